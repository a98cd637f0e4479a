"""Differentiable fast-path powder average and gradient-based fitting (K6).

The reference fits by re-running ``ExperimentRunner`` per objective
evaluation and letting scipy difference it numerically
(muspinsim/fitting.py:67-179).  Here the powder average of
``Hamiltonian.fast_evolve`` (muspinsim/hamiltonian.py:166-217) is a
``torch.autograd.Function`` whose backward pass is the CUDA adjoint
``msp_adjoint_fast``: dL/dHsys and dL/dB_lab for an upstream dL/dP(t).
Couplings enter through :class:`TorchSpinHamiltonian`, a torch restatement of
the term matrices of ``SpinSystem`` (muspinsim/spinsys.py:34-69, 354-442),
so gradients reach hyperfine tensors, dipolar vectors and the field by
ordinary autograd on the host side.
"""

import numpy as np
import scipy.constants as cnst
import torch

from muspinsim_gb300 import _lib, kernels
from muspinsim_gb300 import quaternion as Q
from muspinsim_gb300.constants import EFG_2_MHZ
from muspinsim_gb300.orientations import orientation_rows_to_quats
from muspinsim_gb300.spinsys import MuonSpinSystem

_PREC = {"fp64": _lib.PREC_FP64, "mixed": _lib.PREC_MIXED}


class FastPowder(torch.autograd.Function):
    """P(t) = sum_s wscale_s P_s(t) on the fast path; differentiable in
    Hsys (complex (n, n)) and the lab-frame fields (S, 3)."""

    @staticmethod
    def forward(ctx, Hsys, field, Z, pol, wscale, times, precision):
        n = Hsys.shape[-1]
        S = field.shape[0]
        slot = torch.zeros(S, dtype=torch.int32, device=field.device)
        plan = kernels.PowderPlan(n, Hsys.detach(), Z, field.detach(), pol, wscale, slot, 1,
                                  times, mode=_lib.MODE_FAST, precision=precision)
        out = plan.run().reshape(-1).clone()
        st = int(plan.status[:S].max().item()) if S else 0
        if st & _lib.MSP_ITEM_NOT_CONVERGED:
            raise RuntimeError("fast powder: an eigensolve reached its sweep cap")
        ctx.save_for_backward(Hsys.detach(), field.detach(), Z, pol, wscale, times)
        return out

    @staticmethod
    def backward(ctx, grad_out):
        Hsys, field, Z, pol, wscale, times = ctx.saved_tensors
        S = field.shape[0]
        slot = torch.zeros(S, dtype=torch.int32, device=field.device)
        gH, gF, _ = kernels.adjoint_fast(Hsys.shape[-1], Hsys, Z, field, pol, wscale, slot, 1,
                                         times, grad_out.reshape(1, -1).contiguous(),
                                         want_field=ctx.needs_input_grad[1])
        return (gH if ctx.needs_input_grad[0] else None, gF, None, None, None, None, None)


def fast_powder(Hsys, field, Z, pol, wscale, times, precision="fp64"):
    """Differentiable powder average on the fast path (muon first, T = inf).

    Hsys: (n, n) complex128 tensor; field: (S, 3) float64 lab-frame fields;
    Z: (3, n, n) complex; pol: (S, 3); wscale: (S,) weights (sum_s w_s P_s);
    times: 1-D.  Returns P(t) as a float64 tensor on the device."""
    d = kernels.device()
    Z = kernels.dev(Z, torch.complex128)
    pol = kernels.dev(pol, torch.float64).reshape(-1, 3)
    wscale = kernels.dev(wscale, torch.float64).reshape(-1)
    times = kernels.dev(times, torch.float64).reshape(-1)
    return FastPowder.apply(Hsys.to(d), field.to(d), Z, pol, wscale, times, _PREC[precision])


class TorchSpinHamiltonian:
    """Term matrices of a spin system as differentiable torch functions.

    Same conventions as ``SpinSystem``: spin 0 is the slowest index, a
    bilinear term is sum_ab T_ab S^a_i S^b_j (the matrix product when
    i == j), the dipolar tensor is -(mu0 hbar gamma_i gamma_j 1e6 /
    (2 |r|^3)) (3 r r^T / |r|^2 - 1) with r in Angstrom, and the Zeeman
    operators are Z_a = sum_i gamma_i S^a_i (MHz, T)."""

    def __init__(self, spins, device=None):
        self.system = MuonSpinSystem(spins)
        self.device = device if device is not None else kernels.device()
        n = int(np.prod(self.system.dimension))
        self.n = n
        self.S = [[torch.as_tensor(self.system.operator({i: ax}).matrix.toarray(),
                                   dtype=torch.complex128, device=self.device)
                   for ax in "xyz"] for i in range(len(self.system))]
        self.Z = torch.as_tensor(self.system.zeeman_operators(), dtype=torch.complex128,
                                 device=self.device)
        self._prod = {}

    def gamma(self, i):
        return float(self.system.gamma(i))

    def _pair(self, i, j):
        key = (i, j)
        if key not in self._prod:
            self._prod[key] = torch.stack([torch.stack([self.S[i][a] @ self.S[j][b]
                                                        for b in range(3)]) for a in range(3)])
        return self._prod[key]

    def bilinear(self, i, j, T):
        """sum_ab T_ab S^a_i S^b_j for a real (3, 3) tensor T (MHz)."""
        T = torch.as_tensor(T, dtype=torch.float64, device=self.device)
        return torch.einsum("ab,abij->ij", T.to(torch.complex128), self._pair(i, j))

    def zeeman(self, i, B):
        B = torch.as_tensor(B, dtype=torch.float64, device=self.device)
        g = self.gamma(i)
        return sum(g * B[a].to(torch.complex128) * self.S[i][a] for a in range(3))

    def hyperfine(self, i, j, A):
        return self.bilinear(i, j, A)

    def dipolar(self, i, j, r):
        r = torch.as_tensor(r, dtype=torch.float64, device=self.device)
        rn = torch.linalg.norm(r)
        D = -(torch.eye(3, dtype=torch.float64, device=self.device)
              - 3.0 / rn**2 * torch.outer(r, r))
        dij = -(cnst.mu_0 * cnst.hbar * (self.gamma(i) * self.gamma(j) * 1e6)) / (2 * (rn * 1e-10) ** 3)
        return self.bilinear(i, j, D * dij)

    def quadrupolar(self, i, EFG):
        Qm = self.system.Q(i)
        I = self.system.I(i)
        if I == 0.5:
            raise ValueError("Can not set up quadrupolar coupling for spin 1/2 particle")
        return self.bilinear(i, i, EFG_2_MHZ * Qm / (2 * I * (2 * I - 1)) * torch.as_tensor(EFG))


def powder_geometry(orientations, polarization=(1.0, 0.0, 0.0), mode="zyz"):
    """Rotation matrices, weights and lab-frame polarisations of an
    orientation list (same conventions as powder_average): (R (N, 3, 3),
    wscale (N,), pol (N, 3)) with B_lab = R @ B."""
    qs, ws = orientation_rows_to_quats(orientations, mode)
    N = len(qs)
    ws = ws * (N / ws.sum()) if N > 1 else np.ones(1)
    p = np.asarray(polarization, dtype=float)
    p = p / np.linalg.norm(p)
    R = Q.rotation_matrix(qs).reshape(N, 3, 3)
    return R, ws / N, Q.rotate(qs, p)


class GradientFitter:
    """Least-squares fit of fast-path powder data with analytic gradients
    (the gradient-based counterpart of the reference's FittingRunner
    objective, muspinsim/fitting.py:67-124).

    ``model(params) -> (Hsys, B)``: torch functions of the parameter
    tensors (Hsys complex (n, n), B the crystal-frame field (3,)).
    Loss: sum_t (P(t) - data(t))^2."""

    def __init__(self, model, Z, orientations, times, data, polarization=(1.0, 0.0, 0.0),
                 precision="fp64"):
        self.model = model
        d = kernels.device()
        R, w, p = powder_geometry(orientations, polarization)
        self.R = torch.as_tensor(R, dtype=torch.float64, device=d)
        self.w = torch.as_tensor(w, dtype=torch.float64, device=d)
        self.pol = torch.as_tensor(p, dtype=torch.float64, device=d)
        self.Z = kernels.dev(Z, torch.complex128)
        self.times = kernels.dev(times, torch.float64)
        self.data = kernels.dev(data, torch.float64)
        self.precision = precision
        self.evaluations = 0

    def signal(self, params):
        Hsys, B = self.model(params)
        B_lab = torch.einsum("sab,b->sa", self.R, B)
        return fast_powder(Hsys, B_lab, self.Z, self.pol, self.w, self.times, self.precision)

    def loss(self, params):
        self.evaluations += 1
        r = self.signal(params) - self.data
        return (r * r).sum()

    def loss_and_grad(self, params):
        """(loss, [d loss / d p for p in params]) with params requiring grad."""
        L = self.loss(params)
        grads = torch.autograd.grad(L, params)
        return L, grads

    def fit(self, x0, method="L-BFGS-B", **kw):
        """Minimise over a flat float64 vector split like ``x0`` (a list of
        arrays); returns the scipy result with ``x`` split back."""
        from scipy.optimize import minimize

        shapes = [np.shape(x) for x in x0]
        sizes = [int(np.prod(s)) for s in shapes]
        d = kernels.device()

        def unpack(x):
            out, k = [], 0
            for s, m in zip(shapes, sizes):
                out.append(torch.tensor(x[k:k + m].reshape(s), dtype=torch.float64, device=d,
                                        requires_grad=True))
                k += m
            return out

        def fun(x):
            ps = unpack(x)
            L, gs = self.loss_and_grad(ps)
            g = np.concatenate([gg.detach().cpu().numpy().ravel() for gg in gs])
            return float(L.item()), g

        x = np.concatenate([np.ravel(v) for v in x0]).astype(float)
        res = minimize(fun, x, jac=True, method=method, **kw)
        res.params = [p.detach().cpu().numpy() for p in unpack(res.x)]
        return res
