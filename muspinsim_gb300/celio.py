"""Celio's method, API-compatible with ``muspinsim/celio.py``.

The Hamiltonian is split into contributions that each act on one or two
spins; one time step is the Trotter product (prod_c U_c)^k with U_c =
exp(-2 pi i H_c dt / k) (Phys. Rev. Lett. 56, 2720 (1986)).  Building the
contributions and exponentiating the field-independent ones are small host
computations, as in the reference; every evolution runs on the GPU through
``msp_celio_run`` -- FP64, or double-word FP32 on the FP32 pipe for the
'mixed' precision -- with the field-dependent factors of a batch of
snapshots exponentiated on the device (``msp_celio_expm``).

* ``CelioHamiltonian.fast_evolve``: averaged random initial states (the
  reference's native module, muspinsim/cpp/celio.cpp:23-64).  The random
  numbers are drawn with ``np.random.rand(d)`` per average, as the
  reference draws them, so a seeded run reproduces the reference's.
* ``CelioHamiltonian.evolve``: the density-matrix variant, rho(t_i) =
  T^dag rho0 T with T = E^i, applied factor by factor on the GPU.
"""

import itertools
import logging
from dataclasses import dataclass
from typing import List

import numpy as np
from scipy import sparse
from scipy.linalg import expm

from muspinsim_gb300 import _lib, kernels
from muspinsim_gb300.spinop import spin_projectors
from muspinsim_gb300.validation import validate_celio_params, validate_evolve_params, \
    validate_times


@dataclass
class CelioHContrib:
    """One contribution H_c (muspinsim/celio.py:28-51): its matrix over the
    spins it involves, the dimension of the others, the order of the
    Kronecker factors (involved spins first) and their dimensions."""

    matrix: sparse.csr_matrix
    other_dimension: int
    spin_order: List[int]
    spin_dimensions: List[int]


class CelioEvolveContrib:
    """A Trotter factor as the reference's ``Celio_EvolveContrib``
    (muspinsim/cpp/celio.cpp:4-11): dense matrix, dimension of the
    remaining spins and the index map of the reordered Kronecker product
    (built on first access; the GPU enumerates the groups from the digit
    strides instead)."""

    def __init__(self, matrix, other_dim, spin_order, dimension):
        self.matrix = np.asarray(matrix, dtype=complex)
        self.other_dim = int(other_dim)
        self.spin_order = list(spin_order)
        self._dimension = tuple(dimension)
        self._indices = None

    @property
    def indices(self):
        if self._indices is None:
            n = int(np.prod(self._dimension))
            self._indices = np.transpose(
                np.arange(n, dtype=np.uint64).reshape(self._dimension),
                axes=self.spin_order).flatten()
        return self._indices


def _dense(m):
    return m.toarray() if sparse.issparse(m) else np.asarray(m)


def _field_zero(B):
    return np.array_equal(np.asarray(B, dtype=float), [0.0, 0.0, 0.0])


class CelioHamiltonian:
    """Hamiltonian for Celio's method (muspinsim/celio.py:54-486)."""

    def __init__(self, terms, k, spinsys):
        self._terms = list(terms)
        self._k = k
        self._spinsys = spinsys

    def __add__(self, x):
        return CelioHamiltonian(self._terms + x._terms, self._k, self._spinsys)

    # ----------------------------------------------------------- contributions
    def _groups(self):
        """Runs of terms forming each contribution (muspinsim/celio.py:73-143):
        per spin i, the terms whose first index is i, split into runs of equal
        index tuples (only consecutive terms merge)."""
        L = len(self._spinsys.spins)
        out = []
        for i in range(L):
            spin_ints = [t for t in self._terms if i == t.indices[0]]
            other = [s for s in range(L) if s != i]
            for indices, grp in itertools.groupby(spin_ints, lambda t: t.indices):
                grp = list(grp)
                unin = list(other)
                for t in grp:
                    for j in t.indices:
                        if j in unin:
                            unin.remove(j)
                indices = [int(j) for j in indices]
                if len(indices) == 2 and indices[0] == indices[1]:
                    indices.pop()
                out.append((grp, unin, indices + unin))
        return out

    def _calc_H_contribs(self):
        dims = self._spinsys.dimension
        out = []
        for grp, unin, order in self._groups():
            H = grp[0].matrix
            for t in grp[1:]:
                H = H + t.matrix
            other = int(np.prod([dims[j] for j in unin])) if unin else 1
            out.append(CelioHContrib(sparse.csr_matrix(H), other, order,
                                     [dims[s] for s in order]))
        return out

    def _calc_trotter_evol_op_contribs(self, time_step, cpp):
        """U_c = expm(-2 pi i H_c dt / k) (muspinsim/celio.py:145-208): as
        ``CelioEvolveContrib`` for ``cpp``, else as the full-space sparse
        matrix (U_c (x) 1 reordered to the system's spin order)."""
        dims = tuple(self._spinsys.dimension)
        out = []
        for hc in self._calc_H_contribs():
            U = expm(-2j * np.pi * _dense(hc.matrix) * time_step / self._k)
            if cpp:
                out.append(CelioEvolveContrib(U, hc.other_dimension, hc.spin_order, dims))
            else:
                out.append(sparse.csr_matrix(_full_factor(U, dims, hc.spin_order)))
        return out

    # ----------------------------------------------------------- evolution
    def evolve(self, rho0, times, operators):
        """Density-matrix variant on the GPU (muspinsim/celio.py:210-293):
        returns complex [T, n_ops] expectation values of rho(t_i) =
        T^dag rho0 T, T = E^i, E = (prod_c F_c)^k."""
        times = np.array(times)
        if not operators:
            raise ValueError("At least one SpinOperator must be present in 'operators'")
        if not isinstance(operators, (list, tuple)):
            operators = [operators]
        validate_evolve_params(rho0, times, operators)
        validate_celio_params(self._terms, times)
        dt = times[1] - times[0]
        dims = list(self._spinsys.dimension)
        factors = self._calc_trotter_evol_op_contribs(dt, True)
        plan = _density_plan(dims, [(f.matrix, f.spin_order) for f in factors])
        N = int(np.prod(dims))
        meas = np.stack([_dense(o.matrix).T for o in operators])[None]
        series, _ = kernels.celio_run(
            _lib.CELIO_DENSITY, dims + dims, plan["digits"], plan["mat"], plan["block"][None],
            False, 1, 1, self._k, len(times), rho0=_dense(rho0.matrix).reshape(1, N, N),
            meas=meas, meas_per_snapshot=False)
        return series[0].cpu().numpy()

    def fast_evolve(self, sigma_mu, times, averages, cpp=True):
        """Averaged random-state variant on the GPU (muspinsim/celio.py:
        318-476): returns float64 [T], 0.5 x the mean over ``averages``
        initial states of Re <psi(t)|(sigma_mu (x) 1)|psi(t)>."""
        times = np.array(times)
        validate_times(times)
        validate_celio_params(self._terms, times)
        if averages <= 0:
            raise ValueError("averages must be a positive integer")
        if self._spinsys.muon_index != 0:
            raise ValueError("Muon must be the first spin in the system in order to use "
                             "the fast Celio method")
        dt = times[1] - times[0]
        dims = list(self._spinsys.dimension)
        half = int(np.prod(dims)) // 2
        sig = _dense(sigma_mu).astype(complex)
        mu_psi = _mu_psi(sig)
        phases = np.random.rand(int(averages) * half).reshape(1, int(averages), half)
        factors = self._calc_trotter_evol_op_contribs(dt, True)
        plan = _pure_plan(dims, [(f.matrix, f.spin_order) for f in factors])
        _, rows = kernels.celio_run(
            _lib.CELIO_PURE, dims, plan["digits"], plan["mat"], plan["block"][None], False, 1,
            int(averages), self._k, len(times), mu_psi=mu_psi[None], sigma=sig[None],
            phases=phases, row_start=np.array([0, 1]), num_rows=1)
        return rows[0].cpu().numpy()

    def integrate_decaying(self, rho0, tau, operators):
        raise NotImplementedError("integrate_decaying is not implemented for Celio's method")


# ---------------------------------------------------------------- factor tables
def _full_factor(U, dims, order):
    """(U (x) 1) in the permuted spin order, reordered to the system's
    (muspinsim/celio.py:180-206)."""
    N = int(np.prod(dims))
    D = U.shape[0]
    F = np.kron(U, np.eye(N // D))
    sd = [dims[s] for s in order]
    L = len(dims)
    perm = [int(p) for p in np.argsort(order)]
    return F.reshape(sd + sd).transpose(perm + [L + p for p in perm]).reshape(N, N)


def _involved(order, D, dims):
    """Digits a factor of dimension D acts on, in its own order."""
    d0 = int(order[0])
    return (d0, int(order[1])) if D != dims[d0] else (d0, -1)


def _pure_plan(dims, factors):
    """Factor descriptors and one matrix block for CELIO_PURE."""
    digits, mat, block, off = [], [], [], 0
    for U, order in factors:
        D = U.shape[0]
        digits.append(_involved(order, D, dims))
        mat.append(off)
        block.append(np.asarray(U, dtype=complex).reshape(-1))
        off += D * D
    block = np.concatenate(block) if block else np.zeros(1, dtype=complex)
    return {"digits": np.array(digits, dtype=np.int32).reshape(-1, 2),
            "mat": np.array(mat, dtype=np.int64), "block": block}


def _density_plan(dims, factors):
    """CELIO_DENSITY: per factor U^dagger on the row digits and U^T on the
    column digits, so that a pass maps rho to U^dagger rho U."""
    L = len(dims)
    digits, mat, block, off = [], [], [], 0
    for U, order in factors:
        U = np.asarray(U, dtype=complex)
        D = U.shape[0]
        d0, d1 = _involved(order, D, dims)
        digits.append((d0, d1))
        mat.append(off)
        block.append(U.conj().T.reshape(-1))
        off += D * D
        digits.append((L + d0, L + d1 if d1 >= 0 else -1))
        mat.append(off)
        block.append(U.T.reshape(-1))
        off += D * D
    block = np.concatenate(block) if block else np.zeros(1, dtype=complex)
    return {"digits": np.array(digits, dtype=np.int32).reshape(-1, 2),
            "mat": np.array(mat, dtype=np.int64), "block": block}


def _mu_psi(sig):
    """Muon state of eigenvalue +1 of sigma_mu, chosen as the reference does
    (muspinsim/celio.py:361-363); one 2 x 2 matrix or a stack of them."""
    sig = np.asarray(sig, dtype=complex)
    evals, evecs = np.linalg.eig(sig + np.eye(2))
    if sig.ndim == 2:
        return evecs[:, 1] if np.real(evals[1]) > 0.1 else evecs[:, 0]
    pick = np.where(np.real(evals[:, 1]) > 0.1, 1, 0)
    return evecs[np.arange(len(sig)), :, pick]


# ---------------------------------------------------------------- batched snapshots
class CelioBatch:
    """Every snapshot of an ExperimentRunner with Celio's method, prepared
    once and run as one batch (muspinsim/experiment.py:239-269, 434-471).

    The Trotter pass holds the system's terms plus, when any snapshot has a
    field, every spin's Zeeman term; factors holding a Zeeman term are
    exponentiated per snapshot on the GPU (``msp_celio_expm``), the others
    once on the host.  With ``averages`` > 0 (random initial states) the
    uniform numbers come from np.random.rand in the reference's order --
    snapshot by snapshot, average by average -- or, with
    ``device_phases``, from the library's counter-based generator keyed by
    ``seed``.  Construction uploads everything; :meth:`run` launches
    ``msp_celio_run`` only and returns the (nrows, T) results on the
    device."""

    def __init__(self, system, k, averages, B_lab, p_lab, T, wscale, rows, nrows, times,
                 device_phases=False, seed=0, precision="fp64"):
        import torch

        from muspinsim_gb300.spinsys import SingleTerm

        times = np.asarray(times, dtype=float)
        B_lab = np.asarray(B_lab, dtype=float).reshape(-1, 3)
        p_lab = np.asarray(p_lab, dtype=float).reshape(-1, 3)
        S = len(B_lab)
        dims = list(system.dimension)
        L = len(dims)
        N = int(np.prod(dims))
        any_field = any(not _field_zero(b) for b in B_lab)
        zterms = []
        if any_field:
            zterms = [SingleTerm(system, i, np.array([0.0, 0.0, 1.0]) * system.gammas[i],
                                 label="Zeeman") for i in range(L)]
        H = CelioHamiltonian(system.terms + zterms, k, system)
        # a snapshot without field evolves under the system's terms alone
        all_field = all(not _field_zero(b) for b in B_lab)
        validate_celio_params(H._terms if all_field else system.terms, times)
        dt = times[1] - times[0]
        pure = averages > 0
        if pure:
            if np.any(np.asarray(T, dtype=float) != np.inf):
                raise ValueError("The fast version of Celio's method requires T -> inf. Either "
                                 "remove the number of averages or don't use celio.")
            if system.muon_index != 0:
                raise ValueError("Muon must be the first spin in the system in order to use "
                                 "the fast Celio method")

        # contributions; those holding a Zeeman term depend on the snapshot's field
        zids = {id(t) for t in zterms}
        static, field = [], []
        for pos, (grp, unin, order) in enumerate(H._groups()):
            Hs = None
            for t in grp:
                if id(t) not in zids:
                    Hs = _dense(t.matrix) if Hs is None else Hs + _dense(t.matrix)
            zs = [t for t in grp if id(t) in zids]
            if zs:
                i = int(zs[0].indices[0])
                D = dims[i]
                G = np.array([system.gammas[i] * _dense(system._operators[i][ax].matrix)
                              for ax in "xyz"], dtype=complex)
                field.append((pos, np.zeros((D, D), dtype=complex) if Hs is None else Hs, G,
                              order))
            else:
                static.append((pos, expm(-2j * np.pi * Hs * dt / k), order))

        per = 1 if pure else 2
        Ds = {pos: (U.shape[0], order) for pos, U, order in static}
        Ds.update({pos: (H0.shape[0], order) for pos, H0, G, order in field})
        nfac = len(Ds)
        offs, off = {}, 0
        for pos in range(nfac):
            offs[pos] = off
            off += per * Ds[pos][0] ** 2
        mats_len = max(off, 1)
        digits, mat = [], []
        for pos in range(nfac):
            D, order = Ds[pos]
            d0, d1 = _involved(order, D, dims)
            digits.append((d0, d1))
            mat.append(offs[pos])
            if not pure:
                digits.append((L + d0, L + d1 if d1 >= 0 else -1))
                mat.append(offs[pos] + D * D)
        block = np.zeros(mats_len, dtype=complex)
        for pos, U, order in static:
            D = U.shape[0]
            o = offs[pos]
            if pure:
                block[o:o + D * D] = U.reshape(-1)
            else:
                block[o:o + D * D] = U.conj().T.reshape(-1)
                block[o + D * D:o + 2 * D * D] = U.T.reshape(-1)

        d = kernels.device()
        order_s = np.argsort(np.asarray(rows), kind="stable")
        rows_sorted = np.asarray(rows)[order_s]
        self.row_start = kernels.dev(
            np.searchsorted(rows_sorted, np.arange(nrows + 1)).astype(np.int32), torch.int32)
        if field:
            mats = kernels.dev(np.broadcast_to(block, (S, mats_len)), torch.complex128).clone()
            out_off = []
            for pos, H0, G, order in field:
                D = H0.shape[0]
                o = offs[pos]
                out_off.append((o, -1, -1) if pure else (-1, o, o + D * D))
            kernels.celio_expm([f[1].shape[0] for f in field], [f[1] for f in field],
                               [f[2] for f in field], B_lab[order_s], dt / k, out_off, mats)
            self.per_snap = True
        else:
            mats = kernels.dev(block[None], torch.complex128)
            self.per_snap = False
        self.mats = mats
        self.digits = np.array(digits, dtype=np.int32).reshape(-1, 2)
        self.mat = np.array(mat, dtype=np.int64)
        self.dims, self.k, self.S, self.T = dims, int(k), S, len(times)
        self.precision = _lib.PREC_MIXED if precision == "mixed" else _lib.PREC_FP64
        self.nrows = int(nrows)
        self.pure = pure
        self.averages = int(averages)
        self.wscale = kernels.dev(np.asarray(wscale, dtype=float)[order_s], torch.float64)
        p_sorted = p_lab[order_s]
        if pure:
            half = N // 2
            sig = np.empty((S, 2, 2), dtype=complex)
            sig[:, 0, 0] = p_lab[:, 2]
            sig[:, 0, 1] = p_lab[:, 0] - 1j * p_lab[:, 1]
            sig[:, 1, 0] = p_lab[:, 0] + 1j * p_lab[:, 1]
            sig[:, 1, 1] = -p_lab[:, 2]
            mu = _mu_psi(sig) if S else np.zeros((0, 2), dtype=complex)
            self.sigma = kernels.dev(sig[order_s], torch.complex128)
            self.mu_psi = kernels.dev(mu[order_s], torch.complex128)
            self.seed = int(seed)
            self.phases = None
            if not device_phases:
                ph = np.random.rand(S * self.averages * half).reshape(S, self.averages, half)
                self.phases = kernels.dev(ph[order_s], torch.float64)
            return

        from muspinsim_gb300.experiment import thermal_state

        rho = np.empty((S, N, N), dtype=complex)
        for s_i, s in enumerate(order_s):
            fac = []
            for i in range(L):
                if i == system.muon_index:
                    fac.append(spin_projectors(system.I(i), p_lab[s])[0][1])
                else:
                    fac.append(thermal_state(system.I(i), system.gamma(i), B_lab[s], T[s]))
            M = fac[0]
            for m in fac[1:]:
                M = np.kron(M, m)
            rho[s_i] = M
        self.rho0 = kernels.dev(rho, torch.complex128)
        self.meas = kernels.dev(np.stack([_dense(system.operator({system.muon_index: ax}).matrix).T
                                          for ax in "xyz"])[None], torch.complex128)
        self.pol = torch.as_tensor(p_sorted, dtype=torch.complex128, device=d)
        self.rows_sorted = torch.as_tensor(rows_sorted, dtype=torch.int64, device=d)

    def run(self, path=0):
        import torch

        if self.pure:
            _, out = kernels.celio_run(
                _lib.CELIO_PURE, self.dims, self.digits, self.mat, self.mats, self.per_snap, self.S,
                self.averages, self.k, self.T, mu_psi=self.mu_psi, sigma=self.sigma,
                phases=self.phases, seed=self.seed, wscale=self.wscale, row_start=self.row_start,
                num_rows=self.nrows, path=path, precision=self.precision)
            return out
        series, _ = kernels.celio_run(
            _lib.CELIO_DENSITY, self.dims + self.dims, self.digits, self.mat, self.mats,
            self.per_snap, self.S, 1, self.k, self.T, rho0=self.rho0, meas=self.meas, path=path,
            precision=self.precision)
        vals = torch.real(torch.einsum("sta,sa->st", series, self.pol))
        out = torch.zeros((self.nrows, self.T), dtype=torch.float64, device=vals.device)
        out.index_add_(0, self.rows_sorted, vals * self.wscale[:, None])
        return out


def run_snapshots(system, k, averages, B_lab, p_lab, T, wscale, rows, nrows, times,
                  precision="fp64"):
    """All snapshots of an ExperimentRunner with Celio's method: the
    (nrows, T) float64 results on the device (see CelioBatch).  'mixed'
    runs double-word FP32 where the state fits in shared memory."""
    return CelioBatch(system, k, averages, B_lab, p_lab, T, wscale, rows, nrows, times,
                      precision=precision).run()


logging.getLogger(__name__).addHandler(logging.NullHandler())
