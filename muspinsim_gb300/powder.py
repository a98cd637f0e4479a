"""Batched snapshot engine: many (orientation, field, temperature) snapshots
of one spin system evaluated in one GPU pipeline.

This is the GB300 replacement of the reference's per-snapshot Python loop
(``ExperimentRunner.run`` -> ``run_single``, muspinsim/experiment.py:358-498):
the host prepares per-snapshot 3-vectors (rotated field and polarisation),
weights and output rows, picks the evolution path of every snapshot with the
reference's rule, and hands each path group to ``msp_powder_run``, which
assembles, diagonalises and evolves all snapshots and reduces them into the
output rows on the device.
"""

import numpy as np
import scipy.constants as cnst
import torch

from muspinsim_gb300 import _lib, kernels
from muspinsim_gb300 import quaternion as Q
from muspinsim_gb300.constants import MU_TAU
from muspinsim_gb300.orientations import orientation_rows_to_quats

PRECISIONS = {"fp64": _lib.PREC_FP64, "mixed": _lib.PREC_MIXED}


def precision_code(precision):
    if isinstance(precision, str):
        try:
            return PRECISIONS[precision]
        except KeyError as exc:
            raise ValueError(f"precision must be one of {list(PRECISIONS)}") from exc
    return int(precision)


def t_inf_speedup(B_lab, T, mu_index):
    """Per-snapshot fast-path flag: e hbar^2 |B| / (2 m_p k T) == 0 and the
    muon is spin 0 (muspinsim/experiment.py:413-430)."""
    Bn = np.linalg.norm(np.atleast_2d(B_lab), axis=1)
    T = np.broadcast_to(np.asarray(T, dtype=float), Bn.shape)
    with np.errstate(divide="ignore", invalid="ignore"):
        check = (cnst.e * (cnst.hbar**2) * Bn) / (2 * cnst.m_p * cnst.k * T)
    return (check == 0) & (mu_index == 0)


def _rows_sorted(slot):
    order = np.argsort(slot, kind="stable")
    return order


_PLANS = {}
_ORIENT_BUFFERS = {}


def _orient_buffers(N, L):
    """OrientBuffers for N rows of length L on the current device, reused
    across powder_average calls (every call synchronises before it returns,
    so the pinned rows are free again by the next call)."""
    key = (N, L, torch.cuda.current_device())
    b = _ORIENT_BUFFERS.get(key)
    if b is None:
        if len(_ORIENT_BUFFERS) >= 8:
            _ORIENT_BUFFERS.clear()
        b = _ORIENT_BUFFERS[key] = kernels.OrientBuffers(N, L)
    return b


def _cached_plan(system, Hs, Zd, n, F, Pl, W, slot, num_slots, times, mode, prec, dims, mu, Tarr,
                 max_sweeps):
    """A PowderPlan for the device-side powder_average path, reused across
    calls with the same system matrices and sizes (its output, status and
    workspace stay allocated; only the per-call inputs are re-pointed and
    the time grid re-uploaded).  Plans with finite temperatures are not
    cached."""
    th = np.asarray(times, dtype=float)
    key = (Hs.data_ptr(), Zd.data_ptr(), int(F.shape[0]), th.size, int(num_slots), mode, prec,
           max_sweeps, Tarr is None)
    plan = _PLANS.get(key) if Tarr is None else None
    if plan is None:
        plan = kernels.PowderPlan(n, Hs, Zd, F, Pl, W, slot, num_slots, th, mode=mode,
                                  precision=prec, dims=dims, mu_index=mu, gammas=system.gammas,
                                  temperature=Tarr, tau=MU_TAU, max_sweeps=max_sweeps)
        if Tarr is None:
            if len(_PLANS) >= 8:
                _PLANS.clear()
            _PLANS[key] = plan
        return plan
    plan.rebind(F, Pl, W, slot)
    last = getattr(plan, "_times_host", None)
    if last is None or not np.array_equal(last, th):  # the grid only moves when it changed
        uni, t0, dt = kernels.uniform_grid(th)
        plan.T.copy_(torch.as_tensor(th), non_blocking=False)
        a = plan.args
        a.uniform, a.t0, a.dt = (1 if uni else 0), t0, dt
        plan._times_host = th.copy()
    return plan


def run_snapshots(system, B_lab, p_lab, T, wscale, slot, num_slots, times,
                  y_axis="asymmetry", precision="fp64", max_sweeps=0, Hsys=None, Z=None,
                  fast_mask=None, host_out=False):
    """Evaluate and reduce a batch of snapshots on the GPU.

    B_lab, p_lab: (S, 3) lab-frame field (incl. intrinsic) and muon
    polarisation; T: scalar or (S,) temperatures; wscale: (S,) weight /
    averaged count; slot: (S,) output row.  Returns a device tensor of shape
    (num_slots, len(times)) for 'asymmetry' or (num_slots,) for 'integral',
    and the per-snapshot status (host int array, original order).

    ``fast_mask``: a precomputed fast-path decision (bool, one for all
    snapshots); B_lab, p_lab and wscale may then be device tensors and
    ``slot`` None (every snapshot in row 0).  ``host_out``: return the
    output as a host numpy array (on that path fetched together with the
    status after a single synchronisation)."""
    prec = precision_code(precision)
    dev = kernels.device()
    if fast_mask is not None and isinstance(B_lab, torch.Tensor):
        S = int(B_lab.shape[0])
        if slot is None:
            slot = torch.zeros(S, dtype=torch.int32, device=dev)
    else:
        B_lab = np.ascontiguousarray(np.atleast_2d(B_lab), dtype=float)
        p_lab = np.ascontiguousarray(np.atleast_2d(p_lab), dtype=float)
        S = len(B_lab)
        wscale = np.broadcast_to(np.asarray(wscale, dtype=float), (S,))
        slot = np.broadcast_to(np.asarray(0 if slot is None else slot, dtype=np.int64), (S,))
    Tarr = np.broadcast_to(np.asarray(T, dtype=float), (S,))
    if Hsys is None and Z is None:
        Hs, Zd = system.device_matrices(dev)
        n = int(Hs.shape[0])
    else:
        if Hsys is None:
            Hsys = system.hamiltonian_matrix()
        if Z is None:
            Z = system.zeeman_operators()
        n = Hsys.shape[0]
        Hs = kernels.dev(Hsys, torch.complex128)
        Zd = kernels.dev(Z, torch.complex128)
    dims = list(system.dimension)
    mu = system.muon_index
    if fast_mask is not None and isinstance(B_lab, torch.Tensor):
        mode = _lib.MODE_INTEGRAL if y_axis == "integral" else (
            _lib.MODE_FAST if fast_mask else _lib.MODE_EVOLVE)
        plan = _cached_plan(system, Hs, Zd, n, B_lab, p_lab, wscale, slot, num_slots, times, mode,
                            prec, dims, mu, None if mode == _lib.MODE_FAST else Tarr, max_sweeps)
        out = plan.run()
        if host_out:
            return plan.fetch()
        return out, plan.status[:S].cpu().numpy()

    if y_axis == "integral":
        groups = [(_lib.MODE_INTEGRAL, np.ones(S, dtype=bool))]
        out = torch.zeros((num_slots,), dtype=torch.float64, device=dev)
    else:
        fast = t_inf_speedup(B_lab, Tarr, mu)
        groups = [(_lib.MODE_FAST, fast), (_lib.MODE_EVOLVE, ~fast)]
        out = torch.zeros((num_slots, len(times)), dtype=torch.float64, device=dev)
    status = np.zeros(S, dtype=np.int32)
    first = True
    for mode, mask in groups:
        idx = np.nonzero(mask)[0]
        if idx.size == 0:
            continue
        idx = idx[_rows_sorted(slot[idx])]
        res, st = kernels.powder_run(
            n, Hs, Zd, B_lab[idx], p_lab[idx], wscale[idx], slot[idx].astype(np.int32),
            num_slots, times, mode=mode, precision=prec, dims=dims, mu_index=mu,
            gammas=system.gammas, temperature=Tarr[idx], tau=MU_TAU, max_sweeps=max_sweeps)
        if first:
            out = res
            first = False
        else:
            out += res
        status[idx] = st.cpu().numpy()
    if host_out:
        return out.cpu().numpy(), status
    return out, status


def _fast_rule_uniform(field, intrinsic_field, temperature, mu_index):
    """The reference's per-snapshot fast-path rule when it is the same for
    every orientation, else None: T = inf makes the check 0 for any field;
    with no intrinsic field |B_lab| = |B| for every orientation
    (muspinsim/experiment.py:413-430)."""
    T = np.asarray(temperature, dtype=float)
    if T.ndim != 0:
        return None
    if np.isinf(T):
        return mu_index == 0
    if np.any(np.asarray(intrinsic_field, dtype=float) != 0.0):
        return None
    return bool(t_inf_speedup(np.atleast_2d(field), float(T), mu_index)[0])


class OrientationGrid:
    """A powder grid the GPU generates itself: the input language's
    ``orientation zcw(N)`` / ``eulrange(N)`` (muspinsim/utils.py:34-50).
    ``kind``: 'zcw', 'zcw-hemisphere' or 'eulrange' (n^3 points, sin(beta)
    weights); ``mode``: Euler convention of eulrange rows."""

    def __init__(self, kind, n, mode="zyz"):
        if kind not in ("zcw", "zcw-hemisphere", "eulrange"):
            raise ValueError(f"Unknown orientation grid {kind}")
        self.kind, self.n, self.mode = kind, int(n), mode

    def __len__(self):
        return self.n**3 if self.kind == "eulrange" else self.n

    def rows(self):
        """The same grid as host rows (for host-side code and the oracle)."""
        from muspinsim_gb300.orientations import eulrange_gen, zcw_gen

        if self.kind == "eulrange":
            return eulrange_gen(self.n)
        return zcw_gen(self.n, "hemisphere" if self.kind == "zcw-hemisphere" else "sphere")


def powder_scan(system, orientations, fields, polarization=(1.0, 0.0, 0.0), times=None,
                temperature=np.inf, intrinsic_field=(0.0, 0.0, 0.0), y_axis="asymmetry",
                precision="fp64", max_sweeps=0):
    """One orientation-averaged result per field: a field scan (the field as
    x axis or file range, orientations averaged; MuSpinConfig's snapshot
    product, muspinsim/simconfig.py:299-321, run by ExperimentRunner,
    muspinsim/experiment.py:358-498) in one msp_powder_run.

    ``orientations``: an :class:`OrientationGrid` (points and the field x
    orientation product generated on the device, msp_orient_grid_snapshots)
    or explicit rows (product built on the host).  ``fields``: (F, 3) or
    scalars along z (T).  Returns (F, len(times)), or (F,) for 'integral'."""
    F = np.asarray(fields, dtype=float)
    F = np.stack([np.zeros_like(F), np.zeros_like(F), F], axis=1) if F.ndim == 1 else F
    p = np.asarray(polarization, dtype=float)
    p = p / np.linalg.norm(p)
    intr = np.atleast_1d(np.asarray(intrinsic_field, dtype=float))
    if intr.size == 1:
        intr = np.array([0.0, 0.0, intr[0]])
    if y_axis == "integral":
        times = np.array([np.inf])
    times = np.asarray(times, dtype=float)
    nf = len(F)
    T = float(temperature)
    # T = inf: the fast path wherever the muon comes first; a finite
    # temperature: the general path, exact for every field
    fast = bool(np.isinf(T) and system.muon_index == 0)
    if isinstance(orientations, OrientationGrid):
        B_lab, p_lab, W, slot = kernels.orient_grid_snapshots(
            orientations.kind, orientations.n, F, p, intr, orientations.mode)
        res, status = run_snapshots(system, B_lab, p_lab, T, W, slot, nf, times, y_axis,
                                    precision, max_sweeps, fast_mask=fast, host_out=True)
    else:
        qs, ws = orientation_rows_to_quats(orientations)
        N = len(qs)
        ws = ws * (N / ws.sum()) if N > 1 else np.ones(1)
        B_lab = np.concatenate([Q.rotate(qs, f) + intr for f in F])
        p_lab = np.tile(Q.rotate(qs, p), (nf, 1))
        W = np.tile(ws / N, nf)
        slot = np.repeat(np.arange(nf), N)
        res, status = run_snapshots(system, B_lab, p_lab, T, W, slot, nf, times, y_axis,
                                    precision, max_sweeps, host_out=True)
    if np.any(status & _lib.MSP_ITEM_NOT_CONVERGED):
        raise RuntimeError("powder_scan: an eigensolve reached its sweep cap")
    if np.any(status & _lib.MSP_ITEM_BAD_SLOT):
        raise RuntimeError("powder_scan: invalid output rows")
    return res


def powder_average(system, orientations, field=(0.0, 0.0, 0.0), polarization=(1.0, 0.0, 0.0),
                   times=None, temperature=np.inf, intrinsic_field=(0.0, 0.0, 0.0),
                   y_axis="asymmetry", precision="fp64", mode="zyz", max_sweeps=0):
    """Orientation-averaged muon polarisation of one spin system.

    ``orientations``: rows (theta, phi), (a, b, c) or (a, b, c, w) as in the
    reference's ``orientation`` keyword; weights are normalised to sum to N
    and the result is sum_k w_k P_k / N (muspinsim/simconfig.py:152-159,
    347-368).  ``field``: one 3-vector or a scalar along z (T).  Returns a
    float64 numpy array over ``times`` (or a scalar for 'integral').

    A regular grid of rows is rotated on the device (msp_orient_snapshots)
    and the system's matrices stay on the device between calls, so a call
    moves the rows, the time grid and the result across the bus.  Plans and
    orientation buffers are cached per process and reused by the next call
    of the same sizes: calls from several host threads at once must be
    serialised by the caller."""
    if isinstance(orientations, OrientationGrid):
        f = np.atleast_1d(np.asarray(field, dtype=float))
        f = np.array([0.0, 0.0, f[0]]) if f.size == 1 else f
        return powder_scan(system, orientations, f[None, :], polarization, times, temperature,
                           intrinsic_field, y_axis, precision, max_sweeps)[0]
    f = np.atleast_1d(np.asarray(field, dtype=float))
    if f.size == 1:
        f = np.array([0.0, 0.0, f[0]])
    p = np.asarray(polarization, dtype=float)
    p = p / np.linalg.norm(p)
    intr = np.atleast_1d(np.asarray(intrinsic_field, dtype=float))
    if intr.size == 1:
        intr = np.array([0.0, 0.0, intr[0]])
    if y_axis == "integral":
        times = np.array([np.inf])
    times = np.asarray(times, dtype=float)
    rows = None
    if not _ragged_rows(orientations):
        rows = np.ascontiguousarray(orientations, dtype=float)
        if rows.ndim != 2 or rows.shape[1] not in (2, 3, 4):
            rows = None
    fast = _fast_rule_uniform(f + intr, intr, temperature, system.muon_index)
    if rows is not None and fast is not None and len(rows) > 0:
        N = len(rows)
        wnorm = 1.0 / float(rows[:, 3].sum()) if (rows.shape[1] == 4 and N > 1) else 1.0 / N
        bufs = _orient_buffers(N, rows.shape[1])
        F, Pl, W = kernels.orient_snapshots(rows, f, p, intr, mode, wnorm, buffers=bufs)
        res, status = run_snapshots(system, F, Pl, temperature, W, bufs.slot, 1, times, y_axis,
                                    precision, max_sweeps, fast_mask=fast, host_out=True)
    else:
        qs, ws = orientation_rows_to_quats(orientations, mode)
        N = len(qs)
        ws = ws * (N / ws.sum()) if N > 1 else np.ones(1)
        B_lab = Q.rotate(qs, f) + intr
        p_lab = Q.rotate(qs, p)
        res, status = run_snapshots(system, B_lab, p_lab, temperature, ws / N,
                                    np.zeros(N, np.int64), 1, times, y_axis, precision,
                                    max_sweeps, host_out=True)
    if np.any(status & _lib.MSP_ITEM_BAD_SLOT):
        raise RuntimeError("powder_average: invalid output rows")
    return res[0]


def _ragged_rows(rows):
    if isinstance(rows, np.ndarray):
        return rows.dtype == object
    try:
        return len({len(np.atleast_1d(r)) for r in rows}) > 1
    except TypeError:
        return True
