"""Thin Python layer over the C ABI: torch CUDA tensors in, torch tensors out.

Each function here launches one entry point of ``libmspgpu.so`` on the
current torch CUDA stream.  Inputs may be numpy arrays (copied to the
device) or CUDA tensors (used in place).  Nothing here computes on the CPU.
"""

import ctypes

import numpy as np
import torch

from muspinsim_gb300 import _lib

_CUDA_READY = False


def device():
    """The CUDA device the library runs on; raises when there is none.  (The
    availability check and the library load run once; both are slow enough
    to show in a per-call profile.)"""
    global _CUDA_READY
    if not _CUDA_READY:
        if not torch.cuda.is_available():
            raise RuntimeError(
                "muspinsim_gb300 needs a CUDA device: the polarisation kernels have no CPU path"
            )
        _lib.load()
        _CUDA_READY = True
    return torch.device("cuda", torch.cuda.current_device())


def stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else ctypes.c_void_p(0)


def dev(a, dtype):
    """Contiguous device tensor of `dtype` from a numpy array or tensor."""
    d = device()
    if isinstance(a, torch.Tensor):
        return a.to(device=d, dtype=dtype).contiguous()
    arr = np.ascontiguousarray(a)
    if not arr.flags.writeable:  # e.g. a broadcast view: torch wants its own copy
        arr = arr.copy()
    return torch.as_tensor(arr, dtype=dtype).to(d)


def eigh(H, precision=_lib.PREC_FP64, max_sweeps=0):
    """Batched Hermitian eigensolve of (batch, n, n) complex matrices.

    Returns (evals (batch, n) float64 ascending, evecs (batch, n, n)
    complex128 with eigenvectors as columns, status (batch,) int32)."""
    Hd = dev(H, torch.complex128)
    if Hd.dim() == 2:
        Hd = Hd[None]
    b, n, _ = Hd.shape
    evals = torch.empty((b, n), dtype=torch.float64, device=Hd.device)
    evecs = torch.empty((b, n, n), dtype=torch.complex128, device=Hd.device)
    status = torch.empty((b,), dtype=torch.int32, device=Hd.device)
    if n <= _lib.MAX_DIM:
        _lib.call("msp_eigh_batched", ptr(Hd), n, b, int(precision), int(max_sweeps), ptr(evals),
                  ptr(evecs), ptr(status), stream())
        return evals, evecs, status
    # n > 64: Householder + QL in FP64 with caller scratch
    nbytes = ctypes.c_size_t(0)
    _lib.call("msp_eigh_workspace", n, b, ctypes.byref(nbytes))
    ws = torch.empty(int(nbytes.value) + 256, dtype=torch.uint8, device=Hd.device)
    wp = ws.data_ptr() + ((-ws.data_ptr()) % 256)
    _lib.call("msp_eigh_batched_ws", ptr(Hd), n, b, int(precision), int(max_sweeps), ptr(evals),
              ptr(evecs), ptr(status), ctypes.c_void_p(wp), int(nbytes.value), stream())
    return evals, evecs, status


def assemble(Hsys, Z, fields):
    """H[b] = Hsys + sum_a fields[b, a] Z[a]."""
    Hs = dev(Hsys, torch.complex128)
    Zd = dev(Z, torch.complex128)
    F = dev(fields, torch.float64).reshape(-1, 3)
    n = Hs.shape[-1]
    out = torch.empty((F.shape[0], n, n), dtype=torch.complex128, device=Hs.device)
    _lib.call("msp_assemble", ptr(Hs), ptr(Zd), ptr(F), n, F.shape[0], ptr(out), stream())
    return out


def assemble_rotated(system, rotations):
    """Hamiltonians of rotated copies of ``system`` (msp_assemble_rotated):
    for each 3x3 rotation R_s, the Hamiltonian of ``system.rotate(R_s)``
    (bilinear tensors R T R^T, vectors R v).  Returns (S, n, n) complex128
    on the device."""
    tensors, vectors, B = system.rotation_basis()
    d = device()
    R = dev(np.asarray(rotations, dtype=float) if not isinstance(rotations, torch.Tensor)
            else rotations, torch.float64).reshape(-1, 9)
    S, n = int(R.shape[0]), int(B.shape[-1])
    Td = dev(tensors.reshape(-1), torch.float64) if len(tensors) else None
    Vd = dev(vectors.reshape(-1), torch.float64) if len(vectors) else None
    Bd = dev(B, torch.complex128)
    out = torch.empty((S, n, n), dtype=torch.complex128, device=d)
    _lib.call("msp_assemble_rotated", ptr(R), S, ptr(Td), len(tensors), ptr(Vd), len(vectors),
              ptr(Bd), n, ptr(out), stream())
    return out


def basis_change(U, M, adjoint=False):
    """U^dag M U (or U M U^dag when adjoint) for batched or single matrices."""
    Ud = dev(U, torch.complex128)
    Md = dev(M, torch.complex128)
    n = Ud.shape[-1]
    ub = Ud.reshape(-1, n, n).shape[0]
    mb = Md.reshape(-1, n, n).shape[0]
    batch = max(ub, mb)
    if ub not in (1, batch) or mb not in (1, batch):
        raise ValueError("basis_change: incompatible batch sizes")
    out = torch.empty((batch, n, n), dtype=torch.complex128, device=Ud.device)
    _lib.call("msp_basis_change", ptr(Ud), 0 if ub == 1 else n * n, ptr(Md),
              0 if mb == 1 else n * n, n, batch, 1 if adjoint else 0, ptr(out), stream())
    return out


def fast_cos_sum(times, d, A, W):
    t = dev(times, torch.float64)
    Ad = dev(A, torch.float64)
    Wd = dev(W, torch.float64)
    out = torch.empty(t.shape[0], dtype=torch.float64, device=t.device)
    _lib.call("msp_fast_cos_sum", ptr(t), t.shape[0], int(d), ptr(Ad), ptr(Wd), Ad.shape[0],
              ptr(out), stream())
    return out


def fast_amplitudes(evals, evecs, sigma, d):
    ev = dev(evals, torch.float64)
    U = dev(evecs, torch.complex128)
    s = dev(sigma, torch.complex128)
    n = ev.shape[-1]
    A = torch.empty((n, n), dtype=torch.float64, device=ev.device)
    W = torch.empty((n, n), dtype=torch.float64, device=ev.device)
    _lib.call("msp_fast_amplitudes", ptr(ev), ptr(U), ptr(s), n, int(d), ptr(A), ptr(W), stream())
    return A, W


def evolve_expect(evals, rho, ops, times):
    ev = dev(evals, torch.float64)
    r = dev(rho, torch.complex128)
    o = dev(ops, torch.complex128)
    t = dev(times, torch.float64)
    n = ev.shape[-1]
    nops = o.reshape(-1, n, n).shape[0]
    out = torch.empty((t.shape[0], nops), dtype=torch.complex128, device=ev.device)
    _lib.call("msp_evolve_expect", ptr(ev), ptr(r), ptr(o), n, nops, ptr(t), t.shape[0],
              ptr(out), stream())
    return out


def evolve_phases(evals, rho, times):
    ev = dev(evals, torch.float64)
    r = dev(rho, torch.complex128)
    t = dev(times, torch.float64)
    n = ev.shape[-1]
    out = torch.empty((t.shape[0], n, n), dtype=torch.complex128, device=ev.device)
    _lib.call("msp_evolve_phases", ptr(ev), ptr(r), n, ptr(t), t.shape[0], ptr(out), stream())
    return out


def integrate_decaying(evals, rho, ops, tau):
    ev = dev(evals, torch.float64)
    r = dev(rho, torch.complex128)
    o = dev(ops, torch.complex128)
    n = ev.shape[-1]
    nops = o.reshape(-1, n, n).shape[0]
    out = torch.empty((nops,), dtype=torch.complex128, device=ev.device)
    _lib.call("msp_integrate_decaying", ptr(ev), ptr(r), ptr(o), n, nops, float(tau), ptr(out),
              stream())
    return out


class OrientBuffers:
    """Reusable buffers of orient_snapshots for N rows of length L: a pinned
    host copy of the rows (so the upload is asynchronous), the device rows
    and the three outputs.  A caller that reuses them must not overwrite
    the host rows while an upload from them may still run (the powder
    path synchronises at the end of every call)."""

    def __init__(self, N, L):
        d = device()
        self.host = torch.empty((N, L), dtype=torch.float64, pin_memory=True)
        self.host_np = self.host.numpy()
        self.rows = torch.empty((N, L), dtype=torch.float64, device=d)
        self.field = torch.empty((N, 3), dtype=torch.float64, device=d)
        self.pol = torch.empty((N, 3), dtype=torch.float64, device=d)
        self.w = torch.empty((N,), dtype=torch.float64, device=d)
        self.slot = torch.zeros((N,), dtype=torch.int32, device=d)
        self.uploaded = None  # event after the last upload from `host`


def orient_snapshots(rows, B, p, B_intr=(0.0, 0.0, 0.0), mode="zyz", weight_norm=None,
                     buffers=None):
    """Lab-frame field, polarisation and weight/N of every orientation row on
    the device (msp_orient_snapshots).  ``rows``: (N, 2 | 3 | 4) array or
    tensor.  Returns three device tensors: (N, 3), (N, 3), (N,).
    ``buffers``: an OrientBuffers of the same N and row length, whose
    pinned copy, device rows and outputs are used instead of new ones (the
    outputs are then overwritten by the next call with the same buffers)."""
    d = device()
    if buffers is not None and isinstance(rows, np.ndarray):
        if buffers.uploaded is not None:
            buffers.uploaded.synchronize()  # the previous upload has read `host`
        np.copyto(buffers.host_np, rows)
        buffers.rows.copy_(buffers.host, non_blocking=True)
        if buffers.uploaded is None:
            buffers.uploaded = torch.cuda.Event()
        buffers.uploaded.record(torch.cuda.current_stream())
        R = buffers.rows
    else:
        R = dev(rows, torch.float64)
    if R.dim() != 2 or R.shape[1] not in (2, 3, 4):
        raise ValueError("orientation rows must be (theta, phi), (a, b, c) or (a, b, c, w)")
    N, L = int(R.shape[0]), int(R.shape[1])
    if weight_norm is None:
        if L == 4 and N > 1:
            weight_norm = 1.0 / float(R[:, 3].sum().item())
        else:
            weight_norm = 1.0 / max(N, 1)
    if buffers is not None:
        if tuple(buffers.field.shape) != (N, 3):
            raise ValueError("orient_snapshots: buffers are for another row count")
        field, pol, w = buffers.field, buffers.pol, buffers.w
    else:
        field = torch.empty((N, 3), dtype=torch.float64, device=d)
        pol = torch.empty((N, 3), dtype=torch.float64, device=d)
        w = torch.empty((N,), dtype=torch.float64, device=d)
    vec = ctypes.c_double * 3
    _lib.call("msp_orient_snapshots", ptr(R), N, L, 0 if mode == "zyz" else 1,
              vec(*np.asarray(B, dtype=float)), vec(*np.asarray(p, dtype=float)),
              vec(*np.asarray(B_intr, dtype=float)), float(weight_norm), ptr(field), ptr(pol),
              ptr(w), stream())
    return field, pol, w


def orient_grid_snapshots(kind, n, fields, p, B_intr=(0.0, 0.0, 0.0), mode="zyz",
                          generator=None):
    """Snapshots of a device-generated orientation grid times a field list
    (msp_orient_grid_snapshots): kind 'zcw', 'zcw-hemisphere' or 'eulrange'
    with n points (n^3 for eulrange), fields (F, 3).  Returns device tensors
    field (F*No, 3), pol (F*No, 3), weight (F*No,) (weights normalised over
    the grid) and slot (F*No,) int32 (the field index)."""
    from muspinsim_gb300.orientations import zcw_generator

    d = device()
    code = {"zcw": _lib.GRID_ZCW_SPHERE, "zcw-hemisphere": _lib.GRID_ZCW_HEMISPHERE,
            "eulrange": _lib.GRID_EULRANGE}[kind]
    n = int(n)
    No = n**3 if code == _lib.GRID_EULRANGE else n
    if code == _lib.GRID_EULRANGE:
        b = np.linspace(0, np.pi, n + 2)[1:-1]
        wsum = float(np.sin(b).sum()) * n * n
        wnorm = 1.0 / wsum if No > 1 else 1.0
        gen = 1
    else:
        wnorm = 1.0 / No
        gen = zcw_generator(n) if generator is None else int(generator)
    F = dev(np.atleast_2d(np.asarray(fields, dtype=float)), torch.float64).reshape(-1, 3)
    nf = int(F.shape[0])
    field = torch.empty((nf * No, 3), dtype=torch.float64, device=d)
    pol = torch.empty((nf * No, 3), dtype=torch.float64, device=d)
    w = torch.empty((nf * No,), dtype=torch.float64, device=d)
    slot = torch.empty((nf * No,), dtype=torch.int32, device=d)
    vec = ctypes.c_double * 3
    _lib.call("msp_orient_grid_snapshots", code, n, gen, 0 if mode == "zyz" else 1, ptr(F), nf,
              vec(*np.asarray(p, dtype=float)), vec(*np.asarray(B_intr, dtype=float)),
              float(wnorm), ptr(field), ptr(pol), ptr(w), ptr(slot), stream())
    return field, pol, w, slot


def uniform_grid(times, rtol=1e-12):
    """(is_uniform, t0, dt) for a 1-D time array."""
    t = np.asarray(times, dtype=np.float64)
    if t.size == 0:
        return False, 0.0, 0.0
    if t.size == 1:
        return True, float(t[0]), 0.0
    dt = (t[-1] - t[0]) / (t.size - 1)
    grid = t[0] + dt * np.arange(t.size)
    scale = max(np.abs(t).max(), 1e-300)
    ok = bool(np.all(np.abs(grid - t) <= rtol * scale)) and dt != 0.0
    return ok, float(t[0]), float(dt)


class StageTimer:
    """CUDA-event timer that msp_powder_run fills per stage (snapshots,
    schedule, phase sum, reduction), recorded on the launch stream."""

    def __init__(self):
        lib = _lib.load()
        h = ctypes.c_void_p(0)
        _lib.check(lib.msp_timer_create(ctypes.byref(h)), "msp_timer_create")
        self.handle = h

    def read(self):
        """Summed milliseconds per stage since the last read, and the run count."""
        ms = (ctypes.c_double * _lib.TIMER_STAGES)()
        runs = ctypes.c_int(0)
        _lib.check(_lib.load().msp_timer_read(self.handle, ms, ctypes.byref(runs)), "msp_timer_read")
        return dict(zip(_lib.TIMER_STAGE_NAMES, list(ms))), runs.value

    def close(self):
        if self.handle:
            _lib.load().msp_timer_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class PowderPlan:
    """Device-resident inputs, outputs and scratch of one msp_powder_run
    batch, reusable for repeated runs (benchmarks, fits).

    field, pol: (S, 3); wscale: (S,); slot: (S,) non-decreasing; times: 1-D.
    ``out`` has shape (num_slots,) for MODE_INTEGRAL, else
    (num_slots, len(times)).
    """

    def __init__(self, n, Hsys, Z, field, pol, wscale, slot, num_slots, times,
                 mode=_lib.MODE_FAST, precision=_lib.PREC_FP64, dims=None, mu_index=0,
                 gammas=None, temperature=None, rho_fac=None, tau=1.0, max_sweeps=0,
                 max_refine=0):
        d = device()
        a = _lib.PowderArgs()
        a.n = int(n)
        if dims is not None:
            a.num_spins = len(dims)
            for i, x in enumerate(dims):
                a.dims[i] = int(x)
        a.mu_index = int(mu_index)
        if gammas is not None:
            for i, g in enumerate(gammas):
                a.gammas[i] = float(g)
        self.Hs = dev(Hsys, torch.complex128)
        self.Zd = dev(Z, torch.complex128)
        self.F = dev(field, torch.float64).reshape(-1, 3)
        self.Pl = dev(pol, torch.float64).reshape(-1, 3)
        self.W = dev(wscale, torch.float64).reshape(-1)
        self.Sl = dev(slot, torch.int32).reshape(-1)
        S = self.F.shape[0]
        self.num_snap = S
        a.Hsys, a.Z = self.Hs.data_ptr(), self.Zd.data_ptr()
        a.num_snap = S
        a.field, a.pol = self.F.data_ptr(), self.Pl.data_ptr()
        a.wscale, a.slot = self.W.data_ptr(), self.Sl.data_ptr()
        self.R = None
        if rho_fac is not None:
            self.R = dev(rho_fac, torch.complex128)
            a.rho_fac = self.R.data_ptr()
        self.Tp = None
        if temperature is not None:
            tarr = np.broadcast_to(np.asarray(temperature, dtype=np.float64), (S,))
            self.Tp = dev(np.ascontiguousarray(tarr), torch.float64)
            a.temperature = self.Tp.data_ptr()
        a.num_slots = int(num_slots)
        self.T = None
        if mode == _lib.MODE_INTEGRAL:
            a.num_times = 1
            a.uniform = 1
            shape = (int(num_slots),)
        else:
            th = times.detach().cpu().numpy() if isinstance(times, torch.Tensor) else np.asarray(times)
            uni, t0, dt = uniform_grid(th)
            self.T = dev(times, torch.float64).reshape(-1)
            a.times = self.T.data_ptr()
            a.num_times = self.T.shape[0]
            a.uniform = 1 if uni else 0
            a.t0, a.dt = t0, dt
            shape = (int(num_slots), self.T.shape[0])
        a.tau = float(tau)
        a.mode = int(mode)
        a.precision = int(precision)
        a.max_sweeps = int(max_sweeps)
        a.max_refine = int(max_refine)
        self.out = torch.empty(shape, dtype=torch.float64, device=d)
        self.status = torch.zeros((max(S, 1),), dtype=torch.int32, device=d)
        a.out = self.out.data_ptr()
        a.status = self.status.data_ptr()
        nbytes = ctypes.c_size_t(0)
        _lib.check(_lib.load().msp_powder_workspace(ctypes.byref(a), ctypes.byref(nbytes)),
                   "msp_powder_workspace")
        self.ws = torch.empty(int(nbytes.value) + 256, dtype=torch.uint8, device=d)
        off = (-self.ws.data_ptr()) % 256
        a.workspace = self.ws.data_ptr() + off
        a.workspace_bytes = int(nbytes.value)
        self.workspace_bytes = int(nbytes.value)
        self.args = a

    def rebind(self, field, pol, wscale, slot):
        """Point the plan at new per-snapshot inputs of the same sizes (device
        tensors), keeping its output, status and workspace."""
        if all(isinstance(t, torch.Tensor) and t.is_cuda for t in (field, pol, wscale, slot)) and \
                (field.data_ptr(), pol.data_ptr(), wscale.data_ptr(), slot.data_ptr()) == \
                (self.F.data_ptr(), self.Pl.data_ptr(), self.W.data_ptr(), self.Sl.data_ptr()):
            return self  # the same buffers as last time
        F = dev(field, torch.float64).reshape(-1, 3)
        if F.shape[0] != self.num_snap:
            raise ValueError("rebind: the snapshot count changed")
        self.F, self.Pl = F, dev(pol, torch.float64).reshape(-1, 3)
        self.W, self.Sl = dev(wscale, torch.float64).reshape(-1), dev(slot, torch.int32).reshape(-1)
        a = self.args
        a.field, a.pol = self.F.data_ptr(), self.Pl.data_ptr()
        a.wscale, a.slot = self.W.data_ptr(), self.Sl.data_ptr()
        return self

    def fetch(self):
        """The output and the per-snapshot status on the host after one
        synchronisation: asynchronous copies into pinned staging buffers
        kept with the plan.  Returns two numpy arrays (copies)."""
        if getattr(self, "_host", None) is None:
            self._host = (torch.empty(tuple(self.out.shape), dtype=torch.float64, pin_memory=True),
                          torch.empty(tuple(self.status.shape), dtype=torch.int32,
                                      pin_memory=True))
        ho, hs = self._host
        ho.copy_(self.out, non_blocking=True)
        hs.copy_(self.status, non_blocking=True)
        torch.cuda.current_stream().synchronize()
        return ho.numpy().copy(), hs.numpy()[:self.num_snap].copy()

    def run(self, timer=None):
        """Enqueue the batch on the current stream; returns the output tensor."""
        self.args.stream = torch.cuda.current_stream().cuda_stream
        self.args.timer = timer.handle.value if timer is not None else None
        _lib.check(_lib.load().msp_powder_run(ctypes.byref(self.args)), "msp_powder_run")
        return self.out


def powder_run(n, Hsys, Z, field, pol, wscale, slot, num_slots, times, mode=_lib.MODE_FAST,
               precision=_lib.PREC_FP64, dims=None, mu_index=0, gammas=None, temperature=None,
               rho_fac=None, tau=1.0, max_sweeps=0, max_refine=0):
    """One msp_powder_run on fresh device buffers; returns (out, status)."""
    plan = PowderPlan(n, Hsys, Z, field, pol, wscale, slot, num_slots, times, mode, precision,
                      dims, mu_index, gammas, temperature, rho_fac, tau, max_sweeps, max_refine)
    out = plan.run()
    return out, plan.status[:plan.num_snap]


def adjoint_fast(n, Hsys, Z, field, pol, wscale, slot, num_slots, times, grad_out, max_sweeps=0,
                 want_field=True):
    """Gradient of L through the fast-path powder average (msp_adjoint_fast).

    ``grad_out``: dL/dP, shape (num_slots, len(times)) (or (len(times),) for
    one slot).  Returns (dL/dHsys (n, n) complex128, dL/dfield (S, 3) float64
    or None, status (S,) int32), gradients in PyTorch's complex convention
    dL = Re sum conj(G) dH."""
    d = device()
    a = _lib.AdjointArgs()
    a.n = int(n)
    Hs = dev(Hsys, torch.complex128)
    Zd = dev(Z, torch.complex128)
    F = dev(field, torch.float64).reshape(-1, 3)
    Pl = dev(pol, torch.float64).reshape(-1, 3)
    W = dev(wscale, torch.float64).reshape(-1)
    Sl = dev(slot, torch.int32).reshape(-1)
    S = F.shape[0]
    th = times.detach().cpu().numpy() if isinstance(times, torch.Tensor) else np.asarray(times)
    uni, t0, dt = uniform_grid(th)
    Td = dev(th, torch.float64).reshape(-1)
    g = dev(grad_out, torch.float64).reshape(int(num_slots), -1)
    if g.shape[1] != Td.shape[0]:
        raise ValueError("grad_out must have one row of len(times) values per slot")
    gH = torch.empty((a.n, a.n), dtype=torch.complex128, device=d)
    gF = torch.empty((S, 3), dtype=torch.float64, device=d) if want_field else None
    status = torch.zeros((max(S, 1),), dtype=torch.int32, device=d)
    a.Hsys, a.Z = Hs.data_ptr(), Zd.data_ptr()
    a.num_snap = S
    a.field, a.pol, a.wscale, a.slot = F.data_ptr(), Pl.data_ptr(), W.data_ptr(), Sl.data_ptr()
    a.num_slots = int(num_slots)
    a.times, a.num_times = Td.data_ptr(), Td.shape[0]
    a.uniform, a.t0, a.dt = 1 if uni else 0, t0, dt
    a.grad_out = g.data_ptr()
    a.grad_hsys = gH.data_ptr()
    a.grad_field = gF.data_ptr() if gF is not None else None
    a.status = status.data_ptr()
    a.max_sweeps = int(max_sweeps)
    nbytes = ctypes.c_size_t(0)
    lib = _lib.load()
    _lib.check(lib.msp_adjoint_workspace(ctypes.byref(a), ctypes.byref(nbytes)),
               "msp_adjoint_workspace")
    ws = torch.empty(int(nbytes.value) + 256, dtype=torch.uint8, device=d)
    a.workspace = ws.data_ptr() + ((-ws.data_ptr()) % 256)
    a.workspace_bytes = int(nbytes.value)
    a.stream = torch.cuda.current_stream().cuda_stream
    _lib.check(lib.msp_adjoint_fast(ctypes.byref(a)), "msp_adjoint_fast")
    return gH, gF, status[:S]


class MultiPlan:
    """A heterogeneous batch on the device (msp_multi_*): several spin
    systems of uneven Hilbert dimension, each with its own snapshots, reduced
    into one output row per system.

    Hsys_list, Z_list: per system (n_k, n_k) and (3, n_k, n_k) complex
    matrices; field, pol: (S, 3) lab-frame vectors of all snapshots, system
    by system; wscale: (S,); snap_first: (num_systems + 1,) prefix of the
    systems' snapshot counts; tuning: None or a list of dicts with keys n,
    snap_threads, ctas_per_sm, snaps_per_item.  ``out`` has shape
    (num_systems, len(times)).
    """

    def __init__(self, Hsys_list, Z_list, field, pol, wscale, snap_first, times,
                 precision=_lib.PREC_MIXED, tuning=None, max_pairs_per_chunk=0, max_sweeps=0):
        d = device()
        lib = _lib.load()
        ns = len(Hsys_list)
        if len(Z_list) != ns or len(snap_first) != ns + 1:
            raise ValueError("MultiPlan: one Hsys, one Z and one snapshot range per system")
        dims = np.array([np.shape(h)[-1] for h in Hsys_list], dtype=np.int32)
        first = np.ascontiguousarray(snap_first, dtype=np.int32)
        th = times.detach().cpu().numpy() if isinstance(times, torch.Tensor) else np.asarray(times)
        uni, t0, dt = uniform_grid(th)
        desc = _lib.MultiDesc()
        desc.num_systems = ns
        desc.sys_n = dims.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
        desc.sys_snap_first = first.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
        desc.num_times = int(th.size)
        desc.uniform = 1 if uni else 0
        desc.t0, desc.dt = t0, dt
        desc.precision = int(precision)
        desc.max_sweeps = int(max_sweeps)
        desc.max_pairs_per_chunk = int(max_pairs_per_chunk)
        self._tuning = None
        if tuning:
            arr = (_lib.MultiTuning * len(tuning))()
            for i, t in enumerate(tuning):
                arr[i].n = int(t["n"])
                arr[i].snap_threads = int(t.get("snap_threads", 0))
                arr[i].ctas_per_sm = int(t.get("ctas_per_sm", 0))
                arr[i].snaps_per_item = int(t.get("snaps_per_item", 0))
            self._tuning = arr
            desc.tuning = ctypes.cast(arr, ctypes.POINTER(_lib.MultiTuning))
            desc.num_tuning = len(tuning)
        h = ctypes.c_void_p(0)
        _lib.check(lib.msp_multi_plan_create(ctypes.byref(desc), ctypes.byref(h)),
                   "msp_multi_plan_create")
        self.handle = h
        self.dims = dims
        self.snap_first = first
        self.num_snap = int(first[-1])
        self.Hs = torch.cat([dev(hm, torch.complex128).reshape(-1) for hm in Hsys_list])
        self.Zd = torch.cat([dev(z, torch.complex128).reshape(-1) for z in Z_list])
        self.F = dev(field, torch.float64).reshape(-1, 3)
        self.Pl = dev(pol, torch.float64).reshape(-1, 3)
        self.W = dev(wscale, torch.float64).reshape(-1)
        if self.F.shape[0] != self.num_snap or self.Pl.shape[0] != self.num_snap or \
                self.W.shape[0] != self.num_snap:
            raise ValueError("MultiPlan: field, pol and wscale need one entry per snapshot")
        self.T = dev(th, torch.float64).reshape(-1)
        self.out = torch.empty((ns, int(th.size)), dtype=torch.float64, device=d)
        self.status = torch.zeros((max(self.num_snap, 1),), dtype=torch.int32, device=d)
        nbytes = ctypes.c_size_t(0)
        _lib.check(lib.msp_multi_workspace(h, ctypes.byref(nbytes)), "msp_multi_workspace")
        self.ws = torch.empty(int(nbytes.value) + 256, dtype=torch.uint8, device=d)
        io = _lib.MultiIO()
        io.Hsys_all, io.Z_all = self.Hs.data_ptr(), self.Zd.data_ptr()
        io.field, io.pol, io.wscale = self.F.data_ptr(), self.Pl.data_ptr(), self.W.data_ptr()
        io.times = self.T.data_ptr()
        io.out, io.status = self.out.data_ptr(), self.status.data_ptr()
        io.workspace = self.ws.data_ptr() + ((-self.ws.data_ptr()) % 256)
        io.workspace_bytes = int(nbytes.value)
        self.io = io
        self.workspace_bytes = int(nbytes.value)

    def info(self):
        """Buckets in launch order: list of dicts (n, num_systems, num_snap,
        num_chunks, snap_threads, grid, pairs_per_item, max_items,
        scratch_bytes)."""
        lib = _lib.load()
        nb = ctypes.c_int(0)
        _lib.check(lib.msp_multi_plan_info(self.handle, ctypes.byref(nb), None, 0),
                   "msp_multi_plan_info")
        arr = (_lib.MultiBucketInfo * max(nb.value, 1))()
        _lib.check(lib.msp_multi_plan_info(self.handle, ctypes.byref(nb), arr, nb.value),
                   "msp_multi_plan_info")
        return [{f: getattr(arr[i], f) for f, _ in _lib.MultiBucketInfo._fields_}
                for i in range(nb.value)]

    def run(self, graph=False):
        """Enqueue the batch on the current stream (through a CUDA graph when
        ``graph``); returns ``out``."""
        st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        name = "msp_multi_run_graph" if graph else "msp_multi_run"
        _lib.check(getattr(_lib.load(), name)(self.handle, ctypes.byref(self.io), st), name)
        return self.out

    def close(self):
        if getattr(self, "handle", None) and self.handle.value:
            _lib.load().msp_multi_plan_destroy(self.handle)
            self.handle = ctypes.c_void_p(0)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _superop_ws(n, num_ops):
    nbytes = ctypes.c_size_t(0)
    _lib.call("msp_superop_workspace", int(n), int(num_ops), ctypes.byref(nbytes))
    ws = torch.empty(int(nbytes.value) + 256, dtype=torch.uint8, device=device())
    return ws, ctypes.c_void_p(ws.data_ptr() + ((-ws.data_ptr()) % 256)), int(nbytes.value)


def superop_evolve(L, n, rho0, ops, times):
    """rho(t) = exp(2 pi L t) rho0 (msp_superop_evolve): (T, n_ops) complex
    expectations Tr(O rho(t)), or (T, n*n) vec(rho(t)) when ``ops`` is empty."""
    Ld = dev(L, torch.complex128)
    r = dev(rho0, torch.complex128)
    th = np.asarray(times, dtype=float)
    o = dev(ops, torch.complex128).reshape(-1, n, n) if len(ops) else None
    nops = 0 if o is None else int(o.shape[0])
    uni, t0, dt = uniform_grid(th)
    Td = dev(th, torch.float64)
    out = torch.empty((th.size, nops if nops else n * n), dtype=torch.complex128, device=Ld.device)
    ws, wp, nb = _superop_ws(n, nops)
    _lib.call("msp_superop_evolve", ptr(Ld), int(n), ptr(r), ptr(o), nops, ptr(Td), int(th.size),
              1 if uni else 0, t0, dt, ptr(out), wp, nb, stream())
    return out


def superop_integrate(L, n, rho0, ops, tau):
    """int_0^inf Tr(O rho(t)) e^{-t/tau} dt for each operator
    (msp_superop_integrate): (n_ops,) complex."""
    Ld = dev(L, torch.complex128)
    r = dev(rho0, torch.complex128)
    o = dev(ops, torch.complex128).reshape(-1, n, n)
    nops = int(o.shape[0])
    out = torch.empty((nops,), dtype=torch.complex128, device=Ld.device)
    ws, wp, nb = _superop_ws(n, nops)
    _lib.call("msp_superop_integrate", ptr(Ld), int(n), ptr(r), ptr(o), nops, float(tau),
              ptr(out), wp, nb, stream())
    return out


def lindblad_run(n, Hsys, Z, spin_ops, dims, mu_index, gammas, dissipation, field, pol, wscale,
                 slot, num_slots, times, temperature=None, mode=_lib.MODE_EVOLVE, tau=1.0,
                 precision=_lib.PREC_FP64):
    """A batch of dissipative snapshots reduced into output rows
    (msp_lindblad_run).  ``dissipation``: {spin index: rate}; ``spin_ops``:
    (num_spins, 3, n, n).  ``precision`` PREC_MIXED propagates in
    double-word FP32 where it applies (evolution on a uniform grid,
    n^2 <= 64).  Returns (out, status): out (num_slots, T) or (num_slots,)
    for MODE_INTEGRAL."""
    d = device()
    a = _lib.LindbladArgs()
    a.n, a.num_spins, a.mu_index = int(n), len(dims), int(mu_index)
    for i, x in enumerate(dims):
        a.dims[i] = int(x)
        a.gammas[i] = float(gammas[i])
    keep = [dev(Hsys, torch.complex128), dev(Z, torch.complex128), dev(spin_ops, torch.complex128)]
    a.Hsys, a.Z, a.spin_ops = (t.data_ptr() for t in keep)
    a.num_dissipative = len(dissipation)
    for k, (i, rate) in enumerate(sorted(dissipation.items())):
        a.dissipative_spin[k] = int(i)
        a.dissipative_rate[k] = float(rate)
    F = dev(field, torch.float64).reshape(-1, 3)
    S = int(F.shape[0])
    vecs = [F, dev(pol, torch.float64).reshape(-1, 3), dev(wscale, torch.float64).reshape(-1),
            dev(slot, torch.int32).reshape(-1)]
    keep += vecs
    a.num_snap = S
    a.field, a.pol, a.wscale, a.slot = (t.data_ptr() for t in vecs)
    if temperature is not None:
        Tp = dev(np.ascontiguousarray(np.broadcast_to(np.asarray(temperature, float), (S,))),
                 torch.float64)
        keep.append(Tp)
        a.temperature = Tp.data_ptr()
    a.num_slots = int(num_slots)
    if mode == _lib.MODE_INTEGRAL:
        a.num_times, a.uniform = 1, 1
        shape = (int(num_slots),)
    else:
        th = np.asarray(times, dtype=float)
        uni, t0, dt = uniform_grid(th)
        Td = dev(th, torch.float64)
        keep.append(Td)
        a.times, a.num_times, a.uniform, a.t0, a.dt = Td.data_ptr(), int(th.size), int(uni), t0, dt
        shape = (int(num_slots), int(th.size))
    a.tau, a.mode = float(tau), int(mode)
    a.precision = int(precision)
    out = torch.empty(shape, dtype=torch.float64, device=d)
    status = torch.zeros((max(S, 1),), dtype=torch.int32, device=d)
    a.out, a.status = out.data_ptr(), status.data_ptr()
    nbytes = ctypes.c_size_t(0)
    _lib.check(_lib.load().msp_lindblad_workspace(ctypes.byref(a), ctypes.byref(nbytes)),
               "msp_lindblad_workspace")
    ws = torch.empty(int(nbytes.value) + 256, dtype=torch.uint8, device=d)
    a.workspace = ws.data_ptr() + ((-ws.data_ptr()) % 256)
    a.workspace_bytes = int(nbytes.value)
    a.stream = torch.cuda.current_stream().cuda_stream
    _lib.check(_lib.load().msp_lindblad_run(ctypes.byref(a)), "msp_lindblad_run")
    out_status = (out, status[:S])
    del keep  # inputs may be freed once the stream has consumed them (caching allocator)
    return out_status


def celio_run(mode, digit_dims, factor_digits, factor_mat, mats, mats_per_snapshot,
              num_snapshots, states_per_snapshot, trotter_k, num_times, mu_psi=None, sigma=None,
              phases=None, seed=0, rho0=None, meas=None, meas_per_snapshot=False,
              wscale=None, row_start=None, num_rows=0, path=0, precision=_lib.PREC_FP64):
    """Celio's method through ``msp_celio_run`` (FP64, or double-word FP32
    with ``precision`` = PREC_MIXED).

    ``digit_dims``: multiplicity of each digit of a state (spins for
    CELIO_PURE, row then column spins for CELIO_DENSITY);
    ``factor_digits``: [(d0, d1 or -1)] per factor application of one
    Trotter pass; ``factor_mat``: each factor's matrix offset (complex
    entries) in a snapshot's block of ``mats`` ((S or 1, mats_len) complex).
    Returns (series, rows): series (S, A, T) float64 for PURE or (S, T,
    num_ops) complex128 for DENSITY; rows (num_rows, T) when ``row_start``
    is given, else None."""
    d = device()
    digit_dims = np.ascontiguousarray(digit_dims, dtype=np.int32)
    fd = np.ascontiguousarray(np.asarray(factor_digits, dtype=np.int32).reshape(-1, 2))
    fm = np.ascontiguousarray(np.asarray(factor_mat, dtype=np.int64).reshape(-1))
    nf = fd.shape[0]
    mats_d = dev(mats, torch.complex128) if nf > 0 else None
    mats_len = int(mats_d.shape[-1]) if mats_d is not None else 0
    S, A, T = int(num_snapshots), int(states_per_snapshot), int(num_times)
    a = _lib.CelioArgs()
    a.mode = int(mode)
    a.num_digits = len(digit_dims)
    a.digit_dims = digit_dims.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
    a.num_factors = nf
    a.factor_digits = fd.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
    a.factor_mat = fm.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong))
    a.mats = ptr(mats_d)
    a.mats_len = mats_len
    a.mats_per_snapshot = int(bool(mats_per_snapshot))
    a.num_snapshots = S
    a.states_per_snapshot = A
    a.trotter_k = int(trotter_k)
    a.num_times = T
    keep = []
    if mode == _lib.CELIO_PURE:
        mu = dev(mu_psi, torch.complex128)
        sg = dev(sigma, torch.complex128)
        keep += [mu, sg]
        a.mu_psi, a.sigma = ptr(mu), ptr(sg)
        if phases is not None:
            ph = dev(phases, torch.float64)
            keep.append(ph)
            a.phases = ptr(ph)
        a.seed = int(seed) & 0xFFFFFFFFFFFFFFFF
        series = torch.empty((S, A, T), dtype=torch.float64, device=d)
    else:
        r0 = dev(rho0, torch.complex128)
        ms = dev(meas, torch.complex128)
        keep += [r0, ms]
        a.rho0, a.meas = ptr(r0), ptr(ms)
        a.num_ops = int(ms.shape[-3]) if ms.dim() >= 3 else 1
        a.meas_per_snapshot = int(bool(meas_per_snapshot))
        series = torch.empty((S, T, a.num_ops), dtype=torch.complex128, device=d)
    a.series = ptr(series)
    rows = None
    if row_start is not None:
        rs = dev(row_start, torch.int32)
        keep.append(rs)
        rows = torch.empty((int(num_rows), T), dtype=torch.float64, device=d)
        a.row_start, a.num_rows, a.rows_out = ptr(rs), int(num_rows), ptr(rows)
        if wscale is not None:
            ws_ = dev(wscale, torch.float64)
            keep.append(ws_)
            a.wscale = ptr(ws_)
    a.path = int(path)
    a.precision = int(precision)
    nbytes = ctypes.c_size_t(0)
    _lib.call("msp_celio_workspace", ctypes.byref(a), ctypes.byref(nbytes))
    ws = torch.empty(int(nbytes.value) + 256, dtype=torch.uint8, device=d)
    base = ws.data_ptr()
    aligned = (base + 255) & ~255
    _lib.call("msp_celio_run", ctypes.byref(a), ctypes.c_void_p(aligned),
              ctypes.c_size_t(int(nbytes.value)), stream())
    return series, rows


def celio_expm(dims, H0, G, fields, tau, out_offsets, mats):
    """Field-dependent Trotter factors in place: for every snapshot s and
    factor f, exp(-2 pi i tau (H0_f + sum_a B[s, a] G_f[a])) written into
    ``mats[s]`` (complex (S, mats_len), device) at out_offsets[f] (U,
    U^dagger, U^T; -1 skips).  ``H0``: list of (D, D), ``G``: list of
    (3, D, D) complex arrays."""
    dims = np.ascontiguousarray(dims, dtype=np.int32)
    h = np.concatenate([np.asarray(m, dtype=complex).reshape(-1) for m in H0])
    g = np.concatenate([np.asarray(m, dtype=complex).reshape(-1) for m in G])
    hd, gd = dev(h, torch.complex128), dev(g, torch.complex128)
    B = dev(np.asarray(fields, dtype=float).reshape(-1, 3), torch.float64)
    oo = np.ascontiguousarray(np.asarray(out_offsets, dtype=np.int64).reshape(-1, 3))
    _lib.call("msp_celio_expm", int(B.shape[0]), len(dims),
              dims.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), ptr(hd), ptr(gd), ptr(B),
              float(tau), oo.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong)), ptr(mats),
              int(mats.shape[-1]), stream())
    return mats
