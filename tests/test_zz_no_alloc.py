"""msp_powder_run_static: the powder pipeline for callers that cannot
allocate device memory.

Such a caller -- for example a host whose GPU memory is managed by another
runtime, or a loop that must not let a cudaMalloc synchronise the device --
passes only inputs and outputs; the scratch comes from an array built into
the library.  This test drives the entry point through the C ABI and checks
that two calls in a row give the same results as msp_powder_run with a
caller-provided workspace (FP64 within 1e-10, mixed within 1e-6), and that a
batch larger than the built-in scratch is refused with a clear message.  It
sits in a file collected last, and passes alone in a fresh process as well.
"""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _plan(precision, n_orient=48, n_times=512):
    from muspinsim_gb300 import _lib, kernels, workloads
    from muspinsim_gb300 import quaternion as Q
    from muspinsim_gb300.orientations import orientation_rows_to_quats

    wl = workloads.config2(n_orient=n_orient, n_times=n_times)
    sy = wl.system()
    qs, ws = orientation_rows_to_quats(wl.orientations)
    N = len(qs)
    B = Q.rotate(qs, wl.fields[0])
    p = Q.rotate(qs, wl.polarization / np.linalg.norm(wl.polarization))
    return kernels.PowderPlan(sy.hamiltonian_matrix().shape[0], sy.hamiltonian_matrix(),
                              sy.zeeman_operators(), B, p, ws / N, np.zeros(N, np.int32), 1,
                              wl.times, mode=_lib.MODE_FAST, precision=precision,
                              dims=list(sy.dimension), mu_index=sy.muon_index,
                              gammas=sy.gammas)


def _static_args(plan, out):
    import torch

    from muspinsim_gb300 import _lib

    a = _lib.PowderArgs()
    ctypes.memmove(ctypes.byref(a), ctypes.byref(plan.args), ctypes.sizeof(_lib.PowderArgs))
    a.out = out.data_ptr()
    a.workspace = None  # ignored by the static entry point
    a.workspace_bytes = 0
    a.timer = None
    a.stream = torch.cuda.current_stream().cuda_stream
    return a


@pytest.mark.parametrize("precision,tol", [(0, 1e-10), (1, 1e-6)])
def test_static_scratch_matches_caller_workspace(precision, tol):
    import torch

    from muspinsim_gb300 import _lib

    lib = _lib.load()
    plan = _plan(precision)
    ref = plan.run().clone()
    torch.cuda.synchronize()
    for _ in range(2):  # two calls in a row share (and reuse) the scratch
        out = torch.full_like(ref, float("nan"))
        a = _static_args(plan, out)
        rc = lib.msp_powder_run_static(ctypes.byref(a))
        assert rc == _lib.MSP_OK, _lib.last_error()
        torch.cuda.synchronize()
        assert int(plan.status[: plan.num_snap].max().item()) == 0
        assert float((out - ref).abs().max().item()) <= tol


def test_static_scratch_refuses_oversized_batch():
    import torch

    from muspinsim_gb300 import _lib

    lib = _lib.load()
    plan = _plan(0, n_orient=4000, n_times=4096)  # scratch need well above the limit
    out = torch.empty_like(plan.out)
    a = _static_args(plan, out)
    rc = lib.msp_powder_run_static(ctypes.byref(a))
    assert rc == _lib.MSP_ERR_WORKSPACE
    msg = _lib.last_error()
    assert "scratch" in msg and str(_lib.STATIC_SCRATCH_BYTES) in msg
