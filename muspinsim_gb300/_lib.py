"""ctypes binding of ``libmspgpu.so`` (the C ABI in ``include/mspgpu.h``).

The library is the only compute path: if it cannot be loaded, or no CUDA
device is present, every call raises ``RuntimeError`` -- there is no CPU
fallback.  Device buffers are torch CUDA tensors; their data pointers are
handed to the C functions together with the current CUDA stream.
"""

import ctypes
import os
import threading

from muspinsim_gb300 import build as _build

MSP_OK = 0
MSP_ERR_ARG = 1
MSP_ERR_CUDA = 2
MSP_ERR_WORKSPACE = 3
MSP_ERR_UNSUPPORTED = 4

MSP_ITEM_OK = 0
MSP_ITEM_NOT_CONVERGED = 1
MSP_ITEM_BAD_SLOT = 2
MSP_ITEM_REFINE_LIMIT = 4

GRID_ZCW_SPHERE = 0
GRID_ZCW_HEMISPHERE = 1
GRID_EULRANGE = 2

PREC_FP64 = 0
PREC_MIXED = 1

MODE_FAST = 0
MODE_EVOLVE = 1
MODE_INTEGRAL = 2

MAX_DIM = 64
MAX_DIM_LARGE = 1024  # MSP_MAX_DIM_LARGE: Householder + QL path (FP64)
STATIC_SCRATCH_BYTES = 32 << 20  # MSP_STATIC_SCRATCH_BYTES
MAX_SPINS = 16

_c_dp = ctypes.c_void_p  # device pointers travel as void*


class PowderArgs(ctypes.Structure):
    """Mirror of ``msp_powder_args`` (include/mspgpu.h)."""

    _fields_ = [
        ("n", ctypes.c_int),
        ("num_spins", ctypes.c_int),
        ("mu_index", ctypes.c_int),
        ("dims", ctypes.c_int * MAX_SPINS),
        ("Hsys", _c_dp),
        ("Z", _c_dp),
        ("num_snap", ctypes.c_int),
        ("field", _c_dp),
        ("pol", _c_dp),
        ("wscale", _c_dp),
        ("slot", _c_dp),
        ("temperature", _c_dp),
        ("gammas", ctypes.c_double * MAX_SPINS),
        ("rho_fac", _c_dp),
        ("num_slots", ctypes.c_int),
        ("times", _c_dp),
        ("num_times", ctypes.c_int),
        ("uniform", ctypes.c_int),
        ("t0", ctypes.c_double),
        ("dt", ctypes.c_double),
        ("tau", ctypes.c_double),
        ("mode", ctypes.c_int),
        ("precision", ctypes.c_int),
        ("max_sweeps", ctypes.c_int),
        ("out", _c_dp),
        ("status", _c_dp),
        ("workspace", _c_dp),
        ("workspace_bytes", ctypes.c_size_t),
        ("stream", _c_dp),
        ("timer", _c_dp),
        ("max_refine", ctypes.c_int),
    ]


class AdjointArgs(ctypes.Structure):
    """Mirror of ``msp_adjoint_args`` (include/mspgpu.h)."""

    _fields_ = [
        ("n", ctypes.c_int),
        ("Hsys", _c_dp),
        ("Z", _c_dp),
        ("num_snap", ctypes.c_int),
        ("field", _c_dp),
        ("pol", _c_dp),
        ("wscale", _c_dp),
        ("slot", _c_dp),
        ("num_slots", ctypes.c_int),
        ("times", _c_dp),
        ("num_times", ctypes.c_int),
        ("uniform", ctypes.c_int),
        ("t0", ctypes.c_double),
        ("dt", ctypes.c_double),
        ("grad_out", _c_dp),
        ("grad_hsys", _c_dp),
        ("grad_field", _c_dp),
        ("status", _c_dp),
        ("max_sweeps", ctypes.c_int),
        ("workspace", _c_dp),
        ("workspace_bytes", ctypes.c_size_t),
        ("stream", _c_dp),
    ]


class MultiTuning(ctypes.Structure):
    """Mirror of ``msp_multi_tuning``."""

    _fields_ = [
        ("n", ctypes.c_int),
        ("snap_threads", ctypes.c_int),
        ("ctas_per_sm", ctypes.c_int),
        ("snaps_per_item", ctypes.c_int),
    ]


class MultiDesc(ctypes.Structure):
    """Mirror of ``msp_multi_desc`` (host pointers)."""

    _fields_ = [
        ("num_systems", ctypes.c_int),
        ("sys_n", ctypes.POINTER(ctypes.c_int)),
        ("sys_snap_first", ctypes.POINTER(ctypes.c_int)),
        ("num_times", ctypes.c_int),
        ("uniform", ctypes.c_int),
        ("t0", ctypes.c_double),
        ("dt", ctypes.c_double),
        ("precision", ctypes.c_int),
        ("max_sweeps", ctypes.c_int),
        ("max_pairs_per_chunk", ctypes.c_longlong),
        ("tuning", ctypes.POINTER(MultiTuning)),
        ("num_tuning", ctypes.c_int),
    ]


class MultiIO(ctypes.Structure):
    """Mirror of ``msp_multi_io`` (device pointers)."""

    _fields_ = [
        ("Hsys_all", _c_dp),
        ("Z_all", _c_dp),
        ("field", _c_dp),
        ("pol", _c_dp),
        ("wscale", _c_dp),
        ("times", _c_dp),
        ("out", _c_dp),
        ("status", _c_dp),
        ("workspace", _c_dp),
        ("workspace_bytes", ctypes.c_size_t),
    ]


class MultiBucketInfo(ctypes.Structure):
    """Mirror of ``msp_multi_bucket_info``."""

    _fields_ = [
        ("n", ctypes.c_int),
        ("num_systems", ctypes.c_int),
        ("num_snap", ctypes.c_longlong),
        ("num_chunks", ctypes.c_int),
        ("snap_threads", ctypes.c_int),
        ("grid", ctypes.c_int),
        ("pairs_per_item", ctypes.c_int),
        ("max_items", ctypes.c_int),
        ("scratch_bytes", ctypes.c_size_t),
    ]


class LindbladArgs(ctypes.Structure):
    """Mirror of ``msp_lindblad_args``."""

    _fields_ = [
        ("n", ctypes.c_int),
        ("num_spins", ctypes.c_int),
        ("mu_index", ctypes.c_int),
        ("dims", ctypes.c_int * MAX_SPINS),
        ("gammas", ctypes.c_double * MAX_SPINS),
        ("Hsys", _c_dp),
        ("Z", _c_dp),
        ("spin_ops", _c_dp),
        ("num_dissipative", ctypes.c_int),
        ("dissipative_spin", ctypes.c_int * MAX_SPINS),
        ("dissipative_rate", ctypes.c_double * MAX_SPINS),
        ("num_snap", ctypes.c_int),
        ("field", _c_dp),
        ("pol", _c_dp),
        ("wscale", _c_dp),
        ("slot", _c_dp),
        ("temperature", _c_dp),
        ("num_slots", ctypes.c_int),
        ("times", _c_dp),
        ("num_times", ctypes.c_int),
        ("uniform", ctypes.c_int),
        ("t0", ctypes.c_double),
        ("dt", ctypes.c_double),
        ("tau", ctypes.c_double),
        ("mode", ctypes.c_int),
        ("out", _c_dp),
        ("status", _c_dp),
        ("workspace", _c_dp),
        ("workspace_bytes", ctypes.c_size_t),
        ("stream", _c_dp),
        ("precision", ctypes.c_int),
    ]


CELIO_PURE = 0
CELIO_DENSITY = 1


class CelioArgs(ctypes.Structure):
    """Mirror of ``msp_celio_args``."""

    _fields_ = [
        ("mode", ctypes.c_int),
        ("num_digits", ctypes.c_int),
        ("digit_dims", ctypes.POINTER(ctypes.c_int)),
        ("num_factors", ctypes.c_int),
        ("factor_digits", ctypes.POINTER(ctypes.c_int)),
        ("factor_mat", ctypes.POINTER(ctypes.c_longlong)),
        ("mats", _c_dp),
        ("mats_len", ctypes.c_longlong),
        ("mats_per_snapshot", ctypes.c_int),
        ("num_snapshots", ctypes.c_int),
        ("states_per_snapshot", ctypes.c_int),
        ("trotter_k", ctypes.c_int),
        ("num_times", ctypes.c_int),
        ("mu_psi", _c_dp),
        ("sigma", _c_dp),
        ("phases", _c_dp),
        ("seed", ctypes.c_ulonglong),
        ("rho0", _c_dp),
        ("meas", _c_dp),
        ("num_ops", ctypes.c_int),
        ("meas_per_snapshot", ctypes.c_int),
        ("series", _c_dp),
        ("wscale", _c_dp),
        ("row_start", _c_dp),
        ("num_rows", ctypes.c_int),
        ("rows_out", _c_dp),
        ("path", ctypes.c_int),
        ("precision", ctypes.c_int),
    ]


TIMER_STAGES = 5
TIMER_STAGE_NAMES = ("eigensolve", "snapshots", "schedule", "phase", "reduce")


# name -> (restype, argtypes)
_SIGNATURES = {
    "msp_version": (ctypes.c_int, []),
    "msp_last_error": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_size_t]),
    "msp_assemble": (ctypes.c_int, [_c_dp, _c_dp, _c_dp, ctypes.c_int, ctypes.c_int, _c_dp, _c_dp]),
    "msp_assemble_rotated": (
        ctypes.c_int,
        [_c_dp, ctypes.c_int, _c_dp, ctypes.c_int, _c_dp, ctypes.c_int, _c_dp, ctypes.c_int, _c_dp,
         _c_dp]),
    "msp_eigh_batched": (
        ctypes.c_int,
        [_c_dp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, _c_dp, _c_dp, _c_dp, _c_dp],
    ),
    "msp_eigh_workspace": (
        ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_size_t)]),
    "msp_eigh_batched_ws": (
        ctypes.c_int,
        [_c_dp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, _c_dp, _c_dp, _c_dp, _c_dp,
         ctypes.c_size_t, _c_dp],
    ),
    "msp_basis_change": (
        ctypes.c_int,
        [_c_dp, ctypes.c_longlong, _c_dp, ctypes.c_longlong, ctypes.c_int, ctypes.c_int,
         ctypes.c_int, _c_dp, _c_dp],
    ),
    "msp_orient_grid_snapshots": (
        ctypes.c_int,
        [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, _c_dp, ctypes.c_int, _c_dp,
         _c_dp, ctypes.c_double, _c_dp, _c_dp, _c_dp, _c_dp, _c_dp],
    ),
    "msp_fast_cos_sum": (
        ctypes.c_int,
        [_c_dp, ctypes.c_int, ctypes.c_int, _c_dp, _c_dp, ctypes.c_int, _c_dp, _c_dp],
    ),
    "msp_fast_amplitudes": (
        ctypes.c_int,
        [_c_dp, _c_dp, _c_dp, ctypes.c_int, ctypes.c_int, _c_dp, _c_dp, _c_dp],
    ),
    "msp_evolve_expect": (
        ctypes.c_int,
        [_c_dp, _c_dp, _c_dp, ctypes.c_int, ctypes.c_int, _c_dp, ctypes.c_int, _c_dp, _c_dp],
    ),
    "msp_evolve_phases": (
        ctypes.c_int,
        [_c_dp, _c_dp, ctypes.c_int, _c_dp, ctypes.c_int, _c_dp, _c_dp],
    ),
    "msp_integrate_decaying": (
        ctypes.c_int,
        [_c_dp, _c_dp, _c_dp, ctypes.c_int, ctypes.c_int, ctypes.c_double, _c_dp, _c_dp],
    ),
    "msp_powder_workspace": (
        ctypes.c_int,
        [ctypes.POINTER(PowderArgs), ctypes.POINTER(ctypes.c_size_t)],
    ),
    "msp_powder_run": (ctypes.c_int, [ctypes.POINTER(PowderArgs)]),
    "msp_powder_run_static": (ctypes.c_int, [ctypes.POINTER(PowderArgs)]),
    "msp_adjoint_workspace": (
        ctypes.c_int,
        [ctypes.POINTER(AdjointArgs), ctypes.POINTER(ctypes.c_size_t)],
    ),
    "msp_adjoint_fast": (ctypes.c_int, [ctypes.POINTER(AdjointArgs)]),
    "msp_multi_plan_create": (
        ctypes.c_int, [ctypes.POINTER(MultiDesc), ctypes.POINTER(ctypes.c_void_p)]),
    "msp_multi_plan_destroy": (ctypes.c_int, [_c_dp]),
    "msp_multi_workspace": (ctypes.c_int, [_c_dp, ctypes.POINTER(ctypes.c_size_t)]),
    "msp_multi_plan_info": (
        ctypes.c_int,
        [_c_dp, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(MultiBucketInfo), ctypes.c_int]),
    "msp_multi_run": (ctypes.c_int, [_c_dp, ctypes.POINTER(MultiIO), _c_dp]),
    "msp_multi_run_graph": (ctypes.c_int, [_c_dp, ctypes.POINTER(MultiIO), _c_dp]),
    "msp_orient_snapshots": (
        ctypes.c_int,
        [_c_dp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_double),
         ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double), ctypes.c_double,
         _c_dp, _c_dp, _c_dp, _c_dp]),
    "msp_superop_workspace": (
        ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_size_t)]),
    "msp_superop_evolve": (
        ctypes.c_int,
        [_c_dp, ctypes.c_int, _c_dp, _c_dp, ctypes.c_int, _c_dp, ctypes.c_int, ctypes.c_int,
         ctypes.c_double, ctypes.c_double, _c_dp, _c_dp, ctypes.c_size_t, _c_dp]),
    "msp_superop_integrate": (
        ctypes.c_int,
        [_c_dp, ctypes.c_int, _c_dp, _c_dp, ctypes.c_int, ctypes.c_double, _c_dp, _c_dp,
         ctypes.c_size_t, _c_dp]),
    "msp_lindblad_workspace": (
        ctypes.c_int, [ctypes.POINTER(LindbladArgs), ctypes.POINTER(ctypes.c_size_t)]),
    "msp_lindblad_run": (ctypes.c_int, [ctypes.POINTER(LindbladArgs)]),
    "msp_celio_workspace": (
        ctypes.c_int, [ctypes.POINTER(CelioArgs), ctypes.POINTER(ctypes.c_size_t)]),
    "msp_celio_run": (
        ctypes.c_int, [ctypes.POINTER(CelioArgs), _c_dp, ctypes.c_size_t, _c_dp]),
    "msp_celio_expm": (
        ctypes.c_int,
        [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int), _c_dp, _c_dp, _c_dp,
         ctypes.c_double, ctypes.POINTER(ctypes.c_longlong), _c_dp, ctypes.c_longlong, _c_dp]),
    "msp_timer_create": (ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p)]),
    "msp_timer_destroy": (ctypes.c_int, [_c_dp]),
    "msp_timer_read": (
        ctypes.c_int,
        [_c_dp, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int)],
    ),
}

EXPORTED = tuple(_SIGNATURES)

_lib = None
_lock = threading.Lock()


def library_path():
    return _build.lib_path()


def load(build_if_missing=True):
    """Load (building first if needed) and return the ctypes library."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = library_path()
        if not os.path.exists(path):
            if not build_if_missing:
                raise RuntimeError(f"libmspgpu not built ({path}); run muspinsim_gb300.build")
            path = _build.build()
        lib = ctypes.CDLL(path)
        for name, (res, args) in _SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def last_error():
    buf = ctypes.create_string_buffer(512)
    load().msp_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(rc, what):
    """Turn an msp status code into an exception."""
    if rc == MSP_OK:
        return
    msg = f"{what}: {last_error()}"
    if rc == MSP_ERR_ARG:
        raise ValueError(msg)
    raise RuntimeError(msg)


def call(name, *args):
    rc = getattr(load(), name)(*args)
    check(rc, name)
    return rc
