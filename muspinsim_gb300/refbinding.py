"""The binding a maintainer of the reference adds to run its native cosine
sum on the GPU.

The reference's ``Hamiltonian.fast_evolve`` (muspinsim/hamiltonian.py:166-217)
calls ``parallel_fast_time_evolve(times, other_dimension, A, W)`` from its
Cython extension (muspinsim/cython/parallel.pyx:16-69, imported at
muspinsim/hamiltonian.py:10).  This module is a drop-in for that one
function: same arguments (float64 arrays, C order), same float64 result of
shape (len(times),), computed by ``msp_fast_cos_sum`` with the Cython
kernel's summation order.  Copied into the reference as ``muspinsim/gpu.py``,
the import at muspinsim/hamiltonian.py:10 becomes
``from muspinsim.gpu import parallel_fast_time_evolve``.
"""

import ctypes

import numpy as np
import torch

from muspinsim_gb300 import _lib

_vp = ctypes.c_void_p


def parallel_fast_time_evolve(times, other_dimension, A, W):
    """sum_{j > k} A_jk cos(W_jk t) + sum_j A_jj / 2, divided by
    other_dimension (the reference kernel's result, before fast_evolve's
    factor 0.5), for every t in times."""
    lib = _lib.load()
    t = torch.as_tensor(np.ascontiguousarray(times, dtype=np.float64), device="cuda")
    a = torch.as_tensor(np.ascontiguousarray(A, dtype=np.float64), device="cuda")
    w = torch.as_tensor(np.ascontiguousarray(W, dtype=np.float64), device="cuda")
    if a.ndim != 2 or a.shape[0] != a.shape[1] or w.shape != a.shape:
        raise ValueError("A and W must be square matrices of the same shape")
    out = torch.empty_like(t)
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.msp_fast_cos_sum(_vp(t.data_ptr()), t.numel(), int(other_dimension),
                              _vp(a.data_ptr()), _vp(w.data_ptr()), a.shape[0],
                              _vp(out.data_ptr()), _vp(stream))
    if rc != 0:
        raise RuntimeError(f"msp_fast_cos_sum failed: {_lib.last_error()}")
    return out.cpu().numpy()
