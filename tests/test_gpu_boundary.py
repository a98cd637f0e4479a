"""The GPU side of the drop-in boundary against fixtures made by running the
reference itself (tests/golden/make_golden.py):

* msp_assemble_rotated against SpinSystem.rotate(R).hamiltonian
  (muspinsim/spinsys.py:103-135, 594-626);
* the reference-side binding (muspinsim_gb300.refbinding, the stub a
  maintainer adds at muspinsim/hamiltonian.py:10) fed with the exact
  arguments the reference's Hamiltonian.fast_evolve passed to its Cython
  kernel, against that kernel's output and fast_evolve's result
  (muspinsim/hamiltonian.py:195-217, muspinsim/cython/parallel.pyx:16-69).
"""

import os

import numpy as np
import pytest

from tests.helpers import GOLDEN

pytestmark = pytest.mark.gpu


def test_assemble_rotated_matches_reference():
    from muspinsim_gb300 import kernels, workloads

    z = np.load(os.path.join(GOLDEN, "rotated_dim24.npz"))
    sy = workloads.config2(n_orient=1, n_times=8).system()
    H = kernels.assemble_rotated(sy, z["R"]).cpu().numpy()
    scale = np.abs(z["H"]).max()
    assert np.abs(H - z["HR"]).max() <= 1e-12 * scale


def test_reference_binding_fast_evolve():
    from muspinsim_gb300.refbinding import parallel_fast_time_evolve

    z = np.load(os.path.join(GOLDEN, "fast_binding_dim24.npz"))
    got = parallel_fast_time_evolve(z["times"], int(z["d"]), z["A"], z["W"])
    assert got.shape == z["kernel"].shape and got.dtype == np.float64
    assert np.abs(got - z["kernel"]).max() <= 1e-13
    # fast_evolve returns the kernel's result times 0.5
    assert np.abs(0.5 * got - z["fast"]).max() <= 1e-13
