"""Gradient-based FittingRunner against the reference's own FittingRunner
(tests/golden/fit_fmuf.npz, made by running muspinsim/fitting.py:15-179 on
the F-mu-F problem): the objective at the start point, the analytic
gradient against the reference objective's central differences, and the
L-BFGS-B and Nelder-Mead fits."""

import os

import numpy as np
import pytest

from tests.helpers import GOLDEN

pytestmark = pytest.mark.gpu

FIT_TIMES = np.linspace(0.0, 10.0, 150)


def fit_params(r1, r2):
    """The F-mu-F problem of tests/golden/make_golden.py:fit_params, built
    with the package's make_params."""
    from muspinsim_gb300 import workloads
    from muspinsim_gb300.simconfig import make_params

    wl = workloads.config5(n_orient=12, n_times=150)
    (k1, a1, v1), (k2, a2, v2), third = wl.couplings
    u1, u2 = np.asarray(v1) / np.linalg.norm(v1), np.asarray(v2) / np.linalg.norm(v2)
    coup = [(k1, a1, u1 * r1), (k2, a2, u2 * r2), third]
    return make_params(spins=wl.spins, couplings=coup, time=FIT_TIMES,
                       orientation=wl.orientations, field=[wl.fields[0]],
                       polarization=[wl.polarization])


@pytest.fixture(scope="module")
def golden():
    return np.load(os.path.join(GOLDEN, "fit_fmuf.npz"))


def _runner(golden, method, gradient=True):
    from muspinsim_gb300.fitting import FitInput, FittingRunner, FittingVariable

    inp = FitInput(fit_params, [FittingVariable("r1", 1.10, 0.8, 2.0),
                                FittingVariable("r2", 1.32, 0.8, 2.0)],
                   golden["data"], method=method, rtol=1e-8)
    return FittingRunner(inp, gradient=gradient)


def test_objective_and_gradient_at_start(golden):
    fr = _runner(golden, "lbfgs")
    x0 = golden["x0"]
    assert fr._adjoint_applies()
    f, g = fr._targfun_with_gradient(x0)
    assert abs(f - float(golden["f0"])) <= 1e-10
    assert fr.adjoint_evaluations == 1
    # the reference objective's central differences (h = 1e-6)
    assert np.abs(g - golden["g0"]).max() <= 1e-5 * max(1.0, np.abs(golden["g0"]).max())


def test_lbfgs_fit_with_adjoint_gradients(golden):
    fr = _runner(golden, "lbfgs")
    sol = fr.run()
    assert sol.success
    f_ref = float(golden["f_lbfgs"])
    assert sol.fun <= f_ref * (1 + 1e-4)
    assert np.abs(sol.x - golden["x_lbfgs"]).max() <= 2e-3
    # one forward simulation and one adjoint per objective evaluation,
    # against the reference's 1 + n_variables simulations
    assert fr.simulations < int(golden["nfev_lbfgs"])
    res = fr.runner.config.results
    assert res.shape == (len(FIT_TIMES),)


def test_nelder_mead_fit_matches_reference(golden):
    fr = _runner(golden, "nelder-mead")
    sol = fr.run()
    assert abs(sol.fun - float(golden["f_nm"])) <= 1e-6
    assert np.abs(sol.x - golden["x_nm"]).max() <= 1e-3
