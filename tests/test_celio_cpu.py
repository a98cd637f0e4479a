"""Celio's method on the CPU: the oracle pinned to the reference, and the
host logic of the GPU path.

* the oracle (oracle/port.py, numpy, and oracle/celio.c, the C restatement
  of the reference's native module) reproduces the golden fixtures made by
  running the reference's ExperimentRunner with Celio's method
  (tests/golden/make_golden.py, save_celio) to 1e-10;
* the known answers of muspinsim/tests/test_celio.py (contributions,
  Trotter factors) hold for the host mirror (muspinsim_gb300/celio.py);
* argument errors are raised with the reference's exception types before
  any device is touched.
"""

import ctypes

import numpy as np
import pytest

from oracle import port
from tests.helpers import celio_phases, golden_oracle, load_golden, oracle_system

TOL = 1e-10


@pytest.mark.parametrize("name", ["celio_fast_muVV", "celio_fast_field", "celio_rho_T",
                                  "celio_rho_desc"])
def test_oracle_matches_reference_goldens(name):
    g = load_golden(name)
    got = golden_oracle(g)
    assert got.shape == g["result"].shape
    assert np.abs(got - g["result"]).max() <= TOL


def test_c_restatement_matches_numpy_oracle():
    """oracle/celio.c against the numpy restatement: mu + V (I = 7/2) + N
    (I = 1), a descending-index dipolar term between spins of different
    dimension, quadrupoles and a field."""
    rng = np.random.default_rng(3)
    q = rng.normal(size=(3, 3)) * 0.05
    q = q + q.T
    coup = [("dipolar", {"i": 1, "j": 2}, [0.2, 1.1, 0.7]),
            ("dipolar", {"i": 3, "j": 1}, [1.0, 0.3, 0.4]),
            ("quadrupolar", {"i": 2}, q), ("quadrupolar", {"i": 3}, q * 2)]
    sy = oracle_system(["mu", "V", "N"], coup)
    t = np.linspace(0, 3.0, 20)
    fac = port.celio_snapshot_factors(sy, [0.001, 0.0, 0.003], t[1] - t[0], 4)
    ph = celio_phases(11, 1, 3, sy.n // 2)[0]
    sig = port.sigma_mu([0.3, 0.5, 0.81])
    a = port.celio_fast_evolve(fac, list(sy.dims), sig, t, 4, ph)
    b = port.celio_fast_evolve_c(fac, list(sy.dims), sig, t, 4, ph, nthreads=2)
    assert np.abs(a - b).max() <= 1e-12
    assert abs(a[0] - 0.5 * np.linalg.norm([0.3, 0.5, 0.81])) <= 1e-12


def _ref_test_system():
    """muspinsim/tests/test_celio.py:21-26."""
    from muspinsim_gb300.spinsys import SpinSystem

    ssys = SpinSystem(["mu", "F", ("e", 2)], celio_k=10)
    ssys.add_linear_term(0, [1, 0, 0])
    ssys.add_bilinear_term(0, 1, [[0, 0, 1], [0, 0, 1], [0, 0, 1]])
    ssys.add_bilinear_term(0, 2, [[0, 0, -1], [0, 0, -1], [0, 0, -1]])
    return ssys


def test_contributions_known_answer():
    """muspinsim/tests/test_celio.py:21-75 on the host mirror."""
    from muspinsim_gb300.celio import CelioHamiltonian

    H = _ref_test_system().hamiltonian
    assert isinstance(H, CelioHamiltonian)
    hc = H._calc_H_contribs()
    assert len(hc) == 3
    want = [
        ([[0, 0.5], [0.5, 0]], 6, [0, 1, 2], [2, 2, 3]),
        ([[0.25, 0, 0.25 - 0.25j, 0], [0, -0.25, 0, -0.25 + 0.25j],
          [0.25 + 0.25j, 0, -0.25, 0], [0, -0.25 - 0.25j, 0, 0.25]], 3, [0, 1, 2], [2, 2, 3]),
        ([[-0.5, 0, 0, -0.5 + 0.5j, 0, 0], [0, 0, 0, 0, 0, 0], [0, 0, 0.5, 0, 0, 0.5 - 0.5j],
          [-0.5 - 0.5j, 0, 0, 0.5, 0, 0], [0, 0, 0, 0, 0, 0], [0, 0, 0.5 + 0.5j, 0, 0, -0.5]],
         2, [0, 2, 1], [2, 3, 2]),
    ]
    for c, (m, od, order, sd) in zip(hc, want):
        assert np.allclose(c.matrix.toarray(), m)
        assert c.other_dimension == od
        assert list(c.spin_order) == order
        assert list(c.spin_dimensions) == sd


def test_trotter_factor_known_answer():
    """muspinsim/tests/test_celio.py:77-119: exp(-2 pi i Sx / 10) on the
    muon, as a full-space matrix and as a 2 x 2 factor with its index map."""
    from muspinsim_gb300.celio import CelioEvolveContrib
    from muspinsim_gb300.spinsys import SpinSystem

    ssys = SpinSystem(["mu", "e"], celio_k=10)
    ssys.add_linear_term(0, [1, 0, 0])
    full = ssys.hamiltonian._calc_trotter_evol_op_contribs(1, False)
    assert len(full) == 1
    c, s = 0.95105652, -0.30901699j
    assert np.allclose(full[0].toarray(), [[c, 0, s, 0], [0, c, 0, s], [s, 0, c, 0],
                                           [0, s, 0, c]])
    fast = ssys.hamiltonian._calc_trotter_evol_op_contribs(1, True)
    assert isinstance(fast[0], CelioEvolveContrib)
    assert np.allclose(fast[0].matrix, [[c, s], [s, c]])
    assert fast[0].other_dim == 2
    assert np.array_equal(fast[0].indices, [0, 1, 2, 3])


def test_host_factors_match_oracle():
    """The host mirror's contributions, factors and index maps equal the
    oracle's for a system with a merged Zeeman run and a descending-index
    term."""
    from muspinsim_gb300.spinsys import MuonSpinSystem

    A = np.array([[10.0, 1.0, 0.0], [1.0, 8.0, 0.5], [0.0, 0.5, 12.0]])
    sy = MuonSpinSystem(["mu", "e", "H", "N"], celio_k=3)
    sy.add_hyperfine_term(0, A)
    sy.add_dipolar_term(3, 0, [0.4, 1.0, 0.9])
    sy.add_zeeman_term(3, [0.0, 0.0, 0.02])
    sy.add_quadrupolar_term(3, np.diag([0.1, 0.2, -0.3]))
    coup = [("hyperfine", {"i": 1}, A), ("dipolar", {"i": 4, "j": 1}, [0.4, 1.0, 0.9]),
            ("zeeman", {"i": 4}, [0.0, 0.0, 0.02]), ("quadrupolar", {"i": 4}, np.diag([0.1, 0.2, -0.3]))]
    osy = oracle_system(["mu", "e", "H", "N"], coup)
    dt = 0.05
    want = port.celio_factors(port.celio_contribs(list(osy.dims), port.celio_terms(osy)), dt, 3)
    got = sy.hamiltonian._calc_trotter_evol_op_contribs(dt, True)
    assert len(got) == len(want)
    for g, (U, od, order, _) in zip(got, want):
        assert g.spin_order == list(order) and g.other_dim == od
        assert np.abs(g.matrix - U).max() <= 1e-13
        assert np.array_equal(g.indices, port.celio_index_map(list(osy.dims), order))
    full = sy.hamiltonian._calc_trotter_evol_op_contribs(dt, False)
    for f, (U, _, order, _) in zip(full, want):
        assert np.abs(f.toarray() - port.celio_full_factor(U, list(osy.dims), order)).max() <= 1e-13


def test_factor_plans():
    """Digits and matrix offsets handed to msp_celio_run: one digit for a
    one-spin factor, two (in the factor's own order) for a pair; the
    density form applies U^dagger on the row digits and U^T on the columns."""
    from muspinsim_gb300.celio import _density_plan, _pure_plan

    dims = [2, 8, 3]
    U1 = np.eye(8) * (1 + 1j)
    U2 = np.arange(36).reshape(6, 6) * (1 - 2j)
    p = _pure_plan(dims, [(U1, [1, 0, 2]), (U2, [2, 0, 1])])
    assert p["digits"].tolist() == [[1, -1], [2, 0]]
    assert p["mat"].tolist() == [0, 64]
    assert np.array_equal(p["block"][64:], U2.reshape(-1))
    d = _density_plan(dims, [(U2, [2, 0, 1])])
    assert d["digits"].tolist() == [[2, 0], [5, 3]]
    assert np.array_equal(d["block"][:36], U2.conj().T.reshape(-1))
    assert np.array_equal(d["block"][36:], U2.T.reshape(-1))


def test_validation_errors():
    from muspinsim_gb300.validation import validate_celio_params

    with pytest.raises(ValueError, match="No interaction terms"):
        validate_celio_params([], np.linspace(0, 1, 5))
    with pytest.raises(ValueError, match="non-zero start time"):
        validate_celio_params([1], np.linspace(0.1, 1, 5))
    with pytest.raises(ValueError, match="uneven spacing"):
        validate_celio_params([1], np.array([0.0, 0.1, 0.3]))


def _runner(**kw):
    from muspinsim_gb300.experiment import ExperimentRunner
    from muspinsim_gb300.simconfig import make_params

    return ExperimentRunner(make_params(**kw))


def test_experiment_errors_before_any_device_work():
    """muspinsim/tests/test_experiment.py:340-470: an empty system, a muon
    that is not first with averages, finite temperature with averages,
    dissipation and the integral all fail as in the reference."""
    zee = [("zeeman", {"i": 2}, [0, 0, 1.0 / 135.53880943285955])]
    with pytest.raises(ValueError):
        _runner(spins=["e", "mu"], time=np.linspace(0, 10, 11), celio=(10, 0)).run()
    with pytest.raises(ValueError):
        _runner(spins=["e", "mu"], couplings=zee, time=np.linspace(0, 10, 11),
                celio=(10, 8)).run()
    with pytest.raises(ValueError):
        _runner(spins=["mu", "e"], couplings=[("zeeman", {"i": 1}, [0, 0, 0.01])],
                time=np.linspace(0, 10, 11), celio=(10, 8), temperature=[1.0]).run()
    with pytest.raises(NotImplementedError):
        _runner(spins=["e", "mu"], couplings=zee + [("dissipation", {"i": 1}, [0.5])],
                time=np.linspace(0, 10, 11), celio=(10, 0)).run()
    with pytest.raises(NotImplementedError):
        _runner(spins=["e", "mu"], couplings=zee, y_axis="integral", x_axis="field",
                field=[0.0, 0.1], celio=(10, 0)).run()


def test_capi_validation_without_device():
    from muspinsim_gb300 import _lib

    lib = _lib.load()
    a = _lib.CelioArgs()
    nbytes = ctypes.c_size_t(0)
    a.mode = 7
    assert lib.msp_celio_workspace(ctypes.byref(a), ctypes.byref(nbytes)) == _lib.MSP_ERR_ARG
    dims = (ctypes.c_int * 2)(3, 2)
    a.mode = _lib.CELIO_PURE
    a.num_digits = 2
    a.digit_dims = dims
    a.num_snapshots, a.states_per_snapshot, a.trotter_k, a.num_times = 1, 1, 1, 4
    assert lib.msp_celio_workspace(ctypes.byref(a), ctypes.byref(nbytes)) == _lib.MSP_ERR_ARG
    assert "muon" in _lib.last_error()
