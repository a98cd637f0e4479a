"""Pins the CPU oracle (oracle/port.py) to the reference.

The golden fixtures were produced by running the reference itself
(tests/golden/make_golden.py); the oracle must reproduce them to 1e-10 (both
are FP64 on the CPU; observed differences are ~1e-13, eigenvector-basis and
summation-order effects at phases ~1e4 rad).  The analytic known-answer
cases of the reference suite are restated at the end.
"""

import numpy as np
import pytest

from oracle import port
from tests.helpers import golden_oracle, load_golden, oracle_system

TOL = 1e-10


@pytest.mark.parametrize("name", ["config1_fast", "config2_powder16", "config2_powder8_T10K",
                                  "config5_fmuf", "e_mu_H_weighted"])
def test_time_domain_goldens(name):
    g = load_golden(name)
    got = golden_oracle(g)
    assert got.shape == g["result"].shape
    assert np.abs(got - g["result"]).max() <= TOL


def test_alc_integral_golden():
    g = load_golden("config3_alc")
    got = np.array([golden_oracle(g, field_index=f) for f in range(len(g["fields"]))])
    assert np.abs(got - g["result"]).max() <= TOL


def test_file_range_golden():
    # field x temperature file ranges, results indexed [field, temperature, t]
    g = load_golden("file_ranges")
    assert g["result"].shape == (2, 2, 100)
    for f in range(2):
        for t in range(2):
            got = golden_oracle(g, field_index=f, temp_index=t)
            assert np.abs(got - g["result"][f, t]).max() <= TOL


def test_direct_api_golden():
    g = load_golden("direct_dim24")
    H = g["H"]
    lam, U = np.linalg.eigh(H)
    assert np.abs(lam - g["evals"]).max() <= 1e-12 * np.abs(lam).max()
    ev = port.evolve(H, g["rho0"], g["times"], list(g["ops"]))
    assert np.abs(ev - g["evolve"]).max() <= TOL
    fast = port.fast_evolve(H, g["sigma"], g["times"], 12)
    assert np.abs(fast - g["fast"]).max() <= TOL
    integ = port.integrate_decaying(H, g["rho0"], 2.19703, list(g["ops"]))
    assert np.abs(integ - g["integral"]).max() <= TOL
    # density matrices: U exp(-i l t) U^dag rho U exp(i l t) U^dag
    for k in range(4):
        ph = np.exp(-2j * np.pi * lam * g["times"][k])
        Ut = (U * ph) @ U.conj().T
        rho_t = Ut @ g["rho0"] @ Ut.conj().T
        assert np.abs(rho_t - g["density"][k]).max() <= TOL


# ---- analytic known answers (muspinsim/tests/test_hamiltonian.py:34-128,
#      muspinsim/tests/test_experiment.py:118-200)

def _single_e_precession():
    sy = port.System(["e"], [port.ELEC_GAMMA], [0.5], [0.0])
    sy.add_term([0], [1.0, 0.0, 0.0])
    return sy


def test_known_evolve_cosine():
    sy = _single_e_precession()
    H = sy.hamiltonian()
    t = np.linspace(0, 1, 100)
    rho = port.density_from_vector(0.5, [0, 0, 1])
    res = port.evolve(H, rho, t, [port.embed(sy.Is, {0: "z"})])[:, 0]
    assert np.allclose(res, 0.5 * np.cos(2 * np.pi * t))


def test_known_integral():
    sy = _single_e_precession()
    H = sy.hamiltonian()
    rho = port.density_from_vector(0.5, [0, 0, 1])
    avg = port.integrate_decaying(H, rho, 1.0, [port.embed(sy.Is, {0: "z"})])
    assert np.isclose(avg[0], 0.5 / (1.0 + 4 * np.pi**2))


def test_known_fast_evolve():
    sy = port.System(["mu", "e"], [port.MU_GAMMA, port.ELEC_GAMMA], [0.5, 0.5], [0, 0])
    sy.add_term([0], [1.0, 0.0, 0.0])
    t = np.linspace(0, 1, 100)
    res = port.fast_evolve(sy.hamiltonian(), port.sigma_mu([0, 0, 1]), t, 2)
    assert np.allclose(res, 0.5 * np.cos(2 * np.pi * t))


def test_known_driver_integral():
    # muon Zeeman at 1/gamma_mu T: integral 0.5 / (1 + 4 pi^2 tau^2)
    sy = oracle_system(["e", "mu"], [("zeeman", {"i": 2}, [0, 0, 1.0 / port.MU_GAMMA])])
    r = port.powder_average(sy, [(0.0, 0.0, 0.0)], np.zeros(3), np.array([1.0, 0, 0]), np.inf,
                            [np.inf], y="integral")
    tau = port.MU_TAU
    assert np.isclose(r, 0.5 / (1.0 + 4 * np.pi**2 * tau**2))


def test_fast_path_rule():
    # muspinsim/tests/test_experiment.py:470-580
    assert port.t_inf_speedup([0, 0, 0.01], np.inf, 0)
    assert port.t_inf_speedup([0, 0, 0.0], 1.0, 0)
    assert not port.t_inf_speedup([0, 0, 0.01], 1.0, 0)
    assert not port.t_inf_speedup([0, 0, 0.01], np.inf, 1)


def test_cos_sum_c_matches_reference_formula():
    rng = np.random.default_rng(0)
    n, d = 8, 4
    A = rng.uniform(0, 1, (n, n))
    W = rng.normal(0, 30, (n, n))
    t = np.linspace(0, 3, 50)
    ref = np.array([(0.5 * np.trace(A) + sum(A[j, k] * np.cos(W[j, k] * ti)
                                             for j in range(n) for k in range(j))) / d
                    for ti in t])
    assert np.abs(port.fast_cos_sum(t, d, A, W) - ref).max() <= 1e-13


# ---- Lindblad dissipation (muspinsim/lindbladian.py, muspinsim/experiment.py:272-341)

def test_lindblad_experiment_goldens():
    g = load_golden("lindblad_mu_e")
    assert g["result"].shape == (2, 80)  # temperature file range x time
    for t in range(2):
        got = golden_oracle(g, temp_index=t)
        assert np.abs(got - g["result"][t]).max() <= TOL
    g = load_golden("lindblad_alc")
    got = np.array([golden_oracle(g, field_index=f) for f in range(len(g["fields"]))])
    assert np.abs(got - g["result"]).max() <= TOL


def test_lindblad_direct_golden():
    g = load_golden("lindblad_direct")
    L = port.lindblad_matrix(g["H"], list(zip(g["dops"], g["rates"])))
    assert np.abs(L - g["L"]).max() <= 1e-12 * np.abs(L).max()
    ev = port.lindblad_evolve(L, g["rho0"], g["times"], list(g["ops"]))
    assert np.abs(ev - g["evolve"]).max() <= TOL
    dens = port.lindblad_states(L, g["rho0"], g["times"][:5])
    assert np.abs(dens - g["density"]).max() <= TOL
    integ = port.lindblad_integrate(L, g["rho0"], 2.19703, list(g["ops"]))
    assert np.abs(integ - g["integral"]).max() <= TOL


def test_lindblad_known_answers():
    """muspinsim/tests/test_lindbladian.py:10-85 restated: the superoperator
    of S_z with an S_x dissipator, damped precession, thermalisation."""
    sx, sy_, sz = (port.spin_matrix(0.5, a) for a in "xyz")
    sp, sm = sx + 1j * sy_, sx - 1j * sy_
    assert np.allclose(port.lindblad_matrix(sz), 1j * np.diag([0, -1, 1, 0]))
    assert np.allclose(port.lindblad_matrix(sz, [(sx, 0.1)]),
                       [[-0.025, 0, 0, 0.025], [0, -0.025 - 1j, 0.025, 0],
                        [0, 0.025, -0.025 + 1j, 0], [0.025, 0, 0, -0.025]])
    rho0 = port.density_from_vector(0.5, [1, 0, 0])
    t = np.linspace(0, 1, 100)
    for g in [1.0, 2.0, 5.0, 10.0]:
        ap = -0.5 * np.pi * g + complex((0.5 * np.pi * g) ** 2 - 4 * np.pi ** 2) ** 0.5
        am = -0.5 * np.pi * g - complex((0.5 * np.pi * g) ** 2 - 4 * np.pi ** 2) ** 0.5
        A = ap * am / (am - ap)
        solx = np.real(0.5 * A * (np.exp(ap * t) / ap - np.exp(am * t) / am))
        ev = port.lindblad_evolve(port.lindblad_matrix(sz, [(sx, g)]), rho0, t, [sx])
        assert np.allclose(ev[:, 0], solx)
        ev = port.lindblad_evolve(port.lindblad_matrix(sz, [(sp, 1.5 * g), (sm, 0.5 * g)]), rho0,
                                  t, [sx, sz])
        assert np.allclose(ev[:, 0], 0.5 * np.cos(2 * np.pi * t) * np.exp(-2 * np.pi * g * t))
        assert np.allclose(ev[:, 1], 0.25 * (1 - np.exp(-4 * np.pi * g * t)))
