"""GPU parity of the Lindblad (dissipation) path against the reference.

The reference diagonalises the superoperator (muspinsim/lindbladian.py);
libmspgpu propagates exp(2 pi L t) and solves (1/tau - 2 pi L) x = rho0
instead.  Checked against the reference's goldens (tests/golden/
lindblad_*.npz, produced by running the reference) to 1e-10, against its
analytic known answers (muspinsim/tests/test_lindbladian.py,
test_experiment.py:581-640) and against the oracle."""

import numpy as np
import pytest

from tests.helpers import golden_oracle, load_golden

pytestmark = pytest.mark.gpu

TOL = 1e-10


def test_direct_lindbladian_golden():
    from muspinsim_gb300.hamiltonian import Hamiltonian
    from muspinsim_gb300.lindbladian import Lindbladian
    from muspinsim_gb300.spinop import DensityOperator, SpinOperator

    g = load_golden("lindblad_direct")
    dim = (2, 2)
    H = Hamiltonian(g["H"], dim=dim)
    dops = [(SpinOperator(m, dim=dim), r) for m, r in zip(g["dops"], g["rates"])]
    L = Lindbladian.from_hamiltonian(H, dops)
    assert np.abs(L.matrix.toarray() - g["L"]).max() <= 1e-12 * np.abs(g["L"]).max()
    rho0 = DensityOperator(g["rho0"], dim)
    ops = [SpinOperator(o, dim=dim) for o in g["ops"]]
    ev = L.evolve(rho0, g["times"], ops)
    assert ev.shape == g["evolve"].shape
    assert np.abs(ev - g["evolve"]).max() <= TOL
    dens = L.evolve(rho0, g["times"][:5])
    got = np.array([d.matrix.toarray() for d in dens])
    assert np.abs(got - g["density"]).max() <= TOL
    integ = L.integrate_decaying(rho0, 2.19703, ops)
    assert np.abs(integ - g["integral"]).max() <= TOL
    # a non-uniform grid: one propagator per interval
    t = np.array([0.0, 0.013, 0.5, 0.51, 1.2])
    from oracle import port

    ref = port.lindblad_evolve(g["L"], g["rho0"], t, list(g["ops"]))
    assert np.abs(L.evolve(rho0, t, ops) - ref).max() <= TOL


def test_lindbladian_known_answers():
    """muspinsim/tests/test_lindbladian.py:10-85 on the GPU."""
    from muspinsim_gb300.hamiltonian import Hamiltonian
    from muspinsim_gb300.lindbladian import Lindbladian
    from muspinsim_gb300.spinop import DensityOperator, SpinOperator

    sx = SpinOperator.from_axes()
    sp = SpinOperator.from_axes(0.5, "+")
    sm = SpinOperator.from_axes(0.5, "-")
    sz = SpinOperator.from_axes(0.5, "z")
    H = Hamiltonian(sz.matrix)
    L = Lindbladian.from_hamiltonian(H)
    assert L.dimension == (2, 2)
    assert np.all(L.matrix.toarray() == 1.0j * np.diag([0, -1, 1, 0]))
    rho0 = DensityOperator.from_vectors(0.5, [1, 0, 0], 0)
    t = np.linspace(0, 1, 100)
    assert np.allclose(L.evolve(rho0, t, sx)[:, 0], 0.5 * np.cos(2 * np.pi * t), atol=1e-12)
    for g in [1.0, 2.0, 5.0, 10.0]:
        L = Lindbladian.from_hamiltonian(H, [(sx, g)])
        ap = -0.5 * np.pi * g + complex((0.5 * np.pi * g) ** 2 - 4 * np.pi ** 2) ** 0.5
        am = -0.5 * np.pi * g - complex((0.5 * np.pi * g) ** 2 - 4 * np.pi ** 2) ** 0.5
        A = ap * am / (am - ap)
        solx = np.real(0.5 * A * (np.exp(ap * t) / ap - np.exp(am * t) / am))
        assert np.abs(L.evolve(rho0, t, sx)[:, 0] - solx).max() <= 1e-10
        L = Lindbladian.from_hamiltonian(H, [(sp, 1.5 * g), (sm, 0.5 * g)])
        ev = L.evolve(rho0, t, [sx, sz])
        assert np.abs(ev[:, 0] - 0.5 * np.cos(2 * np.pi * t) * np.exp(-2 * np.pi * g * t)).max() <= 1e-10
        assert np.abs(ev[:, 1] - 0.25 * (1 - np.exp(-4 * np.pi * g * t))).max() <= 1e-10


def _runner(g, **over):
    from muspinsim_gb300.experiment import ExperimentRunner
    from muspinsim_gb300.simconfig import make_params

    coup = list(g["couplings"]) + [("dissipation", {"i": int(k)}, [float(v)])
                                   for k, v in g["dissipation"].items()]
    kw = dict(spins=g["spins"], couplings=coup, time=g["times"],
              orientation=list(g["orientations"]), field=list(g["fields"]),
              intrinsic_field=list(g["intrinsic"]), polarization=[g["polarization"]],
              temperature=list(g["temperatures"]), y_axis=g["y_axis"], x_axis=g["x_axis"],
              average_axes=g["average_axes"])
    kw.update(over)
    return ExperimentRunner(make_params(**kw))


@pytest.mark.parametrize("name", ["lindblad_mu_e", "lindblad_alc"])
def test_experiment_runner_lindblad_goldens(name):
    g = load_golden(name)
    res = _runner(g).run()
    assert res.shape == g["result"].shape
    assert np.abs(res - g["result"]).max() <= TOL


def test_experiment_dissipation_known_answers():
    """muspinsim/tests/test_experiment.py:581-640: a lone muon with
    dissipation g decays as 0.5 exp(-g t); at temperature T in a field
    its polarisation relaxes to 0.5 (1 - Z) / (1 + Z)."""
    import scipy.constants as cnst

    from muspinsim_gb300 import constants
    from muspinsim_gb300.experiment import ExperimentRunner
    from muspinsim_gb300.simconfig import make_params

    g = 1.0
    er = ExperimentRunner(make_params(spins=["mu"], couplings=[("dissipation", {"i": 1}, [g])]))
    times = er.config.x_axis_values
    assert np.abs(er.run() - 0.5 * np.exp(-g * times)).max() <= 1e-10
    T = 0.1
    er = ExperimentRunner(make_params(spins=["mu"], couplings=[("dissipation", {"i": 1}, [g])],
                                      temperature=[T], field=[-1.0], time=np.linspace(0, 20, 101)))
    Z = np.exp(-cnst.h * constants.MU_GAMMA * 1e6 / (cnst.k * T))
    er.load_config(er.config[0])
    Sz = er.system.operator({0: "z"})
    res = er.Htot.evolve(er.rho0, er.config.x_axis_values, operators=[Sz])
    assert abs(np.real(res[-1, 0]) - 0.5 * (1 - Z) / (1 + Z)) <= 1e-7


def test_lindblad_powder_vs_oracle_three_spins():
    """A larger dissipative powder (mu, e, 1H: n = 8, L 64 x 64) at finite
    temperature, against the oracle."""
    from muspinsim_gb300 import workloads

    rng = np.random.default_rng(21)
    coup = [("hyperfine", {"i": 1}, workloads.random_hyperfine(rng, 30.0)),
            ("hyperfine", {"i": 3}, workloads.random_hyperfine(rng, 5.0))]
    orients = [(0.3, 0.5, 0.1, 1.0), (1.1, 2.0, 0.7, 0.5), (2.0, 0.2, 1.9, 2.0)]
    g = {"spins": ["mu", "e", "H"], "couplings": coup, "times": np.linspace(0, 3, 90),
         "orientations": np.array(orients), "fields": np.array([[0.001, 0.0, 0.003]]),
         "intrinsic": np.zeros((1, 3)), "polarization": np.array([0.0, 0.0, 1.0]),
         "temperatures": np.array([15.0]), "y_axis": "asymmetry", "x_axis": "time",
         "average_axes": ["orientation"], "dissipation": {"2": 4.0, "3": 0.5}}
    res = _runner(g).run()
    ref = golden_oracle(g)
    assert np.abs(res - ref).max() <= TOL


MIXED_TOL = 1e-9  # double-word FP32 propagation


@pytest.mark.parametrize("name", ["lindblad_mu_e"])
def test_mixed_precision_golden(name):
    """The double-word propagation against the reference's golden run."""
    g = load_golden(name)
    er = _runner(g)
    er.precision = "mixed"
    res = er.run()
    assert np.abs(res - g["result"]).max() <= MIXED_TOL


def test_mixed_precision_three_spins_against_fp64():
    """mu, e, 1H (L 64 x 64, the largest double-word size) with two
    dissipative spins at finite temperature and a start time t0 > 0: the
    double-word propagation against the FP64 one."""
    from muspinsim_gb300 import workloads

    rng = np.random.default_rng(31)
    coup = [("hyperfine", {"i": 1}, workloads.random_hyperfine(rng, 30.0)),
            ("hyperfine", {"i": 3}, workloads.random_hyperfine(rng, 5.0))]
    orients = [(0.3, 0.5, 0.1, 1.0), (1.1, 2.0, 0.7, 0.5), (2.0, 0.2, 1.9, 2.0)]
    g = {"spins": ["mu", "e", "H"], "couplings": coup, "times": np.linspace(0.2, 4.0, 300),
         "orientations": np.array(orients), "fields": np.array([[0.001, 0.0, 0.003]]),
         "intrinsic": np.zeros((1, 3)), "polarization": np.array([0.0, 0.0, 1.0]),
         "temperatures": np.array([15.0]), "y_axis": "asymmetry", "x_axis": "time",
         "average_axes": ["orientation"], "dissipation": {"2": 4.0, "3": 0.5}}
    out = {}
    for prec in ("fp64", "mixed"):
        er = _runner(g)
        er.precision = prec
        out[prec] = er.run()
    assert np.abs(out["mixed"] - out["fp64"]).max() <= MIXED_TOL
    ref = golden_oracle(g)
    assert np.abs(out["fp64"] - ref).max() <= TOL
