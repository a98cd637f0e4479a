"""The reference-facing API on the GPU: Hamiltonian.diag / evolve /
fast_evolve / integrate_decaying and ExperimentRunner.run, against the
reference's golden outputs (tests/golden/, produced by running the reference)
and the known answers of its suite (muspinsim/tests/test_hamiltonian.py,
test_experiment.py).  FP64: max |dP| <= 1e-10; mixed: <= 1e-6."""

import numpy as np
import pytest

from tests.helpers import load_golden

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10
MIXED_TOL = 1e-6


def _runner(g, precision="fp64", **over):
    from muspinsim_gb300.experiment import ExperimentRunner
    from muspinsim_gb300.simconfig import make_params

    kw = dict(spins=g["spins"], couplings=g["couplings"], time=g["times"],
              orientation=list(g["orientations"]), field=list(g["fields"]),
              intrinsic_field=list(g["intrinsic"]), polarization=[g["polarization"]],
              temperature=list(g["temperatures"]), y_axis=g["y_axis"], x_axis=g["x_axis"],
              average_axes=g["average_axes"])
    kw.update(over)
    return ExperimentRunner(make_params(**kw), precision=precision)


@pytest.mark.parametrize("name", ["config1_fast", "config2_powder16", "config2_powder8_T10K",
                                  "config3_alc", "config5_fmuf", "e_mu_H_weighted", "file_ranges"])
def test_experiment_runner_goldens(name):
    g = load_golden(name)
    res = _runner(g).run()
    assert res.shape == g["result"].shape
    assert np.abs(res - g["result"]).max() <= FP64_TOL
    res_m = _runner(g, "mixed").run()
    assert np.abs(res_m - g["result"]).max() <= MIXED_TOL


def test_direct_api_golden():
    from muspinsim_gb300.hamiltonian import Hamiltonian
    from muspinsim_gb300.spinop import DensityOperator, SpinOperator

    g = load_golden("direct_dim24")
    dims = (2, 2, 2, 3)
    H = Hamiltonian(g["H"], dim=dims)
    evals, evecs = H.diag()
    assert np.abs(evals - g["evals"]).max() <= 1e-12 * np.abs(evals).max()
    rho0 = DensityOperator(g["rho0"], dims)
    ops = [SpinOperator(o, dim=dims) for o in g["ops"]]
    ev = H.evolve(rho0, g["times"], ops)
    assert ev.shape == g["evolve"].shape and ev.dtype == np.complex128
    assert np.abs(ev - g["evolve"]).max() <= FP64_TOL
    dens = H.evolve(rho0, g["times"][:4])
    assert len(dens) == 4 and isinstance(dens[0], DensityOperator)
    for k in range(4):
        assert np.abs(dens[k].matrix.toarray() - g["density"][k]).max() <= FP64_TOL
    fast = H.fast_evolve(g["sigma"], g["times"], 12)
    assert np.abs(fast - g["fast"]).max() <= FP64_TOL
    integ = H.integrate_decaying(rho0, 2.19703, ops)
    assert np.abs(integ - g["integral"]).max() <= FP64_TOL


# ---- known answers (muspinsim/tests/test_hamiltonian.py)

def test_hamiltonian_known_answers():
    from muspinsim_gb300.hamiltonian import Hamiltonian
    from muspinsim_gb300.spinop import DensityOperator, SpinOperator
    from muspinsim_gb300.spinsys import MuonSpinSystem, SpinSystem

    Sx = SpinOperator.from_axes()
    H = Hamiltonian(Sx.matrix)
    evals, evecs = H.diag()
    assert np.all(evals == [-0.5, 0.5]) or np.allclose(evals, [-0.5, 0.5], atol=1e-15)
    # columns parallel to the analytic eigenvectors (the reference's check
    # np.dot(evecs, evecsT) also fixes LAPACK's arbitrary signs)
    analytic = np.array([[1.0, 1.0], [-1.0, 1.0]]) / 2**0.5  # columns: l = -0.5, +0.5
    assert np.allclose(abs(evecs.conj().T @ analytic), np.eye(2))
    assert np.all(np.isclose(H.basis_change(evecs).matrix, np.diag(evals)))

    ssys = SpinSystem(["e"])
    ssys.add_linear_term(0, [1, 0, 0])
    H = ssys.hamiltonian
    rho0 = DensityOperator.from_vectors()
    t = np.linspace(0, 1, 100)
    evol = H.evolve(rho0, t, ssys.operator({0: "z"}))
    assert np.all(np.isclose(evol[:, 0], 0.5 * np.cos(2 * np.pi * t)))
    t4 = np.linspace(0, 1, 4)
    evol = H.evolve(rho0, t4)
    assert len(evol) == 4
    assert np.allclose(evol[1].matrix.toarray(), [[0.25, 0.433012702j], [-0.433012702j, 0.75]])
    assert np.allclose(evol[2].matrix.toarray(), [[0.25, -0.433012702j], [0.433012702j, 0.75]])
    assert np.allclose(evol[3].matrix.toarray(), [[1.0, 0.0], [0.0, 0.0]])
    avg = H.integrate_decaying(rho0, 1.0, ssys.operator({0: "z"}))
    assert np.isclose(avg[0], 0.5 / (1.0 + 4 * np.pi**2))

    msys = MuonSpinSystem(["mu", "e"])
    msys.add_linear_term(0, [1, 0, 0])
    evol = msys.hamiltonian.fast_evolve(msys.sigma_mu([0, 0, 1]), t, 2)
    assert np.all(np.isclose(evol, 0.5 * np.cos(2 * np.pi * t)))

    with pytest.raises(TypeError):
        H.evolve(np.eye(2), t)
    with pytest.raises(ValueError):
        H.integrate_decaying(rho0, -1.0, ssys.operator({0: "z"}))


# ---- known answers (muspinsim/tests/test_experiment.py)

def _mk(**kw):
    from muspinsim_gb300.experiment import ExperimentRunner
    from muspinsim_gb300.simconfig import make_params

    return ExperimentRunner(make_params(**kw))


def test_experiment_known_answers():
    from muspinsim_gb300 import constants

    t = np.linspace(0, 10, 100)
    res = _mk(spins=["e", "mu"], time=t).run()
    assert np.all(np.isclose(res, 0.5))
    zmn = [("zeeman", {"i": 2}, [0, 0, 1.0 / constants.MU_GAMMA])]
    er = _mk(spins=["e", "mu"], time=t, couplings=zmn)
    res = er.run()
    assert np.all(np.isclose(res, 0.5 * np.cos(2 * np.pi * er.config.x_axis_values)))
    assert not er._T_inf_speedup  # muon not first
    zmn1 = [("zeeman", {"i": 1}, [0, 0, 1.0 / constants.MU_GAMMA])]
    er = _mk(spins=["mu", "e"], time=t, couplings=zmn1)
    res = er.run()
    assert er._T_inf_speedup
    assert np.all(np.isclose(res, 0.5 * np.cos(2 * np.pi * t)))
    er = _mk(spins=["mu", "e"], time=t, couplings=zmn1, temperature=[1.0])
    er.run()
    assert er._T_inf_speedup  # no field: fast even at low T
    er = _mk(spins=["mu", "e"], time=t, couplings=zmn1, field=[(0.01,)])
    er.run()
    assert er._T_inf_speedup
    er = _mk(spins=["mu", "e"], time=t, couplings=zmn1, field=[(0.01,)], temperature=[1.0])
    er.run()
    assert not er._T_inf_speedup
    tau = constants.MU_TAU
    for axis in ("field", "intrinsic_field"):
        kw = {axis: [(0.0,), (1.0,)]}
        res = _mk(spins=["e", "mu"], time=t, couplings=zmn, y_axis="integral", x_axis=axis,
                  **kw).run()
        assert np.isclose(res[0], 0.5 / (1.0 + 4 * np.pi**2 * tau**2))
    res = _mk(spins=["e", "mu"], time=t, field=[(0.0,), (10.0,)], temperature=[np.inf, 0.0]).run()
    assert res.shape == (2, 2, 100)
    # the external field turns with the crystallite, the intrinsic one does
    # not (muspinsim/tests/test_experiment.py:283-326; an explicit tilted
    # orientation instead of a one-point powder grid)
    r1 = _mk(spins=["e", "mu"], time=t, couplings=zmn, orientation=[(0.3, 1.1, 0.0)],
             field=[(0.01, 0.0, 0.0)]).run()
    r2 = _mk(spins=["e", "mu"], time=t, couplings=zmn, orientation=[(0.3, 1.1, 0.0)],
             intrinsic_field=[(0.01, 0.0, 0.0)]).run()
    assert not np.allclose(r1, r2)


def test_run_single_matches_batched():
    g = load_golden("config2_powder8_T10K")
    er = _runner(g)
    batched = er.run()
    acc = np.zeros_like(batched)
    for snap in er.config:
        acc += er.run_single(snap) / er.config.avg_N
    assert np.abs(acc - batched).max() <= FP64_TOL


# ---- n > 64 (Householder + QL; global-memory basis changes)

def test_direct_api_large_against_oracle():
    """Hamiltonian.evolve / integrate_decaying / fast_evolve at n = 96
    (mu, e, 1H x 3, 14N dimensions) against the oracle's numpy
    restatement."""
    from oracle import port
    from muspinsim_gb300.hamiltonian import Hamiltonian
    from muspinsim_gb300.spinop import DensityOperator, SpinOperator
    from tests.helpers import random_hermitian

    rng = np.random.default_rng(960)
    dims = (2, 2, 2, 2, 2, 3)
    n = int(np.prod(dims))
    # spectral width ~ 60 MHz and unit-norm operators, as for spin systems
    Hm = random_hermitian(rng, n)
    Hm *= 30.0 / np.abs(np.linalg.eigvalsh(Hm)).max()
    R = random_hermitian(rng, n)
    rho = R @ R.conj().T
    rho /= np.trace(rho).real
    ops = [o / np.abs(np.linalg.eigvalsh(o)).max()
           for o in (random_hermitian(rng, n), random_hermitian(rng, n))]
    t = np.linspace(0.0, 2.0, 37)
    H = Hamiltonian(Hm, dim=dims)
    rho0 = DensityOperator(rho, dims)
    sops = [SpinOperator(o, dim=dims) for o in ops]
    ev = H.evolve(rho0, t, sops)
    assert ev.shape == (len(t), 2)
    assert np.abs(ev - port.evolve(Hm, rho, t, ops)).max() <= FP64_TOL
    dens = H.evolve(rho0, t[:3])
    assert len(dens) == 3
    evals, U = np.linalg.eigh(Hm)
    for k in range(3):
        ph = np.exp(-2j * np.pi * np.subtract.outer(evals, evals) * t[k])
        want = U @ ((U.conj().T @ rho @ U) * ph) @ U.conj().T
        assert np.abs(dens[k].matrix.toarray() - want).max() <= FP64_TOL
    integ = H.integrate_decaying(rho0, 2.19703, sops)
    assert np.abs(integ - port.integrate_decaying(Hm, rho, 2.19703, ops)).max() <= FP64_TOL
    sig = port.sigma_mu([0.3, 0.4, np.sqrt(0.75)])
    fast = H.fast_evolve(sig, t, n // 2)
    assert np.abs(fast - port.fast_evolve(Hm, sig, t, n // 2)).max() <= FP64_TOL
