"""GPU parity of Celio's method (msp_celio_run, msp_celio_expm) against the
reference and the oracle.

* ExperimentRunner with Celio's method reproduces the reference's golden
  runs (tests/golden/celio_*.npz: averaged random states seeded exactly as
  the reference seeds them, and the density-matrix variant) to 1e-10;
* the analytic cases of muspinsim/tests/test_celio.py and
  test_experiment.py:340-470 hold;
* larger systems with factors of every size class (thread form D <= 16,
  warp form D = 7, 14, 64), the shared-memory and global-memory paths, and
  the device-built field factors agree with the oracle to 1e-10.
"""

import numpy as np
import pytest

from oracle import port
from tests.helpers import celio_phases, golden_oracle, load_golden, oracle_system

pytestmark = pytest.mark.gpu

TOL = 1e-10


def _runner(g, **over):
    from muspinsim_gb300.experiment import ExperimentRunner
    from muspinsim_gb300.simconfig import make_params

    kw = dict(spins=g["spins"], couplings=list(g["couplings"]), time=g["times"],
              orientation=list(g["orientations"]), field=list(g["fields"]),
              intrinsic_field=list(g["intrinsic"]), polarization=[g["polarization"]],
              temperature=list(g["temperatures"]), y_axis=g["y_axis"], x_axis=g["x_axis"],
              average_axes=g["average_axes"], celio=tuple(g["celio"]))
    kw.update(over)
    return ExperimentRunner(make_params(**kw))


@pytest.mark.parametrize("name", ["celio_fast_muVV", "celio_fast_field", "celio_rho_T",
                                  "celio_rho_desc"])
def test_experiment_runner_goldens(name):
    g = load_golden(name)
    er = _runner(g)
    if g.get("seed") is not None:
        np.random.seed(g["seed"])
    res = er.run()
    assert res.shape == g["result"].shape
    assert np.abs(res - g["result"]).max() <= TOL


def test_direct_api_known_answers():
    """muspinsim/tests/test_celio.py:121-158: precession about x of a spin
    started along z, through evolve and fast_evolve."""
    from muspinsim_gb300.spinop import DensityOperator
    from muspinsim_gb300.spinsys import MuonSpinSystem, SpinSystem

    ssys = SpinSystem(["e"], celio_k=10)
    ssys.add_linear_term(0, [1, 0, 0])
    t = np.linspace(0, 1, 100)
    ev = ssys.hamiltonian.evolve(DensityOperator.from_vectors(), t, [ssys.operator({0: "z"})])
    assert np.abs(ev[:, 0] - 0.5 * np.cos(2 * np.pi * t)).max() <= 1e-12
    with pytest.raises(ValueError):
        ssys.hamiltonian.evolve(DensityOperator.from_vectors(), t, [])
    with pytest.raises(NotImplementedError):
        ssys.hamiltonian.integrate_decaying(DensityOperator.from_vectors(), 1.0,
                                            ssys.operator({0: "z"}))
    msys = MuonSpinSystem(["mu", "e"], celio_k=10)
    msys.add_linear_term(0, [1, 0, 0])
    fe = msys.hamiltonian.fast_evolve(msys.sigma_mu([0, 0, 1]), t, 10)
    assert np.abs(fe - 0.5 * np.cos(2 * np.pi * t)).max() <= 1e-12


def test_experiment_known_answers():
    """muspinsim/tests/test_experiment.py:340-440: a muon precessing at 1 MHz
    with Celio's method, with and without averages."""
    from muspinsim_gb300.experiment import ExperimentRunner
    from muspinsim_gb300.simconfig import make_params

    t = np.linspace(0, 10, 101)
    for spins, i, celio in ((["e", "mu"], 2, (10, 0)), (["mu", "e"], 1, (10, 8))):
        er = ExperimentRunner(make_params(
            spins=spins, couplings=[("zeeman", {"i": i}, [0, 0, 1.0 / 135.53880943285955])],
            time=t, celio=celio))
        res = er.run()
        assert np.abs(res - 0.5 * np.cos(2 * np.pi * t)).max() <= 1e-8


def _big_system():
    """mu, V (I = 7/2), N (I = 1), H: quadrupoles on V and N, mu-V, N-V,
    H-N and mu-H dipolar terms, the N-V one with descending indices (factor
    dimensions 16, 8, 24, 3, 6, 4)."""
    rng = np.random.default_rng(42)
    qv = rng.normal(size=(3, 3)) * 0.02
    qn = rng.normal(size=(3, 3)) * 0.5
    coup = [("dipolar", {"i": 1, "j": 2}, [0.2, 1.1, 0.7]), ("quadrupolar", {"i": 2}, qv + qv.T),
            ("dipolar", {"i": 3, "j": 2}, [1.4, 0.3, 0.9]), ("quadrupolar", {"i": 3}, qn + qn.T),
            ("dipolar", {"i": 4, "j": 3}, [0.5, 0.6, 1.0]), ("dipolar", {"i": 1, "j": 4}, [1.0, 0.2, 0.3])]
    return ["mu", "V", "N", "H"], coup


@pytest.mark.parametrize("path", [0, 2])
def test_pure_against_oracle(path):
    """Averaged random states, two snapshots in a field, shared-memory and
    global-memory paths."""
    from muspinsim_gb300 import _lib, kernels
    from muspinsim_gb300.celio import _mu_psi, _pure_plan

    spins, coup = _big_system()
    osy = oracle_system(spins, coup)
    dims = list(osy.dims)
    t = np.linspace(0, 2.0, 25)
    k, A = 3, 2
    fields = np.array([[0.001, 0.0, 0.003], [0.0, 0.002, -0.001]])
    pols = np.array([[0.0, 0.6, 0.8], [1.0, 0.0, 0.0]])
    half = osy.n // 2
    ph = celio_phases(5, 2, A, half)
    blocks, ref = [], []
    for s in range(2):
        fac = port.celio_snapshot_factors(osy, fields[s], t[1] - t[0], k)
        plan = _pure_plan(dims, [(U, order) for U, _, order, _ in fac])
        blocks.append(plan["block"])
        ref.append(port.celio_fast_evolve(fac, dims, port.sigma_mu(pols[s]), t, k, ph[s]))
    sig = np.array([port.sigma_mu(p) for p in pols])
    series, rows = kernels.celio_run(
        _lib.CELIO_PURE, dims, plan["digits"], plan["mat"], np.stack(blocks), True, 2, A, k,
        len(t), mu_psi=_mu_psi(sig), sigma=sig, phases=ph, wscale=np.array([1.0, 1.0]),
        row_start=np.array([0, 1, 2]), num_rows=2, path=path)
    assert np.abs(rows.cpu().numpy() - np.array(ref)).max() <= TOL
    assert np.abs(series.cpu().numpy()[:, :, 0] - np.linalg.norm(pols, axis=1)[:, None]).max() <= 1e-12


def test_warp_form_factors_against_oracle():
    """Factor dimensions outside the register-resident set: D = 7 (spin
    3, one digit), 14 (muon x spin 3) and 64 (two I = 7/2 spins)."""
    from muspinsim_gb300 import _lib, kernels
    from muspinsim_gb300.celio import _mu_psi, _pure_plan

    rng = np.random.default_rng(8)
    D7 = 7
    dims = [2, D7, 8, 8]
    N = int(np.prod(dims))
    t = np.linspace(0, 1.0, 6)

    def unitary(D):
        H = rng.normal(size=(D, D)) + 1j * rng.normal(size=(D, D))
        H = H + H.conj().T
        w, V = np.linalg.eigh(H)
        return (V * np.exp(-1j * 0.3 * w)) @ V.conj().T

    facs = [(unitary(14), [0, 1, 2, 3]), (unitary(7), [1, 0, 2, 3]),
            (unitary(64), [3, 2, 0, 1]), (unitary(16), [0, 2, 1, 3])]
    ofac = [(U, N // U.shape[0], order, [dims[s] for s in order]) for U, order in facs]
    ph = celio_phases(9, 1, 1, N // 2)
    sig = port.sigma_mu([0.0, 0.0, 1.0])
    ref = port.celio_fast_evolve(ofac, dims, sig, t, 2, ph[0])
    plan = _pure_plan(dims, facs)
    for path in (0, 2):
        _, rows = kernels.celio_run(
            _lib.CELIO_PURE, dims, plan["digits"], plan["mat"], plan["block"][None], False, 1, 1,
            2, len(t), mu_psi=_mu_psi(sig)[None], sigma=sig[None], phases=ph,
            row_start=np.array([0, 1]), num_rows=1, path=path)
        assert np.abs(rows.cpu().numpy()[0] - ref).max() <= TOL


@pytest.mark.parametrize("path", [0, 2])
def test_density_against_oracle(path):
    """Density-matrix variant with two measured operators, both paths."""
    from muspinsim_gb300 import _lib, kernels
    from muspinsim_gb300.celio import _density_plan

    spins = ["mu", "e", "N"]
    coup = [("hyperfine", {"i": 1}, 30 * np.diag([1.0, 1.2, 0.8])),
            ("hyperfine", {"i": 3}, 3 * np.eye(3)), ("quadrupolar", {"i": 3}, np.diag([0.3, 0.2, -0.5]))]
    osy = oracle_system(spins, coup)
    dims = list(osy.dims)
    t = np.linspace(0, 0.5, 12)
    fac = port.celio_snapshot_factors(osy, [0.0, 0.0, 0.01], t[1] - t[0], 4)
    rho = port.rho0(osy, np.array([0.0, 0.0, 0.01]), np.array([1.0, 0.0, 0.0]), 30.0)
    ops = [osy.muon_operator([1.0, 0, 0]), osy.muon_operator([0.0, 1.0, 0])]
    ref = port.celio_evolve(fac, dims, rho, t, ops, 4)
    plan = _density_plan(dims, [(U, order) for U, _, order, _ in fac])
    N = osy.n
    series, _ = kernels.celio_run(
        _lib.CELIO_DENSITY, dims + dims, plan["digits"], plan["mat"], plan["block"][None], False,
        1, 1, 4, len(t), rho0=rho.reshape(1, N, N), meas=np.stack([o.T for o in ops])[None],
        path=path)
    assert np.abs(series.cpu().numpy()[0] - ref).max() <= TOL


def test_field_factor_exponentials():
    """msp_celio_expm against scipy's expm for spins 1/2, 1 and 7/2."""
    from scipy.linalg import expm

    import torch

    from muspinsim_gb300 import kernels

    rng = np.random.default_rng(4)
    dims = [2, 3, 8]
    H0, G = [], []
    for D in dims:
        h = rng.normal(size=(D, D)) + 1j * rng.normal(size=(D, D))
        H0.append(h + h.conj().T)
        g = rng.normal(size=(3, D, D)) + 1j * rng.normal(size=(3, D, D))
        G.append(20.0 * (g + np.conj(np.transpose(g, (0, 2, 1)))))
    B = rng.normal(size=(5, 3)) * 0.3
    tau = 0.013
    offs, o = [], 0
    for D in dims:
        offs.append((o, o + D * D, o + 2 * D * D))
        o += 3 * D * D
    mats = torch.zeros((5, o), dtype=torch.complex128, device=kernels.device())
    kernels.celio_expm(dims, H0, G, B, tau, offs, mats)
    m = mats.cpu().numpy()
    for s in range(5):
        for f, D in enumerate(dims):
            U = expm(-2j * np.pi * tau * (H0[f] + np.einsum("a,aij->ij", B[s], G[f])))
            a, b, c = offs[f]
            assert np.abs(m[s, a:a + D * D].reshape(D, D) - U).max() <= 1e-13
            assert np.abs(m[s, b:b + D * D].reshape(D, D) - U.conj().T).max() <= 1e-13
            assert np.abs(m[s, c:c + D * D].reshape(D, D) - U.T).max() <= 1e-13


def test_device_generated_states():
    """Without phases the initial states come from the device generator:
    P(0) is 0.5 exactly, different seeds give different curves, and the same
    seed the same curve."""
    from muspinsim_gb300 import _lib, kernels
    from muspinsim_gb300.celio import _mu_psi, _pure_plan

    spins, coup = _big_system()
    osy = oracle_system(spins, coup)
    dims = list(osy.dims)
    t = np.linspace(0, 2.0, 15)
    fac = port.celio_snapshot_factors(osy, None, t[1] - t[0], 2)
    plan = _pure_plan(dims, [(U, order) for U, _, order, _ in fac])
    sig = port.sigma_mu([0.0, 0.0, 1.0])
    outs = []
    for seed in (1, 1, 2):
        _, rows = kernels.celio_run(
            _lib.CELIO_PURE, dims, plan["digits"], plan["mat"], plan["block"][None], False, 1, 4,
            2, len(t), mu_psi=_mu_psi(sig)[None], sigma=sig[None], seed=seed,
            row_start=np.array([0, 1]), num_rows=1)
        outs.append(rows.cpu().numpy()[0])
    assert abs(outs[0][0] - 0.5) <= 1e-12
    assert np.array_equal(outs[0], outs[1])
    assert np.abs(outs[0] - outs[2]).max() > 1e-6
    assert np.abs(outs[0]).max() <= 0.5 + 1e-12


MIXED_TOL = 1e-9  # double-word FP32: ~2^-44 per factor application


@pytest.mark.parametrize("name", ["celio_fast_muVV", "celio_fast_field", "celio_rho_desc"])
def test_mixed_precision_goldens(name):
    """The double-word FP32 form against the reference's golden runs."""
    g = load_golden(name)
    er = _runner(g)
    er.precision = "mixed"
    if g.get("seed") is not None:
        np.random.seed(g["seed"])
    res = er.run()
    assert np.abs(res - g["result"]).max() <= MIXED_TOL


@pytest.mark.parametrize("path", [0, 2])
def test_mixed_precision_all_factor_forms(path):
    """Double-word FP32 with every factor form (register groups of D = 16,
    8, 3, 4, 6 and the FP64 warp fallback of D = 24) against FP64, many
    Trotter passes, in shared memory and from global memory."""
    from muspinsim_gb300 import _lib, kernels
    from muspinsim_gb300.celio import _mu_psi, _pure_plan

    spins, coup = _big_system()
    osy = oracle_system(spins, coup)
    dims = list(osy.dims)
    t = np.linspace(0, 4.0, 80)
    k = 10
    fac = port.celio_snapshot_factors(osy, [0.001, 0.0, 0.003], t[1] - t[0], k)
    plan = _pure_plan(dims, [(U, order) for U, _, order, _ in fac])
    sig = port.sigma_mu([0.0, 0.6, 0.8])
    ph = celio_phases(21, 1, 3, osy.n // 2)
    outs = {}
    for prec in (_lib.PREC_FP64, _lib.PREC_MIXED):
        series, _ = kernels.celio_run(
            _lib.CELIO_PURE, dims, plan["digits"], plan["mat"], plan["block"][None], False, 1, 3,
            k, len(t), mu_psi=_mu_psi(sig)[None], sigma=sig[None], phases=ph, precision=prec,
            path=path if prec == _lib.PREC_MIXED else 0)
        outs[prec] = series.cpu().numpy()
    assert np.abs(outs[_lib.PREC_MIXED] - outs[_lib.PREC_FP64]).max() <= MIXED_TOL


def test_mixed_precision_density_global():
    """The density-matrix form in double-word FP32 from global memory, with
    the warp fallback for its D = 24 factors, against the oracle."""
    from muspinsim_gb300 import _lib, kernels
    from muspinsim_gb300.celio import _density_plan

    spins, coup = _big_system()
    osy = oracle_system(spins, coup)
    dims = list(osy.dims)
    t = np.linspace(0, 0.4, 6)
    fac = port.celio_snapshot_factors(osy, [0.0, 0.0, 0.002], t[1] - t[0], 2)
    rho = port.rho0(osy, np.array([0.0, 0.0, 0.002]), np.array([0.0, 0.0, 1.0]), np.inf)
    ops = [osy.muon_operator([0.0, 0.0, 1.0])]
    ref = port.celio_evolve(fac, dims, rho, t, ops, 2)
    plan = _density_plan(dims, [(U, order) for U, _, order, _ in fac])
    N = osy.n
    series, _ = kernels.celio_run(
        _lib.CELIO_DENSITY, dims + dims, plan["digits"], plan["mat"], plan["block"][None], False,
        1, 1, 2, len(t), rho0=rho.reshape(1, N, N), meas=np.stack([o.T for o in ops])[None],
        path=2, precision=_lib.PREC_MIXED)
    assert np.abs(series.cpu().numpy()[0] - ref).max() <= MIXED_TOL
