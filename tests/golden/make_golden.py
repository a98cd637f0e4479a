"""Generate the golden fixtures of tests/golden/ by running the REFERENCE.

Needs the reference tree (imported through tests/golden/refshim.py) and its
Cython kernel built by oracle/build.py; run it only where the reference is
present:

    python tests/golden/make_golden.py

Each fixture is a small .npz with the inputs (spins, couplings as JSON,
orientations, fields, times, polarisation, temperature, axes) and the
reference's output of ExperimentRunner.run() -- or of Hamiltonian.diag /
evolve / fast_evolve / integrate_decaying for the direct-API cases.  The
synthetic systems come from muspinsim_gb300.workloads (seeded), reduced in
size so that the CPU oracle and the reference finish in seconds.
"""

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, HERE)

import refshim  # noqa: E402


def _jsonable_couplings(couplings):
    return [[k, dict(a), np.asarray(v, dtype=float).tolist()] for k, a, v in couplings]


def _run_reference(spins, couplings, times, orientations, fields, pol, temps, y_axis,
                   x_axis, intrinsic=((0.0, 0.0, 0.0),), average_axes=("orientation",),
                   dissipation=None, celio=(0, 0), seed=None):
    from muspinsim.experiment import ExperimentRunner

    p = refshim.make_params(spins, couplings, times, orientations, field=fields,
                            intrinsic_field=intrinsic, polarization=pol, temperature=temps,
                            y_axis=y_axis, x_axis=x_axis, average_axes=average_axes,
                            dissipation=dissipation, celio=celio)
    er = ExperimentRunner(refshim.ParamsInput(p))
    if seed is not None:
        np.random.seed(seed)
    return np.array(er.run())


def save_experiment(name, spins, couplings, times, orientations, fields=((0.0, 0.0, 0.0),),
                    pol=(1.0, 0.0, 0.0), temps=(np.inf,), y_axis="asymmetry", x_axis="time",
                    intrinsic=((0.0, 0.0, 0.0),), average_axes=("orientation",),
                    dissipation=None, celio=(0, 0), seed=None):
    """Run the reference's ExperimentRunner and store inputs and result.
    With Celio's method and averages, ``seed`` seeds numpy's global
    generator before the run, so the random initial states are reproducible
    (the reference draws np.random.rand(d) per snapshot and average)."""
    out = _run_reference(spins, couplings, times, orientations, fields, pol, temps, y_axis,
                         x_axis, intrinsic, average_axes, dissipation, celio, seed)
    meta = {"spins": list(spins), "couplings": _jsonable_couplings(couplings),
            "y_axis": y_axis, "x_axis": x_axis, "average_axes": list(average_axes),
            "dissipation": {str(k): float(v) for k, v in (dissipation or {}).items()},
            "celio": [int(c) for c in celio], "seed": seed}
    np.savez_compressed(
        os.path.join(HERE, name + ".npz"),
        meta=np.array(json.dumps(meta)),
        times=np.asarray(times, dtype=float),
        orientations=np.asarray(orientations, dtype=float),
        fields=np.asarray([np.atleast_1d(f) for f in fields], dtype=float),
        intrinsic=np.asarray([np.atleast_1d(f) for f in intrinsic], dtype=float),
        polarization=np.asarray(pol, dtype=float),
        temperatures=np.asarray(temps, dtype=float),
        result=out,
    )
    print(f"{name}: result shape {out.shape}")


def save_direct(name):
    """Direct-API goldens: diag, evolve (with and without operators),
    fast_evolve, integrate_decaying of one random dim-24 Hamiltonian."""
    from muspinsim.spinop import DensityOperator
    from muspinsim.spinsys import MuonSpinSystem

    from muspinsim_gb300 import workloads

    wl = workloads.config2(n_orient=1, n_times=64)
    sy = MuonSpinSystem(list(wl.spins))
    for kind, args, val in wl.couplings:
        i, j = args["i"] - 1, args.get("j")
        j = None if j is None else j - 1
        {"hyperfine": lambda: sy.add_hyperfine_term(i, val, j),
         "dipolar": lambda: sy.add_dipolar_term(i, j, val),
         "quadrupolar": lambda: sy.add_quadrupolar_term(i, val)}[kind]()
    sy.add_zeeman_term(0, [0.001, 0.002, 0.01])
    sy.add_zeeman_term(1, [0.001, 0.002, 0.01])
    # a fresh Hamiltonian per call: the reference's diag() cache-hit branch
    # fails under scipy >= 1.15 (muspinsim/spinop.py:61-66)
    evals, evecs = sy.hamiltonian.diag()
    Hm = sy.hamiltonian.matrix.toarray()
    t = np.linspace(0, 2.0, 64)
    rho0 = DensityOperator.from_vectors([0.5, 0.5, 0.5, 1.0], [[0, 0, 1], [1, 0, 0], [0, 1, 0],
                                                             [0, 0, 1]], [0, 0, 0, 0.5])
    ops = [sy.operator({0: "x"}), sy.operator({0: "z"}), sy.operator({2: "+"})]
    ev = sy.hamiltonian.evolve(rho0, t, ops)
    dens = sy.hamiltonian.evolve(rho0, t[:4])
    dens = np.array([d.matrix.toarray() for d in dens])
    fast = sy.hamiltonian.fast_evolve(sy.sigma_mu([0.3, 0.4, 0.5]), t, 12)
    integ = sy.hamiltonian.integrate_decaying(rho0, 2.19703, ops)
    np.savez_compressed(
        os.path.join(HERE, name + ".npz"),
        H=Hm, evals=evals, times=t, rho0=rho0.matrix.toarray(),
        ops=np.array([o.matrix.toarray() for o in ops]), evolve=ev, density=dens,
        sigma=sy.sigma_mu([0.3, 0.4, 0.5]).toarray(), fast=fast, integral=integ)
    print(f"{name}: dim {Hm.shape[0]}")


def save_lindblad_direct(name):
    """Direct-API goldens of the Lindbladian: evolve with and without
    operators and integrate_decaying, for a mu + e system in a field with
    two dissipators (muspinsim/lindbladian.py:17-173)."""
    from muspinsim.lindbladian import Lindbladian
    from muspinsim.spinop import DensityOperator
    from muspinsim.spinsys import MuonSpinSystem

    sy = MuonSpinSystem(["mu", "e"])
    sy.add_hyperfine_term(0, np.array([[120.0, 10.0, 0.0], [10.0, 80.0, 5.0], [0.0, 5.0, 60.0]]))
    sy.add_zeeman_term(0, [0.001, 0.0, 0.004])
    sy.add_zeeman_term(1, [0.001, 0.0, 0.004])
    H = sy.hamiltonian
    dops = [(sy.operator({1: "x"}), 0.7), (sy.operator({1: "+"}), 0.3),
            (sy.operator({0: "z"}), 0.05)]
    L = Lindbladian.from_hamiltonian(H, dops)
    rho0 = DensityOperator.from_vectors([0.5, 0.5], [[0, 0, 1], [1, 0, 0]], [0, 0.3])
    t = np.linspace(0, 1.5, 60)
    ops = [sy.operator({0: "x"}), sy.operator({0: "z"}), sy.operator({1: "+"})]
    ev = L.evolve(rho0, t, ops)
    dens = np.array([d.matrix.toarray() for d in L.evolve(rho0, t[:5])])
    integ = L.integrate_decaying(rho0, 2.19703, ops)
    np.savez_compressed(
        os.path.join(HERE, name + ".npz"),
        H=H.matrix.toarray(), L=L.matrix.toarray(), rho0=rho0.matrix.toarray(), times=t,
        ops=np.array([o.matrix.toarray() for o in ops]),
        dops=np.array([o.matrix.toarray() for o, _ in dops]),
        rates=np.array([g for _, g in dops]), evolve=ev, density=dens, integral=integ)
    print(f"{name}: L {L.matrix.shape}")


def save_celio():
    """Celio's method through ExperimentRunner (muspinsim/celio.py,
    muspinsim/experiment.py:434-471): averaged random states (the native
    module) and the density-matrix variant, with and without a field."""
    # mu + 2 V (I = 7/2): mu-V dipolar (16 x 16 factors) and V quadrupoles
    # (8 x 8), zero field, polarisation along x; 3 orientations x 4 averages
    rng = np.random.default_rng(505)
    coup = []
    for v in (2, 3):
        r = rng.normal(size=3)
        coup.append(("dipolar", {"i": 1, "j": v}, 1.3 * r / np.linalg.norm(r)))
        q = rng.normal(size=(3, 3)) * 0.02
        q = q + q.T
        coup.append(("quadrupolar", {"i": v}, q - np.trace(q) / 3 * np.eye(3)))
    save_experiment("celio_fast_muVV", ["mu", "V", "V"], coup, np.linspace(0, 6.0, 40),
                    [(0.1, 0.2, 0.3, 1.0), (1.0, 2.0, 0.5, 2.0), (2.5, 0.4, 1.5, 0.5)],
                    [(0.0, 0.0, 0.0)], (1.0, 0.0, 0.0), celio=(10, 4), seed=1234)
    # mu + e + H + F in a field: hyperfine, a descending-index dipolar term
    # (F -> mu) and a user Zeeman term on F that merges with the field's
    # Zeeman term into one factor; 4 orientations x 3 averages
    A1 = 40.0 * np.array([[1.0, 0.1, 0.0], [0.1, 0.8, 0.05], [0.0, 0.05, 1.2]])
    A2 = 5.0 * np.array([[0.3, 0.0, 0.1], [0.0, -0.2, 0.0], [0.1, 0.0, 0.5]])
    coup = [("hyperfine", {"i": 1}, A1), ("hyperfine", {"i": 3}, A2),
            ("dipolar", {"i": 4, "j": 1}, [0.4, 1.0, 0.9]), ("zeeman", {"i": 4}, [0.0, 0.0, 0.02])]
    save_experiment("celio_fast_field", ["mu", "e", "H", "F"], coup, np.linspace(0, 1.5, 25),
                    [(0.1, 0.2, 0.3, 1.0), (1.0, 2.0, 0.5, 2.0), (2.5, 0.4, 1.5, 0.5),
                     (0.7, 1.1, 2.9, 1.5)],
                    [(0.002, 0.001, 0.01)], (0.0, 0.0, 1.0), celio=(4, 3), seed=99)
    # density-matrix variant at finite temperature in a field (mu, e, H)
    save_experiment("celio_rho_T", ["mu", "e", "H"], coup[:2] + [("dipolar", {"i": 3, "j": 1},
                                                                   [0.5, 1.1, 0.2])],
                    np.linspace(0, 1.0, 30), [(0.1, 0.2, 0.3, 1.0), (1.0, 2.0, 0.5, 2.0)],
                    [(0.0, 0.0, 0.003)], (1.0, 0.0, 0.0), temps=(20.0,), celio=(6, 0))
    # density-matrix variant with a descending-index dipolar term between
    # spins of different dimension (N -> mu) and a quadrupole, zero field
    q = np.array([[0.2, 0.05, 0.0], [0.05, -0.5, 0.1], [0.0, 0.1, 0.3]])
    save_experiment("celio_rho_desc", ["mu", "H", "N"],
                    [("dipolar", {"i": 3, "j": 1}, [0.3, 0.9, 1.1]),
                     ("dipolar", {"i": 2, "j": 1}, [1.0, 0.2, 0.3]), ("quadrupolar", {"i": 3}, q)],
                    np.linspace(0, 3.0, 35), [(0.3, 0.6, 0.9, 1.0), (2.0, 1.0, 0.4, 1.0)],
                    [(0.0, 0.0, 0.0)], (0.0, 1.0, 0.0), celio=(5, 0))


CONFIG_LAYOUTS = [
    # (times, orientations, fields, temperatures, y axis, x axis, averaged axes)
    (np.linspace(0, 5, 7).tolist(), [(0, 0, 0, 1.0), (0.3, 0.2, 0.1, 2.0), (1, 2, 0.5, 1.0)],
     [(0, 0, 0.01), (0, 0, 0.02)], [np.inf], "asymmetry", "time", ["orientation"]),
    ([0.0], [(0, 0, 0), (0.3, 0.2, 0.1)], [(0, 0, 0.01), (0, 0, 0.02), (0, 0, 0.03)],
     [np.inf, 10.0], "integral", "field", ["orientation", "temperature"]),
    (np.linspace(0, 1, 5).tolist(), [(0, 0, 0)], [(0, 0, 0.01), (0, 0, 0.02)], [np.inf],
     "asymmetry", "field", ["time"]),
    (np.linspace(0, 1, 5).tolist(), [(0, 0, 0)], [(0, 0, 0.01), (0.005, 0, 0.01)],
     [np.inf, 5.0], "asymmetry", "time", ["none"]),
]
CONFIG_SPINS = ["mu", "e", "H"]
CONFIG_COUPLINGS = [("hyperfine", {"i": 1}, 100.0 * np.eye(3)),
                    ("dipolar", {"i": 1, "j": 3}, [0.0, 0.0, 1.5]),
                    ("zeeman", {"i": 3}, [0.0, 0.0, 0.01])]


def save_config_layouts(name):
    """The reference MuSpinConfig's snapshot grid for four axis layouts: the
    configuration indices, result shape, range keys in order, constants,
    averaged count and per-snapshot orientation quaternions and weights
    (muspinsim/simconfig.py:78-321); and the .dat files its save_output
    writes for set results (muspinsim/simconfig.py:370-429), with the date
    line blanked."""
    import tempfile

    from muspinsim.simconfig import MuSpinConfig

    layouts = []
    for times, orients, fields, temps, y, x, avg in CONFIG_LAYOUTS:
        p = refshim.make_params(CONFIG_SPINS, CONFIG_COUPLINGS, times, orients, field=fields,
                                polarization=(1.0, 0.0, 0.0), temperature=temps, y_axis=y,
                                x_axis=x, average_axes=avg)
        cfg = MuSpinConfig(p)
        cfgs = [[[None if isinstance(i, slice) else int(i) for i in part] for part in c]
                for c in cfg._configurations]
        snaps = []
        for k in range(len(cfg)):
            o = cfg[k].orient
            snaps.append([list(map(float, o[0].q)), float(o[1])])
        cfg.results = np.arange(cfg.results.size, dtype=float).reshape(cfg.results.shape) * 0.25
        files = {}
        with tempfile.TemporaryDirectory() as d:
            cfg.save_output(name="out", path=d)
            for fn in sorted(os.listdir(d)):
                with open(os.path.join(d, fn)) as f:
                    lines = f.read().splitlines()
                files[fn] = [("# Output file written on <date>" if ln.startswith(
                    "# Output file written on") else ln) for ln in lines]
        layouts.append({
            "layout": [times, [list(o) for o in orients], [list(f) for f in fields],
                       [float(t) for t in temps], y, x, avg],
            "configurations": cfgs, "shape": list(cfg.results.shape),
            "file_ranges": list(cfg._file_ranges.keys()),
            "avg_ranges": list(cfg._avg_ranges.keys()), "x": list(cfg._x_range.keys())[0],
            "avg_N": int(cfg._avg_N), "time_N": int(cfg._time_N),
            "constants": sorted(cfg._constants.keys()), "orient": snaps, "files": files})
    with open(os.path.join(HERE, name + ".json"), "w") as f:
        json.dump({"spins": CONFIG_SPINS, "couplings": _jsonable_couplings(CONFIG_COUPLINGS),
                   "layouts": layouts}, f, indent=0, default=float)
    print(f"{name}: {len(layouts)} layouts")


def _reference_system(wl):
    from muspinsim.spinsys import MuonSpinSystem

    sy = MuonSpinSystem(list(wl.spins))
    for kind, args, val in wl.couplings:
        i, j = args["i"] - 1, args.get("j")
        j = None if j is None else j - 1
        {"hyperfine": lambda: sy.add_hyperfine_term(i, val, j),
         "dipolar": lambda: sy.add_dipolar_term(i, j, val),
         "quadrupolar": lambda: sy.add_quadrupolar_term(i, val)}[kind]()
    return sy


def save_rotated(name):
    """SpinSystem.rotate(R).hamiltonian of the dim-24 system for seeded
    rotation matrices (muspinsim/spinsys.py:103-135, 594-626)."""
    from muspinsim_gb300 import quaternion as Q
    from muspinsim_gb300 import workloads

    wl = workloads.config2(n_orient=1, n_times=8)
    sy = _reference_system(wl)
    rng = np.random.default_rng(4242)
    qs = Q.from_euler(*rng.uniform(0, 2 * np.pi, (3, 6)), "zyz")
    Rs = Q.rotation_matrix(qs)
    H0 = sy.hamiltonian.matrix.toarray()
    HR = np.array([sy.rotate(R).hamiltonian.matrix.toarray() for R in Rs])
    np.savez_compressed(os.path.join(HERE, name + ".npz"), R=Rs, H=H0, HR=HR,
                        meta=np.array(json.dumps({"spins": list(wl.spins),
                                                  "couplings": _jsonable_couplings(wl.couplings)})))
    print(f"{name}: {len(Rs)} rotations of a dim-{H0.shape[0]} system")


def save_fast_binding(name):
    """The arguments Hamiltonian.fast_evolve passes to its native kernel
    parallel_fast_time_evolve (muspinsim/hamiltonian.py:195-217), that
    kernel's output and fast_evolve's result, for the dim-24 system in a
    field: what a GPU stub bound at muspinsim/hamiltonian.py:10 receives."""
    import muspinsim.hamiltonian as hm

    from muspinsim_gb300 import workloads

    wl = workloads.config2(n_orient=1, n_times=8)
    sy = _reference_system(wl)
    sy.add_zeeman_term(0, [0.002, -0.001, 0.01])
    sy.add_zeeman_term(1, [0.002, -0.001, 0.01])
    calls = []
    native = hm.parallel_fast_time_evolve

    def spy(times, other_dimension, A, W):
        out = native(times, other_dimension, A, W)
        calls.append((np.array(times), int(other_dimension), np.array(A), np.array(W),
                      np.array(out)))
        return out

    hm.parallel_fast_time_evolve = spy
    try:
        t = np.linspace(0.0, 10.0, 777)
        fast = sy.hamiltonian.fast_evolve(sy.sigma_mu([0.3, -0.4, 0.866]), t, 12)
    finally:
        hm.parallel_fast_time_evolve = native
    times, d, A, W, kout = calls[0]
    np.savez_compressed(os.path.join(HERE, name + ".npz"), times=times, d=d, A=A, W=W,
                        kernel=kout, fast=fast)
    print(f"{name}: n = {A.shape[0]}, {len(times)} times")


FIT_TIMES = np.linspace(0.0, 10.0, 150)
FIT_TRUE = {"r1": 1.18, "r2": 1.25}
FIT_START = {"r1": 1.10, "r2": 1.32}


def fit_params(make_params, r1, r2):
    """The F-mu-F fit problem's evaluated parameters (as a function of the two
    mu-F distances, Angstrom): the config-5 geometry with its dipolar
    directions kept and lengths set; 12 orientations; 150 times.  Used with
    the reference's refshim.make_params here and with the package's
    simconfig.make_params in the tests."""
    from muspinsim_gb300 import workloads

    wl = workloads.config5(n_orient=12, n_times=150)
    (k1, a1, v1), (k2, a2, v2), third = wl.couplings
    u1, u2 = np.asarray(v1) / np.linalg.norm(v1), np.asarray(v2) / np.linalg.norm(v2)
    coup = [(k1, a1, u1 * r1), (k2, a2, u2 * r2), third]
    return make_params(wl.spins, coup, FIT_TIMES, wl.orientations, wl.fields[0],
                       wl.polarization)


def save_fit(name):
    """The reference's FittingRunner on the F-mu-F problem
    (muspinsim/fitting.py:15-179): target = its own P(t) at FIT_TRUE plus
    N(0, 0.01^2) noise; L-BFGS-B (its scipy difference quotients) and
    Nelder-Mead results from FIT_START, the objective there and its central
    differences (h = 1e-6)."""
    from muspinsim.experiment import ExperimentRunner
    from muspinsim.fitting import FittingRunner
    from muspinsim.input.variables import FittingVariable

    def mk(spins, coup, times, orients, field, pol):
        return refshim.make_params(spins, coup, times, orients, field=[field],
                                   polarization=pol)

    truth = np.array(ExperimentRunner(refshim.ParamsInput(fit_params(mk, **FIT_TRUE))).run())
    rng = np.random.default_rng(5151)
    data = np.stack([FIT_TIMES, truth + rng.normal(0.0, 0.01, truth.shape)], axis=1)

    class FitIn:
        def __init__(self, method):
            self.fitting_info = {"fit": True, "data": data, "method": method, "rtol": 1e-8,
                                 "function": None, "single_simulation": False,
                                 "evaluate_x_axis": False}
            self.variables = {k: FittingVariable(k, v, 0.8, 2.0) for k, v in FIT_START.items()}

        def evaluate(self, **v):
            p = fit_params(mk, **v)
            p["fitting_info"] = dict(self.fitting_info)
            return p

    out = {}
    for method in ("lbfgs", "nelder-mead"):
        fr = FittingRunner(FitIn(method))
        sol = fr.run()
        out[method] = (np.asarray(sol["x"], dtype=float), float(sol["fun"]), int(sol["nfev"]))
    fr = FittingRunner(FitIn("lbfgs"))
    x0 = np.array([FIT_START[k] for k in sorted(FIT_START)])
    f0 = fr._targfun_minimise(x0)
    g0 = np.zeros(2)
    for k in range(2):
        up, dn = x0.copy(), x0.copy()
        up[k] += 1e-6
        dn[k] -= 1e-6
        g0[k] = (fr._targfun_minimise(up) - fr._targfun_minimise(dn)) / 2e-6
    np.savez_compressed(os.path.join(HERE, name + ".npz"), data=data, truth=truth, x0=x0, f0=f0,
                        g0=g0, x_lbfgs=out["lbfgs"][0], f_lbfgs=out["lbfgs"][1],
                        nfev_lbfgs=out["lbfgs"][2], x_nm=out["nelder-mead"][0],
                        f_nm=out["nelder-mead"][1], nfev_nm=out["nelder-mead"][2])
    print(f"{name}: lbfgs x={out['lbfgs'][0]} f={out['lbfgs'][1]:.6g} nfev={out['lbfgs'][2]}; "
          f"nelder-mead x={out['nelder-mead'][0]} f={out['nelder-mead'][1]:.6g}")


def main(only=None):
    refshim.install()
    if only == "fit":
        save_fit("fit_fmuf")
        return
    if only == "celio":
        save_celio()
        return
    if only == "boundary":
        save_config_layouts("config_layouts")
        save_rotated("rotated_dim24")
        save_fast_binding("fast_binding_dim24")
        return
    from muspinsim_gb300 import workloads

    w1 = workloads.config1()
    save_experiment("config1_fast", w1.spins, w1.couplings, w1.times, w1.orientations,
                    w1.fields, w1.polarization)
    w2 = workloads.config2(n_orient=16, n_times=512)
    save_experiment("config2_powder16", w2.spins, w2.couplings, w2.times, w2.orientations,
                    w2.fields, w2.polarization)
    save_experiment("config2_powder8_T10K", w2.spins, w2.couplings, w2.times[:300],
                    w2.orientations[:8], w2.fields, (1.0, 0.0, 0.0), temps=(10.0,))
    w3 = workloads.config3(n_fields=6, n_orient=5)
    save_experiment("config3_alc", w3.spins, w3.couplings, [0.0], w3.orientations,
                    [tuple(f) for f in w3.fields], w3.polarization, y_axis="integral",
                    x_axis="field")
    w5 = workloads.config5(n_orient=24, n_times=300)
    save_experiment("config5_fmuf", w5.spins, w5.couplings, w5.times, w5.orientations,
                    w5.fields, w5.polarization)
    # muon not first (general evolve path), Euler rows with weights, intrinsic field
    rng = np.random.default_rng(77)
    A1 = workloads.random_hyperfine(rng)
    A2 = workloads.random_hyperfine(rng, 5.0)
    save_experiment("e_mu_H_weighted", ["e", "mu", "H"],
                    [("hyperfine", {"i": 2, "j": 1}, A1), ("hyperfine", {"i": 3, "j": 1}, A2)],
                    np.linspace(0, 5, 200),
                    [(0.1, 0.2, 0.3, 1.0), (1.0, 2.0, 0.5, 2.0), (2.5, 0.4, 1.5, 0.5)],
                    [(0.0, 0.01, 0.02)], (1.0, 1.0, 0.0), intrinsic=[(0.0, 0.0, 0.005)])
    # file ranges: field x temperature, time axis (muspinsim/tests/test_experiment.py:269)
    save_experiment("file_ranges", ["e", "mu"], [("zeeman", {"i": 2}, [0, 0, 1.0 / 135.53880943285955])],
                    np.linspace(0, 10, 100), [(0.0, 0.0, 0.0)],
                    [(0.0, 0.0, 0.0), (0.0, 0.0, 10.0)], (1.0, 0.0, 0.0), temps=(np.inf, 0.0))
    save_direct("direct_dim24")
    # Lindblad dissipation on the electron (muspinsim/experiment.py:272-341): finite and
    # infinite temperature (file range), three orientations, powder average
    save_experiment("lindblad_mu_e", ["mu", "e"], [("hyperfine", {"i": 1}, 50.0 * np.eye(3))],
                    np.linspace(0, 2.0, 80),
                    [(0.1, 0.2, 0.3, 1.0), (1.0, 2.0, 0.5, 2.0), (2.5, 0.4, 1.5, 0.5)],
                    [(0.0, 0.0, 0.002)], (1.0, 0.0, 0.0), temps=(np.inf, 20.0),
                    dissipation={2: 3.0})
    save_experiment("lindblad_alc", ["mu", "e"], [("hyperfine", {"i": 1}, 80.0 * np.eye(3))],
                    [0.0], [(0.0, 0.0, 0.0)], [(0.0, 0.0, b) for b in (0.0, 0.002, 0.005)],
                    (0.0, 0.0, 1.0), temps=(5.0,), y_axis="integral", x_axis="field",
                    dissipation={2: 1.5})
    save_lindblad_direct("lindblad_direct")
    save_celio()
    save_config_layouts("config_layouts")
    save_rotated("rotated_dim24")
    save_fast_binding("fast_binding_dim24")
    save_fit("fit_fmuf")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else None)
