"""The host side of the drop-in boundary against fixtures made by running
the reference itself (tests/golden/make_golden.py):

* MuSpinConfig: snapshot grid, result shape, range order, constants,
  orientation quaternions and weights for four axis layouts
  (muspinsim/simconfig.py:78-321), and the .dat files save_output writes
  (muspinsim/simconfig.py:370-429) byte for byte apart from the date line;
* SpinSystem.rotate(R).hamiltonian on the host
  (muspinsim/spinsys.py:103-135, 594-626).
"""

import json
import os
import tempfile

import numpy as np

from tests.helpers import GOLDEN


def _layouts():
    with open(os.path.join(GOLDEN, "config_layouts.json")) as f:
        return json.load(f)


def _config(g, layout):
    from muspinsim_gb300.simconfig import MuSpinConfig, make_params

    times, orients, fields, temps, y, x, avg = layout
    couplings = [(k, a, np.array(v)) for k, a, v in g["couplings"]]
    p = make_params(spins=g["spins"], couplings=couplings, time=times, orientation=orients,
                    field=fields, polarization=[(1.0, 0.0, 0.0)], temperature=temps,
                    y_axis=y, x_axis=x, average_axes=avg)
    return MuSpinConfig(p)


def test_config_layouts_match_reference():
    g = _layouts()
    for ref in g["layouts"]:
        cfg = _config(g, ref["layout"])
        got = [[[None if isinstance(i, slice) else int(i) for i in part] for part in c]
               for c in cfg.configurations]
        assert got == ref["configurations"]
        assert list(cfg.results.shape) == ref["shape"]
        assert list(cfg.file_ranges.keys()) == ref["file_ranges"]
        assert list(cfg.avg_ranges.keys()) == ref["avg_ranges"]
        assert cfg.x_axis == ref["x"]
        assert cfg.avg_N == ref["avg_N"] and cfg.time_N == ref["time_N"]
        assert sorted(cfg.constants.keys()) == ref["constants"]
        for k, (q, w) in enumerate(ref["orient"]):
            o = cfg[k].orient
            qq = np.asarray(o[0].q)
            # a quaternion and its negative are the same rotation
            assert min(np.abs(qq - q).max(), np.abs(qq + q).max()) <= 1e-14
            assert abs(o[1] - w) <= 1e-14


def test_save_output_matches_reference_writer():
    g = _layouts()
    for ref in g["layouts"]:
        cfg = _config(g, ref["layout"])
        cfg.results = np.arange(cfg.results.size, dtype=float).reshape(cfg.results.shape) * 0.25
        with tempfile.TemporaryDirectory() as d:
            cfg.save_output(name="out", path=d)
            names = sorted(os.listdir(d))
            assert names == sorted(ref["files"].keys())
            for fn in names:
                with open(os.path.join(d, fn)) as f:
                    lines = f.read().splitlines()
                lines = [("# Output file written on <date>" if ln.startswith(
                    "# Output file written on") else ln) for ln in lines]
                assert lines == ref["files"][fn], fn


def test_rotate_host_matches_reference():
    from muspinsim_gb300 import workloads

    z = np.load(os.path.join(GOLDEN, "rotated_dim24.npz"))
    meta = json.loads(str(z["meta"]))
    wl = workloads.config2(n_orient=1, n_times=8)
    assert list(wl.spins) == meta["spins"]
    for (k, a, v), (k2, a2, v2) in zip(wl.couplings, meta["couplings"]):
        assert k == k2 and dict(a) == a2 and np.allclose(np.asarray(v, float), v2, rtol=0, atol=0)
    sy = wl.system()
    scale = np.abs(z["H"]).max()
    assert np.abs(sy.hamiltonian_matrix() - z["H"]).max() <= 1e-12 * scale
    for R, HR in zip(z["R"], z["HR"]):
        assert np.abs(sy.rotate(R).hamiltonian_matrix() - HR).max() <= 1e-12 * scale


def test_fit_config_uses_experimental_axis():
    """Fitting (muspinsim/simconfig.py:180-233): the x axis becomes the
    data's first column; file ranges are refused; FittingVariable checks
    its bounds (muspinsim/input/variables.py:4-40)."""
    import pytest

    from muspinsim_gb300.fitting import FitInput, FittingVariable
    from muspinsim_gb300.simconfig import MuSpinConfig, MuSpinConfigError, make_params

    data = np.stack([np.linspace(0, 5, 11), np.zeros(11)], axis=1)

    def build(a):
        return make_params(spins=["mu", "e"], couplings=[("hyperfine", {"i": 1}, a * np.eye(3))],
                           time=np.linspace(0, 1, 3))

    inp = FitInput(build, [FittingVariable("a", 10.0, 0.0, 50.0)], data)
    cfg = MuSpinConfig(inp.evaluate(a=10.0))
    assert np.allclose(cfg.x_axis_values, data[:, 0]) and cfg.time_N == 11
    bad = dict(inp.evaluate(a=10.0))
    bad.update(make_params(spins=["mu", "e"], time=np.linspace(0, 1, 3),
                           field=[0.0, 0.01]))  # a field file range
    bad["fitting_info"] = inp.fitting_info
    with pytest.raises(MuSpinConfigError, match="file ranges"):
        MuSpinConfig(bad)
    with pytest.raises(ValueError, match="invalid range"):
        FittingVariable("b", 1.0, 2.0, 1.0)
    with pytest.raises(ValueError, match="starting value"):
        FittingVariable("b", 3.0, 0.0, 1.0)
