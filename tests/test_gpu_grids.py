"""Orientation grids and the field x orientation product generated on the
device (msp_orient_grid_snapshots): against the host grids
(muspinsim/utils.py:34-50 restated in muspinsim_gb300/orientations.py) fed
through the row kernel, and powder_scan against the reference's ALC field
scan (tests/golden/config3_alc.npz: fields x ZCW orientations, decaying
integral, muspinsim/experiment.py:358-498)."""

import numpy as np
import pytest

from tests.helpers import load_golden

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind,n", [("zcw", 1), ("zcw", 50), ("zcw", 377), ("zcw-hemisphere", 40),
                                    ("eulrange", 1), ("eulrange", 5)])
def test_device_grid_matches_host_rows(kind, n):
    from muspinsim_gb300 import kernels
    from muspinsim_gb300.powder import OrientationGrid

    grid = OrientationGrid(kind, n)
    fields = np.array([[0.0, 0.0, 0.01], [0.003, -0.002, 0.02], [0.0, 0.0, 0.0]])
    p, intr = np.array([0.6, 0.0, 0.8]), np.array([0.0, 0.001, 0.0])
    F, P, W, slot = kernels.orient_grid_snapshots(kind, n, fields, p, intr)
    F, P, W, slot = (x.cpu().numpy() for x in (F, P, W, slot))
    rows = grid.rows()
    No = len(rows)
    assert F.shape == (3 * No, 3) and np.array_equal(slot, np.repeat(np.arange(3), No))
    for f in range(3):
        Fr, Pr, Wr = (x.cpu().numpy() for x in kernels.orient_snapshots(rows, fields[f], p, intr))
        sl = slice(f * No, (f + 1) * No)
        assert np.abs(F[sl] - Fr).max() <= 1e-14
        assert np.abs(P[sl] - Pr).max() <= 1e-14
        assert np.abs(W[sl] - Wr).max() <= 1e-15
    assert abs(W[:No].sum() - 1.0) <= 1e-12


def test_powder_scan_matches_reference_alc():
    from muspinsim_gb300 import workloads
    from muspinsim_gb300.powder import OrientationGrid, powder_scan

    g = load_golden("config3_alc")
    wl = workloads.config3(n_fields=6, n_orient=5)
    assert np.allclose(wl.orientations, g["orientations"], rtol=0, atol=1e-15)
    sy = wl.system()
    for prec, tol in (("fp64", 1e-10), ("mixed", 1e-6)):
        got = powder_scan(sy, OrientationGrid("zcw", 5), g["fields"], g["polarization"],
                          y_axis="integral", precision=prec)
        assert got.shape == g["result"].shape
        assert np.abs(got - g["result"]).max() <= tol
        rows = powder_scan(sy, g["orientations"], g["fields"], g["polarization"],
                           y_axis="integral", precision=prec)
        # the device grid and the host rows agree to ~1e-16 rad; integrals
        # at a level anticrossing amplify that, within the precision's gate
        assert np.abs(rows - got).max() <= tol


def test_powder_average_with_grid():
    from muspinsim_gb300 import workloads
    from muspinsim_gb300.powder import OrientationGrid, powder_average

    wl = workloads.config2(n_orient=30, n_times=200)
    sy = wl.system()
    grid = OrientationGrid("zcw", 30)
    a = powder_average(sy, grid, wl.fields[0], wl.polarization, wl.times)
    b = powder_average(sy, grid.rows(), wl.fields[0], wl.polarization, wl.times)
    assert np.abs(a - b).max() <= 1e-12
    e = OrientationGrid("eulrange", 3)
    a = powder_average(sy, e, wl.fields[0], wl.polarization, wl.times, temperature=20.0)
    b = powder_average(sy, e.rows(), wl.fields[0], wl.polarization, wl.times, temperature=20.0)
    assert np.abs(a - b).max() <= 1e-10
