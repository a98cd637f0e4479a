"""GPU parity of heterogeneous batches (msp_multi_*) against the oracle.

Every row of a batch of systems with uneven dimension (4 ... 96, the Jacobi
and the Householder eigensolvers both in play) must equal the oracle's
powder average of that system alone: FP64 max|dP| <= 1e-10, mixed <= 1e-6.
Graph replay, chunking (a system split across chunks) and non-default
launch parameters must not change the result beyond rounding.
"""

import numpy as np
import pytest

from tests.helpers import oracle_powder

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10
MIXED_TOL = 1e-6


def _batch(seed=41, n_orient=6, n_times=300, dims=(4, 8, 12, 24, 48, 96)):
    from muspinsim_gb300 import workloads
    from muspinsim_gb300.orientations import zcw_gen

    rng = np.random.default_rng(seed)
    orients = zcw_gen(n_orient)
    times = np.linspace(0.0, 8.0, n_times)
    # every dimension once, then a few repeats so buckets hold several systems
    order = list(dims) + [24, 4, 8]
    return [workloads.random_system_workload(rng, d, orients, times) for d in order]


@pytest.fixture(scope="module")
def batch():
    wls = _batch()
    refs = [oracle_powder(w) for w in wls]
    return wls, refs


@pytest.mark.parametrize("precision,tol", [("fp64", FP64_TOL), ("mixed", MIXED_TOL)])
def test_multi_matches_oracle(batch, precision, tol):
    from muspinsim_gb300.multi import powder_average_multi

    wls, refs = batch
    got = powder_average_multi([w.system() for w in wls], wls[0].orientations,
                               field=wls[0].fields[0], polarization=wls[0].polarization,
                               times=wls[0].times, precision=precision)
    assert got.shape == (len(wls), len(wls[0].times))
    for k, (w, ref) in enumerate(zip(wls, refs)):
        err = np.abs(got[k] - ref).max()
        assert err <= tol, (k, w.name, err)


def test_multi_graph_chunks_and_tuning_agree(batch):
    from muspinsim_gb300.multi import MultiSystemBatch

    wls, refs = batch
    args = ([w.system() for w in wls], wls[0].orientations, wls[0].fields[0],
            wls[0].polarization, wls[0].times)
    base = MultiSystemBatch(*args, precision="fp64")
    r0 = base.result()
    g1 = base.result(graph=True)
    g2 = base.result(graph=True)  # replay of the captured graph
    assert np.abs(g1 - r0).max() <= 1e-13
    assert np.abs(g2 - r0).max() <= 1e-13
    # a 300-pair chunk budget splits every dimension >= 32 snapshot by snapshot
    # and the small ones across chunks
    chunked = MultiSystemBatch(*args, precision="fp64", max_pairs_per_chunk=300)
    info = chunked.plan.info()
    assert any(b["num_chunks"] > 1 for b in info)
    assert np.abs(chunked.result() - r0).max() <= 1e-12
    tuned = MultiSystemBatch(*args, precision="fp64", tuning=[
        {"n": 4, "snap_threads": 64, "ctas_per_sm": 1, "snaps_per_item": 1},
        {"n": 24, "snap_threads": 256, "ctas_per_sm": 2, "snaps_per_item": 3},
        {"n": 96, "snap_threads": 128, "ctas_per_sm": 2},
    ])
    assert np.abs(tuned.result() - r0).max() <= 1e-12
    for k, ref in enumerate(refs):
        assert np.abs(r0[k] - ref).max() <= FP64_TOL


def test_multi_mixed_graph_and_status(batch):
    from muspinsim_gb300.multi import MultiSystemBatch

    wls, refs = batch
    b = MultiSystemBatch([w.system() for w in wls], wls[0].orientations, wls[0].fields[0],
                         wls[0].polarization, wls[0].times, precision="mixed")
    r = b.result(graph=True)
    st = b.plan.status[:b.plan.num_snap].cpu().numpy()
    assert np.all(st == 0)
    for k, ref in enumerate(refs):
        assert np.abs(r[k] - ref).max() <= MIXED_TOL


def test_multi_per_system_orientations_and_empty_rows():
    from muspinsim_gb300.multi import powder_average_multi
    from muspinsim_gb300.orientations import zcw_gen
    from muspinsim_gb300 import workloads

    rng = np.random.default_rng(5)
    times = np.linspace(0.0, 5.0, 128)
    o1, o2 = zcw_gen(3), zcw_gen(10)
    w1 = workloads.random_system_workload(rng, 8, o1, times)
    w2 = workloads.random_system_workload(rng, 12, o2, times)
    got = powder_average_multi([w1.system(), w2.system()], [o1, o2], field=w1.fields[0],
                               polarization=w1.polarization, times=times, precision="fp64")
    assert np.abs(got[0] - oracle_powder(w1)).max() <= FP64_TOL
    assert np.abs(got[1] - oracle_powder(w2)).max() <= FP64_TOL


def test_autotune_caches_choices(tmp_path, monkeypatch, batch):
    import os

    from muspinsim_gb300 import autotune
    from muspinsim_gb300.multi import MultiSystemBatch

    wls, _ = batch
    sub = [w for w in wls if len(w.spins) <= 3][:3]  # dimensions 4, 8, 12
    path = str(tmp_path / "tune.json")
    monkeypatch.setenv("MSP_AUTOTUNE_CACHE", path)
    args = ([w.system() for w in sub], sub[0].orientations, sub[0].fields[0],
            sub[0].polarization, sub[0].times)
    b = MultiSystemBatch(*args, precision="mixed", tuning="auto")
    data = autotune.load_cache(path)
    dims = sorted({w.system().hamiltonian_matrix().shape[0] for w in sub})
    assert len(data) == len(dims)
    assert sorted(t["n"] for t in b.tuning) == dims
    res = b.result()
    for k, w in enumerate(sub):
        assert np.abs(res[k] - oracle_powder(w)).max() <= MIXED_TOL
    # a second batch reads the cache instead of measuring again
    mtime = os.path.getmtime(path)
    b2 = MultiSystemBatch(*args, precision="mixed", tuning="auto")
    assert os.path.getmtime(path) == mtime
    assert b2.tuning == b.tuning


@pytest.mark.parametrize("precision,tol", [("fp64", FP64_TOL), ("mixed", MIXED_TOL)])
def test_multi_with_dim192_systems(precision, tol):
    """Two 192-dimensional systems (the blocked FP32 reduction of the mixed
    large-n kernel) between smaller ones, as multi-system segments."""
    from muspinsim_gb300.multi import powder_average_multi

    wls = _batch(seed=192, n_orient=3, n_times=200, dims=(192, 24, 192, 96))[:4]
    refs = [oracle_powder(w) for w in wls]
    got = powder_average_multi([w.system() for w in wls], wls[0].orientations,
                               field=wls[0].fields[0], polarization=wls[0].polarization,
                               times=wls[0].times, precision=precision)
    for k, (w, ref) in enumerate(zip(wls, refs)):
        err = np.abs(got[k] - ref).max()
        assert err <= tol, (k, w.name, err)


def test_multi_buckets_through_the_ql_eigensolve():
    """Buckets of 4,500 snapshots (three systems x 1,500 orientations each,
    interleaved with the other bucket's systems in the input) take the
    batched Householder + QL first stage, whose four-matrix warp tasks then
    straddle segment boundaries: mixed rows against the FP64 rows."""
    from muspinsim_gb300 import workloads
    from muspinsim_gb300.multi import powder_average_multi
    from muspinsim_gb300.orientations import zcw_gen

    rng = np.random.default_rng(77)
    orients = zcw_gen(1500)
    times = np.linspace(0.0, 8.0, 32)
    wls = [workloads.random_system_workload(rng, d, orients, times) for d in (8, 24, 8, 24, 8, 24)]
    systems = [w.system() for w in wls]
    kw = dict(field=wls[0].fields[0], polarization=wls[0].polarization, times=times)
    fp64 = powder_average_multi(systems, orients, precision="fp64", **kw)
    mixed = powder_average_multi(systems, orients, precision="mixed", **kw)
    err = np.abs(mixed - fp64).max(axis=1)
    print("QL buckets: per-system max|dP| mixed vs FP64:", err)
    assert err.max() <= MIXED_TOL
