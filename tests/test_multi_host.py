"""Host logic of heterogeneous batches and the autotuner (no GPU needed):
plan bucketing, chunking and argument checks through the C ABI, and the
tuner's search and cache."""

import ctypes

import numpy as np
import pytest

from muspinsim_gb300 import _lib, autotune


def _plan(dims, counts, num_times=64, precision=_lib.PREC_MIXED, max_pairs=0, tuning=None):
    lib = _lib.load()
    n = np.ascontiguousarray(dims, dtype=np.int32)
    first = np.ascontiguousarray(np.concatenate([[0], np.cumsum(counts)]), dtype=np.int32)
    d = _lib.MultiDesc()
    d.num_systems = len(dims)
    d.sys_n = n.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
    d.sys_snap_first = first.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
    d.num_times = num_times
    d.uniform = 1
    d.t0, d.dt = 0.0, 0.01
    d.precision = precision
    d.max_pairs_per_chunk = max_pairs
    keep = None
    if tuning:
        keep = (_lib.MultiTuning * len(tuning))(*[_lib.MultiTuning(*t) for t in tuning])
        d.tuning = ctypes.cast(keep, ctypes.POINTER(_lib.MultiTuning))
        d.num_tuning = len(tuning)
    h = ctypes.c_void_p(0)
    rc = lib.msp_multi_plan_create(ctypes.byref(d), ctypes.byref(h))
    return rc, h


def _info(h):
    lib = _lib.load()
    nb = ctypes.c_int(0)
    arr = (_lib.MultiBucketInfo * 16)()
    assert lib.msp_multi_plan_info(h, ctypes.byref(nb), arr, 16) == 0
    return [{f: getattr(arr[i], f) for f, _ in _lib.MultiBucketInfo._fields_}
            for i in range(nb.value)]


def test_plan_buckets_by_dimension():
    lib = _lib.load()
    rc, h = _plan([4, 24, 8, 24, 96, 4], [10, 20, 5, 0, 7, 3])
    assert rc == 0, _lib.last_error()
    info = _info(h)
    by_n = {b["n"]: b for b in info}
    assert sorted(by_n) == [4, 8, 24, 96]
    assert by_n[4]["num_systems"] == 2 and by_n[4]["num_snap"] == 13
    assert by_n[24]["num_systems"] == 2 and by_n[24]["num_snap"] == 20
    assert by_n[96]["num_snap"] == 7
    # launch order: most pair work first
    assert info[0]["n"] == 96
    # mixed precision: FP32 partial sums never hold more than 1024 pairs
    assert all(b["pairs_per_item"] <= 1024 for b in info)
    ws = ctypes.c_size_t(0)
    assert lib.msp_multi_workspace(h, ctypes.byref(ws)) == 0
    assert ws.value >= sum(b["scratch_bytes"] for b in info)
    assert lib.msp_multi_plan_destroy(h) == 0


def test_plan_chunks_split_systems():
    # 24-dim systems (276 pairs) with a budget of 3 snapshots per chunk
    rc, h = _plan([24, 24], [5, 4], max_pairs=3 * 276)
    assert rc == 0
    (b,) = _info(h)
    assert b["num_chunks"] == 3  # 9 snapshots in chunks of 3
    _lib.load().msp_multi_plan_destroy(h)


def test_plan_applies_tuning():
    rc, h = _plan([24, 8], [4, 4], tuning=[(24, 256, 2, 2), (8, 64, 0, 0)])
    assert rc == 0
    by_n = {b["n"]: b for b in _info(h)}
    assert by_n[24]["snap_threads"] == 256
    assert by_n[24]["pairs_per_item"] == 2 * 276
    assert by_n[8]["snap_threads"] == 64
    _lib.load().msp_multi_plan_destroy(h)


@pytest.mark.parametrize("dims,counts,tuning,code", [
    ([5], [3], None, _lib.MSP_ERR_ARG),            # odd n: the muon-first path needs n even
    ([2048], [1], None, _lib.MSP_ERR_UNSUPPORTED),  # beyond the large-n solver
    ([24], [3], [(24, 100, 0, 0)], _lib.MSP_ERR_ARG),  # threads not a multiple of 32
    ([24], [3], [(24, 1024, 0, 0)], _lib.MSP_ERR_ARG),
])
def test_plan_rejects_bad_arguments(dims, counts, tuning, code):
    rc, h = _plan(dims, counts, tuning=tuning)
    assert rc == code
    assert h.value is None or h.value == 0
    assert _lib.last_error()


def test_plan_rejects_decreasing_ranges():
    lib = _lib.load()
    n = np.array([4, 4], dtype=np.int32)
    first = np.array([0, 5, 3], dtype=np.int32)
    d = _lib.MultiDesc()
    d.num_systems = 2
    d.sys_n = n.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
    d.sys_snap_first = first.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
    d.num_times = 8
    d.uniform = 1
    d.dt = 0.1
    h = ctypes.c_void_p(0)
    assert lib.msp_multi_plan_create(ctypes.byref(d), ctypes.byref(h)) == _lib.MSP_ERR_ARG


def test_coordinate_descent_finds_separable_minimum():
    cands = {"a": [0, 1, 2, 3], "b": [10, 20, 30]}
    seen = []

    def measure(p):
        seen.append(dict(p))
        return (p["a"] - 2) ** 2 + (p["b"] - 30) ** 2 * 0.01

    best, t, evals = autotune.coordinate_descent(measure, cands)
    assert best == {"a": 2, "b": 30}
    assert evals == 1 + 3 + 2 == len(seen)


def test_candidates_are_valid_launches():
    for n in (4, 8, 12, 24, 48, 64, 96, 192):
        c = autotune.candidates(n)
        assert c["snap_threads"][0] == 0
        assert all(t == 0 or (t % 32 == 0 and 32 <= t <= 512) for t in c["snap_threads"])
        assert all(0 <= x <= 32 for x in c["ctas_per_sm"])


def test_cache_round_trip(tmp_path, monkeypatch):
    path = str(tmp_path / "sub" / "tune.json")
    monkeypatch.setenv("MSP_AUTOTUNE_CACHE", path)
    assert autotune.cache_path() == path
    assert autotune.load_cache() == {}
    key = autotune.cache_key("GB300", 24, 2048, True, 1, 10000)
    autotune.save_cache({key: {"params": {"snap_threads": 128}}})
    assert autotune.load_cache()[key]["params"]["snap_threads"] == 128
    assert key != autotune.cache_key("GB300", 24, 4096, True, 1, 10000)
