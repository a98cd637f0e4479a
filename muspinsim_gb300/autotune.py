"""Autotuner for the launch parameters of heterogeneous batches.

For every Hilbert dimension of a batch it times ``msp_multi_run`` on a
sample of that dimension's snapshots under candidate parameters -- threads
per snapshot CTA (the Jacobi block size), persistent CTAs per SM, snapshots
per phase-sum work item -- by coordinate descent (one parameter at a time,
the others at their best so far), with CUDA events on the launch stream.
The winners are cached in a JSON file keyed by GPU, dimension, time-grid
length, precision and library version, so a dimension is tuned once per
machine.  The reference has no counterpart (it runs on the CPU with fixed
OpenMP scheduling, muspinsim/cython/parallel.pyx:59).
"""

import json
import os
import statistics
import threading

import numpy as np

# bump when a kernel change invalidates cached choices
TUNER_VERSION = 1

_lock = threading.Lock()


def cache_path():
    """The tuning cache: $MSP_AUTOTUNE_CACHE, else
    ~/.cache/muspinsim_gb300/autotune.json."""
    p = os.environ.get("MSP_AUTOTUNE_CACHE")
    if p:
        return p
    return os.path.join(os.path.expanduser("~"), ".cache", "muspinsim_gb300", "autotune.json")


def load_cache(path=None):
    path = path or cache_path()
    try:
        with open(path) as f:
            data = json.load(f)
        return data if isinstance(data, dict) else {}
    except (OSError, ValueError):
        return {}


def save_cache(data, path=None):
    """Write the cache atomically (write a temporary file, then rename)."""
    path = path or cache_path()
    d = os.path.dirname(path)
    if d:
        os.makedirs(d, exist_ok=True)
    tmp = f"{path}.{os.getpid()}.tmp"
    with open(tmp, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def cache_key(device_name, n, num_times, uniform, precision, lib_version):
    return (f"{device_name}|n={n}|T={num_times}|uniform={int(uniform)}|prec={int(precision)}"
            f"|lib={lib_version}|tuner={TUNER_VERSION}")


def candidates(n):
    """Candidate values per parameter for dimension n (first = default)."""
    if n > 64:  # default: 128 threads, as many CTAs per SM as fit
        return {"snap_threads": [0, 64, 256], "ctas_per_sm": [0, 2, 4, 8],
                "snaps_per_item": [0]}
    m = n + (n & 1)
    base = 32 if m <= 8 else 64 if m <= 16 else 128 if m <= 32 else 256
    threads = [0] + sorted({t for t in (base // 2, base, 2 * base, 3 * base // 2)
                            if 32 <= t <= 512 and t % 32 == 0 and t != base})
    return {"snap_threads": threads, "ctas_per_sm": [0, 2, 4],
            "snaps_per_item": [0, 1, 4, 16]}


def coordinate_descent(measure, cands):
    """Minimise measure(params) over the candidate grid one parameter at a
    time (in the order of ``cands``), starting from the first candidate of
    each.  Returns (best params, best time, evaluations)."""
    best = {k: v[0] for k, v in cands.items()}
    best_t = measure(dict(best))
    evals = 1
    for key, vals in cands.items():
        for v in vals[1:]:
            trial = dict(best)
            trial[key] = v
            t = measure(trial)
            evals += 1
            if t < best_t:
                best, best_t = trial, t
    return best, best_t, evals


def _sample(first, systems, budget):
    """Systems (indices) of one dimension whose snapshots fill about
    ``budget`` snapshots, and their prefix."""
    chosen, acc = [], 0
    for k in systems:
        cnt = int(first[k + 1] - first[k])
        if cnt == 0:
            continue
        chosen.append(k)
        acc += cnt
        if acc >= budget:
            break
    return chosen


def tune_multi(Hs, Zs, field, pol, wscale, first, times, precision, cache=True, repeats=3,
               sample_snapshots=None, path=None):
    """Tuning entries (list of dicts for ``MultiPlan``) for the dimensions
    of a batch, from the cache where present, else measured now."""
    import torch

    from muspinsim_gb300 import _lib, kernels

    kernels.device()
    lib = _lib.load()
    dev = torch.cuda.current_device()
    props = torch.cuda.get_device_properties(dev)
    name = props.name
    sms = props.multi_processor_count
    dims = np.array([h.shape[-1] for h in Hs])
    first = np.asarray(first)
    th = np.asarray(times, dtype=float)
    uni = kernels.uniform_grid(th)[0]
    version = lib.msp_version()
    with _lock:
        data = load_cache(path) if cache else {}
    out, dirty = [], False
    for n in sorted(set(dims.tolist())):
        key = cache_key(name, n, th.size, uni, precision, version)
        if key in data:
            out.append(dict(data[key]["params"], n=int(n)))
            continue
        systems = [k for k in range(len(Hs)) if dims[k] == n]
        budget = sample_snapshots or (2 * sms if n > 64 else 8 * sms)
        chosen = _sample(first, systems, budget)
        if not chosen:
            continue
        sub_first = [0]
        idx = []
        for k in chosen:
            idx.extend(range(int(first[k]), int(first[k + 1])))
            sub_first.append(len(idx))
        idx = np.array(idx)
        sub = ([Hs[k] for k in chosen], [Zs[k] for k in chosen], field[idx], pol[idx],
               wscale[idx], np.array(sub_first, dtype=np.int32))

        def measure(params, sub=sub, n=n):
            tun = [dict(params, n=int(n))]
            plan = kernels.MultiPlan(*sub, th, precision=precision, tuning=tun)
            stream = torch.cuda.current_stream()
            plan.run()
            ts = []
            for _ in range(repeats):
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                plan.run()
                e1.record(stream)
                e1.synchronize()
                ts.append(e0.elapsed_time(e1))
            plan.close()
            return statistics.median(ts)

        best, best_t, evals = coordinate_descent(measure, candidates(int(n)))
        data[key] = {"params": best, "ms": best_t, "evaluations": evals,
                     "sample_snapshots": int(sub_first[-1])}
        dirty = True
        out.append(dict(best, n=int(n)))
    if cache and dirty:
        with _lock:
            merged = load_cache(path)
            merged.update(data)
            try:
                save_cache(merged, path)
            except OSError:
                pass
    return out
