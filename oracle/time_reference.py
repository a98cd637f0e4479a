"""Times the reference's own ExperimentRunner.run() against the CPU-baseline
loop that bench.py runs on the GPU host (numpy eigh per orientation plus the
reference's compiled Cython cosine sum), on the same orientations of the
dim-24 powder workload, and prints both rates and their results' largest
difference.

The reference is Python and cannot travel to the GPU host, so the timed
baseline there is that loop; this script, run where the reference tree is
(python oracle/time_reference.py [orientations] [times]), shows how close
the loop's rate is to the reference's own driver on one machine.  It
imports the reference through tests/golden/refshim.py and is test
infrastructure, like the oracle.
"""

import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))


def main(n_orient=100, n_times=4096):
    import argparse

    import refshim

    import bench

    refshim.install()
    from muspinsim.experiment import ExperimentRunner

    threads = os.cpu_count() or 1
    os.environ["OMP_NUM_THREADS"] = str(threads)
    args = argparse.Namespace(orientations=n_orient, times=n_times)
    wl, sy, B_lab, p_lab, wscale = bench.build_workload(args)
    p = refshim.make_params(wl.spins, wl.couplings, wl.times, wl.orientations,
                            field=[wl.fields[0]], polarization=wl.polarization)
    runner = ExperimentRunner(refshim.ParamsInput(p))
    t0 = time.perf_counter()
    ref = np.asarray(runner.run())
    t_ref = time.perf_counter() - t0
    rate, t_loop, kind, avg = bench.cpu_reference_rate(sy, B_lab, p_lab, wl.times, n_orient,
                                                       threads, wscale)
    out = {"orientations": n_orient, "times": n_times, "threads": threads,
           "cpu_model": bench.cpu_model(),
           "reference_experimentrunner_samples_per_s": n_orient * n_times / t_ref,
           "baseline_loop_samples_per_s": rate, "baseline_kind": kind,
           "loop_over_reference": (n_orient * n_times / t_ref) and rate / (n_orient * n_times / t_ref),
           "max_abs_dP_loop_vs_reference": float(np.abs(avg - ref).max())}
    print(json.dumps(out, indent=1))
    return out


if __name__ == "__main__":
    main(*(int(x) for x in sys.argv[1:3]))
