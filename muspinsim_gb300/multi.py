"""Powder averages of many spin systems of uneven dimension in one GPU batch.

The reference evaluates one spin system per ``ExperimentRunner`` and one
snapshot at a time (muspinsim/experiment.py:358-498); comparing candidate
muon sites, isotopologues or coupling sets means running that loop once per
system.  ``MultiSystemBatch`` hands all of them to ``msp_multi_run``: systems
are bucketed by Hilbert dimension, each bucket runs as one persistent launch
over all its snapshots, buckets run concurrently, and the launch sequence can
be replayed from a CUDA graph.  Every system gets its own output row, the
orientation-weighted mean of the reference (muspinsim/simconfig.py:152-159,
347-368).

Scope: the muon-first, T = inf path that ``ExperimentRunner`` picks by
default (``Hamiltonian.fast_evolve``, muspinsim/hamiltonian.py:166-217).
"""

import numpy as np
import torch

from muspinsim_gb300 import _lib, kernels
from muspinsim_gb300 import quaternion as Q
from muspinsim_gb300.orientations import orientation_rows_to_quats
from muspinsim_gb300.powder import precision_code


def _as_field(field):
    f = np.atleast_1d(np.asarray(field, dtype=float))
    if f.size == 1:
        f = np.array([0.0, 0.0, f[0]])
    return f


class MultiSystemBatch:
    """Device-resident batch of spin systems x orientations.

    ``systems``: MuonSpinSystem objects with the muon first.
    ``orientations``: one array of orientation rows shared by all systems,
    or a list with one array per system (rows as in the reference's
    ``orientation`` keyword: (theta, phi), (a, b, c) or (a, b, c, w)).
    ``field``: one 3-vector (or a scalar along z, T) for all systems, or one
    per system.  ``tuning``: None, a list of per-dimension dicts (see
    ``MultiPlan``), or ``"auto"`` to run the autotuner (results cached on
    disk).
    """

    def __init__(self, systems, orientations, field=(0.0, 0.0, 0.0),
                 polarization=(1.0, 0.0, 0.0), times=None, intrinsic_field=(0.0, 0.0, 0.0),
                 precision="mixed", mode="zyz", tuning=None, max_pairs_per_chunk=0,
                 max_sweeps=0):
        systems = list(systems)
        if not systems:
            raise ValueError("MultiSystemBatch: no systems")
        for k, sy in enumerate(systems):
            if sy.muon_index != 0:
                raise ValueError(
                    f"MultiSystemBatch: system {k} has the muon at index {sy.muon_index}; "
                    "the batched fast path needs the muon first")
        ns = len(systems)
        if isinstance(orientations, (list, tuple)) and len(orientations) == ns and \
                all(np.ndim(o) == 2 for o in orientations):
            orients = [np.asarray(o, dtype=float) for o in orientations]
        else:
            orients = [np.asarray(orientations, dtype=float)] * ns
        fields = np.asarray(field, dtype=float)
        if fields.ndim == 2 and fields.shape[0] == ns:
            fields = [_as_field(f) for f in fields]
        else:
            fields = [_as_field(field)] * ns
        p = np.asarray(polarization, dtype=float)
        p = p / np.linalg.norm(p)
        intr = _as_field(intrinsic_field)
        B_all, p_all, w_all, first = [], [], [], [0]
        for k in range(ns):
            qs, ws = orientation_rows_to_quats(orients[k], mode)
            N = len(qs)
            ws = ws * (N / ws.sum()) if N > 1 else np.ones(N)
            B_all.append(Q.rotate(qs, fields[k]) + intr)
            p_all.append(Q.rotate(qs, p))
            w_all.append(ws / N)
            first.append(first[-1] + N)
        self.systems = systems
        self.times = np.asarray(times, dtype=float)
        self.precision = precision_code(precision)
        Hs = [sy.hamiltonian_matrix() for sy in systems]
        Zs = [sy.zeeman_operators() for sy in systems]
        if isinstance(tuning, str) and tuning == "auto":
            from muspinsim_gb300 import autotune

            tuning = autotune.tune_multi(Hs, Zs, np.concatenate(B_all), np.concatenate(p_all),
                                         np.concatenate(w_all), np.array(first), self.times,
                                         self.precision)
        self.tuning = tuning
        self.plan = kernels.MultiPlan(Hs, Zs, np.concatenate(B_all), np.concatenate(p_all),
                                      np.concatenate(w_all), np.array(first, dtype=np.int32),
                                      self.times, precision=self.precision, tuning=tuning,
                                      max_pairs_per_chunk=max_pairs_per_chunk,
                                      max_sweeps=max_sweeps)

    def run(self, graph=False):
        """Enqueue the batch; returns the (num_systems, len(times)) device tensor."""
        return self.plan.run(graph=graph)

    def result(self, graph=False):
        """Run and return the powder averages as a float64 numpy array; raises
        if an eigensolve hit its sweep cap."""
        out = self.run(graph=graph)
        res = out.cpu().numpy()
        st = self.plan.status[:self.plan.num_snap]
        if self.plan.num_snap and int(st.max().item()) & _lib.MSP_ITEM_NOT_CONVERGED:
            raise RuntimeError("MultiSystemBatch: an eigensolve reached its sweep cap")
        return res


def powder_average_multi(systems, orientations, field=(0.0, 0.0, 0.0),
                         polarization=(1.0, 0.0, 0.0), times=None,
                         intrinsic_field=(0.0, 0.0, 0.0), precision="mixed", mode="zyz",
                         graph=False, tuning=None, max_pairs_per_chunk=0, max_sweeps=0):
    """Orientation-averaged muon polarisation of several systems at once:
    a (len(systems), len(times)) float64 array, row k for systems[k]."""
    batch = MultiSystemBatch(systems, orientations, field, polarization, times, intrinsic_field,
                             precision, mode, tuning, max_pairs_per_chunk, max_sweeps)
    res = batch.result(graph=graph)
    batch.plan.close()
    torch.cuda.current_stream().synchronize()
    return res
