"""Shared test helpers: oracle systems built from the same inputs the GPU
library receives, and random Hermitian matrices."""

import json
import os

import numpy as np

from muspinsim_gb300 import constants as C
from oracle import port


def oracle_system(spins, couplings):
    """oracle.port.System for a spin list and input-file style couplings."""
    gam, Is, Qs = [], [], []
    for s in spins:
        el, iso = s if isinstance(s, tuple) else (s, None)
        gam.append(C.gyromagnetic_ratio(el, iso))
        Is.append(C.spin(el, iso))
        Qs.append(C.quadrupole_moment(el, iso))
    sy = port.System(spins, gam, Is, Qs)
    for kind, args, val in couplings:
        i = args["i"] - 1
        j = args.get("j")
        j = None if j is None else j - 1
        if kind == "hyperfine":
            if j is None:
                j = spins.index("e")
            sy.add_hyperfine(i, val, j)
        elif kind == "dipolar":
            sy.add_dipolar(i, j, val)
        elif kind == "quadrupolar":
            sy.add_quadrupolar(i, val)
        elif kind == "zeeman":
            sy.add_zeeman(i, val)
        else:
            raise ValueError(kind)
    return sy


def oracle_powder(wl, orientations=None, times=None, field=None, temperature=None,
                  y_axis=None):
    """Oracle powder average of a muspinsim_gb300.workloads.Workload."""
    sy = oracle_system(wl.spins, wl.couplings)
    o = wl.orientations if orientations is None else orientations
    t = wl.times if times is None else times
    B = wl.fields[0] if field is None else field
    T = wl.temperature if temperature is None else temperature
    y = wl.y_axis if y_axis is None else y_axis
    p = wl.polarization / np.linalg.norm(wl.polarization)
    return port.powder_average(sy, o, np.asarray(B, float), p, T, t, y=y)


GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load_golden(name):
    """A fixture written by tests/golden/make_golden.py: the meta JSON
    unpacked (spins, couplings with numpy tensors, axes) plus the arrays."""
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    out = {k: z[k] for k in z.files if k != "meta"}
    if "meta" in z.files:
        meta = json.loads(str(z["meta"]))
        meta["couplings"] = [(k, {kk: int(vv) for kk, vv in a.items()}, np.array(v))
                             for k, a, v in meta["couplings"]]
        out.update(meta)
    return out


def golden_oracle(g, field_index=0, temp_index=0):
    """Oracle evaluation of one (field, temperature) row of a golden fixture."""
    sy = oracle_system(g["spins"], g["couplings"])
    p = g["polarization"] / np.linalg.norm(g["polarization"])
    B = g["fields"][field_index]
    if B.size == 1:
        B = np.array([0.0, 0.0, B[0]])
    intr = g["intrinsic"][0]
    if intr.size == 1:
        intr = np.array([0.0, 0.0, intr[0]])
    y = "integral" if g["y_axis"] == "integral" else "asymmetry"
    diss = {int(k) - 1: float(v) for k, v in g.get("dissipation", {}).items()} or None
    celio = tuple(g.get("celio") or (0, 0))
    phases = None
    if celio[0] and celio[1]:
        phases = celio_phases(g["seed"], len(g["orientations"]), celio[1], sy.n // 2)
    return port.powder_average(sy, list(g["orientations"]), B, p, g["temperatures"][temp_index],
                               g["times"], intrinsic_B=intr, y=y, dissipation=diss, celio=celio,
                               phases=phases)


def celio_phases(seed, snapshots, averages, half):
    """The uniform numbers the reference draws for Celio's random initial
    states after np.random.seed(seed): np.random.rand(half) per snapshot and
    average, in that order (muspinsim/celio.py:295-316, 471)."""
    rs = np.random.RandomState(seed)
    return rs.random_sample(snapshots * averages * half).reshape(snapshots, averages, half)


def random_hermitian(rng, n, scale=100.0):
    A = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
    return scale * (A + A.conj().T) / 2.0
