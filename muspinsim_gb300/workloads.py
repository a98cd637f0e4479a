"""Seeded synthetic workloads with the shapes of the benchmark configurations.

No public dataset is involved: each configuration is a spin system with
random couplings drawn from a fixed ``numpy.random.default_rng(seed)``,
plus its orientation grid, field(s) and time axis.  The same objects feed the
GPU library and the CPU oracle, so both see identical inputs.

* ``config1`` -- mu + e (dim 4), isotropic hyperfine A ~ U(100, 500) MHz,
  B = 0.01 T along z, one orientation, p = z, 1000 times on 0-10 us.
* ``config2`` -- mu, e, 1H, 14N (dim 24): anisotropic hyperfine
  Q diag(N(0, 50)) Q^T (Haar Q) for mu, H and N; point dipoles between the
  non-electron spins at random distances U(1, 3) A; 14N quadrupole from a
  random traceless EFG with |V_zz| ~ U(0.1, 1) a.u.; ZCW-style grid of
  10,000 orientations; 4096 times on 0-20 us; B = 0.01 T along z, p = z.
* ``config3`` -- mu, e, 1H x 3 (dim 32), random anisotropic hyperfine,
  2,000 fields on 0-1 T x 1,000 orientations, decaying integral (ALC).
* ``config5`` -- mu, 19F, 19F (dim 8), dipoles at U(1.0, 1.4) A,
  2,000 orientations, 1000 times on 0-20 us.
* ``celio_v3si`` -- Celio's method on mu + 4 51V (I = 7/2, dim
  2 x 8^4 = 8192), the shape of the reference's Celio example: mu-V point
  dipoles at U(1.6, 2.0) A, random traceless V EFGs with |V_zz| ~
  U(0.02, 0.06) a.u., zero field, ZCW orientations (only the polarisation
  turns), k = 10, random initial states averaged, 50 times on 0-10 us.
"""

from dataclasses import dataclass, field
from typing import List, Tuple

import numpy as np

from muspinsim_gb300.orientations import zcw_gen


@dataclass
class Workload:
    name: str
    spins: List
    # (kind, {"i": 1-based, "j": 1-based}, value) exactly as input-file couplings
    couplings: List[Tuple[str, dict, np.ndarray]]
    orientations: np.ndarray  # rows (theta, phi) or (a, b, c[, w])
    fields: np.ndarray  # (F, 3) lab-frame fields (T)
    polarization: np.ndarray  # (3,)
    times: np.ndarray
    temperature: float = np.inf
    y_axis: str = "asymmetry"
    x_axis: str = "time"
    meta: dict = field(default_factory=dict)

    @property
    def num_orientations(self):
        return len(self.orientations)

    def system(self, celio_k=0):
        """The workload's MuonSpinSystem (muspinsim_gb300.spinsys)."""
        from muspinsim_gb300.spinsys import MuonSpinSystem

        sy = MuonSpinSystem(list(self.spins), celio_k)
        for kind, args, val in self.couplings:
            i = args["i"] - 1
            j = args.get("j")
            j = None if j is None else j - 1
            if kind == "hyperfine":
                sy.add_hyperfine_term(i, val, j)
            elif kind == "dipolar":
                sy.add_dipolar_term(i, j, val)
            elif kind == "quadrupolar":
                sy.add_quadrupolar_term(i, val)
            elif kind == "zeeman":
                sy.add_zeeman_term(i, val)
            else:
                raise ValueError(kind)
        return sy


def _haar(rng):
    Qm, R = np.linalg.qr(rng.normal(size=(3, 3)))
    return Qm * np.sign(np.diag(R))


def random_hyperfine(rng, sigma=50.0):
    """Symmetric 3x3 with eigenvalues ~ N(0, sigma) MHz in a Haar frame."""
    Qm = _haar(rng)
    return Qm @ np.diag(rng.normal(0.0, sigma, 3)) @ Qm.T


def random_vector(rng, rmin, rmax):
    v = rng.normal(size=3)
    return v / np.linalg.norm(v) * rng.uniform(rmin, rmax)


def random_efg(rng, vzz_min=0.1, vzz_max=1.0):
    """Random traceless symmetric EFG (a.u.) with |V_zz| ~ U(vzz_min, vzz_max)."""
    V = rng.normal(size=(3, 3))
    V = 0.5 * (V + V.T)
    V -= np.trace(V) / 3.0 * np.eye(3)
    w = np.linalg.eigvalsh(V)
    return V * (rng.uniform(vzz_min, vzz_max) / np.abs(w).max())


def config1(seed=1001, n_times=1000):
    rng = np.random.default_rng(seed)
    a = rng.uniform(100.0, 500.0)
    return Workload(
        name="mu_e_dim4",
        spins=["mu", "e"],
        couplings=[("hyperfine", {"i": 1}, a * np.eye(3))],
        orientations=np.array([[0.0, 0.0, 0.0]]),
        fields=np.array([[0.0, 0.0, 0.01]]),
        polarization=np.array([0.0, 0.0, 1.0]),
        times=np.linspace(0.0, 10.0, n_times),
        meta={"A_MHz": a},
    )


def config2(seed=1002, n_orient=10000, n_times=4096):
    rng = np.random.default_rng(seed)
    coup = [
        ("hyperfine", {"i": 1}, random_hyperfine(rng)),
        ("hyperfine", {"i": 3}, random_hyperfine(rng)),
        ("hyperfine", {"i": 4}, random_hyperfine(rng)),
    ]
    for i, j in [(1, 3), (1, 4), (3, 4)]:
        coup.append(("dipolar", {"i": i, "j": j}, random_vector(rng, 1.0, 3.0)))
    coup.append(("quadrupolar", {"i": 4}, random_efg(rng)))
    return Workload(
        name="mu_e_H_N_dim24_powder",
        spins=["mu", "e", "H", "N"],
        couplings=coup,
        orientations=zcw_gen(n_orient),
        fields=np.array([[0.0, 0.0, 0.01]]),
        polarization=np.array([0.0, 0.0, 1.0]),
        times=np.linspace(0.0, 20.0, n_times),
    )


def config3(seed=1003, n_fields=2000, n_orient=1000):
    rng = np.random.default_rng(seed)
    coup = [("hyperfine", {"i": 1}, random_hyperfine(rng))]
    for i in (3, 4, 5):
        coup.append(("hyperfine", {"i": i}, random_hyperfine(rng)))
    B = np.linspace(0.0, 1.0, n_fields)
    return Workload(
        name="mu_e_3H_dim32_alc",
        spins=["mu", "e", "H", "H", "H"],
        couplings=coup,
        orientations=zcw_gen(n_orient),
        fields=np.stack([np.zeros_like(B), np.zeros_like(B), B], axis=1),
        polarization=np.array([0.0, 0.0, 1.0]),
        times=np.array([np.inf]),
        y_axis="integral",
        x_axis="field",
    )


def config5(seed=1005, n_orient=2000, n_times=1000):
    rng = np.random.default_rng(seed)
    coup = [
        ("dipolar", {"i": 1, "j": 2}, random_vector(rng, 1.0, 1.4)),
        ("dipolar", {"i": 1, "j": 3}, random_vector(rng, 1.0, 1.4)),
        ("dipolar", {"i": 2, "j": 3}, random_vector(rng, 2.0, 2.8)),
    ]
    return Workload(
        name="F_mu_F_dim8_fit",
        spins=["mu", "F", "F"],
        couplings=coup,
        orientations=zcw_gen(n_orient),
        fields=np.array([[0.0, 0.0, 0.0]]),
        polarization=np.array([0.0, 0.0, 1.0]),
        times=np.linspace(0.0, 20.0, n_times),
    )


# Spin lists of the heterogeneous batch, by Hilbert dimension: the muon,
# at most one electron, one to five nuclei with I = 1/2 (1H) or I = 1 (14N).
CONFIG4_SPINS = {
    4: ["mu", "H"],
    8: ["mu", "e", "H"],
    12: ["mu", "e", "N"],
    24: ["mu", "e", "H", "N"],
    48: ["mu", "e", "H", "H", "N"],
    96: ["mu", "e", "H", "H", "H", "N"],
    192: ["mu", "e", "H", "H", "H", "H", "N"],
}


def random_system_workload(rng, dim, orientations, times, field=(0.0, 0.0, 0.01)):
    """One seeded system of the heterogeneous batch: hyperfine of the muon
    and of every nucleus to the electron (random anisotropic tensors as
    above), muon-nucleus point dipoles at U(1, 3) A, and the 14N quadrupole
    from a random EFG."""
    spins = CONFIG4_SPINS[dim]
    coup = []
    has_e = "e" in spins
    for i, s in enumerate(spins, start=1):
        if s == "e":
            continue
        if has_e:
            coup.append(("hyperfine", {"i": i}, random_hyperfine(rng)))
        if i > 1:
            coup.append(("dipolar", {"i": 1, "j": i}, random_vector(rng, 1.0, 3.0)))
        if s == "N":
            coup.append(("quadrupolar", {"i": i}, random_efg(rng)))
    return Workload(
        name=f"system_dim{dim}",
        spins=list(spins),
        couplings=coup,
        orientations=orientations,
        fields=np.array([field], dtype=float),
        polarization=np.array([0.0, 0.0, 1.0]),
        times=times,
    )


def config4(seed=1004, n_systems=4096, n_orient=256, n_times=2048,
            dims=(4, 8, 12, 24, 48, 96, 192)):
    """The heterogeneous batch: ``n_systems`` systems with dimensions drawn
    uniformly from ``dims``, each on the same ZCW-style grid of
    ``n_orient`` orientations, ``n_times`` times on 0-20 us, B = 0.01 T
    along z, p = z.  Returns a list of Workloads."""
    rng = np.random.default_rng(seed)
    orients = zcw_gen(n_orient)
    times = np.linspace(0.0, 20.0, n_times)
    draws = rng.choice(np.asarray(dims), size=n_systems)
    return [random_system_workload(rng, int(d), orients, times) for d in draws]


def celio_v3si(seed=1006, n_orient=8, n_times=50, k=10, averages=19, n_vanadium=4):
    """Celio's method on mu + n_vanadium V (dim 2 x 8^n; 8192 for the
    default 4); see the module docstring."""
    rng = np.random.default_rng(seed)
    spins = ["mu"] + ["V"] * n_vanadium
    coup = []
    for v in range(2, 2 + n_vanadium):
        coup.append(("dipolar", {"i": 1, "j": v}, random_vector(rng, 1.6, 2.0)))
        coup.append(("quadrupolar", {"i": v}, random_efg(rng, 0.02, 0.06)))
    orients = zcw_gen(n_orient) if n_orient > 1 else np.array([[0.0, 0.0]])
    return Workload("celio_v3si", spins, coup, orients, np.zeros((1, 3)),
                    np.array([1.0, 0.0, 0.0]), np.linspace(0, 10.0, n_times),
                    meta={"celio": (int(k), int(averages))})
