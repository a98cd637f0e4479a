"""Powder orientation grids.

``zcw_gen`` restates the Zaremba-Conroy-Wolfsberg lattice as published
(Cheng, Suwelack & Vold 1973; Eden & Levitt, J. Magn. Reson. 132 (1998) 220,
eqs. 5-6, full-sphere constants c = (1, 2, 1)): for N points and generator
g coprime with N,
    beta_j  = arccos(c1 (c2 frac(j / N) - 1)),
    alpha_j = 2 pi / c3 * frac(j g / N),
with N a Fibonacci number F_{M+2} and g = F_M in the original scheme.  Any
N is accepted here: g is the integer nearest N / phi^2 that is coprime with
N, which reduces to the Fibonacci choice when N is a Fibonacci number.  The
reference delegates this grid to a third-party library
(``muspinsim/utils.py:34-37``); its ``(theta, phi)`` rows feed
``quat_from_polar`` exactly like the reference's.

``eulrange_gen`` follows ``muspinsim/utils.py:40-50``.
"""

import math

import numpy as np

from muspinsim_gb300 import quaternion as Q


def zcw_generator(N):
    """The ZCW generator g used for N points (coprime with N, nearest
    N / phi^2)."""
    return _generator(int(N))


def _generator(N):
    phi2 = ((1.0 + 5**0.5) / 2.0) ** 2
    g0 = max(1, int(round(N / phi2)))
    for delta in range(N):
        for g in (g0 + delta, g0 - delta):
            if 1 <= g < max(N, 2) and math.gcd(g, N) == 1:
                return g
    return 1


def zcw_gen(N, mode="sphere"):
    """(N, 2) array of polar angles (theta, phi) of a ZCW-style grid."""
    N = int(N)
    if N < 1:
        raise ValueError("ZCW grid needs at least one point")
    if mode == "sphere":
        c1, c2, c3 = 1.0, 2.0, 1.0
    elif mode == "hemisphere":
        c1, c2, c3 = -1.0, 1.0, 1.0
    else:
        raise ValueError(f"Unknown ZCW mode {mode}")
    j = np.arange(N, dtype=np.int64)
    g = _generator(N)
    # frac(j / N) = j / N for j < N; frac(j g / N) from the exact integer
    # remainder (the device grid generator, msp_orient_grid_snapshots, uses
    # the same two expressions)
    beta = np.arccos(np.clip(c1 * (c2 * (j / N) - 1.0), -1.0, 1.0))
    alpha = 2.0 * np.pi / c3 * (((j * g) % N) / N)
    return np.stack([beta, alpha], axis=1)


def eulrange_gen(N):
    """N^3 ZYZ Euler angles with sin(beta) weights (muspinsim/utils.py:40-50)."""
    N = int(N)
    a = np.linspace(0, 2 * np.pi, N)
    b = np.linspace(0, np.pi, N + 2)[1:-1]
    c = np.linspace(0, 2 * np.pi, N)
    a, b, c = np.array(np.meshgrid(a, b, c)).reshape((3, -1))
    w = np.sin(b)
    return np.array([a, b, c, w]).T


def quat_from_polar(theta, phi):
    """Quaternion turning z towards (theta, phi): Euler (phi, theta, phi) in
    ZYZ (muspinsim/utils.py:53-68)."""
    return Q.Quaternion.from_euler_angles(phi, theta, phi, "zyz")


def _ragged(rows):
    if isinstance(rows, np.ndarray):
        return rows.dtype == object
    lens = {len(np.atleast_1d(r)) for r in rows}
    return len(lens) > 1


def orientation_rows_to_quats(rows, mode="zyz"):
    """Stored orientations of a list of input rows: the CONJUGATE rotation
    quaternions (N, 4) and weights (N,), as MuSpinConfig._validate_orient
    keeps them (muspinsim/simconfig.py:596-613).  Rows are (theta, phi),
    (a, b, c) or (a, b, c, w)."""
    arr = np.asarray(rows, dtype=object if _ragged(rows) else float)
    if arr.dtype != object and arr.ndim == 2 and arr.shape[1] in (2, 3, 4):
        # one kind of row: convert the whole grid at once
        if arr.shape[1] == 2:
            q = Q.from_euler(arr[:, 1], arr[:, 0], arr[:, 1], "zyz")
            ws = np.ones(len(arr))
        else:
            q = Q.from_euler(arr[:, 0], arr[:, 1], arr[:, 2], mode)
            ws = arr[:, 3].copy() if arr.shape[1] == 4 else np.ones(len(arr))
        return Q.qconj(q), ws
    rows = [np.atleast_1d(np.asarray(r, dtype=float)) for r in rows]
    qs = np.empty((len(rows), 4))
    ws = np.ones(len(rows))
    for k, r in enumerate(rows):
        if len(r) == 2:
            q = Q.from_euler(r[1], r[0], r[1], "zyz")
        elif len(r) == 3:
            q = Q.from_euler(r[0], r[1], r[2], mode)
        elif len(r) == 4:
            q = Q.from_euler(r[0], r[1], r[2], mode)
            ws[k] = r[3]
        else:
            raise ValueError(f"Invalid orientation row {r}")
        qs[k] = Q.qconj(q)
    return qs, ws
