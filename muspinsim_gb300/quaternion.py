"""Unit quaternions for crystallite orientations.

Convention of the reference (through ase.quaternions, pinned by
muspinsim/tests/test_config.py:233-285 and muspinsim/tests/test_utils.py:
43-65): q = [w, x, y, z], Hamilton product, ``rotate(v) = q v q*`` (the
matrix R(q) applied to v), Euler angles (a, b, c) in mode 'zyz' give
q_z(c) q_y(b) q_z(a) ('zxz': q_z(c) q_x(b) q_z(a)).

Batched helpers work on (N, 4) arrays so that a whole powder grid is
converted at once.
"""

import numpy as np


def qmul(a, b):
    """Hamilton product of (..., 4) arrays."""
    a = np.asarray(a, dtype=float)
    b = np.asarray(b, dtype=float)
    w1, x1, y1, z1 = np.moveaxis(a, -1, 0)
    w2, x2, y2, z2 = np.moveaxis(b, -1, 0)
    return np.stack(
        [
            w1 * w2 - x1 * x2 - y1 * y2 - z1 * z2,
            w1 * x2 + x1 * w2 + y1 * z2 - z1 * y2,
            w1 * y2 - x1 * z2 + y1 * w2 + z1 * x2,
            w1 * z2 + x1 * y2 - y1 * x2 + z1 * w2,
        ],
        axis=-1,
    )


def qconj(q):
    return np.asarray(q, dtype=float) * np.array([1.0, -1.0, -1.0, -1.0])


def axis_angle(axis, angle):
    """(..., 4) quaternions of rotations by `angle` about unit `axis`."""
    angle = np.asarray(angle, dtype=float)
    axis = np.asarray(axis, dtype=float)
    axis = axis / np.linalg.norm(axis)
    half = angle[..., None] / 2.0
    return np.concatenate([np.cos(half), np.sin(half) * axis], axis=-1)


def from_euler(a, b, c, mode="zyz"):
    """q_z(c) q_{y|x}(b) q_z(a) for arrays of angles (radians)."""
    if mode == "zyz":
        bax = [0.0, 1.0, 0.0]
    elif mode == "zxz":
        bax = [1.0, 0.0, 0.0]
    else:
        raise ValueError(f"Unsupported Euler mode {mode}")
    z = [0.0, 0.0, 1.0]
    return qmul(qmul(axis_angle(z, c), axis_angle(bax, b)), axis_angle(z, a))


def rotation_matrix(q):
    """(..., 3, 3) matrices R with R v = q v q*."""
    q = np.asarray(q, dtype=float)
    w, x, y, z = np.moveaxis(q, -1, 0)
    R = np.stack(
        [
            np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)], -1),
            np.stack([2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)], -1),
            np.stack([2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)], -1),
        ],
        axis=-2,
    )
    return R


def rotate(q, v):
    """q v q* for (N, 4) quaternions and a 3-vector or (N, 3) vectors."""
    q = np.asarray(q, dtype=float)
    v = np.asarray(v, dtype=float)
    zero = np.zeros(v.shape[:-1] + (1,))
    qv = np.concatenate([zero, v], axis=-1)
    return qmul(qmul(q, qv), qconj(q))[..., 1:]


class Quaternion:
    """Single quaternion with the interface the reference uses
    (``q``, ``conjugate``, ``rotate``, ``rotation_matrix``, ``*``,
    ``from_axis_angle``, ``from_euler_angles``, ``euler_angles``)."""

    def __init__(self, qin=(1.0, 0.0, 0.0, 0.0)):
        self.q = np.array(qin, dtype=float)

    def __mul__(self, other):
        return Quaternion(qmul(self.q, other.q))

    def __repr__(self):
        return "Quaternion({0}, {1}, {2}, {3})".format(*self.q)

    def conjugate(self):
        return Quaternion(qconj(self.q))

    def rotate(self, vector):
        return rotate(self.q, np.asarray(vector, dtype=float))

    def rotation_matrix(self):
        return rotation_matrix(self.q)

    def euler_angles(self, mode="zyz"):
        """(a, b, c) with from_euler_angles(a, b, c, mode) == self, up to sign."""
        R = self.rotation_matrix()
        if mode == "zyz":
            b = np.arccos(np.clip(R[2, 2], -1.0, 1.0))
            if np.isclose(np.sin(b), 0.0):
                a = np.arctan2(R[1, 0], R[0, 0])
                c = 0.0
            else:
                a = np.arctan2(R[2, 1], -R[2, 0])
                c = np.arctan2(R[1, 2], R[0, 2])
            # R = Rz(c) Ry(b) Rz(a): recover with the matching composition
            return np.array([a, b, c])
        raise ValueError(f"Unsupported Euler mode {mode}")

    @staticmethod
    def from_axis_angle(axis, angle):
        return Quaternion(axis_angle(axis, angle))

    @staticmethod
    def from_euler_angles(a, b, c, mode="zyz"):
        return Quaternion(from_euler(a, b, c, mode))
