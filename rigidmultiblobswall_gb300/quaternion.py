"""Quaternion with the conventions of quaternion_integrator/quaternion.py:7-84
(s, p) storage, from_rotation, product, rotation matrix, inverse.  Host-side FP64
(one 4-vector per body; the GPU path carries orientations as (Nb,4) arrays)."""
import numpy as np


class Quaternion(object):

    def __init__(self, entries):
        self.entries = entries
        self.s = np.array(entries[0])
        self.p = np.array(entries[1:4])

    @classmethod
    def from_rotation(cls, phi):
        """Quaternion of a rotation by |phi| about phi (quaternion.py:16-27)."""
        phi = np.asarray(phi, dtype=np.float64)
        phi_norm = np.linalg.norm(phi)
        s = np.array([np.cos(phi_norm / 2.)])
        if phi_norm != 0:
            p = np.sin(phi_norm / 2) * (phi / phi_norm)
        else:
            p = np.zeros(3)
        return cls(np.concatenate([s, p]))

    def __mul__(self, other):
        """Quaternion product, other on the right (quaternion.py:30-39)."""
        s = self.s * other.s - np.dot(self.p, other.p)
        p = self.s * other.p + other.s * self.p + np.cross(self.p, other.p)
        return Quaternion(np.concatenate(([s], p)))

    def rotation_matrix(self):
        """Rotation matrix of this quaternion (quaternion.py:42-51)."""
        diag = self.s ** 2 - 0.5
        p, s = self.p, self.s
        return 2.0 * np.array([[p[0] ** 2 + diag, p[0] * p[1] - s * p[2], p[0] * p[2] + s * p[1]],
                               [p[1] * p[0] + s * p[2], p[1] ** 2 + diag, p[1] * p[2] - s * p[0]],
                               [p[2] * p[0] - s * p[1], p[2] * p[1] + s * p[0], p[2] ** 2 + diag]])

    def inverse(self):
        return Quaternion([self.s, -1. * self.p[0], -1. * self.p[1], -1. * self.p[2]])

    def __str__(self):
        return '[ %f, %f, %f, %f ]' % (self.s, self.p[0], self.p[1], self.p[2])
