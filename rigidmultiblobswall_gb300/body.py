"""Rigid body with the interface of body/body.py:13-255 (the parts the
mobility solve uses): blob positions from location + orientation, the geometric
matrix K = [J, R], the wall check.  Host-side FP64 per body; the GPU solve
path takes the concatenated blob positions and locations of all bodies."""
import copy

import numpy as np

from .quaternion import Quaternion  # noqa: F401  (re-export for callers)


class Body(object):

    def __init__(self, location, orientation, reference_configuration, blob_radius):
        self.location = np.copy(location)
        self.location_new = np.copy(location)
        self.location_old = np.copy(location)
        self.orientation = copy.copy(orientation)
        self.orientation_new = copy.copy(orientation)
        self.orientation_old = copy.copy(orientation)
        self.Nblobs = reference_configuration.shape[0]
        self.reference_configuration = np.reshape(reference_configuration[:, 0:3], (self.Nblobs, 3))
        self.blob_masses = np.ones(self.Nblobs)
        self.blob_radius = blob_radius
        self.blobs_radius = np.ones(self.Nblobs) * blob_radius
        self.prescribed_velocity = np.zeros(6)
        self.prescribed_kinematics = False
        self.mobility_blobs = None
        self.ID = None

    def get_r_vectors(self, location=None, orientation=None):
        """r = R(q) r_ref + x (body.py:64-78)."""
        location = self.location if location is None else location
        orientation = self.orientation if orientation is None else orientation
        R = orientation.rotation_matrix()
        return np.dot(self.reference_configuration, R.T) + location

    def calc_rot_matrix(self, location=None, orientation=None):
        """(3 Nblobs, 3) matrix with R_i x = -(r_i - x_body) cross x (body.py:81-96)."""
        r = self.get_r_vectors(location, orientation) - (self.location if location is None else location)
        rot = np.zeros((r.shape[0], 3, 3))
        rot[:, 0, 1] = r[:, 2]
        rot[:, 0, 2] = -r[:, 1]
        rot[:, 1, 0] = -r[:, 2]
        rot[:, 1, 2] = r[:, 0]
        rot[:, 2, 0] = r[:, 1]
        rot[:, 2, 1] = -r[:, 0]
        return np.reshape(rot, (3 * self.Nblobs, 3))

    def calc_J_matrix(self):
        J = np.zeros((3 * self.Nblobs, 3))
        J[0::3, 0] = 1.0
        J[1::3, 1] = 1.0
        J[2::3, 2] = 1.0
        return J

    def calc_K_matrix(self, location=None, orientation=None):
        """K = [J, R], shape (3 Nblobs, 6) (body.py:111-115)."""
        return np.concatenate([self.calc_J_matrix(), self.calc_rot_matrix(location, orientation)], axis=1)

    def check_function(self, location=None, orientation=None, distance=None):
        """True if every blob has z >= distance (default 0) (body.py:118-140)."""
        distance = 0.0 if not distance else distance
        r = self.get_r_vectors(location, orientation)
        return bool(np.all(r[:, 2] >= distance))
