"""Oracle (test infrastructure only): numpy restatement of the reference's
blob forces, multi_bodies/multi_bodies_functions.py:
* blob_blob_forces  - calc_blob_blob_forces_python + blob_blob_force (:297-345):
  soft repulsion from U(r) = U0 exp(-(r - 2a)/b) for r > 2a, linear below,
  minimum periodic image;
* external_forces   - blob_external_forces (:153-189): gravity -g m e_z plus
  the wall repulsion of U(h) = U0 exp(-(h - a)/b) (constant force for h <= a);
* body_force_torque - the body reduction of force_torque_calculator_sort_by_bodies
  (:411-445): per body the sum of blob forces and the sum of (r - x) x f.
Pinned to tests/golden/forces.npz."""
import numpy as np


def _project(d, L):
    out = d.copy()
    for c in range(3):
        if L[c] > 0:
            q = d[..., c] / L[c] + 0.5 * np.sign(d[..., c])
            out[..., c] = d[..., c] - np.trunc(q) * L[c]
    return out


def blob_blob_forces(r, repulsion_strength, debye_length, blob_radius, periodic_length=None):
    r = np.asarray(r, dtype=np.float64).reshape(-1, 3)
    L = np.zeros(3) if periodic_length is None else np.asarray(periodic_length, dtype=np.float64)
    d = r[None, :, :] - r[:, None, :]          # d[i, j] = r_j - r_i
    d = _project(d, L)
    rn = np.linalg.norm(d, axis=-1)
    eps, b, a = repulsion_strength, debye_length, blob_radius
    safe = np.maximum(rn, np.finfo(float).eps)
    mag = np.where(rn > 2 * a, (eps / b) * np.exp(-(rn - 2 * a) / b) / safe, (eps / b) / safe)
    np.fill_diagonal(mag, 0.0)
    return -(mag[:, :, None] * d).sum(axis=1)


def external_forces(r, blob_mass, blob_radius, g, repulsion_strength_wall, debye_length_wall):
    r = np.asarray(r, dtype=np.float64).reshape(-1, 3)
    f = np.zeros_like(r)
    f[:, 2] = -g * blob_mass
    h = r[:, 2]
    e, b, a = repulsion_strength_wall, debye_length_wall, blob_radius
    f[:, 2] += np.where(h > a, (e / b) * np.exp(-(h - a) / b), e / b)
    return f


def body_force_torque(r, locations, offsets, f_blobs):
    """(2 Nb, 3): [F_1, T_1, F_2, T_2, ...]."""
    r = np.asarray(r, dtype=np.float64).reshape(-1, 3)
    f = np.asarray(f_blobs, dtype=np.float64).reshape(-1, 3)
    x = np.asarray(locations, dtype=np.float64).reshape(-1, 3)
    out = np.zeros((2 * x.shape[0], 3))
    for k in range(x.shape[0]):
        sl = slice(offsets[k], offsets[k + 1])
        out[2 * k] = f[sl].sum(axis=0)
        out[2 * k + 1] = np.cross(r[sl] - x[k], f[sl]).sum(axis=0)
    return out
