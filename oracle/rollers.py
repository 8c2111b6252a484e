"""Oracle (test infrastructure only): rollers at a prescribed angular velocity,
QuaternionIntegratorRollers.compute_deterministic_velocity_and_torque
(quaternion_integrator/quaternion_integrator_rollers.py:905-983) in numpy on
the C wall products: M_WT T = omega - M_WF F by unpreconditioned GMRES (the
RHS scaled to norm 1), U = M_UF F + M_UT T; free kinematics T = omega 8 pi eta a^3
(:1586-1597); forward Euler x += U dt (:119-152).  Pinned to
tests/golden/rollers.npz."""
import numpy as np

from . import rigid as orig
from . import wall


def _product(kind, r, v, eta, a, L, wall_present):
    if wall_present:
        return wall.wall_product(kind, r, v, eta, a, periodic_length=L)
    return wall.no_wall_product(kind, r, v, eta, a, periodic_length=L)


def velocity_and_torque(r, force, omega, eta, a, L=None, tol=1e-12, wall_present=True, free_kinematics=False):
    r = np.asarray(r, dtype=np.float64).reshape(-1, 3)
    n = r.shape[0]
    L = np.zeros(3) if L is None else np.asarray(L, dtype=np.float64)
    f = np.asarray(force, dtype=np.float64).reshape(-1)
    w = np.tile(np.asarray(omega, dtype=np.float64).reshape(-1)[:3], n) if np.size(omega) == 3 else \
        np.asarray(omega, dtype=np.float64).reshape(-1)
    if free_kinematics:
        t = w * 8.0 * np.pi * eta * a ** 3
    else:
        rhs = w - _product("wf", r, f, eta, a, L, wall_present)
        nrm = np.linalg.norm(rhs)
        t = np.zeros(3 * n)
        if nrm > 0:
            t, _, _ = orig.gmres_right(lambda x: _product("wt", r, x, eta, a, L, wall_present), lambda x: x,
                                       rhs / nrm, tol=tol, restart=20)
            t = t * nrm
    u = _product("uf", r, f, eta, a, L, wall_present) + _product("ut", r, t, eta, a, L, wall_present)
    return u, t
