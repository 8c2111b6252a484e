"""GPU parity of the rollers solve (rmw_rollers_velocity_and_torque) and the
rollers forward Euler step against the reference's QuaternionIntegratorRollers
(tests/golden/rollers.npz, GMRES tolerance 1e-12 there and here) and the
quaternion_integrator/gmres.py drop-in.

Bars (max-norm relative): FP64 velocities and torques 1e-10, df64 1e-9,
mixed 1e-5 (the torque solve is then converged on the FP32-pair operator);
positions after two steps 1e-11 absolute."""
import functools

import numpy as np
import pytest

from conftest import golden
from oracle import rollers as ro
from rigidmultiblobswall_gb300 import forces, rollers

pytestmark = pytest.mark.gpu
CASES = {"wall": ("single_wall", False), "wall_free": ("single_wall", True), "periodic": ("single_wall", False),
         "no_wall": ("no_wall", False)}
BARS = {"fp64": 1e-10, "df64": 1e-9, "mixed": 1e-5}


def rel(x, y):
    return np.abs(np.asarray(x) - np.asarray(y)).max() / np.abs(np.asarray(y)).max()


@pytest.mark.parametrize("mode", list(BARS))
@pytest.mark.parametrize("c", list(CASES))
def test_rollers_solve_matches_reference(cuda_device, c, mode):
    g = golden("rollers.npz")
    eta, a = g[c + "_params"]
    domain, free = CASES[c]
    u, t, its = rollers.compute_deterministic_velocity_and_torque(
        g[c + "_r"], g[c + "_force"], g[c + "_omega"], eta, a, periodic_length=g[c + "_L"], tolerance=1e-12,
        domain=domain, free_kinematics=free, mode=mode)
    assert rel(u, g[c + "_velocity"]) <= BARS[mode]
    assert rel(t, g[c + "_torque"]) <= BARS[mode]
    assert (its == 0) == free


@pytest.mark.parametrize("c", list(CASES))
def test_rollers_forward_euler_matches_reference(cuda_device, c):
    g = golden("rollers.npz")
    eta, a = g[c + "_params"]
    gg, ew, bw, e, b = g[c + "_force_params"]
    domain, free = CASES[c]
    it = rollers.QuaternionIntegratorRollers(g[c + "_r"], "deterministic_forward_euler_rollers", tolerance=1e-12,
                                             domain=domain)
    it.eta, it.a = eta, a
    it.omega_one_roller = g[c + "_omega"]
    it.free_kinematics = "True" if free else "False"
    it.periodic_length = g[c + "_L"]
    it.calc_one_blob_forces = functools.partial(forces.blob_external_forces, blob_mass=1.0, blob_radius=a, g=gg,
                                                repulsion_strength_wall=ew, debye_length_wall=bw)
    it.calc_blob_blob_forces = functools.partial(forces.calc_blob_blob_forces_pycuda, blob_radius=a,
                                                 repulsion_strength=e, debye_length=b, periodic_length=g[c + "_L"])
    for step in range(2):
        it.advance_time_step(0.01)
        np.testing.assert_allclose(it.x.cpu().numpy(), g[c + "_x%d" % step], rtol=0, atol=1e-11)
    assert (it.det_iterations_count > 0) == (not free)


def test_rollers_larger_against_oracle(cuda_device):
    rng = np.random.default_rng(4)
    n, a = 900, 0.5
    r = np.column_stack([rng.uniform(0, 40, (n, 2)), rng.uniform(0.6, 4, n)])
    f = rng.standard_normal(3 * n)
    uo, to = ro.velocity_and_torque(r, f, [0.0, 1.0, 0.0], 1.0, a, tol=1e-10)
    u, t, its = rollers.compute_deterministic_velocity_and_torque(r, f, [0.0, 1.0, 0.0], 1.0, a, tolerance=1e-10)
    assert its > 0
    assert rel(u, uo) <= 1e-8 and rel(t, to) <= 1e-8


def test_quaternion_integrator_gmres_dropin(cuda_device):
    """gmres.gmres / gmres.right_gmres return (x, info, resnorms)."""
    from rigidmultiblobswall_gb300 import gmres
    rng = np.random.default_rng(2)
    n = 200
    A = np.eye(n) * 4 + rng.standard_normal((n, n)) / np.sqrt(n)
    P = np.diag(1.0 / np.diag(A))
    b = rng.standard_normal(n)
    x_ref = np.linalg.solve(A, b)
    for conv in ("resid", "presid"):
        x, info, res = gmres.gmres(lambda v: A @ v, b, convergence=conv, tol=1e-10, M=lambda v: P @ v, restart=50)
        assert info == 0 and len(res) > 0
        assert np.linalg.norm(x - x_ref) <= 1e-8 * np.linalg.norm(x_ref)
    x, info, res = gmres.right_gmres(lambda v: A @ v, b, M=lambda v: P @ v, tol=1e-10)
    assert info == 0 and np.linalg.norm(x - x_ref) <= 1e-8 * np.linalg.norm(x_ref)
    with pytest.raises(Exception):
        gmres.right_gmres(lambda v: A @ v, b, tol=1e-10)
