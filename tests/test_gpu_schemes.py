"""GPU parity of the time integrators (integrator.QuaternionIntegrator) with the
reference's QuaternionIntegrator: two steps of every GMRES-based scheme from
the same recorded normal draws (tests/golden/schemes.npz, tolerance 1e-12 on
both sides), compared on body locations and quaternions:

  FP64                 absolute 1e-8 (the random finite differences divide
                       solver-level differences by rf_delta = 1e-3)
  df64 / mixed         absolute 1e-6
  rejected steps, free space: against the oracle fed the same draws, 1e-8
"""
import numpy as np
import pytest

from conftest import golden
from rigidmultiblobswall_gb300 import forces, integrator
from rigidmultiblobswall_gb300.rigid import RigidSystem
from test_oracle_schemes import SCHEMES, Draws, make

pytestmark = pytest.mark.gpu


class DeviceDraws(Draws):
    def __call__(self, n):
        import torch
        return torch.as_tensor(super().__call__(n), device="cuda")


def gpu_integrator(g, scheme, draws, mode="fp64", wall=True, kT=None):
    ref = g["ref_cfg"]
    nb = g["locs"].shape[0]
    eta, a, kT0, dt, delta, tol = g["params"]
    sys_ = RigidSystem([ref.shape[0]] * nb, eta, a, wall=wall)
    it = integrator.QuaternionIntegrator(sys_, scheme, g["locs"], g["quats"], np.tile(ref, (nb, 1)), tolerance=tol,
                                         domain="single_wall" if wall else "no_wall",
                                         kT=kT0 if kT is None else kT, rf_delta=delta, mode=mode, normal=draws)
    m, gg, ew, bw, e, b = g["force_params"]
    it.force_torque_calculator = lambda s, r: forces.force_torque_calculator_sort_by_bodies(
        s, r, blob_mass=m, g=gg, repulsion_strength_wall=ew, debye_length_wall=bw, repulsion_strength=e,
        debye_length=b, periodic_length=np.zeros(3))
    return it, dt


def test_body_length_matches_reference(cuda_device):
    g = golden("schemes.npz")
    ref = g["ref_cfg"]
    eta, a = g["params"][:2]
    bl = integrator.body_lengths([ref.shape[0]] * 3, __import__("torch").as_tensor(np.tile(ref, (3, 1))).cuda(), a)
    np.testing.assert_allclose(bl.cpu().numpy(), g["body_length"][0], rtol=1e-14)


@pytest.mark.parametrize("scheme", SCHEMES)
def test_scheme_matches_reference(cuda_device, scheme):
    g = golden("schemes.npz")
    draws = DeviceDraws(g[scheme + "_draws"], g[scheme + "_draw_sizes"])
    it, dt = gpu_integrator(g, scheme, draws)
    for step in range(2):
        it.advance_time_step(dt)
        np.testing.assert_allclose(it.x.cpu().numpy(), g["%s_locs%d" % (scheme, step)], rtol=0, atol=1e-8)
        np.testing.assert_allclose(it.q.cpu().numpy(), g["%s_quats%d" % (scheme, step)], rtol=0, atol=1e-8)
    assert draws.done()
    assert it.invalid_configuration_count == 0
    assert it.det_iterations_count > 0
    assert (it.stoch_iterations_count > 0) == scheme.startswith("stochastic")
    it.close()


@pytest.mark.parametrize("mode", ["df64", "mixed"])
@pytest.mark.parametrize("scheme", ["stochastic_traction_EM", "stochastic_Slip_Trapz", "stochastic_first_order_RFD"])
def test_scheme_reduced_precision_modes(cuda_device, scheme, mode):
    g = golden("schemes.npz")
    draws = DeviceDraws(g[scheme + "_draws"], g[scheme + "_draw_sizes"])
    it, dt = gpu_integrator(g, scheme, draws, mode=mode)
    for step in range(2):
        it.advance_time_step(dt)
        np.testing.assert_allclose(it.x.cpu().numpy(), g["%s_locs%d" % (scheme, step)], rtol=0, atol=1e-6)
        np.testing.assert_allclose(it.q.cpu().numpy(), g["%s_quats%d" % (scheme, step)], rtol=0, atol=1e-6)


def test_rejected_step_is_redrawn_like_the_oracle(cuda_device):
    """A first Brownian draw scaled by 300 pushes a shell through the wall: the
    step is rejected and redrawn with the next draws, on both sides."""
    g = golden("schemes.npz")
    scheme = "stochastic_Slip_Trapz"
    rng = np.random.default_rng(7)
    n3 = 3 * g["ref_cfg"].shape[0] * g["locs"].shape[0]
    vals = rng.standard_normal(8 * n3)
    vals[:n3] *= 300.0
    sizes = [n3] * 8
    it, dt = gpu_integrator(g, scheme, DeviceDraws(vals, sizes))
    o, _ = make(g, scheme, Draws(vals, sizes))
    it.advance_time_step(dt)
    o.advance_time_step(dt)
    assert o.invalid_configuration_count >= 1
    assert it.invalid_configuration_count == o.invalid_configuration_count
    np.testing.assert_allclose(it.x.cpu().numpy(), o.x, rtol=0, atol=1e-8)
    np.testing.assert_allclose(it.q.cpu().numpy(), o.q, rtol=0, atol=1e-8)


@pytest.mark.parametrize("scheme", ["stochastic_traction_EM", "stochastic_Slip_Mid", "deterministic_midpoint"])
def test_free_space_scheme_matches_oracle(cuda_device, scheme):
    g = golden("schemes.npz")
    sizes = g[scheme + "_draw_sizes"]
    vals = g[scheme + "_draws"]
    it, dt = gpu_integrator(g, scheme, DeviceDraws(vals, sizes), wall=False)
    o, _ = make(g, scheme, Draws(vals, sizes))
    o.wall = False
    for _ in range(2):
        it.advance_time_step(dt)
        o.advance_time_step(dt)
    np.testing.assert_allclose(it.x.cpu().numpy(), o.x, rtol=0, atol=1e-8)
    np.testing.assert_allclose(it.q.cpu().numpy(), o.q, rtol=0, atol=1e-8)


def test_zero_temperature_traction_is_forward_euler(cuda_device):
    """kT = 0: the random force and the Brownian slip vanish (the Lanczos call
    draws nothing) and stochastic_traction_EM reduces to forward Euler."""
    g = golden("schemes.npz")
    nb = g["locs"].shape[0]
    vals = np.random.default_rng(3).standard_normal(6 * nb)
    a, _ = gpu_integrator(g, "stochastic_traction_EM", DeviceDraws(vals, [6 * nb]), kT=0.0)
    b, dt = gpu_integrator(g, "deterministic_forward_euler", DeviceDraws(np.zeros(0), []))
    a.advance_time_step(dt)
    b.advance_time_step(dt)
    np.testing.assert_allclose(a.x.cpu().numpy(), b.x.cpu().numpy(), rtol=0, atol=1e-12)
    np.testing.assert_allclose(a.q.cpu().numpy(), b.q.cpu().numpy(), rtol=0, atol=1e-12)


def test_run_saves_and_resumes_on_device(cuda_device, tmp_path):
    """clones.run with the device integrator: 4 steps of stochastic_traction_EM
    saved every 2 steps to a .config trajectory, against 2 steps, a resume from
    the saved frame at initial_step 2 and 2 more steps with the same draws."""
    import os
    from rigidmultiblobswall_gb300 import clones
    g = golden("schemes.npz")
    scheme = "stochastic_traction_EM"
    nb = g["locs"].shape[0]
    n3 = 3 * g["ref_cfg"].shape[0] * nb
    sizes = [6 * nb, n3] * 4
    vals = np.random.default_rng(11).standard_normal(sum(sizes))
    it, dt = gpu_integrator(g, scheme, DeviceDraws(vals, sizes))
    full = os.path.join(str(tmp_path), "full")
    clones.run(it, dt, 4, n_save=2, output_name=full, save_clones="one_file")
    frames = clones.read_config_file(full + ".body.config")
    assert len(frames) == 3
    np.testing.assert_array_equal(frames[0][0], g["locs"])
    np.testing.assert_array_equal(frames[2][0], it.x.cpu().numpy())
    np.testing.assert_array_equal(frames[2][1], it.q.cpu().numpy())
    half = sum(sizes[:4])
    a, _ = gpu_integrator(g, scheme, DeviceDraws(vals[:half], sizes[:4]))
    clones.run(a, dt, 2, n_save=2, output_name=os.path.join(str(tmp_path), "p1"), save_clones="one_file")
    loc, ori = clones.resume_state(os.path.join(str(tmp_path), "p1.body.config"))
    b, _ = gpu_integrator(g, scheme, DeviceDraws(vals[half:], sizes[4:]))
    b.x.copy_(__import__("torch").as_tensor(loc))
    b.q.copy_(__import__("torch").as_tensor(ori))
    clones.run(b, dt, 4, n_save=2, output_name=os.path.join(str(tmp_path), "p2"), initial_step=2,
               save_clones="one_file")
    np.testing.assert_allclose(b.x.cpu().numpy(), it.x.cpu().numpy(), rtol=0, atol=1e-12)
    np.testing.assert_allclose(b.q.cpu().numpy(), it.q.cpu().numpy(), rtol=0, atol=1e-12)
    assert "invalid_configuration_count    = 0" in open(full + ".info").read()
