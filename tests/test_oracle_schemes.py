"""CPU: the oracle's time integrators against two steps of the reference's own
QuaternionIntegrator schemes, fed the same recorded normal draws
(tests/golden/schemes.npz), and its rotation matrix against the reference's."""
import numpy as np
import pytest

from conftest import golden
from oracle import schemes

SCHEMES = ["deterministic_forward_euler", "deterministic_adams_bashforth", "deterministic_midpoint",
           "stochastic_EM", "stochastic_first_order_RFD", "stochastic_adams_bashforth", "stochastic_traction_EM",
           "stochastic_traction_AB", "stochastic_Slip_Trapz", "stochastic_Slip_Mid"]


class Draws:
    """Replays a recorded draw sequence; checks every request's size."""

    def __init__(self, values, sizes):
        self.values, self.sizes = values, list(sizes)
        self.pos, self.k = 0, 0

    def __call__(self, n):
        assert self.k < len(self.sizes) and self.sizes[self.k] == n, "draw %d of size %d" % (self.k, n)
        out = self.values[self.pos:self.pos + n].copy()
        self.pos += n
        self.k += 1
        return out

    def done(self):
        return self.k == len(self.sizes)


def make(g, scheme, draws):
    ref = g["ref_cfg"]
    nb = g["locs"].shape[0]
    eta, a, kT, dt, delta, tol = g["params"]
    return schemes.Integrator(scheme, g["locs"], g["quats"], np.tile(ref, (nb, 1)), np.arange(nb + 1) * ref.shape[0],
                              eta, a, kT, g["body_length"][0], draws, g["force_params"], tolerance=tol,
                              rf_delta=delta), dt


def test_rotation_matrix_matches_reference():
    g = golden("quaternion.npz")
    for q, R in zip(g["q"], g["rot"]):
        np.testing.assert_allclose(schemes.rotation_matrix(q), R, rtol=0, atol=1e-14)


@pytest.mark.parametrize("scheme", SCHEMES)
def test_oracle_scheme_matches_reference(scheme):
    g = golden("schemes.npz")
    draws = Draws(g[scheme + "_draws"], g[scheme + "_draw_sizes"])
    it, dt = make(g, scheme, draws)
    for step in range(2):
        it.advance_time_step(dt)
        np.testing.assert_allclose(it.x, g["%s_locs%d" % (scheme, step)], rtol=0, atol=1e-9)
        np.testing.assert_allclose(it.q, g["%s_quats%d" % (scheme, step)], rtol=0, atol=1e-9)
    assert draws.done()
    assert it.invalid_configuration_count == g[scheme + "_counts"][0]
