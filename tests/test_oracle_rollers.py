"""CPU: the oracle's rollers solve and forward Euler step against the
reference's QuaternionIntegratorRollers (tests/golden/rollers.npz)."""
import numpy as np
import pytest

from conftest import golden
from oracle import forces as of
from oracle import rollers as ro

CASES = {"wall": (True, False), "wall_free": (True, True), "periodic": (True, False), "no_wall": (False, False)}


def rel(x, y):
    return np.abs(np.asarray(x) - np.asarray(y)).max() / np.abs(np.asarray(y)).max()


def oracle_forces(g, c, r):
    eta, a = g[c + "_params"]
    gg, ew, bw, e, b = g[c + "_force_params"]
    return (of.external_forces(r, 1.0, a, gg, ew, bw) + of.blob_blob_forces(r, e, b, a, g[c + "_L"])).reshape(-1)


@pytest.mark.parametrize("c", list(CASES))
def test_oracle_rollers_match_reference(c):
    g = golden("rollers.npz")
    eta, a = g[c + "_params"]
    wp, free = CASES[c]
    assert rel(oracle_forces(g, c, g[c + "_r"]), g[c + "_force"]) <= 1e-13
    u, t = ro.velocity_and_torque(g[c + "_r"], g[c + "_force"], g[c + "_omega"], eta, a, g[c + "_L"],
                                  wall_present=wp, free_kinematics=free)
    assert rel(u, g[c + "_velocity"]) <= 1e-13
    assert rel(t, g[c + "_torque"]) <= 1e-12
    x = g[c + "_r"].copy()
    for step in range(2):
        u, _ = ro.velocity_and_torque(x, oracle_forces(g, c, x), g[c + "_omega"], eta, a, g[c + "_L"],
                                      wall_present=wp, free_kinematics=free)
        x = x + 0.01 * u.reshape(-1, 3)
        np.testing.assert_allclose(x, g[c + "_x%d" % step], rtol=0, atol=1e-12)
