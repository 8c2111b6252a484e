"""CPU: the force oracle against the reference's own force functions."""
import os

import numpy as np
import pytest

from conftest import rel_err
from oracle import forces as of

G = os.path.join(os.path.dirname(__file__), "golden", "forces.npz")


@pytest.mark.parametrize("case", ["dense", "periodic", "far"])
def test_oracle_forces_match_reference_golden(case):
    g = np.load(G)
    eps, b, a = g[case + "_params"]
    bb = of.blob_blob_forces(g[case + "_r"], eps, b, a, periodic_length=g[case + "_L"])
    assert rel_err(bb, g[case + "_bb"]) <= 1e-13
    m, ra, gg, e, bw = g[case + "_ext_params"]
    assert rel_err(of.external_forces(g[case + "_r"], m, ra, gg, e, bw), g[case + "_ext"]) <= 1e-15


def test_body_reduction_is_force_and_moment():
    rng = np.random.default_rng(0)
    r = rng.standard_normal((10, 3))
    x = np.array([[0.0, 0.0, 0.0], [1.0, 1.0, 1.0]])
    f = rng.standard_normal((10, 3))
    ft = of.body_force_torque(r, x, [0, 4, 10], f)
    assert np.allclose(ft[0], f[:4].sum(0)) and np.allclose(ft[3], np.cross(r[4:] - x[1], f[4:]).sum(0))
