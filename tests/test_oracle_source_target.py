"""CPU: the oracle's source-target products (per-blob radii; wall, free space,
free surface) and single-radius free-surface product against the reference's
own numba and Python functions (tests/golden/source_target.npz)."""
import numpy as np
import pytest

from conftest import golden
from oracle import source_target as st

CASES = ["far", "close", "periodic"]
GEOMS = {"wall": "wall", "no_wall": "nowall", "free_surface": "free_surface"}


def rel(x, y):
    return np.abs(np.asarray(x) - np.asarray(y)).max() / np.abs(np.asarray(y)).max()


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("geom", list(GEOMS))
def test_oracle_source_target_matches_reference(case, geom):
    g = golden("source_target.npz")
    u = st.source_target(geom, g[case + "_source"], g[case + "_target"], g[case + "_f"], g[case + "_rs"],
                         g[case + "_rt"], g[case + "_eta"][0], g[case + "_L"])
    assert rel(u, g[case + "_" + GEOMS[geom]]) <= 1e-14


@pytest.mark.parametrize("case", ["far", "close"])
def test_reference_python_forms_agree_with_numba(case):
    g = golden("source_target.npz")
    assert rel(g[case + "_one_wall_py"], g[case + "_wall"]) <= 1e-14
    assert rel(g[case + "_unbounded_py"], g[case + "_nowall"]) <= 1e-14


@pytest.mark.parametrize("case", ["fs", "fs_periodic"])
def test_oracle_free_surface_matches_reference(case):
    g = golden("source_target.npz")
    a, eta = g[case + "_params"]
    u = st.free_surface(g[case + "_r"], g[case + "_f"], eta, a, g[case + "_L"])
    assert rel(u, g[case + "_u"]) <= 1e-14
    # the same product as the source-target form with every radius a
    n = g[case + "_r"].shape[0]
    v = st.source_target("free_surface", g[case + "_r"], g[case + "_r"], g[case + "_f"], np.full(n, a),
                         np.full(n, a), eta, g[case + "_L"])
    assert rel(v, g[case + "_u"]) <= 1e-13
