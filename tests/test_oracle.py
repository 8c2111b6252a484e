"""CPU: the oracle against the golden vectors made from the reference's own code."""
import os

import numpy as np
import pytest

from conftest import golden, rel_err
from oracle import wall
from rigidmultiblobswall_gb300 import suspensions as S

CASES = ["far", "damped", "touching", "periodic", "single"]
KINDS = ["uf", "ut", "wf", "wt"]


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("kind", KINDS)
def test_oracle_matches_reference_golden(case, kind):
    g = golden("products.npz")
    a, eta = g[case + "_params"]
    L = g[case + "_L"]
    out = wall.wall_product(kind, g[case + "_r"], g[case + "_v"], eta, a, periodic_length=L)
    assert rel_err(out, g[case + "_" + kind]) <= 1e-14


@pytest.mark.parametrize("case", ["damped", "touching", "single"])
def test_oracle_matches_reference_dense_mobility(case):
    g = golden("products.npz")
    a, eta = g[case + "_params"]
    ref = g[case + "_dense"] @ g[case + "_v"].reshape(-1)
    assert rel_err(wall.wall_product("uf", g[case + "_r"], g[case + "_v"], eta, a), ref) <= 1e-13


def test_symmetric_cpu_baseline_matches_oracle():
    r, f, eta, a = S.blobs_wall_matvec(300, seed=5)
    r[:5, 2] = 0.2  # damping active
    ref = wall.wall_product("uf", r, f, eta, a)
    assert rel_err(wall.uf_symmetric_fast(r, f, eta, a, threads=2), ref) <= 1e-12


def test_oracle_mobility_symmetry():
    """The full wall mobility is symmetric: M_UF = M_UF^T, M_WT = M_WT^T and M_WF = M_UT^T."""
    rng = np.random.default_rng(7)
    r, _, eta, a = S.blobs_wall_matvec(120, seed=7)
    r[:10, 2] = rng.uniform(0.1, 0.5, 10)
    f, g = rng.standard_normal(360), rng.standard_normal(360)
    for k in ("uf", "wt"):
        lhs = f @ wall.wall_product(k, r, g, eta, a)
        rhs = g @ wall.wall_product(k, r, f, eta, a)
        assert abs(lhs - rhs) <= 1e-12 * abs(lhs)
    lhs = f @ wall.wall_product("ut", r, g, eta, a)
    rhs = g @ wall.wall_product("wf", r, f, eta, a)
    assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), 1e-300)


def test_row_sampled_oracle_matches_full():
    r, f, eta, a = S.blobs_wall_matvec(200, seed=9)
    full = wall.wall_product("wf", r, f, eta, a)
    rows = np.array([0, 17, 199, 54])
    part = wall.wall_product("wf", r, f, eta, a, rows=rows)
    np.testing.assert_array_equal(part.reshape(-1, 3), full.reshape(-1, 3)[rows])


def test_generated_shells_match_reference_vertex_files():
    g = golden("shells.npz")
    for mine, ref in ((S.icosahedron(1.0), g["shell12"]), (S.icosphere_42(), g["shell42"])):
        assert mine.shape == ref.shape
        d = np.linalg.norm(mine[:, None] - ref[None], axis=-1)
        assert d.min(axis=1).max() < 1e-12 and d.min(axis=0).max() < 1e-12
    assert abs(S.blob_radius_of(S.icosphere_42()) - 0.243553056072) < 1e-9


def test_rotation_matrices_match_reference_quaternion():
    g = golden("quaternion.npz")
    np.testing.assert_allclose(S.rotation_matrices(g["q"]), g["rot"], rtol=0, atol=1e-15)


def test_workloads_are_seeded_and_non_overlapping():
    s1, s2 = S.shells_42_256(), S.shells_42_256()
    np.testing.assert_array_equal(s1.r_vectors(), s2.r_vectors())
    c = s1.locations
    d = np.linalg.norm(c[:, None] - c[None], axis=-1) + np.eye(len(c)) * 1e9
    R = np.linalg.norm(s1.shell[0])
    assert d.min() > 2 * R + 2 * s1.a
    assert s1.n_blobs == 10752


def test_oracle_point_particle_limit_is_blake():
    """Property test of mobility/mobility_test.py:70-82 (finite-size limit),
    against the full Blake image system: off-diagonal blocks agree to O(a^2)."""
    rng = np.random.default_rng(0)
    r = rng.normal(5.0, 1.0, (4, 3))
    M = wall.dense_mobility(r, 1.0, 1e-4)
    B = wall.blake_point_mobility(r, 1.0)
    off = ~np.kron(np.eye(4, dtype=bool), np.ones((3, 3), dtype=bool))
    assert np.abs(M - B)[off].max() <= 1e-7 * np.abs(B[off]).max()


@pytest.mark.parametrize("case", ["far", "touching", "periodic", "single"])
@pytest.mark.parametrize("kind", ["uf", "ut", "wf", "wt"])
def test_oracle_no_wall_matches_reference_golden(case, kind):
    """The C restatement of the free-space products against the reference's
    own no-wall numba functions (tests/golden/nowall.npz)."""
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "nowall.npz"))
    a, eta = g[case + "_params"]
    got = wall.no_wall_product(kind, g[case + "_r"], g[case + "_v"], eta, a, periodic_length=g[case + "_L"])
    assert rel_err(got, g[case + "_" + kind]) <= 1e-14


@pytest.mark.parametrize("case", ["far", "touching"])
def test_oracle_free_space_dense_matches_rotne_prager_tensor(case):
    """Dense free-space blob mobility against the reference's rotne_prager_tensor."""
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "nowall.npz"))
    a, eta = g[case + "_params"]
    assert rel_err(wall.no_wall_dense(g[case + "_r"], eta, a), g[case + "_dense"]) <= 1e-14
