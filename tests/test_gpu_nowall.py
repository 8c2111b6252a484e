"""GPU: free-space (no-wall) RPY products against the reference's own no-wall
numba functions (golden vectors) and the oracle, in every precision mode:
far, exact-contact (r = 2a) and periodic cases, blobs below z = 0 (there is
no wall), tile tails, the force-torque drop-in, and the symmetric positive
definiteness of the free-space 6N mobility."""
import os

import numpy as np
import pytest

from conftest import rel_err
from oracle import wall as owall
from rigidmultiblobswall_gb300 import mobility as mob

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-12, "df64": 1e-12, "mixed": 1e-6}
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "nowall.npz")


@pytest.mark.parametrize("mode", ["fp64", "df64", "mixed"])
@pytest.mark.parametrize("case", ["far", "touching", "periodic", "single"])
@pytest.mark.parametrize("kind", ["uf", "ut", "wf", "wt"])
def test_no_wall_matches_reference_golden(cuda_device, kind, case, mode):
    g = np.load(GOLDEN)
    a, eta = g[case + "_params"]
    got = mob.no_wall_product(kind, g[case + "_r"], g[case + "_v"], eta, a, mode=mode,
                              periodic_length=g[case + "_L"])
    assert rel_err(got, g[case + "_" + kind]) <= TOL[mode]


@pytest.mark.parametrize("mode", ["fp64", "df64", "mixed"])
@pytest.mark.parametrize("n", [129, 700])
def test_no_wall_tile_tails_match_oracle(cuda_device, mode, n):
    import torch
    rng = np.random.default_rng(n)
    r = rng.uniform(-6.0, 6.0, (n, 3))
    for kind in ("uf", "ut", "wf", "wt"):
        v = rng.standard_normal(3 * n)
        got = mob.no_wall_product(kind, torch.tensor(r, device="cuda"), torch.tensor(v, device="cuda"), 0.8, 0.35,
                                  mode=mode)
        assert got.is_cuda
        assert rel_err(got.cpu().numpy(), owall.no_wall_product(kind, r, v, 0.8, 0.35)) <= TOL[mode]


@pytest.mark.parametrize("mode,n", [("fp64", 4100), ("df64", 4100), ("mixed", 8200)])
@pytest.mark.parametrize("kind", ["uf", "ut", "wf", "wt"])
def test_no_wall_symmetric_kernel_rows_match_oracle(cuda_device, mode, n, kind):
    """From 4,096 blobs (8,192 in mixed) the free-space products take the
    symmetric kernel (each unordered pair once: M_ji = M_ij(-d)); blobs on both
    sides of z = 0 and a few touching pairs, sampled rows against the oracle."""
    rng = np.random.default_rng(n + len(kind))
    side = 2.2 * np.cbrt(n)
    r = rng.uniform(-side / 2, side / 2, (n, 3))
    r[1::97] = r[0::97][: len(r[1::97])] + np.array([0.7, 0.0, 0.0])  # r = 2a pairs (a = 0.35)
    v = rng.standard_normal(3 * n)
    got = mob.no_wall_product(kind, r, v, 1.0, 0.35, mode=mode)
    rows = np.concatenate([np.arange(0, n, 97)[:20], rng.choice(n, 20, replace=False)])
    ref = owall.no_wall_product(kind, r, v, 1.0, 0.35, rows=rows)
    assert rel_err(got.reshape(-1, 3)[rows].reshape(-1), ref) <= TOL[mode]


def test_no_wall_force_torque_drop_in(cuda_device):
    rng = np.random.default_rng(3)
    r = rng.uniform(-4.0, 4.0, (200, 3))
    F, T = rng.standard_normal(600), rng.standard_normal(600)
    got = mob.no_wall_mobility_trans_times_force_torque_pycuda(r, F, T, 1.0, 0.3)
    ref = owall.no_wall_product("uf", r, F, 1.0, 0.3) + owall.no_wall_product("ut", r, T, 1.0, 0.3)
    assert rel_err(got, ref) <= 1e-12


def test_free_space_mobility_with_rotation_is_spd(cuda_device):
    rng = np.random.default_rng(4)
    r = rng.normal(0.0, 1.2, (6, 3))
    a = 0.3

    def dense(kind):
        cols = []
        for c in range(18):
            e = np.zeros(18)
            e[c] = 1.0
            cols.append(mob.no_wall_product(kind, r, e, 1.0, a, mode="fp64"))
        return np.stack(cols, axis=1)

    M = np.block([[dense("uf"), dense("ut")], [dense("wf"), dense("wt")]])
    assert np.abs(M - M.T).max() <= 1e-12 * np.abs(M).max()
    assert np.linalg.eigvalsh(0.5 * (M + M.T)).min() > 0
