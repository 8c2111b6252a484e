"""GPU: the property tests of the reference's mobility/mobility_test.py,
restated for the GPU products (dense matrices assembled column by column
from the C-ABI products):
  * symmetric positive definite translational mobility (:116-130), and the
    full mobility with rotations [[UF, UT], [WF, WT]] (:145-160);
  * zero coupling to a vanishing blob at the wall (:132-143);
  * point-particle limit: the off-diagonal blocks tend to the Blake image
    system as a -> 0 (:70-82, with the full image system)."""
import numpy as np
import pytest

from oracle import wall as owall
from rigidmultiblobswall_gb300 import mobility as mob

pytestmark = pytest.mark.gpu

MODES = [("fp64", 1e-12), ("df64", 1e-12), ("mixed", 1e-6)]


def _dense(kind, r, eta, a, mode):
    import torch
    rt = torch.tensor(np.asarray(r, dtype=np.float64), device="cuda")
    n = rt.shape[0]
    cols = []
    for c in range(3 * n):
        e = torch.zeros(3 * n, dtype=torch.float64, device="cuda")
        e[c] = 1.0
        cols.append(mob.wall_product(kind, rt, e, eta, a, mode=mode))
    return torch.stack(cols, dim=1).cpu().numpy()


@pytest.mark.parametrize("mode,tol", MODES)
def test_translational_mobility_is_spd(cuda_device, mode, tol):
    rng = np.random.default_rng(1)
    r = rng.normal(10.0, 1.0, (5, 3))
    M = _dense("uf", r, 1.0, 1.0, mode)
    assert np.abs(M - M.T).max() <= tol * np.abs(M).max()
    assert np.linalg.eigvalsh(0.5 * (M + M.T)).min() > 0


@pytest.mark.parametrize("mode,tol", MODES)
def test_mobility_with_rotation_is_spd(cuda_device, mode, tol):
    """Near-wall and wall-overlapping blobs included (the damped regime)."""
    rng = np.random.default_rng(2)
    r = rng.normal(0.0, 1.5, (6, 3))
    r[:, 2] = rng.uniform(0.1, 3.0, 6)
    a = 0.25
    M = np.block([[_dense("uf", r, 1.0, a, mode), _dense("ut", r, 1.0, a, mode)],
                  [_dense("wf", r, 1.0, a, mode), _dense("wt", r, 1.0, a, mode)]])
    assert np.abs(M - M.T).max() <= tol * np.abs(M).max()
    assert np.linalg.eigvalsh(0.5 * (M + M.T)).min() > 0


@pytest.mark.parametrize("mode", ["fp64", "df64"])
def test_vanishing_blob_at_the_wall_decouples(cuda_device, mode):
    a = 1e-4
    r = np.array([[0.0, 0.0, a], [1.0, 1.0, 8.0]])
    M = _dense("uf", r, 1.0, a, mode)
    assert np.abs(M[0:3, 3:6]).max() < 1e-6
    assert np.abs(M[3:6, 0:3]).max() < 1e-6


@pytest.mark.parametrize("mode", ["fp64", "df64"])
def test_point_particle_limit_is_blake(cuda_device, mode):
    rng = np.random.default_rng(0)
    r = rng.normal(5.0, 1.0, (4, 3))
    M = _dense("uf", r, 1.0, 1e-4, mode)
    B = owall.blake_point_mobility(r, 1.0)
    off = ~np.kron(np.eye(4, dtype=bool), np.ones((3, 3), dtype=bool))
    assert np.abs(M - B)[off].max() <= 1e-7 * np.abs(B[off]).max()
