"""GPU: batched (segmented) products and the lockstep batched GMRES over many
independent suspensions of uneven size, against per-suspension oracle results.

Tolerances as for single suspensions: products 1e-12 (FP64, df64) / 1e-6 (mixed);
every suspension's true FP64 residual <= 1.05e-8 (checked by the oracle operator)
and body velocities within 1e-6 of the oracle's own solve.
"""
import numpy as np
import pytest

from conftest import rel_err
from oracle import rigid as orc
from oracle import wall
from rigidmultiblobswall_gb300 import mobility as mb
from rigidmultiblobswall_gb300 import suspensions as S
from rigidmultiblobswall_gb300.rigid import RigidSystem

pytestmark = pytest.mark.gpu
TOL = {"fp64": 1e-12, "df64": 1e-12, "mixed": 1e-6}


@pytest.mark.parametrize("mode", ["fp64", "df64", "mixed"])
@pytest.mark.parametrize("kind", ["uf", "ut", "wf", "wt"])
def test_batched_product_matches_per_suspension_oracle(cuda_device, kind, mode):
    import torch
    sizes = [1, 0, 77, 300, 129, 1000, 5]
    rs, vs = [], []
    for k, m in enumerate(sizes):
        r, f, eta, a = S.blobs_wall_matvec(max(m, 1), seed=100 + k)
        rs.append(r[:m])
        vs.append(f[:m])
    r = np.concatenate(rs)
    v = np.concatenate(vs)
    r[::17, 2] = 0.3 * a  # some blobs overlap the wall
    off = np.concatenate([[0], np.cumsum(sizes)])
    batch = mb.SuspensionBatch(off)
    out = batch.product(kind, torch.tensor(r, device=cuda_device), torch.tensor(v, device=cuda_device), eta, a,
                        mode=mode).cpu().numpy()
    for k in range(len(sizes)):
        sl = slice(3 * off[k], 3 * off[k + 1])
        if sizes[k] == 0:
            continue
        ref = wall.wall_product(kind, r[off[k]:off[k + 1]], v[off[k]:off[k + 1]], eta, a)
        assert rel_err(out[sl], ref) <= TOL[mode], (k, sizes[k])


@pytest.mark.parametrize("mode", ["fp64", "mixed"])
def test_batched_solve_matches_per_suspension_oracle(cuda_device, mode):
    counts = [3, 1, 7, 2, 5]
    susps = [S.shells_42_256(seed=200 + k, n_bodies=c) for k, c in enumerate(counts)]
    r = np.concatenate([s.r_vectors() for s in susps])
    locs = np.concatenate([s.locations for s in susps])
    eta, a = susps[0].eta, susps[0].a
    nb = sum(counts)
    sys_ = RigidSystem([42] * nb, eta, a)
    sys_.set_configuration(r, locs)
    sys_.set_suspensions(counts)
    sys_.build_pc()
    rng = np.random.default_rng(5)
    FT = rng.standard_normal((nb, 6))
    FT[3] = 0.0  # suspension 1 is the single body 3: zero force -> zero solution
    rhs = np.concatenate([np.zeros(3 * sys_.n_blobs), -FT.reshape(-1)])
    x, it, rr, stt = sys_.solve_batched(rhs, tol=1e-8, mode=mode)
    assert (stt == 0).all() and (rr <= 1e-8).all()
    x = x.cpu().numpy()
    N3 = 3 * sys_.n_blobs
    boff = sys_.suspension_body_offsets
    for k, c in enumerate(counts):
        b0, b1 = boff[k], boff[k + 1]
        bl0, bl1 = sys_.offsets[b0], sys_.offsets[b1]
        o = orc.Rigid(r[bl0:bl1], locs[b0:b1], np.arange(c + 1) * 42, eta, a)
        xk = np.concatenate([x[3 * bl0:3 * bl1], x[N3 + 6 * b0:N3 + 6 * b1]])
        bk = np.concatenate([np.zeros(3 * (bl1 - bl0)), -FT[b0:b1].reshape(-1)])
        nb_ = np.linalg.norm(bk)
        if nb_ == 0:
            assert np.abs(xk).max() == 0.0
            continue
        assert np.linalg.norm(bk - o.apply(xk)) <= 1.05e-8 * nb_
        xo, _, _ = orc.gmres_right(o.apply, o.apply_pc, bk / nb_, tol=1e-8)
        assert rel_err(xk[3 * (bl1 - bl0):], xo[3 * (bl1 - bl0):] * nb_) <= 1e-6


def test_batched_product_rejects_bad_offsets(cuda_device):
    from rigidmultiblobswall_gb300._native import RMWError
    with pytest.raises(RMWError):
        mb.SuspensionBatch([0, 5, 3])
    with pytest.raises(RMWError):
        mb.SuspensionBatch([1, 5])
