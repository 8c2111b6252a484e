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
        true_rr = np.linalg.norm(bk - o.apply(xk)) / nb_
        assert true_rr <= 1.05e-8
        # the reported residual (a recurrence once it is small) is the true one
        assert abs(rr[k] - true_rr) <= 1e-9, (k, rr[k], true_rr)
        xo, _, _ = orc.gmres_right(o.apply, o.apply_pc, bk / nb_, tol=1e-8)
        assert rel_err(xk[3 * (bl1 - bl0):], xo[3 * (bl1 - bl0):] * nb_) <= 1e-6


def test_batched_product_rejects_bad_offsets(cuda_device):
    from rigidmultiblobswall_gb300._native import RMWError
    with pytest.raises(RMWError):
        mb.SuspensionBatch([0, 5, 3])
    with pytest.raises(RMWError):
        mb.SuspensionBatch([1, 5])


@pytest.mark.parametrize("nrhs", [1, 3, 8, 11, 16, 19])
def test_multi_rhs_product_matches_single_products(cuda_device, nrhs):
    import torch
    r, _, eta, a = S.blobs_wall_matvec(900, seed=31)
    r[::13, 2] = 0.3 * a
    rng = np.random.default_rng(nrhs)
    V = rng.standard_normal((nrhs, r.size))
    rt = torch.tensor(r, device=cuda_device)
    Y = mb.uf_multi(rt, torch.tensor(V, device=cuda_device), eta, a).cpu().numpy()
    for q in range(nrhs):
        assert rel_err(Y[q], wall.wall_product("uf", r, V[q], eta, a)) <= 1e-6
    # segmented: two suspensions in one array
    off = np.array([0, 400, 900])
    Yb = mb.uf_multi(rt, torch.tensor(V, device=cuda_device), eta, a, batch=mb.SuspensionBatch(off)).cpu().numpy()
    for q in range(nrhs):
        for k in range(2):
            sl = slice(3 * off[k], 3 * off[k + 1])
            ref = wall.wall_product("uf", r[off[k]:off[k + 1]], V[q][sl], eta, a)
            assert rel_err(Yb[q][sl], ref) <= 1e-6


def _batched_system(counts, seed0):
    susps = [S.shells_42_256(seed=seed0 + k, n_bodies=c) for k, c in enumerate(counts)]
    r = np.concatenate([s.r_vectors() for s in susps])
    locs = np.concatenate([s.locations for s in susps])
    eta, a = susps[0].eta, susps[0].a
    sys_ = RigidSystem([42] * sum(counts), eta, a)
    sys_.set_configuration(r, locs)
    sys_.set_suspensions(counts)
    return sys_, r, locs, eta, a


def test_batched_lanczos_matches_per_suspension_oracle(cuda_device):
    counts = [2, 5, 1, 3]
    sys_, r, locs, eta, a = _batched_system(counts, 300)
    sys_.build_pc(stochastic=True)
    nrhs = 3
    Z = np.random.default_rng(9).standard_normal((nrhs, 3 * sys_.n_blobs))
    factor = np.sqrt(2.0 / 1e-3)
    noise, it = sys_.lanczos_batched(Z, factor=factor, tol=1e-3, mode="fp64")
    noise = noise.cpu().numpy()
    boff = sys_.suspension_body_offsets
    for k, c in enumerate(counts):
        bl0, bl1 = sys_.offsets[boff[k]], sys_.offsets[boff[k + 1]]
        o = orc.Rigid(r[bl0:bl1], locs[boff[k]:boff[k + 1]], np.arange(c + 1) * 42, eta, a)
        for q in range(nrhs):
            nz, itk = orc.lanczos(o.mobility_pc, Z[q][3 * bl0:3 * bl1], factor=factor, tol=1e-3)
            nz = o.P_inv_mult(nz)
            assert it[q, k] == itk
            assert rel_err(noise[q][3 * bl0:3 * bl1], nz) <= 1e-8
    # mixed precision (multi-right-hand-side kernel) against the FP64 result
    noise32, it32 = sys_.lanczos_batched(Z, factor=factor, tol=1e-3, mode="mixed")
    assert np.abs(it32 - it).max() <= 1
    assert rel_err(noise32.cpu().numpy(), noise) <= 1e-4
    # the FP32-built stochastic preconditioner, whose FP32 copy of L^-1 the multi-vector multiplies read
    sys_.build_pc(stochastic=True, mode="mixed")
    noise32b, it32b = sys_.lanczos_batched(Z, factor=factor, tol=1e-3, mode="mixed")
    assert np.abs(it32b - it).max() <= 1
    assert rel_err(noise32b.cpu().numpy(), noise) <= 1e-4
