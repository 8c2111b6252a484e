"""GPU: launch-shape autotuning of the pair products and CUDA-graph replay of
the solvers' per-iteration operators - both must leave results unchanged."""
import numpy as np
import pytest

from conftest import rel_err
from oracle import wall as owall
from rigidmultiblobswall_gb300 import _native
from rigidmultiblobswall_gb300 import mobility as mob
from rigidmultiblobswall_gb300 import suspensions as S
from rigidmultiblobswall_gb300.rigid import RigidSystem

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind,mode,n", [("uf", "df64", 3000), ("wt", "mixed", 5000), ("ut", "fp64", 1200)])
def test_autotune_picks_a_split_and_keeps_results(cuda_device, kind, mode, n):
    import torch
    mob.autotune_clear()
    c0, tuned0 = mob.autotune_lookup(kind, n, mode)
    assert not tuned0 and c0 >= 1
    res = mob.autotune(kind, n, mode, reps=2)
    sym_ok = True  # the symmetric kernels cover every block in every precision mode
    assert (1 <= res["nchunks"] <= 64 or (sym_ok and res["nchunks"] == -1))
    assert res["ms"] > 0 and res["default_ms"] > 0
    assert res["ms"] <= res["default_ms"] * 1.0001
    c1, tuned1 = mob.autotune_lookup(kind, n, mode)
    assert tuned1 and c1 == (-1 if res["nchunks"] == -1 else min(res["nchunks"], max(1, n // 128)))
    # a size in the same bucket uses the tuned split and still matches the oracle
    rng = np.random.default_rng(9)
    m = n + 7
    r = np.empty((m, 3))
    r[:, :2] = rng.uniform(0, 30, (m, 2))
    r[:, 2] = rng.uniform(1.5, 9, m)
    v = rng.standard_normal(3 * m)
    got = mob.wall_product(kind, torch.tensor(r, device="cuda"), torch.tensor(v, device="cuda"), 1.0, 0.5,
                           mode=mode).cpu().numpy()
    ref = owall.wall_product(kind, r, v, 1.0, 0.5)
    assert rel_err(got, ref) <= (1e-6 if mode == "mixed" else 1e-12)
    mob.autotune_clear()
    assert not mob.autotune_lookup(kind, n, mode)[1]


def _suspension_system(n_bodies=48, seed=5):
    susp = S.shells(n_bodies, S.icosahedron(1.0), seed, 20.0, 1.2, 4.0, a=0.4)
    sys_ = RigidSystem([12] * n_bodies, 1.0, 0.4)
    sys_.set_configuration(susp.r_vectors(), susp.locations)
    sys_.build_pc()
    return susp, sys_


@pytest.mark.parametrize("mode", ["fp64", "mixed"])
def test_graph_replayed_solve_matches_direct(cuda_device, mode):
    susp, sys_ = _suspension_system()
    FT = np.zeros((susp.n_bodies, 6))
    FT[:, 2] = -1.0
    rhs = np.concatenate([np.zeros(3 * sys_.n_blobs), -FT.reshape(-1)])
    try:
        _native.use_graphs(False)
        _native.graph_stats(reset=True)
        x0, info0, it0, rr0 = sys_.solve(rhs, tol=1e-8, mode=mode)
        assert _native.graph_stats() == (0, 0)
        _native.use_graphs(True)
        x1, info1, it1, rr1 = sys_.solve(rhs, tol=1e-8, mode=mode)
        caps, reps = _native.graph_stats(reset=True)
    finally:
        _native.use_graphs(True)
    # device-resident GMRES: one graph launch per restart cycle (every Arnoldi step of the cycle inside it)
    assert caps >= 1 and reps >= 1
    assert info0 == info1 == 0 and it0 == it1
    assert rel_err(x1.cpu().numpy(), x0.cpu().numpy()) <= 1e-13


def test_graph_replayed_batched_solve_and_lanczos(cuda_device):
    import torch
    counts = [9, 20, 14]
    shells = [S.shells(c, S.icosahedron(1.0), 40 + k, 15.0, 1.2, 4.0, a=0.4) for k, c in enumerate(counts)]
    r = np.concatenate([s.r_vectors() for s in shells])
    x = np.concatenate([s.locations for s in shells])
    sys_ = RigidSystem([12] * sum(counts), 1.0, 0.4)
    sys_.set_configuration(r, x)
    sys_.set_suspensions(counts)
    sys_.build_pc(stochastic=True)
    rng = np.random.default_rng(3)
    rhs = rng.standard_normal(sys_.size)
    Z = rng.standard_normal((4, 3 * sys_.n_blobs))
    out = {}
    try:
        for on in (False, True):
            _native.use_graphs(on)
            _native.graph_stats(reset=True)
            sol, it, rr, stt = sys_.solve_batched(rhs, tol=1e-8, mode="mixed")
            noise, itl = sys_.lanczos_batched(Z, factor=1.0, tol=1e-3, mode="mixed")
            out[on] = (sol.cpu().numpy(), np.asarray(it), noise.cpu().numpy(), np.asarray(itl),
                       _native.graph_stats(reset=True))
    finally:
        _native.use_graphs(True)
    assert out[False][4] == (0, 0)
    assert out[True][4][0] >= 2 and out[True][4][1] > 0
    assert (out[True][1] == out[False][1]).all() and (out[True][3] == out[False][3]).all()
    assert rel_err(out[True][0], out[False][0]) <= 1e-13
    assert rel_err(out[True][2], out[False][2]) <= 1e-13
