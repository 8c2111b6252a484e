"""GPU: the near-field augmented preconditioner - two-body mode couplings
(training targets) and the augmented apply against the oracle, the BF16
tensor-core forward and the training gradients against the CPU oracle,
training progress, and what the exact and the learned couplings gain over the
plain block-diagonal preconditioner (with the fallback rule)."""
import numpy as np
import pytest

from conftest import rel_err
from oracle import nearfield as onf
from oracle import rigid as orig
from rigidmultiblobswall_gb300 import nearfield as nf
from rigidmultiblobswall_gb300 import suspensions as S
from rigidmultiblobswall_gb300.rigid import RigidSystem

pytestmark = pytest.mark.gpu


def _pairs_within(locs, lo, hi):
    d = np.linalg.norm(locs[:, None] - locs[None], axis=-1)
    n = locs.shape[0]
    return [(i, j) for i in range(n) for j in range(n) if i != j and lo <= d[i, j] < hi]


def test_pair_coupling_matches_oracle(cuda_device):
    import torch
    from rigidmultiblobswall_gb300 import _native
    rng = np.random.default_rng(3)
    shell = S.icosahedron(1.0)
    a = 0.4
    ns = 3
    cen = np.array([[0.0, 0.0, 1.3], [2.9, 0.4, 1.9], [5.0, 5.0, 1.2], [5.3, 7.6, 2.7], [9.0, 0.0, 3.0],
                    [9.0, 4.5, 1.1]])
    q = S.random_quaternions(rng, 2 * ns)
    r = S.blob_positions(cen, q, shell)
    sys_ = RigidSystem([12] * (2 * ns), 1.0, a)
    sys_.set_configuration(r, cen)
    sys_.build_pc()
    out = torch.empty(ns * 242, dtype=torch.float64, device=sys_.device)
    _native.call("rmw_rigid_pair_coupling", sys_._h, out.data_ptr())
    got = out.cpu().numpy().reshape(ns, 2, 11, 11)
    for s in range(ns):
        ri, rj = r[24 * s:24 * s + 12], r[24 * s + 12:24 * s + 24]
        g01 = onf.pair_coupling(ri, rj, cen[2 * s], cen[2 * s + 1], 1.0, a)
        g10 = onf.pair_coupling(rj, ri, cen[2 * s + 1], cen[2 * s], 1.0, a)
        assert rel_err(got[s, 0], g01) <= 1e-10
        assert rel_err(got[s, 1], g10) <= 1e-10
    sys_.close()


def _dense_suspension(n_bodies, seed):
    susp = S.shells_42_4096(seed=seed, n_bodies=n_bodies)
    sys_ = RigidSystem([42] * susp.n_bodies, susp.eta, susp.a)
    sys_.set_configuration(susp.r_vectors(), susp.locations)
    sys_.build_pc()
    R = np.linalg.norm(susp.shell[0])
    return susp, sys_, R


def test_exact_nearfield_apply_matches_oracle(cuda_device):
    susp, sys_, R = _dense_suspension(12, 31)
    n_ex, n_ln = nf.attach_exact(sys_, 3 * R)
    pairs = _pairs_within(susp.locations, 0.0, 3 * R)
    assert n_ex == len(pairs) > 0 and n_ln == 0
    rng = np.random.default_rng(2)
    x = rng.standard_normal(sys_.size)
    got = sys_.apply_pc(x).cpu().numpy()
    rig = orig.Rigid(susp.r_vectors(), susp.locations, np.arange(13) * 42, susp.eta, susp.a)
    ref = onf.augmented_pc(rig, x, pairs, {})
    assert rel_err(got, ref) <= 1e-10
    nf.detach(sys_)
    assert rel_err(sys_.apply_pc(x).cpu().numpy(), rig.apply_pc(x)) <= 1e-11
    sys_.close()


def test_fp32_apply_of_mixed_solves_matches_oracle(cuda_device):
    """The mixed solves' FP32 preconditioner apply (one kernel plain, two fused kernels augmented) against
    the oracle's FP64 apply: plain, with exact near pairs, and with the periodic images of a periodic box."""
    susp, sys_, R = _dense_suspension(12, 31)
    rig = orig.Rigid(susp.r_vectors(), susp.locations, np.arange(13) * 42, susp.eta, susp.a)
    rng = np.random.default_rng(7)
    for _ in range(2):  # the second call reuses the FP32 copies
        x = rng.standard_normal(sys_.size)
        assert rel_err(sys_.apply_pc(x, mode="mixed").cpu().numpy(), rig.apply_pc(x)) <= 2e-6
    nf.attach_exact(sys_, 3 * R)
    pairs = _pairs_within(susp.locations, 0.0, 3 * R)
    for _ in range(2):
        x = rng.standard_normal(sys_.size)
        ref = onf.augmented_pc(rig, x, pairs, {})
        assert rel_err(sys_.apply_pc(x, mode="mixed").cpu().numpy(), ref) <= 2e-6
        assert rel_err(sys_.apply_pc(x, mode="fp64").cpu().numpy(), ref) <= 1e-10
    # a rebuilt preconditioner refreshes the FP32 copies
    nf.detach(sys_)
    r2 = susp.r_vectors() + 0.05 * rng.standard_normal(susp.r_vectors().shape) * np.array([1.0, 1.0, 0.0])
    sys_.set_configuration(r2, susp.locations)
    sys_.build_pc()
    rig2 = orig.Rigid(r2, susp.locations, np.arange(13) * 42, susp.eta, susp.a)
    x = rng.standard_normal(sys_.size)
    assert rel_err(sys_.apply_pc(x, mode="mixed").cpu().numpy(), rig2.apply_pc(x)) <= 2e-6
    sys_.close()


def test_nearfield_on_independent_suspensions(cuda_device):
    """Two suspensions in one handle that occupy the same region: the exact near field couples bodies of
    the same suspension only.  FP64 and FP32 augmented applies against the oracle suspension by
    suspension, and the batched mixed solve with the augmented preconditioner meets the oracle's
    residual bar in each suspension."""
    susps = [S.shells_42_4096(seed=31, n_bodies=12), S.shells_42_4096(seed=32, n_bodies=12)]
    R = float(np.linalg.norm(susps[0].shell[0]))
    r = np.concatenate([s.r_vectors() for s in susps])
    locs = np.concatenate([s.locations for s in susps])
    sys_ = RigidSystem([42] * 24, susps[0].eta, susps[0].a)
    sys_.set_configuration(r, locs)
    sys_.set_suspensions([12, 12])
    sys_.build_pc()
    n_ex, n_ln = nf.attach_exact(sys_, 3 * R)
    pairs = [_pairs_within(s.locations, 0.0, 3 * R) for s in susps]
    assert n_ex == sum(len(p) for p in pairs) > 0 and n_ln == 0
    n3 = 3 * sys_.n_blobs
    x = np.random.default_rng(8).standard_normal(sys_.size)
    for mode, tol in ((None, 1e-10), ("mixed", 2e-6)):
        got = sys_.apply_pc(x, mode=mode).cpu().numpy()
        for k, s in enumerate(susps):
            rig = orig.Rigid(s.r_vectors(), s.locations, np.arange(13) * 42, s.eta, s.a)
            xk = np.concatenate([x[3 * 504 * k:3 * 504 * (k + 1)], x[n3 + 72 * k:n3 + 72 * (k + 1)]])
            gk = np.concatenate([got[3 * 504 * k:3 * 504 * (k + 1)], got[n3 + 72 * k:n3 + 72 * (k + 1)]])
            assert rel_err(gk, onf.augmented_pc(rig, xk, pairs[k], {})) <= tol, (mode, k)
    FT = np.zeros((24, 6))
    FT[:, 2] = -1.0
    rhs = np.concatenate([np.zeros(n3), -FT.reshape(-1)])
    sol, its, rr, stt = sys_.solve_batched(rhs, tol=1e-8, mode="mixed")
    assert (np.asarray(stt) == 0).all()
    sol = sol.cpu().numpy()
    for k, s in enumerate(susps):
        rig = orig.Rigid(s.r_vectors(), s.locations, np.arange(13) * 42, s.eta, s.a)
        xk = np.concatenate([sol[3 * 504 * k:3 * 504 * (k + 1)], sol[n3 + 72 * k:n3 + 72 * (k + 1)]])
        bk = np.concatenate([np.zeros(3 * 504), -FT[12 * k:12 * (k + 1)].reshape(-1)])
        assert np.linalg.norm(bk - rig.apply(xk)) <= 1.05e-8 * np.linalg.norm(bk)
    nf.detach(sys_)
    sys_.close()


def _random_graph(rng, R=1.0):
    """Three clusters of 3..6 bodies: message edges < 3R, band edges in [2.2R, 6R)."""
    from oracle import mpnn
    cents, cid = [], []
    for k in range(3):
        n = 3 + k
        c = [np.array([0.0, 0.0, 1.5])]
        while len(c) < n:
            p = c[rng.integers(len(c))] + np.array([*rng.uniform(-3.5, 3.5, 2), 0.0])
            p[2] = rng.uniform(1.1, 3.0)
            if all(np.linalg.norm(p - q) >= 2.2 * R for q in c):
                c.append(p)
        c = np.array(c) + np.array([100.0 * k, 0.0, 0.0])
        cents.append(c)
        cid += [k] * n
    cen = np.concatenate(cents)
    arrays = nf.graph_arrays(cen, np.array(cid), R, 3 * R, 2.2 * R, 6 * R)
    og = mpnn.graph_from_positions(cen, np.array(cid), R, 3 * R, 2.2 * R, 6 * R)
    return arrays, og


def test_forward_and_gradients_match_oracle(cuda_device):
    """The message-passing network on the GPU (BF16 tensor-core GEMMs forward and backward) against the
    BF16-emulating oracle: outputs, loss and every weight and bias gradient."""
    from oracle import mpnn
    rng = np.random.default_rng(1)
    arrays, og = _random_graph(rng)
    for k in ("mp_src", "mp_dst", "band_i", "band_j"):
        assert np.array_equal(arrays[k], og[k])
    nb_edges = len(arrays["band_i"])
    T = rng.standard_normal((nb_edges, onf.N_TARGET)).astype(np.float32)
    m = nf.NearfieldModel(body_radius=1.0, cutoff=6.0, seed=5)
    w, b, norm = m.get_params()
    b = (rng.standard_normal(b.size) * 0.1).astype(np.float32)
    norm = np.concatenate([[1.8, 0.3], [0.6, 0.2], [3.0, 1.9, 1.9], [1.4, 0.6, 0.6],
                           rng.uniform(0.5, 2.0, onf.N_TARGET)]).astype(np.float32)
    m.set_params(w, b, norm)
    g = nf.DeviceGraph(arrays, T)
    Y = m.forward(g)
    Yref, _ = mpnn.forward(w, b, norm, og)
    assert rel_err(Y, Yref) <= 5e-3
    gW, gb, loss = m.grad(g)
    gWr, gbr, lossr = mpnn.grad(w, b, norm, og, T / norm[-onf.N_TARGET:])
    assert abs(loss - lossr) <= 2e-3 * lossr
    assert rel_err(gW, gWr) <= 2e-2
    assert rel_err(gb, gbr) <= 2e-2
    # every layer's block of the gradient, not only the whole vector
    ofs = np.cumsum([0] + [ni * no for _, ni, no, _ in mpnn.LAYERS])
    for l in range(len(mpnn.LAYERS)):
        blk = slice(ofs[l], ofs[l + 1])
        assert rel_err(gW[blk], gWr[blk]) <= 5e-2, mpnn.LAYERS[l][0]


@pytest.fixture(scope="module")
def trained(cuda_device):
    shell = S.icosphere_42()
    a = S.blob_radius_of(shell)
    R = np.linalg.norm(shell[0])
    graphs = nf.cluster_training_data(shell, a, 1.0, 512, d_range=(2 * R + 2 * a, 6 * R),
                                      z_range=(1.1 * R, 3 * R), seed=11)
    m = nf.NearfieldModel(body_radius=R, cutoff=6 * R, seed=2)
    hist = m.train(graphs, steps=1500, lr=2e-3)
    return m, hist, R


def test_training_reduces_the_loss(trained):
    m, hist, _ = trained
    assert np.isfinite(hist).all()
    assert hist[-50:].mean() < 0.1 * hist[:10].mean()


def test_learned_apply_matches_oracle(trained):
    """The attached blocks are the network's outputs (on the suspension's own message-passing graph)
    rotated into the lab frame: the apply matches the oracle fed with the network's outputs."""
    m, _, R = trained
    susp, sys_, _ = _dense_suspension(12, 31)
    n_ex, n_ln = m.attach(sys_, exact_cutoff=3 * R)
    locs = susp.locations
    ex = _pairs_within(locs, 0.0, 3 * R)
    ln = _pairs_within(locs, 3 * R, 6 * R)
    assert (n_ex, n_ln) == (len(ex), len(ln)) and n_ln > 0
    _, _, norm = m.get_params()
    tscale = norm[-onf.N_TARGET:]
    arrays = nf.graph_arrays(locs, np.zeros(len(locs), dtype=int), R, 3 * R, 3 * R, 6 * R)
    assert [(int(i), int(j)) for i, j in zip(arrays["band_i"], arrays["band_j"])] == ln
    Y = m.forward(nf.DeviceGraph(arrays)).astype(np.float64) * tscale
    learned = {}
    for k, (i, j) in enumerate(ln):
        d = locs[j] - locs[i]
        rho = np.hypot(d[0], d[1])
        Q = onf.mode_rotation(d[0] / rho, d[1] / rho)
        learned[(i, j)] = Q @ Y[k].reshape(11, 11) @ Q.T
    rng = np.random.default_rng(5)
    x = rng.standard_normal(sys_.size)
    got = sys_.apply_pc(x).cpu().numpy()
    rig = orig.Rigid(susp.r_vectors(), locs, np.arange(13) * 42, susp.eta, susp.a)
    ref = onf.augmented_pc(rig, x, ex, learned)
    assert rel_err(got, ref) <= 1e-4  # a feature may round to a neighbouring BF16 value
    # the mixed solves' FP32 apply of the same couplings: FP32 rounding on top of the FP64 apply
    assert rel_err(sys_.apply_pc(x, mode="mixed").cpu().numpy(), got) <= 2e-6
    only = m.attach(sys_, exact_cutoff=0.0)
    assert only[0] == 0 and only[1] > n_ln
    assert rel_err(sys_.apply_pc(x, mode="mixed").cpu().numpy(), sys_.apply_pc(x).cpu().numpy()) <= 2e-6
    sys_.close()


def test_augmented_preconditioner_gain_and_fallback(trained):
    """A dense suspension (area fraction 0.3, heights in [1.1R, 3R]): the exact near field (< 3R), the
    learned couplings (< 6R), the learned outer band alone (3R..6R) and exact + learned band each need
    fewer GMRES iterations than the plain block-diagonal preconditioner at the same 1e-8 residual; the
    learned band adds a gain on top of the exact near field; a reference that no preconditioner can beat
    triggers the fallback."""
    m, _, R = trained
    susp, sys_, _ = _dense_suspension(96, 21)
    FT = np.zeros((susp.n_bodies, 6))
    FT[:, 2] = -1.0
    rhs = np.concatenate([np.zeros(3 * sys_.n_blobs), -FT.reshape(-1)])
    rhs /= np.linalg.norm(rhs)
    exact = nf.solve_with_fallback(sys_, None, rhs, mode="fp64", exact_cutoff=3 * R)
    plain = exact["plain"]
    ref = (plain["iterations"], plain["relres"])
    learned = nf.solve_with_fallback(sys_, m, rhs, mode="fp64", reference=ref)
    band = nf.solve_with_fallback(sys_, m, rhs, mode="fp64", reference=ref, learned_from=3 * R)
    both = nf.solve_with_fallback(sys_, m, rhs, mode="fp64", reference=ref, exact_cutoff=3 * R)
    print("iterations: plain", plain["iterations"], "exact<3R", exact["augmented"]["iterations"],
          "learned<6R", learned["augmented"]["iterations"], "learned 3R..6R", band["augmented"]["iterations"],
          "exact<3R+learned", both["augmented"]["iterations"])
    assert plain["relres"] <= 1e-8
    for res in (exact, learned, band, both):
        assert res["augmented"]["relres"] <= 1e-8
        assert res["augmented"]["iterations"] < plain["iterations"]
        assert res["kept"] == "augmented"
    assert band["augmented"]["pairs"][0] == 0 and band["augmented"]["pairs"][1] > 0
    assert both["augmented"]["iterations"] < exact["augmented"]["iterations"]
    x_plain = plain["x"].cpu().numpy()
    assert rel_err(both["augmented"]["x"].cpu().numpy(), x_plain) <= 1e-6
    res2 = nf.solve_with_fallback(sys_, m, rhs, mode="fp64", reference=(1, 1e-12))
    assert res2["kept"] == "plain"
    sys_.close()
