"""CPU: the near-field network oracle's gradient against finite differences
(no rounding), so that it can serve as the check of the GPU kernels."""
import numpy as np

from oracle import nearfield as onf


def _graph(rng):
    from oracle import mpnn
    cen = np.array([[0.0, 0.0, 1.3], [2.4, 0.5, 1.9], [4.6, -0.4, 1.2], [2.0, 3.1, 2.6],
                    [40.0, 0.0, 1.5], [42.9, 1.0, 1.1]])
    return mpnn.graph_from_positions(cen, [0, 0, 0, 0, 1, 1], 1.0, 3.0, 2.2, 6.0)


def test_mpnn_oracle_gradient_matches_finite_differences():
    """The message-passing oracle's backward pass (the check of the GPU training kernels) against central
    differences of its loss, with the BF16 rounding switched off."""
    from oracle import mpnn
    rng = np.random.default_rng(0)
    g = _graph(rng)
    assert len(g["mp_src"]) > 0 and len(g["band_i"]) > 0
    nw, nb = mpnn.sizes()
    w = rng.standard_normal(nw) * 0.15
    b = rng.standard_normal(nb) * 0.1
    norm = np.concatenate([[1.8, 0.2], [0.5, 0.1], [3.0, 1.8, 1.8], [1.5, 0.5, 0.5], np.ones(mpnn.TARGET)])
    T = rng.standard_normal((len(g["band_i"]), mpnn.TARGET))
    gW, gb, loss = mpnn.grad(w, b, norm, g, T, rounding=False)
    ofs = np.cumsum([0] + [ni * no for _, ni, no, _ in mpnn.LAYERS])
    picks = [ofs[0] + 1, ofs[1] + 3, ofs[1] + 70, ofs[2] + 5, ofs[2] + 100, ofs[5] + 7, ofs[7] + 130,
             ofs[8] + 9, ofs[9] + 11]
    for idx in picks:
        e = np.zeros(nw)
        e[idx] = 1e-6
        fd = (mpnn.grad(w + e, b, norm, g, T, rounding=False)[2] -
              mpnn.grad(w - e, b, norm, g, T, rounding=False)[2]) / 2e-6
        assert abs(fd - gW[idx]) <= 1e-6 * max(1.0, abs(fd)), idx
    bofs = np.cumsum([0] + [no for _, _, no, _ in mpnn.LAYERS])
    for idx in (bofs[0] + 2, bofs[2] + 3, bofs[6] + 1, bofs[9] + 4):
        e = np.zeros(nb)
        e[idx] = 1e-6
        fd = (mpnn.grad(w, b + e, norm, g, T, rounding=False)[2] -
              mpnn.grad(w, b - e, norm, g, T, rounding=False)[2]) / 2e-6
        assert abs(fd - gb[idx]) <= 1e-6 * max(1.0, abs(fd)), idx


def test_mpnn_messages_stay_inside_clusters_and_change_predictions():
    """Edges join bodies of one cluster only; a body added near a pair (a message neighbour, not itself
    in the pair) changes the pair's prediction - the network sees neighbourhoods."""
    from oracle import mpnn
    rng = np.random.default_rng(1)
    g = _graph(rng)
    cl = np.array([0, 0, 0, 0, 1, 1])
    assert (cl[g["mp_src"]] == cl[g["mp_dst"]]).all() and (cl[g["band_i"]] == cl[g["band_j"]]).all()
    assert (g["mp_dst"][g["mp_rev"]] == g["mp_src"]).all() and (g["band_i"][g["band_rev"]] == g["band_j"]).all()
    nw, nb = mpnn.sizes()
    w = rng.standard_normal(nw) * 0.2
    b = rng.standard_normal(nb) * 0.1
    norm = np.concatenate([[1.8, 0.2], [0.5, 0.1], [3.0, 1.8, 1.8], [1.5, 0.5, 0.5], np.ones(mpnn.TARGET)])
    cen2 = np.array([[0.0, 0.0, 1.3], [4.0, 0.0, 1.3]])
    two = mpnn.graph_from_positions(cen2, [0, 0], 1.0, 3.0, 2.2, 6.0)
    three = mpnn.graph_from_positions(np.vstack([cen2, [[2.0, 2.0, 1.3]]]), [0, 0, 0], 1.0, 3.0, 2.2, 6.0)
    y2, _ = mpnn.forward(w, b, norm, two, rounding=False)
    y3, _ = mpnn.forward(w, b, norm, three, rounding=False)
    k = [e for e in range(len(three["band_i"])) if (three["band_i"][e], three["band_j"][e]) == (0, 1)][0]
    assert np.abs(y3[k] - y2[0]).max() > 1e-6


def test_bf16_rounding_is_round_to_nearest_even():
    x = np.array([1.0, 1.00390625, 1.005859375, -2.5, 3.0e-3], dtype=np.float32)
    y = onf.bf16(x)
    assert y[0] == 1.0 and y[1] == 1.0  # tie to even
    assert y[2] == np.float32(1.0078125)
    assert y[3] == -2.5


def test_mode_coupling_rotates_with_the_pair():
    """Turning a two-body configuration about the wall normal by theta turns
    the mode coupling by Q(theta) = diag(Rz, Rz, R5): the covariance the
    network's pair frame relies on."""
    from rigidmultiblobswall_gb300 import suspensions as S
    rng = np.random.default_rng(4)
    shell = S.icosahedron(1.0)
    a = 0.4
    q = S.random_quaternions(rng, 2)
    c0, c1 = np.array([0.3, -0.2, 1.6]), np.array([2.1, 1.5, 2.4])
    r0 = S.blob_positions(c0[None], q[0:1], shell)
    r1 = S.blob_positions(c1[None], q[1:2], shell)
    G = onf.pair_coupling(r0, r1, c0, c1, 1.0, a)
    th = 0.7
    c, s = np.cos(th), np.sin(th)
    Rz = np.array([[c, -s, 0], [s, c, 0], [0, 0, 1.0]])
    Gr = onf.pair_coupling(r0 @ Rz.T, r1 @ Rz.T, Rz @ c0, Rz @ c1, 1.0, a)
    Q = onf.mode_rotation(c, s)
    assert np.allclose(Q @ Q.T, np.eye(11), atol=1e-14)
    assert np.abs(Gr - Q @ G @ Q.T).max() <= 1e-10 * np.abs(G).max()
    # pi rotation is the diagonal sign pattern the training data uses
    from rigidmultiblobswall_gb300.nearfield import Q_PI
    assert np.allclose(onf.mode_rotation(-1.0, 0.0), np.diag(Q_PI), atol=1e-15) or \
        np.allclose(onf.mode_rotation(-1.0, 0.0), Q_PI, atol=1e-15)


def test_translation_block_of_far_pair_is_stokeslet_like():
    """Far from each other and very far from the wall, the translation block
    of G approaches the Oseen coupling of the two centres."""
    from rigidmultiblobswall_gb300 import suspensions as S
    shell = S.icosahedron(1.0)
    a = 0.4
    c0, c1 = np.array([0.0, 0.0, 5000.0]), np.array([12.0, 0.0, 5000.0])
    r0 = shell + c0
    r1 = shell + c1
    G = onf.pair_coupling(r0, r1, c0, c1, 1.0, a)
    # Oseen tensor of the separation, 1/(8 pi eta d) (I + e e)
    d = 12.0
    oseen = (np.eye(3) + np.diag([1.0, 0.0, 0.0])) / (8 * np.pi * d)
    assert np.abs(G[:3, :3] - oseen).max() <= 0.05 * np.abs(oseen).max()
