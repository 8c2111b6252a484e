"""CPU: the near-field network oracle's gradient against finite differences
(no rounding), so that it can serve as the check of the GPU kernels."""
import numpy as np

from oracle import nearfield as onf


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    nw = sum(i * o for i, o in onf.LAYERS)
    w = rng.standard_normal(nw) * 0.2
    b = rng.standard_normal(3 * onf.WIDTH + onf.N_OUT) * 0.1
    X = np.zeros((8, onf.N_IN))
    X[:, :3] = rng.standard_normal((8, 3))
    T = rng.standard_normal((8, onf.N_TARGET))
    saved = onf.bf16
    onf.bf16 = lambda x: np.asarray(x, dtype=np.float64)  # exact arithmetic for the check
    try:
        gW, gb, loss = onf.grad(w, b, X, T)
        for idx in (0, 5, 200, 1500, nw - 3):
            e = np.zeros(nw)
            e[idx] = 1e-6
            fd = (onf.grad(w + e, b, X, T)[2] - onf.grad(w - e, b, X, T)[2]) / 2e-6
            assert abs(fd - gW[idx]) <= 1e-6 * max(1.0, abs(fd))
        for idx in (0, 70, 3 * onf.WIDTH + 5):
            e = np.zeros(b.size)
            e[idx] = 1e-6
            fd = (onf.grad(w, b + e, X, T)[2] - onf.grad(w, b - e, X, T)[2]) / 2e-6
            assert abs(fd - gb[idx]) <= 1e-6 * max(1.0, abs(fd))
    finally:
        onf.bf16 = saved


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
