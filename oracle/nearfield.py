"""Oracle (test infrastructure only) for the near-field augmented
preconditioner: numpy restatements of
* BF16 rounding (round to nearest even) and the activation the network uses
  (its forward and backward passes are restated in oracle/mpnn.py);
* the two-body mode coupling G_ij (11 modes: translations, rotations,
  strains) used as training target;
* the augmented preconditioner apply y = P0 x - P0 [v; 0] with
  v_i = sum_j M_ij lambda_j (exact pairs) + X_i G_ij X_j^T lambda_j (learned
  pairs), on top of the block-diagonal oracle (rigid.Rigid.apply_pc)."""
import numpy as np

from . import wall

N_MODES = 11
N_TARGET = N_MODES * N_MODES


def bf16(x):
    x = np.ascontiguousarray(x, dtype=np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).reshape(x.shape)


def silu(z):
    return z / (1.0 + np.exp(-z))


def silu_grad(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


_S2, _S6 = 1.0 / np.sqrt(2.0), 1.0 / np.sqrt(6.0)
STRAINS = [np.diag([_S2, -_S2, 0.0]), np.diag([-_S6, -_S6, 2.0 * _S6]),
           np.array([[0, _S2, 0], [_S2, 0, 0], [0, 0, 0]]), np.array([[0, 0, _S2], [0, 0, 0], [_S2, 0, 0]]),
           np.array([[0, 0, 0], [0, 0, _S2], [0, _S2, 0]])]


def modes(r_body, centre):
    """X (3n x 11): blob velocities of the unit translations, rotations (e_c x d)
    and strains E_k d of one body."""
    d = np.asarray(r_body, dtype=np.float64).reshape(-1, 3) - np.asarray(centre)
    n = d.shape[0]
    X = np.zeros((3 * n, N_MODES))
    for c in range(3):
        X[c::3, c] = 1.0
    for c in range(3):
        e = np.zeros(3)
        e[c] = 1.0
        X[:, 3 + c] = np.cross(e, d).reshape(-1)
    for k, E in enumerate(STRAINS):
        X[:, 6 + k] = (d @ E.T).reshape(-1)
    return X


def mode_rotation(c, s):
    """diag(Rz, Rz, R5) for the rotation about z with cos c, sin s."""
    Rz = np.array([[c, -s, 0.0], [s, c, 0.0], [0.0, 0.0, 1.0]])
    Q = np.zeros((N_MODES, N_MODES))
    Q[:3, :3] = Rz
    Q[3:6, 3:6] = Rz
    for l, El in enumerate(STRAINS):
        T = Rz @ El @ Rz.T
        for k, Ek in enumerate(STRAINS):
            Q[6 + k, 6 + l] = (Ek * T).sum()
    return Q


def pair_coupling(r_i, r_j, c_i, c_j, eta, a):
    """G_ij = (X_i^T M_i^-1 X_i)^-1 X_i^T M_i^-1 M_ij M_j^-1 X_j (X_j^T M_j^-1 X_j)^-1 (11 x 11)."""
    r_i = np.asarray(r_i, dtype=np.float64).reshape(-1, 3)
    r_j = np.asarray(r_j, dtype=np.float64).reshape(-1, 3)
    m = 3 * r_i.shape[0]
    M = wall.dense_mobility(np.concatenate([r_i, r_j]), eta, a)
    Mi_inv = np.linalg.inv(M[:m, :m])
    Mj_inv = np.linalg.inv(M[m:, m:])
    Xi, Xj = modes(r_i, c_i), modes(r_j, c_j)
    Ai, Aj = Mi_inv @ Xi, Mj_inv @ Xj
    return np.linalg.solve(Xi.T @ Ai, Ai.T @ M[:m, m:] @ Aj @ np.linalg.inv(Xj.T @ Aj))


def augmented_pc(rig, x, exact_pairs, learned):
    """y = P0 x - P0 [v; 0] on the oracle rigid system rig (rigid.Rigid):
    exact_pairs: list of ordered (i, j); learned: dict (i, j) -> G_ij (lab frame)."""
    off = rig.offsets
    y = rig.apply_pc(x)
    lam = y[:3 * rig.N]
    v = np.zeros(3 * rig.N + 6 * rig.Nb)
    for (i, j) in exact_pairs:
        ri, rj = rig.r[off[i]:off[i + 1]], rig.r[off[j]:off[j + 1]]
        m = 3 * ri.shape[0]
        M = wall.dense_mobility(np.concatenate([ri, rj]), rig.eta, rig.a)
        v[3 * off[i]:3 * off[i + 1]] += M[:m, m:] @ lam[3 * off[j]:3 * off[j + 1]]
    for (i, j), G in learned.items():
        Xi = modes(rig.r[off[i]:off[i + 1]], rig.locs[i])
        Xj = modes(rig.r[off[j]:off[j + 1]], rig.locs[j])
        v[3 * off[i]:3 * off[i + 1]] += Xi @ (G @ (Xj.T @ lam[3 * off[j]:3 * off[j + 1]]))
    return y - rig.apply_pc(v)
