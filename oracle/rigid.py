"""Oracle (test infrastructure only): numpy restatement of the reference's
rigid-body mobility solve and Lanczos noise, on top of the C wall products.

* K_bodies, K_mult, KT_mult        multi_bodies/multi_bodies.py:306-371, body/body.py:81-115
* linear_operator                  multi_bodies/multi_bodies.py:424-471
* block_pc                         multi_bodies/multi_bodies.py:752-903 (Cholesky, M^-1, pinv(K^T M^-1 K))
* det_stoch                        multi_bodies/multi_bodies.py:480-618 (mobility_pc, P_inv_mult)
* gmres_right                      general_application_utils.py:514-635 (right PC, zero initial guess,
                                   restarted, true-residual stop) - an own numpy GMRES, not scipy's
* lanczos                          stochastic_forcing/stochastic_forcing.py:112-264
* em_step                          quaternion_integrator_multi_bodies.py:262-322 (no wall-crossing retry)

Only tests, smoke() and bench.py's CPU legs use it.
"""
import numpy as np
import scipy.linalg

from . import wall


def K_bodies(r, locs, offsets):
    Ks = []
    for b in range(len(offsets) - 1):
        d = r[offsets[b]:offsets[b + 1]] - locs[b]
        nb = d.shape[0]
        K = np.zeros((3 * nb, 6))
        K[0::3, 0] = 1.0
        K[1::3, 1] = 1.0
        K[2::3, 2] = 1.0
        rot = np.zeros((nb, 3, 3))
        rot[:, 0, 1] = d[:, 2]
        rot[:, 0, 2] = -d[:, 1]
        rot[:, 1, 0] = -d[:, 2]
        rot[:, 1, 2] = d[:, 0]
        rot[:, 2, 0] = d[:, 1]
        rot[:, 2, 1] = -d[:, 0]
        K[:, 3:] = rot.reshape(3 * nb, 3)
        Ks.append(K)
    return Ks


def K_mult(Ks, offsets, u):
    out = np.empty(3 * offsets[-1])
    for b, K in enumerate(Ks):
        out[3 * offsets[b]:3 * offsets[b + 1]] = K @ u[6 * b:6 * b + 6]
    return out


def KT_mult(Ks, offsets, lam):
    out = np.empty(6 * len(Ks))
    for b, K in enumerate(Ks):
        out[6 * b:6 * b + 6] = K.T @ lam[3 * offsets[b]:3 * offsets[b + 1]]
    return out


class Rigid:
    """One suspension: blob positions r (N,3), body locations (Nb,3), blob offsets."""

    def __init__(self, r, locs, offsets, eta, a, wall_present=True):
        self.r = np.ascontiguousarray(r, dtype=np.float64).reshape(-1, 3)
        self.locs = np.asarray(locs, dtype=np.float64).reshape(-1, 3)
        self.offsets = np.asarray(offsets, dtype=np.int64)
        self.eta, self.a = float(eta), float(a)
        self.N = int(self.offsets[-1])
        self.Nb = len(self.offsets) - 1
        self.size = 3 * self.N + 6 * self.Nb
        self.Ks = K_bodies(self.r, self.locs, self.offsets)
        self._pc = None
        self.wall_present = wall_present  # False: free space (the *_no_wall implementations)

    def mobility(self, v):
        if not self.wall_present:
            return wall.no_wall_product("uf", self.r, v, self.eta, self.a)
        return wall.wall_product("uf", self.r, v, self.eta, self.a)

    def apply(self, x):
        n3 = 3 * self.N
        y = np.empty(self.size)
        y[:n3] = self.mobility(x[:n3]) - K_mult(self.Ks, self.offsets, x[n3:])
        y[n3:] = -KT_mult(self.Ks, self.offsets, x[:n3])
        return y

    def build_pc(self):
        minv, nmat, lfac, linv = [], [], [], []
        for b in range(self.Nb):
            rb = self.r[self.offsets[b]:self.offsets[b + 1]]
            M = (wall.dense_mobility(rb, self.eta, self.a) if self.wall_present
                 else wall.no_wall_dense(rb, self.eta, self.a))
            U, lower = scipy.linalg.cho_factor(M)
            U = np.triu(U)
            Uinv = scipy.linalg.solve_triangular(U, np.eye(M.shape[0]))
            Mi = Uinv @ Uinv.T
            K = self.Ks[b]
            minv.append(Mi)
            nmat.append(np.linalg.pinv(K.T @ Mi @ K))
            lfac.append(U.T)
            linv.append(Uinv.T)
        self._pc = (minv, nmat, lfac, linv)

    def apply_pc(self, x):
        if self._pc is None:
            self.build_pc()
        minv, nmat, _, _ = self._pc
        n3 = 3 * self.N
        y = np.empty(self.size)
        for b in range(self.Nb):
            s = x[3 * self.offsets[b]:3 * self.offsets[b + 1]]
            F = x[n3 + 6 * b:n3 + 6 * b + 6]
            lt = minv[b] @ s
            Y = nmat[b] @ (-F - self.Ks[b].T @ lt)
            y[3 * self.offsets[b]:3 * self.offsets[b + 1]] = minv[b] @ (s + self.Ks[b] @ Y)
            y[n3 + 6 * b:n3 + 6 * b + 6] = Y
        return y

    def mobility_pc(self, w):
        """L^-1 M L^-T w per body blocks (P = L^-T)."""
        if self._pc is None:
            self.build_pc()
        _, _, _, linv = self._pc
        t = np.empty_like(w)
        for b in range(self.Nb):
            sl = slice(3 * self.offsets[b], 3 * self.offsets[b + 1])
            t[sl] = linv[b].T @ w[sl]
        m = self.mobility(t)
        out = np.empty_like(w)
        for b in range(self.Nb):
            sl = slice(3 * self.offsets[b], 3 * self.offsets[b + 1])
            out[sl] = linv[b] @ m[sl]
        return out

    def P_inv_mult(self, w):
        if self._pc is None:
            self.build_pc()
        _, _, lfac, _ = self._pc
        out = np.empty_like(w)
        for b in range(self.Nb):
            sl = slice(3 * self.offsets[b], 3 * self.offsets[b + 1])
            out[sl] = lfac[b] @ w[sl]
        return out


def gmres_right(A, P, b, tol=1e-8, restart=60, maxiter=1000):
    """Right-preconditioned restarted GMRES, zero initial guess, stops when the
    true residual |b - A x| <= tol |b|.  Returns (x, iterations, rel residual)."""
    n = b.size
    bn = np.linalg.norm(b)
    x = np.zeros(n)
    if bn == 0:
        return x, 0, 0.0
    r = b.copy()
    it = 0
    while True:
        beta = np.linalg.norm(r)
        V = np.zeros((restart + 1, n))
        H = np.zeros((restart + 1, restart))
        V[0] = r / beta
        g = np.zeros(restart + 1)
        g[0] = beta
        cs, sn = np.zeros(restart), np.zeros(restart)
        j_done = 0
        for j in range(restart):
            w = A(P(V[j]))
            for _ in range(2):  # CGS2
                h = V[:j + 1] @ w
                w = w - V[:j + 1].T @ h
                H[:j + 1, j] += h
            H[j + 1, j] = np.linalg.norm(w)
            if H[j + 1, j] > 0:
                V[j + 1] = w / H[j + 1, j]
            for q in range(j):
                t = cs[q] * H[q, j] + sn[q] * H[q + 1, j]
                H[q + 1, j] = -sn[q] * H[q, j] + cs[q] * H[q + 1, j]
                H[q, j] = t
            den = np.hypot(H[j, j], H[j + 1, j])
            cs[j], sn[j] = (1.0, 0.0) if den == 0 else (H[j, j] / den, H[j + 1, j] / den)
            H[j, j] = cs[j] * H[j, j] + sn[j] * H[j + 1, j]
            H[j + 1, j] = 0.0
            g[j + 1] = -sn[j] * g[j]
            g[j] = cs[j] * g[j]
            it += 1
            j_done = j + 1
            if abs(g[j + 1]) <= tol * bn or it >= maxiter:
                break
        y = scipy.linalg.solve_triangular(H[:j_done, :j_done], g[:j_done])
        x = x + P(V[:j_done].T @ y)
        r = b - A(x)
        rel = np.linalg.norm(r) / bn
        if rel <= tol or it >= maxiter:
            return x, it, rel


def lanczos(mult, z, factor=1.0, tol=1e-6, max_iter=1000):
    """factor * M^(1/2) z, returns (noise, iterations) (stochastic_forcing.py:112-264)."""
    dim = z.size
    v = [z / np.linalg.norm(z)]
    vn = np.linalg.norm(z)
    hd, hs = [], []
    noise_old = np.zeros(dim)
    noise = noise_old
    for i in range(max_iter + 1):
        w = mult(v[i])
        if i > 0:
            w = w - hs[i - 1] * v[i - 1]
        hd.append(w @ v[i])
        w = w - hd[i] * v[i]
        hs.append(np.linalg.norm(w))
        if hs[i] > 0:
            w = w / hs[i]
        else:
            w[0] = 1.0
        T = np.diag(hd) + np.diag(hs[:i], -1) + np.diag(hs[:i], 1)
        lam, Q = np.linalg.eigh(T)
        sq = np.sqrt(np.maximum(lam, 0.0))
        V = np.array(v)
        noise = V.T @ (Q @ (vn * factor * sq * Q[0, :]))
        for row in V:
            w = w - (row @ w) * row
        v.append(w)
        if i > 0:
            if np.linalg.norm(noise - noise_old) / max(np.linalg.norm(noise_old), np.finfo(float).eps) < tol:
                return noise, i
        noise_old = noise.copy()
    return noise, max_iter


def quat_mult(q1, q2):
    s1, p1 = q1[0], q1[1:]
    s2, p2 = q2[0], q2[1:]
    return np.concatenate([[s1 * s2 - p1 @ p2], s1 * p2 + s2 * p1 + np.cross(p1, p2)])


def quat_from_rotation(phi):
    n = np.linalg.norm(phi)
    if n == 0:
        return np.array([1.0, 0.0, 0.0, 0.0])
    return np.concatenate([[np.cos(n / 2)], np.sin(n / 2) * phi / n])


def em_update(locs, quats, vel, dt):
    nl = locs + vel.reshape(-1, 6)[:, :3] * dt
    nq = np.array([quat_mult(quat_from_rotation(w * dt), q) for w, q in zip(vel.reshape(-1, 6)[:, 3:], quats)])
    return nl, nq
