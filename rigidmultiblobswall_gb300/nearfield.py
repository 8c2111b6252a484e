"""Near-field augmented preconditioner (GPU): the first Neumann term of the
near inter-body blocks of M on top of the block-diagonal preconditioner, with
exact blob-level couplings for close pairs and network-predicted couplings of
the bodies' 11 low-order modes (translations, rotations, strains) further out.
The network is trained on the GPU on two-body couplings that the plain
method's own machinery computes.

Use::

    sys_.build_pc()
    attach_exact(sys_, cutoff=3 * R)                   # exact near field only
    model = NearfieldModel(body_radius=R, cutoff=6 * R)
    feat, targ = pair_training_data(shell, a, eta, 2048, d_range=(2 * R + 2 * a, 6 * R),
                                    z_range=(1.1 * R, 3 * R))
    model.train(feat, targ, steps=3000)
    model.attach(sys_, exact_cutoff=3 * R)             # exact < 3R <= learned < 6R
    result = solve_with_fallback(sys_, model, rhs, exact_cutoff=3 * R)

The network predicts, for a pair of bodies at horizontal distance d and
heights z_i, z_j (units of the body radius), the 11x11 response G_ij of body
i's modes to body j's mode moments (force, torque, stresslet) in the frame
whose x axis is the horizontal separation; the kernels rotate it into the lab
frame.  Changing only the rigid-body (6x6) part of the preconditioner - even
with the exact many-body mobility - was found to cost GMRES iterations: the
blob rows of the correction must stay consistent, which the Neumann form
guarantees.
"""
import ctypes

import numpy as np

from . import _native
from . import suspensions as S
from .rigid import RigidSystem

N_FEAT, N_MODES = 3, 11
N_TARGET = N_MODES * N_MODES
# rotation by pi about the wall normal in the mode basis (translations,
# rotations, strains (xx-yy), (2zz-xx-yy), xy, xz, yz)
Q_PI = np.diag([-1.0, -1.0, 1.0, -1.0, -1.0, 1.0, 1.0, 1.0, 1.0, -1.0, -1.0])


def _sizes():
    vals = [ctypes.c_int(0) for _ in range(6)]
    _native.call("rmw_nearfield_sizes", *[ctypes.byref(v) for v in vals])
    return [v.value for v in vals]


class NearfieldModel:
    """Owner of an rmw near-field network on the current CUDA device."""

    def __init__(self, body_radius, cutoff, seed=0):
        h = ctypes.c_void_p()
        _native.call("rmw_nearfield_create", ctypes.byref(h), float(body_radius), float(cutoff), int(seed))
        self._h = h
        self.body_radius = float(body_radius)
        self.cutoff = float(cutoff)
        self.n_weights, self.n_biases, self.n_in, self.width, self.n_out, self.n_target = _sizes()

    def __del__(self):
        try:
            if self._h is not None and self._h.value:
                _native.load().rmw_nearfield_destroy(self._h)
        except Exception:
            pass

    # -- parameters --------------------------------------------------------------
    def get_params(self):
        w = np.zeros(self.n_weights, dtype=np.float32)
        b = np.zeros(self.n_biases, dtype=np.float32)
        nrm = np.zeros(2 * N_FEAT + N_TARGET, dtype=np.float32)
        _native.call("rmw_nearfield_get", self._h, w.ctypes.data, b.ctypes.data, nrm.ctypes.data)
        return w, b, nrm

    def set_params(self, w=None, b=None, norm=None):
        def p(x):
            return None if x is None else np.ascontiguousarray(x, dtype=np.float32).ctypes.data
        keep = [np.ascontiguousarray(x, dtype=np.float32) if x is not None else None for x in (w, b, norm)]
        _native.call("rmw_nearfield_set", self._h, *[None if k is None else k.ctypes.data for k in keep])

    def save(self, path):
        w, b, nrm = self.get_params()
        np.savez(path, w=w, b=b, norm=nrm, radius=self.body_radius, cutoff=self.cutoff)

    @classmethod
    def load(cls, path):
        d = np.load(path)
        m = cls(float(d["radius"]), float(d["cutoff"]))
        m.set_params(d["w"], d["b"], d["norm"])
        return m

    # -- network -------------------------------------------------------------------
    def forward(self, X_norm):
        """Outputs (P, 121) for normalised, zero-padded inputs (P, 16) (host)."""
        X = np.ascontiguousarray(X_norm, dtype=np.float32).reshape(-1, self.n_in)
        Y = np.zeros((X.shape[0], N_TARGET), dtype=np.float32)
        _native.call("rmw_nearfield_forward", self._h, X.ctypes.data, X.shape[0], Y.ctypes.data)
        return Y

    def grad(self, X_norm, T):
        """Gradients (weights, biases) and loss of the mean squared error (host)."""
        X = np.ascontiguousarray(X_norm, dtype=np.float32).reshape(-1, self.n_in)
        T = np.ascontiguousarray(T, dtype=np.float32).reshape(-1, N_TARGET)
        gW = np.zeros(self.n_weights, dtype=np.float32)
        gb = np.zeros(self.n_biases, dtype=np.float32)
        loss = np.zeros(1, dtype=np.float32)
        _native.call("rmw_nearfield_grad", self._h, X.ctypes.data, T.ctypes.data, X.shape[0], gW.ctypes.data,
                     gb.ctypes.data, loss.ctypes.data)
        return gW, gb, float(loss[0])

    def train(self, feat, targ, steps=3000, batch=1024, lr=2e-3, seed=1):
        """Adam on device tensors feat (S, 3) and targ (S, 121), float32.  Returns the loss history."""
        import torch
        f = torch.as_tensor(feat, dtype=torch.float32).contiguous()
        t = torch.as_tensor(targ, dtype=torch.float32).contiguous()
        if not f.is_cuda:
            f, t = f.cuda(), t.cuda()
        hist = np.zeros(steps, dtype=np.float32)
        _native.call("rmw_nearfield_train", self._h, f.data_ptr(), t.data_ptr(), f.shape[0], int(steps), int(batch),
                     float(lr), int(seed), hist.ctypes.data, torch.cuda.current_stream(f.device).cuda_stream)
        return hist

    def attach(self, sys_: RigidSystem, exact_cutoff=0.0):
        """Augment sys_'s preconditioner (already built): exact couplings below
        exact_cutoff, learned ones up to the network's cutoff.  Returns the
        (exact, learned) ordered pair counts."""
        return _set(sys_, self._h, exact_cutoff)


def _set(sys_, net, exact_cutoff):
    n = (ctypes.c_int64 * 2)()
    _native.call("rmw_rigid_set_nearfield", sys_._h, net, float(exact_cutoff), n)
    return int(n[0]), int(n[1])


def attach_exact(sys_: RigidSystem, cutoff):
    """Exact near-field couplings only (no network)."""
    return _set(sys_, None, cutoff)


def detach(sys_: RigidSystem):
    """Back to the plain block-diagonal preconditioner."""
    _set(sys_, None, 0.0)


def pair_training_data(shell, a, eta, n_samples, d_range, z_range, seed=0, device="cuda"):
    """Two-body training set from the plain method on the GPU.

    Each sample places body 0 at (0, 0, z0) and body 1 at (d, 0, z1) (random
    orientations, centre distance in d_range, heights in z_range); the
    handle's block-diagonal preconditioner forms each body's M^-1 and
    rmw_rigid_pair_coupling the 11x11 couplings G_01 and G_10.  G_10 is
    turned by pi about the wall normal into its own pair frame.  Returns
    float32 CUDA tensors feat (2S, 3) = (d, z_i, z_j)/R and targ (2S, 121).
    """
    import torch
    rng = np.random.default_rng(seed)
    R = float(np.linalg.norm(shell[0]))
    z0 = np.empty(n_samples)
    z1 = np.empty(n_samples)
    d = np.empty(n_samples)
    k = 0
    while k < n_samples:
        a0, a1 = rng.uniform(*z_range, size=2)
        dist = rng.uniform(*d_range)
        dz = a1 - a0
        if dz * dz >= dist * dist:
            continue
        z0[k], z1[k], d[k] = a0, a1, np.sqrt(dist * dist - dz * dz)
        k += 1
    q = S.random_quaternions(rng, 2 * n_samples)
    cen = np.empty((2 * n_samples, 3))
    cen[0::2] = np.stack([np.zeros(n_samples), np.zeros(n_samples), z0], axis=1)
    cen[1::2] = np.stack([d, np.zeros(n_samples), z1], axis=1)
    r = S.blob_positions(cen, q, shell)
    nb = shell.shape[0]
    sys_ = RigidSystem([nb] * (2 * n_samples), eta, a, device=device)
    try:
        sys_.set_configuration(r, cen)
        sys_.build_pc()
        out = torch.empty(n_samples * 242, dtype=torch.float64, device=sys_.device)
        _native.call("rmw_rigid_pair_coupling", sys_._h, out.data_ptr())
    finally:
        sys_.close()
    G = out.reshape(n_samples, 2, N_MODES, N_MODES)
    Qpi = torch.tensor(Q_PI, dtype=torch.float64, device=out.device)
    G10 = Qpi @ G[:, 1] @ Qpi.T
    feat = torch.tensor(np.concatenate([np.stack([d, z0, z1], 1), np.stack([d, z1, z0], 1)]) / R,
                        dtype=torch.float32, device=out.device)
    targ = torch.cat([G[:, 0].reshape(n_samples, -1), G10.reshape(n_samples, -1)]).to(torch.float32)
    return feat, targ


def solve_with_fallback(sys_, model, rhs, tol=1e-8, restart=60, maxiter=1000, mode="mixed", reference=None,
                        exact_cutoff=0.0):
    """Solve with the augmented preconditioner and keep it only when it helps.

    model may be None (exact near field only).  reference: (iterations,
    relative residual) of the plain block-diagonal solve on the same system, if
    known; otherwise it is measured here.  Returns a dict with both solves and
    the one kept ("plain" or "augmented"); the handle is left with that
    preconditioner.
    """
    import time
    import torch
    if reference is None:
        detach(sys_)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        xp, infop, itp, rrp = sys_.solve(rhs, tol=tol, restart=restart, maxiter=maxiter, mode=mode)
        torch.cuda.synchronize()
        plain = {"iterations": itp, "relres": rrp, "info": infop, "s": time.perf_counter() - t0, "x": xp}
    else:
        plain = {"iterations": reference[0], "relres": reference[1], "info": 0, "s": None, "x": None}
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    pairs = model.attach(sys_, exact_cutoff) if model is not None else attach_exact(sys_, exact_cutoff)
    xl, infol, itl, rrl = sys_.solve(rhs, tol=tol, restart=restart, maxiter=maxiter, mode=mode)
    torch.cuda.synchronize()
    aug = {"iterations": itl, "relres": rrl, "info": infol, "s": time.perf_counter() - t0, "x": xl,
           "pairs": pairs}
    worse = infol != 0 or itl > plain["iterations"] or rrl > max(plain["relres"], tol)
    if worse:
        detach(sys_)
    return {"plain": plain, "augmented": aug, "kept": "plain" if worse else "augmented"}
