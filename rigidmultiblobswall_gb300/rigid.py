"""Device-resident rigid-body suspension: a thin owner of an ``rmw_rigid`` handle.

All vectors are CUDA float64 torch tensors.  Saddle-point vectors have the
layout of the reference's linear_operator_rigid (multi_bodies/multi_bodies.py:424-471):
``[lambda (3N); U (6 Nb)]`` with ``U_b = (velocity, angular velocity)``.
"""
import ctypes

import numpy as np

from . import _native

MODES = {"fp64": _native.MODE_FP64, "mixed": _native.MODE_MIXED, "df64": _native.MODE_DF64}


def _mode(mode):
    if mode not in MODES:
        raise ValueError("mode must be 'fp64', 'df64' or 'mixed'")
    return MODES[mode]


def _dev(x, device):
    import torch
    if type(x) is torch.Tensor and x.dtype == torch.float64 and x.device == device and x.is_contiguous():
        return x  # already a contiguous float64 tensor on the suspension's device
    t = torch.as_tensor(x, dtype=torch.float64, device=device)
    return t.contiguous()


class RigidSystem:
    """One suspension of rigid multiblob bodies on one GPU.

    blobs_per_body: sequence of blob counts (body b owns the next n_b blobs).
    wall: False for free-space (no-wall) mobilities.
    """

    def __init__(self, blobs_per_body, eta, a, periodic_length=None, device="cuda", wall=True):
        import torch
        self.device = torch.device(device)
        if self.device.index is None:
            self.device = torch.device("cuda", torch.cuda.current_device())
        counts = np.asarray(blobs_per_body, dtype=np.int64).reshape(-1)
        if counts.size == 0 or (counts <= 0).any():
            raise ValueError("every body needs at least one blob")
        self.blobs_per_body = counts
        self.offsets = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
        self.n_bodies = int(counts.size)
        self.n_blobs = int(self.offsets[-1])
        self.eta = float(eta)
        self.a = float(a)
        self.L = np.zeros(3) if periodic_length is None else np.ascontiguousarray(periodic_length, dtype=np.float64)
        self.stream = torch.cuda.current_stream(self.device)
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _native.call("rmw_rigid_create", ctypes.byref(h), self.n_bodies,
                         self.offsets.ctypes.data_as(ctypes.c_void_p), self.eta, self.a,
                         self.L.ctypes.data_as(ctypes.c_void_p), self.stream.cuda_stream)
        self._h = h
        self.size = 3 * self.n_blobs + 6 * self.n_bodies
        self.wall = True
        if not wall:
            self.set_wall(False)

    def set_wall(self, wall):
        """Mobility above the wall (True) or in free space (False, the reference's
        *_no_wall implementations).  Invalidates the preconditioners."""
        _native.call("rmw_rigid_set_wall", self._h, 1 if wall else 0)
        self.wall = bool(wall)

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            _native.load().rmw_rigid_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- state -------------------------------------------------------------
    def set_configuration(self, r_blobs, x_bodies):
        """Blob positions (N,3) and body locations (Nb,3); invalidates the preconditioner."""
        import torch
        r = _dev(r_blobs, self.device).reshape(-1, 3)
        x = _dev(x_bodies, self.device).reshape(-1, 3)
        if r.shape[0] != self.n_blobs or x.shape[0] != self.n_bodies:
            raise ValueError("configuration sizes do not match the suspension")
        self._r, self._x = r, x  # keep alive until the copy is done
        with torch.cuda.device(self.device):
            _native.call("rmw_rigid_set_configuration", self._h, r.data_ptr(), x.data_ptr())

    def build_pc(self, stochastic=False, mode="fp64"):
        """Block-diagonal preconditioner(s) at the current configuration; mode
        'mixed' factorises the body blocks in FP32 for the mixed solves."""
        import torch
        with torch.cuda.device(self.device):
            _native.call("rmw_rigid_build_pc_mode", self._h, 1 if stochastic else 0, _mode(mode))

    # -- operators -------------------------------------------------------------
    def _out(self, n):
        import torch
        return torch.empty(n, dtype=torch.float64, device=self.device)

    def apply(self, x, mode="fp64"):
        """linear_operator_rigid: [M l - K U; -K^T l]."""
        x = _dev(x, self.device).reshape(-1)
        y = self._out(self.size)
        _native.call("rmw_rigid_apply", self._h, x.data_ptr(), y.data_ptr(), _mode(mode))
        return y

    def apply_pc(self, x, mode=None):
        """Block-diagonal preconditioner apply (with the attached near-field
        augmentation).  mode=None or "fp64": FP64; mode="mixed": the FP32 apply
        of the mixed-precision solves."""
        x = _dev(x, self.device).reshape(-1)
        y = self._out(self.size)
        if mode is None:
            _native.call("rmw_rigid_apply_pc", self._h, x.data_ptr(), y.data_ptr())
        else:
            _native.call("rmw_rigid_apply_pc_mode", self._h, x.data_ptr(), y.data_ptr(), _mode(mode))
        return y

    def mobility_pc(self, w, mode="fp64"):
        """L^-1 M L^-T w (det_stoch mobility_pc)."""
        w = _dev(w, self.device).reshape(-1)
        y = self._out(3 * self.n_blobs)
        _native.call("rmw_rigid_mobility_pc", self._h, w.data_ptr(), y.data_ptr(), _mode(mode))
        return y

    def P_inv_mult(self, w):
        """L w (det_stoch P_inv_mult)."""
        w = _dev(w, self.device).reshape(-1)
        y = self._out(3 * self.n_blobs)
        _native.call("rmw_rigid_P_inv_mult", self._h, w.data_ptr(), y.data_ptr())
        return y

    def K_mult(self, u):
        u = _dev(u, self.device).reshape(-1)
        y = self._out(3 * self.n_blobs)
        _native.call("rmw_rigid_K_mult", self._h, u.data_ptr(), y.data_ptr())
        return y

    def KT_mult(self, lam):
        lam = _dev(lam, self.device).reshape(-1)
        y = self._out(6 * self.n_bodies)
        _native.call("rmw_rigid_KT_mult", self._h, lam.data_ptr(), y.data_ptr())
        return y

    def body_mobility(self):
        """List of the dense per-body wall mobility matrices (torch, on device)."""
        m2 = 9 * self.blobs_per_body ** 2
        out = self._out(int(m2.sum()))
        _native.call("rmw_rigid_body_mobility", self._h, out.data_ptr())
        res, o = [], 0
        for nb, sz in zip(self.blobs_per_body, m2):
            res.append(out[o:o + sz].reshape(3 * nb, 3 * nb))
            o += sz
        return res

    # -- body kinematics --------------------------------------------------------
    def blob_positions(self, x_bodies, q_bodies, r_ref):
        """(N,3) blob positions R(q) r_ref + x on the device."""
        x = _dev(x_bodies, self.device).reshape(-1)
        q = _dev(q_bodies, self.device).reshape(-1)
        rr = _dev(r_ref, self.device).reshape(-1)
        out = self._out(3 * self.n_blobs)
        _native.call("rmw_rigid_blob_positions", self._h, x.data_ptr(), q.data_ptr(), rr.data_ptr(),
                     out.data_ptr())
        return out.reshape(-1, 3)

    def euler_update(self, x_bodies, q_bodies, velocities, dt):
        """x + U dt and from_rotation(w dt) * q for every body."""
        x = _dev(x_bodies, self.device).reshape(-1)
        q = _dev(q_bodies, self.device).reshape(-1)
        v = _dev(velocities, self.device).reshape(-1)
        xn = self._out(3 * self.n_bodies)
        qn = self._out(4 * self.n_bodies)
        _native.call("rmw_rigid_euler_update", self._h, x.data_ptr(), q.data_ptr(), v.data_ptr(), float(dt),
                     xn.data_ptr(), qn.data_ptr())
        return xn.reshape(-1, 3), qn.reshape(-1, 4)

    def count_below(self, r, zmin=0.0):
        r = _dev(r, self.device).reshape(-1)
        c = ctypes.c_int(0)
        _native.call("rmw_count_below", r.data_ptr(), r.numel() // 3, float(zmin), ctypes.byref(c),
                     self.stream.cuda_stream)
        return c.value

    # -- independent suspensions -----------------------------------------------
    def set_suspensions(self, bodies_per_suspension):
        """Declare consecutive groups of bodies as independent suspensions
        (block-diagonal mobility); enables solve_batched."""
        counts = np.asarray(bodies_per_suspension, dtype=np.int64).reshape(-1)
        if counts.sum() != self.n_bodies or (counts < 0).any():
            raise ValueError("suspension body counts must add up to the number of bodies")
        off = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
        _native.call("rmw_rigid_set_suspensions", self._h, counts.size, off.ctypes.data_as(ctypes.c_void_p))
        self.suspension_body_offsets = off
        blob_off = self.offsets[off]
        self.suspension_blob_offsets = blob_off
        self.n_suspensions = int(counts.size)

    def solve_batched(self, rhs, tol=1e-8, restart=60, maxiter=1000, mode="fp64"):
        """Every suspension solved by its own GMRES (lockstep).  Returns
        (solution, iterations[k], relative residual[k], status[k]); status 0 = converged."""
        import torch
        b = _dev(rhs, self.device).reshape(-1)
        x = self._out(self.size)
        k = self.n_suspensions
        it = np.zeros(k, dtype=np.int32)
        rr = np.zeros(k)
        stt = np.zeros(k, dtype=np.int32)
        with torch.cuda.device(self.device):
            rc = _native.load().rmw_rigid_solve_batched(
                self._h, b.data_ptr(), x.data_ptr(), float(tol), int(restart), int(maxiter), _mode(mode),
                it.ctypes.data_as(ctypes.c_void_p), rr.ctypes.data_as(ctypes.c_void_p),
                stt.ctypes.data_as(ctypes.c_void_p))
        if rc not in (_native.RMW_OK, _native.RMW_ERR_NOT_CONVERGED):
            _native.check(rc)
        return x, it, rr, stt

    def lanczos_batched(self, Z, factor=1.0, tol=1e-3, max_iter=95, mode="fp64"):
        """Brownian noise for several right-hand sides of every suspension:
        Z (nrhs, 3N) -> (noise (nrhs, 3N), iterations (nrhs, n_suspensions))."""
        import torch
        Zt = _dev(Z, self.device).reshape(-1, 3 * self.n_blobs).contiguous()
        nrhs = Zt.shape[0]
        out = torch.empty_like(Zt)
        it = np.zeros(nrhs * self.n_suspensions, dtype=np.int32)
        with torch.cuda.device(self.device):
            _native.call("rmw_rigid_lanczos_batched", self._h, Zt.data_ptr(), out.data_ptr(), nrhs, float(factor),
                         float(tol), int(max_iter), _mode(mode), it.ctypes.data_as(ctypes.c_void_p))
        return out, it.reshape(nrhs, self.n_suspensions)

    # -- solvers -----------------------------------------------------------------
    def solve(self, rhs, tol=1e-8, restart=60, maxiter=1000, mode="fp64", raise_on_fail=False, scaled=False):
        """GMRES with the block-diagonal preconditioner.  Returns (solution, info, iterations, rel_residual);
        info = 0 on convergence, else the iteration count (the reference's convention).  scaled: solve
        for rhs / |rhs| and scale the solution back by |rhs| on the device (solve_mobility_problem's
        normalisation)."""
        import torch
        b = _dev(rhs, self.device).reshape(-1)
        x = self._out(self.size)
        it = ctypes.c_int(0)
        rr = ctypes.c_double(0.0)
        fn = _native.load().rmw_rigid_solve_scaled if scaled else _native.load().rmw_rigid_solve
        with torch.cuda.device(self.device):
            rc = fn(self._h, b.data_ptr(), x.data_ptr(), float(tol), int(restart), int(maxiter), _mode(mode),
                    ctypes.byref(it), ctypes.byref(rr))
        if rc == _native.RMW_ERR_NOT_CONVERGED and not raise_on_fail:
            return x, it.value, it.value, rr.value
        _native.check(rc)
        return x, 0, it.value, rr.value

    def lanczos(self, z, factor=1.0, tol=1e-3, max_iter=1000, mode="fp64"):
        """factor * L (L^-1 M L^-T)^(1/2) z: (noise, iterations)."""
        import torch
        z = _dev(z, self.device).reshape(-1)
        out = self._out(3 * self.n_blobs)
        it = ctypes.c_int(0)
        with torch.cuda.device(self.device):
            _native.call("rmw_rigid_lanczos", self._h, z.data_ptr(), out.data_ptr(), float(factor), float(tol),
                         int(max_iter), _mode(mode), ctypes.byref(it))
        return out, it.value
