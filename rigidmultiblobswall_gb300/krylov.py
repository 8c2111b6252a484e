"""Generic GPU Krylov solvers behind the reference's entry points:

* gmres(A, b, ...)                  general_application_utils.py:514-635
* stochastic_forcing_lanczos(...)   stochastic_forcing/stochastic_forcing.py:112-264

The operators may be any callables (or objects with ``matvec``) acting on CUDA
torch vectors; numpy-only callables are wrapped with a host round trip.  The
Krylov vector work (Arnoldi / reorthogonalisation, norms, updates) runs in
librmw_gb300's kernels; the solver calls back into Python only to apply the
operators.
"""
import ctypes

import numpy as np

from . import _native


class _DevView:
    def __init__(self, ptr, n):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": "<f8", "data": (ptr, False), "version": 3,
                                         "strides": None}


def _view(ptr, n, device):
    import torch
    return torch.as_tensor(_DevView(ptr, n), device=device)


def _as_fn(op):
    if op is None:
        return None
    if hasattr(op, "matvec"):
        return op.matvec
    return op


class _Callback:
    """Wraps a Python operator as an rmw_operator_fn."""

    def __init__(self, fn, n, device):
        self.fn = fn
        self.n = n
        self.device = device
        self.error = None
        self.host_only = False
        self.c = _native.OPERATOR_FN(self._call)

    def _apply(self, x):
        import torch
        if not self.host_only:
            try:
                y = self.fn(x)
            except (TypeError, AttributeError, ValueError):
                self.host_only = True
        if self.host_only:
            y = self.fn(x.cpu().numpy())
        y = torch.as_tensor(y, dtype=torch.float64, device=self.device).reshape(-1)
        return y

    def _call(self, ctx, xp, yp):
        try:
            x = _view(xp, self.n, self.device)
            y = _view(yp, self.n, self.device)
            y.copy_(self._apply(x))
            return 0
        except Exception as e:  # reported after the native call returns
            self.error = e
            return 1


def gmres(A, b, x0=None, tol=1e-05, restart=None, maxiter=None, xtype=None, M=None, callback=None, restrt=None,
          PC_side="right"):
    """Solve A x = b with right-preconditioned restarted GMRES (M = P^-1).

    Same arguments and return value (x, info) as the reference wrapper; info = 0
    on convergence, > 0 the number of iterations when maxiter is reached.  The
    initial guess is zero, as in the reference (which does not pass x0 on).
    PC_side 'left' solves M A x = M b without a right preconditioner.
    callback(rk) is called once per iteration with the relative residual estimate.
    """
    import torch
    is_t = type(b).__module__.startswith("torch")
    device = b.device if is_t and b.is_cuda else torch.device("cuda", torch.cuda.current_device())
    bt = torch.as_tensor(b, dtype=torch.float64, device=device).reshape(-1).contiguous()
    n = bt.numel()
    restart = restart if restart is not None else (restrt if restrt is not None else 20)
    maxiter = maxiter if maxiter is not None else 10 * n
    Af, Mf = _as_fn(A), _as_fn(M)
    if PC_side in ("left", "left_res") and Mf is not None:
        # M A x = M b; either operator may take tensors or only numpy arrays
        A0, M0 = _Callback(Af, n, device), _Callback(Mf, n, device)
        Af = lambda x: M0._apply(A0._apply(x))  # noqa: E731
        bt = M0._apply(bt).contiguous()
        Mf = None
    cbA = _Callback(Af, n, device)
    cbM = _Callback(Mf, n, device) if Mf is not None else None
    x = torch.empty(n, dtype=torch.float64, device=device)
    it = ctypes.c_int(0)
    rr = ctypes.c_double(0.0)
    cap = int(min(maxiter, 100000))
    hist = np.zeros(max(cap, 1))
    stream = torch.cuda.current_stream(device).cuda_stream
    rc = _native.load().rmw_gmres(n, ctypes.cast(cbA.c, ctypes.c_void_p), None,
                                  ctypes.cast(cbM.c, ctypes.c_void_p) if cbM else None, None, bt.data_ptr(),
                                  x.data_ptr(), float(tol), int(restart), int(maxiter), stream, ctypes.byref(it),
                                  ctypes.byref(rr), hist.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), cap)
    for cb in (cbA, cbM):
        if cb is not None and cb.error is not None:
            raise cb.error
    if rc not in (_native.RMW_OK, _native.RMW_ERR_NOT_CONVERGED):
        _native.check(rc)
    info = 0 if rc == _native.RMW_OK else it.value
    if callback is not None:
        for k in range(min(it.value, cap)):
            callback(hist[k])
    return (x if is_t else x.cpu().numpy()), info


def stochastic_forcing_lanczos(factor=1.0, tolerance=1e-06, max_iter=1000, dim=None, mobility=None,
                               mobility_mult=None, L_mult=None, z=None, print_residual=False):
    """factor * M^(1/2) z by Lanczos; returns (noise, iterations) like the reference.

    mobility: dense matrix (used only if mobility_mult is None); mobility_mult:
    callable v -> M v; L_mult: callable applied to the result (M ~ L L^T);
    z: the random vector (drawn from numpy's global normal generator if None).
    """
    import torch
    if dim is None:
        dim = len(z)
    if factor == 0.0:
        return (np.zeros(dim), 0)
    is_t = z is not None and type(z).__module__.startswith("torch")
    device = z.device if is_t and z.is_cuda else torch.device("cuda", torch.cuda.current_device())
    if z is None:
        z = np.random.randn(dim)
    zt = torch.as_tensor(z, dtype=torch.float64, device=device).reshape(-1).contiguous()
    if mobility_mult is None:
        Mt = torch.as_tensor(np.asarray(mobility, dtype=np.float64) if not type(mobility).__module__.startswith(
            "torch") else mobility, dtype=torch.float64, device=device)
        fn = lambda v: Mt @ v  # noqa: E731
    else:
        fn = _as_fn(mobility_mult)
    cb = _Callback(fn, dim, device)
    out = torch.empty(dim, dtype=torch.float64, device=device)
    it = ctypes.c_int(0)
    stream = torch.cuda.current_stream(device).cuda_stream
    rc = _native.load().rmw_lanczos(dim, ctypes.cast(cb.c, ctypes.c_void_p), None, zt.data_ptr(), out.data_ptr(),
                                    float(factor), float(tolerance), int(max_iter), stream, ctypes.byref(it))
    if cb.error is not None:
        raise cb.error
    _native.check(rc)
    if L_mult is not None:
        out = torch.as_tensor(_Callback(_as_fn(L_mult), dim, device)._apply(out), device=device)
    noise = out if is_t else out.cpu().numpy()
    return (np.reshape(noise, dim) if not is_t else noise.reshape(dim)), it.value
