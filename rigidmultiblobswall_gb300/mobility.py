"""Drop-in for the wall-RPY part of the reference's ``mobility/mobility.py``.

Same names, argument meaning and return convention as the reference:
``f(r_vectors, vector, eta, a, *args, **kwargs)`` with ``r_vectors`` an (N,3)
array, ``vector`` (N,3) or (3N,), the keyword ``periodic_length`` (3 lengths,
> 0 means pseudo-periodic) and a NEW flat (3N,) float64 result.  Inputs are
never modified.

All products run on the GPU through librmw_gb300.so:

* numpy inputs take the host path (copy in, launch, copy out; synchronous), the
  contract of the reference's pycuda wrappers (mobility/mobility_pycuda.py:2235-2267);
* CUDA torch tensors stay on the device; the call is asynchronous on the current
  torch stream and returns a CUDA tensor.

The extra keyword ``mode`` selects 'fp64' (default, every pair in FP64),
'df64' (double-float pair arithmetic on the FP32 pipe with FP64 accumulation;
error <= 1e-12 relative to FP64, several times faster on GB300, whose FP64
rate is 1/64 of FP32) or 'mixed' (FP32 pair evaluation with double-float
position differences and compensated accumulation; error <= 1e-6 relative to
FP64).

The ``_pycuda``, ``_numba`` and ``_cpp`` suffixes of the reference are all
aliases of the GPU implementation, so ``set_mobility_vector_prod`` callers can
swap the backend without changing their implementation string.
"""
import ctypes

import numpy as np
import scipy.sparse

from . import _native

_MODES = {"fp64": _native.MODE_FP64, "mixed": _native.MODE_MIXED, "df64": _native.MODE_DF64}


def _mode(kwargs):
    m = kwargs.get("mode", "fp64")
    if m not in _MODES:
        raise ValueError("mode must be 'fp64', 'df64' or 'mixed'")
    return _MODES[m]


def _periodic(kwargs):
    L = kwargs.get("periodic_length", None)
    if L is None:
        return np.zeros(3)
    L = np.ascontiguousarray(np.asarray(L, dtype=np.float64).reshape(-1))
    if L.size != 3:
        raise ValueError("periodic_length must have 3 entries")
    return L


def _is_torch(x):
    return type(x).__module__.startswith("torch")


def wall_product(kind, r_vectors, vector, eta, a, **kwargs):
    """B M(z_eff) B v for kind in {'uf','ut','wf','wt'} (see module docstring)."""
    L = _periodic(kwargs)
    mode = _mode(kwargs)
    k = _native.KINDS[kind]
    Lp = L.ctypes.data_as(ctypes.c_void_p)
    if _is_torch(r_vectors) or _is_torch(vector):
        import torch
        r = torch.as_tensor(r_vectors, dtype=torch.float64)
        v = torch.as_tensor(vector, dtype=torch.float64)
        if not (r.is_cuda and v.is_cuda):
            raise ValueError("torch inputs must both be CUDA tensors")
        r = r.reshape(-1, 3).contiguous()
        n = r.shape[0]
        v = v.reshape(-1).contiguous()
        if v.numel() != 3 * n:
            raise ValueError("vector must have 3N entries")
        out = torch.empty(3 * n, dtype=torch.float64, device=r.device)
        stream = torch.cuda.current_stream(r.device).cuda_stream
        with torch.cuda.device(r.device):
            _native.call("rmw_wall_product", k, r.data_ptr(), v.data_ptr(), out.data_ptr(), n, float(eta),
                         float(a), Lp, mode, stream)
        return out
    r = np.ascontiguousarray(np.asarray(r_vectors, dtype=np.float64).reshape(-1, 3))
    n = r.shape[0]
    v = np.ascontiguousarray(np.asarray(vector, dtype=np.float64).reshape(-1))
    if v.size != 3 * n:
        raise ValueError("vector must have 3N entries")
    out = np.empty(3 * n)
    _native.call("rmw_wall_product_host", k, r.ctypes.data_as(ctypes.c_void_p), v.ctypes.data_as(ctypes.c_void_p),
                 out.ctypes.data_as(ctypes.c_void_p), n, float(eta), float(a), Lp, mode)
    return out


def wall_force_torque(r_vectors, force, torque, eta, a, with_rotation=True, **kwargs):
    """U = M_UF F + M_UT T and (with_rotation) W = M_WF F + M_WT T in one pass
    over the pairs, with the wall regularisation of the single products.
    Returns U, or (U, W); numpy in -> numpy out, CUDA tensors stay on the device."""
    import torch
    L = _periodic(kwargs)
    mode = _mode(kwargs)
    on_device = _is_torch(r_vectors) or _is_torch(force) or _is_torch(torque)
    dev = None
    for x in (r_vectors, force, torque):
        if _is_torch(x) and x.is_cuda:
            dev = x.device
    if dev is None:
        if on_device:
            raise ValueError("torch inputs must be CUDA tensors")
        dev = torch.device("cuda", torch.cuda.current_device())
    r = torch.as_tensor(r_vectors, dtype=torch.float64, device=dev).reshape(-1, 3).contiguous()
    n = r.shape[0]
    f = torch.as_tensor(force, dtype=torch.float64, device=dev).reshape(-1).contiguous()
    t = torch.as_tensor(torque, dtype=torch.float64, device=dev).reshape(-1).contiguous()
    if f.numel() != 3 * n or t.numel() != 3 * n:
        raise ValueError("force and torque must have 3N entries")
    U = torch.empty(3 * n, dtype=torch.float64, device=dev)
    W = torch.empty(3 * n, dtype=torch.float64, device=dev) if with_rotation else None
    with torch.cuda.device(dev):
        _native.call("rmw_wall_force_torque", r.data_ptr(), f.data_ptr(), t.data_ptr(), U.data_ptr(),
                     W.data_ptr() if W is not None else None, n, float(eta), float(a),
                     L.ctypes.data_as(ctypes.c_void_p), mode, torch.cuda.current_stream(dev).cuda_stream)
    if not on_device:
        U = U.cpu().numpy()
        W = W.cpu().numpy() if W is not None else None
    return (U, W) if with_rotation else U


def no_wall_product(kind, r_vectors, vector, eta, a, **kwargs):
    """Free-space RPY product M_kind v (no wall, no regularisation), kind in
    {'uf','ut','wf','wt'}; numpy in -> numpy out, CUDA tensors stay on the device."""
    import torch
    L = _periodic(kwargs)
    mode = _mode(kwargs)
    on_device = _is_torch(r_vectors) or _is_torch(vector)
    dev = None
    for x in (r_vectors, vector):
        if _is_torch(x) and x.is_cuda:
            dev = x.device
    if dev is None:
        if on_device:
            raise ValueError("torch inputs must be CUDA tensors")
        dev = torch.device("cuda", torch.cuda.current_device())
    r = torch.as_tensor(r_vectors, dtype=torch.float64, device=dev).reshape(-1, 3).contiguous()
    n = r.shape[0]
    v = torch.as_tensor(vector, dtype=torch.float64, device=dev).reshape(-1).contiguous()
    if v.numel() != 3 * n:
        raise ValueError("vector must have 3N entries")
    out = torch.empty(3 * n, dtype=torch.float64, device=dev)
    with torch.cuda.device(dev):
        _native.call("rmw_nowall_product", _native.KINDS[kind], r.data_ptr(), v.data_ptr(), out.data_ptr(), n,
                     float(eta), float(a), L.ctypes.data_as(ctypes.c_void_p), mode,
                     torch.cuda.current_stream(dev).cuda_stream)
    return out if on_device else out.cpu().numpy()


def no_wall_mobility_trans_times_force_gb300(r_vectors, force, eta, a, *args, **kwargs):
    """Free-space RPY M_UF F (mobility/mobility.py:288-297)."""
    return no_wall_product("uf", r_vectors, force, eta, a, **kwargs)


def no_wall_mobility_trans_times_torque_gb300(r_vectors, torque, eta, a, *args, **kwargs):
    """Free-space RPY M_UT T (mobility/mobility.py:482-491)."""
    return no_wall_product("ut", r_vectors, torque, eta, a, **kwargs)


def no_wall_mobility_rot_times_force_gb300(r_vectors, force, eta, a, *args, **kwargs):
    """Free-space RPY M_WF F (mobility/mobility.py:328-337)."""
    return no_wall_product("wf", r_vectors, force, eta, a, **kwargs)


def no_wall_mobility_rot_times_torque_gb300(r_vectors, torque, eta, a, *args, **kwargs):
    """Free-space RPY M_WT T (mobility/mobility.py:370-379)."""
    return no_wall_product("wt", r_vectors, torque, eta, a, **kwargs)


def no_wall_mobility_trans_times_force_torque_gb300(r_vectors, force, torque, eta, a, *args, **kwargs):
    """Free-space U = M_UF F + M_UT T (mobility/mobility.py:413-423)."""
    return (no_wall_product("uf", r_vectors, force, eta, a, **kwargs) +
            no_wall_product("ut", r_vectors, torque, eta, a, **kwargs))


def single_wall_mobility_trans_times_force_torque_gb300(r_vectors, force, torque, eta, a, *args, **kwargs):
    """U = M_UF F + M_UT T (mobility/mobility.py:384-411)."""
    return wall_force_torque(r_vectors, force, torque, eta, a, with_rotation=False, **kwargs)


def wall_mobility_mult(r_vectors, X, eta, a, **kwargs):
    """[U_1 W_1 U_2 W_2 ...] = M [F_1 T_1 F_2 T_2 ...], the layout of
    Lub_Solver.Wall_Mobility_Mult (Lubrication/Lub_Solver.py:277-305), in one
    fused pass instead of four products."""
    xp = X
    if _is_torch(X):
        FT = X.reshape(-1, 6)
    else:
        FT = np.asarray(xp, dtype=np.float64).reshape(-1, 6)
    U, W = wall_force_torque(r_vectors, FT[:, 0:3].reshape(-1), FT[:, 3:6].reshape(-1), eta, a, **kwargs)
    if _is_torch(U):
        import torch
        return torch.cat([U.reshape(-1, 3), W.reshape(-1, 3)], dim=1).reshape(-1)
    return np.concatenate([U.reshape(-1, 3), W.reshape(-1, 3)], axis=1).reshape(-1)


class SuspensionBatch:
    """Segmented products of many independent suspensions stored in one (N,3)
    array: suspension k owns blobs [blob_offsets[k], blob_offsets[k+1]) and
    interacts only with itself.  One launch serves all suspensions."""

    def __init__(self, blob_offsets):
        off = np.ascontiguousarray(blob_offsets, dtype=np.int64).reshape(-1)
        h = ctypes.c_void_p()
        _native.call("rmw_wall_batch_create", ctypes.byref(h), off.size - 1, off.ctypes.data_as(ctypes.c_void_p))
        self._h = h
        self.offsets = off
        self.n = int(off[-1])

    def __del__(self):
        try:
            if self._h is not None and self._h.value:
                _native.load().rmw_wall_batch_destroy(self._h)
        except Exception:
            pass

    def product(self, kind, r_vectors, vector, eta, a, mode="fp64"):
        """Block-diagonal B M B v (CUDA torch tensors in and out)."""
        import torch
        r = torch.as_tensor(r_vectors, dtype=torch.float64).reshape(-1, 3).contiguous()
        v = torch.as_tensor(vector, dtype=torch.float64).reshape(-1).contiguous()
        if not (r.is_cuda and v.is_cuda) or r.shape[0] != self.n or v.numel() != 3 * self.n:
            raise ValueError("expected CUDA tensors of the batch's size")
        out = torch.empty(3 * self.n, dtype=torch.float64, device=r.device)
        with torch.cuda.device(r.device):
            _native.call("rmw_wall_product_batched", self._h, _native.KINDS[kind], r.data_ptr(), v.data_ptr(),
                         out.data_ptr(), float(eta), float(a), _MODES[mode],
                         torch.cuda.current_stream(r.device).cuda_stream)
        return out


def uf_multi(r_vectors, V, eta, a, batch=None):
    """M_UF applied to the rows of V (nrhs, 3N) at once, mixed precision
    (each pair block formed once for all right-hand sides).  CUDA tensors."""
    import torch
    r = torch.as_tensor(r_vectors, dtype=torch.float64).reshape(-1, 3).contiguous()
    n = r.shape[0]
    Vt = torch.as_tensor(V, dtype=torch.float64).reshape(-1, 3 * n).contiguous()
    Y = torch.empty_like(Vt)
    with torch.cuda.device(r.device):
        _native.call("rmw_wall_uf_multi", r.data_ptr(), Vt.data_ptr(), Y.data_ptr(), n, Vt.shape[0], float(eta),
                     float(a), batch._h if batch is not None else None, torch.cuda.current_stream(r.device).cuda_stream)
    return Y


def autotune(kind="uf", n=10752, mode="df64", reps=3, device=None):
    """Time every admissible source split of the `kind` product in `mode` on n
    synthetic blobs and cache the fastest for n's size bucket on the device;
    later products of that size use it.  Returns {"nchunks", "ms",
    "default_ms"}."""
    import torch
    dev = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
    best = ctypes.c_int(0)
    ms = ctypes.c_double(0.0)
    dms = ctypes.c_double(0.0)
    with torch.cuda.device(dev):
        _native.call("rmw_wall_autotune", _native.KINDS[kind], _MODES[mode], int(n), int(reps),
                     torch.cuda.current_stream(dev).cuda_stream, ctypes.byref(best), ctypes.byref(ms),
                     ctypes.byref(dms))
    return {"nchunks": best.value, "ms": ms.value, "default_ms": dms.value}


def autotune_lookup(kind="uf", n=10752, mode="df64"):
    """(source split the products use for this size, whether it was tuned)."""
    c = ctypes.c_int(0)
    t = ctypes.c_int(0)
    _native.call("rmw_wall_autotune_lookup", _native.KINDS[kind], _MODES[mode], int(n), ctypes.byref(c),
                 ctypes.byref(t))
    return c.value, bool(t.value)


def autotune_set(kind="uf", n=10752, mode="df64", nchunks=-1):
    """Pin the launch choice for this size bucket: a source split in [1, 64]
    or -1 for the symmetric kernel (non-periodic products of 256 or more
    blobs, any block and precision mode)."""
    _native.call("rmw_wall_autotune_set", _native.KINDS[kind], _MODES[mode], int(n), int(nchunks))


def autotune_clear():
    _native.call("rmw_wall_autotune_clear")


# ---------------------------------------------------------------------------
# wall regularisation helpers (mobility/mobility.py:52-84)
def shift_heights(r_vectors, blob_radius, *args, **kwargs):
    """z_effective = blob_radius wherever z <= blob_radius (copy; input untouched)."""
    r_effective = np.copy(r_vectors)
    r_effective[r_vectors[:, 2] <= blob_radius, 2] = blob_radius
    return r_effective


def damping_matrix_B(r_vectors, blob_radius, *args, **kwargs):
    """(sparse diag B, overlap): B_ii = z_i/blob_radius where z_i < blob_radius, else 1."""
    r = np.asarray(r_vectors).reshape(-1, 3)
    b = np.where(r[:, 2] < blob_radius, r[:, 2] / blob_radius, 1.0)
    B = np.repeat(b, 3)
    overlap = bool(np.any(r[:, 2] < blob_radius))
    return (scipy.sparse.dia_matrix((B, 0), shape=(B.size, B.size)), overlap)


# ---------------------------------------------------------------------------
# the four wall products under the reference's names
def single_wall_mobility_trans_times_force_gb300(r_vectors, force, eta, a, *args, **kwargs):
    """u = M_UF F  (reference: mobility/mobility.py:222-252, kernel mobility_pycuda.py:150-254)."""
    return wall_product("uf", r_vectors, force, eta, a, **kwargs)


def single_wall_mobility_trans_times_torque_gb300(r_vectors, torque, eta, a, *args, **kwargs):
    """u = M_UT T  (reference: mobility/mobility.py:427-452, kernel mobility_pycuda.py:1516-1622)."""
    return wall_product("ut", r_vectors, torque, eta, a, **kwargs)


def single_wall_mobility_rot_times_force_gb300(r_vectors, force, eta, a, *args, **kwargs):
    """w = M_WF F  (reference: mobility/mobility.py:300-325, kernel mobility_pycuda.py:926-1031)."""
    return wall_product("wf", r_vectors, force, eta, a, **kwargs)


def single_wall_mobility_rot_times_torque_gb300(r_vectors, torque, eta, a, *args, **kwargs):
    """w = M_WT T  (reference: mobility/mobility.py:342-367, kernel mobility_pycuda.py:593-697)."""
    return wall_product("wt", r_vectors, torque, eta, a, **kwargs)


# Reference backend names: all served by the GPU implementation.
single_wall_mobility_trans_times_force_pycuda = single_wall_mobility_trans_times_force_gb300
single_wall_mobility_trans_times_force_numba = single_wall_mobility_trans_times_force_gb300
single_wall_mobility_trans_times_force_cpp = single_wall_mobility_trans_times_force_gb300
single_wall_mobility_trans_times_torque_pycuda = single_wall_mobility_trans_times_torque_gb300
single_wall_mobility_trans_times_torque_numba = single_wall_mobility_trans_times_torque_gb300
single_wall_mobility_rot_times_force_pycuda = single_wall_mobility_rot_times_force_gb300
single_wall_mobility_rot_times_force_numba = single_wall_mobility_rot_times_force_gb300
single_wall_mobility_rot_times_torque_pycuda = single_wall_mobility_rot_times_torque_gb300
single_wall_mobility_rot_times_torque_numba = single_wall_mobility_rot_times_torque_gb300
single_wall_mobility_trans_times_force_torque_pycuda = single_wall_mobility_trans_times_force_torque_gb300
no_wall_mobility_trans_times_force_pycuda = no_wall_mobility_trans_times_force_gb300
no_wall_mobility_trans_times_force_numba = no_wall_mobility_trans_times_force_gb300
no_wall_mobility_trans_times_torque_pycuda = no_wall_mobility_trans_times_torque_gb300
no_wall_mobility_trans_times_torque_numba = no_wall_mobility_trans_times_torque_gb300
no_wall_mobility_rot_times_force_pycuda = no_wall_mobility_rot_times_force_gb300
no_wall_mobility_rot_times_force_numba = no_wall_mobility_rot_times_force_gb300
no_wall_mobility_rot_times_torque_pycuda = no_wall_mobility_rot_times_torque_gb300
no_wall_mobility_rot_times_torque_numba = no_wall_mobility_rot_times_torque_gb300
no_wall_mobility_trans_times_force_torque_pycuda = no_wall_mobility_trans_times_force_torque_gb300


# -- per-blob radii, sources -> targets; free surface --------------------------
_GEOMETRIES = {"no_wall": 0, "wall": 1, "free_surface": 2}


def _device_for(*xs):
    import torch
    on_device = any(_is_torch(x) for x in xs)
    for x in xs:
        if _is_torch(x) and x.is_cuda:
            return x.device, True
    if on_device:
        raise ValueError("torch inputs must be CUDA tensors")
    return torch.device("cuda", torch.cuda.current_device()), False


def source_target_product(geometry, source, target, force, radius_source, radius_target, eta, **kwargs):
    """Velocities (3 Nt,) of targets of radii radius_target from forces on
    sources of radii radius_source; geometry 'no_wall', 'wall' (shifted heights
    and damping on both sides) or 'free_surface'.  Keywords periodic_length and
    mode as the other products; numpy in -> numpy out, CUDA tensors stay on the
    device."""
    import torch
    L = _periodic(kwargs)
    mode = _mode(kwargs)
    dev, on_device = _device_for(source, target, force, radius_source, radius_target)
    t = lambda x: torch.as_tensor(x, dtype=torch.float64, device=dev)  # noqa: E731
    src = t(source).reshape(-1, 3).contiguous()
    trg = t(target).reshape(-1, 3).contiguous()
    ns, nt = src.shape[0], trg.shape[0]
    f = t(force).reshape(-1).contiguous()

    def radii(x, n):  # one radius per blob, or one for all
        v = t(x).reshape(-1)
        return (v.expand(n) if v.numel() == 1 else v).contiguous()

    rs, rt = radii(radius_source, ns), radii(radius_target, nt)
    if f.numel() != 3 * ns or rs.numel() != ns or rt.numel() != nt:
        raise ValueError("force must have 3 Ns entries and one radius per blob")
    out = torch.empty(3 * nt, dtype=torch.float64, device=dev)
    with torch.cuda.device(dev):
        _native.call("rmw_source_target_product", _GEOMETRIES[geometry], src.data_ptr(), trg.data_ptr(),
                     f.data_ptr(), rs.data_ptr(), rt.data_ptr(), ns, nt, float(eta),
                     L.ctypes.data_as(ctypes.c_void_p), mode, out.data_ptr(),
                     torch.cuda.current_stream(dev).cuda_stream)
    return out if on_device else out.cpu().numpy()


def single_wall_mobility_trans_times_force_source_target_gb300(source, target, force, radius_source, radius_target,
                                                               eta, *args, **kwargs):
    """Wall source-target product (mobility/mobility.py:494-530, 551-590)."""
    return source_target_product("wall", source, target, force, radius_source, radius_target, eta, **kwargs)


def no_wall_mobility_trans_times_force_source_target_gb300(source, target, force, radius_source, radius_target,
                                                           eta, *args, **kwargs):
    """Free-space source-target product (mobility/mobility.py:593-616)."""
    return source_target_product("no_wall", source, target, force, radius_source, radius_target, eta, **kwargs)


def free_surface_mobility_trans_times_force_source_target_gb300(source, target, force, radius_source,
                                                                radius_target, eta, *args, **kwargs):
    """Free-surface source-target product (mobility/mobility.py:1409-1429)."""
    return source_target_product("free_surface", source, target, force, radius_source, radius_target, eta,
                                 **kwargs)


def mobility_vector_product_source_target_one_wall(source, target, force, radius_source, radius_target, eta,
                                                   *args, **kwargs):
    """The Python form of the wall source-target product (mobility/mobility.py:830-902);
    returns (Nt, 3)."""
    out = single_wall_mobility_trans_times_force_source_target_gb300(source, target, force, radius_source,
                                                                     radius_target, eta, **kwargs)
    return out.reshape(-1, 3)


def mobility_vector_product_source_target_unbounded(source, target, force, radius_source, radius_target, eta,
                                                    *args, **kwargs):
    """The Python form of the free-space source-target product (mobility/mobility.py:905-946);
    returns (Nt, 3)."""
    out = no_wall_mobility_trans_times_force_source_target_gb300(source, target, force, radius_source,
                                                                 radius_target, eta, **kwargs)
    return out.reshape(-1, 3)


def free_surface_mobility_trans_times_force_gb300(r_vectors, force, eta, a, *args, **kwargs):
    """Free-surface product of blobs of radius a (mobility/mobility.py:533-548, 1390-1406)."""
    import torch
    L = _periodic(kwargs)
    mode = _mode(kwargs)
    dev, on_device = _device_for(r_vectors, force)
    r = torch.as_tensor(r_vectors, dtype=torch.float64, device=dev).reshape(-1, 3).contiguous()
    n = r.shape[0]
    f = torch.as_tensor(force, dtype=torch.float64, device=dev).reshape(-1).contiguous()
    if f.numel() != 3 * n:
        raise ValueError("force must have 3N entries")
    out = torch.empty(3 * n, dtype=torch.float64, device=dev)
    with torch.cuda.device(dev):
        _native.call("rmw_free_surface_product", r.data_ptr(), f.data_ptr(), out.data_ptr(), n, float(eta),
                     float(a), L.ctypes.data_as(ctypes.c_void_p), mode, torch.cuda.current_stream(dev).cuda_stream)
    return out if on_device else out.cpu().numpy()


def shift_heights_different_radius(r_vectors, blob_radius, *args, **kwargs):
    """Heights raised to each blob's radius (mobility/mobility.py:87-99)."""
    r = np.array(r_vectors, dtype=np.float64).reshape(-1, 3)
    rad = np.asarray(blob_radius, dtype=np.float64).reshape(-1)
    r[:, 2] = np.where(r[:, 2] > rad, r[:, 2], rad)
    return r


def damping_matrix_B_different_radius(r_vectors, blob_radius, *args, **kwargs):
    """(diagonal B with z/radius below the radius, any overlap) (mobility/mobility.py:102-119)."""
    r = np.asarray(r_vectors, dtype=np.float64).reshape(-1, 3)
    rad = np.asarray(blob_radius, dtype=np.float64).reshape(-1)
    d = np.where(r[:, 2] < rad, r[:, 2] / rad, 1.0)
    return scipy.sparse.dia_matrix((np.repeat(d, 3), 0), shape=(3 * d.size, 3 * d.size)), bool((d != 1.0).any())


single_wall_mobility_trans_times_force_source_target_pycuda = single_wall_mobility_trans_times_force_source_target_gb300
single_wall_mobility_trans_times_force_source_target_numba = single_wall_mobility_trans_times_force_source_target_gb300
no_wall_mobility_trans_times_force_source_target_numba = no_wall_mobility_trans_times_force_source_target_gb300
free_surface_mobility_trans_times_force_source_target_numba = free_surface_mobility_trans_times_force_source_target_gb300
free_surface_mobility_trans_times_force_pycuda = free_surface_mobility_trans_times_force_gb300
free_surface_mobility_trans_times_force_numba = free_surface_mobility_trans_times_force_gb300


# -- dense matrices ---------------------------------------------------------------
def _dense(wall, r_vectors, eta, a):
    import torch
    dev, on_device = _device_for(r_vectors)
    r = torch.as_tensor(r_vectors, dtype=torch.float64, device=dev).reshape(-1, 3).contiguous()
    n = r.shape[0]
    M = torch.empty((3 * n, 3 * n), dtype=torch.float64, device=dev)
    with torch.cuda.device(dev):
        _native.call("rmw_dense_mobility", 1 if wall else 0, r.data_ptr(), M.data_ptr(), n, float(eta), float(a),
                     torch.cuda.current_stream(dev).cuda_stream)
    return M if on_device else M.cpu().numpy()


def single_wall_fluid_mobility(r_vectors, eta, a, *args, **kwargs):
    """Dense (3N, 3N) wall mobility with shifted heights and damping
    (mobility/mobility.py:1018-1116); periodic images are not part of it, as
    in the reference."""
    return _dense(True, r_vectors, eta, a)


def rotne_prager_tensor(r_vectors, eta, a, *args, **kwargs):
    """Dense (3N, 3N) free-space RPY mobility (mobility/mobility.py:967-1015)."""
    return _dense(False, r_vectors, eta, a)


def single_wall_fluid_mobility_product(r_vectors, vector, eta, a, *args, **kwargs):
    """M v with the wall mobility (mobility/mobility.py:711-724, the dense
    product); evaluated pairwise without forming M."""
    kwargs.pop("periodic_length", None)
    return wall_product("uf", r_vectors, vector, eta, a, **kwargs)


def no_wall_fluid_mobility_product(r_vectors, vector, eta, a, *args, **kwargs):
    """M v with the free-space mobility (mobility/mobility.py:727-737)."""
    kwargs.pop("periodic_length", None)
    return no_wall_product("uf", r_vectors, vector, eta, a, **kwargs)


single_wall_fluid_mobility_loops = single_wall_fluid_mobility
single_wall_fluid_mobility_cpp = single_wall_fluid_mobility
rotne_prager_tensor_loops = rotne_prager_tensor
rotne_prager_tensor_cpp = rotne_prager_tensor
