"""ctypes binding of librmw_gb300.so (the C ABI declared in include/rmw_gb300.h).

The library is required: importing a compute entry point without it raises.
There is no CPU fallback anywhere in this package.
"""
import ctypes
import os

from . import build as _build

RMW_OK = 0
RMW_ERR_ARG = 1
RMW_ERR_CUDA = 2
RMW_ERR_NOT_CONVERGED = 3
RMW_ERR_BREAKDOWN = 4
RMW_ERR_NONFINITE = 5
RMW_ERR_ALLOC = 6

MODE_FP64 = 0
MODE_MIXED = 1
MODE_DF64 = 2
KINDS = {"uf": 0, "ut": 1, "wf": 2, "wt": 3}

_lib = None


class RMWError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("rmw_gb300 error %d: %s" % (code, msg))
        self.code = code


c_double_p = ctypes.POINTER(ctypes.c_double)
_vp = ctypes.c_void_p
_i64 = ctypes.c_int64
_d = ctypes.c_double
_i = ctypes.c_int

# name -> (restype, argtypes)
SIGNATURES = {
    "rmw_last_error": (ctypes.c_char_p, []),
    "rmw_version": (_i, []),
    "rmw_wall_product": (_i, [_i, _vp, _vp, _vp, _i64, _d, _d, _vp, _i, _vp]),
    "rmw_wall_uf": (_i, [_vp, _vp, _vp, _i64, _d, _d, _vp, _i, _vp]),
    "rmw_wall_ut": (_i, [_vp, _vp, _vp, _i64, _d, _d, _vp, _i, _vp]),
    "rmw_wall_wf": (_i, [_vp, _vp, _vp, _i64, _d, _d, _vp, _i, _vp]),
    "rmw_wall_wt": (_i, [_vp, _vp, _vp, _i64, _d, _d, _vp, _i, _vp]),
    "rmw_wall_batch_create": (_i, [ctypes.POINTER(ctypes.c_void_p), _i64, _vp]),
    "rmw_wall_batch_destroy": (_i, [_vp]),
    "rmw_wall_product_batched": (_i, [_vp, _i, _vp, _vp, _vp, _d, _d, _i, _vp]),
    "rmw_wall_uf_multi": (_i, [_vp, _vp, _vp, _i64, _i, _d, _d, _vp, _vp]),
    "rmw_wall_product_host": (_i, [_i, _vp, _vp, _vp, _i64, _d, _d, _vp, _i]),
    "rmw_wall_force_torque": (_i, [_vp, _vp, _vp, _vp, _vp, _i64, _d, _d, _vp, _i, _vp]),
    "rmw_nowall_product": (_i, [_i, _vp, _vp, _vp, _i64, _d, _d, _vp, _i, _vp]),
    "rmw_source_target_product": (_i, [_i, _vp, _vp, _vp, _vp, _vp, _i64, _i64, _d, _vp, _i, _vp, _vp]),
    "rmw_free_surface_product": (_i, [_vp, _vp, _vp, _i64, _d, _d, _vp, _i, _vp]),
    "rmw_dense_mobility": (_i, [_i, _vp, _vp, _i64, _d, _d, _vp]),
    "rmw_rollers_velocity_and_torque": (_i, [_vp, _vp, _vp, _vp, _vp, _i64, _d, _d, _vp, _i, _d, _i, _i, _i, _vp,
                                            _vp, _vp]),
    "rmw_rigid_set_wall": (_i, [_vp, _i]),
    "rmw_blob_blob_forces": (_i, [_vp, _vp, _i64, _d, _d, _d, _d, _vp, _i, _vp]),
    "rmw_blob_external_forces": (_i, [_vp, _vp, _i64, _d, _d, _d, _d, _d, _i, _vp]),
    "rmw_wall_autotune": (_i, [_i, _i, _i64, _i, _vp, _vp, _vp, _vp]),
    "rmw_wall_autotune_lookup": (_i, [_i, _i, _i64, _vp, _vp]),
    "rmw_wall_autotune_clear": (_i, []),
    "rmw_wall_autotune_set": (_i, [_i, _i, _i64, _i]),
    "rmw_wall_product_route": (_i, [_i, _i, _i64, _vp, _vp]),
    "rmw_use_graphs": (_i, [_i]),
    "rmw_use_device_krylov": (_i, [_i]),
    "rmw_trace_bytes": (_i, [_i, _vp, _i]),
    "rmw_graph_stats": (_i, [_vp, _vp, _i]),
    "rmw_rigid_create": (_i, [ctypes.POINTER(ctypes.c_void_p), _i64, _vp, _d, _d, _vp, _vp]),
    "rmw_rigid_destroy": (_i, [_vp]),
    "rmw_rigid_sizes": (_i, [_vp, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64)]),
    "rmw_rigid_set_configuration": (_i, [_vp, _vp, _vp]),
    "rmw_rigid_build_pc": (_i, [_vp, _i]),
    "rmw_rigid_build_pc_mode": (_i, [_vp, _i, _i]),
    "rmw_rigid_apply": (_i, [_vp, _vp, _vp, _i]),
    "rmw_rigid_apply_pc": (_i, [_vp, _vp, _vp]),
    "rmw_rigid_apply_pc_mode": (_i, [_vp, _vp, _vp, _i]),
    "rmw_rigid_mobility_pc": (_i, [_vp, _vp, _vp, _i]),
    "rmw_rigid_P_inv_mult": (_i, [_vp, _vp, _vp]),
    "rmw_rigid_K_mult": (_i, [_vp, _vp, _vp]),
    "rmw_rigid_KT_mult": (_i, [_vp, _vp, _vp]),
    "rmw_rigid_body_mobility": (_i, [_vp, _vp]),
    "rmw_rigid_blob_positions": (_i, [_vp, _vp, _vp, _vp, _vp]),
    "rmw_rigid_euler_update": (_i, [_vp, _vp, _vp, _vp, _d, _vp, _vp]),
    "rmw_count_below": (_i, [_vp, _i64, _d, ctypes.POINTER(ctypes.c_int), _vp]),
    "rmw_rigid_solve": (_i, [_vp, _vp, _vp, _d, _i, _i, _i, ctypes.POINTER(ctypes.c_int),
                             ctypes.POINTER(ctypes.c_double)]),
    "rmw_rigid_solve_scaled": (_i, [_vp, _vp, _vp, _d, _i, _i, _i, ctypes.POINTER(ctypes.c_int),
                             ctypes.POINTER(ctypes.c_double)]),
    "rmw_rigid_lanczos": (_i, [_vp, _vp, _vp, _d, _d, _i, _i, ctypes.POINTER(ctypes.c_int)]),
    "rmw_wall_lanczos": (_i, [_vp, _vp, _vp, _i64, _d, _d, _vp, _d, _d, _i, _i, _vp,
                              ctypes.POINTER(ctypes.c_int)]),
    "rmw_rigid_set_suspensions": (_i, [_vp, _i64, _vp]),
    "rmw_rigid_solve_batched": (_i, [_vp, _vp, _vp, _d, _i, _i, _i, _vp, _vp, _vp]),
    "rmw_rigid_lanczos_batched": (_i, [_vp, _vp, _vp, _i, _d, _d, _i, _i, _vp]),
    "rmw_rigid_pair_coupling": (_i, [_vp, _vp]),
    "rmw_nearfield_create": (_i, [ctypes.POINTER(ctypes.c_void_p), _d, _d, ctypes.c_ulonglong]),
    "rmw_nearfield_destroy": (_i, [_vp]),
    "rmw_nearfield_sizes": (_i, [_vp, _vp, _vp, _vp, _vp, _vp]),
    "rmw_nearfield_get": (_i, [_vp, _vp, _vp, _vp]),
    "rmw_nearfield_set": (_i, [_vp, _vp, _vp, _vp]),
    "rmw_nearfield_forward": (_i, [_vp, _vp, _vp, _vp]),
    "rmw_nearfield_grad": (_i, [_vp, _vp, _vp, _vp, _vp]),
    "rmw_nearfield_train": (_i, [_vp, _vp, _i, _i, ctypes.c_float, _vp, _vp]),
    "rmw_nearfield_set_cutoffs": (_i, [_vp, _d, _d]),
    "rmw_rigid_set_nearfield": (_i, [_vp, _vp, _d, _vp]),
    "rmw_rigid_set_nearfield_bands": (_i, [_vp, _vp, _d, _d, _vp]),
    "rmw_rigid_pair_coupling_list": (_i, [_vp, _vp, _i64, _vp]),
    "rmw_gmres": (_i, [_i64, _vp, _vp, _vp, _vp, _vp, _vp, _d, _i, _i, _vp, ctypes.POINTER(ctypes.c_int),
                       ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double), _i]),
    "rmw_lanczos": (_i, [_i64, _vp, _vp, _vp, _vp, _d, _d, _i, _vp, ctypes.POINTER(ctypes.c_int)]),
    "rmw_wall_product_noalloc": (_i, [_i, _vp, _vp, _vp, _i64, _d, _d, _vp, _i, _vp]),
    "rmw_fma_peak": (_i, [_i, ctypes.POINTER(ctypes.c_double), _vp]),
    "rmw_set_scratch_limit": (_i, [_i64]),
    "rmw_release_scratch": (_i, []),
    "rmw_trace_enable": (_i, [_i]),
    "rmw_trace_read": (_i, [_i, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int64), _i]),
}


def fma_peak(fp64, stream=None):
    """Measured FP64/FP32 FMA-pipe FLOP/s of the current device."""
    out = ctypes.c_double(0.0)
    call("rmw_fma_peak", 1 if fp64 else 0, ctypes.byref(out), stream)
    return out.value


def trace_enable(on=True):
    call("rmw_trace_enable", 1 if on else 0)


def trace_read(kind=0, reset=True):
    """(total milliseconds, launches) of traced kernels of one class."""
    ms = ctypes.c_double(0.0)
    cnt = ctypes.c_int64(0)
    call("rmw_trace_read", kind, ctypes.byref(ms), ctypes.byref(cnt), 1 if reset else 0)
    return ms.value, cnt.value


def trace_bytes(kind=1, reset=True):
    """Algorithmic bytes moved by traced work of one class."""
    b = ctypes.c_double(0.0)
    call("rmw_trace_bytes", kind, ctypes.byref(b), 1 if reset else 0)
    return b.value


OPERATOR_FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p)


def lib_path():
    return _build.lib_path()


def load(build_if_missing=False):
    """Load the shared library (raises if it is missing and not built)."""
    global _lib
    if _lib is not None:
        return _lib
    p = lib_path()
    if not os.path.exists(p):
        if build_if_missing:
            _build.build()
        else:
            raise RuntimeError("librmw_gb300.so is not built (%s); run rigidmultiblobswall_gb300.build.build()" % p)
    lib = ctypes.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name, None)
        if fn is None:
            continue
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(rc):
    if rc != RMW_OK:
        msg = load().rmw_last_error()
        raise RMWError(rc, msg.decode() if msg else "")
    return rc


def call(name, *args):
    return check(getattr(load(), name)(*args))


def set_scratch_limit(nbytes):
    """Cap one library scratch buffer at nbytes (0 = no cap); symmetric products fall back to one-sided."""
    call("rmw_set_scratch_limit", int(nbytes))


def release_scratch():
    """Free the current device's library scratch buffers."""
    call("rmw_release_scratch")


def use_graphs(on=True):
    """Replay the solvers' per-iteration operators as CUDA graphs (default on)."""
    call("rmw_use_graphs", 1 if on else 0)


def use_device_krylov(on=True):
    """Run the rigid solves' GMRES restart cycles on the device (default on) or host-driven."""
    call("rmw_use_device_krylov", 1 if on else 0)


def graph_stats(reset=False):
    """(graphs captured, graph replays) since the last reset."""
    c = ctypes.c_int64(0)
    r = ctypes.c_int64(0)
    call("rmw_graph_stats", ctypes.byref(c), ctypes.byref(r), 1 if reset else 0)
    return c.value, r.value
