"""Oracle (test infrastructure only): ctypes binding of the C restatement of the
wall-RPY products (``oracle/wall_oracle.c``) and the reference's wall
regularisation helpers.

Only tests, ``__graft_entry__.smoke()`` and the CPU legs of ``bench.py`` use it.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(_HERE, "_build")
KINDS = {"uf": 0, "ut": 1, "wf": 2, "wt": 3}
_libs = {}


def build(quiet=True):
    """Compile the oracle shared libraries (gcc, OpenMP)."""
    cmd = ["make", "-C", _HERE, "-s"]
    subprocess.run(cmd, check=True, stdout=subprocess.DEVNULL if quiet else None)


def _lib(fast=False):
    key = "fast" if fast else "parity"
    if key in _libs:
        return _libs[key]
    path = os.path.join(_BUILD, "liboracle_fast.so" if fast else "liboracle.so")
    if not os.path.exists(path):
        build()
    lib = ctypes.CDLL(path)
    dp = ctypes.POINTER(ctypes.c_double)
    lp = ctypes.POINTER(ctypes.c_long)
    lib.oracle_wall_product_rows.argtypes = [ctypes.c_int, dp, dp, dp, ctypes.c_long, lp, ctypes.c_long,
                                             ctypes.c_double, ctypes.c_double, dp]
    lib.oracle_wall_raw_rows.argtypes = lib.oracle_wall_product_rows.argtypes
    lib.oracle_nowall_rows.argtypes = lib.oracle_wall_product_rows.argtypes
    lib.oracle_wall_uf_symmetric.argtypes = [dp, dp, dp, ctypes.c_long, ctypes.c_double, ctypes.c_double,
                                             ctypes.c_int]
    lib.oracle_max_threads.restype = ctypes.c_int
    lib.oracle_wall_dense.argtypes = [dp, ctypes.c_long, ctypes.c_double, ctypes.c_double, dp]
    _libs[key] = lib
    return lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def wall_product(kind, r_vectors, vector, eta, a, periodic_length=None, rows=None, regularize=True):
    """B M(z_eff) B v for kind in {'uf','ut','wf','wt'} (flat (3N,) or (3*len(rows),))."""
    lib = _lib()
    r = np.ascontiguousarray(np.asarray(r_vectors, dtype=np.float64).reshape(-1, 3))
    v = np.ascontiguousarray(np.asarray(vector, dtype=np.float64).reshape(-1))
    n = r.shape[0]
    assert v.size == 3 * n
    L = np.zeros(3) if periodic_length is None else np.ascontiguousarray(periodic_length, dtype=np.float64)
    if rows is not None:
        rows = np.ascontiguousarray(rows, dtype=np.int64)
        out = np.empty(3 * rows.size)
        rp = rows.ctypes.data_as(ctypes.POINTER(ctypes.c_long))
        nr = rows.size
    else:
        out = np.empty(3 * n)
        rp = ctypes.POINTER(ctypes.c_long)()
        nr = 0
    fn = lib.oracle_wall_product_rows if regularize else lib.oracle_wall_raw_rows
    fn(KINDS[kind], _dp(r), _dp(v), _dp(out), n, rp, nr, float(eta), float(a), _dp(L))
    return out


def no_wall_product(kind, r_vectors, vector, eta, a, periodic_length=None, rows=None):
    """Free-space RPY product M v (no wall, no regularisation) of the no-wall
    numba functions (mobility/mobility_numba.py:13-1190)."""
    lib = _lib()
    r = np.ascontiguousarray(np.asarray(r_vectors, dtype=np.float64).reshape(-1, 3))
    v = np.ascontiguousarray(np.asarray(vector, dtype=np.float64).reshape(-1))
    n = r.shape[0]
    assert v.size == 3 * n
    L = np.zeros(3) if periodic_length is None else np.ascontiguousarray(periodic_length, dtype=np.float64)
    if rows is not None:
        rows = np.ascontiguousarray(rows, dtype=np.int64)
        out = np.empty(3 * rows.size)
        rp = rows.ctypes.data_as(ctypes.POINTER(ctypes.c_long))
        nr = rows.size
    else:
        out = np.empty(3 * n)
        rp = ctypes.POINTER(ctypes.c_long)()
        nr = 0
    lib.oracle_nowall_rows(KINDS[kind], _dp(r), _dp(v), _dp(out), n, rp, nr, float(eta), float(a), _dp(L))
    return out


def no_wall_dense(r_vectors, eta, a):
    """Dense free-space RPY blob mobility (3N, 3N), the reference's
    rotne_prager_tensor (mobility/mobility.py:967-1015), column by column from
    the free-space product."""
    r = np.ascontiguousarray(np.asarray(r_vectors, dtype=np.float64).reshape(-1, 3))
    n = r.shape[0]
    M = np.empty((3 * n, 3 * n))
    e = np.zeros(3 * n)
    for c in range(3 * n):
        e[c] = 1.0
        M[:, c] = no_wall_product("uf", r, e, eta, a)
        e[c] = 0.0
    return M


def dense_mobility(r_vectors, eta, a):
    """Dense regularised wall mobility (3N, 3N) (mobility/mobility.py:1018-1116)."""
    r = np.ascontiguousarray(np.asarray(r_vectors, dtype=np.float64).reshape(-1, 3))
    n = r.shape[0]
    M = np.empty((3 * n, 3 * n))
    _lib().oracle_wall_dense(_dp(r), n, float(eta), float(a), _dp(M))
    return M


def shift_heights(r_vectors, blob_radius):
    """mobility/mobility.py:52-64: z_eff = blob_radius where z <= blob_radius."""
    r = np.array(r_vectors, dtype=np.float64, copy=True).reshape(-1, 3)
    r[r[:, 2] <= blob_radius, 2] = blob_radius
    return r


def damping_vector(r_vectors, blob_radius):
    """Diagonal of mobility/mobility.py:67-84's B (B_ii = z/a where z < a, else 1)."""
    r = np.asarray(r_vectors, dtype=np.float64).reshape(-1, 3)
    b = np.where(r[:, 2] < blob_radius, r[:, 2] / blob_radius, 1.0)
    return np.repeat(b, 3), bool(np.any(r[:, 2] < blob_radius))


def uf_symmetric_fast(r_vectors, force, eta, a, threads=0):
    """Reference-C++-structured symmetric M_UF f (fast-math build), regularised
    like mobility/mobility.py:187-219.  Used as the timed CPU baseline."""
    lib = _lib(fast=True)
    r = np.asarray(r_vectors, dtype=np.float64).reshape(-1, 3)
    reff = np.ascontiguousarray(shift_heights(r, a))
    b, overlap = damping_vector(r, a)
    f = np.ascontiguousarray(np.asarray(force, dtype=np.float64).reshape(-1) * (b if overlap else 1.0))
    out = np.empty(f.size)
    lib.oracle_wall_uf_symmetric(_dp(reff), _dp(f), _dp(out), r.shape[0], float(eta), float(a), int(threads))
    if overlap:
        out *= b
    return out


def max_threads():
    return _lib(fast=True).oracle_max_threads()


def blake_point_mobility(r_vectors, eta):
    """Off-diagonal 3x3 blocks of the point-particle (Blake 1971) image system
    above a no-slip wall at z = 0: S(r) - S(R) + 2h SD(R) - h^2 PD(R), with R
    the separation from the image of the source at height h, S the Stokeslet
    (I/|r| + r r^T/|r|^3)/(8 pi eta), SD the Stokes doublet and PD the
    potential dipole with the sign flips of the image system's wall-parallel
    forcing (helpers of mobility/mobility.py:152-171).  Diagonal blocks zero.
    The finite-size wall mobility tends to it as a -> 0."""
    r = np.asarray(r_vectors, dtype=np.float64).reshape(-1, 3)
    n = r.shape[0]
    e3 = np.array([0.0, 0.0, 1.0])
    M = np.zeros((3 * n, 3 * n))
    for j in range(n):
        for k in range(n):
            if j == k:
                continue
            d = r[j] - r[k]
            rn = np.linalg.norm(d)
            h = r[k, 2]
            R = r[j] - (r[k] - 2.0 * h * e3)
            Rn = np.linalg.norm(R)
            S = (np.eye(3) / rn + np.outer(d, d) / rn ** 3 - (np.eye(3) / Rn + np.outer(R, R) / Rn ** 3)) / (8 * np.pi)
            SD = np.outer(R, e3) + R[2] * np.eye(3) - np.outer(e3, R) - 3.0 * R[2] * np.outer(R, R) / Rn ** 2
            SD[:, 0:2] *= -1.0
            SD /= 8 * np.pi * Rn ** 3
            PD = np.eye(3) - 3.0 * np.outer(R, R) / Rn ** 2
            PD[:, 0:2] *= -1.0
            PD /= 4 * np.pi * Rn ** 3
            M[3 * j:3 * j + 3, 3 * k:3 * k + 3] = (S + 2.0 * h * SD - h * h * PD) / eta
    return M


def force_torque(r_vectors, force, torque, eta, a, periodic_length=None, rows=None):
    """(U, W) = (M_UF F + M_UT T, M_WF F + M_WT T): the reference's
    single_wall_mobility_trans_times_force_torque (mobility/mobility.py:384-411)
    for U and the four products of Lub_Solver.Wall_Mobility_Mult
    (Lubrication/Lub_Solver.py:277-305) for both, composed from the oracle
    products."""
    kw = {"periodic_length": periodic_length, "rows": rows}
    U = wall_product("uf", r_vectors, force, eta, a, **kw) + wall_product("ut", r_vectors, torque, eta, a, **kw)
    W = wall_product("wf", r_vectors, force, eta, a, **kw) + wall_product("wt", r_vectors, torque, eta, a, **kw)
    return U, W
