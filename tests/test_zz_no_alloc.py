"""GPU: the allocation-free product entry point (rmw_wall_product_noalloc).

It serves callers that cannot call cudaMalloc - an application whose device
memory is owned by another allocator, code that must keep a fixed device
footprint after start-up, or a loop that cannot take cudaMalloc's implicit
device synchronisation - by keeping its scratch in a fixed 16 MiB device array
instead of allocating.  This file is collected last on purpose, and it must
pass both alone in a fresh process and after every other test.

Checks, through the C ABI: two calls in a row agree with the standard entry
point rmw_wall_product (within the tolerances of the other product tests:
1e-12 relative for FP64 and df64, 1e-6 for mixed), the second call with
different inputs so that the array's leftover contents from the first call
cannot leak in; a product just below RMW_NOALLOC_MAX_BLOBS, where the source
split shrinks until the scratch fits the array; and sizes above the limit are
rejected with a clear error.
"""
import ctypes

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

TOL = {0: 1e-12, 1: 1e-6, 2: 1e-12}  # mode 0 = FP64, 1 = mixed, 2 = df64 (double-float, FP64-accurate)


def _inputs(torch, dev, n, seed):
    from rigidmultiblobswall_gb300 import suspensions as S
    r, f, eta, a = S.blobs_wall_matvec(n, seed=seed)
    r[: n // 10, 2] = 0.3 * a  # some blobs overlap the wall: damping path on
    return torch.tensor(r, device=dev), torch.tensor(f, device=dev), eta, a


@pytest.mark.parametrize("mode", [0, 1, 2])
@pytest.mark.parametrize("kind", [0, 1, 2, 3])
def test_noalloc_matches_standard_entry_point_twice(cuda_device, kind, mode):
    import torch
    from rigidmultiblobswall_gb300 import _native
    lib = _native.load()
    stream = torch.cuda.current_stream(cuda_device).cuda_stream
    L = np.zeros(3)
    Lp = L.ctypes.data_as(ctypes.c_void_p)
    for call, (n, seed) in enumerate(((3000, 21), (1777, 22))):
        r, f, eta, a = _inputs(torch, cuda_device, n, seed + 10 * kind)
        ref = torch.empty(3 * n, dtype=torch.float64, device=cuda_device)
        out = torch.full((3 * n,), float("nan"), dtype=torch.float64, device=cuda_device)
        _native.check(lib.rmw_wall_product(kind, r.data_ptr(), f.data_ptr(), ref.data_ptr(), n, eta, a, Lp, mode,
                                           stream))
        _native.check(lib.rmw_wall_product_noalloc(kind, r.data_ptr(), f.data_ptr(), out.data_ptr(), n, eta, a,
                                                   Lp, mode, stream))
        torch.cuda.synchronize()
        assert torch.isfinite(out).all(), "call %d left non-finite output" % call
        assert rel_err(out.cpu().numpy(), ref.cpu().numpy()) <= TOL[mode], "call %d" % call


@pytest.mark.parametrize("mode", [1, 2])
def test_noalloc_near_its_limit_matches_standard_entry_point(cuda_device, mode):
    """179,999 blobs: 88 B per blob of packed sources and one chunk of partial
    sums is 15.8 MB, so the source split drops to the one chunk the 16 MiB
    array holds; the result still matches the standard entry point."""
    import torch
    from rigidmultiblobswall_gb300 import _native
    lib = _native.load()
    stream = torch.cuda.current_stream(cuda_device).cuda_stream
    n = 179999
    r, f, eta, a = _inputs(torch, cuda_device, n, 31)
    ref = torch.empty(3 * n, dtype=torch.float64, device=cuda_device)
    out = torch.full((3 * n,), float("nan"), dtype=torch.float64, device=cuda_device)
    _native.check(lib.rmw_wall_product(0, r.data_ptr(), f.data_ptr(), ref.data_ptr(), n, eta, a, None, mode,
                                       stream))
    _native.check(lib.rmw_wall_product_noalloc(0, r.data_ptr(), f.data_ptr(), out.data_ptr(), n, eta, a, None,
                                               mode, stream))
    torch.cuda.synchronize()
    assert torch.isfinite(out).all()
    assert rel_err(out.cpu().numpy(), ref.cpu().numpy()) <= TOL[mode]


def test_noalloc_rejects_sizes_above_its_limit(cuda_device):
    from rigidmultiblobswall_gb300 import _native
    lib = _native.load()
    limit = 180000  # RMW_NOALLOC_MAX_BLOBS in include/rmw_gb300.h
    rc = lib.rmw_wall_product_noalloc(0, 16, 16, 16, limit + 1, 1.0, 0.5, None, 0, None)
    assert rc == _native.RMW_ERR_ARG
    assert b"RMW_NOALLOC_MAX_BLOBS" in lib.rmw_last_error()
