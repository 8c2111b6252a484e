"""GPU: products whose symmetric partial sums cannot get their scratch fall back to the one-sided kernels.

rmw_set_scratch_limit caps one scratch request; with a 10 MB cap at 8,300 blobs the symmetric partial sums
(ceil(n/128) x 3n doubles = 12.9 MB for one block, 25.9 MB for the fused [U; W]) are refused, which is the
same path a failed cudaMalloc takes under memory pressure.  Every entry point with a symmetric kernel (wall
products, the fused force-torque product, the free-space products) must still return the oracle's result
through its one-sided kernels, and a request that even the one-sided kernels cannot fit must fail cleanly."""
import numpy as np
import pytest

from conftest import rel_err
from oracle import wall as owall
from rigidmultiblobswall_gb300 import _native
from rigidmultiblobswall_gb300 import mobility as mob

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-12, "df64": 1e-12, "mixed": 1e-6}
CAP = 10 * 1024 * 1024


def _case(n, seed):
    rng = np.random.default_rng(seed)
    r = np.empty((n, 3))
    side = 2.5 * np.cbrt(n)
    r[:, :2] = rng.uniform(0, side, (n, 2))
    r[:, 2] = rng.uniform(0.1, 4.0, n)
    return r, rng.standard_normal(3 * n), rng.standard_normal(3 * n)


@pytest.fixture
def capped(cuda_device):
    _native.set_scratch_limit(CAP)
    try:
        yield CAP
    finally:
        _native.set_scratch_limit(0)


@pytest.mark.parametrize("mode", ["df64", "mixed"])
def test_capped_products_fall_back_and_match_oracle(capped, mode):
    n, a = 8300, 0.3
    r, F, T = _case(n, 41)
    rows = np.random.default_rng(3).choice(n, 30, replace=False)
    pick = lambda x: np.asarray(x).reshape(-1, 3)[rows].reshape(-1)  # noqa: E731
    u = mob.wall_product("uf", r, F, 1.0, a, mode=mode)
    assert rel_err(pick(u), owall.wall_product("uf", r, F, 1.0, a, rows=rows)) <= TOL[mode]
    U, W = mob.wall_force_torque(r, F, T, 1.0, a, mode=mode)
    Ur, Wr = owall.force_torque(r, F, T, 1.0, a, rows=rows)
    assert rel_err(pick(U), Ur) <= TOL[mode]
    assert rel_err(pick(W), Wr) <= TOL[mode]
    v = mob.no_wall_product("wt", r, T, 1.0, a, mode=mode)
    assert rel_err(pick(v), owall.no_wall_product("wt", r, T, 1.0, a, rows=rows)) <= TOL[mode]


def test_request_above_cap_fails_cleanly_and_lifting_it_recovers(cuda_device):
    n, a = 60000, 0.3  # one-sided UF scratch: packed sources + 3n doubles per source chunk > 1 MB
    r, F, _ = _case(n, 5)
    _native.set_scratch_limit(1 << 20)
    try:
        with pytest.raises(_native.RMWError) as e:
            mob.wall_product("uf", r, F, 1.0, a, mode="mixed")
        assert e.value.code == _native.RMW_ERR_ALLOC
    finally:
        _native.set_scratch_limit(0)
    _native.release_scratch()
    rows = np.arange(0, n, 4999)
    u = mob.wall_product("uf", r, F, 1.0, a, mode="mixed")
    ref = owall.wall_product("uf", r, F, 1.0, a, rows=rows)
    assert rel_err(np.asarray(u).reshape(-1, 3)[rows].reshape(-1), ref) <= 1e-6
