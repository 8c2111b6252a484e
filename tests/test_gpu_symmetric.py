"""GPU: the symmetric kernels of all four blocks, FP64, df64 and mixed (each
unordered pair evaluated once and applied both ways: M_UF with f3 and f4
exchanged, the rotation blocks with d -> -d and the heights exchanged)
against the oracle and against the standard kernels:
tile tails, diagonal-tile pairing, wall-overlapping (damped) blobs, a shell
suspension, determinism, and the fallback where it does not apply."""
import numpy as np
import pytest

from conftest import rel_err
from oracle import wall as owall
from rigidmultiblobswall_gb300 import mobility as mob
from rigidmultiblobswall_gb300 import suspensions as S

pytestmark = pytest.mark.gpu


def _blobs(n, seed, damped=False):
    rng = np.random.default_rng(seed)
    r = np.empty((n, 3))
    side = 2.0 * np.cbrt(n)
    r[:, :2] = rng.uniform(0, side, (n, 2))
    r[:, 2] = rng.uniform(0.1 if damped else 0.8, 4.0, n)
    return r, rng.standard_normal(3 * n)


def _product(r, v, a, pin, mode="df64", kind="uf"):
    import torch
    mob.autotune_clear()
    if pin is not None:
        mob.autotune_set(kind, len(r), mode, pin)
    out = mob.wall_product(kind, torch.tensor(r, device="cuda"), torch.tensor(v, device="cuda"), 1.0, a,
                           mode=mode).cpu().numpy()
    mob.autotune_clear()
    return out


KINDS = ["uf", "ut", "wf", "wt"]


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("n", [256, 257, 300, 383, 1000, 2049])
@pytest.mark.parametrize("damped", [False, True])
def test_symmetric_matches_oracle_and_standard(cuda_device, kind, n, damped):
    r, v = _blobs(n, n, damped)
    a = 0.35
    sym = _product(r, v, a, -1, kind=kind)
    std = _product(r, v, a, 8, kind=kind)
    ref = owall.wall_product(kind, r, v, 1.0, a)
    assert rel_err(sym, ref) <= 1e-12
    assert rel_err(sym, std) <= 1e-13


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("n", [256, 383, 1000])
@pytest.mark.parametrize("damped", [False, True])
def test_fp64_symmetric_matches_oracle_and_standard(cuda_device, kind, n, damped):
    r, v = _blobs(n, n + 2, damped)
    a = 0.35
    sym = _product(r, v, a, -1, "fp64", kind)
    std = _product(r, v, a, 8, "fp64", kind)
    ref = owall.wall_product(kind, r, v, 1.0, a)
    assert rel_err(sym, ref) <= 1e-12
    assert rel_err(sym, std) <= 1e-13


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("n", [256, 300, 1000, 2049])
@pytest.mark.parametrize("damped", [False, True])
def test_mixed_symmetric_matches_oracle_and_standard(cuda_device, kind, n, damped):
    r, v = _blobs(n, n + 1, damped)
    a = 0.35
    sym = _product(r, v, a, -1, "mixed", kind)
    std = _product(r, v, a, 8, "mixed", kind)
    ref = owall.wall_product(kind, r, v, 1.0, a)
    assert rel_err(sym, ref) <= 1e-6
    assert rel_err(sym, std) <= 1e-6


@pytest.mark.parametrize("kind", KINDS)
def test_symmetric_shell_suspension_and_determinism(cuda_device, kind):
    s = S.shells_42_256(n_bodies=64)
    r = s.r_vectors()
    v = np.random.default_rng(1).standard_normal(3 * len(r))
    a = s.a
    x1 = _product(r, v, a, -1, kind=kind)
    x2 = _product(r, v, a, -1, kind=kind)
    assert np.array_equal(x1, x2)
    rows = np.arange(0, len(r), 7)
    ref = owall.wall_product(kind, r, v, 1.0, a, rows=rows)
    got = x1.reshape(-1, 3)[rows].reshape(-1)
    assert rel_err(got, ref) <= 1e-12


def test_symmetric_choice_rules(cuda_device):
    import torch
    from rigidmultiblobswall_gb300._native import RMWError
    with pytest.raises(RMWError):
        mob.autotune_set("uf", 100, "df64", -1)  # fewer than 256 blobs
    with pytest.raises(RMWError):
        mob.autotune_set("wt", 255, "mixed", -1)
    mob.autotune_set("uf", 1000, "fp64", -1)  # every precision mode has a symmetric kernel
    assert mob.autotune_lookup("uf", 1000, "fp64") == (-1, True)
    mob.autotune_clear()
    mob.autotune_set("uf", 1000, "df64", -1)
    assert mob.autotune_lookup("uf", 1000, "df64") == (-1, True)
    # periodic products fall back to the standard kernel and stay correct
    r, v = _blobs(1000, 5)
    L = np.array([30.0, 30.0, 0.0])
    got = mob.wall_product("uf", torch.tensor(r, device="cuda"), torch.tensor(v, device="cuda"), 1.0, 0.35,
                           mode="df64", periodic_length=L).cpu().numpy()
    mob.autotune_clear()
    ref = owall.wall_product("uf", r, v, 1.0, 0.35, periodic_length=L)
    assert rel_err(got, ref) <= 1e-12


def test_symmetric_beyond_six_gib_of_partial_sums(cuda_device):
    """200,000 blobs: 7.5 GB of partial sums, above the former fixed 6 GiB
    budget and inside the device-scaled one; sampled rows against the oracle."""
    import torch
    n = 200_000
    rng = np.random.default_rng(17)
    r = np.empty((n, 3))
    r[:, :2] = rng.uniform(0, 400.0, (n, 2))
    r[:, 2] = rng.uniform(0.6, 6.0, n)
    v = rng.standard_normal(3 * n)
    a = 0.35
    mob.autotune_clear()
    assert mob.autotune_lookup("uf", n, "mixed")[0] == -1
    got = mob.wall_product("uf", torch.tensor(r, device="cuda"), torch.tensor(v, device="cuda"), 1.0, a,
                           mode="mixed").cpu().numpy()
    rows = rng.choice(n, 40, replace=False)
    ref = owall.wall_product("uf", r, v, 1.0, a, rows=rows)
    assert rel_err(got.reshape(-1, 3)[rows].reshape(-1), ref) <= 1e-6


def _route(kind, mode, n):
    import ctypes
    from rigidmultiblobswall_gb300 import _native
    out = ctypes.c_int(-1)
    _native.call("rmw_wall_product_route", _native.KINDS[kind], {"fp64": 0, "mixed": 1, "df64": 2}[mode], n, None,
                 ctypes.byref(out))
    return out.value


@pytest.mark.parametrize("kind", ["uf", "ut", "wf", "wt"])
def test_banded_symmetric_product_matches_oracle(cuda_device, kind):
    """Above the partial-sum budget the df64 products run the symmetric kernel band by band of tile rows
    (bands summed in a fixed order).  A 48 MB scratch cap makes 20,000 blobs (59 MB of per-tile partial
    sums) take that route; all blocks against the oracle, the wall overlapping some blobs, and a second
    call bit-identical to the first."""
    from rigidmultiblobswall_gb300 import _native
    n = 20_000
    rng = np.random.default_rng(23)
    r = np.empty((n, 3))
    r[:, :2] = rng.uniform(0, 120.0, (n, 2))
    r[:, 2] = rng.uniform(0.1, 6.0, n)
    v = rng.standard_normal(3 * n)
    a = 0.35
    mob.autotune_clear()
    _native.set_scratch_limit(48 << 20)
    try:
        assert _route(kind, "df64", n) == 2
        got = mob.wall_product(kind, r, v, 1.0, a, mode="df64")
        again = mob.wall_product(kind, r, v, 1.0, a, mode="df64")
    finally:
        _native.set_scratch_limit(0)
    assert _route(kind, "df64", n) == 1
    rows = np.concatenate([rng.choice(n, 60, replace=False), [0, 127, 128, n - 1]])
    ref = owall.wall_product(kind, r, v, 1.0, a, rows=rows)
    assert rel_err(got.reshape(-1, 3)[rows].reshape(-1), ref) <= 1e-12
    assert np.array_equal(got, again)
    full = mob.wall_product(kind, r, v, 1.0, a, mode="df64")
    assert rel_err(got, full) <= 1e-13


def test_half_million_blob_df64_product_runs_symmetric(cuda_device):
    """500,000 blobs: 47 GB of per-tile partial sums, far above the budget; the df64 product still
    evaluates each unordered pair once (banded route), sampled rows against the oracle."""
    import torch
    n = 500_000
    assert _route("uf", "df64", n) == 2
    rng = np.random.default_rng(29)
    r = np.empty((n, 3))
    r[:, :2] = rng.uniform(0, 700.0, (n, 2))
    r[:, 2] = rng.uniform(0.6, 6.0, n)
    v = rng.standard_normal(3 * n)
    a = 0.35
    got = mob.wall_product("uf", torch.tensor(r, device="cuda"), torch.tensor(v, device="cuda"), 1.0, a,
                           mode="df64").cpu().numpy()
    rows = rng.choice(n, 24, replace=False)
    ref = owall.wall_product("uf", r, v, 1.0, a, rows=rows)
    assert rel_err(got.reshape(-1, 3)[rows].reshape(-1), ref) <= 1e-12
