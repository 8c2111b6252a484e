"""GPU: the fused force-and-torque product (rmw_wall_force_torque) against
the oracle's composition of the four single products, in every precision
mode, with wall-overlapping blobs, periodic images, tile tails, the U-only
form (single_wall_mobility_trans_times_force_torque) and the
[F_1 T_1 F_2 T_2 ...] layout of Lub_Solver.Wall_Mobility_Mult."""
import numpy as np
import pytest

from conftest import rel_err
from oracle import wall as owall
from rigidmultiblobswall_gb300 import mobility as mob
from rigidmultiblobswall_gb300 import suspensions as S

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-12, "df64": 1e-12, "mixed": 1e-6}


def _case(n, seed, damped):
    rng = np.random.default_rng(seed)
    r = np.empty((n, 3))
    side = 2.5 * np.cbrt(max(n, 1))
    r[:, :2] = rng.uniform(0, side, (n, 2))
    r[:, 2] = rng.uniform(0.1 if damped else 0.8, 4.0, n)
    return r, rng.standard_normal(3 * n), rng.standard_normal(3 * n)


@pytest.mark.parametrize("mode", ["fp64", "df64", "mixed"])
@pytest.mark.parametrize("damped", [False, True])
@pytest.mark.parametrize("n", [1, 129, 700])
def test_fused_matches_four_products(cuda_device, mode, damped, n):
    r, F, T = _case(n, n + 3, damped)
    a = 0.3
    U, W = mob.wall_force_torque(r, F, T, 1.0, a, mode=mode)
    Ur, Wr = owall.force_torque(r, F, T, 1.0, a)
    assert rel_err(U, Ur) <= TOL[mode]
    assert rel_err(W, Wr) <= TOL[mode]
    Uonly = mob.single_wall_mobility_trans_times_force_torque_pycuda(r, F, T, 1.0, a, mode=mode)
    assert rel_err(Uonly, Ur) <= TOL[mode]


@pytest.mark.parametrize("mode", ["fp64", "df64", "mixed"])
@pytest.mark.parametrize("damped", [False, True])
def test_symmetric_route_matches_oracle(cuda_device, mode, damped):
    """With the symmetric kernels chosen for all four blocks (the default from
    4,096 blobs in FP64 and df64 and 8,192 in mixed; pinned here at 700), the
    FP64 and df64 [U; W] are sums of the four symmetric single products (mixed
    below 8,192 blobs keeps the one-sided fused pass)."""
    r, F, T = _case(700, 11, damped)
    a = 0.3
    mob.autotune_clear()
    try:
        for kind in ("uf", "ut", "wf", "wt"):
            mob.autotune_set(kind, len(r), mode, -1)
        U, W = mob.wall_force_torque(r, F, T, 1.0, a, mode=mode)
        Uonly = mob.single_wall_mobility_trans_times_force_torque_pycuda(r, F, T, 1.0, a, mode=mode)
    finally:
        mob.autotune_clear()
    Ur, Wr = owall.force_torque(r, F, T, 1.0, a)
    assert rel_err(U, Ur) <= TOL[mode]
    assert rel_err(W, Wr) <= TOL[mode]
    assert rel_err(Uonly, Ur) <= TOL[mode]


@pytest.mark.parametrize("damped", [False, True])
def test_mixed_symmetric_force_torque_rows_match_oracle(cuda_device, damped):
    """From 8,192 blobs the mixed [U; W] runs the symmetric fused kernel (all
    four blocks per unordered pair, both ways); sampled rows against the
    oracle, and the U-only form."""
    n = 8300
    r, F, T = _case(n, 23, damped)
    a = 0.3
    U, W = mob.wall_force_torque(r, F, T, 1.0, a, mode="mixed")
    Uonly = mob.single_wall_mobility_trans_times_force_torque_pycuda(r, F, T, 1.0, a, mode="mixed")
    rows = np.random.default_rng(5).choice(n, 40, replace=False)
    Ur, Wr = owall.force_torque(r, F, T, 1.0, a, rows=rows)
    pick = lambda x: x.reshape(-1, 3)[rows].reshape(-1)  # noqa: E731
    assert rel_err(pick(U), Ur) <= 1e-6
    assert rel_err(pick(W), Wr) <= 1e-6
    assert rel_err(pick(Uonly), Ur) <= 1e-6


@pytest.mark.parametrize("mode", ["fp64", "df64", "mixed"])
def test_fused_periodic(cuda_device, mode):
    r, F, T = _case(300, 7, True)
    L = np.array([9.0, 11.0, 0.0])
    U, W = mob.wall_force_torque(r, F, T, 1.0, 0.3, mode=mode, periodic_length=L)
    Ur, Wr = owall.force_torque(r, F, T, 1.0, 0.3, periodic_length=L)
    assert rel_err(U, Ur) <= TOL[mode]
    assert rel_err(W, Wr) <= TOL[mode]


def test_wall_mobility_mult_layout(cuda_device):
    r, F, T = _case(64, 5, False)
    X = np.concatenate([F.reshape(-1, 3), T.reshape(-1, 3)], axis=1).reshape(-1)
    out = mob.wall_mobility_mult(r, X, 1.0, 0.3, mode="df64").reshape(-1, 6)
    Ur, Wr = owall.force_torque(r, F, T, 1.0, 0.3)
    assert rel_err(out[:, 0:3].reshape(-1), Ur) <= 1e-12
    assert rel_err(out[:, 3:6].reshape(-1), Wr) <= 1e-12


def test_fused_shell_suspension_rows_and_device_path(cuda_device):
    import torch
    s = S.shells_42_256()
    r = s.r_vectors()
    n = len(r)
    rng = np.random.default_rng(2)
    F, T = rng.standard_normal(3 * n), rng.standard_normal(3 * n)
    U, W = mob.wall_force_torque(torch.tensor(r, device="cuda"), torch.tensor(F, device="cuda"),
                                 torch.tensor(T, device="cuda"), 1.0, s.a, mode="df64")
    assert U.is_cuda and W.is_cuda
    rows = np.arange(0, n, 97)
    Ur, Wr = owall.force_torque(r, F, T, 1.0, s.a, rows=rows)
    assert rel_err(U.cpu().numpy().reshape(-1, 3)[rows].reshape(-1), Ur) <= 1e-12
    assert rel_err(W.cpu().numpy().reshape(-1, 3)[rows].reshape(-1), Wr) <= 1e-12


def test_fused_errors_and_empty(cuda_device):
    from rigidmultiblobswall_gb300._native import RMWError
    U, W = mob.wall_force_torque(np.zeros((0, 3)), np.zeros(0), np.zeros(0), 1.0, 0.3)
    assert U.size == 0 and W.size == 0
    with pytest.raises(ValueError):
        mob.wall_force_torque(np.zeros((4, 3)), np.zeros(12), np.zeros(9), 1.0, 0.3)
    with pytest.raises(RMWError):
        mob.wall_force_torque(np.ones((4, 3)), np.zeros(12), np.zeros(12), 1.0, -0.3)
