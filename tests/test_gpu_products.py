"""GPU parity of the four wall-RPY products against the reference golden vectors
and the CPU oracle.

Tolerances (relative 2-norm error of the whole output vector):
  FP64 mode   <= 1e-12
  mixed mode  <= 1e-6
"""

import numpy as np
import pytest

from conftest import golden, rel_err
from oracle import wall
from rigidmultiblobswall_gb300 import mobility as mb
from rigidmultiblobswall_gb300 import suspensions as S

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-12, "df64": 1e-12, "mixed": 1e-6}
CASES = ["far", "damped", "touching", "periodic", "single"]
KINDS = ["uf", "ut", "wf", "wt"]
FN = {
    "uf": mb.single_wall_mobility_trans_times_force_pycuda,
    "ut": mb.single_wall_mobility_trans_times_torque_pycuda,
    "wf": mb.single_wall_mobility_rot_times_force_pycuda,
    "wt": mb.single_wall_mobility_rot_times_torque_pycuda,
}


@pytest.mark.parametrize("mode", ["fp64", "df64", "mixed"])
@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("kind", KINDS)
def test_products_match_reference_golden(cuda_device, kind, case, mode):
    g = golden("products.npz")
    a, eta = g[case + "_params"]
    out = FN[kind](g[case + "_r"], g[case + "_v"], eta, a, periodic_length=g[case + "_L"], mode=mode)
    assert out.shape == (g[case + "_r"].size,)
    assert rel_err(out, g[case + "_" + kind]) <= TOL[mode]


@pytest.mark.parametrize("damped", [False, True])
@pytest.mark.parametrize("mode", ["fp64", "df64", "mixed"])
@pytest.mark.parametrize("kind", KINDS)
def test_plain_matvec_workload_matches_oracle(cuda_device, kind, mode, damped):
    """2048 free blobs; with damped=True every 17th blob sits at z = 0.3a
    (wall regularisation on), where the far-field wall image nearly cancels
    the free-space term and exposes any precision leak in the pair algebra."""
    r, f, eta, a = S.blobs_wall_matvec(2048, seed=0)
    if damped:
        r[::17, 2] = 0.3 * a
    ref = wall.wall_product(kind, r, f, eta, a)
    assert rel_err(FN[kind](r, f, eta, a, mode=mode), ref) <= TOL[mode]


@pytest.mark.parametrize("mode", ["fp64", "df64", "mixed"])
@pytest.mark.parametrize("kind", KINDS)
def test_shell_suspension_rows_match_oracle(cuda_device, kind, mode):
    """256 shells x 42 blobs (blobs below z=a present): 400 sampled target rows."""
    s = S.shells_42_256()
    r = s.r_vectors()
    assert (r[:, 2] < s.a).any()
    rng = np.random.default_rng(3)
    v = rng.standard_normal(r.shape)
    rows = np.sort(rng.choice(len(r), 400, replace=False))
    ref = wall.wall_product(kind, r, v, s.eta, s.a, rows=rows)
    out = FN[kind](r, v, s.eta, s.a, mode=mode).reshape(-1, 3)[rows]
    assert rel_err(out, ref) <= TOL[mode]


def test_device_path_equals_host_path(cuda_device):
    import torch
    r, f, eta, a = S.blobs_wall_matvec(777, seed=4)
    host = mb.single_wall_mobility_rot_times_torque_numba(r, f, eta, a)
    rt = torch.tensor(r, device=cuda_device)
    ft = torch.tensor(f, device=cuda_device)
    dev = mb.single_wall_mobility_rot_times_torque_numba(rt, ft, eta, a)
    assert dev.is_cuda and dev.dtype == torch.float64
    np.testing.assert_array_equal(dev.cpu().numpy(), host)


def test_inputs_are_not_modified(cuda_device):
    r, f, eta, a = S.blobs_wall_matvec(100, seed=6)
    r[:4, 2] = 0.1
    r0, f0 = r.copy(), f.copy()
    mb.single_wall_mobility_trans_times_force_numba(r, f, eta, a)
    np.testing.assert_array_equal(r, r0)
    np.testing.assert_array_equal(f, f0)


def test_empty_and_single_blob(cuda_device):
    out = mb.single_wall_mobility_trans_times_force_pycuda(np.zeros((0, 3)), np.zeros(0), 1.0, 0.5)
    assert out.shape == (0,)
    r = np.array([[0.0, 0.0, 2.0]])
    f = np.array([0.0, 0.0, 1.0])
    ref = wall.wall_product("uf", r, f, 1.0, 0.5)
    assert rel_err(mb.single_wall_mobility_trans_times_force_pycuda(r, f, 1.0, 0.5), ref) <= 1e-15


def test_tile_tail_sizes(cuda_device):
    """Sizes around the 128-target / 128-source tile edges and the chunk split."""
    for n in (127, 128, 129, 255, 257, 1025):
        r, f, eta, a = S.blobs_wall_matvec(n, seed=n)
        for kind in ("uf", "wt"):
            for mode in ("fp64", "df64"):
                assert rel_err(FN[kind](r, f, eta, a, mode=mode), wall.wall_product(kind, r, f, eta, a)) <= 1e-12


def test_errors_raise(cuda_device):
    from rigidmultiblobswall_gb300._native import RMWError
    r, f, eta, a = S.blobs_wall_matvec(10, seed=1)
    with pytest.raises(RMWError):
        mb.single_wall_mobility_trans_times_force_pycuda(r, f, eta, -1.0)
    with pytest.raises(ValueError):
        mb.single_wall_mobility_trans_times_force_pycuda(r, f, eta, a, mode="fp16")


@pytest.mark.parametrize("kind", KINDS)
def test_df64_large_suspension_rows(cuda_device, kind):
    """df64 at 4096 shells x 42 blobs (172,032 blobs): 96 sampled rows against
    the FP64 oracle at the FP64-mode bar (1e-12)."""
    import torch
    s = S.shells_42_4096()
    r = s.r_vectors()
    v = np.random.default_rng(13).standard_normal(r.shape)
    out = mb.wall_product(kind, torch.tensor(r, device=cuda_device), torch.tensor(v, device=cuda_device), s.eta,
                          s.a, mode="df64").cpu().numpy()
    rows = np.random.default_rng(14).choice(s.n_blobs, 96, replace=False)
    ref = wall.wall_product(kind, r, v, s.eta, s.a, rows=rows)
    assert rel_err(out.reshape(-1, 3)[rows], ref) <= 1e-12


def test_large_suspension_linearity_and_sampled_rows(cuda_device):
    """4096 shells x 42 blobs (172,032 blobs), mixed mode: linearity of the
    product and 128 sampled rows against the FP64 oracle."""
    import torch
    s = S.shells_42_4096()
    r = torch.tensor(s.r_vectors(), device=cuda_device)
    g = torch.Generator(device="cpu").manual_seed(11)
    f = torch.randn(r.shape, generator=g, dtype=torch.float64).to(cuda_device)
    h = torch.randn(r.shape, generator=g, dtype=torch.float64).to(cuda_device)
    uf = mb.wall_product("uf", r, f, s.eta, s.a, mode="mixed")
    uh = mb.wall_product("uf", r, h, s.eta, s.a, mode="mixed")
    ufh = mb.wall_product("uf", r, 2.0 * f - 0.5 * h, s.eta, s.a, mode="mixed")
    assert rel_err((ufh).cpu().numpy(), (2.0 * uf - 0.5 * uh).cpu().numpy()) <= 1e-6
    rows = np.random.default_rng(12).choice(s.n_blobs, 128, replace=False)
    ref = wall.wall_product("uf", s.r_vectors(), f.cpu().numpy(), s.eta, s.a, rows=rows)
    assert rel_err(uf.cpu().numpy().reshape(-1, 3)[rows], ref) <= 1e-6
