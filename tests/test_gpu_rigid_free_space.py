"""GPU: the rigid-body handle in free space (set_wall(False), the reference's
*_no_wall implementations): dense body blocks, operator, block-diagonal
preconditioner, GMRES solve in every mode and Lanczos noise against the
oracle; wall-only features are refused; switching back restores the wall."""
import numpy as np
import pytest

from conftest import rel_err
from oracle import rigid as orig
from oracle import wall as owall
from rigidmultiblobswall_gb300 import suspensions as S
from rigidmultiblobswall_gb300._native import RMWError
from rigidmultiblobswall_gb300.rigid import RigidSystem

pytestmark = pytest.mark.gpu


def _system(nb=10, seed=4):
    susp = S.shells(nb, S.icosahedron(1.0), seed, 9.0, -2.0, 3.0, a=0.4)  # free space: no wall, z may be < 0
    sys_ = RigidSystem([12] * nb, 1.0, 0.4, wall=False)
    sys_.set_configuration(susp.r_vectors(), susp.locations)
    rig = orig.Rigid(susp.r_vectors(), susp.locations, np.arange(nb + 1) * 12, 1.0, 0.4, wall_present=False)
    return susp, sys_, rig


def test_free_space_blocks_operator_and_pc(cuda_device):
    susp, sys_, rig = _system()
    blocks = sys_.body_mobility()
    ref0 = owall.no_wall_dense(susp.r_vectors()[:12], 1.0, 0.4)
    assert rel_err(blocks[0].cpu().numpy(), ref0) <= 1e-13
    rng = np.random.default_rng(1)
    x = rng.standard_normal(sys_.size)
    assert rel_err(sys_.apply(x, mode="fp64").cpu().numpy(), rig.apply(x)) <= 1e-12
    sys_.build_pc()
    assert rel_err(sys_.apply_pc(x).cpu().numpy(), rig.apply_pc(x)) <= 1e-9


@pytest.mark.parametrize("mode", ["fp64", "df64", "mixed"])
def test_free_space_solve_matches_oracle(cuda_device, mode):
    susp, sys_, rig = _system()
    FT = np.zeros((susp.n_bodies, 6))
    FT[:, 2] = -1.0
    rhs = np.concatenate([np.zeros(3 * sys_.n_blobs), -FT.reshape(-1)])
    rhs /= np.linalg.norm(rhs)
    sys_.build_pc()
    x, info, it, rr = sys_.solve(rhs, tol=1e-8, mode=mode)
    assert info == 0 and rr <= 1e-8
    xo = x.cpu().numpy()
    true_res = np.linalg.norm(rhs - rig.apply(xo)) / np.linalg.norm(rhs)
    assert true_res <= 1.05e-8
    xr, itr, rrr = orig.gmres_right(rig.apply, rig.apply_pc, rhs, tol=1e-8)
    U, Ur = xo[3 * sys_.n_blobs:], xr[3 * sys_.n_blobs:]
    assert rel_err(U, Ur) <= 1e-6


def test_free_space_lanczos_and_guards(cuda_device):
    susp, sys_, rig = _system()
    sys_.build_pc(stochastic=True)
    rng = np.random.default_rng(2)
    z = rng.standard_normal(3 * sys_.n_blobs)
    noise, it = sys_.lanczos(z, factor=1.0, tol=1e-6, mode="fp64")
    ref, itr = orig.lanczos(rig.mobility_pc, z, factor=1.0, tol=1e-6)
    assert it == itr
    assert rel_err(noise.cpu().numpy(), rig.P_inv_mult(ref)) <= 1e-8
    with pytest.raises(RMWError):
        sys_.set_suspensions([5, 5])
    # back to the wall: the wall blocks return (heights must be above it)
    sys_.set_wall(True)
    r = susp.r_vectors()
    r[:, 2] += 5.0
    x = susp.locations.copy()
    x[:, 2] += 5.0
    sys_.set_configuration(r, x)
    rigw = orig.Rigid(r, x, np.arange(susp.n_bodies + 1) * 12, 1.0, 0.4)
    v = rng.standard_normal(sys_.size)
    assert rel_err(sys_.apply(v, mode="fp64").cpu().numpy(), rigw.apply(v)) <= 1e-12
