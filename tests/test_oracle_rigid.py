"""CPU: the oracle's rigid-body pieces against the golden vectors of the
reference's own solve (linear operator, preconditioners, GMRES, Lanczos,
one Euler-Maruyama step)."""
import numpy as np
import pytest

from conftest import golden, rel_err
from oracle import rigid

CASES = ["s42", "s12"]


def system(g, c):
    nb = g[c + "_locs"].shape[0]
    n_per = g[c + "_ref_cfg"].shape[0]
    offsets = np.arange(nb + 1) * n_per
    a, eta = g[c + "_params"]
    return rigid.Rigid(g[c + "_r"], g[c + "_locs"], offsets, eta, a)


@pytest.mark.parametrize("c", CASES)
def test_oracle_rigid_pieces_match_reference(c):
    g = golden("rigid.npz")
    S = system(g, c)
    np.testing.assert_allclose(np.array(S.Ks), g[c + "_K"], rtol=0, atol=1e-14)
    assert rel_err(S.apply(g[c + "_x"]), g[c + "_Ax"]) <= 1e-13
    assert rel_err(S.apply_pc(g[c + "_x"]), g[c + "_Px"]) <= 1e-10
    assert rel_err(S.mobility_pc(g[c + "_w"]), g[c + "_mob_pc_w"]) <= 1e-10
    assert rel_err(S.P_inv_mult(g[c + "_w"]), g[c + "_P_inv_w"]) <= 1e-12


@pytest.mark.parametrize("c", CASES)
def test_oracle_gmres_matches_reference_solution(c):
    g = golden("rigid.npz")
    S = system(g, c)
    FT = g[c + "_FT"]
    rhs = np.concatenate([np.zeros(3 * S.N), -FT.flatten()])
    nrm = np.linalg.norm(rhs)
    x, it, rel = rigid.gmres_right(S.apply, S.apply_pc, rhs / nrm, tol=1e-8, restart=60)
    x *= nrm
    assert rel <= 1e-8
    U, Uref = x[3 * S.N:], g[c + "_sol"][3 * S.N:]
    assert rel_err(U, Uref) <= 1e-6  # both solutions are within the 1e-8 residual tolerance
    assert abs(it - int(g[c + "_info"][1])) <= 2


@pytest.mark.parametrize("c", CASES)
def test_oracle_lanczos_and_em_step_match_reference(c):
    g = golden("rigid.npz")
    S = system(g, c)
    noise, it = rigid.lanczos(S.mobility_pc, g[c + "_z"], factor=np.sqrt(2.0 / 1e-3), tol=1e-3)
    noise = S.P_inv_mult(noise)
    assert it == int(g[c + "_lanczos_iters"][0])
    assert rel_err(noise, g[c + "_noise"]) <= 1e-9
    rhs = np.concatenate([-noise, -g[c + "_FT"].flatten()])
    nrm = np.linalg.norm(rhs)
    x, _, rel = rigid.gmres_right(S.apply, S.apply_pc, rhs / nrm, tol=1e-8)
    vel = (x * nrm)[3 * S.N:]
    nl, nq = rigid.em_update(g[c + "_locs"], g[c + "_quats"], vel, float(g[c + "_bd_dt"][0]))
    assert np.abs(nl - g[c + "_bd_locs"]).max() <= 1e-9
    assert np.abs(nq - g[c + "_bd_quats"]).max() <= 1e-9


@pytest.mark.parametrize("case", ["small", "tight", "loose"])
def test_oracle_lanczos_dense_matches_reference(case):
    g = golden("lanczos.npz")
    M = g[case + "_M"]
    tol, factor = g[case + "_tol"]
    noise, it = rigid.lanczos(lambda v: M @ v, g[case + "_z"], factor=factor, tol=tol)
    assert it == int(g[case + "_iters"][0])
    assert rel_err(noise, g[case + "_noise"]) <= 1e-10
