"""GPU parity of the rigid-body path (operator, preconditioners, GMRES solve,
Lanczos noise, Euler-Maruyama step) against the golden vectors of the
reference's own solve and against the oracle on larger suspensions.

Tolerances (relative 2-norm):
  operator / K / K^T            1e-12
  block-diagonal PC apply       1e-9   (explicit inverses of 126x126 SPD blocks, cond ~1e4)
  GMRES body velocities         1e-6   (both sides stop at a 1e-8 relative residual)
  Lanczos noise (same z)        1e-8, identical iteration count
  mixed-precision solve         same 1e-8 FP64 residual, velocities within 1e-6 of FP64
"""
import numpy as np
import pytest

from conftest import golden, rel_err
from oracle import rigid as orc
from rigidmultiblobswall_gb300 import integrator
from rigidmultiblobswall_gb300 import suspensions as S
from rigidmultiblobswall_gb300.rigid import RigidSystem

pytestmark = pytest.mark.gpu
CASES = ["s42", "s12"]


def gpu_system(g, c):
    nb = g[c + "_locs"].shape[0]
    n_per = g[c + "_ref_cfg"].shape[0]
    a, eta = g[c + "_params"]
    s = RigidSystem([n_per] * nb, eta, a)
    s.set_configuration(g[c + "_r"], g[c + "_locs"])
    return s


@pytest.mark.parametrize("c", CASES)
def test_operator_and_K_match_reference(cuda_device, c):
    g = golden("rigid.npz")
    s = gpu_system(g, c)
    assert rel_err(s.apply(g[c + "_x"]).cpu().numpy(), g[c + "_Ax"]) <= 1e-12
    n3 = 3 * s.n_blobs
    u = g[c + "_x"][n3:]
    Ku = np.concatenate([K @ u[6 * b:6 * b + 6] for b, K in enumerate(g[c + "_K"])])
    assert rel_err(s.K_mult(u).cpu().numpy(), Ku) <= 1e-13
    lam = g[c + "_x"][:n3]
    nper = g[c + "_K"].shape[1] // 3
    KTl = np.concatenate([K.T @ lam[3 * nper * b:3 * nper * (b + 1)] for b, K in enumerate(g[c + "_K"])])
    assert rel_err(s.KT_mult(lam).cpu().numpy(), KTl) <= 1e-13


@pytest.mark.parametrize("c", CASES)
def test_preconditioners_match_reference(cuda_device, c):
    g = golden("rigid.npz")
    s = gpu_system(g, c)
    s.build_pc(stochastic=True)
    assert rel_err(s.apply_pc(g[c + "_x"]).cpu().numpy(), g[c + "_Px"]) <= 1e-9
    assert rel_err(s.mobility_pc(g[c + "_w"]).cpu().numpy(), g[c + "_mob_pc_w"]) <= 1e-9
    assert rel_err(s.P_inv_mult(g[c + "_w"]).cpu().numpy(), g[c + "_P_inv_w"]) <= 1e-12


@pytest.mark.parametrize("c", CASES)
def test_body_mobility_blocks_match_oracle(cuda_device, c):
    from oracle import wall
    g = golden("rigid.npz")
    s = gpu_system(g, c)
    blocks = s.body_mobility()
    nper = g[c + "_ref_cfg"].shape[0]
    a, eta = g[c + "_params"]
    for b in (0, len(blocks) - 1):
        ref = wall.dense_mobility(g[c + "_r"][b * nper:(b + 1) * nper], eta, a)
        assert rel_err(blocks[b].cpu().numpy(), ref) <= 1e-13


@pytest.mark.parametrize("mode", ["fp64", "df64", "mixed"])
@pytest.mark.parametrize("c", CASES)
def test_solve_matches_reference(cuda_device, c, mode):
    g = golden("rigid.npz")
    s = gpu_system(g, c)
    sol, info, its, rr = integrator.solve_mobility_problem(s, g[c + "_FT"], tol=1e-8, mode=mode)
    assert info == 0 and rr <= 1e-8
    sol = sol.cpu().numpy()
    n3 = 3 * s.n_blobs
    assert rel_err(sol[n3:], g[c + "_sol"][n3:]) <= 1e-6
    # the FP64 residual of the GPU solution, checked by the oracle operator
    o = orc.Rigid(g[c + "_r"], g[c + "_locs"], s.offsets, s.eta, s.a)
    rhs = np.concatenate([np.zeros(n3), -g[c + "_FT"].flatten()])
    assert np.linalg.norm(rhs - o.apply(sol)) <= 1.05e-8 * np.linalg.norm(rhs)


@pytest.mark.parametrize("mode", ["fp64", "mixed"])
def test_scaled_solve_of_device_inputs(cuda_device, mode):
    """Device inputs take rmw_rigid_solve_scaled (|b|, b / |b| and the scaling back in the library): the
    same solution as the host path, which scales on the host; zero and unconverged cases keep the
    reference's return convention."""
    import torch
    g = golden("rigid.npz")
    s = gpu_system(g, "s42")
    ft = torch.as_tensor(g["s42_FT"], device="cuda")
    noise = torch.randn(3 * s.n_blobs, dtype=torch.float64, device="cuda", generator=torch.Generator(
        device="cuda").manual_seed(5)) * 1e-2
    x_dev, info, its, rr = integrator.solve_mobility_problem(s, ft, noise=noise, tol=1e-8, mode=mode)
    x_host, info_h, its_h, rr_h = integrator.solve_mobility_problem(s, g["s42_FT"], noise=noise.cpu().numpy(),
                                                                     tol=1e-8, mode=mode)
    assert info == 0 and info_h == 0 and abs(its - its_h) <= 1 and rr <= 1e-8
    assert rel_err(x_dev.cpu().numpy(), x_host.cpu().numpy()) <= 1e-10
    o = orc.Rigid(g["s42_r"], g["s42_locs"], s.offsets, s.eta, s.a)
    n3 = 3 * s.n_blobs
    rhs = np.concatenate([-noise.cpu().numpy(), -g["s42_FT"].flatten()])
    assert np.linalg.norm(rhs - o.apply(x_dev.cpu().numpy())) <= 1.05e-8 * np.linalg.norm(rhs)
    z, info, its, rr = integrator.solve_mobility_problem(s, torch.zeros_like(ft), mode=mode)
    assert info == 0 and its == 0 and float(z.abs().max()) == 0.0
    b = torch.as_tensor(np.random.default_rng(0).standard_normal(s.size), device="cuda")
    x, info, its, rr = s.solve(b, tol=1e-14, maxiter=1, scaled=True)
    assert info == 1 and its == 1 and rr > 1e-14 and bool(torch.isfinite(x).all())


@pytest.mark.parametrize("c", CASES)
def test_lanczos_and_em_step_match_reference(cuda_device, c):
    g = golden("rigid.npz")
    s = gpu_system(g, c)
    s.build_pc(stochastic=True)
    noise, it = s.lanczos(g[c + "_z"], factor=np.sqrt(2.0 / 1e-3), tol=1e-3)
    assert it == int(g[c + "_lanczos_iters"][0])
    assert rel_err(noise.cpu().numpy(), g[c + "_noise"]) <= 1e-8
    nper = g[c + "_ref_cfg"].shape[0]
    nb = g[c + "_locs"].shape[0]
    # body-frame coordinates: r_ref = R(q)^T (r - x)
    Rm = S.rotation_matrices(g[c + "_quats"])
    rref = np.einsum("bji,bkj->bki", Rm, g[c + "_r"].reshape(nb, nper, 3) - g[c + "_locs"][:, None, :])
    step = integrator.BrownianStepper(s, g[c + "_locs"], g[c + "_quats"], rref.reshape(-1, 3), kT=1.0)
    np.testing.assert_allclose(step.r_vectors().cpu().numpy(), g[c + "_r"], rtol=0, atol=1e-13)
    out = step.step(float(g[c + "_bd_dt"][0]), g[c + "_FT"], z=g[c + "_z"])
    assert out["lanczos_iterations"] == int(g[c + "_lanczos_iters"][0])
    assert np.abs(step.x.cpu().numpy() - g[c + "_bd_locs"]).max() <= 1e-9
    assert np.abs(step.q.cpu().numpy() - g[c + "_bd_quats"]).max() <= 1e-9


@pytest.mark.parametrize("case", ["small", "tight", "loose"])
def test_generic_lanczos_matches_reference(cuda_device, case):
    from rigidmultiblobswall_gb300.stochastic_forcing import stochastic_forcing_lanczos
    g = golden("lanczos.npz")
    tol, factor = g[case + "_tol"]
    noise, it = stochastic_forcing_lanczos(factor=factor, tolerance=tol, mobility=g[case + "_M"], z=g[case + "_z"])
    assert it == int(g[case + "_iters"][0])
    assert rel_err(noise, g[case + "_noise"]) <= 1e-9


def test_generic_gmres_with_reference_style_operators(cuda_device):
    """utils.gmres drop-in with numpy-only operators (the reference's calling
    convention): linear_operator_rigid + the block-diagonal preconditioner."""
    from rigidmultiblobswall_gb300 import multi_bodies as mbs
    from rigidmultiblobswall_gb300.general_application_utils import gmres
    from rigidmultiblobswall_gb300.body import Body
    from rigidmultiblobswall_gb300.quaternion import Quaternion
    g = golden("rigid.npz")
    c = "s12"
    a, eta = g[c + "_params"]
    bodies = [Body(l, Quaternion(q), g[c + "_ref_cfg"], a) for l, q in zip(g[c + "_locs"], g[c + "_quats"])]
    N = sum(b.Nblobs for b in bodies)
    r = mbs.get_blobs_r_vectors(bodies, N)
    assert np.abs(r - g[c + "_r"]).max() <= 1e-13
    PC = mbs.build_block_diagonal_preconditioner(bodies, [], r, N, eta, a)
    A = lambda x: mbs.linear_operator_rigid(x, bodies, [], r, eta, a)  # noqa: E731
    rhs = np.concatenate([np.zeros(3 * N), -g[c + "_FT"].flatten()])
    nrm = np.linalg.norm(rhs)
    count = []
    x, info = gmres(A, rhs / nrm, tol=1e-8, M=PC, maxiter=1000, restart=60, callback=lambda rk: count.append(rk))
    assert info == 0 and len(count) > 0
    assert rel_err((x * nrm)[3 * N:], g[c + "_sol"][3 * N:]) <= 1e-6


def test_larger_suspension_matches_oracle(cuda_device):
    """32 shells x 42 blobs: GPU solve (FP64 and mixed) against the oracle's solve."""
    susp = S.shells_42_256(n_bodies=32, seed=7)
    r = susp.r_vectors()
    s = RigidSystem([42] * 32, susp.eta, susp.a)
    s.set_configuration(r, susp.locations)
    FT = np.zeros((32, 6))
    FT[:, 2] = -1.0
    o = orc.Rigid(r, susp.locations, s.offsets, susp.eta, susp.a)
    rhs = np.concatenate([np.zeros(3 * s.n_blobs), -FT.flatten()])
    xo, ito, relo = orc.gmres_right(o.apply, o.apply_pc, rhs / np.linalg.norm(rhs), tol=1e-8)
    xo *= np.linalg.norm(rhs)
    for mode in ("fp64", "df64", "mixed"):
        sol, info, its, rr = integrator.solve_mobility_problem(s, FT, tol=1e-8, mode=mode)
        sol = sol.cpu().numpy()
        assert info == 0
        assert np.linalg.norm(rhs - o.apply(sol)) <= 1.05e-8 * np.linalg.norm(rhs)
        assert rel_err(sol[3 * s.n_blobs:], xo[3 * s.n_blobs:]) <= 1e-6
        if mode != "mixed":
            assert abs(its - ito) <= 2


def test_solver_error_paths(cuda_device):
    from rigidmultiblobswall_gb300._native import RMWError
    with pytest.raises(ValueError):
        RigidSystem([], 1.0, 0.5)
    s = RigidSystem([3], 1.0, 0.5)
    r = np.array([[0.0, 0.0, 2.0], [1.0, 0.0, 2.0], [0.0, 1.0, 2.0]])
    s.set_configuration(r, r.mean(axis=0, keepdims=True))
    with pytest.raises(RMWError):
        s.apply_pc(np.ones(s.size))  # preconditioner not built
    # a zero right-hand side returns the zero solution
    sol, info, its, rr = integrator.solve_mobility_problem(s, np.zeros((1, 6)))
    assert info == 0 and float(sol.abs().max()) == 0.0
    # maxiter reached: info > 0, no exception (several bodies, so the
    # block-diagonal preconditioner is not exact)
    g = golden("rigid.npz")
    s2 = gpu_system(g, "s12")
    s2.build_pc()
    x, info, its, rr = s2.solve(np.random.default_rng(0).standard_normal(s2.size), tol=1e-14, maxiter=1)
    assert info == 1 and its == 1 and rr > 1e-14


@pytest.mark.parametrize("tol", [1e-6, 1e-8, 1e-11])
def test_mixed_refinement_reports_the_true_residual(cuda_device, tol):
    """The mixed refinement updates its residual as r - A32 d (FP32-pair
    product of the correction) once |r| / |b| <= 1e4 tol, instead of
    recomputing b - A x in double-float: the reported relative residual stays
    within a tenth of the tolerance of the oracle's FP64 residual of the
    returned solution, which meets the tolerance."""
    susp = S.shells_42_256(n_bodies=20, seed=21)
    r = susp.r_vectors()
    s = RigidSystem([42] * 20, susp.eta, susp.a)
    s.set_configuration(r, susp.locations)
    FT = np.random.default_rng(4).standard_normal((20, 6))
    rhs = np.concatenate([np.zeros(3 * s.n_blobs), -FT.flatten()])
    o = orc.Rigid(r, susp.locations, s.offsets, susp.eta, susp.a)
    sol, info, its, rr = integrator.solve_mobility_problem(s, FT, tol=tol, mode="mixed")
    true_rr = np.linalg.norm(rhs - o.apply(sol.cpu().numpy())) / np.linalg.norm(rhs)
    assert info == 0 and rr <= tol
    assert true_rr <= 1.05 * tol
    assert abs(rr - true_rr) <= 0.1 * tol


def test_fp32_preconditioner_for_mixed_solves(cuda_device):
    """build_pc(mode='mixed') factorises the body blocks in FP32: the mixed
    solve still reaches the FP64 residual bar with the same body velocities,
    and an FP64 solve afterwards rebuilds the FP64 preconditioner (same
    iterations and solution as with a fresh FP64 build)."""
    susp = S.shells_42_256(n_bodies=24, seed=12)
    r = susp.r_vectors()
    s = RigidSystem([42] * 24, susp.eta, susp.a)
    s.set_configuration(r, susp.locations)
    FT = np.zeros((24, 6))
    FT[:, 2] = -1.0
    rhs = np.concatenate([np.zeros(3 * s.n_blobs), -FT.flatten()])
    o = orc.Rigid(r, susp.locations, s.offsets, susp.eta, susp.a)
    s.build_pc(mode="fp64")
    x64, info64, it64, _ = integrator.solve_mobility_problem(s, FT, tol=1e-8, mode="fp64")
    s.build_pc(mode="mixed")
    xm, infom, itm, _ = integrator.solve_mobility_problem(s, FT, tol=1e-8, mode="mixed")
    assert infom == 0 and abs(itm - it64) <= 2
    xm = xm.cpu().numpy()
    assert np.linalg.norm(rhs - o.apply(xm)) <= 1.05e-8 * np.linalg.norm(rhs)
    assert rel_err(xm[3 * s.n_blobs:], x64.cpu().numpy()[3 * s.n_blobs:]) <= 1e-6
    s.build_pc(mode="mixed")
    x2, info2, it2, _ = integrator.solve_mobility_problem(s, FT, tol=1e-8, mode="fp64")
    assert info2 == 0 and it2 == it64
    assert rel_err(x2.cpu().numpy(), x64.cpu().numpy()) <= 1e-12


@pytest.mark.parametrize("stochastic", [False, True])
def test_fp32_built_preconditioner_matches_oracle(cuda_device, stochastic):
    """The FP32-built blocks of the mixed solves against the oracle's FP64 preconditioner apply: the
    deterministic build inverts each block by register-resident Gauss-Jordan sweeps, the stochastic one
    through the FP32 Cholesky (it also needs L and L^-1).  A handle of 12- and 42-blob bodies exercises the
    padded sweep of the smaller blocks.  FP32 inverses of blocks with condition numbers ~1e4: 5e-3."""
    rng = np.random.default_rng(21)
    sh12, sh42 = S.icosahedron(1.0), S.icosphere_42(1.0)
    counts = [12, 42, 42, 12, 42, 12]
    cen = np.array([[3.0 * k, 0.0, 1.6 + 0.3 * k] for k in range(len(counts))])
    q = S.random_quaternions(rng, len(counts))
    r = np.concatenate([S.blob_positions(cen[k:k + 1], q[k:k + 1], sh12 if c == 12 else sh42)
                        for k, c in enumerate(counts)])
    a = 0.25
    s = RigidSystem(counts, 1.0, a)
    s.set_configuration(r, cen)
    s.build_pc(stochastic=stochastic, mode="mixed")
    o = orc.Rigid(r, cen, s.offsets, 1.0, a)
    for _ in range(2):
        x = rng.standard_normal(s.size)
        err = rel_err(s.apply_pc(x).cpu().numpy(), o.apply_pc(x))
        assert err <= 5e-3, err
    s.close()


def test_mixed_operator_matches_oracle(cuda_device):
    """The operator of the mixed inner solves (FP32-pair product, K U and K^T lambda in FP32 on offsets
    formed in FP64) against the oracle's FP64 operator, on a random vector and on a solution of the
    mobility problem (constraint forces whose body sums cancel): body rows <= 1e-5 relative; blob rows
    <= 1e-5 of |M lambda| (at a solution M lambda - K U cancels to the residual)."""
    susp = S.shells_42_256(n_bodies=24, seed=12)
    r = susp.r_vectors()
    s = RigidSystem([42] * 24, susp.eta, susp.a)
    s.set_configuration(r, susp.locations)
    o = orc.Rigid(r, susp.locations, s.offsets, susp.eta, susp.a)
    FT = np.zeros((24, 6))
    FT[:, 2] = -1.0
    sol, info, _, _ = integrator.solve_mobility_problem(s, FT, tol=1e-8, mode="fp64")
    assert info == 0
    n3 = 3 * s.n_blobs
    for x in (np.random.default_rng(5).standard_normal(s.size), sol.cpu().numpy()):
        got = s.apply(x, mode="mixed").cpu().numpy()
        ref = o.apply(x)
        m_lam = o.apply(np.concatenate([x[:n3], np.zeros(s.size - n3)]))[:n3]
        assert np.linalg.norm(got[:n3] - ref[:n3]) <= 1e-5 * np.linalg.norm(m_lam)
        assert rel_err(got[n3:], ref[n3:]) <= 1e-5
    s.close()
