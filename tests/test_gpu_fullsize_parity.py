"""GPU parity at the full sizes of the benchmark workloads, checked by the oracle.

The smaller rigid-body tests pin the solver against the reference's own goldens on a few bodies; these
run the three solver workloads at their full sizes and let the oracle (the C restatement of the wall
products plus the numpy restatement of K, the operator, the preconditioners, GMRES and Lanczos) judge:

* 256 shells x 42 blobs (10,752 blobs): the mobility solve to a 1e-8 relative residual in FP64, df64,
  mixed and mixed with the near-field augmented preconditioner.  The oracle's FP64 residual
  |b - A x| / |b| of every returned solution is <= 1.05e-8, and the body velocities agree with the
  oracle's own solve (general_application_utils.py:514-635 with the block-diagonal preconditioner of
  multi_bodies.py:752-903) within 1e-6.
* 1024 shells x 12 blobs (12,288 blobs): one Euler-Maruyama step (quaternion_integrator_multi_bodies.py:
  262-322) against the oracle's step fed the same z: Lanczos iterations, noise, velocities, new
  locations and quaternions.
* 64 suspensions of 16..512 42-blob shells (658,140 blobs): every suspension's batched solution meets
  the oracle's residual bar; two suspensions' velocities and Lanczos noise against the oracle's own.
"""
import numpy as np
import pytest

from conftest import rel_err
from oracle import rigid as orc
from rigidmultiblobswall_gb300 import integrator
from rigidmultiblobswall_gb300 import suspensions as S
from rigidmultiblobswall_gb300.rigid import RigidSystem

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cfg2(cuda_device):
    s2 = S.shells_42_256()
    r = s2.r_vectors()
    sys2 = RigidSystem([42] * s2.n_bodies, s2.eta, s2.a)
    sys2.set_configuration(r, s2.locations)
    o = orc.Rigid(r, s2.locations, sys2.offsets, s2.eta, s2.a)
    FT = np.zeros((s2.n_bodies, 6))
    FT[:, 2] = -1.0
    rhs = np.concatenate([np.zeros(3 * sys2.n_blobs), -FT.flatten()])
    nrm = np.linalg.norm(rhs)
    xo, ito, relo = orc.gmres_right(o.apply, o.apply_pc, rhs / nrm, tol=1e-8)
    return s2, sys2, o, FT, rhs, xo * nrm, ito


@pytest.mark.parametrize("arm", ["fp64", "df64", "mixed", "mixed+nearfield"])
def test_shells42x256_solve_meets_oracle_residual(cfg2, arm):
    s2, sys2, o, FT, rhs, xo, ito = cfg2
    mode = arm.split("+")[0]
    sys2.build_pc(mode=mode)
    if arm.endswith("nearfield"):
        from rigidmultiblobswall_gb300 import nearfield as nf
        R = float(np.linalg.norm(s2.shell[0]))
        graphs = nf.cluster_training_data(s2.shell, s2.a, 1.0, 256, d_range=(2 * R + 2 * s2.a, 6 * R),
                                          z_range=(1.1 * R, 5 * R), seed=11, device=sys2.device)
        model = nf.NearfieldModel(body_radius=R, cutoff=6 * R, seed=2)
        model.train(graphs, steps=600, lr=2e-3)
        model.attach(sys2, exact_cutoff=3 * R)
    try:
        sol, info, its, rr = integrator.solve_mobility_problem(sys2, FT, tol=1e-8, mode=mode)
    finally:
        if arm.endswith("nearfield"):
            nf.detach(sys2)
    sol = sol.cpu().numpy()
    n3 = 3 * sys2.n_blobs
    assert info == 0 and rr <= 1e-8
    true_rr = np.linalg.norm(rhs - o.apply(sol)) / np.linalg.norm(rhs)
    assert true_rr <= 1.05e-8, true_rr
    assert rel_err(sol[n3:], xo[n3:]) <= 1e-6
    if mode != "mixed":
        assert abs(its - ito) <= 2


@pytest.mark.parametrize("mode", ["fp64", "mixed"])
def test_shells12x1024_em_step_matches_oracle(cuda_device, mode):
    import torch
    s3 = S.shells_12_1024()
    nb = s3.n_bodies
    sys3 = RigidSystem([12] * nb, s3.eta, s3.a)
    r_ref = np.tile(s3.shell, (nb, 1))
    dt, kT = 1e-3, 1.0
    FT = np.zeros((nb, 6))
    FT[:, 2] = -1.0
    z = np.random.default_rng(3).standard_normal(3 * s3.n_blobs)
    step = integrator.BrownianStepper(sys3, s3.locations, s3.quaternions, r_ref, kT=kT, mode=mode)
    r0 = step.r_vectors().cpu().numpy()
    out = step.step(dt, FT, z=torch.tensor(z, device=sys3.device))
    vel = out["velocities"].cpu().numpy()
    # the GPU noise of the same draw (the step's configuration, before the update)
    sysn = RigidSystem([12] * nb, s3.eta, s3.a)
    sysn.set_configuration(r0, s3.locations)
    sysn.build_pc(stochastic=True, mode=mode)
    noise, itl = sysn.lanczos(z, factor=np.sqrt(2 * kT / dt), tol=1e-3, mode=mode)
    noise = noise.cpu().numpy()
    # oracle step
    o = orc.Rigid(r0, s3.locations, sysn.offsets, s3.eta, s3.a)
    o.build_pc()
    raw, ito_l = orc.lanczos(o.mobility_pc, z, factor=np.sqrt(2 * kT / dt), tol=1e-3)
    onoise = o.P_inv_mult(raw)
    rhs = np.concatenate([-onoise, -FT.flatten()])
    nrm = np.linalg.norm(rhs)
    xo, _, _ = orc.gmres_right(o.apply, o.apply_pc, rhs / nrm, tol=1e-8)
    ovel = (xo * nrm)[3 * s3.n_blobs:]
    olocs, oquats = orc.em_update(s3.locations, s3.quaternions, ovel, dt)
    tol_noise = 1e-8 if mode == "fp64" else 1e-6
    assert abs(out["lanczos_iterations"] - ito_l) <= (0 if mode == "fp64" else 1)
    assert abs(itl - ito_l) <= (0 if mode == "fp64" else 1)
    assert rel_err(noise, onoise) <= tol_noise
    assert rel_err(vel, ovel) <= 1e-6
    assert np.abs(step.x.cpu().numpy() - olocs).max() <= 1e-8
    assert np.abs(step.q.cpu().numpy() - oquats).max() <= 1e-8


def test_batched_64_suspensions_meet_oracle_residual(cuda_device):
    susps = S.shells_42_batch()
    counts = [s.n_bodies for s in susps]
    r = np.concatenate([s.r_vectors() for s in susps])
    locs = np.concatenate([s.locations for s in susps])
    sysb = RigidSystem([42] * sum(counts), susps[0].eta, susps[0].a)
    sysb.set_configuration(r, locs)
    sysb.set_suspensions(counts)
    sysb.build_pc(mode="mixed")
    FT = np.zeros((sum(counts), 6))
    FT[:, 2] = -1.0
    n3 = 3 * sysb.n_blobs
    rhs = np.concatenate([np.zeros(n3), -FT.flatten()])
    sol, its, rr, stt = sysb.solve_batched(rhs, tol=1e-8, mode="mixed")
    sol = sol.cpu().numpy()
    assert (np.asarray(stt) == 0).all()
    boff = np.concatenate([[0], np.cumsum(counts)])
    blob_off = 42 * boff
    worst = 0.0
    small = np.argsort(counts)[:2]
    for k, s in enumerate(susps):
        lam = sol[3 * blob_off[k]:3 * blob_off[k + 1]]
        U = sol[n3 + 6 * boff[k]:n3 + 6 * boff[k + 1]]
        offs = 42 * np.arange(counts[k] + 1)
        o = orc.Rigid(r[blob_off[k]:blob_off[k + 1]], s.locations, offs, s.eta, s.a)
        bk = np.concatenate([np.zeros(3 * blob_off[k + 1] - 3 * blob_off[k]), -FT[boff[k]:boff[k + 1]].flatten()])
        res = np.linalg.norm(bk - o.apply(np.concatenate([lam, U]))) / np.linalg.norm(bk)
        worst = max(worst, res)
        if k in small:
            xo, _, _ = orc.gmres_right(o.apply, o.apply_pc, bk / np.linalg.norm(bk), tol=1e-8)
            assert rel_err(U, (xo * np.linalg.norm(bk))[3 * (blob_off[k + 1] - blob_off[k]):]) <= 1e-6
    assert worst <= 1.05e-8, worst


def test_batched_lanczos_noise_matches_oracle_on_two_suspensions(cuda_device):
    susps = S.shells_42_batch()
    counts = [s.n_bodies for s in susps]
    r = np.concatenate([s.r_vectors() for s in susps])
    locs = np.concatenate([s.locations for s in susps])
    sysb = RigidSystem([42] * sum(counts), susps[0].eta, susps[0].a)
    sysb.set_configuration(r, locs)
    sysb.set_suspensions(counts)
    sysb.build_pc(stochastic=True)
    Z = np.random.default_rng(4).standard_normal((2, 3 * sysb.n_blobs))
    noise, itl = sysb.lanczos_batched(Z, factor=np.sqrt(2.0 / 1e-3), tol=1e-3, mode="fp64")
    noise = noise.cpu().numpy()
    itl = np.asarray(itl).reshape(2, len(counts))
    boff = np.concatenate([[0], np.cumsum(counts)])
    blob_off = 42 * boff
    for k in np.argsort(counts)[:2]:
        offs = 42 * np.arange(counts[k] + 1)
        rk = r[blob_off[k]:blob_off[k + 1]]
        o = orc.Rigid(rk, susps[k].locations, offs, susps[k].eta, susps[k].a)
        o.build_pc()
        for q in range(2):
            zk = Z[q, 3 * blob_off[k]:3 * blob_off[k + 1]]
            raw, it = orc.lanczos(o.mobility_pc, zk, factor=np.sqrt(2.0 / 1e-3), tol=1e-3)
            assert itl[q, k] == it
            assert rel_err(noise[q, 3 * blob_off[k]:3 * blob_off[k + 1]], o.P_inv_mult(raw)) <= 1e-8
