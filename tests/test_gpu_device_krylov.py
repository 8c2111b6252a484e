"""GPU: device-resident GMRES restart cycles against the host-driven Arnoldi loop and the oracle.

The rigid solves run each restart cycle on the device: the operator A P^-1 and a fused cooperative
Arnoldi step kernel (CGS2, Givens rotations, stopping test), repeated by a CUDA graph while node.  The
host-driven loop (rmw_use_device_krylov(0)) does the same algorithm with one host round trip per step.
Both must give the same iteration counts and solutions within round-off, in every precision mode, with
CUDA graphs on and off, and the oracle's FP64 residual of the solution must meet the tolerance
(general_application_utils.py:514-635: right preconditioning, relative tolerance, zero start)."""
import numpy as np
import pytest

from conftest import rel_err
from oracle import rigid as orc
from rigidmultiblobswall_gb300 import _native
from rigidmultiblobswall_gb300 import integrator
from rigidmultiblobswall_gb300 import suspensions as S
from rigidmultiblobswall_gb300.rigid import RigidSystem

pytestmark = pytest.mark.gpu


def _suspension(nb, seed):
    susp = S.shells_42_256(n_bodies=nb, seed=seed)
    r = susp.r_vectors()
    s = RigidSystem([42] * nb, susp.eta, susp.a)
    s.set_configuration(r, susp.locations)
    o = orc.Rigid(r, susp.locations, s.offsets, susp.eta, susp.a)
    return s, o


@pytest.fixture
def switches(cuda_device):
    yield
    _native.use_device_krylov(True)
    _native.use_graphs(True)


@pytest.mark.parametrize("mode", ["fp64", "df64", "mixed"])
@pytest.mark.parametrize("graphs", [True, False])
def test_device_cycles_match_host_loop_and_oracle(switches, mode, graphs):
    s, o = _suspension(24, 31)
    FT = np.random.default_rng(2).standard_normal((24, 6))
    rhs = np.concatenate([np.zeros(3 * s.n_blobs), -FT.flatten()])
    _native.use_graphs(graphs)
    res = {}
    for dev in (True, False):
        _native.use_device_krylov(dev)
        sol, info, its, rr = integrator.solve_mobility_problem(s, FT, tol=1e-8, mode=mode)
        assert info == 0 and rr <= 1e-8
        res[dev] = (sol.cpu().numpy(), its)
    (xd, itd), (xh, ith) = res[True], res[False]
    assert abs(itd - ith) <= (0 if mode != "mixed" else 1)
    assert rel_err(xd, xh) <= 1e-9
    assert np.linalg.norm(rhs - o.apply(xd)) <= 1.05e-8 * np.linalg.norm(rhs)


def test_device_cycles_restart_and_maxiter(switches):
    """A short restart forces several device cycles; a tiny maxiter stops mid-cycle with info > 0."""
    s, o = _suspension(16, 5)
    FT = np.zeros((16, 6))
    FT[:, 2] = -1.0
    rhs = np.concatenate([np.zeros(3 * s.n_blobs), -FT.flatten()])
    s.build_pc()
    b = rhs / np.linalg.norm(rhs)
    out = {}
    for dev in (True, False):
        _native.use_device_krylov(dev)
        x, info, its, rr = s.solve(b, tol=1e-10, restart=4, mode="fp64")
        assert info == 0 and its > 4
        out[dev] = (x.cpu().numpy(), its)
        x1, info1, its1, rr1 = s.solve(b, tol=1e-14, maxiter=3, mode="fp64")
        assert info1 == 3 and its1 == 3 and rr1 > 1e-14
    assert out[True][1] == out[False][1]
    assert rel_err(out[True][0], out[False][0]) <= 1e-9
    assert np.linalg.norm(b - o.apply(out[True][0])) <= 1.05e-10


def test_device_cycles_are_deterministic(switches):
    s, _ = _suspension(20, 9)
    FT = np.random.default_rng(8).standard_normal((20, 6))
    a = integrator.solve_mobility_problem(s, FT, tol=1e-8, mode="mixed")[0].cpu().numpy()
    b = integrator.solve_mobility_problem(s, FT, tol=1e-8, mode="mixed")[0].cpu().numpy()
    assert np.array_equal(a, b)


@pytest.mark.parametrize("mode", ["fp64", "mixed"])
@pytest.mark.parametrize("tol", [1e-3, 1e-10])
def test_device_lanczos_matches_host_loop(switches, mode, tol):
    """Device-resident Lanczos (fused step kernel with the reorthogonalisation pass and the tridiagonal
    eigen-solve on the device, graph while loop) against the host-driven recurrence: same iteration count,
    same noise to round-off.  tol 1e-10 runs past the basis' first 32 vectors (the host doubles it)."""
    s, _ = _suspension(24, 13)
    s.build_pc(stochastic=True, mode=mode)
    z = np.random.default_rng(6).standard_normal(3 * s.n_blobs)
    out = {}
    for dev in (True, False):
        _native.use_device_krylov(dev)
        noise, it = s.lanczos(z, factor=np.sqrt(2.0 / 1e-3), tol=tol, mode=mode, max_iter=200)
        out[dev] = (noise.cpu().numpy(), it)
    assert out[True][1] == out[False][1]
    assert rel_err(out[True][0], out[False][0]) <= 1e-9


def test_device_lanczos_grows_its_basis(switches):
    """A tolerance no iteration meets runs max_iter = 50 iterations: past the first 32 basis vectors, where
    the device loop returns to the host to double the basis and continues; same result as the host loop."""
    s, _ = _suspension(12, 17)
    s.build_pc(stochastic=True)
    z = np.random.default_rng(9).standard_normal(3 * s.n_blobs)
    out = {}
    for dev in (True, False):
        _native.use_device_krylov(dev)
        noise, it = s.lanczos(z, factor=1.0, tol=1e-16, max_iter=50)
        out[dev] = (noise.cpu().numpy(), it)
    assert out[True][1] == out[False][1] == 50
    assert rel_err(out[True][0], out[False][0]) <= 1e-8


def test_device_lanczos_max_iter_and_zero_factor(switches):
    s, _ = _suspension(8, 2)
    s.build_pc(stochastic=True)
    z = np.random.default_rng(1).standard_normal(3 * s.n_blobs)
    res = {}
    for dev in (True, False):
        _native.use_device_krylov(dev)
        noise, it = s.lanczos(z, factor=1.0, tol=1e-16, max_iter=5)
        res[dev] = (noise.cpu().numpy(), it)
        zero, it0 = s.lanczos(z, factor=0.0)
        assert it0 == 0 and float(zero.abs().max()) == 0.0
    assert res[True][1] == res[False][1] == 5
    assert rel_err(res[True][0], res[False][0]) <= 1e-10


def test_device_batched_solve_and_lanczos_match_host_loop(switches):
    counts = [9, 20, 14, 5]
    shells = [S.shells(c, S.icosahedron(1.0), 60 + k, 15.0, 1.2, 4.0, a=0.4) for k, c in enumerate(counts)]
    r = np.concatenate([sh.r_vectors() for sh in shells])
    x = np.concatenate([sh.locations for sh in shells])
    s = RigidSystem([12] * sum(counts), 1.0, 0.4)
    s.set_configuration(r, x)
    s.set_suspensions(counts)
    s.build_pc(stochastic=True)
    rng = np.random.default_rng(11)
    rhs = rng.standard_normal(s.size)
    Z = rng.standard_normal((5, 3 * s.n_blobs))
    out = {}
    for dev in (True, False):
        _native.use_device_krylov(dev)
        for mode in ("fp64", "mixed"):
            sol, it, rr, stt = s.solve_batched(rhs, tol=1e-8, mode=mode)
            noise, itl = s.lanczos_batched(Z, factor=1.0, tol=1e-4, mode=mode)
            assert (np.asarray(stt) == 0).all() and (np.asarray(rr) <= 1e-8).all()
            out[(dev, mode)] = (sol.cpu().numpy(), np.asarray(it), noise.cpu().numpy(), np.asarray(itl))
    for mode in ("fp64", "mixed"):
        d, h = out[(True, mode)], out[(False, mode)]
        assert (d[3] == h[3]).all()
        assert rel_err(d[2], h[2]) <= 1e-9
        assert np.abs(d[1] - h[1]).max() <= (0 if mode == "fp64" else 1)
        assert rel_err(d[0], h[0]) <= 1e-8
