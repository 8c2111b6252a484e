"""GPU parity of the source-target products with per-blob radii (wall, free
space, free surface; rmw_source_target_product) and the single-radius
free-surface product (rmw_free_surface_product) against the reference's own
outputs (tests/golden/source_target.npz) and the oracle on larger inputs.

Bars (max-norm error relative to the largest velocity): FP64 1e-12, df64
1e-11, mixed 1e-5."""
import numpy as np
import pytest

from conftest import golden
from oracle import source_target as st
from rigidmultiblobswall_gb300 import mobility as mb

pytestmark = pytest.mark.gpu
CASES = ["far", "close", "periodic"]
FNS = {"wall": mb.single_wall_mobility_trans_times_force_source_target_numba,
       "no_wall": mb.no_wall_mobility_trans_times_force_source_target_numba,
       "free_surface": mb.free_surface_mobility_trans_times_force_source_target_numba}
KEYS = {"wall": "wall", "no_wall": "nowall", "free_surface": "free_surface"}
BARS = {"fp64": 1e-12, "df64": 1e-11, "mixed": 1e-5}


def rel(x, y):
    return np.abs(np.asarray(x) - np.asarray(y)).max() / np.abs(np.asarray(y)).max()


@pytest.mark.parametrize("mode", list(BARS))
@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("geom", list(FNS))
def test_source_target_matches_reference(cuda_device, geom, case, mode):
    g = golden("source_target.npz")
    u = FNS[geom](g[case + "_source"], g[case + "_target"], g[case + "_f"], g[case + "_rs"], g[case + "_rt"],
                  g[case + "_eta"][0], periodic_length=g[case + "_L"], mode=mode)
    assert u.shape == (3 * g[case + "_target"].shape[0],)
    assert rel(u, g[case + "_" + KEYS[geom]]) <= BARS[mode]


@pytest.mark.parametrize("case", ["far", "close"])
def test_python_forms_return_rows(cuda_device, case):
    g = golden("source_target.npz")
    args = (g[case + "_source"], g[case + "_target"], g[case + "_f"], g[case + "_rs"], g[case + "_rt"],
            g[case + "_eta"][0])
    u = mb.mobility_vector_product_source_target_one_wall(*args)
    assert u.shape == (g[case + "_target"].shape[0], 3)
    assert rel(u.reshape(-1), g[case + "_one_wall_py"]) <= 1e-12
    v = mb.mobility_vector_product_source_target_unbounded(*args)
    assert rel(v.reshape(-1), g[case + "_unbounded_py"]) <= 1e-12


@pytest.mark.parametrize("mode", list(BARS))
@pytest.mark.parametrize("case", ["fs", "fs_periodic"])
def test_free_surface_matches_reference(cuda_device, case, mode):
    g = golden("source_target.npz")
    a, eta = g[case + "_params"]
    u = mb.free_surface_mobility_trans_times_force_pycuda(g[case + "_r"], g[case + "_f"], eta, a,
                                                          periodic_length=g[case + "_L"], mode=mode)
    assert rel(u, g[case + "_u"]) <= BARS[mode]


@pytest.mark.parametrize("ns,nt", [(1500, 1000), (3000, 7), (1, 300), (129, 257)])
@pytest.mark.parametrize("geom", list(FNS))
def test_source_target_larger_against_oracle(cuda_device, geom, ns, nt):
    """Tile tails, a single source, few targets (sources split over many CTAs)."""
    rng = np.random.default_rng(ns + 7 * nt)
    src = np.column_stack([rng.uniform(0, 30, (ns, 2)), rng.uniform(0.05, 5, ns)])
    trg = np.column_stack([rng.uniform(0, 30, (nt, 2)), rng.uniform(0.05, 5, nt)])
    rs, rt = rng.uniform(0.1, 0.8, ns), rng.uniform(0.1, 0.8, nt)
    f = rng.standard_normal(3 * ns)
    ref = st.source_target(geom, src, trg, f, rs, rt, 1.3)
    for mode in BARS:
        u = FNS[geom](src, trg, f, rs, rt, 1.3, mode=mode)
        assert rel(u, ref) <= BARS[mode], mode


def test_device_tensors_and_edge_cases(cuda_device):
    import torch
    from rigidmultiblobswall_gb300._native import RMWError
    rng = np.random.default_rng(5)
    src = torch.as_tensor(rng.uniform(0.5, 3, (50, 3)), device="cuda")
    trg = torch.as_tensor(rng.uniform(0.5, 3, (40, 3)), device="cuda")
    f = torch.as_tensor(rng.standard_normal(150), device="cuda")
    u = mb.single_wall_mobility_trans_times_force_source_target_pycuda(src, trg, f, 0.3, 0.4, 1.0)
    assert isinstance(u, torch.Tensor) and u.is_cuda
    ref = st.source_target("wall", src.cpu().numpy(), trg.cpu().numpy(), f.cpu().numpy(), np.full(50, 0.3),
                           np.full(40, 0.4), 1.0)
    assert rel(u.cpu().numpy(), ref) <= 1e-12
    # no sources: zero velocities; no targets: empty result
    z = mb.no_wall_mobility_trans_times_force_source_target_numba(np.zeros((0, 3)), trg.cpu().numpy(), np.zeros(0),
                                                                  np.zeros(0), np.full(40, 0.4), 1.0)
    assert z.shape == (120,) and not z.any()
    e = mb.no_wall_mobility_trans_times_force_source_target_numba(src.cpu().numpy(), np.zeros((0, 3)),
                                                                  f.cpu().numpy(), np.full(50, 0.3), np.zeros(0), 1.0)
    assert e.shape == (0,)
    with pytest.raises(ValueError):
        mb.source_target_product("wall", src, trg, f[:10], 0.3, 0.4, 1.0)
    with pytest.raises(RMWError):
        mb.free_surface_mobility_trans_times_force_numba(trg, torch.zeros(120, dtype=torch.float64, device="cuda"),
                                                         1.0, -0.5)
