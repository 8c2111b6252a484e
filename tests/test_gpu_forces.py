"""GPU: blob forces against the reference's own force functions (golden
vectors) and the oracle: blob-blob repulsion with and without periodic
images, both sides of the exact FP32 screen (compact CTAs, and CTAs whose
blobs span 3e7 so the screen must switch itself off), external gravity and
wall forces, accumulation, argument errors, and the per-body reduction."""
import os

import numpy as np
import pytest

from conftest import rel_err
from oracle import forces as of
from rigidmultiblobswall_gb300 import forces as F
from rigidmultiblobswall_gb300 import suspensions as S
from rigidmultiblobswall_gb300.rigid import RigidSystem

pytestmark = pytest.mark.gpu

G = os.path.join(os.path.dirname(__file__), "golden", "forces.npz")


@pytest.mark.parametrize("case", ["dense", "periodic", "far"])
def test_forces_match_reference_golden(cuda_device, case):
    g = np.load(G)
    eps, b, a = g[case + "_params"]
    bb = F.calc_blob_blob_forces_pycuda(g[case + "_r"], periodic_length=g[case + "_L"], repulsion_strength=eps,
                                        debye_length=b, blob_radius=a)
    assert bb.shape == (len(g[case + "_r"]), 3)
    assert rel_err(bb, g[case + "_bb"]) <= 1e-12
    m, ra, gg, e, bw = g[case + "_ext_params"]
    ext = F.blob_external_forces(g[case + "_r"], blob_mass=m, blob_radius=ra, g=gg, repulsion_strength_wall=e,
                                 debye_length_wall=bw)
    assert rel_err(ext, g[case + "_ext"]) <= 1e-14


@pytest.mark.parametrize("case", ["dense", "periodic", "far"])
def test_cutoff_variant_matches_reference_tree_golden(cuda_device, case):
    """calc_blob_blob_forces_tree_numba: pairs within 2a + 30 b only."""
    g = np.load(G)
    eps, b, a = g[case + "_params"]
    got = F.calc_blob_blob_forces_tree_numba(g[case + "_r"], periodic_length=g[case + "_L"], repulsion_strength=eps,
                                             debye_length=b, blob_radius=a)
    assert rel_err(got, g[case + "_tree"]) <= 1e-12


@pytest.mark.parametrize("spread", [False, True])
@pytest.mark.parametrize("periodic", [False, True])
def test_blob_blob_matches_oracle_both_screen_paths(cuda_device, spread, periodic):
    """spread: every other blob is moved 3e7 away, so each CTA's blobs span
    3e7, the FP32 screen cannot bound its error and must fall back to FP64
    distances - the result must still match the oracle."""
    rng = np.random.default_rng(5)
    n = 1300
    r = rng.uniform(0.0, 14.0, (n, 3))
    if spread:
        r[1::2, :2] += 3.0e7
    L = np.array([14.0, 14.0, 0.0]) if periodic and not spread else None
    got = F.calc_blob_blob_forces_pycuda(r, periodic_length=L, repulsion_strength=0.8, debye_length=0.004,
                                         blob_radius=0.2)
    ref = of.blob_blob_forces(r, 0.8, 0.004, 0.2, periodic_length=L)
    assert rel_err(got, ref) <= 1e-12


def test_accumulate_and_device_path(cuda_device):
    import torch
    from rigidmultiblobswall_gb300 import _native
    rng = np.random.default_rng(6)
    r = torch.tensor(rng.uniform(0.0, 5.0, (400, 3)), device="cuda")
    f = torch.ones_like(r)
    st = torch.cuda.current_stream().cuda_stream
    _native.call("rmw_blob_external_forces", r.data_ptr(), f.data_ptr(), 400, 1.0, 0.3, 2.0, 0.5, 0.2, 1, st)
    _native.call("rmw_blob_blob_forces", r.data_ptr(), f.data_ptr(), 400, 1.0, 0.1, 0.3, 0.0, None, 1, st)
    rn = r.cpu().numpy()
    ref = 1.0 + of.external_forces(rn, 1.0, 0.3, 2.0, 0.5, 0.2) + of.blob_blob_forces(rn, 1.0, 0.1, 0.3)
    assert rel_err(f.cpu().numpy(), ref) <= 1e-12
    ft = F.calc_blob_blob_forces_pycuda(r, repulsion_strength=1.0, debye_length=0.1, blob_radius=0.3)
    assert ft.is_cuda
    with pytest.raises(_native.RMWError):
        _native.call("rmw_blob_blob_forces", r.data_ptr(), f.data_ptr(), 400, 1.0, 0.0, 0.3, 0.0, None, 0, st)


def test_body_force_torque_reduction(cuda_device):
    s = S.shells(12, S.icosahedron(1.0), 8, 10.0, 1.2, 3.0, a=0.4)
    r = s.r_vectors()
    sys_ = RigidSystem([12] * s.n_bodies, 1.0, 0.4)
    sys_.set_configuration(r, s.locations)
    kw = dict(blob_mass=1.0, g=1.5, repulsion_strength_wall=0.3, debye_length_wall=0.2, repulsion_strength=0.5,
              debye_length=0.1, periodic_length=np.zeros(3))
    ft = F.force_torque_calculator_sort_by_bodies(sys_, r, **kw)
    fb = of.external_forces(r, 1.0, 0.4, 1.5, 0.3, 0.2) + of.blob_blob_forces(r, 0.5, 0.1, 0.4)
    ref = of.body_force_torque(r, s.locations, np.arange(s.n_bodies + 1) * 12, fb)
    assert ft.shape == (2 * s.n_bodies, 3)
    assert rel_err(ft, ref) <= 1e-12
