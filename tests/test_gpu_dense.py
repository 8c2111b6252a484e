"""GPU parity of the dense blob mobilities (rmw_dense_mobility) with the
reference's single_wall_fluid_mobility and rotne_prager_tensor
(tests/golden/products.npz, nowall.npz: far, wall-overlapping (damped), exact
contact and single-blob cases), bar 1e-13 relative; and of the dense-product
drop-ins with the reference's numba products."""
import numpy as np
import pytest

from conftest import golden, rel_err
from rigidmultiblobswall_gb300 import mobility as mb

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", ["damped", "touching", "single"])
def test_single_wall_fluid_mobility_matches_reference(cuda_device, case):
    g = golden("products.npz")
    a, eta = g[case + "_params"]
    M = mb.single_wall_fluid_mobility(g[case + "_r"], eta, a)
    assert M.shape == g[case + "_dense"].shape
    assert rel_err(M, g[case + "_dense"]) <= 1e-13
    assert rel_err(M, M.T) <= 1e-14
    u = mb.single_wall_fluid_mobility_product(g[case + "_r"], g[case + "_v"], eta, a)
    assert rel_err(u, g[case + "_uf"]) <= 1e-12


@pytest.mark.parametrize("case", ["far", "touching", "single"])
def test_rotne_prager_tensor_matches_reference(cuda_device, case):
    g = golden("nowall.npz")
    a, eta = g[case + "_params"]
    M = mb.rotne_prager_tensor(g[case + "_r"], eta, a)
    assert rel_err(M, g[case + "_dense"]) <= 1e-13
    u = mb.no_wall_fluid_mobility_product(g[case + "_r"], g[case + "_v"], eta, a)
    assert rel_err(u, g[case + "_uf"]) <= 1e-12


def test_dense_mobility_is_spd_and_matches_the_product(cuda_device):
    import torch
    rng = np.random.default_rng(9)
    n, a = 700, 0.5
    r = np.column_stack([rng.uniform(0, 20, (n, 2)), rng.uniform(0.2, 3, n)])
    M = mb.single_wall_fluid_mobility(torch.as_tensor(r, device="cuda"), 1.0, a)
    assert isinstance(M, torch.Tensor)
    assert float(torch.linalg.eigvalsh(M).min()) > 0
    v = rng.standard_normal(3 * n)
    u = mb.single_wall_mobility_trans_times_force_pycuda(r, v, 1.0, a)
    assert rel_err((M @ torch.as_tensor(v, device="cuda")).cpu().numpy(), u) <= 1e-12
