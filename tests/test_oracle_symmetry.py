"""CPU: the pair identities the symmetric kernels rely on, checked on the
oracle's own blocks (the restatement of mobility/mobility_numba.py):

* single wall: M_UF,ji = M_UF,ij^T and M_WT,ji = M_WT,ij^T (each unordered
  pair's coefficients serve both blobs, M_UF with f3 and f4 exchanged), and
  the grand mobility's symmetry M_UT,ji = M_WF,ij^T that makes [U; W] = M [F; T]
  symmetric as a 6N x 6N matrix;
* free space: M_ji = M_ij(-d), i.e. UF and WT blocks equal for both orders,
  UT and WF blocks opposite.

Blocks of two-blob systems over far, near-wall (z < a, damped), touching
(r = 2a) and overlapping pairs; tolerance 1e-13 relative to the block norm."""
import numpy as np
import pytest

from oracle import wall as owall


def _pairs(seed, a):
    rng = np.random.default_rng(seed)
    out = []
    for k in range(40):
        zi, zj = rng.uniform(0.3 * a, 6 * a, 2) if k % 4 == 1 else rng.uniform(1.2 * a, 8 * a, 2)
        if k % 4 == 2:  # touching: |r_i - r_j| = 2a
            d = rng.standard_normal(3)
            d *= 2 * a / np.linalg.norm(d)
        elif k % 4 == 3:  # overlapping
            d = rng.standard_normal(3)
            d *= rng.uniform(0.3, 1.9) * a / np.linalg.norm(d)
        else:
            d = rng.uniform(-10 * a, 10 * a, 3)
        ri = np.array([0.0, 0.0, zi])
        rj = ri - d
        if k % 4 in (0, 1):
            rj[2] = zj  # far or near-wall pairs: both heights drawn above the wall plane
        else:
            rj[2] = max(rj[2], 0.5 * a)  # keep the blob above the wall plane
        out.append(np.array([ri, rj]))
    return out


def _block(fn, kind, r, tgt, src, a):
    """3x3 block mapping blob src's vector to blob tgt's output."""
    B = np.zeros((3, 3))
    for c in range(3):
        v = np.zeros(6)
        v[3 * src + c] = 1.0
        B[:, c] = fn(kind, r, v, 1.0, a)[3 * tgt:3 * tgt + 3]
    return B


def _close(A, B):
    return np.linalg.norm(A - B) <= 1e-13 * max(np.linalg.norm(A), np.linalg.norm(B), 1e-300)


@pytest.mark.parametrize("kind", ["uf", "wt"])
def test_wall_blocks_transpose_under_exchange(kind):
    a = 0.35
    for r in _pairs(3, a):
        Mij = _block(owall.wall_product, kind, r, 0, 1, a)
        Mji = _block(owall.wall_product, kind, r, 1, 0, a)
        assert _close(Mji, Mij.T), (kind, r)


def test_wall_grand_mobility_symmetry():
    a = 0.35
    for r in _pairs(4, a):
        UTji = _block(owall.wall_product, "ut", r, 1, 0, a)
        WFij = _block(owall.wall_product, "wf", r, 0, 1, a)
        assert _close(UTji, WFij.T), r


@pytest.mark.parametrize("kind,sign", [("uf", 1.0), ("wt", 1.0), ("ut", -1.0), ("wf", -1.0)])
def test_free_space_blocks_under_exchange(kind, sign):
    a = 0.35
    for r in _pairs(5, a):
        Mij = _block(owall.no_wall_product, kind, r, 0, 1, a)
        Mji = _block(owall.no_wall_product, kind, r, 1, 0, a)
        assert _close(Mji, sign * Mij), (kind, r)
