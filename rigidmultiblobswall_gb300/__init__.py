"""GB300-native (sm_103a) wall-corrected RPY blob mobility hot path of
RigidMultiblobsWall: the four wall pair products, the block-diagonal
preconditioned GMRES rigid-body mobility solve, and the Lanczos M^(1/2) z.

Compute runs in librmw_gb300.so (hand-written CUDA, C ABI in include/rmw_gb300.h).
"""
from . import _native  # noqa: F401

__all__ = ["mobility"]
