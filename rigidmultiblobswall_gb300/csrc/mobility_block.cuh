// The 3x3 translational mobility block M_ij (without 1/(8 pi eta a)) of two
// blobs, as the dense matrices of the reference build it:
// * above the wall (mobility/mobility.py:1018-1116, single_wall_fluid_mobility):
//   heights shifted to max(z, a), the RPY + Swan-Brady wall block between
//   distinct blobs and the wall-corrected self block on the diagonal; the
//   damping factors b_i b_j (z / a below a) are returned in *scale;
// * free space (mobility/mobility.py:967-1015, rotne_prager_tensor): RPY,
//   4/3 I on the diagonal.
#pragma once

#include "pair_math.cuh"

namespace rmw {

// T = float evaluates the pair block in FP32 (from FP64 position differences):
// the preconditioner blocks of the mixed-precision solves.
template <typename T = double>
__device__ __forceinline__ void uf_block(const double *__restrict__ r, int i, int j, double a, bool wall,
                                         double blk[3][3], double *scale)
{
    const double inva = 1.0 / a;
    for (int u = 0; u < 3; ++u)
        for (int w = 0; w < 3; ++w) blk[u][w] = 0.0;
    *scale = 1.0;
    if (wall) {
        const double zi = r[3 * i + 2], zj = r[3 * j + 2];
        *scale = ((zi < a) ? zi / a : 1.0) * ((zj < a) ? zj / a : 1.0);
        const double zie = (zi <= a) ? a : zi, zje = (zj <= a) ? a : zj;
        if (i == j) {
            const double iz = a / zie, iz3 = iz * iz * iz, iz5 = iz3 * iz * iz;
            const double mxx = 4.0 / 3.0 - (9.0 * iz - 2.0 * iz3 + iz5) / 12.0;
            blk[0][0] = mxx;
            blk[1][1] = mxx;
            blk[2][2] = 4.0 / 3.0 - (9.0 * iz - 4.0 * iz3 + iz5) / 6.0;
            return;
        }
        const T dx = (T)((r[3 * i] - r[3 * j]) * inva), dy = (T)((r[3 * i + 1] - r[3 * j + 1]) * inva);
        const T dz = (T)((zie - zje) * inva);
        const T hi = (T)(zie * inva), hj = (T)(zje * inva), Rz = (T)((zie + zje) * inva);
        for (int w = 0; w < 3; ++w) {
            T c[3] = {T(0), T(0), T(0)};
            pair_contrib<RMW_UF, T>(dx, dy, dz, Rz, hi, hj, w == 0 ? T(1) : T(0), w == 1 ? T(1) : T(0),
                                    w == 2 ? T(1) : T(0), c[0], c[1], c[2]);
            blk[0][w] = c[0];
            blk[1][w] = c[1];
            blk[2][w] = c[2];
        }
        return;
    }
    if (i == j) {
        blk[0][0] = blk[1][1] = blk[2][2] = 4.0 / 3.0;
        return;
    }
    const T dx = (T)((r[3 * i] - r[3 * j]) * inva), dy = (T)((r[3 * i + 1] - r[3 * j + 1]) * inva),
            dz = (T)((r[3 * i + 2] - r[3 * j + 2]) * inva);
    for (int w = 0; w < 3; ++w) {
        T c[3] = {T(0), T(0), T(0)};
        pair_rpy<RMW_UF, T>(dx, dy, dz, w == 0 ? T(1) : T(0), w == 1 ? T(1) : T(0), w == 2 ? T(1) : T(0), c[0], c[1],
                            c[2]);
        blk[0][w] = c[0];
        blk[1][w] = c[1];
        blk[2][w] = c[2];
    }
}

}  // namespace rmw
