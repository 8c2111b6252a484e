// Near-field augmented block-diagonal preconditioner, and the learned
// coupling network that feeds it.
//
// The block-diagonal preconditioner P0 is the exact inverse of the saddle-point
// operator with every inter-body blob block of M dropped:
//   A0 = [[Mbd, -K], [-K^T, 0]],   A P0 = I + [[M - Mbd, 0], [0, 0]] A0^-1 .
// The error lives in the blob rows only: the velocities that other bodies'
// blob forces induce on a body.  The augmented preconditioner takes the first
// Neumann term of (A0 + E)^-1 with E the near part of M - Mbd:
//   y = P0 x;   v_i = sum_{j near i} M_ij lambda_j(y);   y <- y - P0 [v; 0] .
// It stays an exact-inverse-like operator (the force rows of the correction
// are consistent), which is why it helps where changing only the body
// velocities - even with the exact many-body mobility - costs iterations.
//
// Two kinds of near pairs:
//  * exact pairs (centre distance below the exact cutoff): M_ij lambda_j
//    evaluated blob by blob in double-float arithmetic (same pair formulas
//    and periodic images as the all-pairs product, ~1e-14 relative);
//  * learned pairs (from the exact cutoff to the network's cutoff): M_ij is
//    replaced by its projection on the 11 low-order modes of each body -
//    3 translations, 3 rotations, 5 strains E_k d (d = blob - centre):
//      v_i ~ X_i G_ij X_j^T lambda_j,  X_b the mode velocities of body b,
//    with G_ij = (X_i^T M_i^-1 X_i)^-1 X_i^T M_i^-1  M_ij  M_j^-1 X_j (X_j^T M_j^-1 X_j)^-1,
//    the response of body i's modes to body j's force, torque and stresslet
//    above the wall.  A small network predicts G_ij from the horizontal
//    distance and both heights (units of the body radius) in the frame
//    rotated about the wall normal so that the separation lies along +x;
//    the kernels rotate it back (translations and rotations as vectors,
//    strains by the 5x5 representation of the rotation).
// GMRES with right preconditioning accepts any nonsingular P^-1, so a poor
// prediction only costs iterations; the caller compares against the plain
// solve and falls back.
//
// Training data come from two- to eight-body clusters through the plain
// method's own machinery on the GPU: a handle whose bodies are the clusters'
// shells builds each body's M^-1 (rmw_rigid_build_pc) and pair_list_kernel
// forms G_ij of every ordered pair of a cluster in the learned band.
//
// The network (mpnn.cu) is a message-passing network over the bodies: three
// rounds of messages between bodies closer than its message cutoff, then a
// readout per learned pair from both bodies' embeddings and the pair's
// geometry.  Training clusters of two to eight bodies give it neighbourhoods
// of the sizes it meets in a suspension.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "mpnn.cuh"
#include "pair_math.cuh"
#include "pair_math_df.cuh"
#include "rigid.cuh"

namespace rmw {

constexpr int kModes = 11;
constexpr double kS2 = 0.70710678118654752440;  // 1/sqrt(2)
constexpr double kS6 = 0.40824829046386301637;  // 1/sqrt(6)

// velocity of mode c at displacement d from the body centre: 0-2 translations,
// 3-5 rotations (e_c x d), 6-10 strains E_k d with the orthonormal symmetric
// traceless basis (xx-yy)/sqrt2, (2zz-xx-yy)/sqrt6, (xy+yx)/sqrt2,
// (xz+zx)/sqrt2, (yz+zy)/sqrt2
__host__ __device__ __forceinline__ void mode_velocity(int c, double dx, double dy, double dz, double &vx,
                                                       double &vy, double &vz)
{
    switch (c) {
    case 0: vx = 1.0; vy = 0.0; vz = 0.0; break;
    case 1: vx = 0.0; vy = 1.0; vz = 0.0; break;
    case 2: vx = 0.0; vy = 0.0; vz = 1.0; break;
    case 3: vx = 0.0; vy = -dz; vz = dy; break;
    case 4: vx = dz; vy = 0.0; vz = -dx; break;
    case 5: vx = -dy; vy = dx; vz = 0.0; break;
    case 6: vx = kS2 * dx; vy = -kS2 * dy; vz = 0.0; break;
    case 7: vx = -kS6 * dx; vy = -kS6 * dy; vz = 2.0 * kS6 * dz; break;
    case 8: vx = kS2 * dy; vy = kS2 * dx; vz = 0.0; break;
    case 9: vx = kS2 * dz; vy = 0.0; vz = kS2 * dx; break;
    default: vx = 0.0; vy = kS2 * dz; vz = kS2 * dy; break;
    }
}

template <typename T>
__host__ __device__ __forceinline__ void strain_basis(int k, T E[3][3])
{
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) E[a][b] = T(0);
    switch (k) {
    case 0: E[0][0] = T(kS2); E[1][1] = -T(kS2); break;
    case 1: E[0][0] = -T(kS6); E[1][1] = -T(kS6); E[2][2] = T(2.0 * kS6); break;
    case 2: E[0][1] = E[1][0] = T(kS2); break;
    case 3: E[0][2] = E[2][0] = T(kS2); break;
    default: E[1][2] = E[2][1] = T(kS2); break;
    }
}

// Q = diag(Rz, Rz, R5) for the rotation about z with cos c, sin s
template <typename T>
__host__ __device__ inline void mode_rotation(T c, T s, T Q[kModes][kModes])
{
    for (int a = 0; a < kModes; ++a)
        for (int b = 0; b < kModes; ++b) Q[a][b] = T(0);
    for (int blk = 0; blk < 2; ++blk) {
        const int o = 3 * blk;
        Q[o][o] = c; Q[o][o + 1] = -s;
        Q[o + 1][o] = s; Q[o + 1][o + 1] = c;
        Q[o + 2][o + 2] = T(1);
    }
    const T Rz[3][3] = {{c, -s, T(0)}, {s, c, T(0)}, {T(0), T(0), T(1)}};
    for (int l = 0; l < 5; ++l) {
        T El[3][3], R[3][3];
        strain_basis(l, El);
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) {
                T acc = T(0);
                for (int p = 0; p < 3; ++p)
                    for (int q = 0; q < 3; ++q) acc += Rz[a][p] * El[p][q] * Rz[b][q];
                R[a][b] = acc;
            }
        for (int k = 0; k < 5; ++k) {
            T Ek[3][3];
            strain_basis(k, Ek);
            T acc = T(0);
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) acc += Ek[a][b] * R[a][b];
            Q[6 + k][6 + l] = acc;
        }
    }
}

struct Images {
    double Lx, Ly, Lz;
};

// Unscaled single-wall RPY velocity at blob (xi, yi, zie) from blob (xj, yj, zje)
// carrying v (heights already clamped at a, v already damped), summed over the
// periodic images the all-pairs product uses; the caller multiplies by
// b_i / (8 pi eta a).
__device__ __forceinline__ void wall_uf_pair(double xi, double yi, double zie, double xj, double yj, double zje,
                                             double inva, const Images &P, double vx, double vy, double vz,
                                             double &ux, double &uy, double &uz)
{
    const double hi = zie * inva, hj = zje * inva, Rz = (zie + zje) * inva;
    double rx = xi - xj, ry = yi - yj, rz = zie - zje;
    if (!(P.Lx > 0 || P.Ly > 0 || P.Lz > 0)) {
        double cx = 0.0, cy = 0.0, cz = 0.0;
        pair_contrib<RMW_UF, double>(rx * inva, ry * inva, rz * inva, Rz, hi, hj, vx, vy, vz, cx, cy, cz);
        ux += cx; uy += cy; uz += cz;
        return;
    }
    if (P.Lx > 0) rx = project(rx, P.Lx);
    if (P.Ly > 0) ry = project(ry, P.Ly);
    if (P.Lz > 0) rz = project(rz, P.Lz);
    const int px = P.Lx > 0, py = P.Ly > 0, pz = P.Lz > 0;
    for (int bx = -px; bx <= px; ++bx)
        for (int by = -py; by <= py; ++by)
            for (int bz = -pz; bz <= pz; ++bz) {
                double cx = 0.0, cy = 0.0, cz = 0.0;
                pair_contrib<RMW_UF, double>((rx + bx * P.Lx) * inva, (ry + by * P.Ly) * inva,
                                             (rz + bz * P.Lz) * inva, Rz, hi, hj, vx, vy, vz, cx, cy, cz);
                ux += cx; uy += cy; uz += cz;
            }
}

// The same velocity in double-float arithmetic on the FP32 pipe (relative
// error ~1e-14, like the df64 product mode): differences formed in FP64, the
// pair math in df64, the result accumulated in FP64.
__device__ __forceinline__ void wall_uf_pair_df(double xi, double yi, double zie, double xj, double yj, double zje,
                                                double inva, const Images &P, double vx, double vy, double vz,
                                                double &ux, double &uy, double &uz)
{
    const df hi = df_of_double(zie * inva), hj = df_of_double(zje * inva), Rz = df_of_double((zie + zje) * inva);
    const df fx = df_of_double(vx), fy = df_of_double(vy), fz = df_of_double(vz);
    double rx = xi - xj, ry = yi - yj, rz = zie - zje;
    if (!(P.Lx > 0 || P.Ly > 0 || P.Lz > 0)) {
        df cx, cy, cz;
        pair_contrib_df<RMW_UF>(df_of_double(rx * inva), df_of_double(ry * inva), df_of_double(rz * inva), Rz, hi, hj,
                                fx, fy, fz, cx, cy, cz);
        ux += to_double(cx); uy += to_double(cy); uz += to_double(cz);
        return;
    }
    if (P.Lx > 0) rx = project(rx, P.Lx);
    if (P.Ly > 0) ry = project(ry, P.Ly);
    if (P.Lz > 0) rz = project(rz, P.Lz);
    const int px = P.Lx > 0, py = P.Ly > 0, pz = P.Lz > 0;
    for (int bx = -px; bx <= px; ++bx)
        for (int by = -py; by <= py; ++by)
            for (int bz = -pz; bz <= pz; ++bz) {
                df cx, cy, cz;
                pair_contrib_df<RMW_UF>(df_of_double((rx + bx * P.Lx) * inva), df_of_double((ry + by * P.Ly) * inva),
                                        df_of_double((rz + bz * P.Lz) * inva), Rz, hi, hj, fx, fy, fz, cx, cy, cz);
                ux += to_double(cx); uy += to_double(cy); uz += to_double(cz);
            }
}

__device__ __forceinline__ double wall_damp(double z, double a) { return (z < a) ? z / a : 1.0; }
__device__ __forceinline__ double wall_clamp(double z, double a) { return (z <= a) ? a : z; }

// ---------------------------------------------------------------------------
// two-body mode couplings (training targets)

// A = M_b^-1 X_b (m x 11, row-major)
__device__ void body_minv_modes(const double *__restrict__ Mi, const double *__restrict__ r, int o, int nbl,
                                const double *c, double *A)
{
    const int m = 3 * nbl;
    for (int t = threadIdx.x; t < m; t += blockDim.x) {
        double acc[kModes];
        for (int k = 0; k < kModes; ++k) acc[k] = 0.0;
        for (int q = 0; q < nbl; ++q) {
            const int i = o + q;
            const double dx = r[3 * i] - c[0], dy = r[3 * i + 1] - c[1], dz = r[3 * i + 2] - c[2];
            // M^-1 symmetric: column t of rows 3q..3q+2, coalesced across threads
            const double m0 = Mi[(long long)(3 * q) * m + t], m1 = Mi[(long long)(3 * q + 1) * m + t],
                         m2 = Mi[(long long)(3 * q + 2) * m + t];
#pragma unroll
            for (int k = 0; k < kModes; ++k) {
                double vx, vy, vz;
                mode_velocity(k, dx, dy, dz, vx, vy, vz);
                acc[k] += m0 * vx + m1 * vy + m2 * vz;
            }
        }
        for (int k = 0; k < kModes; ++k) A[t * kModes + k] = acc[k];
    }
}

// Ginv = (X_b^T A)^-1 (11 x 11), Gauss-Jordan with partial pivoting by one thread
__device__ void mode_gram_inverse(const double *A, const double *__restrict__ r, int o, int nbl, const double *c,
                                  double *aug, double *Ginv, int *status)
{
    for (int e = threadIdx.x; e < kModes * kModes; e += blockDim.x) {
        const int k = e / kModes, l = e % kModes;
        double g = 0.0;
        for (int q = 0; q < nbl; ++q) {
            const int i = o + q;
            double vx, vy, vz;
            mode_velocity(k, r[3 * i] - c[0], r[3 * i + 1] - c[1], r[3 * i + 2] - c[2], vx, vy, vz);
            g += vx * A[(3 * q) * kModes + l] + vy * A[(3 * q + 1) * kModes + l] + vz * A[(3 * q + 2) * kModes + l];
        }
        aug[k * 2 * kModes + l] = g;
        aug[k * 2 * kModes + kModes + l] = (k == l) ? 1.0 : 0.0;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const int w = 2 * kModes;
        for (int cc = 0; cc < kModes; ++cc) {
            int piv = cc;
            for (int i = cc + 1; i < kModes; ++i)
                if (fabs(aug[i * w + cc]) > fabs(aug[piv * w + cc])) piv = i;
            if (piv != cc)
                for (int j = 0; j < w; ++j) {
                    const double t = aug[cc * w + j];
                    aug[cc * w + j] = aug[piv * w + j];
                    aug[piv * w + j] = t;
                }
            const double dg = aug[cc * w + cc];
            if (!(fabs(dg) > 0.0)) {
                atomicExch(status, 3);
                continue;
            }
            for (int j = 0; j < w; ++j) aug[cc * w + j] /= dg;
            for (int i = 0; i < kModes; ++i) {
                if (i == cc) continue;
                const double f = aug[i * w + cc];
                for (int j = 0; j < w; ++j) aug[i * w + j] -= f * aug[cc * w + j];
            }
        }
    }
    __syncthreads();
    for (int e = threadIdx.x; e < kModes * kModes; e += blockDim.x)
        Ginv[e] = aug[(e / kModes) * 2 * kModes + kModes + e % kModes];
    __syncthreads();
}

// out = Gi^-1 A_i^T M_ij A_j Gj^-1 (11 x 11, row-major): response of body i's
// modes to body j's mode moments.  Lam, V: scratch (m x 11).
__device__ void mode_coupling(const double *__restrict__ r, int oi, int ni, const double *Ai, const double *Giinv,
                              int oj, int nj, const double *Aj, const double *Gjinv, double a, double nf,
                              const Images &P, double *Lam, double *V, double *W, double *out)
{
    const int mj = 3 * nj, mi = 3 * ni;
    const double inva = 1.0 / a;
    for (int e = threadIdx.x; e < mj * kModes; e += blockDim.x) {
        const int t = e / kModes, l = e % kModes;
        double acc = 0.0;
        for (int k = 0; k < kModes; ++k) acc += Aj[t * kModes + k] * Gjinv[k * kModes + l];
        Lam[e] = acc;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < ni * kModes; e += blockDim.x) {
        const int p = e / kModes, l = e % kModes;
        const int i = oi + p;
        const double zi = r[3 * i + 2];
        const double zie = wall_clamp(zi, a);
        double ux = 0.0, uy = 0.0, uz = 0.0;
        for (int q = 0; q < nj; ++q) {
            const int j = oj + q;
            const double zj = r[3 * j + 2];
            const double bj = wall_damp(zj, a);
            wall_uf_pair(r[3 * i], r[3 * i + 1], zie, r[3 * j], r[3 * j + 1], wall_clamp(zj, a), inva, P,
                         bj * Lam[(3 * q) * kModes + l], bj * Lam[(3 * q + 1) * kModes + l],
                         bj * Lam[(3 * q + 2) * kModes + l], ux, uy, uz);
        }
        const double sc = nf * wall_damp(zi, a);
        V[(3 * p) * kModes + l] = sc * ux;
        V[(3 * p + 1) * kModes + l] = sc * uy;
        V[(3 * p + 2) * kModes + l] = sc * uz;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < kModes * kModes; e += blockDim.x) {
        const int k = e / kModes, l = e % kModes;
        double acc = 0.0;
        for (int t = 0; t < mi; ++t) acc += Ai[t * kModes + k] * V[t * kModes + l];
        W[e] = acc;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < kModes * kModes; e += blockDim.x) {
        const int k = e / kModes, l = e % kModes;
        double acc = 0.0;
        for (int p = 0; p < kModes; ++p) acc += Giinv[k * kModes + p] * W[p * kModes + l];
        out[e] = acc;
    }
    __syncthreads();
}

// One CTA per sample s = bodies (2s, 2s+1): out[242 s ..] = G_01, G_10 (lab frame).
__global__ void pair_fts_kernel(const double *__restrict__ r, const double *__restrict__ xb,
                                const int *__restrict__ boff, const long long *__restrict__ moff,
                                const double *__restrict__ minv, double a, double nf, Images P, int max_m,
                                double *__restrict__ out, int *status)
{
    extern __shared__ double sh[];
    const int s = blockIdx.x;
    const int b0 = 2 * s, b1 = 2 * s + 1;
    const int o0 = boff[b0], n0 = boff[b0 + 1] - o0, o1 = boff[b1], n1 = boff[b1 + 1] - o1;
    double *A0 = sh, *A1 = A0 + max_m * kModes, *Lam = A1 + max_m * kModes, *V = Lam + max_m * kModes;
    double *G0 = V + max_m * kModes, *G1 = G0 + kModes * kModes, *W = G1 + kModes * kModes;
    double *aug = W + kModes * kModes;
    __shared__ double c0[3], c1[3];
    if (threadIdx.x < 3) {
        c0[threadIdx.x] = xb[3 * b0 + threadIdx.x];
        c1[threadIdx.x] = xb[3 * b1 + threadIdx.x];
    }
    __syncthreads();
    body_minv_modes(minv + moff[b0], r, o0, n0, c0, A0);
    body_minv_modes(minv + moff[b1], r, o1, n1, c1, A1);
    __syncthreads();
    mode_gram_inverse(A0, r, o0, n0, c0, aug, G0, status);
    mode_gram_inverse(A1, r, o1, n1, c1, aug, G1, status);
    mode_coupling(r, o0, n0, A0, G0, o1, n1, A1, G1, a, nf, P, Lam, V, W, out + 242LL * s);
    mode_coupling(r, o1, n1, A1, G1, o0, n0, A0, G0, a, nf, P, Lam, V, W, out + 242LL * s + 121);
}

// G_ij (lab frame) of listed ordered pairs (i, j) of the handle's bodies; one
// CTA per pair, the same steps as pair_fts_kernel.
__global__ void pair_list_kernel(const double *__restrict__ r, const double *__restrict__ xb,
                                 const int *__restrict__ boff, const long long *__restrict__ moff,
                                 const double *__restrict__ minv, const int *__restrict__ pairs, double a, double nf,
                                 Images P, int max_m, double *__restrict__ out, int *status)
{
    extern __shared__ double sh[];
    const int q = blockIdx.x;
    const int b0 = pairs[2 * q], b1 = pairs[2 * q + 1];
    const int o0 = boff[b0], n0 = boff[b0 + 1] - o0, o1 = boff[b1], n1 = boff[b1 + 1] - o1;
    double *A0 = sh, *A1 = A0 + max_m * kModes, *Lam = A1 + max_m * kModes, *V = Lam + max_m * kModes;
    double *G0 = V + max_m * kModes, *G1 = G0 + kModes * kModes, *W = G1 + kModes * kModes;
    double *aug = W + kModes * kModes;
    __shared__ double c0[3], c1[3];
    if (threadIdx.x < 3) {
        c0[threadIdx.x] = xb[3 * b0 + threadIdx.x];
        c1[threadIdx.x] = xb[3 * b1 + threadIdx.x];
    }
    __syncthreads();
    body_minv_modes(minv + moff[b0], r, o0, n0, c0, A0);
    body_minv_modes(minv + moff[b1], r, o1, n1, c1, A1);
    __syncthreads();
    mode_gram_inverse(A0, r, o0, n0, c0, aug, G0, status);
    mode_gram_inverse(A1, r, o1, n1, c1, aug, G1, status);
    mode_coupling(r, o0, n0, A0, G0, o1, n1, A1, G1, a, nf, P, Lam, V, W, out + 121LL * q);
}

// ---------------------------------------------------------------------------
// neighbour lists: ordered pairs (i, j != i) of one suspension by centre
// distance (minimum image)

// Neighbour bands of every body, one warp per body: the lanes take the
// candidates j of the body's suspension in ascending order, 32 at a time; the
// count pass (cnt != null) counts the exact (d < cut_ex), learned
// (cut_lf <= d < cut_ln, not exact) and message-passing (d < cut_mp) hits; the
// fill pass writes each band's hits at the body's CSR offset, placed by the
// ballot prefix of the lane, so every list is sorted by j.  Distances are
// formed in FP32 from FP32 centres (minimum image in periodic directions).
__global__ void nbr_bands_kernel(const double *__restrict__ xb, int nb, float cut_ex2, float cut_lf2, float cut_ln2,
                                 float cut_mp2, Images P, const int2 *__restrict__ range, int *__restrict__ cnt,
                                 const int *__restrict__ ex_off, int *__restrict__ ex_idx,
                                 const int *__restrict__ ln_off, int *__restrict__ ln_idx,
                                 const int *__restrict__ mp_off, int *__restrict__ mp_idx)
{
    const int i = (int)(((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (i >= nb) return;  // i is uniform across the warp
    const int2 rg = range ? range[i] : make_int2(0, nb);
    const float xi = (float)xb[3 * i], yi = (float)xb[3 * i + 1], zi = (float)xb[3 * i + 2];
    const float Lx = (float)P.Lx, Ly = (float)P.Ly, Lz = (float)P.Lz;
    const bool fill = ex_off != nullptr;
    int ce = fill ? ex_off[i] : 0, cl = fill ? ln_off[i] : 0, cm = fill ? mp_off[i] : 0;
    int ne = 0, nl = 0, nm = 0;
    const unsigned below = (1u << lane) - 1u;
    for (int j0 = rg.x; j0 < rg.y; j0 += 32) {
        const int j = j0 + lane;
        bool ex = false, ln = false, mp = false;
        if (j < rg.y && j != i) {
            float dx = (float)xb[3 * j] - xi, dy = (float)xb[3 * j + 1] - yi, dz = (float)xb[3 * j + 2] - zi;
            if (Lx > 0.f) dx = project(dx, Lx);
            if (Ly > 0.f) dy = project(dy, Ly);
            if (Lz > 0.f) dz = project(dz, Lz);
            const float d2 = dx * dx + dy * dy + dz * dz;
            ex = d2 < cut_ex2;
            ln = !ex && d2 < cut_ln2 && d2 >= cut_lf2;
            mp = d2 < cut_mp2;
        }
        const unsigned me = __ballot_sync(0xffffffffu, ex), ml = __ballot_sync(0xffffffffu, ln),
                       mm = __ballot_sync(0xffffffffu, mp);
        if (fill) {
            if (ex) ex_idx[ce + __popc(me & below)] = j;
            if (ln) ln_idx[cl + __popc(ml & below)] = j;
            if (mp) mp_idx[cm + __popc(mm & below)] = j;
        }
        ce += __popc(me);
        cl += __popc(ml);
        cm += __popc(mm);
        ne += __popc(me);
        nl += __popc(ml);
        nm += __popc(mm);
    }
    if (!fill && lane == 0) {
        cnt[i] = ne;
        cnt[nb + i] = nl;
        cnt[2 * nb + i] = nm;
    }
}

__device__ __forceinline__ int owner_of(const int *__restrict__ off, int nb, int q)
{
    int lo = 0, hi = nb;
    while (hi - lo > 1) {
        const int mid = (lo + hi) / 2;
        if (off[mid] <= q) lo = mid; else hi = mid;
    }
    return lo;
}

// horizontal separation of entry q's pair (owner -> neighbour), minimum image
__device__ __forceinline__ void pair_horizontal(const double *__restrict__ xb, int i, int j, const Images &P,
                                                double &dx, double &dy)
{
    dx = xb[3 * j] - xb[3 * i];
    dy = xb[3 * j + 1] - xb[3 * i + 1];
    if (P.Lx > 0) dx = project(dx, P.Lx);
    if (P.Ly > 0) dy = project(dy, P.Ly);
}

// owner (CSR row) of every entry of a list
__global__ void csr_owner_kernel(const int *__restrict__ off, int nb, int *__restrict__ owner)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nb) return;
    for (int q = off[i]; q < off[i + 1]; ++q) owner[q] = i;
}

// raw edge features (horizontal distance, z_dst, z_src) / R of list entries (dst = owner)
__global__ void edge_raw_features_kernel(const double *__restrict__ xb, const int *__restrict__ owner,
                                         const int *__restrict__ idx, int n, double inv_radius, Images P,
                                         float *__restrict__ feat)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    const int i = owner[q], j = idx[q];
    double dx, dy;
    pair_horizontal(xb, i, j, P, dx, dy);
    feat[3LL * q] = (float)(sqrt(dx * dx + dy * dy) * inv_radius);
    feat[3LL * q + 1] = (float)(xb[3 * i + 2] * inv_radius);
    feat[3LL * q + 2] = (float)(xb[3 * j + 2] * inv_radius);
}

// raw node features (z / R, message neighbours / 8)
__global__ void node_raw_features_kernel(const double *__restrict__ xb, const int *__restrict__ mp_off, int nb,
                                         double inv_radius, float *__restrict__ feat)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nb) return;
    feat[2LL * i] = (float)(xb[3 * i + 2] * inv_radius);
    feat[2LL * i + 1] = (float)(mp_off[i + 1] - mp_off[i]) / 8.0f;
}

// G_lab = Q G' Q^T, G' = network output * target scale (pair frame).  FP32:
// the network's outputs carry BF16-level accuracy.  One thread per (entry,
// row of G_lab).
__global__ void pair_blocks_kernel(const float *__restrict__ Yf, const double *__restrict__ xb,
                                   const int *__restrict__ off, const int *__restrict__ idx, int nb, int npairs,
                                   Images P, const float *__restrict__ tscale, double *__restrict__ G)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)npairs * kModes) return;
    const int q = (int)(t / kModes), a = (int)(t % kModes);
    const int i = owner_of(off, nb, q), j = idx[q];
    double dx, dy;
    pair_horizontal(xb, i, j, P, dx, dy);
    const double rho = sqrt(dx * dx + dy * dy);
    const float c = rho > 0 ? (float)(dx / rho) : 1.f, s = rho > 0 ? (float)(dy / rho) : 0.f;
    float Q[kModes][kModes];
    mode_rotation(c, s, Q);
    const float *y = Yf + (long long)q * kMpOut;
    float row[kModes];  // (Q G')[a][:]
    for (int l = 0; l < kModes; ++l) {
        float acc = 0.f;
        for (int k = 0; k < kModes; ++k) acc += Q[a][k] * y[kModes * k + l] * tscale[kModes * k + l];
        row[l] = acc;
    }
    for (int b = 0; b < kModes; ++b) {
        float acc = 0.f;
        for (int l = 0; l < kModes; ++l) acc += row[l] * Q[b][l];
        G[121LL * q + kModes * a + b] = (double)acc;
    }
}

// ---------------------------------------------------------------------------
// augmented preconditioner apply

// mode moments X_b^T lambda_b of every body (one warp per body)
__global__ void body_moments_kernel(const double *__restrict__ r, const double *__restrict__ xb,
                                    const int *__restrict__ boff, int nb, const double *__restrict__ lam,
                                    double *__restrict__ mom)
{
    const int b = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (b >= nb) return;
    const int o = boff[b], nbl = boff[b + 1] - o;
    double acc[kModes];
#pragma unroll
    for (int k = 0; k < kModes; ++k) acc[k] = 0.0;
    for (int p = lane; p < nbl; p += 32) {
        const int i = o + p;
        const double dx = r[3 * i] - xb[3 * b], dy = r[3 * i + 1] - xb[3 * b + 1], dz = r[3 * i + 2] - xb[3 * b + 2];
        const double lx = lam[3 * i], ly = lam[3 * i + 1], lz = lam[3 * i + 2];
#pragma unroll
        for (int k = 0; k < kModes; ++k) {
            double vx, vy, vz;
            mode_velocity(k, dx, dy, dz, vx, vy, vz);
            acc[k] += vx * lx + vy * ly + vz * lz;
        }
    }
#pragma unroll
    for (int k = 0; k < kModes; ++k) {
        for (int off = 16; off > 0; off >>= 1) acc[k] += __shfl_xor_sync(0xffffffffu, acc[k], off);
        if (lane == 0) mom[kModes * b + k] = acc[k];
    }
}

// Exact near pairs, one CTA per neighbour entry q = (owner i, neighbour j):
// part[q] (3 x blobs of i, unscaled) = sum over j's blobs of the pair
// velocities.  Threads split as (target blob, source subset); the subsets are
// added in a fixed order.
__global__ void nf_pairs_kernel(const double *__restrict__ r, const int *__restrict__ boff,
                                const int *__restrict__ ex_off, const int *__restrict__ ex_idx, int nb,
                                const double *__restrict__ lam, double a, Images P, int part_stride,
                                double *__restrict__ part)
{
    extern __shared__ double acc[];  // nsplit x ni x 3
    const int q = blockIdx.x;
    const int i = owner_of(ex_off, nb, q), j = ex_idx[q];
    const int oi = boff[i], ni = boff[i + 1] - oi, oj = boff[j], nj = boff[j + 1] - oj;
    const int nsplit = max(1, (int)blockDim.x / ni);
    const double inva = 1.0 / a;
    for (int w = threadIdx.x; w < ni * nsplit; w += blockDim.x) {
        const int t = w % ni, sp = w / ni;
        const int ti = oi + t;
        const double zie = wall_clamp(r[3 * ti + 2], a);
        double ux = 0.0, uy = 0.0, uz = 0.0;
        for (int s = sp; s < nj; s += nsplit) {
            const int sj = oj + s;
            const double zj = r[3 * sj + 2], bj = wall_damp(zj, a);
            wall_uf_pair_df(r[3 * ti], r[3 * ti + 1], zie, r[3 * sj], r[3 * sj + 1], wall_clamp(zj, a), inva, P,
                            bj * lam[3 * sj], bj * lam[3 * sj + 1], bj * lam[3 * sj + 2], ux, uy, uz);
        }
        acc[3 * w] = ux;
        acc[3 * w + 1] = uy;
        acc[3 * w + 2] = uz;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < 3 * ni; e += blockDim.x) {
        double sum = 0.0;
        for (int sp = 0; sp < nsplit; ++sp) sum += acc[3 * ni * sp + e];
        part[(long long)q * part_stride + e] = sum;
    }
}

// v_i = nf b_t sum_{exact entries of i} part + X_i sum_{learned j} G_ij mom_j on
// body i's blob rows (one CTA per body; entries in CSR order)
__global__ void nf_gather_kernel(const double *__restrict__ r, const double *__restrict__ xb,
                                 const int *__restrict__ boff, const int *__restrict__ ex_off,
                                 const double *__restrict__ part, int part_stride, const int *__restrict__ ln_off,
                                 const int *__restrict__ ln_idx, const double *__restrict__ G,
                                 const double *__restrict__ mom, double a, double nf, double *__restrict__ v)
{
    __shared__ double cm[kModes];
    const int i = blockIdx.x;
    const int o = boff[i], nbl = boff[i + 1] - o;
    if (threadIdx.x < kModes) {
        double acc = 0.0;
        if (ln_off)
            for (int q = ln_off[i]; q < ln_off[i + 1]; ++q) {
                const double *Gq = G + 121LL * q + kModes * threadIdx.x;
                const double *mj = mom + kModes * ln_idx[q];
                for (int l = 0; l < kModes; ++l) acc += Gq[l] * mj[l];
            }
        cm[threadIdx.x] = acc;
    }
    __syncthreads();
    const int e0 = ex_off ? ex_off[i] : 0, e1 = ex_off ? ex_off[i + 1] : 0;
    for (int p = threadIdx.x; p < nbl; p += blockDim.x) {
        const int ti = o + p;
        double ux = 0.0, uy = 0.0, uz = 0.0;
        for (int q = e0; q < e1; ++q) {
            const double *pq = part + (long long)q * part_stride + 3 * p;
            ux += pq[0]; uy += pq[1]; uz += pq[2];
        }
        const double zi = r[3 * ti + 2];
        const double sc = nf * wall_damp(zi, a);
        double wx = sc * ux, wy = sc * uy, wz = sc * uz;
        const double dx = r[3 * ti] - xb[3 * i], dy = r[3 * ti + 1] - xb[3 * i + 1], dz = zi - xb[3 * i + 2];
#pragma unroll
        for (int k = 0; k < kModes; ++k) {
            double mx, my, mz;
            mode_velocity(k, dx, dy, dz, mx, my, mz);
            wx += mx * cm[k];
            wy += my * cm[k];
            wz += mz * cm[k];
        }
        v[3LL * ti] = wx;
        v[3LL * ti + 1] = wy;
        v[3LL * ti + 2] = wz;
    }
}

__global__ void nf_subtract_kernel(double *__restrict__ y, const double *__restrict__ z, long long n)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] -= z[i];
}

static Images images_of(const RigidSystem &S) { return Images{S.L[0], S.L[1], S.L[2]}; }

int nearfield_apply_pc(RigidSystem &S, const double *x, double *y)
{
    if (int rc = rigid_apply_pc_plain(S, x, y)) return rc;
    const double nf = 1.0 / (8.0 * kPi * S.eta * S.a);
    const int stride = S.max_m;  // 3 x largest blob count per body
    if (S.nf_ln_pairs > 0)
        body_moments_kernel<<<(S.nb * 32 + 127) / 128, 128, 0, S.st>>>(S.r, S.xb, S.boff, S.nb, y, S.nf_mom);
    if (S.nf_ex_pairs > 0) {
        const int nt = 512;  // 42-blob bodies: 12 source subsets of 3-4 blobs per target
        const size_t sm = sizeof(double) * 3 * (size_t)std::max(nt, S.max_m / 3);
        if (sm > 48 * 1024)
            RMW_CUDA(cudaFuncSetAttribute(nf_pairs_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        nf_pairs_kernel<<<S.nf_ex_pairs, nt, sm, S.st>>>(S.r, S.boff, S.nf_ex_off, S.nf_ex_idx, S.nb, y, S.a,
                                                          images_of(S), stride, S.nf_part);
    }
    nf_gather_kernel<<<S.nb, 64, 0, S.st>>>(S.r, S.xb, S.boff, S.nf_ex_pairs ? S.nf_ex_off : nullptr, S.nf_part,
                                             stride, S.nf_ln_pairs ? S.nf_ln_off : nullptr, S.nf_ln_idx, S.nf_G,
                                             S.nf_mom, S.a, nf, S.nf_v);
    RMW_CHECK_LAUNCH("near-field velocities");
    if (int rc = rigid_apply_pc_plain(S, S.nf_v, S.nf_z)) return rc;
    const long long n = S.sys_size();
    nf_subtract_kernel<<<(unsigned)((n + 255) / 256), 256, 0, S.st>>>(y, S.nf_z, n);
    RMW_CHECK_LAUNCH("near-field preconditioner apply");
    return RMW_OK;
}

// ---------------------------------------------------------------------------
// FP32 preconditioner apply of the mixed-precision solves
//
// A mixed solve's inner GMRES runs on FP32 pair products to a 1e-5 relative
// residual and its refinement residual is FP64-accurate, so its preconditioner
// needs no FP64 arithmetic: any fixed approximate inverse serves, and the FP32
// rounding of the apply (~1e-7) stays far below the inner tolerance.  On GB300
// the FP64 pipe runs at 1/64 of the FP32 rate and the FP64 apply's dependent
// multiply-add chains (one m x m block per body) are latency-bound on it.  The
// FP32 form reads FP32 copies of M_b^-1, M_b^-1 K, N_b, of the learned
// couplings and of the blob geometry (offset from the body centre, height),
// so that no FP64 instruction is left in its loops.  The plain apply is one
// kernel, the augmented apply two:
//   pc_apply_f32_kernel<true>  y0 = P0 x, the damped blob forces b lambda(y0)
//                              in FP32 and the 11 mode moments of lambda(y0);
//   nf_correct_f32_kernel      per body i: v_i from the exact pairs (blob by
//                              blob, FP32 pair math) and the learned modes,
//                              z_i = P0_i [v_i; 0], y_i = y0_i - z_i.
// Every sum runs in a fixed order, so the apply is deterministic.

constexpr int kPcF32Threads = 128;
constexpr int kPcF32MaxM = 1536;  // 512 blobs per body: shared-memory layout bound

__device__ __forceinline__ void mode_velocity_f(int c, float dx, float dy, float dz, float &vx, float &vy, float &vz)
{
    const float s2 = (float)kS2, s6 = (float)kS6;
    switch (c) {
    case 0: vx = 1.f; vy = 0.f; vz = 0.f; break;
    case 1: vx = 0.f; vy = 1.f; vz = 0.f; break;
    case 2: vx = 0.f; vy = 0.f; vz = 1.f; break;
    case 3: vx = 0.f; vy = -dz; vz = dy; break;
    case 4: vx = dz; vy = 0.f; vz = -dx; break;
    case 5: vx = -dy; vy = dx; vz = 0.f; break;
    case 6: vx = s2 * dx; vy = -s2 * dy; vz = 0.f; break;
    case 7: vx = -s6 * dx; vy = -s6 * dy; vz = 2.f * s6 * dz; break;
    case 8: vx = s2 * dy; vy = s2 * dx; vz = 0.f; break;
    case 9: vx = s2 * dz; vy = 0.f; vz = s2 * dx; break;
    default: vx = 0.f; vy = s2 * dz; vz = s2 * dy; break;
    }
}

// blob32[i] = (r_i - x_b, z_i) in FP32, b the body of blob i
__global__ void blob_geometry_f32_kernel(const double *__restrict__ r, const double *__restrict__ xb,
                                         const int *__restrict__ blob_body, int n, float4 *__restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int b = blob_body[i];
    out[i] = make_float4((float)(r[3 * i] - xb[3 * b]), (float)(r[3 * i + 1] - xb[3 * b + 1]),
                         (float)(r[3 * i + 2] - xb[3 * b + 2]), (float)r[3 * i + 2]);
}

// unscaled wall-RPY velocity at a blob from a blob carrying v (already damped),
// FP32: d = (centre difference, rounded once) + (offset difference); heights
// clamped at a; periodic directions by the same images as the all-pairs product
__device__ __forceinline__ void wall_uf_pair_f(float dx, float dy, float dz, float zi, float zj, float a, float inva,
                                               const Images &P, float Lx, float Ly, float Lz, float vx, float vy,
                                               float vz, float &ux, float &uy, float &uz)
{
    const float zie = zi <= a ? a : zi, zje = zj <= a ? a : zj;
    const float hi = zie * inva, hj = zje * inva, Rz = (zie + zje) * inva;
    dz = zie - zje;  // the clamped heights' difference, as the FP64 pair uses
    if (!(Lx > 0.f || Ly > 0.f || Lz > 0.f)) {
        float cx = 0.f, cy = 0.f, cz = 0.f;
        pair_contrib<RMW_UF, float>(dx * inva, dy * inva, dz * inva, Rz, hi, hj, vx, vy, vz, cx, cy, cz);
        ux += cx; uy += cy; uz += cz;
        return;
    }
    if (Lx > 0.f) dx = project(dx, Lx);
    if (Ly > 0.f) dy = project(dy, Ly);
    if (Lz > 0.f) dz = project(dz, Lz);
    const int px = Lx > 0.f, py = Ly > 0.f, pz = Lz > 0.f;
    for (int bx = -px; bx <= px; ++bx)
        for (int by = -py; by <= py; ++by)
            for (int bz = -pz; bz <= pz; ++bz) {
                float cx = 0.f, cy = 0.f, cz = 0.f;
                pair_contrib<RMW_UF, float>((dx + bx * Lx) * inva, (dy + by * Ly) * inva, (dz + bz * Lz) * inva, Rz,
                                            hi, hj, vx, vy, vz, cx, cy, cz);
                ux += cx; uy += cy; uz += cz;
            }
}

// lam = M_b^-1 s + (M_b^-1 K) U with U = N_b (-F - K^T M_b^-1 s), in FP32, for
// body b (the whole CTA): s and lam hold m floats in shared memory, part at
// least blockDim.x floats, red 6 (warps + 1) floats, U 6 floats; F holds the
// body's six force rows, or is null for zero forces.
__device__ void pc_block_f32(int o, int m, const float *__restrict__ Mi, const float *__restrict__ MK,
                             const float *__restrict__ Nb, const float4 *__restrict__ geo, const float *s,
                             const float *F, float *lam, float *part, float *red, float *U)
{
    const int tid = threadIdx.x, nt = blockDim.x, nw = nt >> 5;
    // M_b^-1 s, M^-1 symmetric (columns read coalesced); rows shorter than
    // the CTA split their sources over G groups, summed in group order
    const int G = m <= nt ? nt / m : 1;
    if (G > 1) {
        if (tid < G * m) {
            const int g = tid / m, t = tid - g * m;
            float a0 = 0.f, a1 = 0.f;
            int k = g;
            for (; k + G < m; k += 2 * G) {
                a0 = fmaf(Mi[(long long)k * m + t], s[k], a0);
                a1 = fmaf(Mi[(long long)(k + G) * m + t], s[k + G], a1);
            }
            if (k < m) a0 = fmaf(Mi[(long long)k * m + t], s[k], a0);
            part[g * m + t] = a0 + a1;
        }
        __syncthreads();
        for (int t = tid; t < m; t += nt) {
            float acc = 0.f;
            for (int g = 0; g < G; ++g) acc += part[g * m + t];
            lam[t] = acc;
        }
    } else {
        // four independent chains: four column loads in flight per thread (the blocks of large
        // suspensions stream from HBM; eight chains measured slower, 67 -> 83 us at 4096 shells)
        for (int t = tid; t < m; t += nt) {
            float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
            int k = 0;
            for (; k + 3 < m; k += 4) {
                a0 = fmaf(Mi[(long long)k * m + t], s[k], a0);
                a1 = fmaf(Mi[(long long)(k + 1) * m + t], s[k + 1], a1);
                a2 = fmaf(Mi[(long long)(k + 2) * m + t], s[k + 2], a2);
                a3 = fmaf(Mi[(long long)(k + 3) * m + t], s[k + 3], a3);
            }
            for (; k < m; ++k) a0 = fmaf(Mi[(long long)k * m + t], s[k], a0);
            lam[t] = (a0 + a1) + (a2 + a3);
        }
    }
    __syncthreads();
    // K^T M_b^-1 s
    float p6[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (int p = tid; p < m / 3; p += nt) {
        const float4 d = geo[o + p];
        const float lx = lam[3 * p], ly = lam[3 * p + 1], lz = lam[3 * p + 2];
        p6[0] += lx; p6[1] += ly; p6[2] += lz;
        p6[3] += d.y * lz - d.z * ly;
        p6[4] += d.z * lx - d.x * lz;
        p6[5] += d.x * ly - d.y * lx;
    }
    const int lane = tid & 31, wid = tid >> 5;
#pragma unroll
    for (int c = 0; c < 6; ++c) {
        for (int off = 16; off > 0; off >>= 1) p6[c] += __shfl_xor_sync(0xffffffffu, p6[c], off);
        if (lane == 0) red[6 * wid + c] = p6[c];
    }
    __syncthreads();
    if (tid < 6) {
        float ktl = 0.f;
        for (int w = 0; w < nw; ++w) ktl += red[6 * w + tid];
        red[6 * nw + tid] = (F ? -F[tid] : 0.f) - ktl;
    }
    __syncthreads();
    if (tid < 6) {
        float u = 0.f;
        for (int c = 0; c < 6; ++c) u = fmaf(Nb[6 * tid + c], red[6 * nw + c], u);
        U[tid] = u;
    }
    __syncthreads();
    for (int t = tid; t < m; t += nt) {
        float acc = lam[t];
#pragma unroll
        for (int c = 0; c < 6; ++c) acc = fmaf(MK[6 * t + c], U[c], acc);
        lam[t] = acc;
    }
    __syncthreads();
}

// y = P0 x in FP32 (one CTA per body).  NF: also the damped blob forces
// lam32 = b lambda of the result (the exact pairs' sources) and the 11 mode
// moments X_b^T lambda_b (the learned couplings' inputs; mom may be null).
template <bool NF>
__global__ void __launch_bounds__(kPcF32Threads)
    pc_apply_f32_kernel(const double *__restrict__ x, double *__restrict__ y, const float4 *__restrict__ geo,
                        const int *__restrict__ boff, const long long *__restrict__ moff,
                        const float *__restrict__ minv, const float *__restrict__ minvK,
                        const float *__restrict__ nmat, int n, float a, float *__restrict__ lam32,
                        float *__restrict__ mom)
{
    extern __shared__ float shf[];
    __shared__ float U[6], F[6];
    const int b = blockIdx.x, tid = threadIdx.x, nt = blockDim.x, nw = nt >> 5;
    const int o = boff[b], m = 3 * (boff[b + 1] - o);
    float *s = shf, *lam = s + m, *part = lam + m, *red = part + nt;
    for (int t = tid; t < m; t += nt) s[t] = (float)x[3LL * o + t];
    if (tid < 6) F[tid] = (float)x[3LL * n + 6LL * b + tid];
    __syncthreads();
    pc_block_f32(o, m, minv + moff[b], minvK + 18LL * o, nmat + 36LL * b, geo, s, F, lam, part, red, U);
    for (int t = tid; t < m; t += nt) y[3LL * o + t] = (double)lam[t];
    if (tid < 6) y[3LL * n + 6LL * b + tid] = (double)U[tid];
    if constexpr (NF) {
        const float inva = 1.f / a;
        for (int t = tid; t < m; t += nt) {
            const float z = geo[o + t / 3].w;
            lam32[3LL * o + t] = (z < a ? z * inva : 1.f) * lam[t];
        }
        if (mom) {
            float acc[kModes];
#pragma unroll
            for (int k = 0; k < kModes; ++k) acc[k] = 0.f;
            for (int p = tid; p < m / 3; p += nt) {
                const float4 d = geo[o + p];
                const float lx = lam[3 * p], ly = lam[3 * p + 1], lz = lam[3 * p + 2];
#pragma unroll
                for (int k = 0; k < kModes; ++k) {
                    float vx, vy, vz;
                    mode_velocity_f(k, d.x, d.y, d.z, vx, vy, vz);
                    acc[k] = fmaf(vx, lx, fmaf(vy, ly, fmaf(vz, lz, acc[k])));
                }
            }
            const int lane = tid & 31, wid = tid >> 5;
#pragma unroll
            for (int k = 0; k < kModes; ++k) {
                for (int off = 16; off > 0; off >>= 1) acc[k] += __shfl_xor_sync(0xffffffffu, acc[k], off);
                if (lane == 0) part[kModes * wid + k] = acc[k];  // part is free again (nw x 11 <= nt floats)
            }
            __syncthreads();
            if (tid < kModes) {
                float sum = 0.f;
                for (int w = 0; w < nw; ++w) sum += part[kModes * w + tid];
                mom[kModes * b + tid] = sum;
            }
        }
    }
}

// y = y0 - P0 [v; 0] with v the near-field blob velocities of lambda(y0):
// exact pairs blob by blob (threads split as target blob x source subset,
// subsets summed in order), learned pairs through the mode moments.
__global__ void __launch_bounds__(kPcF32Threads)
    nf_correct_f32_kernel(const double *__restrict__ y0, double *__restrict__ y, const float4 *__restrict__ geo,
                          const double *__restrict__ xb, const int *__restrict__ boff,
                          const long long *__restrict__ moff, const float *__restrict__ minv,
                          const float *__restrict__ minvK, const float *__restrict__ nmat, int n,
                          const int *__restrict__ ex_off, const int *__restrict__ ex_idx,
                          const float *__restrict__ lam32, const int *__restrict__ ln_off,
                          const int *__restrict__ ln_idx, const float *__restrict__ G, const float *__restrict__ mom,
                          float a, float nfac, Images P)
{
    extern __shared__ float shf[];
    __shared__ float U[6], cm[kModes], cmp[kModes * kModes];
    const int b = blockIdx.x, tid = threadIdx.x, nt = blockDim.x;
    const int o = boff[b], nbl = boff[b + 1] - o, m = 3 * nbl;
    float *v = shf, *lam = v + m, *part = lam + m, *red = part + 3 * max(nt, nbl);
    const float inva = 1.f / a;
    const float Lx = (float)P.Lx, Ly = (float)P.Ly, Lz = (float)P.Lz;
    // exact pairs
    const int nsplit = max(1, nt / nbl);
    const int e0 = ex_off ? ex_off[b] : 0, e1 = ex_off ? ex_off[b + 1] : 0;
    for (int w = tid; w < nbl * nsplit; w += nt) {
        const int t = w % nbl, sp = w / nbl;
        const float4 gt = geo[o + t];
        float ux = 0.f, uy = 0.f, uz = 0.f;
        for (int q = e0; q < e1; ++q) {
            const int j = ex_idx[q], oj = boff[j], nj = boff[j + 1] - oj;
            // centre difference in FP64, rounded once per neighbour
            const float cx = (float)(xb[3 * b] - xb[3 * j]), cy = (float)(xb[3 * b + 1] - xb[3 * j + 1]);
            for (int s = sp; s < nj; s += nsplit) {
                const float4 gs = geo[oj + s];
                const float *ls = lam32 + 3LL * (oj + s);
                wall_uf_pair_f(cx + (gt.x - gs.x), cy + (gt.y - gs.y), 0.f, gt.w, gs.w, a, inva, P, Lx, Ly, Lz,
                               ls[0], ls[1], ls[2], ux, uy, uz);
            }
        }
        part[3 * w] = ux;
        part[3 * w + 1] = uy;
        part[3 * w + 2] = uz;
    }
    // learned pairs: cm = sum_q G_q mom_j(q), entry (k, l) per thread, then rows in order
    if (tid < kModes * kModes) {
        float acc = 0.f;
        if (ln_off)
            for (int q = ln_off[b]; q < ln_off[b + 1]; ++q)
                acc = fmaf(G[121LL * q + tid], mom[kModes * ln_idx[q] + tid % kModes], acc);
        cmp[tid] = acc;
    }
    __syncthreads();
    if (tid < kModes) {
        float c = 0.f;
        for (int l = 0; l < kModes; ++l) c += cmp[kModes * tid + l];
        cm[tid] = c;
    }
    __syncthreads();
    for (int t = tid; t < nbl; t += nt) {
        float ux = 0.f, uy = 0.f, uz = 0.f;
        for (int sp = 0; sp < nsplit; ++sp) {
            const float *pp = part + 3 * (sp * nbl + t);
            ux += pp[0]; uy += pp[1]; uz += pp[2];
        }
        const float4 gt = geo[o + t];
        const float sc = nfac * (gt.w < a ? gt.w * inva : 1.f);
        float wx = sc * ux, wy = sc * uy, wz = sc * uz;
#pragma unroll
        for (int k = 0; k < kModes; ++k) {
            float mx, my, mz;
            mode_velocity_f(k, gt.x, gt.y, gt.z, mx, my, mz);
            wx = fmaf(mx, cm[k], wx);
            wy = fmaf(my, cm[k], wy);
            wz = fmaf(mz, cm[k], wz);
        }
        v[3 * t] = wx;
        v[3 * t + 1] = wy;
        v[3 * t + 2] = wz;
    }
    __syncthreads();
    pc_block_f32(o, m, minv + moff[b], minvK + 18LL * o, nmat + 36LL * b, geo, v, nullptr, lam, part, red, U);
    for (int t = tid; t < m; t += nt) y[3LL * o + t] = y0[3LL * o + t] - (double)lam[t];
    if (tid < 6) y[3LL * n + 6LL * b + tid] = y0[3LL * n + 6LL * b + tid] - (double)U[tid];
}

__global__ void to_f32_kernel(const double *__restrict__ x, float *__restrict__ y, long long n)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        y[i] = (float)x[i];
}

static void to_f32(const double *x, float *y, long long n, cudaStream_t st)
{
    if (n <= 0) return;
    const unsigned g = (unsigned)std::min<long long>((n + 255) / 256, 152LL * 16);
    to_f32_kernel<<<g, 256, 0, st>>>(x, y, n);
}

int rigid_pc_prepare_f32(RigidSystem &S)
{
    if (!S.pc_ready) return fail(RMW_ERR_ARG, "preconditioner not built (call rmw_rigid_build_pc)");
    if (S.pc32_ready || S.max_m > kPcF32MaxM) return RMW_OK;
    const long long tot = S.moff_h[S.nb];
    if (int rc = alloc_pc32(S)) return rc;
    if (!S.pc32_blocks) {
        to_f32(S.minv, S.minv32, tot, S.st);
        to_f32(S.minvK, S.minvK32, 18LL * S.n, S.st);
        to_f32(S.nmat, S.nmat32, 36LL * S.nb, S.st);
    }
    blob_geometry_f32_kernel<<<(S.n + 255) / 256, 256, 0, S.st>>>(S.r, S.xb, S.blob_body, S.n, S.blob32);
    RMW_CHECK_LAUNCH("FP32 preconditioner copies");
    S.pc32_ready = true;
    return RMW_OK;
}

int rigid_apply_pc_mixed(RigidSystem &S, const double *x, double *y)
{
    if (!S.pc_ready) return fail(RMW_ERR_ARG, "preconditioner not built (call rmw_rigid_build_pc)");
    if (S.max_m > kPcF32MaxM) return rigid_apply_pc(S, x, y);
    if (!S.pc32_ready) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        RMW_CUDA(cudaStreamIsCapturing(S.st, &cs));
        if (cs != cudaStreamCaptureStatusNone) return rigid_apply_pc(S, x, y);
        if (int rc = rigid_pc_prepare_f32(S)) return rc;
    }
    const int nt = kPcF32Threads, nw = nt / 32;
    void *tok = nullptr;
    if (int rc = trace_begin(TRACE_PC, S.st, &tok)) return rc;
    const size_t sm2 = sizeof(float) * (2 * (size_t)S.max_m + nt + 6 * (nw + 1));
    const float a = (float)S.a;
    if (!S.nf_on) {
        pc_apply_f32_kernel<false><<<S.nb, nt, sm2, S.st>>>(x, y, S.blob32, S.boff, S.moff, S.minv32, S.minvK32,
                                                             S.nmat32, S.n, a, nullptr, nullptr);
    } else {
        const bool ln = S.nf_ln_pairs > 0;
        pc_apply_f32_kernel<true><<<S.nb, nt, sm2, S.st>>>(x, S.nf_z, S.blob32, S.boff, S.moff, S.minv32, S.minvK32,
                                                            S.nmat32, S.n, a, S.nf_lam32, ln ? S.nf_mom32 : nullptr);
        const size_t sm3 = sizeof(float) * (2 * (size_t)S.max_m + 3 * (size_t)std::max(nt, S.max_m / 3) +
                                            6 * (nw + 1));
        const float nf = (float)(1.0 / (8.0 * kPi * S.eta * S.a));
        nf_correct_f32_kernel<<<S.nb, nt, sm3, S.st>>>(
            S.nf_z, y, S.blob32, S.xb, S.boff, S.moff, S.minv32, S.minvK32, S.nmat32, S.n,
            S.nf_ex_pairs ? S.nf_ex_off : nullptr, S.nf_ex_idx, S.nf_lam32, ln ? S.nf_ln_off : nullptr, S.nf_ln_idx,
            S.nf_G32, S.nf_mom32, a, nf, images_of(S));
    }
    if (int rc = trace_end(tok, S.st)) return rc;
    RMW_CHECK_LAUNCH("FP32 preconditioner apply");
    return RMW_OK;
}

// grow-only per-entry arrays of the two lists: capacities in entries, shared
// by the index array and the per-entry data (pair velocities, mode couplings)
static int grow_lists(RigidSystem &S, size_t need_ex, size_t need_ln)
{
    if (!S.nf_ex_idx || need_ex > S.nf_cap_ex) {
        if (S.nf_ex_idx) RMW_CUDA(cudaFree(S.nf_ex_idx));
        if (S.nf_part) RMW_CUDA(cudaFree(S.nf_part));
        S.nf_ex_idx = nullptr;
        S.nf_part = nullptr;
        S.nf_cap_ex = 0;
        const size_t want = std::max<size_t>(need_ex + need_ex / 4, 64);
        RMW_CUDA(cudaMalloc(&S.nf_ex_idx, sizeof(int) * want));
        RMW_CUDA(cudaMalloc(&S.nf_part, sizeof(double) * (size_t)S.max_m * want));
        S.nf_cap_ex = want;
    }
    if (!S.nf_ln_idx || need_ln > S.nf_cap_ln) {
        if (S.nf_ln_idx) RMW_CUDA(cudaFree(S.nf_ln_idx));
        if (S.nf_G) RMW_CUDA(cudaFree(S.nf_G));
        if (S.nf_G32) RMW_CUDA(cudaFree(S.nf_G32));
        S.nf_G32 = nullptr;
        S.nf_ln_idx = nullptr;
        S.nf_G = nullptr;
        S.nf_cap_ln = 0;
        const size_t want = std::max<size_t>(need_ln + need_ln / 4, 64);
        RMW_CUDA(cudaMalloc(&S.nf_ln_idx, sizeof(int) * want));
        RMW_CUDA(cudaMalloc(&S.nf_G, sizeof(double) * 121 * want));
        RMW_CUDA(cudaMalloc(&S.nf_G32, sizeof(float) * 121 * want));
        S.nf_cap_ln = want;
    }
    return RMW_OK;
}

// exact (d < cut_ex), learned (cut_ex <= d < cut_ln, d >= cut_lf) and
// message-passing (d < cut_mp) neighbour lists of the handle's bodies: one
// counting pass, one host round trip, one filling pass
static int build_bands(RigidSystem &S, double cut_ex, double cut_lf, double cut_ln, double cut_mp)
{
    cudaStream_t st = S.st;
    const int nb = S.nb;
    if (!S.nf_off) {
        RMW_CUDA(cudaMalloc(&S.nf_off, sizeof(int) * 3 * (nb + 1)));
        RMW_CUDA(cudaMalloc(&S.nf_cnt, sizeof(int) * 3 * nb));
    }
    S.nf_ex_off = S.nf_off;
    S.nf_ln_off = S.nf_off + nb + 1;
    S.nf_mp_off = S.nf_off + 2 * (nb + 1);
    const int2 *range = nullptr;
    if (!S.susp_body_off.empty()) {
        std::vector<int2> rg(nb);
        for (size_t k = 0; k + 1 < S.susp_body_off.size(); ++k)
            for (long long b = S.susp_body_off[k]; b < S.susp_body_off[k + 1]; ++b)
                rg[b] = make_int2((int)S.susp_body_off[k], (int)S.susp_body_off[k + 1]);
        if (!S.nf_range) RMW_CUDA(cudaMalloc(&S.nf_range, sizeof(int2) * nb));
        RMW_CUDA(cudaMemcpyAsync(S.nf_range, rg.data(), sizeof(int2) * nb, cudaMemcpyHostToDevice, st));
        range = S.nf_range;
    }
    const Images P = images_of(S);
    const float e2 = (float)(cut_ex * cut_ex), f2 = (float)(cut_lf * cut_lf), l2 = (float)(cut_ln * cut_ln),
                m2 = (float)(cut_mp * cut_mp);
    const unsigned g = (unsigned)(((long long)nb * 32 + 255) / 256);  // one warp per body
    nbr_bands_kernel<<<g, 256, 0, st>>>(S.xb, nb, e2, f2, l2, m2, P, range, S.nf_cnt, nullptr, nullptr, nullptr,
                                         nullptr, nullptr, nullptr);
    RMW_CHECK_LAUNCH("neighbour count");
    std::vector<int> cnt(3 * (size_t)nb), off(3 * ((size_t)nb + 1), 0);
    RMW_CUDA(cudaMemcpyAsync(cnt.data(), S.nf_cnt, sizeof(int) * 3 * nb, cudaMemcpyDeviceToHost, st));
    RMW_CUDA(cudaStreamSynchronize(st));
    for (int band = 0; band < 3; ++band) {
        int *o = off.data() + (size_t)band * (nb + 1);
        for (int b = 0; b < nb; ++b) o[b + 1] = o[b] + cnt[(size_t)band * nb + b];
    }
    S.nf_ex_pairs = off[nb];
    S.nf_ln_pairs = off[2 * (size_t)nb + 1];
    S.nf_mp_pairs = off[3 * (size_t)nb + 2];
    RMW_CUDA(cudaMemcpyAsync(S.nf_off, off.data(), sizeof(int) * off.size(), cudaMemcpyHostToDevice, st));
    if (int rc = grow_lists(S, (size_t)S.nf_ex_pairs, (size_t)S.nf_ln_pairs)) return rc;
    if (!S.nf_mp_idx || (size_t)S.nf_mp_pairs > S.nf_cap_mp) {
        if (S.nf_mp_idx) RMW_CUDA(cudaFree(S.nf_mp_idx));
        S.nf_mp_idx = nullptr;
        S.nf_cap_mp = 0;
        const size_t want = std::max<size_t>((size_t)S.nf_mp_pairs + S.nf_mp_pairs / 4, 64);
        RMW_CUDA(cudaMalloc(&S.nf_mp_idx, sizeof(int) * want));
        S.nf_cap_mp = want;
    }
    // the count pass wrote the offsets' sources; the fill pass writes the lists
    nbr_bands_kernel<<<g, 256, 0, st>>>(S.xb, nb, e2, f2, l2, m2, P, range, nullptr, S.nf_ex_off, S.nf_ex_idx,
                                         S.nf_ln_off, S.nf_ln_idx, S.nf_mp_off, S.nf_mp_idx);
    RMW_CHECK_LAUNCH("neighbour fill");
    return RMW_OK;
}

// Network couplings of every learned pair into S.nf_G (lab frame): the
// message-passing graph of the handle's bodies (message neighbours, learned
// pairs as band edges), the network's forward pass, the rotation out of each
// pair's frame.
static int learned_couplings(RigidSystem &S, MpnnNet &N)
{
    cudaStream_t st = S.st;
    const int nb = S.nb, np = S.nf_ln_pairs, nm = S.nf_mp_pairs;
    const Images P = images_of(S);
    const double invR = 1.0 / N.radius;
    auto al = [](size_t b) { return (b + 255) / 256 * 256; };
    const size_t bytes = al(sizeof(float) * 2 * nb) + al(sizeof(int) * std::max(nm, 1)) +
                         al(sizeof(float) * 3 * std::max(nm, 1)) + al(sizeof(int) * np) + al(sizeof(float) * 3 * np);
    void *buf = nullptr;
    RMW_CUDA(rmw::dmalloc_async(&buf, bytes, st));
    char *p = (char *)buf;
    float *node = (float *)p;
    p += al(sizeof(float) * 2 * nb);
    int *mp_dst = (int *)p;
    p += al(sizeof(int) * std::max(nm, 1));
    float *mp_feat = (float *)p;
    p += al(sizeof(float) * 3 * std::max(nm, 1));
    int *band_i = (int *)p;
    p += al(sizeof(int) * np);
    float *band_feat = (float *)p;
    const unsigned gb = (unsigned)((nb + 127) / 128);
    node_raw_features_kernel<<<gb, 128, 0, st>>>(S.xb, S.nf_mp_off, nb, invR, node);
    if (nm > 0) {
        csr_owner_kernel<<<gb, 128, 0, st>>>(S.nf_mp_off, nb, mp_dst);
        edge_raw_features_kernel<<<(unsigned)((nm + 127) / 128), 128, 0, st>>>(S.xb, mp_dst, S.nf_mp_idx, nm, invR, P,
                                                                              mp_feat);
    }
    csr_owner_kernel<<<gb, 128, 0, st>>>(S.nf_ln_off, nb, band_i);
    edge_raw_features_kernel<<<(unsigned)((np + 127) / 128), 128, 0, st>>>(S.xb, band_i, S.nf_ln_idx, np, invR, P,
                                                                          band_feat);
    RMW_CHECK_LAUNCH("near-field graph");
    MpGraph g;
    g.n_nodes = nb;
    g.n_mp = nm;
    g.n_band = np;
    g.node_feat = node;
    g.mp_src = S.nf_mp_idx;
    g.mp_dst = mp_dst;
    g.mp_off = S.nf_mp_off;
    g.mp_feat = mp_feat;
    g.band_i = band_i;
    g.band_j = S.nf_ln_idx;
    g.band_off = S.nf_ln_off;
    g.band_feat = band_feat;
    MpWork *W = nullptr;
    int rc = mp_work_create(&W, nb, nm, np, st);
    if (rc == RMW_OK) rc = mp_forward(N, g, *W, st);
    if (rc == RMW_OK) {
        pair_blocks_kernel<<<(unsigned)(((long long)np * kModes + 127) / 128), 128, 0, st>>>(
            mp_outputs(*W), S.xb, S.nf_ln_off, S.nf_ln_idx, nb, np, P, N.dnorm + 2 * kNodeFeat + 2 * kEdgeFeat,
            S.nf_G);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) rc = cuda_fail(e, "near-field coupling blocks");
    }
    mp_work_destroy(W);
    cudaFreeAsync(buf, st);
    return rc;
}

}  // namespace rmw

// ---------------------------------------------------------------------------
// C ABI
using rmw::MpnnNet;
using rmw::RigidSystem;

extern "C" {

int rmw_rigid_pair_coupling(void *sys, double *out)
{
    if (!sys || !out) return rmw::fail(RMW_ERR_ARG, "null argument");
    RigidSystem &S = *(RigidSystem *)sys;
    if (!S.pc_ready) return rmw::fail(RMW_ERR_ARG, "build the preconditioner first (it forms each body's M^-1)");
    if (S.nb % 2) return rmw::fail(RMW_ERR_ARG, "two-body samples need an even body count");
    const int nt = 128;
    const size_t sm = sizeof(double) * (4 * (size_t)S.max_m * rmw::kModes + 3 * rmw::kModes * rmw::kModes +
                                        2 * rmw::kModes * rmw::kModes);
    if (sm > 227 * 1024) return rmw::fail(RMW_ERR_ARG, "bodies too large for the two-body coupling kernel");
    if (sm > 48 * 1024)
        RMW_CUDA(cudaFuncSetAttribute(rmw::pair_fts_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    RMW_CUDA(cudaMemsetAsync(S.dstatus, 0, sizeof(int), S.st));
    const double nf = 1.0 / (8.0 * rmw::kPi * S.eta * S.a);
    rmw::pair_fts_kernel<<<S.nb / 2, nt, sm, S.st>>>(S.r, S.xb, S.boff, S.moff, S.minv, S.a, nf,
                                                      rmw::Images{S.L[0], S.L[1], S.L[2]}, S.max_m, out, S.dstatus);
    RMW_CHECK_LAUNCH("two-body mode coupling");
    int h = 0;
    RMW_CUDA(cudaMemcpyAsync(&h, S.dstatus, sizeof(int), cudaMemcpyDeviceToHost, S.st));
    RMW_CUDA(cudaStreamSynchronize(S.st));
    if (h) return rmw::fail(RMW_ERR_NONFINITE, "singular mode Gram matrix");
    return RMW_OK;
}

int rmw_rigid_pair_coupling_list(void *sys, const int *pairs, int64_t n_pairs, double *out)
{
    if (!sys || !pairs || !out) return rmw::fail(RMW_ERR_ARG, "null argument");
    RigidSystem &S = *(RigidSystem *)sys;
    if (!S.pc_ready) return rmw::fail(RMW_ERR_ARG, "build the preconditioner first (it forms each body's M^-1)");
    if (n_pairs <= 0) return RMW_OK;
    if (n_pairs > (int64_t(1) << 30)) return rmw::fail(RMW_ERR_ARG, "too many pairs");
    std::vector<int> hp((size_t)2 * n_pairs);
    RMW_CUDA(cudaMemcpyAsync(hp.data(), pairs, sizeof(int) * hp.size(), cudaMemcpyDeviceToHost, S.st));
    RMW_CUDA(cudaStreamSynchronize(S.st));
    for (size_t k = 0; k < hp.size(); ++k)
        if (hp[k] < 0 || hp[k] >= S.nb) return rmw::fail(RMW_ERR_ARG, "pair index out of range");
    const int nt = 128;
    const size_t sm = sizeof(double) * (4 * (size_t)S.max_m * rmw::kModes + 3 * rmw::kModes * rmw::kModes +
                                        2 * rmw::kModes * rmw::kModes);
    if (sm > 227 * 1024) return rmw::fail(RMW_ERR_ARG, "bodies too large for the coupling kernel");
    if (sm > 48 * 1024)
        RMW_CUDA(cudaFuncSetAttribute(rmw::pair_list_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    RMW_CUDA(cudaMemsetAsync(S.dstatus, 0, sizeof(int), S.st));
    const double nf = 1.0 / (8.0 * rmw::kPi * S.eta * S.a);
    rmw::pair_list_kernel<<<(unsigned)n_pairs, nt, sm, S.st>>>(S.r, S.xb, S.boff, S.moff, S.minv, pairs, S.a, nf,
                                                               rmw::Images{S.L[0], S.L[1], S.L[2]}, S.max_m, out,
                                                               S.dstatus);
    RMW_CHECK_LAUNCH("mode coupling of listed pairs");
    int h = 0;
    RMW_CUDA(cudaMemcpyAsync(&h, S.dstatus, sizeof(int), cudaMemcpyDeviceToHost, S.st));
    RMW_CUDA(cudaStreamSynchronize(S.st));
    if (h) return rmw::fail(RMW_ERR_NONFINITE, "singular mode Gram matrix");
    return RMW_OK;
}

// Switch a handle's preconditioner (after rmw_rigid_build_pc) to the
// near-field augmented form: exact blob-level couplings for body pairs closer
// than exact_cutoff, network-predicted mode couplings for pairs from
// max(exact_cutoff, learned_from) to the network's cutoff (net may be NULL:
// exact pairs only).  Pairs are found within one suspension.  net == NULL and
// exact_cutoff <= 0 switch back to the block-diagonal form.  n_pairs_host
// (optional, 2 entries) receives the numbers of ordered exact and learned
// pairs.
int rmw_rigid_set_nearfield_bands(void *sys, void *net, double exact_cutoff, double learned_from,
                                  int64_t *n_pairs_host)
{
    if (!sys) return rmw::fail(RMW_ERR_ARG, "null handle");
    RigidSystem &S = *(RigidSystem *)sys;
    if (n_pairs_host) n_pairs_host[0] = n_pairs_host[1] = 0;
    const double lo = exact_cutoff > 0 ? exact_cutoff : 0.0;
    if (!net && !(lo > 0)) {
        S.nf_on = false;
        return RMW_OK;
    }
    if (!S.pc_ready) return rmw::fail(RMW_ERR_ARG, "build the preconditioner first");
    if (!S.wall) return rmw::fail(RMW_ERR_ARG, "the near-field preconditioner models bodies above the wall");
    MpnnNet *N = (MpnnNet *)net;
    const double hi = N ? std::max(N->cutoff, lo) : lo;
    const double lf = N ? std::max(learned_from, 0.0) : hi;
    const double mp = N ? N->mp_cutoff : 0.0;
    cudaStream_t st = S.st;
    S.nf_on = false;
    if (int rc = rmw::build_bands(S, lo, lf, hi, mp)) return rc;
    if (!S.nf_mom) RMW_CUDA(cudaMalloc(&S.nf_mom, sizeof(double) * rmw::kModes * S.nb));
    if (!S.nf_mom32) RMW_CUDA(cudaMalloc(&S.nf_mom32, sizeof(float) * rmw::kModes * S.nb));
    if (!S.nf_lam32) RMW_CUDA(cudaMalloc(&S.nf_lam32, sizeof(float) * 3 * (size_t)S.n));
    if (!S.nf_v) {
        RMW_CUDA(cudaMalloc(&S.nf_v, sizeof(double) * S.sys_size()));
        RMW_CUDA(cudaMemset(S.nf_v, 0, sizeof(double) * S.sys_size()));  // force rows stay zero
    }
    if (!S.nf_z) RMW_CUDA(cudaMalloc(&S.nf_z, sizeof(double) * S.sys_size()));
    if (N && S.nf_ln_pairs > 0) {
        if (int rc = rmw::learned_couplings(S, *N)) return rc;
        rmw::to_f32(S.nf_G, S.nf_G32, 121LL * S.nf_ln_pairs, st);  // the mixed solves' FP32 apply
    }
    if (!N) S.nf_ln_pairs = 0;
    RMW_CHECK_LAUNCH("near-field attach");
    RMW_CUDA(cudaStreamSynchronize(st));
    S.nf_on = true;
    if (n_pairs_host) {
        n_pairs_host[0] = S.nf_ex_pairs;
        n_pairs_host[1] = S.nf_ln_pairs;
    }
    return RMW_OK;
}

int rmw_rigid_set_nearfield(void *sys, void *net, double exact_cutoff, int64_t *n_pairs_host)
{
    return rmw_rigid_set_nearfield_bands(sys, net, exact_cutoff, 0.0, n_pairs_host);
}

}  // extern "C"
