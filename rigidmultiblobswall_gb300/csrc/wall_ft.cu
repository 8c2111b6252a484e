// Fused force-and-torque wall product:
//
//   U = M_UF F + M_UT T,    W = M_WF F + M_WT T     (W optional)
//
// in one pass over the pairs.  The reference's pycuda kernel
// velocity_from_force_and_torque (mobility/mobility_pycuda.py:1266-1392,
// wrapper mobility/mobility.py:384-411) returns U only; the 6N product
// [U; W] is what Lub_Solver.Wall_Mobility_Mult (Lubrication/Lub_Solver.py:
// 277-305) and the rollers' GMRES assemble from four separate products.  Here
// the four pair blocks are evaluated back to back on the same pair inputs:
// the pair functions are inlined, so the distances, the two reciprocal square
// roots and the powers of 1/R they share are formed once per pair.
//
// Scaling: with F' = b F and T' = b T / a (b the wall damping), and nf =
// 1/(8 pi eta a),
//   U_i = b_i nf       [ sum_j M_UF F'_j + M_UT T'_j + self(F'_i, T'_i) ]
//   W_i = b_i nf / a   [ sum_j M_WF F'_j + M_WT T'_j + self(F'_i, T'_i) ]
// because the four blocks carry 1/(8 pi eta a^p) with p = 1, 2, 2, 3.
//
// Same structure as the single products (wall_pair.cu): pack -> pair kernel
// over (target tiles) x (source chunks) -> finalize summing the chunks in
// fixed order (deterministic), adding the self terms and the scale.
// Precision modes as there: FP64; df64 (double-float on the FP32 pipe,
// <= 1e-12 against FP64); mixed (FP32 pairs from double-float position
// differences, compensated sums, <= 1e-6).
#include <algorithm>

#include "pair_math.cuh"
#include "pair_math_df.cuh"
#include "rmw_common.cuh"
#include "wall_pair.cuh"

namespace rmw {

namespace {

constexpr int kFtThreads = 128;  // targets per CTA
constexpr int kFtTile = 64;      // sources per shared-memory tile
constexpr int kFtDfGroup = 32;   // df64: sources per double-float group sum

struct FtImages {
    double Lx, Ly, Lz;  // periodic lengths over a (0 = not periodic)
};

// source records: positions over a (z clamped at a), F' and T'
struct __align__(16) FtSrcD {
    double x, y, z, pad0;
    double fx, fy, fz, pad1;
    double tx, ty, tz, pad2;
};
struct __align__(16) FtSrcF {
    float4 hi, lo;  // double-float positions over a
    float4 f, t;    // F', T' in FP32
};
struct __align__(16) FtSrcDF {
    float4 hi, lo;    // positions over a
    float4 fhi, flo;  // F'
    float4 thi, tlo;  // T'
};

__device__ __forceinline__ void ft_prep(const double *r, const double *F, const double *T, int i, double a,
                                        double &x, double &y, double &z, double f[3], double t[3])
{
    const double inva = 1.0 / a;
    const double zz = r[3 * i + 2];
    const double b = (zz < a) ? zz / a : 1.0;
    const double ze = (zz <= a) ? a : zz;
    x = r[3 * i] * inva;
    y = r[3 * i + 1] * inva;
    z = ze * inva;
    for (int c = 0; c < 3; ++c) {
        f[c] = b * F[3 * i + c];
        t[c] = b * T[3 * i + c] * inva;
    }
}

__global__ void ft_pack_fp64_kernel(const double *__restrict__ r, const double *__restrict__ F,
                                    const double *__restrict__ T, FtSrcD *__restrict__ src, int n, double a)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double x, y, z, f[3], t[3];
    ft_prep(r, F, T, i, a, x, y, z, f, t);
    FtSrcD s;
    s.x = x; s.y = y; s.z = z; s.pad0 = 0.0;
    s.fx = f[0]; s.fy = f[1]; s.fz = f[2]; s.pad1 = 0.0;
    s.tx = t[0]; s.ty = t[1]; s.tz = t[2]; s.pad2 = 0.0;
    src[i] = s;
}

__global__ void ft_pack_mixed_kernel(const double *__restrict__ r, const double *__restrict__ F,
                                     const double *__restrict__ T, FtSrcF *__restrict__ src, int n, double a)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double x, y, z, f[3], t[3];
    ft_prep(r, F, T, i, a, x, y, z, f, t);
    const float xh = (float)x, yh = (float)y, zh = (float)z;
    FtSrcF s;
    s.hi = make_float4(xh, yh, zh, 0.f);
    s.lo = make_float4((float)(x - (double)xh), (float)(y - (double)yh), (float)(z - (double)zh), 0.f);
    s.f = make_float4((float)f[0], (float)f[1], (float)f[2], 0.f);
    s.t = make_float4((float)t[0], (float)t[1], (float)t[2], 0.f);
    src[i] = s;
}

__global__ void ft_pack_df_kernel(const double *__restrict__ r, const double *__restrict__ F,
                                  const double *__restrict__ T, FtSrcDF *__restrict__ src, int n, double a)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double x, y, z, f[3], t[3];
    ft_prep(r, F, T, i, a, x, y, z, f, t);
    const df X = df_of_double(x), Y = df_of_double(y), Z = df_of_double(z);
    const df f0 = df_of_double(f[0]), f1 = df_of_double(f[1]), f2 = df_of_double(f[2]);
    const df t0 = df_of_double(t[0]), t1 = df_of_double(t[1]), t2 = df_of_double(t[2]);
    FtSrcDF s;
    s.hi = make_float4(X.hi, Y.hi, Z.hi, 0.f);
    s.lo = make_float4(X.lo, Y.lo, Z.lo, 0.f);
    s.fhi = make_float4(f0.hi, f1.hi, f2.hi, 0.f);
    s.flo = make_float4(f0.lo, f1.lo, f2.lo, 0.f);
    s.thi = make_float4(t0.hi, t1.hi, t2.hi, 0.f);
    s.tlo = make_float4(t0.lo, t1.lo, t2.lo, 0.f);
    src[i] = s;
}

// the periodic images the single products use: minimum image, then the
// neighbouring boxes along every periodic direction
template <typename T, typename F>
__device__ __forceinline__ void for_images(T rx, T ry, T rz, T Lx, T Ly, T Lz, bool self_pair, F &&f)
{
    if (Lx > T(0)) rx = project(rx, Lx);
    if (Ly > T(0)) ry = project(ry, Ly);
    if (Lz > T(0)) rz = project(rz, Lz);
    const int px = Lx > T(0), py = Ly > T(0), pz = Lz > T(0);
    for (int bx = -px; bx <= px; ++bx)
        for (int by = -py; by <= py; ++by)
            for (int bz = -pz; bz <= pz; ++bz) {
                const bool self = self_pair && bx == 0 && by == 0 && bz == 0;
                if (!self) f(rx + bx * Lx, ry + by * Ly, rz + bz * Lz);
            }
}

// ---------------------------------------------------------------------------
// FP64
template <bool WITH_W, bool PER>
__global__ void __launch_bounds__(kFtThreads) ft_pair_fp64_kernel(const FtSrcD *__restrict__ src, int n, int chunk,
                                                                   FtImages P, double *__restrict__ partial)
{
    __shared__ FtSrcD tile[kFtTile];
    const int i = blockIdx.x * kFtThreads + threadIdx.x;
    const bool valid = i < n;
    const int j0 = blockIdx.y * chunk, j1 = min(n, j0 + chunk);
    FtSrcD me;
    if (valid) me = src[i];
    else { me.x = 0.0; me.y = 0.0; me.z = 1.0e6; }
    double u[3] = {0.0, 0.0, 0.0}, w[3] = {0.0, 0.0, 0.0};
    for (int t0 = j0; t0 < j1; t0 += kFtTile) {
        const int cnt = min(kFtTile, j1 - t0);
        __syncthreads();
        for (int k = threadIdx.x; k < cnt; k += kFtThreads) tile[k] = src[t0 + k];
        __syncthreads();
        for (int k = 0; k < cnt; ++k) {
            const FtSrcD s = tile[k];
            const int j = t0 + k;
            const double Rz = me.z + s.z;
            auto add = [&](double dx, double dy, double dz) {
                double cu[3] = {0.0, 0.0, 0.0}, cw[3] = {0.0, 0.0, 0.0};
                pair_contrib<RMW_UF, double>(dx, dy, dz, Rz, me.z, s.z, s.fx, s.fy, s.fz, cu[0], cu[1], cu[2]);
                pair_contrib<RMW_UT, double>(dx, dy, dz, Rz, me.z, s.z, s.tx, s.ty, s.tz, cu[0], cu[1], cu[2]);
                if (WITH_W) {
                    pair_contrib<RMW_WF, double>(dx, dy, dz, Rz, me.z, s.z, s.fx, s.fy, s.fz, cw[0], cw[1], cw[2]);
                    pair_contrib<RMW_WT, double>(dx, dy, dz, Rz, me.z, s.z, s.tx, s.ty, s.tz, cw[0], cw[1], cw[2]);
                }
                for (int c = 0; c < 3; ++c) {
                    u[c] += cu[c];
                    w[c] += cw[c];
                }
            };
            const double dx = me.x - s.x, dy = me.y - s.y, dz = me.z - s.z;
            if (!PER) {
                // the self pair is evaluated (coincident points, finite near-field
                // branch) and discarded, so the warp stays convergent
                double cu[3] = {0.0, 0.0, 0.0}, cw[3] = {0.0, 0.0, 0.0};
                pair_contrib<RMW_UF, double>(dx, dy, dz, Rz, me.z, s.z, s.fx, s.fy, s.fz, cu[0], cu[1], cu[2]);
                pair_contrib<RMW_UT, double>(dx, dy, dz, Rz, me.z, s.z, s.tx, s.ty, s.tz, cu[0], cu[1], cu[2]);
                if (WITH_W) {
                    pair_contrib<RMW_WF, double>(dx, dy, dz, Rz, me.z, s.z, s.fx, s.fy, s.fz, cw[0], cw[1], cw[2]);
                    pair_contrib<RMW_WT, double>(dx, dy, dz, Rz, me.z, s.z, s.tx, s.ty, s.tz, cw[0], cw[1], cw[2]);
                }
                if (j != i)
                    for (int c = 0; c < 3; ++c) {
                        u[c] += cu[c];
                        w[c] += cw[c];
                    }
            } else {
                for_images(dx, dy, dz, P.Lx, P.Ly, P.Lz, j == i, add);
            }
        }
    }
    if (valid) {
        double *o = partial + (size_t)blockIdx.y * 6 * n;
        for (int c = 0; c < 3; ++c) {
            o[3 * (size_t)i + c] = u[c];
            o[3 * (size_t)n + 3 * (size_t)i + c] = w[c];
        }
    }
}

// ---------------------------------------------------------------------------
// mixed: FP32 pairs from double-float position differences; the FP32 sum over
// each tile is folded into TwoSum-compensated accumulators
template <bool WITH_W, bool PER>
__global__ void __launch_bounds__(kFtThreads) ft_pair_mixed_kernel(const FtSrcF *__restrict__ src, int n, int chunk,
                                                                    FtImages P, double *__restrict__ partial)
{
    __shared__ FtSrcF tile[kFtTile];
    const int i = blockIdx.x * kFtThreads + threadIdx.x;
    const bool valid = i < n;
    const int j0 = blockIdx.y * chunk, j1 = min(n, j0 + chunk);
    float4 mh = make_float4(0.f, 0.f, 1.0e6f, 0.f), ml = make_float4(0.f, 0.f, 0.f, 0.f);
    if (valid) { mh = src[i].hi; ml = src[i].lo; }
    const float hi = mh.z + ml.z;
    const float Lx = (float)P.Lx, Ly = (float)P.Ly, Lz = (float)P.Lz;
    float sh_[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f}, sl_[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (int t0 = j0; t0 < j1; t0 += kFtTile) {
        const int cnt = min(kFtTile, j1 - t0);
        __syncthreads();
        for (int k = threadIdx.x; k < cnt; k += kFtThreads) tile[k] = src[t0 + k];
        __syncthreads();
        float acc[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        for (int k = 0; k < cnt; ++k) {
            const float4 sh = tile[k].hi, sl = tile[k].lo, sf = tile[k].f, st = tile[k].t;
            const int j = t0 + k;
            const float dx = (mh.x - sh.x) + (ml.x - sl.x);
            const float dy = (mh.y - sh.y) + (ml.y - sl.y);
            const float dz = (mh.z - sh.z) + (ml.z - sl.z);
            const float hj = sh.z + sl.z;
            const float Rz = hi + hj;
            auto add = [&](float ex, float ey, float ez, float *o) {
                pair_contrib<RMW_UF, float>(ex, ey, ez, Rz, hi, hj, sf.x, sf.y, sf.z, o[0], o[1], o[2]);
                pair_contrib<RMW_UT, float>(ex, ey, ez, Rz, hi, hj, st.x, st.y, st.z, o[0], o[1], o[2]);
                if (WITH_W) {
                    pair_contrib<RMW_WF, float>(ex, ey, ez, Rz, hi, hj, sf.x, sf.y, sf.z, o[3], o[4], o[5]);
                    pair_contrib<RMW_WT, float>(ex, ey, ez, Rz, hi, hj, st.x, st.y, st.z, o[3], o[4], o[5]);
                }
            };
            if (!PER) {
                float c[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
                add(dx, dy, dz, c);
                if (j != i)
                    for (int q = 0; q < 6; ++q) acc[q] += c[q];
            } else {
                for_images(dx, dy, dz, Lx, Ly, Lz, j == i, [&](float ex, float ey, float ez) { add(ex, ey, ez, acc); });
            }
        }
        for (int q = 0; q < 6; ++q) comp_add(sh_[q], sl_[q], acc[q]);
    }
    if (valid) {
        double *o = partial + (size_t)blockIdx.y * 6 * n;
        for (int c = 0; c < 3; ++c) {
            o[3 * (size_t)i + c] = (double)sh_[c] + (double)sl_[c];
            o[3 * (size_t)n + 3 * (size_t)i + c] = (double)sh_[3 + c] + (double)sl_[3 + c];
        }
    }
}

// ---------------------------------------------------------------------------
// df64: double-float pairs on the FP32 pipe; each group of kFtDfGroup sources
// is summed in double-float and folded into FP64 accumulators
template <bool WITH_W, bool PER>
__global__ void __launch_bounds__(kFtThreads) ft_pair_df_kernel(const FtSrcDF *__restrict__ src, int n, int chunk,
                                                                 FtImages P, double *__restrict__ partial)
{
    __shared__ FtSrcDF tile[kFtTile];
    const int i = blockIdx.x * kFtThreads + threadIdx.x;
    const bool valid = i < n;
    const int j0 = blockIdx.y * chunk, j1 = min(n, j0 + chunk);
    float4 mh = make_float4(0.f, 0.f, 1.0e6f, 0.f), ml = make_float4(0.f, 0.f, 0.f, 0.f);
    if (valid) { mh = src[i].hi; ml = src[i].lo; }
    const df xi = {mh.x, ml.x}, yi = {mh.y, ml.y}, zi = {mh.z, ml.z};
    double acc[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (int t0 = j0; t0 < j1; t0 += kFtTile) {
        const int cnt = min(kFtTile, j1 - t0);
        __syncthreads();
        for (int k = threadIdx.x; k < cnt; k += kFtThreads) tile[k] = src[t0 + k];
        __syncthreads();
        for (int g0 = 0; g0 < cnt; g0 += kFtDfGroup) {
            const int g1 = min(cnt, g0 + kFtDfGroup);
            df gs[6] = {df_from(0.f), df_from(0.f), df_from(0.f), df_from(0.f), df_from(0.f), df_from(0.f)};
            for (int k = g0; k < g1; ++k) {
                const FtSrcDF s = tile[k];
                const int j = t0 + k;
                const df xj = {s.hi.x, s.lo.x}, yj = {s.hi.y, s.lo.y}, zj = {s.hi.z, s.lo.z};
                const df fx = {s.fhi.x, s.flo.x}, fy = {s.fhi.y, s.flo.y}, fz = {s.fhi.z, s.flo.z};
                const df tx = {s.thi.x, s.tlo.x}, ty = {s.thi.y, s.tlo.y}, tz = {s.thi.z, s.tlo.z};
                const df Rz = zi + zj;
                auto add = [&](df ex, df ey, df ez) {
                    df a0, a1, a2, b0, b1, b2;
                    pair_contrib_df<RMW_UF>(ex, ey, ez, Rz, zi, zj, fx, fy, fz, a0, a1, a2);
                    pair_contrib_df<RMW_UT>(ex, ey, ez, Rz, zi, zj, tx, ty, tz, b0, b1, b2);
                    acc_add(gs[0], a0 + b0);
                    acc_add(gs[1], a1 + b1);
                    acc_add(gs[2], a2 + b2);
                    if (WITH_W) {
                        pair_contrib_df<RMW_WF>(ex, ey, ez, Rz, zi, zj, fx, fy, fz, a0, a1, a2);
                        pair_contrib_df<RMW_WT>(ex, ey, ez, Rz, zi, zj, tx, ty, tz, b0, b1, b2);
                        acc_add(gs[3], a0 + b0);
                        acc_add(gs[4], a1 + b1);
                        acc_add(gs[5], a2 + b2);
                    }
                };
                if (!PER) {
                    if (j != i) {
                        add(xi - xj, yi - yj, zi - zj);
                    } else {
                        // evaluate and discard the self pair so the warp stays convergent
                        df g2[6];
                        for (int q = 0; q < 6; ++q) g2[q] = gs[q];
                        add(xi - xj, yi - yj, zi - zj);
                        for (int q = 0; q < 6; ++q) gs[q] = g2[q];
                    }
                } else {
                    // minimum image in FP64 (rare path), then back to double-float
                    for_images(to_double(xi - xj), to_double(yi - yj), to_double(zi - zj), P.Lx, P.Ly, P.Lz, j == i,
                               [&](double ex, double ey, double ez) {
                                   add(df_of_double(ex), df_of_double(ey), df_of_double(ez));
                               });
                }
            }
            for (int q = 0; q < 6; ++q) acc[q] += to_double(gs[q]);
        }
    }
    if (valid) {
        double *o = partial + (size_t)blockIdx.y * 6 * n;
        for (int c = 0; c < 3; ++c) {
            o[3 * (size_t)i + c] = acc[c];
            o[3 * (size_t)n + 3 * (size_t)i + c] = acc[3 + c];
        }
    }
}

// ---------------------------------------------------------------------------
// finalize: fixed-order chunk sum, FP64 self terms of the four blocks
// (mobility/mobility_numba.py self terms), b_i and the scales
__global__ void ft_finalize_kernel(const double *__restrict__ r, const double *__restrict__ F,
                                   const double *__restrict__ T, const double *__restrict__ partial, int nchunks,
                                   double *__restrict__ U, double *__restrict__ W, int n, double a, double nf)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double u[3] = {0.0, 0.0, 0.0}, w[3] = {0.0, 0.0, 0.0};
    for (int s = 0; s < nchunks; ++s) {
        const double *p = partial + (size_t)s * 6 * n;
        for (int c = 0; c < 3; ++c) {
            u[c] += p[3 * (size_t)i + c];
            w[c] += p[3 * (size_t)n + 3 * (size_t)i + c];
        }
    }
    const double z = r[3 * i + 2];
    const double b = (z < a) ? z / a : 1.0;
    const double ze = (z <= a) ? a : z;
    const double fx = b * F[3 * i], fy = b * F[3 * i + 1], fz = b * F[3 * i + 2];
    const double tx = b * T[3 * i] / a, ty = b * T[3 * i + 1] / a, tz = b * T[3 * i + 2] / a;
    const double iz = a / ze, iz3 = iz * iz * iz, iz5 = iz3 * iz * iz;
    const double mxx = 4.0 / 3.0 - (9.0 * iz - 2.0 * iz3 + iz5) / 12.0;
    const double mzz = 4.0 / 3.0 - (9.0 * iz - 4.0 * iz3 + iz5) / 6.0;
    const double sr = 0.125 * iz3 * iz;  // rotation-translation coupling 1/(8 h^4)
    u[0] += mxx * fx + sr * ty;
    u[1] += mxx * fy - sr * tx;
    u[2] += mzz * fz;
    U[3 * i] = b * nf * u[0];
    U[3 * i + 1] = b * nf * u[1];
    U[3 * i + 2] = b * nf * u[2];
    if (W) {
        w[0] += -sr * fy + (1.0 - 0.3125 * iz3) * tx;
        w[1] += sr * fx + (1.0 - 0.3125 * iz3) * ty;
        w[2] += (1.0 - 0.125 * iz3) * tz;
        const double sw = b * nf / a;
        W[3 * i] = sw * w[0];
        W[3 * i + 1] = sw * w[1];
        W[3 * i + 2] = sw * w[2];
    }
}

// ---------------------------------------------------------------------------
// Symmetric mixed-precision force-torque kernel: the grid and pairing of the
// symmetric single products (one CTA per tile pair T <= S of the upper
// triangle; lane l meets source (l + k) mod 128 at step k; per-warp source
// sums in shared memory), all four blocks per unordered pair, applied to both
// blobs: u_i += UF_ij f_j + UT_ij t_j, w_i += WF_ij f_j + WT_ij t_j and the
// same with i and j exchanged (M_ji = M_ij^T: UF through its transposed
// coefficients, the rotation blocks through pair_rot_sym).  The UF
// coefficients come times 3/2 and are scaled back per pair, so U and W keep
// the one-sided kernels' sums and finalize.  Partial slots: blob b of tile X
// gets one slot per tile, U at slot * 6n + 3b and W at slot * 6n + 3n + 3b.
constexpr int kFtSymWarps = 4;
constexpr int kFtSymTile = 32 * kFtSymWarps;

template <bool WITH_W>
__global__ void __launch_bounds__(kFtSymTile) ft_sym_mixed_kernel(const FtSrcF *__restrict__ src, int n, int nt,
                                                                  double *__restrict__ partial)
{
    __shared__ float4 thi[kFtSymTile], tlo[kFtSymTile], tf[kFtSymTile], tt[kFtSymTile];
    __shared__ float sacc[kFtSymWarps][6][kFtSymTile];
    int T, S;
    sym_tile_pair(blockIdx.x, nt, T, S);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const bool diag = (T == S);
    const int i = T * kFtSymTile + tid;
    const bool valid_i = i < n;
    // a target or source past the end is a dummy far above the wall with zero vectors
    const FtSrcF dummy = {make_float4(1.0e6f, 1.0e6f, 1.0e6f, 0.f), make_float4(0.f, 0.f, 0.f, 0.f),
                          make_float4(0.f, 0.f, 0.f, 0.f), make_float4(0.f, 0.f, 0.f, 0.f)};
    const FtSrcF me = valid_i ? src[i] : dummy;
    const float hi = me.hi.z + me.lo.z;
    {
        const int j = S * kFtSymTile + tid;
        const FtSrcF sj = (j < n) ? src[j] : dummy;
        thi[tid] = sj.hi;
        tlo[tid] = sj.lo;
        tf[tid] = sj.f;
        tt[tid] = sj.t;
    }
    for (int c = 0; c < 6; ++c)
        for (int k = lane; k < kFtSymTile; k += 32) sacc[warp][c][k] = 0.f;
    __syncthreads();
    float u0 = 0.f, u1 = 0.f, u2 = 0.f, w0 = 0.f, w1 = 0.f, w2 = 0.f;
    constexpr float kThird2 = 2.0f / 3.0f;  // undoes the UF coefficients' 3/2
    auto step = [&](int k) {
        const int jl = (lane + k) & (kFtSymTile - 1);
        const float4 sh = thi[jl], sl = tlo[jl], sf = tf[jl], st = tt[jl];
        const float dx = (me.hi.x - sh.x) + (me.lo.x - sl.x);
        const float dy = (me.hi.y - sh.y) + (me.lo.y - sl.y);
        const float dz = (me.hi.z - sh.z) + (me.lo.z - sl.z);
        const float hj = sh.z + sl.z;
        const float Rz = hi + hj;
        float a0 = sacc[warp][0][jl], a1 = sacc[warp][1][jl], a2 = sacc[warp][2][jl];
        UFCoeffs<float> c = uf_coeffs<float>(dx, dy, dz, Rz, hi, hj);
        c.Af *= kThird2; c.Bc *= kThird2; c.c2 *= kThird2; c.c3 *= kThird2; c.c4 *= kThird2; c.Af5 *= kThird2;
        uf_apply<float>(c, dx, dy, dz, Rz, sf.x, sf.y, sf.z, u0, u1, u2);
        const UFCoeffs<float> ct = {c.Af, c.Bc, c.c2, c.c4, c.c3, c.Af5};  // M^T: f3 and f4 trade places
        uf_apply<float>(ct, dx, dy, dz, Rz, me.f.x, me.f.y, me.f.z, a0, a1, a2);
        pair_rot_sym<float, RMW_UT>(dx, dy, dz, Rz, hi, hj, st.x, st.y, st.z, me.t.x, me.t.y, me.t.z, u0, u1, u2, a0,
                                    a1, a2);
        sacc[warp][0][jl] = a0;
        sacc[warp][1][jl] = a1;
        sacc[warp][2][jl] = a2;
        if (WITH_W) {
            float b0 = sacc[warp][3][jl], b1 = sacc[warp][4][jl], b2 = sacc[warp][5][jl];
            pair_rot_sym<float, RMW_WF>(dx, dy, dz, Rz, hi, hj, sf.x, sf.y, sf.z, me.f.x, me.f.y, me.f.z, w0, w1, w2,
                                        b0, b1, b2);
            pair_rot_sym<float, RMW_WT>(dx, dy, dz, Rz, hi, hj, st.x, st.y, st.z, me.t.x, me.t.y, me.t.z, w0, w1, w2,
                                        b0, b1, b2);
            sacc[warp][3][jl] = b0;
            sacc[warp][4][jl] = b1;
            sacc[warp][5][jl] = b2;
        }
    };
    if (diag) {
        for (int k = 0; k < kFtSymTile; ++k) {
            __syncwarp();
            const int off = (k - 32 * warp) & (kFtSymTile - 1);  // (source - target) mod 128, warp-uniform
            if (off == 0 || off > kFtSymTile / 2 || (off == kFtSymTile / 2 && warp >= kFtSymWarps / 2)) continue;
            step(k);
        }
    } else {
        for (int k = 0; k < kFtSymTile; ++k) {
            __syncwarp();
            step(k);
        }
    }
    __syncthreads();
    double q[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (int w = 0; w < kFtSymWarps; ++w)
        for (int c = 0; c < (WITH_W ? 6 : 3); ++c) q[c] += (double)sacc[w][c][tid];
    const double tu[6] = {u0, u1, u2, w0, w1, w2};
    const size_t stride = 6 * (size_t)n;
    if (diag) {
        if (valid_i) {
            double *o = partial + (size_t)T * stride;
            for (int c = 0; c < 3; ++c) {
                o[3 * (size_t)i + c] = tu[c] + q[c];
                o[3 * (size_t)n + 3 * (size_t)i + c] = tu[3 + c] + q[3 + c];
            }
        }
    } else {
        if (valid_i) {
            double *o = partial + (size_t)S * stride;
            for (int c = 0; c < 3; ++c) {
                o[3 * (size_t)i + c] = tu[c];
                o[3 * (size_t)n + 3 * (size_t)i + c] = tu[3 + c];
            }
        }
        const int j = S * kFtSymTile + tid;
        if (j < n) {
            double *o = partial + (size_t)T * stride;
            for (int c = 0; c < 3; ++c) {
                o[3 * (size_t)j + c] = q[c];
                o[3 * (size_t)n + 3 * (size_t)j + c] = q[3 + c];
            }
        }
    }
}

__global__ void ft_add_kernel(const double *__restrict__ x, double *__restrict__ y, long long m)
{
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < m) y[k] += x[k];
}

// U (and W) as sums of single products, each through the symmetric kernel
// (every unordered pair once per block): in FP64 and df64 faster than the
// fused one-sided pass wherever the symmetric kernels apply.
int ft_by_symmetric_products(const double *r, const double *F, const double *T, double *U, double *W, int n,
                             double eta, double a, int mode, cudaStream_t st)
{
    void *tmp = nullptr;
    if (int rc = scratch(SCRATCH_FT_TERM, sizeof(double) * 3 * (size_t)n, &tmp, st)) return rc;
    double *t = (double *)tmp;
    const unsigned g = (unsigned)((3LL * n + 255) / 256);
    if (int rc = wall_product(RMW_UF, r, F, U, n, eta, a, nullptr, mode, st)) return rc;
    if (int rc = wall_product(RMW_UT, r, T, t, n, eta, a, nullptr, mode, st)) return rc;
    ft_add_kernel<<<g, 256, 0, st>>>(t, U, 3LL * n);
    if (W) {
        if (int rc = wall_product(RMW_WF, r, F, W, n, eta, a, nullptr, mode, st)) return rc;
        if (int rc = wall_product(RMW_WT, r, T, t, n, eta, a, nullptr, mode, st)) return rc;
        ft_add_kernel<<<g, 256, 0, st>>>(t, W, 3LL * n);
    }
    RMW_CHECK_LAUNCH("force-torque through symmetric products");
    return RMW_OK;
}

}  // namespace

size_t wall_ft_scratch_bytes(int n, int mode, int nchunks)
{
    const size_t rec = (mode == RMW_MODE_MIXED) ? sizeof(FtSrcF) : (mode == RMW_MODE_DF64 ? sizeof(FtSrcDF)
                                                                                          : sizeof(FtSrcD));
    const size_t packed = ((rec * (size_t)n + 255) / 256) * 256;
    return packed + sizeof(double) * 6 * (size_t)n * (size_t)nchunks;
}

template <bool WITH_W, bool PER>
static void ft_launch(int mode, dim3 grid, cudaStream_t st, void *src, int n, int chunk, FtImages P,
                      double *partial)
{
    if (mode == RMW_MODE_FP64)
        ft_pair_fp64_kernel<WITH_W, PER><<<grid, kFtThreads, 0, st>>>((const FtSrcD *)src, n, chunk, P, partial);
    else if (mode == RMW_MODE_DF64)
        ft_pair_df_kernel<WITH_W, PER><<<grid, kFtThreads, 0, st>>>((const FtSrcDF *)src, n, chunk, P, partial);
    else
        ft_pair_mixed_kernel<WITH_W, PER><<<grid, kFtThreads, 0, st>>>((const FtSrcF *)src, n, chunk, P, partial);
}

int wall_force_torque(const double *r, const double *F, const double *T, double *U, double *W, int64_t n,
                      double eta, double a, const double *L, int mode, cudaStream_t st)
{
    if (int rc = validate_product_args(RMW_UF, r, F, U, n, eta, a, mode)) return rc;
    if (n > 0 && !T) return fail(RMW_ERR_ARG, "null torque array");
    if (n == 0) return RMW_OK;
    const int N = (int)n;
    const bool per = L && (L[0] > 0 || L[1] > 0 || L[2] > 0);
    // mixed: the symmetric fused kernel from 8,192 blobs
    if (!per && mode == RMW_MODE_MIXED && N >= 8192) {
        const int nt = (N + kFtSymTile - 1) / kFtSymTile;
        const size_t packed = ((sizeof(FtSrcF) * (size_t)N + 255) / 256) * 256;
        const size_t part = sizeof(double) * 6 * (size_t)N * (size_t)nt;
        void *ws = nullptr;
        // the partial sums may not fit next to the caller's allocations (or
        // above rmw_set_scratch_limit): then the one-sided pass below, whose
        // scratch is far smaller, does the product
        if (part <= wall_sym_partial_budget() && scratch(SCRATCH_PAIR, packed + part, &ws, st) != RMW_OK) {
            cudaGetLastError();
            ws = nullptr;
        }
        if (ws) {
            double *partial = (double *)((char *)ws + packed);
            const int pb = 256, pg = (N + pb - 1) / pb;
            ft_pack_mixed_kernel<<<pg, pb, 0, st>>>(r, F, T, (FtSrcF *)ws, N, a);
            const unsigned ncta = (unsigned)((long long)nt * (nt + 1) / 2);
            void *tok = nullptr;
            if (int rc = trace_begin(TRACE_PAIR, st, &tok)) return rc;
            if (W) ft_sym_mixed_kernel<true><<<ncta, kFtSymTile, 0, st>>>((const FtSrcF *)ws, N, nt, partial);
            else ft_sym_mixed_kernel<false><<<ncta, kFtSymTile, 0, st>>>((const FtSrcF *)ws, N, nt, partial);
            if (int rc = trace_end(tok, st)) return rc;
            ft_finalize_kernel<<<pg, pb, 0, st>>>(r, F, T, partial, nt, U, W, N, a, 1.0 / (8.0 * kPi * eta * a));
            RMW_CHECK_LAUNCH("symmetric force-torque wall product");
            return RMW_OK;
        }
    }
    // FP64 and df64: the four symmetric products (at 10,752 blobs FP64 39.4 vs
    // 49.5 ms for the one-sided fused pass, df64 5.9 vs 7.6 ms)
    if (!per && (mode == RMW_MODE_FP64 || mode == RMW_MODE_DF64)) {
        bool sym = true;
        for (int kind : {RMW_UF, RMW_UT, RMW_WF, RMW_WT})
            sym = sym && wall_chunks(kind, mode, N) == kSymChunks && wall_sym_applicable(kind, mode, N, nullptr);
        if (sym) return ft_by_symmetric_products(r, F, T, U, W, N, eta, a, mode, st);
    }
    const int nchunks = wall_default_chunks(N);
    void *ws = nullptr;
    if (int rc = scratch(SCRATCH_PAIR, wall_ft_scratch_bytes(N, mode, nchunks), &ws, st)) return rc;
    const size_t rec = (mode == RMW_MODE_MIXED) ? sizeof(FtSrcF) : (mode == RMW_MODE_DF64 ? sizeof(FtSrcDF)
                                                                                          : sizeof(FtSrcD));
    const size_t packed = ((rec * (size_t)N + 255) / 256) * 256;
    double *partial = (double *)((char *)ws + packed);
    const int pb = 256, pg = (N + pb - 1) / pb;
    if (mode == RMW_MODE_FP64) ft_pack_fp64_kernel<<<pg, pb, 0, st>>>(r, F, T, (FtSrcD *)ws, N, a);
    else if (mode == RMW_MODE_DF64) ft_pack_df_kernel<<<pg, pb, 0, st>>>(r, F, T, (FtSrcDF *)ws, N, a);
    else ft_pack_mixed_kernel<<<pg, pb, 0, st>>>(r, F, T, (FtSrcF *)ws, N, a);
    const FtImages P{L ? L[0] / a : 0.0, L ? L[1] / a : 0.0, L ? L[2] / a : 0.0};
    const int chunk = (N + nchunks - 1) / nchunks;
    const dim3 grid((N + kFtThreads - 1) / kFtThreads, nchunks);
    void *tok = nullptr;
    if (int rc = trace_begin(TRACE_PAIR, st, &tok)) return rc;
    if (W) {
        if (per) ft_launch<true, true>(mode, grid, st, ws, N, chunk, P, partial);
        else ft_launch<true, false>(mode, grid, st, ws, N, chunk, P, partial);
    } else {
        if (per) ft_launch<false, true>(mode, grid, st, ws, N, chunk, P, partial);
        else ft_launch<false, false>(mode, grid, st, ws, N, chunk, P, partial);
    }
    if (int rc = trace_end(tok, st)) return rc;
    ft_finalize_kernel<<<pg, pb, 0, st>>>(r, F, T, partial, nchunks, U, W, N, a, 1.0 / (8.0 * kPi * eta * a));
    RMW_CHECK_LAUNCH("force-torque wall product");
    return RMW_OK;
}

}  // namespace rmw

extern "C" {

// U = M_UF F + M_UT T and, if W is not NULL, W = M_WF F + M_WT T, in one pass
// over the pairs (device arrays of 3n doubles; see rmw_gb300.h).
int rmw_wall_force_torque(const double *r, const double *F, const double *T, double *U, double *W, int64_t n,
                          double eta, double a, const double *L_host, int mode, void *stream)
{
    return rmw::wall_force_torque(r, F, T, U, W, n, eta, a, L_host, mode, rmw::as_stream(stream));
}

}  // extern "C"
