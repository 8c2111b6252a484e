// Single-wall Rotne-Prager-Yamakawa blob mobility products on GB300.
//
// u_i = b_i * nf * sum_j M_ij(z_eff) (b_j v_j)
//
// for the four blocks UF, UT, WF, WT of the wall mobility (Swan & Brady wall
// correction on top of the RPY tensor), with the wall regularisation
// z_eff = max(z, a), b = min(z/a, 1) of the reference (mobility/mobility.py:52-84).
// The pair formulas are those of mobility/mobility_numba.py:124-287 (UF),
// 548-686 (UT), 938-1073 (WF), 1189-1328 (WT), rewritten without divisions:
//   h_hat * e_z      = h_j / R        (h_hat = h_j / (h_i + h_j), e_z = (h_i + h_j) / R)
//   (1 - h_hat) e_z  = h_i / R
// so each pair costs two reciprocal square roots and no division.
//
// Kernel structure (all-pairs, O(N^2)):
//   1. pack     : one thread per blob; applies z_eff and b, writes a packed
//                 source record (FP64: x,y,z,bv; mixed: pre-scaled double-float
//                 positions hi/lo + FP32 bv) to scratch.
//   2. pair     : grid (target tiles) x (source chunks).  Each CTA stages source
//                 tiles of kTile records in shared memory; each thread owns one
//                 target and loops over the tile (broadcast shared loads).
//                 Mixed mode evaluates pairs in FP32 from double-float position
//                 differences and folds each tile's FP32 partial sum into a
//                 TwoSum-compensated accumulator.  Each CTA writes its FP64
//                 partial sums to scratch partial[chunk][3n].
//   3. finalize : one thread per blob; sums the chunks in fixed order (the
//                 result is deterministic), adds the FP64 self term, applies
//                 b_i and the 1/(8 pi eta a^p) factor.
#include <algorithm>
#include <atomic>
#include <cstdio>
#include <mutex>
#include <vector>

#include "pair_math.cuh"
#include "pair_math_df.cuh"
#include "rmw_common.cuh"
#include "wall_pair.cuh"

namespace rmw {

constexpr int kThreads = 128;  // targets per CTA
constexpr int kTile = 128;     // sources per shared-memory tile

struct __align__(16) SrcD {
    double x, y, z, pad0;
    double vx, vy, vz, pad1;
};
struct __align__(16) SrcF {
    float4 hi;  // x/a, y/a, z_eff/a (rounded to float), unused
    float4 lo;  // residuals x/a - hi.x, ...
    float4 v;   // b*v
};

struct __align__(16) SrcDF {
    float4 hi;   // x/a, y/a, z_eff/a : high floats
    float4 lo;   //                     low floats
    float4 vhi;  // b*v : high floats
    float4 vlo;  //       low floats
};

struct Periodic {
    double Lx, Ly, Lz;  // already divided by a for the mixed path
};

// Work of one CTA: targets [tbeg, tend) against sources [j0, j1), partial sums
// into chunk slot `slot`.  Without a job table (SEG = false) it follows from
// the 2-D grid: target tile blockIdx.x, source chunk blockIdx.y.  With one
// (segmented products of many independent suspensions) each CTA reads its job.
struct PairRange {
    int tbeg, tend, j0, j1, slot;
};

template <bool SEG>
__device__ __forceinline__ PairRange pair_range(const TileJob *jobs, int n, int chunk)
{
    if (SEG) {
        const TileJob jb = jobs[blockIdx.x];
        return {jb.t0, jb.t1, jb.s0, jb.s1, jb.slot};
    }
    const int tb = blockIdx.x * kThreads;
    const int j0 = blockIdx.y * chunk;
    return {tb, min(n, tb + kThreads), j0, min(n, j0 + chunk), (int)blockIdx.y};
}

// ---------------------------------------------------------------------------
// pack
__global__ void pack_fp64_kernel(const double *__restrict__ r, const double *__restrict__ v, SrcD *__restrict__ src,
                                 int n, double a)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double x = r[3 * i], y = r[3 * i + 1], z = r[3 * i + 2];
    double b = (z < a) ? z / a : 1.0;
    double ze = (z <= a) ? a : z;
    SrcD s;
    s.x = x; s.y = y; s.z = ze; s.pad0 = 0.0;
    s.vx = b * v[3 * i]; s.vy = b * v[3 * i + 1]; s.vz = b * v[3 * i + 2]; s.pad1 = 0.0;
    src[i] = s;
}

__global__ void pack_mixed_kernel(const double *__restrict__ r, const double *__restrict__ v, SrcF *__restrict__ src,
                                  int n, double a)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double inva = 1.0 / a;
    double x = r[3 * i], y = r[3 * i + 1], z = r[3 * i + 2];
    double b = (z < a) ? z / a : 1.0;
    double ze = (z <= a) ? a : z;
    double xs = x * inva, ys = y * inva, zs = ze * inva;
    float xh = (float)xs, yh = (float)ys, zh = (float)zs;
    SrcF s;
    s.hi = make_float4(xh, yh, zh, 0.f);
    s.lo = make_float4((float)(xs - (double)xh), (float)(ys - (double)yh), (float)(zs - (double)zh), 0.f);
    s.v = make_float4((float)(b * v[3 * i]), (float)(b * v[3 * i + 1]), (float)(b * v[3 * i + 2]), 0.f);
    src[i] = s;
}

__global__ void pack_df_kernel(const double *__restrict__ r, const double *__restrict__ v, SrcDF *__restrict__ src,
                               int n, double a)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double inva = 1.0 / a;
    const double z = r[3 * i + 2];
    const double b = (z < a) ? z / a : 1.0;
    const double ze = (z <= a) ? a : z;
    const df x = df_of_double(r[3 * i] * inva), y = df_of_double(r[3 * i + 1] * inva), zz = df_of_double(ze * inva);
    const df vx = df_of_double(b * v[3 * i]), vy = df_of_double(b * v[3 * i + 1]), vz = df_of_double(b * v[3 * i + 2]);
    SrcDF s;
    s.hi = make_float4(x.hi, y.hi, zz.hi, 0.f);
    s.lo = make_float4(x.lo, y.lo, zz.lo, 0.f);
    s.vhi = make_float4(vx.hi, vy.hi, vz.hi, 0.f);
    s.vlo = make_float4(vx.lo, vy.lo, vz.lo, 0.f);
    src[i] = s;
}

// ---------------------------------------------------------------------------
// df64 pair kernel: double-float pair evaluation on the FP32 pipe; the
// double-float sum over each group of kDfGroup sources is folded into FP64
// accumulators (FP64 pipe, a few adds per group).
constexpr int kDfGroup = 32;

template <int KIND, bool PER, bool SEG>
__global__ void __launch_bounds__(kThreads) wall_pair_df_kernel(const SrcDF *__restrict__ src, int n, int chunk,
                                                                 Periodic P, double *__restrict__ partial,
                                                                 const TileJob *__restrict__ jobs)
{
    __shared__ SrcDF tile[kTile];
    const PairRange pr = pair_range<SEG>(jobs, n, chunk);
    const int i = pr.tbeg + threadIdx.x;
    const bool valid = i < pr.tend;
    const int j0 = pr.j0, j1 = pr.j1;
    float4 mh = make_float4(0.f, 0.f, 1.f, 0.f), ml = make_float4(0.f, 0.f, 0.f, 0.f);
    if (valid) { mh = src[i].hi; ml = src[i].lo; }
    const df xi = {mh.x, ml.x}, yi = {mh.y, ml.y}, zi = {mh.z, ml.z};
    double ax = 0.0, ay = 0.0, az = 0.0;
    for (int t0 = j0; t0 < j1; t0 += kTile) {
        const int cnt = min(kTile, j1 - t0);
        __syncthreads();
        for (int k = threadIdx.x; k < cnt; k += kThreads) tile[k] = src[t0 + k];
        __syncthreads();
        const bool self_possible = (t0 < pr.tend) && (t0 + cnt > pr.tbeg);
        for (int g0 = 0; g0 < cnt; g0 += kDfGroup) {
            const int g1 = min(cnt, g0 + kDfGroup);
            df ux = df_from(0.f), uy = df_from(0.f), uz = df_from(0.f);
            if (!PER && !self_possible) {
                // tiles that cannot hold this CTA's targets: no self-pair test
                for (int k = g0; k < g1; ++k) {
                    const float4 sh = tile[k].hi, sl = tile[k].lo, svh = tile[k].vhi, svl = tile[k].vlo;
                    const df xj = {sh.x, sl.x}, yj = {sh.y, sl.y}, zj = {sh.z, sl.z};
                    const df vx = {svh.x, svl.x}, vy = {svh.y, svl.y}, vz = {svh.z, svl.z};
                    pair_acc_df<KIND>(xi - xj, yi - yj, zi - zj, add_u(zi, zj), zi, zj, vx, vy, vz, ux, uy, uz);
                }
                ax += to_double(ux);
                ay += to_double(uy);
                az += to_double(uz);
                continue;
            }
            for (int k = g0; k < g1; ++k) {
                const float4 sh = tile[k].hi, sl = tile[k].lo, svh = tile[k].vhi, svl = tile[k].vlo;
                const int j = t0 + k;
                const df xj = {sh.x, sl.x}, yj = {sh.y, sl.y}, zj = {sh.z, sl.z};
                const df vx = {svh.x, svl.x}, vy = {svh.y, svl.y}, vz = {svh.z, svl.z};
                const df dz = zi - zj;
                const df Rz = zi + zj;
                if (!PER) {
                    // the self pair is evaluated (NaN for coincident points) and the sums
                    // restored, so the warp stays convergent
                    const df kx = ux, ky = uy, kz = uz;
                    pair_acc_df<KIND>(xi - xj, yi - yj, dz, Rz, zi, zj, vx, vy, vz, ux, uy, uz);
                    if (j == i) {
                        ux = kx;
                        uy = ky;
                        uz = kz;
                    }
                } else {
                    // minimum image in FP64 (rare path), then back to double-float
                    double rx = to_double(xi - xj), ry = to_double(yi - yj), rz = to_double(dz);
                    if (P.Lx > 0) rx = project(rx, P.Lx);
                    if (P.Ly > 0) ry = project(ry, P.Ly);
                    if (P.Lz > 0) rz = project(rz, P.Lz);
                    const int px = P.Lx > 0, py = P.Ly > 0, pz = P.Lz > 0;
                    for (int bx = -px; bx <= px; ++bx)
                        for (int by = -py; by <= py; ++by)
                            for (int bz = -pz; bz <= pz; ++bz) {
                                const bool self = (j == i) && bx == 0 && by == 0 && bz == 0;
                                const df kx = ux, ky = uy, kz = uz;
                                pair_acc_df<KIND>(df_of_double(rx + bx * P.Lx), df_of_double(ry + by * P.Ly),
                                                  df_of_double(rz + bz * P.Lz), Rz, zi, zj, vx, vy, vz, ux, uy, uz);
                                if (self) {
                                    ux = kx;
                                    uy = ky;
                                    uz = kz;
                                }
                            }
                }
            }
            ax += to_double(ux);
            ay += to_double(uy);
            az += to_double(uz);
        }
    }
    if (valid) {
        double *o = partial + (size_t)pr.slot * 3 * n + 3 * (size_t)i;
        o[0] = ax; o[1] = ay; o[2] = az;
    }
}

// ---------------------------------------------------------------------------
// Symmetric df64 UF kernel: every unordered pair is evaluated once and applied
// both ways (M_ji = M_ij^T), about half the issued instructions per ordered
// pair of wall_pair_df_kernel.  One CTA per (target tile T, source tile S),
// T <= S, over the upper triangle of tiles.  Within a CTA, lane l of a warp
// meets source (l + k) mod 128 at step k, so the 32 lanes of a warp always
// touch 32 different sources: the source-side sums are per-warp shared-memory
// double-float accumulators updated without atomics (a __syncwarp orders
// consecutive steps).  On diagonal tiles the step offset (source - target) mod 128 is
// warp-uniform, and only offsets 1..63 (and 64 for the lower half of the
// targets) are evaluated: each unordered pair once.
// Partial sums: blob b of tile X receives one write per tile Y - from CTA
// (X, Y) as a target for Y >= X (the diagonal CTA adds both roles), from CTA
// (Y, X) as a source for Y < X - into partial[Y][3n], so the finalize kernel
// sums ntiles slots in fixed order and the result is deterministic.
constexpr int kSymWarps = kThreads / 32;


// The CTA's tile pair: from blockIdx.x over the upper triangle of nt tiles, or
// (SEG) from its job, which also moves src and partial to its suspension.
template <bool SEG, typename Rec>
__device__ __forceinline__ void sym_cta(const SymJob *jobs, int &n, int &nt, int &T, int &S,
                                        const Rec *__restrict__ &src, double *__restrict__ &partial)
{
    if (SEG) {
        const SymJob jb = jobs[blockIdx.x];
        src += jb.base;
        partial += jb.pbase;
        n = jb.n;
        nt = (jb.n + kTile - 1) / kTile;
        T = jb.T;
        S = jb.S;
    } else {
        sym_tile_pair(blockIdx.x, nt, T, S);
    }
}

// A band of tile rows [t0, t1) of the upper triangle (all S >= T), with its
// own compact partial sums: the target-side sums of CTA (T, S) at
// bt[((T - t0) (nt - t0) + S - t0) * 384], the source-side sums at
// bs[((S - t0) (t1 - t0) + T - t0) * 384] (384 = 3 x 128 doubles).  Bands
// are accumulated one after the other in a fixed order (sym_band_accum_kernel),
// so the scratch is O(band x n) instead of O(n^2 / 128) and results stay
// deterministic.
struct SymBand {
    int t0, t1;
    double *bt, *bs;
};

__device__ __forceinline__ void sym_band_pair(long long b, int nt, const SymBand &bd, int &T, int &S)
{
    int t = bd.t0;
    while (t + 1 < bd.t1 && b >= nt - t) {
        b -= nt - t;
        ++t;
    }
    T = t;
    S = t + (int)b;
}

template <bool SEG, int KIND, bool NOWALL = false, bool BAND = false>
__device__ __forceinline__ void df_sym_body(const SrcDF *__restrict__ src, int n, int nt,
                                            double *__restrict__ partial, const SymJob *__restrict__ jobs,
                                            const SymBand bd = SymBand{0, 0, nullptr, nullptr})
{
    // structure-of-arrays source tile: the rotated reads of a warp hit 32
    // consecutive 16-byte entries (no bank conflicts)
    __shared__ float4 thi[kTile], tlo[kTile], tvh[kTile], tvl[kTile];
    __shared__ float2 sacc[kSymWarps][3][kTile];  // per-warp source-side double-float sums (hi, lo)
    int T, S;
    if constexpr (BAND) sym_band_pair(blockIdx.x, nt, bd, T, S);
    else sym_cta<SEG>(jobs, n, nt, T, S, src, partial);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const bool diag = (T == S);
    const int i = T * kTile + tid;
    const bool valid_i = i < n;
    // a target or source past the end is a dummy far above the wall with a zero vector
    const SrcDF dummy = {make_float4(1.0e6f, 1.0e6f, 1.0e6f, 0.f), make_float4(0.f, 0.f, 0.f, 0.f),
                         make_float4(0.f, 0.f, 0.f, 0.f), make_float4(0.f, 0.f, 0.f, 0.f)};
    const SrcDF me = valid_i ? src[i] : dummy;
    const df xi = {me.hi.x, me.lo.x}, yi = {me.hi.y, me.lo.y}, zi = {me.hi.z, me.lo.z};
    const df qx = {me.vhi.x, me.vlo.x}, qy = {me.vhi.y, me.vlo.y}, qz = {me.vhi.z, me.vlo.z};
    {
        const int j = S * kTile + tid;
        const SrcDF sj = (j < n) ? src[j] : dummy;
        thi[tid] = sj.hi;
        tlo[tid] = sj.lo;
        tvh[tid] = sj.vhi;
        tvl[tid] = sj.vlo;
    }
    for (int c = 0; c < 3; ++c)
        for (int k = lane; k < kTile; k += 32) sacc[warp][c][k] = make_float2(0.f, 0.f);
    __syncthreads();
    double ax = 0.0, ay = 0.0, az = 0.0;
    df ux = df_from(0.f), uy = df_from(0.f), uz = df_from(0.f);
    auto fold = [&]() {  // fold each group of 32 double-float sums into FP64
        ax += to_double(ux);
        ay += to_double(uy);
        az += to_double(uz);
        ux = df_from(0.f);
        uy = df_from(0.f);
        uz = df_from(0.f);
    };
    auto step = [&](int k) {
        const int jl = (lane + k) & (kTile - 1);
        const float4 sh = thi[jl], sl = tlo[jl], svh = tvh[jl], svl = tvl[jl];
        const df xj = {sh.x, sl.x}, yj = {sh.y, sl.y}, zj = {sh.z, sl.z};
        const df vx = {svh.x, svl.x}, vy = {svh.y, svl.y}, vz = {svh.z, svl.z};
        // double-float accumulation on the FP32 pipe (no FP64 conversions per pair)
        const float2 a0 = sacc[warp][0][jl], a1 = sacc[warp][1][jl], a2 = sacc[warp][2][jl];
        df wx = {a0.x, a0.y}, wy = {a1.x, a1.y}, wz = {a2.x, a2.y};
        // differences renormalised (a cancelled high part must not leave the value in the low part, whose
        // square a double-float product drops); the sum of two heights cannot cancel
        if constexpr (NOWALL)
            pair_rpy_sym_df<KIND>(xi - xj, yi - yj, zi - zj, vx, vy, vz, qx, qy, qz, ux, uy, uz, wx, wy, wz);
        else if constexpr (KIND == RMW_UF)
            pair_uf_sym_df(xi - xj, yi - yj, zi - zj, add_u(zi, zj), zi, zj, vx, vy, vz, qx, qy, qz, ux, uy, uz, wx,
                           wy, wz);
        else
            pair_rot_sym_df<KIND>(xi - xj, yi - yj, zi - zj, add_u(zi, zj), zi, zj, vx, vy, vz, qx, qy, qz, ux, uy,
                                  uz, wx, wy, wz);
        sacc[warp][0][jl] = make_float2(wx.hi, wx.lo);
        sacc[warp][1][jl] = make_float2(wy.hi, wy.lo);
        sacc[warp][2][jl] = make_float2(wz.hi, wz.lo);
    };
    if (diag) {
        for (int k = 0; k < kTile; ++k) {
            __syncwarp();
            if (k && !(k & 31)) fold();
            const int off = (k - 32 * warp) & (kTile - 1);  // (source - target) mod 128, warp-uniform
            if (off == 0 || off > kTile / 2 || (off == kTile / 2 && warp >= kSymWarps / 2)) continue;
            step(k);
        }
    } else {
        // off-diagonal tiles: no per-step skip test (unrolling measured slower here)
        for (int g = 0; g < kTile; g += 32) {
            if (g) fold();
#pragma unroll 1
            for (int k = g; k < g + 32; ++k) {
                __syncwarp();
                step(k);
            }
        }
    }
    ax += to_double(ux);
    ay += to_double(uy);
    az += to_double(uz);
    __syncthreads();
    // source role of blob S*128 + tid (dummy pairs contributed exact zeros)
    double sx = 0.0, sy = 0.0, sz = 0.0;
    for (int w = 0; w < kSymWarps; ++w) {
        sx += (double)sacc[w][0][tid].x + (double)sacc[w][0][tid].y;
        sy += (double)sacc[w][1][tid].x + (double)sacc[w][1][tid].y;
        sz += (double)sacc[w][2][tid].x + (double)sacc[w][2][tid].y;
    }
    if constexpr (BAND) {
        const int W = nt - bd.t0, C = bd.t1 - bd.t0;
        double *o = bd.bt + ((size_t)(T - bd.t0) * W + (S - bd.t0)) * (3 * kTile) + 3 * tid;
        o[0] = diag ? ax + sx : ax;
        o[1] = diag ? ay + sy : ay;
        o[2] = diag ? az + sz : az;
        if (!diag) {
            double *q = bd.bs + ((size_t)(S - bd.t0) * C + (T - bd.t0)) * (3 * kTile) + 3 * tid;
            q[0] = sx; q[1] = sy; q[2] = sz;
        }
        return;
    }
    const size_t stride = 3 * (size_t)n;
    if (diag) {
        if (valid_i) {
            double *o = partial + (size_t)T * stride + 3 * (size_t)i;
            o[0] = ax + sx; o[1] = ay + sy; o[2] = az + sz;
        }
    } else {
        if (valid_i) {
            double *o = partial + (size_t)S * stride + 3 * (size_t)i;
            o[0] = ax; o[1] = ay; o[2] = az;
        }
        const int j = S * kTile + tid;
        if (j < n) {
            double *o = partial + (size_t)T * stride + 3 * (size_t)j;
            o[0] = sx; o[1] = sy; o[2] = sz;
        }
    }
}

template <bool SEG>
__global__ void __launch_bounds__(kThreads) wall_uf_df_sym_kernel(const SrcDF *__restrict__ src, int n, int nt,
                                                                   double *__restrict__ partial,
                                                                   const SymJob *__restrict__ jobs)
{
    df_sym_body<SEG, RMW_UF>(src, n, nt, partial, jobs);
}

// The rotation blocks (UT, WF, WT) on the same grid: pair_rot_sym_df.
template <bool SEG, int KIND>
__global__ void __launch_bounds__(kThreads) wall_rot_df_sym_kernel(const SrcDF *__restrict__ src, int n, int nt,
                                                                    double *__restrict__ partial,
                                                                    const SymJob *__restrict__ jobs)
{
    df_sym_body<SEG, KIND>(src, n, nt, partial, jobs);
}

// The same kernels over one band of tile rows (SymBand): products whose
// per-tile partial sums would not fit in the scratch budget.
template <int KIND>
__global__ void __launch_bounds__(kThreads) wall_df_sym_band_kernel(const SrcDF *__restrict__ src, int n, int nt,
                                                                     const SymBand bd)
{
    df_sym_body<false, KIND, false, true>(src, n, nt, nullptr, nullptr, bd);
}

// acc (3n doubles, FP64) += the band's contributions to every blob of tiles
// >= t0: its target-side sums (tiles in the band, S ascending) and its
// source-side sums (T ascending), in a fixed order.
__global__ void sym_band_accum_kernel(const SymBand bd, int n, int nt, double *__restrict__ acc)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= n) return;
    const int X = b / kTile, l = b % kTile;
    if (X < bd.t0) return;
    const int W = nt - bd.t0, C = bd.t1 - bd.t0;
    double sx = 0.0, sy = 0.0, sz = 0.0;
    if (X < bd.t1)
        for (int S = X; S < nt; ++S) {
            const double *o = bd.bt + ((size_t)(X - bd.t0) * W + (S - bd.t0)) * (3 * kTile) + 3 * l;
            sx += o[0]; sy += o[1]; sz += o[2];
        }
    for (int T = bd.t0; T < min(bd.t1, X); ++T) {
        const double *o = bd.bs + ((size_t)(X - bd.t0) * C + (T - bd.t0)) * (3 * kTile) + 3 * l;
        sx += o[0]; sy += o[1]; sz += o[2];
    }
    acc[3LL * b] += sx;
    acc[3LL * b + 1] += sy;
    acc[3LL * b + 2] += sz;
}

// Symmetric mixed-precision UF kernel: the same grid, pairing and partial-sum
// slots as wall_uf_df_sym_kernel, FP32 pair math from double-float position
// differences (as wall_pair_mixed_kernel).  The target-side FP32 sum over the
// tile is folded into a TwoSum-compensated accumulator; the source side sums
// its 32 contributions per warp in FP32 shared memory and the four warp
// copies in double-float.  The slots hold double-float values (float2 hi, lo
// in the 8 bytes of a double slot), which the finalize adds on the FP32 pipe:
// summed in FP64, the ceil(n/128) slots of every blob made the finalize
// FP64-bound on GB300.
template <bool SEG, int KIND, bool NOWALL = false>
__device__ __forceinline__ void mixed_sym_body(const SrcF *__restrict__ src, int n, int nt,
                                               double *__restrict__ partial, const SymJob *__restrict__ jobs)
{
    __shared__ float4 thi[kTile], tlo[kTile], tv[kTile];
    __shared__ float sacc[kSymWarps][3][kTile];
    int T, S;
    sym_cta<SEG>(jobs, n, nt, T, S, src, partial);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const bool diag = (T == S);
    const int i = T * kTile + tid;
    const bool valid_i = i < n;
    const SrcF dummy = {make_float4(1.0e6f, 1.0e6f, 1.0e6f, 0.f), make_float4(0.f, 0.f, 0.f, 0.f),
                        make_float4(0.f, 0.f, 0.f, 0.f)};
    const SrcF me = valid_i ? src[i] : dummy;
    const float hi = me.hi.z + me.lo.z;
    {
        const int j = S * kTile + tid;
        const SrcF sj = (j < n) ? src[j] : dummy;
        thi[tid] = sj.hi;
        tlo[tid] = sj.lo;
        tv[tid] = sj.v;
    }
    for (int c = 0; c < 3; ++c)
        for (int k = lane; k < kTile; k += 32) sacc[warp][c][k] = 0.f;
    __syncthreads();
    float ux = 0.f, uy = 0.f, uz = 0.f;
    auto step = [&](int k) {
        const int jl = (lane + k) & (kTile - 1);
        const float4 sh = thi[jl], sl = tlo[jl], sv = tv[jl];
        const float dx = (me.hi.x - sh.x) + (me.lo.x - sl.x);
        const float dy = (me.hi.y - sh.y) + (me.lo.y - sl.y);
        const float dz = (me.hi.z - sh.z) + (me.lo.z - sl.z);
        const float hj = sh.z + sl.z;
        const float Rz = hi + hj;
        float wx = sacc[warp][0][jl], wy = sacc[warp][1][jl], wz = sacc[warp][2][jl];
        if constexpr (NOWALL) {
            pair_rpy_sym<float, KIND>(dx, dy, dz, sv.x, sv.y, sv.z, me.v.x, me.v.y, me.v.z, ux, uy, uz, wx, wy, wz);
        } else if constexpr (KIND == RMW_UF) {
            const UFCoeffs<float> c = uf_coeffs<float>(dx, dy, dz, Rz, hi, hj);
            uf_apply<float>(c, dx, dy, dz, Rz, sv.x, sv.y, sv.z, ux, uy, uz);
            const UFCoeffs<float> ct = {c.Af, c.Bc, c.c2, c.c4, c.c3, c.Af5};  // M^T: f3 and f4 trade places
            uf_apply<float>(ct, dx, dy, dz, Rz, me.v.x, me.v.y, me.v.z, wx, wy, wz);
        } else {
            pair_rot_sym<float, KIND>(dx, dy, dz, Rz, hi, hj, sv.x, sv.y, sv.z, me.v.x, me.v.y, me.v.z, ux, uy, uz, wx,
                                      wy, wz);
        }
        sacc[warp][0][jl] = wx;
        sacc[warp][1][jl] = wy;
        sacc[warp][2][jl] = wz;
    };
    if (diag) {
        for (int k = 0; k < kTile; ++k) {
            __syncwarp();
            const int off = (k - 32 * warp) & (kTile - 1);
            if (off == 0 || off > kTile / 2 || (off == kTile / 2 && warp >= kSymWarps / 2)) continue;
            step(k);
        }
    } else {
        // off-diagonal tiles (all but nt of them): no per-step skip test; two steps per trip
#pragma unroll 2
        for (int k = 0; k < kTile; ++k) {
            __syncwarp();
            step(k);
        }
    }
    float sx = 0.f, sy = 0.f, sz = 0.f, ex_ = 0.f, ey_ = 0.f, ez_ = 0.f;
    comp_add(sx, ex_, ux);
    comp_add(sy, ey_, uy);
    comp_add(sz, ez_, uz);
    const df ax = two_sum_df(sx, ex_), ay = two_sum_df(sy, ey_), az = two_sum_df(sz, ez_);
    __syncthreads();
    df qx = df_from(sacc[0][0][tid]), qy = df_from(sacc[0][1][tid]), qz = df_from(sacc[0][2][tid]);
    for (int w = 1; w < kSymWarps; ++w) {
        qx = qx + sacc[w][0][tid];
        qy = qy + sacc[w][1][tid];
        qz = qz + sacc[w][2][tid];
    }
    float2 *part2 = reinterpret_cast<float2 *>(partial);
    const size_t stride = 3 * (size_t)n;
    auto put = [](float2 *o, df x, df y, df z) {
        o[0] = make_float2(x.hi, x.lo);
        o[1] = make_float2(y.hi, y.lo);
        o[2] = make_float2(z.hi, z.lo);
    };
    if (diag) {
        if (valid_i) put(part2 + (size_t)T * stride + 3 * (size_t)i, ax + qx, ay + qy, az + qz);
    } else {
        if (valid_i) put(part2 + (size_t)S * stride + 3 * (size_t)i, ax, ay, az);
        const int j = S * kTile + tid;
        if (j < n) put(part2 + (size_t)T * stride + 3 * (size_t)j, qx, qy, qz);
    }
}

template <bool SEG>
__global__ void __launch_bounds__(kThreads) wall_uf_mixed_sym_kernel(const SrcF *__restrict__ src, int n, int nt,
                                                                      double *__restrict__ partial,
                                                                      const SymJob *__restrict__ jobs)
{
    mixed_sym_body<SEG, RMW_UF>(src, n, nt, partial, jobs);
}

template <bool SEG, int KIND>
__global__ void __launch_bounds__(kThreads) wall_rot_mixed_sym_kernel(const SrcF *__restrict__ src, int n, int nt,
                                                                       double *__restrict__ partial,
                                                                       const SymJob *__restrict__ jobs)
{
    mixed_sym_body<SEG, KIND>(src, n, nt, partial, jobs);
}

// Symmetric FP64 kernel of any kind: the same grid, pairing and partial-sum
// slots, FP64 pair arithmetic (the FP64 pipe bounds it, so halving the
// coefficient work per ordered pair is the gain); source-side sums per warp
// in FP64 shared memory.
template <bool SEG, int KIND, bool NOWALL = false>
__device__ __forceinline__ void fp64_sym_body(const SrcD *__restrict__ src, int n, int nt, double inva,
                                              double *__restrict__ partial, const SymJob *__restrict__ jobs)
{
    __shared__ double tx[kTile], ty[kTile], tz[kTile], tvx[kTile], tvy[kTile], tvz[kTile];
    __shared__ double sacc[kSymWarps][3][kTile];
    int T, S;
    sym_cta<SEG>(jobs, n, nt, T, S, src, partial);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const bool diag = (T == S);
    const int i = T * kTile + tid;
    const bool valid_i = i < n;
    // a target or source past the end is a dummy far above the wall with a zero vector
    const SrcD dummy = {1.0e6, 1.0e6, 1.0e6, 0.0, 0.0, 0.0, 0.0, 0.0};
    const SrcD me = valid_i ? src[i] : dummy;
    const double xi = me.x * inva, yi = me.y * inva, zi = me.z * inva;
    {
        const int j = S * kTile + tid;
        const SrcD sj = (j < n) ? src[j] : dummy;
        tx[tid] = sj.x * inva;
        ty[tid] = sj.y * inva;
        tz[tid] = sj.z * inva;
        tvx[tid] = sj.vx;
        tvy[tid] = sj.vy;
        tvz[tid] = sj.vz;
    }
    for (int c = 0; c < 3; ++c)
        for (int k = lane; k < kTile; k += 32) sacc[warp][c][k] = 0.0;
    __syncthreads();
    double ux = 0.0, uy = 0.0, uz = 0.0;
    auto step = [&](int k) {
        const int jl = (lane + k) & (kTile - 1);
        const double zj = tz[jl];
        const double dx = xi - tx[jl], dy = yi - ty[jl], dz = zi - zj, Rz = zi + zj;
        const double vx = tvx[jl], vy = tvy[jl], vz = tvz[jl];
        double wx = sacc[warp][0][jl], wy = sacc[warp][1][jl], wz = sacc[warp][2][jl];
        if constexpr (NOWALL) {
            pair_rpy_sym<double, KIND>(dx, dy, dz, vx, vy, vz, me.vx, me.vy, me.vz, ux, uy, uz, wx, wy, wz);
        } else if constexpr (KIND == RMW_UF) {
            const UFCoeffs<double> c = uf_coeffs<double>(dx, dy, dz, Rz, zi, zj);
            uf_apply<double>(c, dx, dy, dz, Rz, vx, vy, vz, ux, uy, uz);
            const UFCoeffs<double> ct = {c.Af, c.Bc, c.c2, c.c4, c.c3, c.Af5};  // M^T: f3 and f4 trade places
            uf_apply<double>(ct, dx, dy, dz, Rz, me.vx, me.vy, me.vz, wx, wy, wz);
        } else {
            pair_rot_sym<double, KIND>(dx, dy, dz, Rz, zi, zj, vx, vy, vz, me.vx, me.vy, me.vz, ux, uy, uz, wx, wy,
                                       wz);
        }
        sacc[warp][0][jl] = wx;
        sacc[warp][1][jl] = wy;
        sacc[warp][2][jl] = wz;
    };
    if (diag) {
        for (int k = 0; k < kTile; ++k) {
            __syncwarp();
            const int off = (k - 32 * warp) & (kTile - 1);
            if (off == 0 || off > kTile / 2 || (off == kTile / 2 && warp >= kSymWarps / 2)) continue;
            step(k);
        }
    } else {
        for (int k = 0; k < kTile; ++k) {
            __syncwarp();
            step(k);
        }
    }
    __syncthreads();
    double qx = 0.0, qy = 0.0, qz = 0.0;
    for (int w = 0; w < kSymWarps; ++w) {
        qx += sacc[w][0][tid];
        qy += sacc[w][1][tid];
        qz += sacc[w][2][tid];
    }
    const size_t stride = 3 * (size_t)n;
    if (diag) {
        if (valid_i) {
            double *o = partial + (size_t)T * stride + 3 * (size_t)i;
            o[0] = ux + qx; o[1] = uy + qy; o[2] = uz + qz;
        }
    } else {
        if (valid_i) {
            double *o = partial + (size_t)S * stride + 3 * (size_t)i;
            o[0] = ux; o[1] = uy; o[2] = uz;
        }
        const int j = S * kTile + tid;
        if (j < n) {
            double *o = partial + (size_t)T * stride + 3 * (size_t)j;
            o[0] = qx; o[1] = qy; o[2] = qz;
        }
    }
}

template <bool SEG, int KIND>
__global__ void __launch_bounds__(kThreads) wall_fp64_sym_kernel(const SrcD *__restrict__ src, int n, int nt,
                                                                  double inva, double *__restrict__ partial,
                                                                  const SymJob *__restrict__ jobs)
{
    fp64_sym_body<SEG, KIND>(src, n, nt, inva, partial, jobs);
}

// Free-space (no wall) symmetric kernels: the same bodies with pair_rpy_sym;
// the no-wall pack writes records of the same layouts (positions over a, no
// height shift or damping), so the FP64 body takes inva = 1.
template <int KIND>
__global__ void __launch_bounds__(kThreads) nowall_df_sym_kernel(const SrcDF *__restrict__ src, int n, int nt,
                                                                  double *__restrict__ partial)
{
    df_sym_body<false, KIND, true>(src, n, nt, partial, nullptr);
}
template <int KIND>
__global__ void __launch_bounds__(kThreads) nowall_mixed_sym_kernel(const SrcF *__restrict__ src, int n, int nt,
                                                                     double *__restrict__ partial)
{
    mixed_sym_body<false, KIND, true>(src, n, nt, partial, nullptr);
}
template <int KIND>
__global__ void __launch_bounds__(kThreads) nowall_fp64_sym_kernel(const SrcD *__restrict__ src, int n, int nt,
                                                                    double *__restrict__ partial)
{
    fp64_sym_body<false, KIND, true>(src, n, nt, 1.0, partial, nullptr);
}

template <int KIND>
static void nowall_sym_launch_kind(int mode, const void *src, int n, int nt, double *partial, cudaStream_t st)
{
    const unsigned ncta = (unsigned)((long long)nt * (nt + 1) / 2);
    if (mode == RMW_MODE_FP64)
        nowall_fp64_sym_kernel<KIND><<<ncta, kThreads, 0, st>>>((const SrcD *)src, n, nt, partial);
    else if (mode == RMW_MODE_DF64)
        nowall_df_sym_kernel<KIND><<<ncta, kThreads, 0, st>>>((const SrcDF *)src, n, nt, partial);
    else
        nowall_mixed_sym_kernel<KIND><<<ncta, kThreads, 0, st>>>((const SrcF *)src, n, nt, partial);
}

int nowall_sym_launch(int kind, int mode, const void *src, int n, double *partial, cudaStream_t st)
{
    const int nt = wall_sym_slots(n);
    switch (kind) {
    case RMW_UF: nowall_sym_launch_kind<RMW_UF>(mode, src, n, nt, partial, st); break;
    case RMW_UT: nowall_sym_launch_kind<RMW_UT>(mode, src, n, nt, partial, st); break;
    case RMW_WF: nowall_sym_launch_kind<RMW_WF>(mode, src, n, nt, partial, st); break;
    default: nowall_sym_launch_kind<RMW_WT>(mode, src, n, nt, partial, st); break;
    }
    RMW_CHECK_LAUNCH("symmetric free-space product");
    return RMW_OK;
}

// ---------------------------------------------------------------------------
// FP64 pair kernel
template <int KIND, bool PER, bool SEG>
__global__ void __launch_bounds__(kThreads) wall_pair_fp64_kernel(const SrcD *__restrict__ src, int n, int chunk,
                                                                   double inva, Periodic P,
                                                                   double *__restrict__ partial,
                                                                   const TileJob *__restrict__ jobs)
{
    __shared__ SrcD tile[kTile];
    const PairRange pr = pair_range<SEG>(jobs, n, chunk);
    const int i = pr.tbeg + threadIdx.x;
    const bool valid = i < pr.tend;
    const int j0 = pr.j0, j1 = pr.j1;
    SrcD me;
    if (valid) me = src[i];
    else { me.x = 0.0; me.y = 0.0; me.z = 1.0; }
    const double hi = me.z * inva;
    double ux = 0.0, uy = 0.0, uz = 0.0;
    for (int t0 = j0; t0 < j1; t0 += kTile) {
        const int cnt = min(kTile, j1 - t0);
        __syncthreads();
        for (int k = threadIdx.x; k < cnt; k += kThreads) tile[k] = src[t0 + k];
        __syncthreads();
#pragma unroll 2
        for (int k = 0; k < cnt; ++k) {
            const SrcD s = tile[k];
            const int j = t0 + k;
            const double hj = s.z * inva;
            const double Rz = (me.z + s.z) * inva;
            if (!PER) {
                double cx = 0.0, cy = 0.0, cz = 0.0;
                pair_contrib<KIND, double>((me.x - s.x) * inva, (me.y - s.y) * inva, (me.z - s.z) * inva, Rz, hi, hj,
                                           s.vx, s.vy, s.vz, cx, cy, cz);
                if (j != i) { ux += cx; uy += cy; uz += cz; }
            } else {
                double rx = me.x - s.x, ry = me.y - s.y, rz = me.z - s.z;
                if (P.Lx > 0) rx = project(rx, P.Lx);
                if (P.Ly > 0) ry = project(ry, P.Ly);
                if (P.Lz > 0) rz = project(rz, P.Lz);
                const int px = P.Lx > 0, py = P.Ly > 0, pz = P.Lz > 0;
                for (int bx = -px; bx <= px; ++bx)
                    for (int by = -py; by <= py; ++by)
                        for (int bz = -pz; bz <= pz; ++bz) {
                            double cx = 0.0, cy = 0.0, cz = 0.0;
                            pair_contrib<KIND, double>((rx + bx * P.Lx) * inva, (ry + by * P.Ly) * inva,
                                                       (rz + bz * P.Lz) * inva, Rz, hi, hj, s.vx, s.vy, s.vz, cx, cy,
                                                       cz);
                            const bool self = (j == i) && bx == 0 && by == 0 && bz == 0;
                            if (!self) { ux += cx; uy += cy; uz += cz; }
                        }
            }
        }
    }
    if (valid) {
        double *o = partial + (size_t)pr.slot * 3 * n + 3 * (size_t)i;
        o[0] = ux; o[1] = uy; o[2] = uz;
    }
}

// ---------------------------------------------------------------------------
// Mixed pair kernel: FP32 pair evaluation, double-float position differences,
// per-tile FP32 sums folded into TwoSum-compensated accumulators.
template <int KIND, bool PER, bool SEG>
__global__ void __launch_bounds__(kThreads) wall_pair_mixed_kernel(const SrcF *__restrict__ src, int n, int chunk,
                                                                    Periodic P, double *__restrict__ partial,
                                                                    const TileJob *__restrict__ jobs)
{
    __shared__ SrcF tile[kTile];
    const PairRange pr = pair_range<SEG>(jobs, n, chunk);
    const int i = pr.tbeg + threadIdx.x;
    const bool valid = i < pr.tend;
    const int j0 = pr.j0, j1 = pr.j1;
    float4 mh = make_float4(0.f, 0.f, 1.f, 0.f), ml = make_float4(0.f, 0.f, 0.f, 0.f);
    if (valid) { mh = src[i].hi; ml = src[i].lo; }
    const float hi = mh.z + ml.z;
    float sx = 0.f, sy = 0.f, sz = 0.f;   // compensated running sums (hi parts)
    float ex_ = 0.f, ey_ = 0.f, ez_ = 0.f;  // compensation terms
    const float Lx = (float)P.Lx, Ly = (float)P.Ly, Lz = (float)P.Lz;
    for (int t0 = j0; t0 < j1; t0 += kTile) {
        const int cnt = min(kTile, j1 - t0);
        __syncthreads();
        for (int k = threadIdx.x; k < cnt; k += kThreads) tile[k] = src[t0 + k];
        __syncthreads();
        float ux = 0.f, uy = 0.f, uz = 0.f;
        // only tiles that overlap this CTA's own targets can hold the self pair
        const bool self_possible = (t0 < pr.tend) && (t0 + cnt > pr.tbeg);
        if (!PER && !self_possible) {
#pragma unroll 4
            for (int k = 0; k < cnt; ++k) {
                const float4 sh = tile[k].hi;
                const float4 sl = tile[k].lo;
                const float4 sv = tile[k].v;
                const float dx = (mh.x - sh.x) + (ml.x - sl.x);
                const float dy = (mh.y - sh.y) + (ml.y - sl.y);
                const float dz = (mh.z - sh.z) + (ml.z - sl.z);
                const float hj = sh.z + sl.z;
                pair_contrib<KIND, float>(dx, dy, dz, hi + hj, hi, hj, sv.x, sv.y, sv.z, ux, uy, uz);
            }
        } else
#pragma unroll 4
        for (int k = 0; k < cnt; ++k) {
            const float4 sh = tile[k].hi;
            const float4 sl = tile[k].lo;
            const float4 sv = tile[k].v;
            const int j = t0 + k;
            const float dx = (mh.x - sh.x) + (ml.x - sl.x);
            const float dy = (mh.y - sh.y) + (ml.y - sl.y);
            const float dz = (mh.z - sh.z) + (ml.z - sl.z);
            const float hj = sh.z + sl.z;
            const float Rz = hi + hj;
            if (!PER) {
                float cx = 0.f, cy = 0.f, cz = 0.f;
                pair_contrib<KIND, float>(dx, dy, dz, Rz, hi, hj, sv.x, sv.y, sv.z, cx, cy, cz);
                if (j != i) { ux += cx; uy += cy; uz += cz; }
            } else {
                float rx = dx, ry = dy, rz = dz;
                if (Lx > 0.f) rx = project(rx, Lx);
                if (Ly > 0.f) ry = project(ry, Ly);
                if (Lz > 0.f) rz = project(rz, Lz);
                const int px = Lx > 0.f, py = Ly > 0.f, pz = Lz > 0.f;
                for (int bx = -px; bx <= px; ++bx)
                    for (int by = -py; by <= py; ++by)
                        for (int bz = -pz; bz <= pz; ++bz) {
                            float cx = 0.f, cy = 0.f, cz = 0.f;
                            pair_contrib<KIND, float>(rx + bx * Lx, ry + by * Ly, rz + bz * Lz, Rz, hi, hj, sv.x,
                                                      sv.y, sv.z, cx, cy, cz);
                            const bool self = (j == i) && bx == 0 && by == 0 && bz == 0;
                            if (!self) { ux += cx; uy += cy; uz += cz; }
                        }
            }
        }
        comp_add(sx, ex_, ux);
        comp_add(sy, ey_, uy);
        comp_add(sz, ez_, uz);
    }
    if (valid) {
        double *o = partial + (size_t)pr.slot * 3 * n + 3 * (size_t)i;
        o[0] = (double)sx + (double)ex_;
        o[1] = (double)sy + (double)ey_;
        o[2] = (double)sz + (double)ez_;
    }
}

// ---------------------------------------------------------------------------
// Multi-right-hand-side M_UF product (mixed precision): the vector-independent
// part of each pair block is computed once and applied to every right-hand
// side of a pass.  Passes are kMultiPass (16) wide; a pass of at most 8
// right-hand sides runs the 8-wide kernel.  vec[(j * width + q) * 3 + c]
// holds component c of b_j v_q,j (3 * width floats per source, a multiple of
// 16 bytes).
__global__ void pack_multi_kernel(const double *__restrict__ r, const double *__restrict__ V, long long ldv, int nrhs,
                                  SrcF *__restrict__ src, float *__restrict__ vec, int n, double a, int width)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double inva = 1.0 / a;
    const double z = r[3 * i + 2];
    const double b = (z < a) ? z / a : 1.0;
    const double ze = (z <= a) ? a : z;
    const double xs = r[3 * i] * inva, ys = r[3 * i + 1] * inva, zs = ze * inva;
    const float xh = (float)xs, yh = (float)ys, zh = (float)zs;
    SrcF s;
    s.hi = make_float4(xh, yh, zh, 0.f);
    s.lo = make_float4((float)(xs - (double)xh), (float)(ys - (double)yh), (float)(zs - (double)zh), 0.f);
    s.v = make_float4(0.f, 0.f, 0.f, 0.f);
    src[i] = s;
    float *o = vec + (long long)i * 3 * width;
    for (int q = 0; q < width; ++q) {
        float w0 = 0.f, w1 = 0.f, w2 = 0.f;
        if (q < nrhs) {
            const double *v = V + (long long)q * ldv + 3LL * i;
            w0 = (float)(b * v[0]);
            w1 = (float)(b * v[1]);
            w2 = (float)(b * v[2]);
        }
        o[3 * q] = w0;
        o[3 * q + 1] = w1;
        o[3 * q + 2] = w2;
    }
}

// One shared-memory tile of sources against this thread's target, for every
// right-hand side: the explicit 3x3 block once per pair, then nine FMAs per
// right-hand side.  DIAG: the tile may contain the target itself, whose pair
// block is zeroed (the self term is added by the finalize kernel).
template <bool DIAG, int NR>
__device__ __forceinline__ void multi_tile(const float4 *tpos, const float4 *tvec, int cnt, int t0, int i, float4 mh,
                                           float4 ml, float hi, float (&acc)[NR][3])
{
#pragma unroll 1
    for (int k = 0; k < cnt; ++k) {
        const float4 shp = tpos[2 * k], slp = tpos[2 * k + 1];
        const float dx = (mh.x - shp.x) + (ml.x - slp.x);
        const float dy = (mh.y - shp.y) + (ml.y - slp.y);
        const float dz = (mh.z - shp.z) + (ml.z - slp.z);
        const float hj = shp.z + slp.z;
        const float Rz = hi + hj;
        UFCoeffs<float> c = uf_coeffs<float>(dx, dy, dz, Rz, hi, hj);
        if (DIAG && t0 + k == i) c = UFCoeffs<float>{0.f, 0.f, 0.f, 0.f, 0.f, 0.f};  // finite inputs
        const UFBlock m = uf_block_f(c, dx, dy, dz, Rz);
        const float4 *vk = tvec + k * (3 * NR / 4);
#pragma unroll
        for (int g = 0; g < NR / 4; ++g) {  // four right-hand sides = three float4
            const float4 a0 = vk[3 * g], a1 = vk[3 * g + 1], a2 = vk[3 * g + 2];
            uf_block_apply(m, a0.x, a0.y, a0.z, acc[4 * g][0], acc[4 * g][1], acc[4 * g][2]);
            uf_block_apply(m, a0.w, a1.x, a1.y, acc[4 * g + 1][0], acc[4 * g + 1][1], acc[4 * g + 1][2]);
            uf_block_apply(m, a1.z, a1.w, a2.x, acc[4 * g + 2][0], acc[4 * g + 2][1], acc[4 * g + 2][2]);
            uf_block_apply(m, a2.y, a2.z, a2.w, acc[4 * g + 3][0], acc[4 * g + 3][1], acc[4 * g + 3][2]);
        }
    }
}

// Dynamic shared memory of the NR-wide kernel: kTile/2 source positions (hi,
// lo), their NR vectors and, for NR > 8, the per-thread compensated sums
// (float2 hi/lo, laid out [component][thread] so a warp's accesses are
// consecutive); up to 8 right-hand sides keep those sums in registers.
template <int NR> constexpr size_t multi_smem_bytes()
{
    return sizeof(float4) * kTile + sizeof(float) * kTile / 2 * 3 * NR +
           (NR > 8 ? sizeof(float2) * NR * 3 * kThreads : 0);
}

template <bool SEG, int NR>
__global__ void __launch_bounds__(kThreads, NR > 8 ? 3 : 4) wall_pair_multi_kernel(const SrcF *__restrict__ src,
                                                                    const float4 *__restrict__ vec, int n, int chunk,
                                                                    double *__restrict__ partial,
                                                                    const TileJob *__restrict__ jobs,
                                                                    const unsigned char *__restrict__ active)
{
    constexpr bool kRegSums = NR <= 8;
    extern __shared__ float4 multi_smem[];
    float4 *tpos = multi_smem;              // 2 * kTile/2
    float4 *tvec = multi_smem + kTile;      // kTile/2 sources x 3 NR floats
    float2 *sums = (float2 *)(tvec + kTile / 2 * (3 * NR / 4));
    if (SEG && active && !active[jobs[blockIdx.x].susp]) return;  // converged suspension: nothing to do
    const PairRange pr = pair_range<SEG>(jobs, n, chunk);
    const int i = pr.tbeg + threadIdx.x;
    const bool valid = i < pr.tend;
    float4 mh = make_float4(0.f, 0.f, 1.f, 0.f), ml = make_float4(0.f, 0.f, 0.f, 0.f);
    if (valid) { mh = src[i].hi; ml = src[i].lo; }
    const float hi = mh.z + ml.z;
    float sh_[kRegSums ? NR : 1][3], sl_[kRegSums ? NR : 1][3];
    if constexpr (kRegSums) {
#pragma unroll
        for (int q = 0; q < NR; ++q)
#pragma unroll
            for (int c = 0; c < 3; ++c) sh_[q][c] = sl_[q][c] = 0.f;
    } else {
        for (int e = 0; e < NR * 3; ++e) sums[e * kThreads + threadIdx.x] = make_float2(0.f, 0.f);
    }
    constexpr int kT = kTile / 2;
    for (int t0 = pr.j0; t0 < pr.j1; t0 += kT) {
        const int cnt = min(kT, pr.j1 - t0);
        __syncthreads();
        for (int k = threadIdx.x; k < cnt; k += kThreads) {
            tpos[2 * k] = src[t0 + k].hi;
            tpos[2 * k + 1] = src[t0 + k].lo;
        }
        for (int k = threadIdx.x; k < cnt * (3 * NR / 4); k += kThreads)
            tvec[k] = vec[(long long)t0 * (3 * NR / 4) + k];
        __syncthreads();
        float acc[NR][3];
#pragma unroll
        for (int q = 0; q < NR; ++q) acc[q][0] = acc[q][1] = acc[q][2] = 0.f;
        // only a tile that overlaps the CTA's targets can hold a self pair
        if (t0 < pr.tend && t0 + cnt > pr.tbeg) multi_tile<true, NR>(tpos, tvec, cnt, t0, i, mh, ml, hi, acc);
        else multi_tile<false, NR>(tpos, tvec, cnt, t0, i, mh, ml, hi, acc);
#pragma unroll
        for (int q = 0; q < NR; ++q)
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                if constexpr (kRegSums) {
                    comp_add(sh_[q][c], sl_[q][c], acc[q][c]);
                } else {
                    float2 &w = sums[(q * 3 + c) * kThreads + threadIdx.x];
                    float h = w.x, l = w.y;
                    comp_add(h, l, acc[q][c]);
                    w = make_float2(h, l);
                }
            }
    }
    if (valid) {
#pragma unroll
        for (int q = 0; q < NR; ++q) {
            double *o = partial + ((size_t)pr.slot * NR + q) * 3 * n + 3 * (size_t)i;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                if constexpr (kRegSums) {
                    o[c] = (double)sh_[q][c] + (double)sl_[q][c];
                } else {
                    const float2 w = sums[(q * 3 + c) * kThreads + threadIdx.x];
                    o[c] = (double)w.x + (double)w.y;
                }
            }
        }
    }
}

// out[q][3i..] = b_i nf (sum_slots partial + self block (b_i v_q,i)) for q < nrhs
__global__ void wall_finalize_multi_kernel(const double *__restrict__ r, const double *__restrict__ V, long long ldv,
                                           int nrhs, int width, const double *__restrict__ partial, int nchunks,
                                           double *__restrict__ out, long long ldo, int n, double a, double nf,
                                           const int *__restrict__ blob_nchunks,
                                           const unsigned char *__restrict__ active = nullptr,
                                           const int *__restrict__ blob_susp = nullptr)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int q = blockIdx.y;
    if (i >= n || q >= nrhs) return;
    if (active && !active[blob_susp[i]]) {  // skipped suspension: zero rows
        double *o = out + (long long)q * ldo + 3LL * i;
        o[0] = o[1] = o[2] = 0.0;
        return;
    }
    const int nc = blob_nchunks ? blob_nchunks[i] : nchunks;
    double ux = 0.0, uy = 0.0, uz = 0.0;
    for (int s = 0; s < nc; ++s) {
        const double *p = partial + ((size_t)s * width + q) * 3 * n + 3 * (size_t)i;
        ux += p[0]; uy += p[1]; uz += p[2];
    }
    ux *= kUFCoeffScale; uy *= kUFCoeffScale; uz *= kUFCoeffScale;  // the pair kernel sums (3/2) M v
    const double z = r[3 * i + 2];
    const double b = (z < a) ? z / a : 1.0;
    const double ze = (z <= a) ? a : z;
    const double *v = V + (long long)q * ldv + 3LL * i;
    const double iz = a / ze, iz3 = iz * iz * iz, iz5 = iz3 * iz * iz;
    const double mxx = 4.0 / 3.0 - (9.0 * iz - 2.0 * iz3 + iz5) / 12.0;
    const double mzz = 4.0 / 3.0 - (9.0 * iz - 4.0 * iz3 + iz5) / 6.0;
    ux += mxx * b * v[0];
    uy += mxx * b * v[1];
    uz += mzz * b * v[2];
    double *o = out + (long long)q * ldo + 3LL * i;
    const double sc = b * nf;
    o[0] = ux * sc;
    o[1] = uy * sc;
    o[2] = uz * sc;
}

// ---------------------------------------------------------------------------
// finalize: fixed-order chunk sum + FP64 self term + b_i * norm factor.
// With pbase / pstride (segmented symmetric layout) blob i's slot s is at
// partial + pbase[i] + s * pstride[i]; otherwise at partial + s * 3n + 3i.
// kFinGroup consecutive threads share a blob: thread g of the group sums slots
// g, g + kFinGroup, ... and a fixed shuffle tree adds the group's sums, so the
// order is fixed (deterministic) and the slot loads run kFinGroup-wide.
constexpr int kFinGroup = 4;
inline unsigned finalize_blocks(int n, int pb) { return (unsigned)(((long long)kFinGroup * n + pb - 1) / pb); }

// DF2: the slots hold double-float values (the mixed symmetric kernels), added
// in double-float on the FP32 pipe
template <int KIND, bool DF2 = false>
__global__ void wall_finalize_kernel(const double *__restrict__ r, const double *__restrict__ v,
                                     const double *__restrict__ partial, int nchunks, double *__restrict__ out,
                                     int n, double a, double nf, const int *__restrict__ blob_nchunks,
                                     const long long *__restrict__ pbase = nullptr,
                                     const int *__restrict__ pstride = nullptr, double pair_scale = 1.0)
{
    const long long gt = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int i = (int)(gt / kFinGroup), g = (int)(gt % kFinGroup);
    double ux = 0.0, uy = 0.0, uz = 0.0;
    if constexpr (DF2) {
        df sx = df_from(0.f), sy = df_from(0.f), sz = df_from(0.f);
        if (i < n) {
            const int nc = blob_nchunks ? blob_nchunks[i] : nchunks;
            const float2 *p0 = reinterpret_cast<const float2 *>(partial) + (pbase ? pbase[i] : 3 * (long long)i);
            const size_t ps = pstride ? (size_t)pstride[i] : 3 * (size_t)n;
#pragma unroll 4
            for (int s = g; s < nc; s += kFinGroup) {
                const float2 *p = p0 + (size_t)s * ps;
                const float2 px = p[0], py = p[1], pz = p[2];
                sx = sx + df{px.x, px.y};
                sy = sy + df{py.x, py.y};
                sz = sz + df{pz.x, pz.y};
            }
        }
#pragma unroll
        for (int o = kFinGroup / 2; o > 0; o >>= 1) {  // every lane of the warp takes part
            sx = sx + df{__shfl_down_sync(0xffffffffu, sx.hi, o, kFinGroup),
                         __shfl_down_sync(0xffffffffu, sx.lo, o, kFinGroup)};
            sy = sy + df{__shfl_down_sync(0xffffffffu, sy.hi, o, kFinGroup),
                         __shfl_down_sync(0xffffffffu, sy.lo, o, kFinGroup)};
            sz = sz + df{__shfl_down_sync(0xffffffffu, sz.hi, o, kFinGroup),
                         __shfl_down_sync(0xffffffffu, sz.lo, o, kFinGroup)};
        }
        ux = (double)sx.hi + (double)sx.lo;
        uy = (double)sy.hi + (double)sy.lo;
        uz = (double)sz.hi + (double)sz.lo;
    } else {
        if (i < n) {
            const int nc = blob_nchunks ? blob_nchunks[i] : nchunks;
            const double *p0 = pbase ? partial + pbase[i] : partial + 3 * (size_t)i;
            const size_t ps = pstride ? (size_t)pstride[i] : 3 * (size_t)n;
#pragma unroll 4
            for (int s = g; s < nc; s += kFinGroup) {  // unrolled: loads of several slots in flight
                const double *p = p0 + (size_t)s * ps;
                ux += p[0]; uy += p[1]; uz += p[2];
            }
        }
#pragma unroll
        for (int o = kFinGroup / 2; o > 0; o >>= 1) {  // every lane of the warp takes part
            ux += __shfl_down_sync(0xffffffffu, ux, o, kFinGroup);
            uy += __shfl_down_sync(0xffffffffu, uy, o, kFinGroup);
            uz += __shfl_down_sync(0xffffffffu, uz, o, kFinGroup);
        }
    }
    if (i >= n || g != 0) return;
    ux *= pair_scale; uy *= pair_scale; uz *= pair_scale;
    const double z = r[3 * i + 2];
    const double b = (z < a) ? z / a : 1.0;
    const double ze = (z <= a) ? a : z;
    const double vx = b * v[3 * i], vy = b * v[3 * i + 1], vz = b * v[3 * i + 2];
    const double iz = a / ze;  // 1/h
    if (KIND == RMW_UF) {
        const double iz3 = iz * iz * iz, iz5 = iz3 * iz * iz;
        const double mxx = 4.0 / 3.0 - (9.0 * iz - 2.0 * iz3 + iz5) / 12.0;
        const double mzz = 4.0 / 3.0 - (9.0 * iz - 4.0 * iz3 + iz5) / 6.0;
        ux += mxx * vx; uy += mxx * vy; uz += mzz * vz;
    } else if (KIND == RMW_UT) {
        const double s = 0.125 * iz * iz * iz * iz;
        ux += s * vy; uy -= s * vx;
    } else if (KIND == RMW_WF) {
        const double s = 0.125 * iz * iz * iz * iz;
        ux -= s * vy; uy += s * vx;
    } else {
        const double iz3 = iz * iz * iz;
        ux += (1.0 - 0.3125 * iz3) * vx; uy += (1.0 - 0.3125 * iz3) * vy; uz += (1.0 - 0.125 * iz3) * vz;
    }
    const double sc = b * nf;
    out[3 * i] = ux * sc;
    out[3 * i + 1] = uy * sc;
    out[3 * i + 2] = uz * sc;
}

// ---------------------------------------------------------------------------
// host side
static int choose_chunks(int n)
{
    const int tiles = (n + kThreads - 1) / kThreads;
    const int want = 152 * 8;  // CTAs to fill the 152 SMs several times over
    int s = (want + tiles - 1) / tiles;
    s = std::min(s, std::max(1, n / 256));  // keep each chunk >= 256 sources
    return std::max(1, std::min(s, 64));
}

int wall_default_chunks(int n) { return choose_chunks(n); }

size_t wall_scratch_bytes(int n, int mode, int nchunks)
{
    size_t rec = (mode == RMW_MODE_FP64) ? sizeof(SrcD) : (mode == RMW_MODE_DF64 ? sizeof(SrcDF) : sizeof(SrcF));
    size_t packed = ((rec * (size_t)n + 255) / 256) * 256;
    return packed + sizeof(double) * 3 * (size_t)n * (size_t)nchunks;
}

template <int KIND>
static int launch_kind(const double *r, const double *v, double *out, int n, double eta, double a, const double *L,
                       int mode, cudaStream_t st, void *scratch_ptr, int nchunks, const WallBatch *B)
{
    const double inva = 1.0 / a;
    const double nf = (KIND == RMW_UF)   ? 1.0 / (8.0 * kPi * eta * a)
                      : (KIND == RMW_WT) ? 1.0 / (8.0 * kPi * eta * a * a * a)
                                         : 1.0 / (8.0 * kPi * eta * a * a);
    const bool per = !B && L && (L[0] > 0 || L[1] > 0 || L[2] > 0);
    Periodic P{L ? L[0] : 0.0, L ? L[1] : 0.0, L ? L[2] : 0.0};
    size_t rec = (mode == RMW_MODE_FP64) ? sizeof(SrcD) : (mode == RMW_MODE_DF64 ? sizeof(SrcDF) : sizeof(SrcF));
    size_t packed = ((rec * (size_t)n + 255) / 256) * 256;
    char *base = (char *)scratch_ptr;
    double *partial = (double *)(base + packed);
    const int chunk = (n + nchunks - 1) / nchunks;
    const dim3 grid = B ? dim3(B->njobs) : dim3((n + kThreads - 1) / kThreads, nchunks);
    const TileJob *jobs = B ? B->jobs : nullptr;
    const int pb = 256, pg = (n + pb - 1) / pb;
    void *tok = nullptr;
    if (mode == RMW_MODE_FP64) {
        SrcD *src = (SrcD *)base;
        pack_fp64_kernel<<<pg, pb, 0, st>>>(r, v, src, n, a);
        if (int rc = trace_begin(TRACE_PAIR, st, &tok)) return rc;
        if (B) wall_pair_fp64_kernel<KIND, false, true><<<grid, kThreads, 0, st>>>(src, n, chunk, inva, P, partial, jobs);
        else if (per) wall_pair_fp64_kernel<KIND, true, false><<<grid, kThreads, 0, st>>>(src, n, chunk, inva, P, partial, jobs);
        else wall_pair_fp64_kernel<KIND, false, false><<<grid, kThreads, 0, st>>>(src, n, chunk, inva, P, partial, jobs);
    } else if (mode == RMW_MODE_DF64) {
        SrcDF *src = (SrcDF *)base;
        pack_df_kernel<<<pg, pb, 0, st>>>(r, v, src, n, a);
        Periodic Ps{P.Lx * inva, P.Ly * inva, P.Lz * inva};
        if (int rc = trace_begin(TRACE_PAIR, st, &tok)) return rc;
        if (B) wall_pair_df_kernel<KIND, false, true><<<grid, kThreads, 0, st>>>(src, n, chunk, Ps, partial, jobs);
        else if (per) wall_pair_df_kernel<KIND, true, false><<<grid, kThreads, 0, st>>>(src, n, chunk, Ps, partial, jobs);
        else wall_pair_df_kernel<KIND, false, false><<<grid, kThreads, 0, st>>>(src, n, chunk, Ps, partial, jobs);
    } else {
        SrcF *src = (SrcF *)base;
        pack_mixed_kernel<<<pg, pb, 0, st>>>(r, v, src, n, a);
        Periodic Ps{P.Lx * inva, P.Ly * inva, P.Lz * inva};
        if (int rc = trace_begin(TRACE_PAIR, st, &tok)) return rc;
        if (B) wall_pair_mixed_kernel<KIND, false, true><<<grid, kThreads, 0, st>>>(src, n, chunk, Ps, partial, jobs);
        else if (per) wall_pair_mixed_kernel<KIND, true, false><<<grid, kThreads, 0, st>>>(src, n, chunk, Ps, partial, jobs);
        else wall_pair_mixed_kernel<KIND, false, false><<<grid, kThreads, 0, st>>>(src, n, chunk, Ps, partial, jobs);
    }
    if (int rc = trace_end(tok, st)) return rc;
    // the df64 UF pair kernel sums (3/2) M v
    const double scale = (KIND == RMW_UF && mode == RMW_MODE_DF64) ? kUFCoeffScale : 1.0;
    wall_finalize_kernel<KIND><<<finalize_blocks(n, pb), pb, 0, st>>>(r, v, partial, nchunks, out, n, a, nf,
                                                                       B ? B->blob_nch : nullptr, nullptr, nullptr,
                                                                       scale);
    RMW_CHECK_LAUNCH("wall product kernels");
    return RMW_OK;
}

int validate_product_args(int kind, const void *r, const void *v, const void *out, int64_t n, double eta, double a,
                          int mode)
{
    if (kind < RMW_UF || kind > RMW_WT) return fail(RMW_ERR_ARG, "unknown product kind");
    if (mode != RMW_MODE_FP64 && mode != RMW_MODE_MIXED && mode != RMW_MODE_DF64)
        return fail(RMW_ERR_ARG, "unknown precision mode");
    if (n < 0 || n > (int64_t(1) << 28)) return fail(RMW_ERR_ARG, "number of blobs out of range [0, 2^28]");
    if (n > 0 && (!r || !v || !out)) return fail(RMW_ERR_ARG, "null array pointer");
    if (!(a > 0) || !(eta > 0)) return fail(RMW_ERR_ARG, "blob radius and viscosity must be positive");
    return RMW_OK;
}

static int launch_dispatch(int kind, const double *r, const double *v, double *out, int n, double eta, double a,
                           const double *L, int mode, cudaStream_t st, void *scratch_ptr, int nchunks,
                           const WallBatch *B)
{
    switch (kind) {
    case RMW_UF: return launch_kind<RMW_UF>(r, v, out, n, eta, a, L, mode, st, scratch_ptr, nchunks, B);
    case RMW_UT: return launch_kind<RMW_UT>(r, v, out, n, eta, a, L, mode, st, scratch_ptr, nchunks, B);
    case RMW_WF: return launch_kind<RMW_WF>(r, v, out, n, eta, a, L, mode, st, scratch_ptr, nchunks, B);
    default: return launch_kind<RMW_WT>(r, v, out, n, eta, a, L, mode, st, scratch_ptr, nchunks, B);
    }
}

int wall_product_with_scratch(int kind, const double *r, const double *v, double *out, int n, double eta, double a,
                              const double *L, int mode, cudaStream_t st, void *scratch_ptr, int nchunks)
{
    return launch_dispatch(kind, r, v, out, n, eta, a, L, mode, st, scratch_ptr, nchunks, nullptr);
}

size_t wall_sym_partial_budget()
{
    // per device, computed once; atomics because several host threads may ask at once
    static std::atomic<size_t> budget[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return kSymMaxPartialBytes;
    size_t b = budget[dev].load();
    if (!b) {
        size_t total = 0;
        cudaDeviceProp prop;
        if (cudaGetDeviceProperties(&prop, dev) == cudaSuccess) total = prop.totalGlobalMem;
        b = std::max(kSymMaxPartialBytes, total / 8);
        budget[dev].store(b);
    }
    // a cap on one scratch buffer (rmw_set_scratch_limit) caps the partial sums too
    const size_t cap = scratch_limit();
    return cap ? std::min(b, cap) : b;
}

bool wall_sym_applicable(int kind, int mode, int n, const double *L)
{
    if (kind < RMW_UF || kind > RMW_WT ||
        (mode != RMW_MODE_FP64 && mode != RMW_MODE_DF64 && mode != RMW_MODE_MIXED))
        return false;
    if (L && (L[0] > 0 || L[1] > 0 || L[2] > 0)) return false;
    if (n < 2 * kTile) return false;
    const double nt = (double)((n + kTile - 1) / kTile);
    return nt * 3.0 * (double)n * sizeof(double) <= (double)wall_sym_partial_budget();
}

int wall_sym_slots(int n) { return (n + kTile - 1) / kTile; }

// the symmetric kernel and finalize of one kind: the UF kernels sum (3/2) M v
template <int KIND>
static void launch_sym(bool seg, int mode, const void *src, int n, int nt, unsigned ncta, double *partial,
                       const SymJob *jobs, cudaStream_t st, double inva)
{
    if (mode == RMW_MODE_FP64) {
        const SrcD *s = (const SrcD *)src;
        if (seg) wall_fp64_sym_kernel<true, KIND><<<ncta, kThreads, 0, st>>>(s, n, nt, inva, partial, jobs);
        else wall_fp64_sym_kernel<false, KIND><<<ncta, kThreads, 0, st>>>(s, n, nt, inva, partial, jobs);
    } else if (mode == RMW_MODE_DF64) {
        const SrcDF *s = (const SrcDF *)src;
        if (KIND == RMW_UF) {
            if (seg) wall_uf_df_sym_kernel<true><<<ncta, kThreads, 0, st>>>(s, n, nt, partial, jobs);
            else wall_uf_df_sym_kernel<false><<<ncta, kThreads, 0, st>>>(s, n, nt, partial, jobs);
        } else {
            if (seg) wall_rot_df_sym_kernel<true, KIND><<<ncta, kThreads, 0, st>>>(s, n, nt, partial, jobs);
            else wall_rot_df_sym_kernel<false, KIND><<<ncta, kThreads, 0, st>>>(s, n, nt, partial, jobs);
        }
    } else {
        const SrcF *s = (const SrcF *)src;
        if (KIND == RMW_UF) {
            if (seg) wall_uf_mixed_sym_kernel<true><<<ncta, kThreads, 0, st>>>(s, n, nt, partial, jobs);
            else wall_uf_mixed_sym_kernel<false><<<ncta, kThreads, 0, st>>>(s, n, nt, partial, jobs);
        } else {
            if (seg) wall_rot_mixed_sym_kernel<true, KIND><<<ncta, kThreads, 0, st>>>(s, n, nt, partial, jobs);
            else wall_rot_mixed_sym_kernel<false, KIND><<<ncta, kThreads, 0, st>>>(s, n, nt, partial, jobs);
        }
    }
}

static double kind_norm(int kind, double eta, double a)
{
    return (kind == RMW_UF)   ? 1.0 / (8.0 * kPi * eta * a)
           : (kind == RMW_WT) ? 1.0 / (8.0 * kPi * eta * a * a * a)
                              : 1.0 / (8.0 * kPi * eta * a * a);
}

template <int KIND, bool DF2>
static void launch_sym_finalize_t(const double *r, const double *v, const double *partial, int nt, double *out,
                                  int n, double a, double nf, const WallBatch *B, cudaStream_t st)
{
    const int pb = 256;
    const double scale = (KIND == RMW_UF) ? kUFCoeffScale : 1.0;
    if (B)
        wall_finalize_kernel<KIND, DF2><<<finalize_blocks(n, pb), pb, 0, st>>>(r, v, partial, 0, out, n, a, nf,
                                                                               B->blob_nslots, B->blob_pbase,
                                                                               B->blob_pstride, scale);
    else
        wall_finalize_kernel<KIND, DF2><<<finalize_blocks(n, pb), pb, 0, st>>>(r, v, partial, nt, out, n, a, nf,
                                                                               nullptr, nullptr, nullptr, scale);
}

// mixed: the symmetric kernels' slots hold double-float values
template <int KIND>
static void launch_sym_finalize(const double *r, const double *v, const double *partial, int nt, double *out, int n,
                                double a, double nf, const WallBatch *B, cudaStream_t st, bool mixed = false)
{
    if (mixed) launch_sym_finalize_t<KIND, true>(r, v, partial, nt, out, n, a, nf, B, st);
    else launch_sym_finalize_t<KIND, false>(r, v, partial, nt, out, n, a, nf, B, st);
}

// pack, symmetric pair kernel and finalize of any kind (B: segmented over its suspensions)
static int sym_product(int kind, const double *r, const double *v, double *out, int n, double eta, double a,
                       int mode, cudaStream_t st, void *scratch_ptr, const WallBatch *B)
{
    const int nt = B ? 0 : wall_sym_slots(n);
    const size_t rec = (mode == RMW_MODE_FP64) ? sizeof(SrcD) : (mode == RMW_MODE_DF64 ? sizeof(SrcDF) : sizeof(SrcF));
    const size_t packed = ((rec * (size_t)n + 255) / 256) * 256;
    char *base = (char *)scratch_ptr;
    double *partial = (double *)(base + packed);
    const int pb = 256, pg = (n + pb - 1) / pb;
    const unsigned ncta = B ? (unsigned)B->nsym : (unsigned)((long long)nt * (nt + 1) / 2);
    const SymJob *jobs = B ? B->sym_jobs : nullptr;
    if (mode == RMW_MODE_FP64) pack_fp64_kernel<<<pg, pb, 0, st>>>(r, v, (SrcD *)base, n, a);
    else if (mode == RMW_MODE_DF64) pack_df_kernel<<<pg, pb, 0, st>>>(r, v, (SrcDF *)base, n, a);
    else pack_mixed_kernel<<<pg, pb, 0, st>>>(r, v, (SrcF *)base, n, a);
    const double inva = 1.0 / a;
    void *tok = nullptr;
    if (int rc = trace_begin(TRACE_PAIR, st, &tok)) return rc;
    switch (kind) {
    case RMW_UF: launch_sym<RMW_UF>(B != nullptr, mode, base, n, nt, ncta, partial, jobs, st, inva); break;
    case RMW_UT: launch_sym<RMW_UT>(B != nullptr, mode, base, n, nt, ncta, partial, jobs, st, inva); break;
    case RMW_WF: launch_sym<RMW_WF>(B != nullptr, mode, base, n, nt, ncta, partial, jobs, st, inva); break;
    default: launch_sym<RMW_WT>(B != nullptr, mode, base, n, nt, ncta, partial, jobs, st, inva); break;
    }
    if (int rc = trace_end(tok, st)) return rc;
    const double nf = kind_norm(kind, eta, a);
    switch (kind) {
    case RMW_UF: launch_sym_finalize<RMW_UF>(r, v, partial, nt, out, n, a, nf, B, st, mode == RMW_MODE_MIXED); break;
    case RMW_UT: launch_sym_finalize<RMW_UT>(r, v, partial, nt, out, n, a, nf, B, st, mode == RMW_MODE_MIXED); break;
    case RMW_WF: launch_sym_finalize<RMW_WF>(r, v, partial, nt, out, n, a, nf, B, st, mode == RMW_MODE_MIXED); break;
    default: launch_sym_finalize<RMW_WT>(r, v, partial, nt, out, n, a, nf, B, st, mode == RMW_MODE_MIXED); break;
    }
    RMW_CHECK_LAUNCH("symmetric wall product kernels");
    return RMW_OK;
}

int wall_product_sym_with_scratch(int kind, const double *r, const double *v, double *out, int n, double eta,
                                  double a, int mode, cudaStream_t st, void *scratch_ptr)
{
    return sym_product(kind, r, v, out, n, eta, a, mode, st, scratch_ptr, nullptr);
}

// Tile rows per band of the banded symmetric product: the band's two partial
// sum blocks (2 x rows x nt x 384 doubles) within a quarter of the symmetric
// partial-sum budget.
int wall_sym_band_rows(int n)
{
    const long long nt = (n + kTile - 1) / kTile;
    const double per_row = 2.0 * (double)nt * 3 * kTile * sizeof(double);
    const long long rows = (long long)((double)wall_sym_partial_budget() / 4.0 / per_row);
    return (int)std::max(1LL, std::min(nt, rows));
}

size_t wall_sym_band_scratch_bytes(int n)
{
    const size_t nt = (n + kTile - 1) / kTile;
    const size_t packed = ((sizeof(SrcDF) * (size_t)n + 255) / 256) * 256;
    const size_t acc = ((sizeof(double) * 3 * (size_t)n + 255) / 256) * 256;
    return packed + acc + 2 * (size_t)wall_sym_band_rows(n) * nt * 3 * kTile * sizeof(double);
}

// The df64 symmetric product band by band (SymBand): the products whose
// per-tile partial sums exceed the scratch budget (from about 430,000 blobs on
// a GB300) keep the symmetric kernel's one evaluation per unordered pair.
static int sym_band_product(int kind, const double *r, const double *v, double *out, int n, double eta, double a,
                            cudaStream_t st, void *scratch_ptr)
{
    const int nt = (n + kTile - 1) / kTile, C = wall_sym_band_rows(n);
    const size_t packed = ((sizeof(SrcDF) * (size_t)n + 255) / 256) * 256;
    const size_t accb = ((sizeof(double) * 3 * (size_t)n + 255) / 256) * 256;
    char *base = (char *)scratch_ptr;
    double *acc = (double *)(base + packed);
    double *bt = (double *)(base + packed + accb);
    double *bs = bt + (size_t)C * nt * 3 * kTile;
    const int pb = 256, pg = (n + pb - 1) / pb;
    pack_df_kernel<<<pg, pb, 0, st>>>(r, v, (SrcDF *)base, n, a);
    RMW_CUDA(cudaMemsetAsync(acc, 0, sizeof(double) * 3 * (size_t)n, st));
    void *tok = nullptr;
    if (int rc = trace_begin(TRACE_PAIR, st, &tok)) return rc;
    for (int t0 = 0; t0 < nt; t0 += C) {
        const int t1 = std::min(nt, t0 + C);
        long long ncta = 0;
        for (int t = t0; t < t1; ++t) ncta += nt - t;
        const SymBand bd{t0, t1, bt, bs};
        const SrcDF *src = (const SrcDF *)base;
        switch (kind) {
        case RMW_UF: wall_df_sym_band_kernel<RMW_UF><<<(unsigned)ncta, kThreads, 0, st>>>(src, n, nt, bd); break;
        case RMW_UT: wall_df_sym_band_kernel<RMW_UT><<<(unsigned)ncta, kThreads, 0, st>>>(src, n, nt, bd); break;
        case RMW_WF: wall_df_sym_band_kernel<RMW_WF><<<(unsigned)ncta, kThreads, 0, st>>>(src, n, nt, bd); break;
        default: wall_df_sym_band_kernel<RMW_WT><<<(unsigned)ncta, kThreads, 0, st>>>(src, n, nt, bd); break;
        }
        sym_band_accum_kernel<<<pg, pb, 0, st>>>(bd, n, nt, acc);
    }
    if (int rc = trace_end(tok, st)) return rc;
    const double nf = kind_norm(kind, eta, a);
    switch (kind) {
    case RMW_UF: launch_sym_finalize<RMW_UF>(r, v, acc, 1, out, n, a, nf, nullptr, st); break;
    case RMW_UT: launch_sym_finalize<RMW_UT>(r, v, acc, 1, out, n, a, nf, nullptr, st); break;
    case RMW_WF: launch_sym_finalize<RMW_WF>(r, v, acc, 1, out, n, a, nf, nullptr, st); break;
    default: launch_sym_finalize<RMW_WT>(r, v, acc, 1, out, n, a, nf, nullptr, st); break;
    }
    RMW_CHECK_LAUNCH("banded symmetric wall product kernels");
    return RMW_OK;
}

int wall_product(int kind, const double *r, const double *v, double *out, int64_t n, double eta, double a,
                 const double *L, int mode, cudaStream_t st)
{
    int rc = validate_product_args(kind, r, v, out, n, eta, a, mode);
    if (rc) return rc;
    if (n == 0) return RMW_OK;
    int nchunks = wall_chunks(kind, mode, (int)n);
    bool sym = nchunks == kSymChunks && wall_sym_applicable(kind, mode, (int)n, L);
    const bool periodic = L && (L[0] > 0 || L[1] > 0 || L[2] > 0);
    void *ws = nullptr;
    if (nchunks == kSymChunks && !sym && mode == RMW_MODE_DF64 && !periodic && n >= 2 * kTile) {
        // too many tiles for one partial-sum slot per tile: the symmetric kernel band by band
        if (scratch(SCRATCH_PAIR, wall_sym_band_scratch_bytes((int)n), &ws, st) == RMW_OK)
            return sym_band_product(kind, r, v, out, (int)n, eta, a, st, ws);
        cudaGetLastError();
    }
    if (nchunks == kSymChunks && !sym) nchunks = wall_default_chunks((int)n);
    rc = scratch(SCRATCH_PAIR, wall_scratch_bytes((int)n, mode, sym ? wall_sym_slots((int)n) : nchunks), &ws, st);
    if (rc && sym) {
        // the symmetric kernel's partial sums did not fit next to the caller's
        // allocations: the standard kernel needs far less scratch
        cudaGetLastError();
        sym = false;
        nchunks = wall_default_chunks((int)n);
        rc = scratch(SCRATCH_PAIR, wall_scratch_bytes((int)n, mode, nchunks), &ws, st);
    }
    if (rc) return rc;
    if (sym) return wall_product_sym_with_scratch(kind, r, v, out, (int)n, eta, a, mode, st, ws);
    return wall_product_with_scratch(kind, r, v, out, (int)n, eta, a, L, mode, st, ws, nchunks);
}

// ---------------------------------------------------------------------------
// segmented products of many suspensions
int wall_batch_build(WallBatch &B, const long long *off, int ninst)
{
    if (ninst <= 0) return fail(RMW_ERR_ARG, "need at least one suspension");
    if (off[0] != 0) return fail(RMW_ERR_ARG, "suspension offsets must start at 0");
    for (int k = 0; k < ninst; ++k)
        if (off[k + 1] < off[k]) return fail(RMW_ERR_ARG, "suspension offsets must not decrease");
    if (off[ninst] > (1LL << 28)) return fail(RMW_ERR_ARG, "too many blobs");
    B.n = (int)off[ninst];
    B.ninst = ninst;
    B.off.assign(off, off + ninst + 1);
    RMW_CUDA(cudaGetDevice(&B.device));
    // one chunk factor for all suspensions, sized so the whole batch fills the GPU,
    // never splitting a suspension's sources below 256 per chunk
    long long tiles = 0;
    for (int k = 0; k < ninst; ++k) tiles += (off[k + 1] - off[k] + kThreads - 1) / kThreads;
    const long long want = 152 * 8;
    const int factor = (int)std::max<long long>(1, std::min<long long>(64, (want + tiles - 1) / std::max(1LL, tiles)));
    std::vector<TileJob> jobs;
    std::vector<int> nch(B.n), bsusp(B.n);
    for (int k = 0; k < ninst; ++k)
        for (long long i = off[k]; i < off[k + 1]; ++i) bsusp[i] = k;
    int max_slots = 1;
    for (int k = 0; k < ninst; ++k) {
        const int b0 = (int)off[k], m = (int)(off[k + 1] - off[k]);
        if (m == 0) continue;
        const int c = std::max(1, std::min(factor, m / 256));
        const int chunk = (m + c - 1) / c;
        max_slots = std::max(max_slots, c);
        for (int i = b0; i < b0 + m; ++i) nch[i] = c;
        for (int t = 0; t < m; t += kThreads)
            for (int q = 0; q < c; ++q) {
                const int s0 = b0 + q * chunk, s1 = std::min(b0 + m, s0 + chunk);
                jobs.push_back({b0 + t, std::min(b0 + m, b0 + t + kThreads), s0, std::max(s0, s1), q, k});
            }
    }
    B.njobs = (int)jobs.size();
    B.max_slots = max_slots;
    RMW_CUDA(cudaMalloc(&B.jobs, sizeof(TileJob) * std::max<size_t>(1, jobs.size())));
    RMW_CUDA(cudaMalloc(&B.blob_nch, sizeof(int) * std::max(1, B.n)));
    RMW_CUDA(cudaMalloc(&B.blob_susp, sizeof(int) * std::max(1, B.n)));
    RMW_CUDA(cudaMemcpy(B.jobs, jobs.data(), sizeof(TileJob) * jobs.size(), cudaMemcpyHostToDevice));
    if (B.n) RMW_CUDA(cudaMemcpy(B.blob_nch, nch.data(), sizeof(int) * B.n, cudaMemcpyHostToDevice));
    if (B.n) RMW_CUDA(cudaMemcpy(B.blob_susp, bsusp.data(), sizeof(int) * B.n, cudaMemcpyHostToDevice));
    // symmetric UF layout: every suspension's upper triangle of tile pairs,
    // partial sums suspension after suspension
    std::vector<SymJob> sj;
    std::vector<long long> pb(B.n);
    std::vector<int> pst(B.n), nsl(B.n);
    long long pbase = 0;
    for (int k = 0; k < ninst; ++k) {
        const int b0 = (int)off[k], m = (int)(off[k + 1] - off[k]);
        if (m == 0) continue;
        const int nt = (m + kTile - 1) / kTile;
        for (int T = 0; T < nt; ++T)
            for (int S = T; S < nt; ++S) sj.push_back({pbase, b0, m, T, S});
        for (int i = 0; i < m; ++i) {
            pb[b0 + i] = pbase + 3LL * i;
            pst[b0 + i] = 3 * m;
            nsl[b0 + i] = nt;
        }
        pbase += (long long)nt * 3 * m;
    }
    B.nsym = (long long)sj.size();
    B.sym_doubles = pbase;
    RMW_CUDA(cudaMalloc(&B.sym_jobs, sizeof(SymJob) * std::max<size_t>(1, sj.size())));
    RMW_CUDA(cudaMalloc(&B.blob_pbase, sizeof(long long) * std::max(1, B.n)));
    RMW_CUDA(cudaMalloc(&B.blob_pstride, sizeof(int) * std::max(1, B.n)));
    RMW_CUDA(cudaMalloc(&B.blob_nslots, sizeof(int) * std::max(1, B.n)));
    if (!sj.empty()) RMW_CUDA(cudaMemcpy(B.sym_jobs, sj.data(), sizeof(SymJob) * sj.size(), cudaMemcpyHostToDevice));
    if (B.n) {
        RMW_CUDA(cudaMemcpy(B.blob_pbase, pb.data(), sizeof(long long) * B.n, cudaMemcpyHostToDevice));
        RMW_CUDA(cudaMemcpy(B.blob_pstride, pst.data(), sizeof(int) * B.n, cudaMemcpyHostToDevice));
        RMW_CUDA(cudaMemcpy(B.blob_nslots, nsl.data(), sizeof(int) * B.n, cudaMemcpyHostToDevice));
    }
    return RMW_OK;
}

void wall_batch_free(WallBatch &B)
{
    int cur = 0;
    cudaGetDevice(&cur);
    cudaSetDevice(B.device);
    if (B.jobs) cudaFree(B.jobs);
    if (B.blob_nch) cudaFree(B.blob_nch);
    for (void *p : {(void *)B.sym_jobs, (void *)B.blob_pbase, (void *)B.blob_pstride, (void *)B.blob_nslots,
                    (void *)B.blob_susp})
        if (p) cudaFree(p);
    cudaSetDevice(cur);
    B.jobs = nullptr;
    B.blob_nch = nullptr;
    B.sym_jobs = nullptr;
    B.blob_pbase = nullptr;
    B.blob_pstride = nullptr;
    B.blob_nslots = nullptr;
    B.blob_susp = nullptr;
}

int wall_product_batched(const WallBatch &B, int kind, const double *r, const double *v, double *out, double eta,
                         double a, int mode, cudaStream_t st)
{
    int rc = validate_product_args(kind, r, v, out, B.n, eta, a, mode);
    if (rc) return rc;
    if (B.n == 0 || B.njobs == 0) return RMW_OK;
    void *ws = nullptr;
    if (B.nsym > 0 && B.sym_doubles * (long long)sizeof(double) <= (long long)wall_sym_partial_budget()) {
        // each suspension's unordered pairs once, applied both ways
        const size_t rec = (mode == RMW_MODE_FP64) ? sizeof(SrcD) : (mode == RMW_MODE_DF64 ? sizeof(SrcDF) : sizeof(SrcF));
        const size_t packed = ((rec * (size_t)B.n + 255) / 256) * 256;
        rc = scratch(SCRATCH_PAIR, packed + sizeof(double) * (size_t)B.sym_doubles, &ws, st);
        if (rc) return rc;
        return sym_product(kind, r, v, out, B.n, eta, a, mode, st, ws, &B);
    }
    rc = scratch(SCRATCH_PAIR, wall_scratch_bytes(B.n, mode, B.max_slots), &ws, st);
    if (rc) return rc;
    return launch_dispatch(kind, r, v, out, B.n, eta, a, nullptr, mode, st, ws, B.max_slots, &B);
}

// M_UF applied to nrhs vectors (rows of V with stride ldv; outputs rows of Y
// with stride ldy), mixed precision, kMultiPass vectors per pass.
int wall_uf_multi(const double *r, const double *V, long long ldv, double *Y, long long ldy, int nrhs, int n,
                  double eta, double a, const WallBatch *B, cudaStream_t st, const unsigned char *active)
{
    if (!B) active = nullptr;
    if (nrhs <= 0 || n <= 0) return RMW_OK;
    const int nchunks = B ? B->max_slots : choose_chunks(n);
    const int wmax = nrhs > 8 ? kMultiPass : 8;
    const size_t pos = ((sizeof(SrcF) * (size_t)n + 255) / 256) * 256;
    const size_t vecb = ((sizeof(float) * 3 * (size_t)n * wmax + 255) / 256) * 256;
    const size_t bytes = pos + vecb + sizeof(double) * 3 * (size_t)n * wmax * nchunks;
    void *ws = nullptr;
    if (int rc = scratch(SCRATCH_PAIR, bytes, &ws, st)) return rc;
    SrcF *src = (SrcF *)ws;
    float *vec = (float *)((char *)ws + pos);
    const float4 *vec4 = (const float4 *)vec;
    double *partial = (double *)((char *)ws + pos + vecb);
    const double nf = 1.0 / (8.0 * kPi * eta * a);
    const int chunk = (n + nchunks - 1) / nchunks;
    const dim3 grid = B ? dim3(B->njobs) : dim3((n + kThreads - 1) / kThreads, nchunks);
    static bool attr_set = false;  // the 16-wide kernel needs more than 48 KB of shared memory
    if (!attr_set) {
        RMW_CUDA(cudaFuncSetAttribute(wall_pair_multi_kernel<true, kMultiPass>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)multi_smem_bytes<kMultiPass>()));
        RMW_CUDA(cudaFuncSetAttribute(wall_pair_multi_kernel<false, kMultiPass>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)multi_smem_bytes<kMultiPass>()));
        attr_set = true;
    }
    for (int q0 = 0; q0 < nrhs; q0 += kMultiPass) {
        const int nr = std::min(kMultiPass, nrhs - q0);
        const int width = nr > 8 ? kMultiPass : 8;
        pack_multi_kernel<<<(n + 255) / 256, 256, 0, st>>>(r, V + (long long)q0 * ldv, ldv, nr, src, vec, n, a,
                                                           width);
        void *tok = nullptr;
        if (int rc = trace_begin(TRACE_PAIR, st, &tok)) return rc;
        const unsigned char *act = active ? active + (size_t)(q0 / kMultiPass) * B->ninst : nullptr;
        const TileJob *jobs = B ? B->jobs : nullptr;
        if (width == kMultiPass) {
            const size_t sm = multi_smem_bytes<kMultiPass>();
            if (B) wall_pair_multi_kernel<true, kMultiPass><<<grid, kThreads, sm, st>>>(src, vec4, n, chunk, partial, jobs, act);
            else wall_pair_multi_kernel<false, kMultiPass><<<grid, kThreads, sm, st>>>(src, vec4, n, chunk, partial, jobs, act);
        } else {
            const size_t sm = multi_smem_bytes<8>();
            if (B) wall_pair_multi_kernel<true, 8><<<grid, kThreads, sm, st>>>(src, vec4, n, chunk, partial, jobs, act);
            else wall_pair_multi_kernel<false, 8><<<grid, kThreads, sm, st>>>(src, vec4, n, chunk, partial, jobs, act);
        }
        if (int rc = trace_end(tok, st)) return rc;
        wall_finalize_multi_kernel<<<dim3((n + 255) / 256, nr), 256, 0, st>>>(
            r, V + (long long)q0 * ldv, ldv, nr, width, partial, nchunks, Y + (long long)q0 * ldy, ldy, n, a, nf,
            B ? B->blob_nch : nullptr, act, B ? B->blob_susp : nullptr);
    }
    RMW_CHECK_LAUNCH("multi-rhs product");
    return RMW_OK;
}

}  // namespace rmw

// ---------------------------------------------------------------------------
// C ABI
extern "C" {

// How a product of (kind, mode, n) is launched on the current device: 0 the
// one-sided kernel, 1 the symmetric kernel (one partial-sum slot per tile),
// 2 the symmetric kernel band by band (beyond the partial-sum budget).
int rmw_wall_product_route(int kind, int mode, int64_t n, const double *L_host, int *route_host)
{
    if (!route_host) return rmw::fail(RMW_ERR_ARG, "null output");
    if (int rc = rmw::validate_product_args(kind, (void *)1, (void *)1, (void *)1, n, 1.0, 1.0, mode)) return rc;
    const int N = (int)n;
    const bool periodic = L_host && (L_host[0] > 0 || L_host[1] > 0 || L_host[2] > 0);
    const int c = rmw::wall_chunks(kind, mode, N);
    int route = 0;
    if (c == rmw::kSymChunks) {
        if (rmw::wall_sym_applicable(kind, mode, N, L_host)) route = 1;
        else if (mode == RMW_MODE_DF64 && !periodic && N >= 2 * rmw::kTile) route = 2;
    }
    *route_host = route;
    return RMW_OK;
}


int rmw_wall_product(int kind, const double *r, const double *v, double *out, int64_t n, double eta, double a,
                     const double *L_host, int mode, void *stream)
{
    return rmw::wall_product(kind, r, v, out, n, eta, a, L_host, mode, rmw::as_stream(stream));
}

int rmw_wall_uf(const double *r, const double *v, double *out, int64_t n, double eta, double a, const double *L_host,
                int mode, void *stream)
{
    return rmw_wall_product(RMW_UF, r, v, out, n, eta, a, L_host, mode, stream);
}
int rmw_wall_ut(const double *r, const double *v, double *out, int64_t n, double eta, double a, const double *L_host,
                int mode, void *stream)
{
    return rmw_wall_product(RMW_UT, r, v, out, n, eta, a, L_host, mode, stream);
}
int rmw_wall_wf(const double *r, const double *v, double *out, int64_t n, double eta, double a, const double *L_host,
                int mode, void *stream)
{
    return rmw_wall_product(RMW_WF, r, v, out, n, eta, a, L_host, mode, stream);
}
int rmw_wall_wt(const double *r, const double *v, double *out, int64_t n, double eta, double a, const double *L_host,
                int mode, void *stream)
{
    return rmw_wall_product(RMW_WT, r, v, out, n, eta, a, L_host, mode, stream);
}

int rmw_wall_batch_create(void **handle, int64_t n_suspensions, const int64_t *blob_offsets_host)
{
    if (!handle || !blob_offsets_host) return rmw::fail(RMW_ERR_ARG, "null argument");
    *handle = nullptr;
    if (n_suspensions <= 0 || n_suspensions > (1 << 20)) return rmw::fail(RMW_ERR_ARG, "bad suspension count");
    std::vector<long long> off(blob_offsets_host, blob_offsets_host + n_suspensions + 1);
    rmw::WallBatch *B = new rmw::WallBatch();
    int rc = rmw::wall_batch_build(*B, off.data(), (int)n_suspensions);
    if (rc) {
        rmw::wall_batch_free(*B);
        delete B;
        return rc;
    }
    *handle = B;
    return RMW_OK;
}

int rmw_wall_batch_destroy(void *handle)
{
    if (handle) {
        rmw::WallBatch *B = (rmw::WallBatch *)handle;
        rmw::wall_batch_free(*B);
        delete B;
    }
    return RMW_OK;
}

int rmw_wall_product_batched(void *handle, int kind, const double *r, const double *v, double *out, double eta,
                             double a, int mode, void *stream)
{
    if (!handle) return rmw::fail(RMW_ERR_ARG, "null batch handle");
    return rmw::wall_product_batched(*(rmw::WallBatch *)handle, kind, r, v, out, eta, a, mode, rmw::as_stream(stream));
}

int rmw_wall_uf_multi(const double *r, const double *V, double *Y, int64_t n, int nrhs, double eta, double a,
                      void *batch, void *stream)
{
    int rc = rmw::validate_product_args(RMW_UF, r, V, Y, n, eta, a, RMW_MODE_MIXED);
    if (rc) return rc;
    if (nrhs < 0) return rmw::fail(RMW_ERR_ARG, "nrhs must be >= 0");
    rmw::WallBatch *B = (rmw::WallBatch *)batch;
    if (B && B->n != n) return rmw::fail(RMW_ERR_ARG, "batch handle does not match n");
    return rmw::wall_uf_multi(r, V, 3 * n, Y, 3 * n, nrhs, (int)n, eta, a, B, rmw::as_stream(stream));
}

int rmw_wall_product_host(int kind, const double *r_host, const double *v_host, double *out_host, int64_t n,
                          double eta, double a, const double *L_host, int mode)
{
    int rc = rmw::validate_product_args(kind, r_host, v_host, out_host, n, eta, a, mode);
    if (rc) return rc;
    if (n == 0) return RMW_OK;
    // Device staging for r, v and out has its own scratch slot.
    const size_t bytes = sizeof(double) * 3 * (size_t)n;
    void *stage = nullptr;
    rc = rmw::scratch(rmw::SCRATCH_HOST_STAGING, 3 * bytes, &stage, 0);
    if (rc) return rc;
    double *dr = (double *)stage, *dv = dr + 3 * n, *dout = dv + 3 * n;
    cudaStream_t st = 0;
    RMW_CUDA(cudaMemcpyAsync(dr, r_host, bytes, cudaMemcpyHostToDevice, st));
    RMW_CUDA(cudaMemcpyAsync(dv, v_host, bytes, cudaMemcpyHostToDevice, st));
    rc = rmw::wall_product(kind, dr, dv, dout, n, eta, a, L_host, mode, st);
    if (rc) return rc;
    RMW_CUDA(cudaMemcpyAsync(out_host, dout, bytes, cudaMemcpyDeviceToHost, st));
    RMW_CUDA(cudaStreamSynchronize(st));
    return RMW_OK;
}

}  // extern "C"
