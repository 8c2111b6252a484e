// Free-space (no wall) RPY blob products: u = M v with the unbounded-domain
// Rotne-Prager-Yamakawa blocks M_UF, M_UT, M_WF, M_WT, the products of the
// reference's *_no_wall_* implementations (mobility/mobility_numba.py:13-1190,
// pycuda kernels mobility/mobility_pycuda.py:371-467 and the no-wall
// variants after it).  Positions are used as given - there is no wall, so
// no height shift and no damping - and pseudo-periodic images follow the
// wall products (minimum image plus the neighbouring boxes).
//
// Structure as the wall products: pack -> pair kernel over (target tiles) x
// (source chunks) -> finalize summing the chunks in fixed order, adding the
// self term (4/3 for UF, 1 for WT, none for UT/WF) and 1/(8 pi eta a^p).
// Precision modes FP64, df64 and mixed as there.
#include <algorithm>

#include "pair_math.cuh"
#include "pair_math_df.cuh"
#include "rmw_common.cuh"
#include "wall_pair.cuh"

namespace rmw {

namespace {

constexpr int kNwThreads = 128;
constexpr int kNwTile = 128;
constexpr int kNwDfGroup = 32;

struct NwImages {
    double Lx, Ly, Lz;  // periodic lengths over a
};

struct __align__(16) NwSrcD {
    double x, y, z, pad0;
    double vx, vy, vz, pad1;
};
struct __align__(16) NwSrcF {
    float4 hi, lo, v;
};
struct __align__(16) NwSrcDF {
    float4 hi, lo, vhi, vlo;
};
// the symmetric kernels (wall_pair.cu) read these records as the wall
// products' SrcD (x, y, z, pad, vx, vy, vz, pad), SrcF (hi, lo, v) and SrcDF
// (hi, lo, vhi, vlo): the same fields in the same order and sizes
static_assert(sizeof(NwSrcD) == 64 && sizeof(NwSrcF) == 48 && sizeof(NwSrcDF) == 64,
              "no-wall records must keep the wall records' layouts");

__global__ void nw_pack_fp64_kernel(const double *__restrict__ r, const double *__restrict__ v,
                                    NwSrcD *__restrict__ src, int n, double inva)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    NwSrcD s;
    s.x = r[3 * i] * inva; s.y = r[3 * i + 1] * inva; s.z = r[3 * i + 2] * inva; s.pad0 = 0.0;
    s.vx = v[3 * i]; s.vy = v[3 * i + 1]; s.vz = v[3 * i + 2]; s.pad1 = 0.0;
    src[i] = s;
}

__global__ void nw_pack_mixed_kernel(const double *__restrict__ r, const double *__restrict__ v,
                                     NwSrcF *__restrict__ src, int n, double inva)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double x = r[3 * i] * inva, y = r[3 * i + 1] * inva, z = r[3 * i + 2] * inva;
    const float xh = (float)x, yh = (float)y, zh = (float)z;
    NwSrcF s;
    s.hi = make_float4(xh, yh, zh, 0.f);
    s.lo = make_float4((float)(x - (double)xh), (float)(y - (double)yh), (float)(z - (double)zh), 0.f);
    s.v = make_float4((float)v[3 * i], (float)v[3 * i + 1], (float)v[3 * i + 2], 0.f);
    src[i] = s;
}

__global__ void nw_pack_df_kernel(const double *__restrict__ r, const double *__restrict__ v,
                                  NwSrcDF *__restrict__ src, int n, double inva)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const df x = df_of_double(r[3 * i] * inva), y = df_of_double(r[3 * i + 1] * inva),
             z = df_of_double(r[3 * i + 2] * inva);
    const df vx = df_of_double(v[3 * i]), vy = df_of_double(v[3 * i + 1]), vz = df_of_double(v[3 * i + 2]);
    NwSrcDF s;
    s.hi = make_float4(x.hi, y.hi, z.hi, 0.f);
    s.lo = make_float4(x.lo, y.lo, z.lo, 0.f);
    s.vhi = make_float4(vx.hi, vy.hi, vz.hi, 0.f);
    s.vlo = make_float4(vx.lo, vy.lo, vz.lo, 0.f);
    src[i] = s;
}

template <typename T, typename F>
__device__ __forceinline__ void nw_images(T rx, T ry, T rz, T Lx, T Ly, T Lz, bool self_pair, F &&f)
{
    if (Lx > T(0)) rx = project(rx, Lx);
    if (Ly > T(0)) ry = project(ry, Ly);
    if (Lz > T(0)) rz = project(rz, Lz);
    const int px = Lx > T(0), py = Ly > T(0), pz = Lz > T(0);
    for (int bx = -px; bx <= px; ++bx)
        for (int by = -py; by <= py; ++by)
            for (int bz = -pz; bz <= pz; ++bz)
                if (!(self_pair && bx == 0 && by == 0 && bz == 0)) f(rx + bx * Lx, ry + by * Ly, rz + bz * Lz);
}

template <int KIND, bool PER>
__global__ void __launch_bounds__(kNwThreads) nw_pair_fp64_kernel(const NwSrcD *__restrict__ src, int n, int chunk,
                                                                   NwImages P, double *__restrict__ partial)
{
    __shared__ NwSrcD tile[kNwTile];
    const int i = blockIdx.x * kNwThreads + threadIdx.x;
    const bool valid = i < n;
    const int j0 = blockIdx.y * chunk, j1 = min(n, j0 + chunk);
    NwSrcD me;
    if (valid) me = src[i];
    else { me.x = 0.0; me.y = 0.0; me.z = 1.0e6; }
    double ux = 0.0, uy = 0.0, uz = 0.0;
    for (int t0 = j0; t0 < j1; t0 += kNwTile) {
        const int cnt = min(kNwTile, j1 - t0);
        __syncthreads();
        for (int k = threadIdx.x; k < cnt; k += kNwThreads) tile[k] = src[t0 + k];
        __syncthreads();
        for (int k = 0; k < cnt; ++k) {
            const NwSrcD s = tile[k];
            const int j = t0 + k;
            if (!PER) {
                // the self pair is evaluated and discarded so the warp stays convergent
                double cx = 0.0, cy = 0.0, cz = 0.0;
                pair_rpy<KIND, double>(me.x - s.x, me.y - s.y, me.z - s.z, s.vx, s.vy, s.vz, cx, cy, cz);
                if (j != i) { ux += cx; uy += cy; uz += cz; }
            } else {
                nw_images(me.x - s.x, me.y - s.y, me.z - s.z, P.Lx, P.Ly, P.Lz, j == i,
                          [&](double ex, double ey, double ez) {
                              pair_rpy<KIND, double>(ex, ey, ez, s.vx, s.vy, s.vz, ux, uy, uz);
                          });
            }
        }
    }
    if (valid) {
        double *o = partial + (size_t)blockIdx.y * 3 * n + 3 * (size_t)i;
        o[0] = ux; o[1] = uy; o[2] = uz;
    }
}

template <int KIND, bool PER>
__global__ void __launch_bounds__(kNwThreads) nw_pair_mixed_kernel(const NwSrcF *__restrict__ src, int n, int chunk,
                                                                    NwImages P, double *__restrict__ partial)
{
    __shared__ NwSrcF tile[kNwTile];
    const int i = blockIdx.x * kNwThreads + threadIdx.x;
    const bool valid = i < n;
    const int j0 = blockIdx.y * chunk, j1 = min(n, j0 + chunk);
    float4 mh = make_float4(0.f, 0.f, 1.0e6f, 0.f), ml = make_float4(0.f, 0.f, 0.f, 0.f);
    if (valid) { mh = src[i].hi; ml = src[i].lo; }
    const float Lx = (float)P.Lx, Ly = (float)P.Ly, Lz = (float)P.Lz;
    float sx = 0.f, sy = 0.f, sz = 0.f, ex_ = 0.f, ey_ = 0.f, ez_ = 0.f;
    for (int t0 = j0; t0 < j1; t0 += kNwTile) {
        const int cnt = min(kNwTile, j1 - t0);
        __syncthreads();
        for (int k = threadIdx.x; k < cnt; k += kNwThreads) tile[k] = src[t0 + k];
        __syncthreads();
        float ux = 0.f, uy = 0.f, uz = 0.f;
        for (int k = 0; k < cnt; ++k) {
            const float4 sh = tile[k].hi, sl = tile[k].lo, sv = tile[k].v;
            const int j = t0 + k;
            const float dx = (mh.x - sh.x) + (ml.x - sl.x);
            const float dy = (mh.y - sh.y) + (ml.y - sl.y);
            const float dz = (mh.z - sh.z) + (ml.z - sl.z);
            if (!PER) {
                float cx = 0.f, cy = 0.f, cz = 0.f;
                pair_rpy<KIND, float>(dx, dy, dz, sv.x, sv.y, sv.z, cx, cy, cz);
                if (j != i) { ux += cx; uy += cy; uz += cz; }
            } else {
                nw_images(dx, dy, dz, Lx, Ly, Lz, j == i, [&](float qx, float qy, float qz) {
                    pair_rpy<KIND, float>(qx, qy, qz, sv.x, sv.y, sv.z, ux, uy, uz);
                });
            }
        }
        comp_add(sx, ex_, ux);
        comp_add(sy, ey_, uy);
        comp_add(sz, ez_, uz);
    }
    if (valid) {
        double *o = partial + (size_t)blockIdx.y * 3 * n + 3 * (size_t)i;
        o[0] = (double)sx + (double)ex_;
        o[1] = (double)sy + (double)ey_;
        o[2] = (double)sz + (double)ez_;
    }
}

template <int KIND, bool PER>
__global__ void __launch_bounds__(kNwThreads) nw_pair_df_kernel(const NwSrcDF *__restrict__ src, int n, int chunk,
                                                                 NwImages P, double *__restrict__ partial)
{
    __shared__ NwSrcDF tile[kNwTile];
    const int i = blockIdx.x * kNwThreads + threadIdx.x;
    const bool valid = i < n;
    const int j0 = blockIdx.y * chunk, j1 = min(n, j0 + chunk);
    float4 mh = make_float4(0.f, 0.f, 1.0e6f, 0.f), ml = make_float4(0.f, 0.f, 0.f, 0.f);
    if (valid) { mh = src[i].hi; ml = src[i].lo; }
    const df xi = {mh.x, ml.x}, yi = {mh.y, ml.y}, zi = {mh.z, ml.z};
    double ax = 0.0, ay = 0.0, az = 0.0;
    for (int t0 = j0; t0 < j1; t0 += kNwTile) {
        const int cnt = min(kNwTile, j1 - t0);
        __syncthreads();
        for (int k = threadIdx.x; k < cnt; k += kNwThreads) tile[k] = src[t0 + k];
        __syncthreads();
        for (int g0 = 0; g0 < cnt; g0 += kNwDfGroup) {
            const int g1 = min(cnt, g0 + kNwDfGroup);
            df ux = df_from(0.f), uy = df_from(0.f), uz = df_from(0.f);
            for (int k = g0; k < g1; ++k) {
                const NwSrcDF s = tile[k];
                const int j = t0 + k;
                const df xj = {s.hi.x, s.lo.x}, yj = {s.hi.y, s.lo.y}, zj = {s.hi.z, s.lo.z};
                const df vx = {s.vhi.x, s.vlo.x}, vy = {s.vhi.y, s.vlo.y}, vz = {s.vhi.z, s.vlo.z};
                if (!PER) {
                    df cx, cy, cz;
                    pair_rpy_df<KIND>(xi - xj, yi - yj, zi - zj, vx, vy, vz, cx, cy, cz);
                    if (j != i) {
                        acc_add(ux, cx);
                        acc_add(uy, cy);
                        acc_add(uz, cz);
                    }
                } else {
                    nw_images(to_double(xi - xj), to_double(yi - yj), to_double(zi - zj), P.Lx, P.Ly, P.Lz, j == i,
                              [&](double qx, double qy, double qz) {
                                  df cx, cy, cz;
                                  pair_rpy_df<KIND>(df_of_double(qx), df_of_double(qy), df_of_double(qz), vx, vy,
                                                    vz, cx, cy, cz);
                                  acc_add(ux, cx);
                                  acc_add(uy, cy);
                                  acc_add(uz, cz);
                              });
                }
            }
            ax += to_double(ux);
            ay += to_double(uy);
            az += to_double(uz);
        }
    }
    if (valid) {
        double *o = partial + (size_t)blockIdx.y * 3 * n + 3 * (size_t)i;
        o[0] = ax; o[1] = ay; o[2] = az;
    }
}

// DF2: double-float slots of the mixed symmetric kernels, added on the FP32 pipe
template <bool DF2 = false>
__global__ void nw_finalize_kernel(const double *__restrict__ v, const double *__restrict__ partial, int nchunks,
                                   double *__restrict__ out, int n, double self_coef, double nf)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double u[3] = {0.0, 0.0, 0.0};
    if constexpr (DF2) {
        const float2 *p2 = reinterpret_cast<const float2 *>(partial);
        df s3[3] = {df_from(0.f), df_from(0.f), df_from(0.f)};
        for (int s = 0; s < nchunks; ++s)
            for (int c = 0; c < 3; ++c) {
                const float2 p = p2[(size_t)s * 3 * n + 3 * (size_t)i + c];
                s3[c] = s3[c] + df{p.x, p.y};
            }
        for (int c = 0; c < 3; ++c) u[c] = (double)s3[c].hi + (double)s3[c].lo;
    } else {
        for (int s = 0; s < nchunks; ++s)
            for (int c = 0; c < 3; ++c) u[c] += partial[(size_t)s * 3 * n + 3 * (size_t)i + c];
    }
    for (int c = 0; c < 3; ++c) out[3 * i + c] = nf * (u[c] + self_coef * v[3 * i + c]);
}

template <int KIND, bool PER>
void nw_launch(int mode, dim3 grid, cudaStream_t st, const void *src, int n, int chunk, NwImages P, double *partial)
{
    if (mode == RMW_MODE_FP64)
        nw_pair_fp64_kernel<KIND, PER><<<grid, kNwThreads, 0, st>>>((const NwSrcD *)src, n, chunk, P, partial);
    else if (mode == RMW_MODE_DF64)
        nw_pair_df_kernel<KIND, PER><<<grid, kNwThreads, 0, st>>>((const NwSrcDF *)src, n, chunk, P, partial);
    else
        nw_pair_mixed_kernel<KIND, PER><<<grid, kNwThreads, 0, st>>>((const NwSrcF *)src, n, chunk, P, partial);
}

template <int KIND>
void nw_dispatch(bool per, int mode, dim3 grid, cudaStream_t st, const void *src, int n, int chunk, NwImages P,
                 double *partial)
{
    if (per) nw_launch<KIND, true>(mode, grid, st, src, n, chunk, P, partial);
    else nw_launch<KIND, false>(mode, grid, st, src, n, chunk, P, partial);
}

}  // namespace

int nowall_product(int kind, const double *r, const double *v, double *out, int64_t n, double eta, double a,
                   const double *L, int mode, cudaStream_t st)
{
    if (int rc = validate_product_args(kind, r, v, out, n, eta, a, mode)) return rc;
    if (n == 0) return RMW_OK;
    const int N = (int)n;
    const bool per = L && (L[0] > 0 || L[1] > 0 || L[2] > 0);
    // the symmetric kernel (each unordered pair once, both ways) from 4,096 blobs
    // in FP64 and df64 and 8,192 in mixed, as the wall products' untuned rule
    bool sym = !per && N >= (mode == RMW_MODE_MIXED ? 8192 : 4096) &&
               wall_sym_applicable(kind, mode, N, nullptr);
    int nchunks = sym ? wall_sym_slots(N) : wall_default_chunks(N);
    const size_t rec = (mode == RMW_MODE_FP64) ? sizeof(NwSrcD) : (mode == RMW_MODE_DF64 ? sizeof(NwSrcDF)
                                                                                          : sizeof(NwSrcF));
    const size_t packed = ((rec * (size_t)N + 255) / 256) * 256;
    void *ws = nullptr;
    int src = scratch(SCRATCH_PAIR, packed + sizeof(double) * 3 * (size_t)N * nchunks, &ws, st);
    if (src && sym) {
        // the symmetric partial sums did not fit next to the caller's
        // allocations (or above rmw_set_scratch_limit): the one-sided kernels
        // need far less scratch
        cudaGetLastError();
        sym = false;
        nchunks = wall_default_chunks(N);
        src = scratch(SCRATCH_PAIR, packed + sizeof(double) * 3 * (size_t)N * nchunks, &ws, st);
    }
    if (src) return src;
    double *partial = (double *)((char *)ws + packed);
    const double inva = 1.0 / a;
    const int pb = 256, pg = (N + pb - 1) / pb;
    if (mode == RMW_MODE_FP64) nw_pack_fp64_kernel<<<pg, pb, 0, st>>>(r, v, (NwSrcD *)ws, N, inva);
    else if (mode == RMW_MODE_DF64) nw_pack_df_kernel<<<pg, pb, 0, st>>>(r, v, (NwSrcDF *)ws, N, inva);
    else nw_pack_mixed_kernel<<<pg, pb, 0, st>>>(r, v, (NwSrcF *)ws, N, inva);
    const NwImages P{L ? L[0] * inva : 0.0, L ? L[1] * inva : 0.0, L ? L[2] * inva : 0.0};
    const int chunk = (N + nchunks - 1) / nchunks;
    const dim3 grid((N + kNwThreads - 1) / kNwThreads, nchunks);
    void *tok = nullptr;
    if (int rc = trace_begin(TRACE_PAIR, st, &tok)) return rc;
    if (sym) {
        // the sym slots have the chunk layout (slot s of blob i at s * 3n + 3i)
        if (int rc = nowall_sym_launch(kind, mode, ws, N, partial, st)) return rc;
    } else {
        switch (kind) {
        case RMW_UF: nw_dispatch<RMW_UF>(per, mode, grid, st, ws, N, chunk, P, partial); break;
        case RMW_UT: nw_dispatch<RMW_UT>(per, mode, grid, st, ws, N, chunk, P, partial); break;
        case RMW_WF: nw_dispatch<RMW_WF>(per, mode, grid, st, ws, N, chunk, P, partial); break;
        default: nw_dispatch<RMW_WT>(per, mode, grid, st, ws, N, chunk, P, partial); break;
        }
    }
    if (int rc = trace_end(tok, st)) return rc;
    const double p = (kind == RMW_UF) ? a : (kind == RMW_WT ? a * a * a : a * a);
    const double self_coef = (kind == RMW_UF) ? 4.0 / 3.0 : (kind == RMW_WT ? 1.0 : 0.0);
    if (sym && mode == RMW_MODE_MIXED)
        nw_finalize_kernel<true><<<pg, pb, 0, st>>>(v, partial, nchunks, out, N, self_coef, 1.0 / (8.0 * kPi * eta * p));
    else
        nw_finalize_kernel<false><<<pg, pb, 0, st>>>(v, partial, nchunks, out, N, self_coef,
                                                     1.0 / (8.0 * kPi * eta * p));
    RMW_CHECK_LAUNCH("free-space product kernels");
    return RMW_OK;
}

}  // namespace rmw

extern "C" {

// Free-space RPY product out = M_kind v (no wall); device arrays of 3n doubles.
int rmw_nowall_product(int kind, const double *r, const double *v, double *out, int64_t n, double eta, double a,
                       const double *L_host, int mode, void *stream)
{
    return rmw::nowall_product(kind, r, v, out, n, eta, a, L_host, mode, rmw::as_stream(stream));
}

}  // extern "C"
