// Rigid multiblob bodies: geometric matrix K, the block-diagonal
// preconditioners of multi_bodies/multi_bodies.py and the saddle-point
// operator of linear_operator_rigid, all on the GPU.
//
//   K [U; w]_i  = U_b + w_b x (r_i - x_b)               (body/body.py:81-115)
//   K^T l       = [sum_i l_i ; sum_i (r_i - x_b) x l_i]  (multi_bodies.py:350-371)
//   A [l; U]    = [M l - K U ; -K^T l]                   (multi_bodies.py:424-471)
//
// Block-diagonal preconditioner (multi_bodies.py:752-903 / 480-618), per body b
// with m = 3 n_b blob unknowns:
//   M_b      dense wall mobility of the body's blobs (mobility/mobility.py:1018-1116)
//   M_b = L L^T (Cholesky), L^-1, M_b^-1 = L^-T L^-1, N_b = (K^T M_b^-1 K)^-1
//   apply:  l~ = M_b^-1 s ; U = N_b (-F - K^T l~) ; l = l~ + (M_b^-1 K) U
// (M_b^-1 K is precomputed, so one apply reads M_b^-1 once instead of twice.)
//
// One CTA per body.  The factorisation runs in shared memory when m^2 doubles
// fit (m <= 160, i.e. up to 53 blobs per body), else in global memory.
#include <algorithm>
#include <cmath>
#include <vector>

#include "pair_math.cuh"
#include "mobility_block.cuh"
#include "rigid.cuh"
#include "wall_pair.cuh"

namespace rmw {

constexpr int kRigidThreads = 256;
constexpr int kSmemMaxM = 160;
constexpr int kSmemMaxM32 = 224;  // FP32 factorisation in shared memory up to 224 x 224 (196 KB)

// ---------------------------------------------------------------------------
// K and K^T
__global__ void k_times_u_kernel(const double *__restrict__ r, const double *__restrict__ xb,
                                 const int *__restrict__ blob_body, const double *__restrict__ u,
                                 double *__restrict__ out, int n, double alpha, double beta)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int b = blob_body[i];
    const double dx = r[3 * i] - xb[3 * b], dy = r[3 * i + 1] - xb[3 * b + 1], dz = r[3 * i + 2] - xb[3 * b + 2];
    const double *U = u + 6 * b;
    const double kx = U[0] + (U[4] * dz - U[5] * dy);
    const double ky = U[1] + (U[5] * dx - U[3] * dz);
    const double kz = U[2] + (U[3] * dy - U[4] * dx);
    if (beta == 0.0) {
        out[3 * i] = alpha * kx;
        out[3 * i + 1] = alpha * ky;
        out[3 * i + 2] = alpha * kz;
    } else {
        out[3 * i] = beta * out[3 * i] + alpha * kx;
        out[3 * i + 1] = beta * out[3 * i + 1] + alpha * ky;
        out[3 * i + 2] = beta * out[3 * i + 2] + alpha * kz;
    }
}

// one warp per body; out_b = alpha * K_b^T l
__global__ void kt_times_lambda_kernel(const double *__restrict__ r, const double *__restrict__ xb,
                                       const int *__restrict__ boff, const double *__restrict__ lam,
                                       double *__restrict__ out, int nb, double alpha)
{
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= nb) return;
    const int b = warp;
    const double cx = xb[3 * b], cy = xb[3 * b + 1], cz = xb[3 * b + 2];
    double s[6] = {0, 0, 0, 0, 0, 0};
    for (int i = boff[b] + lane; i < boff[b + 1]; i += 32) {
        const double lx = lam[3 * i], ly = lam[3 * i + 1], lz = lam[3 * i + 2];
        const double dx = r[3 * i] - cx, dy = r[3 * i + 1] - cy, dz = r[3 * i + 2] - cz;
        s[0] += lx; s[1] += ly; s[2] += lz;
        s[3] += dy * lz - dz * ly;
        s[4] += dz * lx - dx * lz;
        s[5] += dx * ly - dy * lx;
    }
#pragma unroll
    for (int c = 0; c < 6; ++c)
        for (int o = 16; o > 0; o >>= 1) s[c] += __shfl_xor_sync(0xffffffffu, s[c], o);
    if (lane < 6) out[6 * b + lane] = alpha * s[lane];
}

// The K parts of the mixed-precision operator in one pass, one warp per body:
// y_blob -= K U and y_body = -K^T lambda in FP32 arithmetic on offsets formed
// in FP64 (the accuracy class of the FP32-pair product they join)
__global__ void k_ops_f32_kernel(const double *__restrict__ r, const double *__restrict__ xb,
                                 const int *__restrict__ boff, const double *__restrict__ x, double *__restrict__ y,
                                 int n, int nb)
{
    const int b = (int)(((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (b >= nb) return;
    const double cx = xb[3 * b], cy = xb[3 * b + 1], cz = xb[3 * b + 2];
    const double *Ud = x + 3LL * n + 6LL * b;
    const float U0 = (float)Ud[0], U1 = (float)Ud[1], U2 = (float)Ud[2], U3 = (float)Ud[3], U4 = (float)Ud[4],
                U5 = (float)Ud[5];
    float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f, s4 = 0.f, s5 = 0.f;
    for (int i = boff[b] + lane; i < boff[b + 1]; i += 32) {
        const float dx = (float)(r[3 * i] - cx), dy = (float)(r[3 * i + 1] - cy), dz = (float)(r[3 * i + 2] - cz);
        const float lx = (float)x[3LL * i], ly = (float)x[3LL * i + 1], lz = (float)x[3LL * i + 2];
        s0 += lx; s1 += ly; s2 += lz;
        s3 += dy * lz - dz * ly;
        s4 += dz * lx - dx * lz;
        s5 += dx * ly - dy * lx;
        y[3LL * i] -= (double)(U0 + (U4 * dz - U5 * dy));
        y[3LL * i + 1] -= (double)(U1 + (U5 * dx - U3 * dz));
        y[3LL * i + 2] -= (double)(U2 + (U3 * dy - U4 * dx));
    }
    for (int o = 16; o > 0; o >>= 1) {
        s0 += __shfl_xor_sync(0xffffffffu, s0, o);
        s1 += __shfl_xor_sync(0xffffffffu, s1, o);
        s2 += __shfl_xor_sync(0xffffffffu, s2, o);
        s3 += __shfl_xor_sync(0xffffffffu, s3, o);
        s4 += __shfl_xor_sync(0xffffffffu, s4, o);
        s5 += __shfl_xor_sync(0xffffffffu, s5, o);
    }
    if (lane == 0) {
        double *yb = y + 3LL * n + 6LL * b;
        yb[0] = -(double)s0; yb[1] = -(double)s1; yb[2] = -(double)s2;
        yb[3] = -(double)s3; yb[4] = -(double)s4; yb[5] = -(double)s5;
    }
}

// ---------------------------------------------------------------------------
// dense per-body wall mobility M_b = nf * B M~(z_eff) B (row-major m x m)
template <typename T>
__global__ void body_mobility_kernel(const double *__restrict__ r, const int *__restrict__ boff,
                                     const long long *__restrict__ moff, double *__restrict__ M, double eta,
                                     double a)
{
    const int b = blockIdx.x;
    const int o = boff[b], nbl = boff[b + 1] - o, m = 3 * nbl;
    double *Mb = M + moff[b];
    const double nf = 1.0 / (8.0 * kPi * eta * a);
    for (int pq = threadIdx.x; pq < nbl * nbl; pq += blockDim.x) {
        const int p = pq / nbl, q = pq % nbl;
        double blk[3][3], sc;
        uf_block<T>(r, o + p, o + q, a, true, blk, &sc);
        sc *= nf;
        for (int u = 0; u < 3; ++u)
            for (int w = 0; w < 3; ++w) Mb[(long long)(3 * p + u) * m + 3 * q + w] = sc * blk[u][w];
    }
}

// Free-space variant (no wall, no regularisation): the blocks of
// rotne_prager_tensor (mobility/mobility.py:967-1015).
template <typename T>
__global__ void body_mobility_free_kernel(const double *__restrict__ r, const int *__restrict__ boff,
                                          const long long *__restrict__ moff, double *__restrict__ M, double eta,
                                          double a)
{
    const int b = blockIdx.x;
    const int o = boff[b], nbl = boff[b + 1] - o, m = 3 * nbl;
    double *Mb = M + moff[b];
    const double nf = 1.0 / (8.0 * kPi * eta * a);
    for (int pq = threadIdx.x; pq < nbl * nbl; pq += blockDim.x) {
        const int p = pq / nbl, q = pq % nbl;
        double blk[3][3], sc;
        uf_block<T>(r, o + p, o + q, a, false, blk, &sc);
        for (int u = 0; u < 3; ++u)
            for (int w = 0; w < 3; ++w) Mb[(long long)(3 * p + u) * m + 3 * q + w] = nf * blk[u][w];
    }
}

// ---------------------------------------------------------------------------
// Cholesky + inverse of every M_b.  A (m x m, row-major) is the working copy
// (shared memory or global); on exit minv holds M_b^-1, and lfac / linv (if
// non-null) hold L and L^-1 (lower triangles, upper zero).
template <typename T> __device__ __forceinline__ T fsqrt(T x);
template <> __device__ __forceinline__ double fsqrt<double>(double x) { return sqrt(fmax(x, 1e-300)); }
template <> __device__ __forceinline__ float fsqrt<float>(float x) { return sqrtf(fmaxf(x, 1e-30f)); }

// T = float: the preconditioner of the mixed-precision solves (a different but
// equally valid block-diagonal P; the FP64-accurate refinement residual
// decides convergence), factorised on the FP32 pipe; results stored as double.
template <typename T>
__device__ void factor_and_invert(T *A, int m, T *tmp, double *minv, double *lfac, double *linv, int *status)
{
    const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, wid = tid >> 5, nw = nt >> 5;
    // right-looking Cholesky, lower triangle: per column k the scale by the
    // pivot's square root (kept in tmp until the end, so that A[k][k] stays
    // readable for the whole step), then the trailing update with warps over
    // rows and lanes over columns
    for (int k = 0; k < m; ++k) {
        const T d = A[k * m + k];
        if (tid == 0) {
            if (!(d > T(0))) atomicExch(status, 1);  // not positive definite
            tmp[k] = fsqrt<T>(d);
        }
        const T dk = fsqrt<T>(d);
        for (int i = k + 1 + tid; i < m; i += nt) A[i * m + k] /= dk;
        __syncthreads();
        for (int i = k + 1 + wid; i < m; i += nw) {
            const T lik = A[i * m + k];
            for (int j = k + 1 + lane; j <= i; j += 32) A[i * m + j] -= lik * A[j * m + k];
        }
        __syncthreads();
    }
    for (int idx = tid; idx < m * m; idx += nt) {
        const int i = idx / m, j = idx - i * m;
        if (j > i) A[idx] = T(0);
        if (j == i) A[idx] = tmp[i];
        if (lfac) lfac[idx] = (j > i) ? 0.0 : (double)A[idx];
    }
    __syncthreads();
    // in-place inverse of the lower-triangular L, column by column from the right
    for (int j = m - 1; j >= 0; --j) {
        const T ajj = T(1) / A[j * m + j];
        for (int k = j + 1 + tid; k < m; k += nt) tmp[k] = A[k * m + j];
        __syncthreads();
        for (int i = j + 1 + tid; i < m; i += nt) {
            T sum = T(0);
            for (int k = j + 1; k <= i; ++k) sum += A[i * m + k] * tmp[k];
            A[i * m + j] = -ajj * sum;
        }
        if (tid == 0) A[j * m + j] = ajj;
        __syncthreads();
    }
    if (linv)
        for (int idx = tid; idx < m * m; idx += nt) linv[idx] = (double)A[idx];
    // M^-1 = L^-T L^-1 : minv[i][j] = sum_{k >= max(i,j)} X[k][i] X[k][j], warps
    // over the rows i, lanes over the columns j >= i
    for (int i = wid; i < m; i += nw)
        for (int j = i + lane; j < m; j += 32) {
            T sum = T(0);
            for (int k = j; k < m; ++k) sum += A[k * m + i] * A[k * m + j];
            minv[(long long)i * m + j] = (double)sum;
            minv[(long long)j * m + i] = (double)sum;
        }
}

template <typename T>
__global__ void pc_factor_smem_kernel(const double *__restrict__ M, const long long *__restrict__ moff,
                                      const int *__restrict__ boff, double *__restrict__ minv, double *lfac,
                                      double *linv, int *status)
{
    extern __shared__ __align__(16) unsigned char smraw[];
    T *sm = (T *)smraw;
    const int b = blockIdx.x;
    const int m = 3 * (boff[b + 1] - boff[b]);
    T *A = sm, *tmp = sm + m * m;
    const double *Mb = M + moff[b];
    for (int idx = threadIdx.x; idx < m * m; idx += blockDim.x) A[idx] = (T)Mb[idx];
    __syncthreads();
    factor_and_invert<T>(A, m, tmp, minv + moff[b], lfac ? lfac + moff[b] : nullptr, linv ? linv + moff[b] : nullptr,
                         status);
}

// M_b^-1 of the mixed solves' FP32 preconditioner (deterministic builds, m <=
// 16 R): in-place Gauss-Jordan sweeps with the matrix held in registers, one
// CTA of 16 x 16 threads per body, thread (ty, tx) owning rows ty + 16u and
// columns tx + 16w.  Step k publishes row k and column k through shared memory
// (double-buffered: one barrier per step) and updates every element:
//   A[k][k] <- 1/p,  A[k][j] <- A[k][j]/p,  A[i][k] <- -A[i][k]/p,
//   A[i][j] <- A[i][j] - A[i][k] A[k][j] / p,        p = A[k][k],
// which leaves A^-1 after m steps.  An SPD matrix needs no pivoting (every
// pivot is a positive Schur-complement diagonal); a non-positive pivot flags
// the body like the Cholesky does.  M^-1 is written symmetrised (the upper
// triangle both ways), as the apply kernels read it by columns.  m^3 fused
// multiply-adds on the FP32 pipe with no reduction and no dependent chain,
// against the Cholesky route's column loops.
template <int R>
__global__ void __launch_bounds__(256) pc_sweep_f32_kernel(const double *__restrict__ M,
                                                           const long long *__restrict__ moff,
                                                           const int *__restrict__ boff, double *__restrict__ minv,
                                                           float *__restrict__ minv32, int *status)
{
    __shared__ float colb[2][16 * R], rowb[2][16 * R];
    const int b = blockIdx.x;
    const int m = 3 * (boff[b + 1] - boff[b]);
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const double *Mb = M + moff[b];
    float A[R][R];
#pragma unroll
    for (int u = 0; u < R; ++u)
#pragma unroll
        for (int w = 0; w < R; ++w) {
            const int i = ty + 16 * u, j = tx + 16 * w;
            A[u][w] = (i < m && j < m) ? (float)Mb[(long long)i * m + j] : 0.f;
        }
    bool bad = false;
    for (int k = 0; k < m; ++k) {
        const int kb = k & 1, kr = k & 15, kq = k >> 4;
        if (tx == kr) {  // column k
#pragma unroll
            for (int w = 0; w < R; ++w)
                if (w == kq)
#pragma unroll
                    for (int u = 0; u < R; ++u) colb[kb][ty + 16 * u] = A[u][w];
        }
        if (ty == kr) {  // row k
#pragma unroll
            for (int u = 0; u < R; ++u)
                if (u == kq)
#pragma unroll
                    for (int w = 0; w < R; ++w) rowb[kb][tx + 16 * w] = A[u][w];
        }
        __syncthreads();
        const float p = rowb[kb][k];
        bad = bad || !(p > 0.f);
        const float ip = 1.f / p;
        float c[R], rr[R];
#pragma unroll
        for (int u = 0; u < R; ++u) c[u] = colb[kb][ty + 16 * u] * ip;
#pragma unroll
        for (int w = 0; w < R; ++w) rr[w] = rowb[kb][tx + 16 * w];
#pragma unroll
        for (int u = 0; u < R; ++u)
#pragma unroll
            for (int w = 0; w < R; ++w) A[u][w] = fmaf(-c[u], rr[w], A[u][w]);
        // row k, column k and the pivot replace the general update
        if (ty == kr) {
#pragma unroll
            for (int u = 0; u < R; ++u)
                if (u == kq)
#pragma unroll
                    for (int w = 0; w < R; ++w) A[u][w] = rr[w] * ip;
        }
        if (tx == kr) {
#pragma unroll
            for (int w = 0; w < R; ++w)
                if (w == kq)
#pragma unroll
                    for (int u = 0; u < R; ++u) A[u][w] = (ty == kr && u == kq) ? ip : -c[u];
        }
    }
    if (bad && threadIdx.x == 0) atomicExch(status, 1);  // not positive definite
    double *Mi = minv + moff[b];
    float *Mf = minv32 + moff[b];
#pragma unroll
    for (int u = 0; u < R; ++u)
#pragma unroll
        for (int w = 0; w < R; ++w) {
            const int i = ty + 16 * u, j = tx + 16 * w;
            if (i < m && j < m && i <= j) {
                Mi[(long long)i * m + j] = (double)A[u][w];
                Mi[(long long)j * m + i] = (double)A[u][w];
                Mf[(long long)i * m + j] = A[u][w];
                Mf[(long long)j * m + i] = A[u][w];
            }
        }
}

// M^-1 K and N = (K^T M^-1 K)^-1 of the FP32 deterministic build, in FP32
// from the sweep's FP32 M^-1 (as pc_body_kernel): written in both precisions,
// FP32 for the mixed solves' apply, FP64 for the FP64 apply
__global__ void pc_body_f32_kernel(const double *__restrict__ r, const double *__restrict__ xb,
                                   const int *__restrict__ boff, const long long *__restrict__ moff,
                                   const float *__restrict__ minv32, double *__restrict__ minvK,
                                   float *__restrict__ minvK32, double *__restrict__ nmat, float *__restrict__ nmat32,
                                   int *status)
{
    extern __shared__ float foff[];  // 3 per blob
    __shared__ float G[36];
    __shared__ float aug[6][12];
    const int b = blockIdx.x;
    const int o = boff[b], m = 3 * (boff[b + 1] - o);
    const float *Mi = minv32 + moff[b];
    const double cx = xb[3 * b], cy = xb[3 * b + 1], cz = xb[3 * b + 2];
    for (int p = threadIdx.x; p < m / 3; p += blockDim.x) {
        foff[3 * p] = (float)(r[3 * (o + p)] - cx);
        foff[3 * p + 1] = (float)(r[3 * (o + p) + 1] - cy);
        foff[3 * p + 2] = (float)(r[3 * (o + p) + 2] - cz);
    }
    __syncthreads();
    float *MK32 = minvK32 + 18LL * o;
    for (int t = threadIdx.x; t < m; t += blockDim.x) {
        float acc[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        for (int p = 0; p < m / 3; ++p) {
            const float dx = foff[3 * p], dy = foff[3 * p + 1], dz = foff[3 * p + 2];
            const float m0 = Mi[(long long)(3 * p) * m + t], m1 = Mi[(long long)(3 * p + 1) * m + t],
                        m2 = Mi[(long long)(3 * p + 2) * m + t];
            acc[0] += m0; acc[1] += m1; acc[2] += m2;
            acc[3] += -dz * m1 + dy * m2;
            acc[4] += dz * m0 - dx * m2;
            acc[5] += -dy * m0 + dx * m1;
        }
        for (int c = 0; c < 6; ++c) {
            MK32[6LL * t + c] = acc[c];
            minvK[18LL * o + 6LL * t + c] = (double)acc[c];
        }
    }
    __syncthreads();
    if (threadIdx.x < 36) {
        const int rr = threadIdx.x / 6, c = threadIdx.x % 6;
        float sum = 0.f;
        for (int p = 0; p < m / 3; ++p) {
            const float dx = foff[3 * p], dy = foff[3 * p + 1], dz = foff[3 * p + 2];
            const float k0 = MK32[6LL * (3 * p) + c], k1 = MK32[6LL * (3 * p + 1) + c], k2 = MK32[6LL * (3 * p + 2) + c];
            float kr;
            if (rr < 3) kr = (rr == 0) ? k0 : (rr == 1 ? k1 : k2);
            else if (rr == 3) kr = -dz * k1 + dy * k2;
            else if (rr == 4) kr = dz * k0 - dx * k2;
            else kr = -dy * k0 + dx * k1;
            sum += kr;
        }
        G[threadIdx.x] = sum;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int i = 0; i < 6; ++i)
            for (int j = 0; j < 12; ++j) aug[i][j] = (j < 6) ? G[6 * i + j] : (j - 6 == i ? 1.f : 0.f);
        for (int c = 0; c < 6; ++c) {
            int piv = c;
            for (int i = c + 1; i < 6; ++i)
                if (fabsf(aug[i][c]) > fabsf(aug[piv][c])) piv = i;
            if (piv != c)
                for (int j = 0; j < 12; ++j) {
                    const float t = aug[c][j]; aug[c][j] = aug[piv][j]; aug[piv][j] = t;
                }
            const float d = aug[c][c];
            if (d == 0.f) { atomicExch(status, 2); continue; }
            for (int j = 0; j < 12; ++j) aug[c][j] /= d;
            for (int i = 0; i < 6; ++i) {
                if (i == c) continue;
                const float f = aug[i][c];
                for (int j = 0; j < 12; ++j) aug[i][j] -= f * aug[c][j];
            }
        }
        for (int i = 0; i < 6; ++i)
            for (int j = 0; j < 6; ++j) {
                nmat32[36 * b + 6 * i + j] = aug[i][6 + j];
                nmat[36 * b + 6 * i + j] = (double)aug[i][6 + j];
            }
    }
}

int alloc_pc32(RigidSystem &S)
{
    // each array on its own, so that a failed allocation leaves no half-set state behind
    if (!S.minv32) RMW_CUDA(cudaMalloc(&S.minv32, sizeof(float) * (size_t)S.moff_h[S.nb]));
    if (!S.minvK32) RMW_CUDA(cudaMalloc(&S.minvK32, sizeof(float) * 18 * (size_t)S.n));
    if (!S.nmat32) RMW_CUDA(cudaMalloc(&S.nmat32, sizeof(float) * 36 * (size_t)S.nb));
    if (!S.blob32) RMW_CUDA(cudaMalloc(&S.blob32, sizeof(float4) * (size_t)S.n));
    return RMW_OK;
}

static void launch_pc_sweep_f32(int R, int nb, const double *M, const long long *moff, const int *boff,
                                double *minv, float *minv32, int *status, cudaStream_t st)
{
    switch (R) {
    case 1: pc_sweep_f32_kernel<1><<<nb, 256, 0, st>>>(M, moff, boff, minv, minv32, status); break;
    case 2: pc_sweep_f32_kernel<2><<<nb, 256, 0, st>>>(M, moff, boff, minv, minv32, status); break;
    case 3: pc_sweep_f32_kernel<3><<<nb, 256, 0, st>>>(M, moff, boff, minv, minv32, status); break;
    case 4: pc_sweep_f32_kernel<4><<<nb, 256, 0, st>>>(M, moff, boff, minv, minv32, status); break;
    case 5: pc_sweep_f32_kernel<5><<<nb, 256, 0, st>>>(M, moff, boff, minv, minv32, status); break;
    case 6: pc_sweep_f32_kernel<6><<<nb, 256, 0, st>>>(M, moff, boff, minv, minv32, status); break;
    case 7: pc_sweep_f32_kernel<7><<<nb, 256, 0, st>>>(M, moff, boff, minv, minv32, status); break;
    default: pc_sweep_f32_kernel<8><<<nb, 256, 0, st>>>(M, moff, boff, minv, minv32, status); break;
    }
}
constexpr int kSweepMaxM = 128;

// global-memory variant: M is overwritten (it is the working copy), tmp is m doubles per body
__global__ void pc_factor_global_kernel(double *__restrict__ M, const long long *__restrict__ moff,
                                        const int *__restrict__ boff, double *__restrict__ minv, double *lfac,
                                        double *linv, double *tmpg, int *status)
{
    const int b = blockIdx.x;
    const int m = 3 * (boff[b + 1] - boff[b]);
    factor_and_invert<double>(M + moff[b], m, tmpg + 3 * boff[b], minv + moff[b], lfac ? lfac + moff[b] : nullptr,
                              linv ? linv + moff[b] : nullptr, status);
}

// M^-1 K (m x 6) and N = (K^T M^-1 K)^-1 (6 x 6) per body; the blob offsets
// from the centre staged in shared memory (3 doubles per blob)
__global__ void pc_body_kernel(const double *__restrict__ r, const double *__restrict__ xb,
                               const int *__restrict__ boff, const long long *__restrict__ moff,
                               const double *__restrict__ minv, double *__restrict__ minvK,
                               double *__restrict__ nmat, int *status)
{
    extern __shared__ double doff[];
    __shared__ double G[36];
    __shared__ double aug[6][12];
    const int b = blockIdx.x;
    const int o = boff[b], m = 3 * (boff[b + 1] - o);
    const double *Mi = minv + moff[b];
    double *MK = minvK + 6LL * 3 * o;
    const double cx = xb[3 * b], cy = xb[3 * b + 1], cz = xb[3 * b + 2];
    if (threadIdx.x < 36) G[threadIdx.x] = 0.0;
    for (int p = threadIdx.x; p < m / 3; p += blockDim.x) {
        doff[3 * p] = r[3 * (o + p)] - cx;
        doff[3 * p + 1] = r[3 * (o + p) + 1] - cy;
        doff[3 * p + 2] = r[3 * (o + p) + 2] - cz;
    }
    __syncthreads();
    // MK[t][c] = sum_k Minv[t][k] K[k][c]; K row k = 3p+u: J part e_u, rot part
    // R_p row u.  M^-1 is symmetric: Minv[k][t] is read, coalesced over t.
    for (int t = threadIdx.x; t < m; t += blockDim.x) {
        double acc[6] = {0, 0, 0, 0, 0, 0};
        for (int p = 0; p < m / 3; ++p) {
            const double dx = doff[3 * p], dy = doff[3 * p + 1], dz = doff[3 * p + 2];
            const double m0 = Mi[(long long)(3 * p) * m + t], m1 = Mi[(long long)(3 * p + 1) * m + t],
                         m2 = Mi[(long long)(3 * p + 2) * m + t];
            acc[0] += m0; acc[1] += m1; acc[2] += m2;
            // R_p = [[0, dz, -dy], [-dz, 0, dx], [dy, -dx, 0]] (R w = w x d)
            acc[3] += -dz * m1 + dy * m2;
            acc[4] += dz * m0 - dx * m2;
            acc[5] += -dy * m0 + dx * m1;
        }
        for (int c = 0; c < 6; ++c) MK[6LL * t + c] = acc[c];
    }
    __syncthreads();
    // G = K^T (M^-1 K)
    if (threadIdx.x < 36) {
        const int rr = threadIdx.x / 6, c = threadIdx.x % 6;
        double s = 0.0;
        for (int p = 0; p < m / 3; ++p) {
            const double dx = doff[3 * p], dy = doff[3 * p + 1], dz = doff[3 * p + 2];
            const double k0 = MK[6LL * (3 * p) + c], k1 = MK[6LL * (3 * p + 1) + c], k2 = MK[6LL * (3 * p + 2) + c];
            double kr;
            if (rr < 3) kr = (rr == 0) ? k0 : (rr == 1 ? k1 : k2);
            else if (rr == 3) kr = -dz * k1 + dy * k2;
            else if (rr == 4) kr = dz * k0 - dx * k2;
            else kr = -dy * k0 + dx * k1;
            s += kr;
        }
        G[threadIdx.x] = s;
    }
    __syncthreads();
    // invert the symmetric positive definite 6x6 by Gauss-Jordan with partial pivoting
    if (threadIdx.x == 0) {
        for (int i = 0; i < 6; ++i)
            for (int j = 0; j < 12; ++j) aug[i][j] = (j < 6) ? G[6 * i + j] : (j - 6 == i ? 1.0 : 0.0);
        for (int c = 0; c < 6; ++c) {
            int piv = c;
            for (int i = c + 1; i < 6; ++i)
                if (fabs(aug[i][c]) > fabs(aug[piv][c])) piv = i;
            if (piv != c)
                for (int j = 0; j < 12; ++j) {
                    double t = aug[c][j]; aug[c][j] = aug[piv][j]; aug[piv][j] = t;
                }
            const double d = aug[c][c];
            if (d == 0.0) { atomicExch(status, 2); continue; }
            for (int j = 0; j < 12; ++j) aug[c][j] /= d;
            for (int i = 0; i < 6; ++i) {
                if (i == c) continue;
                const double f = aug[i][c];
                for (int j = 0; j < 12; ++j) aug[i][j] -= f * aug[c][j];
            }
        }
        for (int i = 0; i < 6; ++i)
            for (int j = 0; j < 6; ++j) nmat[36 * b + 6 * i + j] = aug[i][6 + j];
    }
}

// ---------------------------------------------------------------------------
// preconditioner apply, one CTA per body
__global__ void pc_apply_kernel(const double *__restrict__ x, double *__restrict__ y,
                                const double *__restrict__ r, const double *__restrict__ xb,
                                const int *__restrict__ boff, const long long *__restrict__ moff,
                                const double *__restrict__ minv, const double *__restrict__ minvK,
                                const double *__restrict__ nmat, int n)
{
    extern __shared__ double sh[];
    const int b = blockIdx.x;
    const int o = boff[b], m = 3 * (boff[b + 1] - o);
    double *s = sh;            // m
    double *lt = sh + m;       // m
    double *red = sh + 2 * m;  // 6 * (blockDim/32)
    __shared__ double Y[6];
    const double *Mi = minv + moff[b];
    const int tid = threadIdx.x, nt = blockDim.x;
    for (int t = tid; t < m; t += nt) s[t] = x[3LL * o + t];
    __syncthreads();
    for (int t = tid; t < m; t += nt) {
        double acc = 0.0;
        for (int k = 0; k < m; ++k) acc += Mi[(long long)k * m + t] * s[k];  // M^-1 symmetric: coalesced
        lt[t] = acc;
    }
    __syncthreads();
    // K^T l~
    const double cx = xb[3 * b], cy = xb[3 * b + 1], cz = xb[3 * b + 2];
    double p6[6] = {0, 0, 0, 0, 0, 0};
    for (int p = tid; p < m / 3; p += nt) {
        const int i = o + p;
        const double dx = r[3 * i] - cx, dy = r[3 * i + 1] - cy, dz = r[3 * i + 2] - cz;
        const double lx = lt[3 * p], ly = lt[3 * p + 1], lz = lt[3 * p + 2];
        p6[0] += lx; p6[1] += ly; p6[2] += lz;
        p6[3] += dy * lz - dz * ly;
        p6[4] += dz * lx - dx * lz;
        p6[5] += dx * ly - dy * lx;
    }
    const int lane = tid & 31, wid = tid >> 5;
#pragma unroll
    for (int c = 0; c < 6; ++c) {
        for (int off = 16; off > 0; off >>= 1) p6[c] += __shfl_xor_sync(0xffffffffu, p6[c], off);
        if (lane == 0) red[6 * wid + c] = p6[c];
    }
    __syncthreads();
    if (tid < 6) {
        double ktl = 0.0;
        for (int w = 0; w < nt / 32; ++w) ktl += red[6 * w + tid];
        red[6 * (nt / 32) + tid] = -x[3LL * n + 6 * b + tid] - ktl;  // -F - K^T l~
    }
    __syncthreads();
    if (tid < 6) {
        const double *Nb = nmat + 36 * b;
        const double *rhs = red + 6 * (nt / 32);
        double u = 0.0;
        for (int c = 0; c < 6; ++c) u += Nb[6 * tid + c] * rhs[c];
        Y[tid] = u;
        y[3LL * n + 6 * b + tid] = u;
    }
    __syncthreads();
    const double *MK = minvK + 6LL * 3 * o;
    for (int t = tid; t < m; t += nt) {
        double acc = lt[t];
        for (int c = 0; c < 6; ++c) acc += MK[6LL * t + c] * Y[c];
        y[3LL * o + t] = acc;
    }
}

// y_b = T_b x_b (T lower triangular, row-major) or T_b^T x_b, per body;
// blockIdx.y selects one of several vectors (stride ld)
__global__ void block_tri_mult_kernel(const double *__restrict__ T, const long long *__restrict__ moff,
                                      const int *__restrict__ boff, const double *__restrict__ x,
                                      double *__restrict__ y, int transpose, long long ld)
{
    extern __shared__ double xs[];
    const int b = blockIdx.x;
    x += (long long)blockIdx.y * ld;
    y += (long long)blockIdx.y * ld;
    const int o = boff[b], m = 3 * (boff[b + 1] - o);
    const double *Tb = T + moff[b];
    for (int t = threadIdx.x; t < m; t += blockDim.x) xs[t] = x[3LL * o + t];
    __syncthreads();
    for (int t = threadIdx.x; t < m; t += blockDim.x) {
        double acc = 0.0;
        if (!transpose)
            for (int k = 0; k <= t; ++k) acc += Tb[(long long)t * m + k] * xs[k];
        else
            for (int k = t; k < m; ++k) acc += Tb[(long long)k * m + t] * xs[k];
        y[3LL * o + t] = acc;
    }
}

// The same products for all nvec vectors of a body in one CTA, in FP32 (the
// mixed-precision Lanczos operator, whose tolerance is 1e-3): the factor
// block is read once, converted into shared memory, and applied to every
// vector, instead of one FP64 pass over the block per vector.  Shared
// memory: m^2 + nvec m floats.  In place (y == x) is safe: the body's slice of
// every vector is staged before any is written.
// y_v = T x_v (or T^T x_v) for nvec vectors per body in FP32, one CTA per
// body.  The factor sits in shared memory as S[k][t] (T transposed for T x,
// as is for T^T x), so that every thread owns one output row t and all rows
// walk k = 0..m-1 together: S reads are consecutive over the threads, the
// vectors' entries x[k][v] are broadcast, and each thread runs sixteen
// independent FMA chains (sixteen vectors at a time).  The walk covers the
// factor's zero triangle too (exact: those entries are zero).
template <typename TT>
__global__ void block_tri_mult_f32_kernel(const TT *__restrict__ T, const long long *__restrict__ moff,
                                          const int *__restrict__ boff, const double *x, double *y, int transpose,
                                          long long ld, int nvec)
{
    extern __shared__ __align__(16) float tsm[];
    const int b = blockIdx.x;
    const int o = boff[b], m = 3 * (boff[b + 1] - o);
    const int nv16 = (nvec + 15) & ~15;
    float *Ss = tsm, *xs = tsm + (((size_t)m * m + 3) & ~(size_t)3);  // xs[k * nv16 + v], 16-byte aligned
    const TT *Tb = T + moff[b];
    // the factor's load is the latency-bound part (a few CTAs per SM): 16-byte
    // loads, four in flight per thread
    constexpr int kV = 16 / sizeof(TT);  // elements per 16-byte load
    const int mm = m * m;
    const bool vec = (mm % kV) == 0 && (moff[b] % kV) == 0;
    auto put = [&](int e, float val) {
        if (transpose) {
            Ss[e] = val;
        } else {
            const int i = e / m, j = e - i * m;
            Ss[j * m + i] = val;
        }
    };
    if (vec) {
        const int nq = mm / kV;
#pragma unroll 4
        for (int q = threadIdx.x; q < nq; q += blockDim.x) {
            if constexpr (sizeof(TT) == 4) {
                const float4 w = reinterpret_cast<const float4 *>(Tb)[q];
                put(4 * q, w.x); put(4 * q + 1, w.y); put(4 * q + 2, w.z); put(4 * q + 3, w.w);
            } else {
                const double2 w = reinterpret_cast<const double2 *>(Tb)[q];
                put(2 * q, (float)w.x); put(2 * q + 1, (float)w.y);
            }
        }
    } else {
#pragma unroll 4
        for (int e = threadIdx.x; e < mm; e += blockDim.x) put(e, (float)Tb[e]);
    }
#pragma unroll 4
    for (int e = threadIdx.x; e < nv16 * m; e += blockDim.x) {
        const int v = e / m, k = e - v * m;
        xs[k * nv16 + v] = (v < nvec) ? (float)x[(long long)v * ld + 3LL * o + k] : 0.f;
    }
    __syncthreads();
    for (int t = threadIdx.x; t < m; t += blockDim.x)
        for (int v0 = 0; v0 < nvec; v0 += 16) {
            float acc[16];
#pragma unroll
            for (int q = 0; q < 16; ++q) acc[q] = 0.f;
#pragma unroll 2
            for (int k = 0; k < m; ++k) {
                const float sk = Ss[k * m + t];
                const float4 *xk = reinterpret_cast<const float4 *>(xs + k * nv16 + v0);
#pragma unroll
                for (int g = 0; g < 4; ++g) {
                    const float4 xv = xk[g];
                    acc[4 * g] = fmaf(sk, xv.x, acc[4 * g]);
                    acc[4 * g + 1] = fmaf(sk, xv.y, acc[4 * g + 1]);
                    acc[4 * g + 2] = fmaf(sk, xv.z, acc[4 * g + 2]);
                    acc[4 * g + 3] = fmaf(sk, xv.w, acc[4 * g + 3]);
                }
            }
#pragma unroll
            for (int q = 0; q < 16; ++q)
                if (v0 + q < nvec) y[(long long)(v0 + q) * ld + 3LL * o + t] = acc[q];
        }
}

// ---------------------------------------------------------------------------
// body kinematics (FP64)
// r_i = R(q_b) r_ref_i + x_b  (body/body.py:64-78, quaternion.py:42-51)
__global__ void blob_positions_kernel(const double *__restrict__ xb, const double *__restrict__ q,
                                      const double *__restrict__ rref, const int *__restrict__ blob_body,
                                      double *__restrict__ r, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int b = blob_body[i];
    const double s = q[4 * b], p0 = q[4 * b + 1], p1 = q[4 * b + 2], p2 = q[4 * b + 3];
    const double dg = s * s - 0.5;
    const double R00 = 2 * (p0 * p0 + dg), R01 = 2 * (p0 * p1 - s * p2), R02 = 2 * (p0 * p2 + s * p1);
    const double R10 = 2 * (p1 * p0 + s * p2), R11 = 2 * (p1 * p1 + dg), R12 = 2 * (p1 * p2 - s * p0);
    const double R20 = 2 * (p2 * p0 - s * p1), R21 = 2 * (p2 * p1 + s * p0), R22 = 2 * (p2 * p2 + dg);
    const double a = rref[3 * i], bb = rref[3 * i + 1], c = rref[3 * i + 2];
    r[3 * i] = R00 * a + R01 * bb + R02 * c + xb[3 * b];
    r[3 * i + 1] = R10 * a + R11 * bb + R12 * c + xb[3 * b + 1];
    r[3 * i + 2] = R20 * a + R21 * bb + R22 * c + xb[3 * b + 2];
}

// x_new = x + U dt ; q_new = from_rotation(w dt) * q   (quaternion_integrator_multi_bodies.py:308-312)
__global__ void euler_update_kernel(const double *__restrict__ x, const double *__restrict__ q,
                                    const double *__restrict__ vel, double dt, double *__restrict__ xn,
                                    double *__restrict__ qn, int nb)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    const double *U = vel + 6 * b;
    xn[3 * b] = x[3 * b] + U[0] * dt;
    xn[3 * b + 1] = x[3 * b + 1] + U[1] * dt;
    xn[3 * b + 2] = x[3 * b + 2] + U[2] * dt;
    const double f0 = U[3] * dt, f1 = U[4] * dt, f2 = U[5] * dt;
    const double ph = sqrt(f0 * f0 + f1 * f1 + f2 * f2);
    const double s1 = cos(ph / 2.0);
    double p0 = 0.0, p1 = 0.0, p2 = 0.0;
    if (ph != 0.0) {
        const double sf = sin(ph / 2.0) / ph;
        p0 = sf * f0; p1 = sf * f1; p2 = sf * f2;
    }
    const double s2 = q[4 * b], r0 = q[4 * b + 1], r1 = q[4 * b + 2], r2 = q[4 * b + 3];
    // (s1, p) * (s2, r) = (s1 s2 - p.r, s1 r + s2 p + p x r)
    qn[4 * b] = s1 * s2 - (p0 * r0 + p1 * r1 + p2 * r2);
    qn[4 * b + 1] = s1 * r0 + s2 * p0 + (p1 * r2 - p2 * r1);
    qn[4 * b + 2] = s1 * r1 + s2 * p1 + (p2 * r0 - p0 * r2);
    qn[4 * b + 3] = s1 * r2 + s2 * p2 + (p0 * r1 - p1 * r0);
}

// count of blobs with z < zmin (Body.check_function, body/body.py:118-140)
__global__ void count_below_kernel(const double *__restrict__ r, int n, double zmin, int *__restrict__ count)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool below = (i < n) && (r[3 * i + 2] < zmin);
    const unsigned m = __ballot_sync(0xffffffffu, below);
    if ((threadIdx.x & 31) == 0 && m) atomicAdd(count, __popc(m));
}

// ---------------------------------------------------------------------------
// host side
__global__ void double_to_float_kernel(const double *__restrict__ x, float *__restrict__ y, long long n)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        y[i] = (float)x[i];
}

static int build_pc(RigidSystem &S, bool stochastic, bool fp32 = false)
{
    cudaStream_t st = S.st;
    S.pc32_ready = S.pc32_blocks = S.linv32_ready = false;  // the FP32 copies follow the arrays rewritten here
    const long long tot = S.moff_h[S.nb];
    // working copy of the dense body mobilities (stream-ordered, freed below)
    void *ws = nullptr;
    const size_t ws_bytes = sizeof(double) * ((size_t)tot + 3 * (size_t)S.n);
    RMW_CUDA(rmw::dmalloc_async(&ws, ws_bytes, st));
    double *M = (double *)ws;
    double *tmpg = M + tot;
    if (!S.minv) {
        RMW_CUDA(cudaMalloc(&S.minv, sizeof(double) * tot));
        RMW_CUDA(cudaMalloc(&S.minvK, sizeof(double) * 6 * 3 * (size_t)S.n));
        RMW_CUDA(cudaMalloc(&S.nmat, sizeof(double) * 36 * (size_t)S.nb));
    }
    if (stochastic && !S.lfac) {
        RMW_CUDA(cudaMalloc(&S.lfac, sizeof(double) * tot));
        RMW_CUDA(cudaMalloc(&S.linv, sizeof(double) * tot));
    }
    RMW_CUDA(cudaMemsetAsync(S.dstatus, 0, sizeof(int), st));
    if (fp32 && S.max_m > kSmemMaxM32) fp32 = false;
    if (fp32) {
        if (S.wall) body_mobility_kernel<float><<<S.nb, kRigidThreads, 0, st>>>(S.r, S.boff, S.moff, M, S.eta, S.a);
        else body_mobility_free_kernel<float><<<S.nb, kRigidThreads, 0, st>>>(S.r, S.boff, S.moff, M, S.eta, S.a);
    } else {
        if (S.wall) body_mobility_kernel<double><<<S.nb, kRigidThreads, 0, st>>>(S.r, S.boff, S.moff, M, S.eta, S.a);
        else body_mobility_free_kernel<double><<<S.nb, kRigidThreads, 0, st>>>(S.r, S.boff, S.moff, M, S.eta, S.a);
    }
    double *lf = stochastic ? S.lfac : nullptr, *li = stochastic ? S.linv : nullptr;
    const bool sweep = fp32 && !stochastic && S.max_m <= kSweepMaxM;
    if (sweep) {
        // the blocks in FP32 directly: M^-1, M^-1 K and N also as the mixed solves' FP32 copies
        if (int rc = alloc_pc32(S)) {
            cudaFreeAsync(ws, st);
            return rc;
        }
        launch_pc_sweep_f32((S.max_m + 15) / 16, S.nb, M, S.moff, S.boff, S.minv, S.minv32, S.dstatus, st);
    } else if (fp32) {
        const size_t sm = sizeof(float) * ((size_t)S.max_m * S.max_m + S.max_m);
        RMW_CUDA(cudaFuncSetAttribute(pc_factor_smem_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)sm));
        pc_factor_smem_kernel<float><<<S.nb, kRigidThreads, sm, st>>>(M, S.moff, S.boff, S.minv, lf, li, S.dstatus);
    } else if (S.max_m <= kSmemMaxM) {
        const size_t sm = sizeof(double) * ((size_t)S.max_m * S.max_m + S.max_m);
        RMW_CUDA(cudaFuncSetAttribute(pc_factor_smem_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)sm));
        pc_factor_smem_kernel<double><<<S.nb, kRigidThreads, sm, st>>>(M, S.moff, S.boff, S.minv, lf, li, S.dstatus);
    } else {
        pc_factor_global_kernel<<<S.nb, kRigidThreads, 0, st>>>(M, S.moff, S.boff, S.minv, lf, li, tmpg, S.dstatus);
    }
    if (sweep) {
        pc_body_f32_kernel<<<S.nb, 128, sizeof(float) * (size_t)S.max_m, st>>>(
            S.r, S.xb, S.boff, S.moff, S.minv32, S.minvK, S.minvK32, S.nmat, S.nmat32, S.dstatus);
    } else {
        const size_t sm = sizeof(double) * (size_t)S.max_m;
        if (sm > 48 * 1024)
            RMW_CUDA(cudaFuncSetAttribute(pc_body_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        pc_body_kernel<<<S.nb, 128, sm, st>>>(S.r, S.xb, S.boff, S.moff, S.minv, S.minvK, S.nmat, S.dstatus);
    }
    RMW_CHECK_LAUNCH("preconditioner build");
    int hstat = 0;
    RMW_CUDA(cudaMemcpyAsync(&hstat, S.dstatus, sizeof(int), cudaMemcpyDeviceToHost, st));
    RMW_CUDA(cudaFreeAsync(ws, st));
    RMW_CUDA(cudaStreamSynchronize(st));
    if (hstat != 0 && fp32) return build_pc(S, stochastic, false);  // FP32 factorisation failed: FP64 instead
    if (hstat == 1) return fail(RMW_ERR_NONFINITE, "body mobility matrix is not positive definite (Cholesky failed)");
    if (hstat == 2) return fail(RMW_ERR_NONFINITE, "singular 6x6 body resistance K^T M^-1 K");
    if (fp32 && stochastic) {
        // the FP32 copy of L^-1 for the mixed multi-vector Lanczos products
        if (!S.linv32) RMW_CUDA(cudaMalloc(&S.linv32, sizeof(float) * (size_t)tot));
        const unsigned g = (unsigned)std::min<long long>((tot + 255) / 256, 152LL * 16);
        double_to_float_kernel<<<g, 256, 0, st>>>(S.linv, S.linv32, tot);
        RMW_CHECK_LAUNCH("FP32 copy of L^-1");
        S.linv32_ready = true;
    }
    S.pc_ready = true;
    S.stoch_ready = stochastic;
    S.pc_fp32 = fp32;
    S.pc32_ready = false;
    S.pc32_blocks = sweep;  // the FP32 copies of the blocks are already written
    return RMW_OK;
}

int rigid_mobility(RigidSystem &S, const double *v, double *y, int mode)
{
    if (!S.wall) return nowall_product(RMW_UF, S.r, v, y, S.n, S.eta, S.a, S.L, mode, S.st);
    if (S.batch) return wall_product_batched(*S.batch, RMW_UF, S.r, v, y, S.eta, S.a, mode, S.st);
    return wall_product(RMW_UF, S.r, v, y, S.n, S.eta, S.a, S.L, mode, S.st);
}

int rigid_apply(RigidSystem &S, const double *x, double *y, int mode)
{
    cudaStream_t st = S.st;
    // y_blob = M l
    if (int rc = rigid_mobility(S, x, y, mode)) return rc;
    const int tb = 256;
    if (mode == RMW_MODE_MIXED) {
        k_ops_f32_kernel<<<(unsigned)(((long long)S.nb * 32 + tb - 1) / tb), tb, 0, st>>>(S.r, S.xb, S.boff, x, y,
                                                                                          S.n, S.nb);
        RMW_CHECK_LAUNCH("rigid operator");
        return RMW_OK;
    }
    // y_blob -= K U
    k_times_u_kernel<<<(S.n + tb - 1) / tb, tb, 0, st>>>(S.r, S.xb, S.blob_body, x + 3LL * S.n, y, S.n, -1.0, 1.0);
    // y_body = -K^T l
    kt_times_lambda_kernel<<<(S.nb * 32 + tb - 1) / tb, tb, 0, st>>>(S.r, S.xb, S.boff, x, y + 3LL * S.n, S.nb,
                                                                       -1.0);
    RMW_CHECK_LAUNCH("rigid operator");
    return RMW_OK;
}

int rigid_apply_pc(RigidSystem &S, const double *x, double *y)
{
    if (!S.pc_ready) return fail(RMW_ERR_ARG, "preconditioner not built (call rmw_rigid_build_pc)");
    if (S.nf_on) return nearfield_apply_pc(S, x, y);
    return rigid_apply_pc_plain(S, x, y);
}

int rigid_apply_pc_plain(RigidSystem &S, const double *x, double *y)
{
    const int nt = 128;
    const size_t sm = sizeof(double) * (2 * (size_t)S.max_m + 6 * (nt / 32 + 1));
    if (sm > 48 * 1024)
        RMW_CUDA(cudaFuncSetAttribute(pc_apply_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    void *tok = nullptr;
    if (int rc = trace_begin(TRACE_PC, S.st, &tok)) return rc;
    pc_apply_kernel<<<S.nb, nt, sm, S.st>>>(x, y, S.r, S.xb, S.boff, S.moff, S.minv, S.minvK, S.nmat, S.n);
    if (int rc = trace_end(tok, S.st)) return rc;
    RMW_CHECK_LAUNCH("preconditioner apply");
    return RMW_OK;
}

static int tri_mult(RigidSystem &S, const double *T, const double *x, double *y, int transpose, int nvec = 1)
{
    const size_t sm = sizeof(double) * (size_t)S.max_m;
    block_tri_mult_kernel<<<dim3(S.nb, nvec), 128, sm, S.st>>>(T, S.moff, S.boff, x, y, transpose, 3LL * S.n);
    RMW_CHECK_LAUNCH("block triangular multiply");
    return RMW_OK;
}

int rigid_mobility_pc(RigidSystem &S, const double *w, double *y, int mode)
{
    if (!S.stoch_ready) return fail(RMW_ERR_ARG, "stochastic preconditioner not built");
    // y = L^-1 M L^-T w   (P = L^-T, reference: P^T M P with P = U^-1, U = L^T)
    if (int rc = tri_mult(S, S.linv, w, S.tmp3n, 1)) return rc;
    if (int rc = rigid_mobility(S, S.tmp3n, y, mode)) return rc;
    // in place is safe per body: each CTA stages its own slice in shared memory first
    return tri_mult(S, S.linv, y, y, 0);
}

// FP32 form of tri_mult for all nvec vectors per body (mixed mode); false when
// a body's block does not fit the shared memory
static size_t tri_mult_f32_smem(const RigidSystem &S, int nvec)
{
    return ((((size_t)S.max_m * S.max_m + 3) & ~(size_t)3) + (size_t)((nvec + 15) & ~15) * S.max_m) * sizeof(float);
}
static bool tri_mult_f32_fits(const RigidSystem &S, int nvec) { return tri_mult_f32_smem(S, nvec) <= 200 * 1024; }
// T: the FP64 factor; its FP32 copy is read instead when the build made one
// (half the bytes, no conversion per element and launch)
static int tri_mult_f32(RigidSystem &S, const double *T, const double *x, double *y, int transpose, int nvec)
{
    const size_t sm = tri_mult_f32_smem(S, nvec);
    const bool f32 = T == S.linv && S.linv32_ready;
    if (sm > 48 * 1024) {
        if (f32)
            RMW_CUDA(cudaFuncSetAttribute(block_tri_mult_f32_kernel<float>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        else
            RMW_CUDA(cudaFuncSetAttribute(block_tri_mult_f32_kernel<double>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    }
    if (f32)
        block_tri_mult_f32_kernel<float><<<S.nb, 256, sm, S.st>>>(S.linv32, S.moff, S.boff, x, y, transpose,
                                                                   3LL * S.n, nvec);
    else
        block_tri_mult_f32_kernel<double><<<S.nb, 256, sm, S.st>>>(T, S.moff, S.boff, x, y, transpose, 3LL * S.n,
                                                                    nvec);
    RMW_CHECK_LAUNCH("block triangular multiply (FP32)");
    return RMW_OK;
}

int rigid_mobility_pc_multi(RigidSystem &S, const double *W, double *Y, int nvec, int mode, double *tmp,
                            const unsigned char *active)
{
    if (!S.stoch_ready) return fail(RMW_ERR_ARG, "stochastic preconditioner not built");
    const long long ld = 3LL * S.n;
    if (mode == RMW_MODE_MIXED && S.wall && tri_mult_f32_fits(S, nvec)) {
        if (int rc = tri_mult_f32(S, S.linv, W, tmp, 1, nvec)) return rc;
        if (int rc = wall_uf_multi(S.r, tmp, ld, Y, ld, nvec, S.n, S.eta, S.a, S.batch, S.st, active)) return rc;
        return tri_mult_f32(S, S.linv, Y, Y, 0, nvec);
    }
    if (int rc = tri_mult(S, S.linv, W, tmp, 1, nvec)) return rc;
    if (mode == RMW_MODE_MIXED && S.wall) {
        if (int rc = wall_uf_multi(S.r, tmp, ld, Y, ld, nvec, S.n, S.eta, S.a, S.batch, S.st, active)) return rc;
    } else {
        for (int q = 0; q < nvec; ++q)
            if (int rc = rigid_mobility(S, tmp + q * ld, Y + q * ld, mode)) return rc;
    }
    return tri_mult(S, S.linv, Y, Y, 0, nvec);
}

int rigid_P_inv_mult_multi(RigidSystem &S, const double *W, double *Y, int nvec, int mode)
{
    if (!S.stoch_ready) return fail(RMW_ERR_ARG, "stochastic preconditioner not built");
    // mixed: the FP32 multiply (each body's factor read once for all vectors)
    if (mode == RMW_MODE_MIXED && tri_mult_f32_fits(S, nvec)) return tri_mult_f32(S, S.lfac, W, Y, 0, nvec);
    return tri_mult(S, S.lfac, W, Y, 0, nvec);
}

int rigid_P_inv_mult(RigidSystem &S, const double *w, double *y)
{
    if (!S.stoch_ready) return fail(RMW_ERR_ARG, "stochastic preconditioner not built");
    return tri_mult(S, S.lfac, w, y, 0);
}

static void free_system(RigidSystem *S)
{
    int cur = 0;
    cudaGetDevice(&cur);
    cudaSetDevice(S->device);
    void *ptrs[] = {S->boff, S->blob_body, S->moff, S->r, S->xb, S->minv, S->minvK, S->nmat, S->lfac, S->linv,
                    S->dstatus, S->tmp3n, S->perm, S->nf_off, S->nf_ex_idx, S->nf_ln_idx, S->nf_mp_idx, S->nf_cnt, S->nf_range,
                    S->nf_G, S->nf_mom, S->nf_v, S->nf_z, S->nf_part, S->minv32, S->minvK32, S->nmat32,
                    S->blob32, S->nf_mom32, S->nf_lam32, S->nf_G32, S->linv32};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    if (S->batch) {
        wall_batch_free(*S->batch);
        delete S->batch;
    }
    cudaSetDevice(cur);
    delete S;
}

}  // namespace rmw

// ---------------------------------------------------------------------------
// C ABI
using rmw::RigidSystem;

extern "C" {

int rmw_rigid_create(void **out, int64_t n_bodies, const int64_t *blob_offsets_host, double eta, double a,
                     const double *L_host, void *stream)
{
    if (!out) return rmw::fail(RMW_ERR_ARG, "null output handle");
    *out = nullptr;
    if (n_bodies <= 0 || n_bodies > (1 << 24)) return rmw::fail(RMW_ERR_ARG, "n_bodies out of range");
    if (!blob_offsets_host) return rmw::fail(RMW_ERR_ARG, "null blob offsets");
    if (!(a > 0) || !(eta > 0)) return rmw::fail(RMW_ERR_ARG, "blob radius and viscosity must be positive");
    if (blob_offsets_host[0] != 0) return rmw::fail(RMW_ERR_ARG, "blob offsets must start at 0");
    RigidSystem *S = new RigidSystem();
    S->nb = (int)n_bodies;
    S->eta = eta;
    S->a = a;
    if (L_host)
        for (int k = 0; k < 3; ++k) S->L[k] = L_host[k];
    S->st = rmw::as_stream(stream);
    cudaGetDevice(&S->device);
    if (int rc = rmw::pool_retain()) {
        delete S;
        return rc;
    }
    S->boff_h.resize(S->nb + 1);
    S->moff_h.resize(S->nb + 1);
    S->moff_h[0] = 0;
    for (int b = 0; b <= S->nb; ++b) {
        S->boff_h[b] = (int)blob_offsets_host[b];
        if (b > 0) {
            const long long nbl = blob_offsets_host[b] - blob_offsets_host[b - 1];
            if (nbl <= 0 || blob_offsets_host[b] > (1LL << 28)) {
                delete S;
                return rmw::fail(RMW_ERR_ARG, "blob offsets must be strictly increasing (every body needs a blob)");
            }
            S->max_m = std::max(S->max_m, (int)(3 * nbl));
            S->moff_h[b] = S->moff_h[b - 1] + 9 * nbl * nbl;
        }
    }
    S->n = S->boff_h[S->nb];
    std::vector<int> bb(S->n);
    for (int b = 0; b < S->nb; ++b)
        for (int i = S->boff_h[b]; i < S->boff_h[b + 1]; ++i) bb[i] = b;
    cudaError_t e = cudaSuccess;
    auto chk = [&](cudaError_t x) {
        if (e == cudaSuccess) e = x;
    };
    chk(cudaMalloc(&S->boff, sizeof(int) * (S->nb + 1)));
    chk(cudaMalloc(&S->blob_body, sizeof(int) * S->n));
    chk(cudaMalloc(&S->moff, sizeof(long long) * (S->nb + 1)));
    chk(cudaMalloc(&S->r, sizeof(double) * 3 * S->n));
    chk(cudaMalloc(&S->xb, sizeof(double) * 3 * S->nb));
    chk(cudaMalloc(&S->dstatus, sizeof(int)));
    chk(cudaMalloc(&S->tmp3n, sizeof(double) * 3 * S->n));
    if (e == cudaSuccess) {
        chk(cudaMemcpy(S->boff, S->boff_h.data(), sizeof(int) * (S->nb + 1), cudaMemcpyHostToDevice));
        chk(cudaMemcpy(S->blob_body, bb.data(), sizeof(int) * S->n, cudaMemcpyHostToDevice));
        chk(cudaMemcpy(S->moff, S->moff_h.data(), sizeof(long long) * (S->nb + 1), cudaMemcpyHostToDevice));
    }
    if (e != cudaSuccess) {
        rmw::free_system(S);
        return rmw::cuda_fail(e, "rmw_rigid_create");
    }
    *out = S;
    return RMW_OK;
}

int rmw_rigid_destroy(void *sys)
{
    if (sys) rmw::free_system((RigidSystem *)sys);
    return RMW_OK;
}

int rmw_rigid_sizes(void *sys, int64_t *n_blobs_host, int64_t *n_bodies_host)
{
    if (!sys || !n_blobs_host || !n_bodies_host) return rmw::fail(RMW_ERR_ARG, "null argument");
    RigidSystem *S = (RigidSystem *)sys;
    *n_blobs_host = S->n;
    *n_bodies_host = S->nb;
    return RMW_OK;
}

// Wall (1, the default) or free space (0) for every mobility of the handle:
// blob products, dense per-body blocks of the preconditioners, solves and
// Lanczos.  Free space is the reference's *_no_wall implementations
// (mobility/mobility.py:288-482, rotne_prager_tensor :967-1015).  Invalidates
// the preconditioners.  Batched suspensions and the near-field augmented
// preconditioner are wall-only.
int rmw_rigid_set_wall(void *sys, int wall)
{
    if (!sys) return rmw::fail(RMW_ERR_ARG, "null handle");
    RigidSystem *S = (RigidSystem *)sys;
    if (!wall && S->batch) return rmw::fail(RMW_ERR_ARG, "batched suspensions are available with the wall only");
    if (S->wall != (wall != 0)) {
        S->wall = wall != 0;
        S->pc_ready = false;
        S->stoch_ready = false;
        S->nf_on = false;
    }
    return RMW_OK;
}

int rmw_rigid_set_configuration(void *sys, const double *r_blobs, const double *x_bodies)
{
    if (!sys || !r_blobs || !x_bodies) return rmw::fail(RMW_ERR_ARG, "null argument");
    RigidSystem *S = (RigidSystem *)sys;
    RMW_CUDA(cudaMemcpyAsync(S->r, r_blobs, sizeof(double) * 3 * S->n, cudaMemcpyDeviceToDevice, S->st));
    RMW_CUDA(cudaMemcpyAsync(S->xb, x_bodies, sizeof(double) * 3 * S->nb, cudaMemcpyDeviceToDevice, S->st));
    S->pc_ready = S->stoch_ready = false;
    S->nf_on = false;  // neighbour pairs and coupling blocks belong to the old configuration
    return RMW_OK;
}

int rmw_rigid_build_pc(void *sys, int stochastic)
{
    if (!sys) return rmw::fail(RMW_ERR_ARG, "null handle");
    return rmw::build_pc(*(RigidSystem *)sys, stochastic != 0);
}

// As rmw_rigid_build_pc for the solves of one precision mode: RMW_MODE_MIXED
// factorises the body blocks on the FP32 pipe (the FP64 pipe runs at 1/64 of
// it on GB300); a block that is not positive definite in FP32 makes it fall
// back to FP64.  Convergence is still judged by the FP64-accurate residual.
int rmw_rigid_build_pc_mode(void *sys, int stochastic, int mode)
{
    if (!sys) return rmw::fail(RMW_ERR_ARG, "null handle");
    if (mode != RMW_MODE_FP64 && mode != RMW_MODE_MIXED && mode != RMW_MODE_DF64)
        return rmw::fail(RMW_ERR_ARG, "unknown precision mode");
    RigidSystem &S = *(RigidSystem *)sys;
    void *tok = nullptr;
    if (int rc = rmw::trace_begin(rmw::TRACE_PCBUILD, S.st, &tok)) return rc;
    const int rc = rmw::build_pc(S, stochastic != 0, mode == RMW_MODE_MIXED);
    if (int rc2 = rmw::trace_end(tok, S.st)) return rc2;
    return rc;
}

int rmw_rigid_apply(void *sys, const double *x, double *y, int mode)
{
    if (!sys || !x || !y) return rmw::fail(RMW_ERR_ARG, "null argument");
    if (x == y) return rmw::fail(RMW_ERR_ARG, "rmw_rigid_apply cannot run in place");
    return rmw::rigid_apply(*(RigidSystem *)sys, x, y, mode);
}

int rmw_rigid_apply_pc(void *sys, const double *x, double *y)
{
    if (!sys || !x || !y) return rmw::fail(RMW_ERR_ARG, "null argument");
    if (x == y) return rmw::fail(RMW_ERR_ARG, "rmw_rigid_apply_pc cannot run in place");
    return rmw::rigid_apply_pc(*(RigidSystem *)sys, x, y);
}

int rmw_rigid_apply_pc_mode(void *sys, const double *x, double *y, int mode)
{
    if (!sys || !x || !y) return rmw::fail(RMW_ERR_ARG, "null argument");
    if (x == y) return rmw::fail(RMW_ERR_ARG, "rmw_rigid_apply_pc_mode cannot run in place");
    if (mode != RMW_MODE_FP64 && mode != RMW_MODE_MIXED && mode != RMW_MODE_DF64)
        return rmw::fail(RMW_ERR_ARG, "unknown precision mode");
    RigidSystem &S = *(RigidSystem *)sys;
    return mode == RMW_MODE_MIXED ? rmw::rigid_apply_pc_mixed(S, x, y) : rmw::rigid_apply_pc(S, x, y);
}

int rmw_rigid_mobility_pc(void *sys, const double *w, double *y, int mode)
{
    if (!sys || !w || !y) return rmw::fail(RMW_ERR_ARG, "null argument");
    return rmw::rigid_mobility_pc(*(RigidSystem *)sys, w, y, mode);
}

int rmw_rigid_P_inv_mult(void *sys, const double *w, double *y)
{
    if (!sys || !w || !y) return rmw::fail(RMW_ERR_ARG, "null argument");
    return rmw::rigid_P_inv_mult(*(RigidSystem *)sys, w, y);
}

int rmw_rigid_K_mult(void *sys, const double *u, double *out)
{
    if (!sys || !u || !out) return rmw::fail(RMW_ERR_ARG, "null argument");
    RigidSystem *S = (RigidSystem *)sys;
    rmw::k_times_u_kernel<<<(S->n + 255) / 256, 256, 0, S->st>>>(S->r, S->xb, S->blob_body, u, out, S->n, 1.0, 0.0);
    RMW_CHECK_LAUNCH("K multiply");
    return RMW_OK;
}

int rmw_rigid_KT_mult(void *sys, const double *lam, double *out)
{
    if (!sys || !lam || !out) return rmw::fail(RMW_ERR_ARG, "null argument");
    RigidSystem *S = (RigidSystem *)sys;
    rmw::kt_times_lambda_kernel<<<(S->nb * 32 + 255) / 256, 256, 0, S->st>>>(S->r, S->xb, S->boff, lam, out, S->nb,
                                                                              1.0);
    RMW_CHECK_LAUNCH("K^T multiply");
    return RMW_OK;
}

int rmw_rigid_blob_positions(void *sys, const double *x_bodies, const double *q_bodies, const double *r_ref,
                             double *r_out)
{
    if (!sys || !x_bodies || !q_bodies || !r_ref || !r_out) return rmw::fail(RMW_ERR_ARG, "null argument");
    RigidSystem *S = (RigidSystem *)sys;
    rmw::blob_positions_kernel<<<(S->n + 255) / 256, 256, 0, S->st>>>(x_bodies, q_bodies, r_ref, S->blob_body,
                                                                       r_out, S->n);
    RMW_CHECK_LAUNCH("blob positions");
    return RMW_OK;
}

int rmw_rigid_euler_update(void *sys, const double *x_bodies, const double *q_bodies, const double *velocities,
                           double dt, double *x_new, double *q_new)
{
    if (!sys || !x_bodies || !q_bodies || !velocities || !x_new || !q_new)
        return rmw::fail(RMW_ERR_ARG, "null argument");
    RigidSystem *S = (RigidSystem *)sys;
    rmw::euler_update_kernel<<<(S->nb + 127) / 128, 128, 0, S->st>>>(x_bodies, q_bodies, velocities, dt, x_new,
                                                                      q_new, S->nb);
    RMW_CHECK_LAUNCH("euler update");
    return RMW_OK;
}

int rmw_count_below(const double *r, int64_t n, double zmin, int *count_host, void *stream)
{
    if (!r || !count_host || n < 0) return rmw::fail(RMW_ERR_ARG, "bad argument");
    cudaStream_t st = rmw::as_stream(stream);
    *count_host = 0;
    if (n == 0) return RMW_OK;
    int *d = nullptr;
    RMW_CUDA(rmw::dmalloc_async(&d, sizeof(int), st));
    RMW_CUDA(cudaMemsetAsync(d, 0, sizeof(int), st));
    rmw::count_below_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(r, (int)n, zmin, d);
    RMW_CHECK_LAUNCH("count below");
    RMW_CUDA(cudaMemcpyAsync(count_host, d, sizeof(int), cudaMemcpyDeviceToHost, st));
    RMW_CUDA(cudaFreeAsync(d, st));
    RMW_CUDA(cudaStreamSynchronize(st));
    return RMW_OK;
}

// Dense per-body wall mobility blocks (each body's 3n_b x 3n_b matrix, bodies
// concatenated) - the matrices the preconditioner factorises.
int rmw_rigid_body_mobility(void *sys, double *out)
{
    if (!sys || !out) return rmw::fail(RMW_ERR_ARG, "null argument");
    RigidSystem *S = (RigidSystem *)sys;
    if (S->wall)
        rmw::body_mobility_kernel<double><<<S->nb, rmw::kRigidThreads, 0, S->st>>>(S->r, S->boff, S->moff, out, S->eta, S->a);
    else
        rmw::body_mobility_free_kernel<double><<<S->nb, rmw::kRigidThreads, 0, S->st>>>(S->r, S->boff, S->moff, out, S->eta,
                                                                               S->a);
    RMW_CHECK_LAUNCH("body mobility");
    return RMW_OK;
}

}  // extern "C"
