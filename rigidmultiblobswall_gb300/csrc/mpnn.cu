// The message-passing network that predicts the near-field mode couplings of
// the augmented preconditioner (nearfield.cu), and its training.
//
// Graph: bodies are nodes; message edges join bodies whose centres are closer
// than the message cutoff (3R by default); band edges are the pairs whose
// 11 x 11 mode coupling G_ij the network predicts (the learned band of the
// preconditioner).  Inputs: per node (z / R, degree / 8), per edge (horizontal
// distance, z_dst, z_src) / R, normalised by statistics of the training data.
//   h0 = silu(W0 x)
//   3 x:  m_e = silu(Wm [h_src; e]);  M_i = mean_{e -> i} m_e;
//         h <- h + silu(Wu [h_i; M_i])
//   G_ij (pair frame) = ro2 silu(ro1 silu(ro0 [h_i; h_j; e_ij]))
// (biases throughout, width 64, inputs zero-padded to 16, 121 outputs padded
// to 128).  The messages let a pair's prediction see how crowded and how high
// both bodies' neighbourhoods are.
//
// Arithmetic: BF16 weights, GEMM inputs and stored activations, FP32
// accumulation on the tensor cores (mma.sync m16n8k16 BF16) in the forward
// and backward passes: the backward GEMMs dX = dZ W and dW = dZ^T X take the
// output gradients rounded to BF16 (straight-through for every rounding);
// bias gradients, aggregation and the residual sums stay FP32.  Every
// reduction runs in a fixed order (CSR edge order, fixed warp trees), so
// training is deterministic.  Sizes are tiny (K <= 144, N <= 128), which is
// why warp-level mma.sync tiles are used rather than tcgen05/TMEM tiles.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "mpnn.cuh"

namespace rmw {

__device__ __forceinline__ float mp_silu(float z) { return z / (1.0f + __expf(-z)); }
__device__ __forceinline__ float mp_silu_grad(float z)
{
    const float s = 1.0f / (1.0f + __expf(-z));
    return s * (1.0f + z * (1.0f - s));
}
__device__ __forceinline__ unsigned mp_pack(__nv_bfloat16 lo, __nv_bfloat16 hi)
{
    return (unsigned)__bfloat16_as_ushort(lo) | ((unsigned)__bfloat16_as_ushort(hi) << 16);
}
__device__ __forceinline__ void mma_bf16(float c[4], unsigned a0, unsigned a1, unsigned a2, unsigned a3,
                                         unsigned b0, unsigned b1)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// Z = X W^T + b (rows [0, P), P a multiple of 16); X: P x nin, W: nout x nin
// (BF16, row-major).  Outputs (each optional): Z (FP32 pre-activation), Y =
// bf16(act(Z)), Yf = act(Z) in FP32; nout a multiple of 16.
__global__ void mp_dense_kernel(const __nv_bfloat16 *__restrict__ X, int nin, const __nv_bfloat16 *__restrict__ Wt,
                                const float *__restrict__ bias, int nout, float *__restrict__ Z,
                                __nv_bfloat16 *__restrict__ Y, float *__restrict__ Yf, int P, int act)
{
    // one warp per 16 rows x 16 output columns: two 16 x 8 tiles sharing the
    // row fragments
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    const int ngrp = nout >> 4;
    const int row0 = (warp / ngrp) * 16, n0 = (warp % ngrp) * 16;
    if (row0 >= P) return;
    const int g = lane >> 2, tq = lane & 3;
    float c[2][4] = {{0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}};
    for (int k0 = 0; k0 < nin; k0 += 16) {
        const int kc = k0 + tq * 2;
        const unsigned a0 = *(const unsigned *)(X + (long long)(row0 + g) * nin + kc);
        const unsigned a1 = *(const unsigned *)(X + (long long)(row0 + g + 8) * nin + kc);
        const unsigned a2 = *(const unsigned *)(X + (long long)(row0 + g) * nin + kc + 8);
        const unsigned a3 = *(const unsigned *)(X + (long long)(row0 + g + 8) * nin + kc + 8);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const unsigned b0 = *(const unsigned *)(Wt + (long long)(n0 + 8 * h + g) * nin + kc);
            const unsigned b1 = *(const unsigned *)(Wt + (long long)(n0 + 8 * h + g) * nin + kc + 8);
            mma_bf16(c[h], a0, a1, a2, a3, b0, b1);
        }
    }
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int col = n0 + 8 * h + tq * 2;
        for (int e = 0; e < 4; ++e) {
            const int rr = row0 + g + (e >= 2 ? 8 : 0), cc = col + (e & 1);
            const float z = c[h][e] + bias[cc];
            const float y = act ? mp_silu(z) : z;
            if (Z) Z[(long long)rr * nout + cc] = z;
            if (Y) Y[(long long)rr * nout + cc] = __float2bfloat16_rn(y);
            if (Yf) Yf[(long long)rr * nout + cc] = y;
        }
    }
}

// C (M x N, FP32) = sum_k A(m, k) B(k, n) on the tensor cores, BF16 operands:
// A(m, k) = AT ? A[k lda + m] : A[m lda + k];  B(k, n) = BT ? B[n ldb + k] : B[k ldb + n].
// M a multiple of 16, N of 8, K of 16.  One warp per 16 x 8 tile.
template <bool AT, bool BT>
__global__ void mp_gemm_kernel(int M, int N, int K, const __nv_bfloat16 *__restrict__ A, int lda,
                               const __nv_bfloat16 *__restrict__ B, int ldb, float *__restrict__ C, int ldc)
{
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    const int tiles_n = N / 8;
    if (warp >= (M / 16) * tiles_n) return;
    const int m0 = (warp / tiles_n) * 16, n0 = (warp % tiles_n) * 8;
    const int g = lane >> 2, tq = lane & 3;
    auto a = [&](int m, int k) { return AT ? A[(long long)k * lda + m] : A[(long long)m * lda + k]; };
    auto b = [&](int k, int n) { return BT ? B[(long long)n * ldb + k] : B[(long long)k * ldb + n]; };
    float c[4] = {0.f, 0.f, 0.f, 0.f};
    for (int k0 = 0; k0 < K; k0 += 16) {
        const int kc = k0 + tq * 2;
        const unsigned a0 = mp_pack(a(m0 + g, kc), a(m0 + g, kc + 1));
        const unsigned a1 = mp_pack(a(m0 + g + 8, kc), a(m0 + g + 8, kc + 1));
        const unsigned a2 = mp_pack(a(m0 + g, kc + 8), a(m0 + g, kc + 9));
        const unsigned a3 = mp_pack(a(m0 + g + 8, kc + 8), a(m0 + g + 8, kc + 9));
        const unsigned b0 = mp_pack(b(kc, n0 + g), b(kc + 1, n0 + g));
        const unsigned b1 = mp_pack(b(kc + 8, n0 + g), b(kc + 9, n0 + g));
        mma_bf16(c, a0, a1, a2, a3, b0, b1);
    }
    const int col = n0 + tq * 2;
    C[(long long)(m0 + g) * ldc + col] = c[0];
    C[(long long)(m0 + g) * ldc + col + 1] = c[1];
    C[(long long)(m0 + g + 8) * ldc + col] = c[2];
    C[(long long)(m0 + g + 8) * ldc + col + 1] = c[3];
}

__global__ void mp_to_bf16_kernel(const float *__restrict__ x, __nv_bfloat16 *__restrict__ y, long long n)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = __float2bfloat16_rn(x[i]);
}

// dZ = dY * silu'(Z) (act) or dY
__global__ void mp_act_grad_kernel(const float *__restrict__ dY, int ldy, const float *__restrict__ Z,
                                   float *__restrict__ dZ, int rows, int cols, int act)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)rows * cols) return;
    const int r = (int)(t / cols), c = (int)(t % cols);
    const float d = dY[(long long)r * ldy + c];
    dZ[t] = act ? d * mp_silu_grad(Z[t]) : d;
}

// gb[c] = sum_r dZ[r][c] (one warp per column, fixed order)
__global__ void mp_bias_grad_kernel(const float *__restrict__ dZ, int rows, int cols, float *__restrict__ gb)
{
    const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (c >= cols) return;
    float s = 0.f;
    for (int r = lane; r < rows; r += 32) s += dZ[(long long)r * cols + c];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) gb[c] = s;
}

// normalised, zero-padded BF16 rows of raw features (rows_pad rows of kMpIn)
__global__ void mp_features_kernel(const float *__restrict__ raw, int nf, int rows, const float *__restrict__ mean,
                                   const float *__restrict__ scale, __nv_bfloat16 *__restrict__ X, int rows_pad)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows_pad) return;
    for (int k = 0; k < kMpIn; ++k) {
        const float v = (r < rows && k < nf) ? (raw[(long long)r * nf + k] - mean[k]) / scale[k] : 0.f;
        X[(long long)r * kMpIn + k] = __float2bfloat16_rn(v);
    }
}

// Xm[e] = [h[src(e)], E[e]]  (80 wide; padded rows zero)
__global__ void mp_gather_msg_kernel(const __nv_bfloat16 *__restrict__ h, const int *__restrict__ src,
                                     const __nv_bfloat16 *__restrict__ E, int ne, int ne_pad,
                                     __nv_bfloat16 *__restrict__ Xm)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int w = kMpW + kMpIn;
    if (t >= (long long)ne_pad * w) return;
    const int e = (int)(t / w), c = (int)(t % w);
    __nv_bfloat16 v = __float2bfloat16_rn(0.f);
    if (e < ne) v = c < kMpW ? h[(long long)src[e] * kMpW + c] : E[(long long)e * kMpIn + c - kMpW];
    Xm[t] = v;
}

// Xu[i] = [h[i], bf16(mean of m over the edges into i)]  (128 wide)
__global__ void mp_aggregate_kernel(const __nv_bfloat16 *__restrict__ h, const __nv_bfloat16 *__restrict__ m,
                                    const int *__restrict__ off, int nn, int nn_pad, __nv_bfloat16 *__restrict__ Xu)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)nn_pad * kMpW) return;
    const int i = (int)(t / kMpW), c = (int)(t % kMpW);
    __nv_bfloat16 hv = __float2bfloat16_rn(0.f), mv = hv;
    if (i < nn) {
        const int e0 = off[i], e1 = off[i + 1];
        float s = 0.f;
        for (int e = e0; e < e1; ++e) s += __bfloat162float(m[(long long)e * kMpW + c]);
        hv = h[(long long)i * kMpW + c];
        mv = __float2bfloat16_rn(s / (float)max(e1 - e0, 1));
    }
    Xu[(long long)i * 2 * kMpW + c] = hv;
    Xu[(long long)i * 2 * kMpW + kMpW + c] = mv;
}

// h_new = bf16(h + u)
__global__ void mp_residual_kernel(const __nv_bfloat16 *__restrict__ h, const float *__restrict__ u, long long n,
                                   __nv_bfloat16 *__restrict__ hn)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) hn[t] = __float2bfloat16_rn(__bfloat162float(h[t]) + u[t]);
}

// Xr[e] = [h[i(e)], h[j(e)], E[e]]  (144 wide)
__global__ void mp_gather_readout_kernel(const __nv_bfloat16 *__restrict__ h, const int *__restrict__ bi,
                                         const int *__restrict__ bj, const __nv_bfloat16 *__restrict__ E, int nb,
                                         int nb_pad, __nv_bfloat16 *__restrict__ Xr)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int w = 2 * kMpW + kMpIn;
    if (t >= (long long)nb_pad * w) return;
    const int e = (int)(t / w), c = (int)(t % w);
    __nv_bfloat16 v = __float2bfloat16_rn(0.f);
    if (e < nb) {
        if (c < kMpW) v = h[(long long)bi[e] * kMpW + c];
        else if (c < 2 * kMpW) v = h[(long long)bj[e] * kMpW + c - kMpW];
        else v = E[(long long)e * kMpIn + c - 2 * kMpW];
    }
    Xr[t] = v;
}

// MSE gradient on the band outputs: dY = 2 (Y - T / tscale) / (nb * 121), loss
// summed per block into *loss (one block's sum per atomic: fixed set of adds)
__global__ void mp_mse_kernel(const float *__restrict__ Yf, const float *__restrict__ T,
                              const float *__restrict__ tscale, int nb, int nb_pad, float *__restrict__ dY,
                              float *__restrict__ part)
{
    __shared__ float sh[8];
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    float g = 0.f, l = 0.f;
    if (t < (long long)nb_pad * kMpOut) {
        const int e = (int)(t / kMpOut), o = (int)(t % kMpOut);
        if (e < nb && o < kMpTarget) {
            const float d = Yf[t] - T[(long long)e * kMpTarget + o] / tscale[o];
            g = 2.0f * d / (float)((long long)nb * kMpTarget);
            l = d * d / (float)((long long)nb * kMpTarget);
        }
        dY[t] = g;
    }
    for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = l;
    __syncthreads();
    if (threadIdx.x == 0) {
        float s = 0.f;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += sh[w];
        part[blockIdx.x] = s;
    }
}

// loss = sum of the block partials (fixed order)
__global__ void mp_sum_kernel(const float *__restrict__ part, int n, float *__restrict__ out)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        float s = 0.f;
        for (int i = 0; i < n; ++i) s += part[i];
        *out = s;
    }
}

// dh[n][c] = sum over band edges f owned by n of dXr[f][c] + dXr[rev f][64 + c]
__global__ void mp_readout_scatter_kernel(const float *__restrict__ dXr, const int *__restrict__ off,
                                          const int *__restrict__ rev, int nn, float *__restrict__ dh)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)nn * kMpW) return;
    const int i = (int)(t / kMpW), c = (int)(t % kMpW);
    const int w = 2 * kMpW + kMpIn;
    float s = 0.f;
    for (int f = off[i]; f < off[i + 1]; ++f) s += dXr[(long long)f * w + c] + dXr[(long long)rev[f] * w + kMpW + c];
    dh[t] = s;
}

// dZm[e][c] = dXu[dst e][64 + c] / deg(dst e) * silu'(Zm[e][c])
__global__ void mp_msg_grad_kernel(const float *__restrict__ dXu, const int *__restrict__ dst,
                                   const int *__restrict__ off, const float *__restrict__ Zm, int ne,
                                   float *__restrict__ dZm)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)ne * kMpW) return;
    const int e = (int)(t / kMpW), c = (int)(t % kMpW);
    const int i = dst[e];
    const float inv = 1.0f / (float)max(off[i + 1] - off[i], 1);
    dZm[t] = dXu[(long long)i * 2 * kMpW + kMpW + c] * inv * mp_silu_grad(Zm[t]);
}

// dh_prev[n][c] = dh[n][c] + dXu[n][c] + sum_{f into n} dXm[rev f][c]
__global__ void mp_node_grad_kernel(const float *__restrict__ dh, const float *__restrict__ dXu,
                                    const float *__restrict__ dXm, const int *__restrict__ off,
                                    const int *__restrict__ rev, int nn, float *__restrict__ dprev)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)nn * kMpW) return;
    const int i = (int)(t / kMpW), c = (int)(t % kMpW);
    float s = dh[t] + dXu[(long long)i * 2 * kMpW + c];
    for (int f = off[i]; f < off[i + 1]; ++f) s += dXm[(long long)rev[f] * (kMpW + kMpIn) + c];
    dprev[t] = s;
}

__global__ void mp_adam_kernel(float *__restrict__ w, const float *__restrict__ g, float *__restrict__ m,
                               float *__restrict__ v, __nv_bfloat16 *__restrict__ wb, int count, float lr, float b1,
                               float b2, float c1, float c2, float eps)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    w[i] = wi;
    if (wb) wb[i] = __float2bfloat16_rn(wi);
}

// ---------------------------------------------------------------------------
// workspace: activations of one graph (rows padded to 16)
static inline int pad16(int n) { return ((std::max(n, 1) + 15) / 16) * 16; }

struct MpWork {
    int cap_n = 0, cap_e = 0, cap_b = 0;
    cudaStream_t st = 0;
    void *base = nullptr;
    __nv_bfloat16 *X0 = nullptr, *Em = nullptr, *Eb = nullptr;
    float *Zemb = nullptr;
    __nv_bfloat16 *h[kMpSteps + 1];
    __nv_bfloat16 *Xm[kMpSteps], *m[kMpSteps], *Xu[kMpSteps];
    float *Zm[kMpSteps], *Zu[kMpSteps];
    float *U = nullptr;  // silu(Zu) of the current step (FP32)
    __nv_bfloat16 *Xr = nullptr, *A0 = nullptr, *A1 = nullptr;
    float *Z0 = nullptr, *Z1 = nullptr, *Yf = nullptr;
    // backward
    float *dY = nullptr, *dZ = nullptr, *dX = nullptr, *dX2 = nullptr, *dh = nullptr, *dh2 = nullptr,
          *part = nullptr, *loss = nullptr;
    __nv_bfloat16 *dZb = nullptr;
};

int mp_work_create(MpWork **out, int nodes, int mp, int band, cudaStream_t st)
{
    MpWork *W = new MpWork();
    W->st = st;
    const size_t N = pad16(nodes), E = pad16(mp), B = pad16(band);
    W->cap_n = (int)N;
    W->cap_e = (int)E;
    W->cap_b = (int)B;
    const size_t rows = std::max(N, std::max(E, B));
    const int kw = 2 * kMpW + kMpIn;  // widest GEMM input (144)
    auto al = [](size_t b) { return (b + 255) / 256 * 256; };
    size_t bytes = 0;
    const size_t hb = sizeof(__nv_bfloat16), fb = sizeof(float);
    bytes += al(hb * N * kMpIn) + al(hb * E * kMpIn) + al(hb * B * kMpIn) + al(fb * N * kMpW);
    bytes += (kMpSteps + 1) * al(hb * N * kMpW);
    bytes += kMpSteps * (al(hb * E * (kMpW + kMpIn)) + al(hb * E * kMpW) + al(hb * N * 2 * kMpW) + al(fb * E * kMpW) +
                         al(fb * N * kMpW));
    bytes += al(fb * N * kMpW);
    bytes += al(hb * B * kw) + 2 * al(hb * B * kMpW) + 2 * al(fb * B * kMpW) + al(fb * B * kMpOut);
    bytes += al(fb * B * kMpOut) + al(fb * rows * kw) + 2 * al(fb * rows * kw) + 2 * al(fb * N * kMpW) +
             al(fb * (B * kMpOut / 256 + 2)) + al(fb * 4) + al(hb * rows * kw);
    if (rmw::dmalloc_async(&W->base, bytes, st) != cudaSuccess) {
        delete W;
        return fail(RMW_ERR_ALLOC, "message-passing network workspace");
    }
    char *p = (char *)W->base;
    auto take = [&](size_t b) {
        char *q = p;
        p += al(b);
        return (void *)q;
    };
    W->X0 = (__nv_bfloat16 *)take(hb * N * kMpIn);
    W->Em = (__nv_bfloat16 *)take(hb * E * kMpIn);
    W->Eb = (__nv_bfloat16 *)take(hb * B * kMpIn);
    W->Zemb = (float *)take(fb * N * kMpW);
    for (int t = 0; t <= kMpSteps; ++t) W->h[t] = (__nv_bfloat16 *)take(hb * N * kMpW);
    for (int t = 0; t < kMpSteps; ++t) {
        W->Xm[t] = (__nv_bfloat16 *)take(hb * E * (kMpW + kMpIn));
        W->m[t] = (__nv_bfloat16 *)take(hb * E * kMpW);
        W->Xu[t] = (__nv_bfloat16 *)take(hb * N * 2 * kMpW);
        W->Zm[t] = (float *)take(fb * E * kMpW);
        W->Zu[t] = (float *)take(fb * N * kMpW);
    }
    W->U = (float *)take(fb * N * kMpW);
    W->Xr = (__nv_bfloat16 *)take(hb * B * kw);
    W->A0 = (__nv_bfloat16 *)take(hb * B * kMpW);
    W->A1 = (__nv_bfloat16 *)take(hb * B * kMpW);
    W->Z0 = (float *)take(fb * B * kMpW);
    W->Z1 = (float *)take(fb * B * kMpW);
    W->Yf = (float *)take(fb * B * kMpOut);
    W->dY = (float *)take(fb * B * kMpOut);
    W->dZ = (float *)take(fb * rows * kw);
    W->dX = (float *)take(fb * rows * kw);
    W->dX2 = (float *)take(fb * rows * kw);
    W->dh = (float *)take(fb * N * kMpW);
    W->dh2 = (float *)take(fb * N * kMpW);
    W->part = (float *)take(fb * (B * kMpOut / 256 + 2));
    W->loss = (float *)take(fb * 4);
    W->dZb = (__nv_bfloat16 *)take(hb * rows * kw);
    *out = W;
    return RMW_OK;
}

void mp_work_destroy(MpWork *W)
{
    if (!W) return;
    if (W->base) cudaFreeAsync(W->base, W->st);
    delete W;
}

const float *mp_outputs(const MpWork &W) { return W.Yf; }

static void dense(MpnnNet &net, int l, const __nv_bfloat16 *X, int rows, float *Z, __nv_bfloat16 *Y, float *Yf,
                  bool act, cudaStream_t st)
{
    const long long warps = (long long)(rows / 16) * (mp_layer_out(l) / 16);
    mp_dense_kernel<<<(unsigned)((warps * 32 + 127) / 128), 128, 0, st>>>(X, mp_layer_in(l), net.wb + mp_wofs(l),
                                                              net.b + mp_bofs(l), mp_layer_out(l), Z, Y, Yf, rows,
                                                              act ? 1 : 0);
}

static inline unsigned blocks(long long n, int t) { return (unsigned)((n + t - 1) / t); }

int mp_forward(MpnnNet &net, const MpGraph &g, MpWork &W, cudaStream_t st)
{
    const int N = pad16(g.n_nodes), E = pad16(g.n_mp), B = pad16(g.n_band);
    if (N > W.cap_n || E > W.cap_e || B > W.cap_b) return fail(RMW_ERR_ARG, "graph larger than its workspace");
    const float *nm = net.dnorm, *ns = nm + kNodeFeat, *em = ns + kNodeFeat, *es = em + kEdgeFeat;
    mp_features_kernel<<<blocks(N, 128), 128, 0, st>>>(g.node_feat, kNodeFeat, g.n_nodes, nm, ns, W.X0, N);
    mp_features_kernel<<<blocks(E, 128), 128, 0, st>>>(g.mp_feat, kEdgeFeat, g.n_mp, em, es, W.Em, E);
    mp_features_kernel<<<blocks(B, 128), 128, 0, st>>>(g.band_feat, kEdgeFeat, g.n_band, em, es, W.Eb, B);
    dense(net, 0, W.X0, N, W.Zemb, W.h[0], nullptr, true, st);
    for (int t = 0; t < kMpSteps; ++t) {
        mp_gather_msg_kernel<<<blocks((long long)E * (kMpW + kMpIn), 256), 256, 0, st>>>(W.h[t], g.mp_src, W.Em,
                                                                                        g.n_mp, E, W.Xm[t]);
        dense(net, 1 + 2 * t, W.Xm[t], E, W.Zm[t], W.m[t], nullptr, true, st);
        mp_aggregate_kernel<<<blocks((long long)N * kMpW, 256), 256, 0, st>>>(W.h[t], W.m[t], g.mp_off, g.n_nodes,
                                                                               N, W.Xu[t]);
        dense(net, 2 + 2 * t, W.Xu[t], N, W.Zu[t], nullptr, W.U, true, st);
        mp_residual_kernel<<<blocks((long long)N * kMpW, 256), 256, 0, st>>>(W.h[t], W.U, (long long)N * kMpW,
                                                                              W.h[t + 1]);
    }
    const int r0 = 2 * kMpSteps + 1;
    mp_gather_readout_kernel<<<blocks((long long)B * (2 * kMpW + kMpIn), 256), 256, 0, st>>>(
        W.h[kMpSteps], g.band_i, g.band_j, W.Eb, g.n_band, B, W.Xr);
    dense(net, r0, W.Xr, B, W.Z0, W.A0, nullptr, true, st);
    dense(net, r0 + 1, W.A0, B, W.Z1, W.A1, nullptr, true, st);
    dense(net, r0 + 2, W.A1, B, nullptr, nullptr, W.Yf, false, st);
    RMW_CHECK_LAUNCH("message-passing forward");
    return RMW_OK;
}

// backward of one dense layer: dZ (rows x nout, FP32, already times act')
// -> gW, gb of layer l (written) and, if dX, dX = bf16(dZ) W (rows x nin)
static void dense_back(MpnnNet &net, int l, const __nv_bfloat16 *X, int rows, const float *dZ, MpWork &W,
                       float *gW, float *gb, float *dX, cudaStream_t st)
{
    const int ni = mp_layer_in(l), no = mp_layer_out(l);
    mp_to_bf16_kernel<<<blocks((long long)rows * no, 256), 256, 0, st>>>(dZ, W.dZb, (long long)rows * no);
    // gW (no x ni) = dZb^T (no x rows) X (rows x ni)
    mp_gemm_kernel<true, false><<<blocks((long long)(no / 16) * (ni / 8) * 32, 128), 128, 0, st>>>(
        no, ni, rows, W.dZb, no, X, ni, gW + mp_wofs(l), ni);
    mp_bias_grad_kernel<<<blocks((long long)no * 32, 128), 128, 0, st>>>(dZ, rows, no, gb + mp_bofs(l));
    if (dX) {
        // dX (rows x ni) = dZb (rows x no) W (no x ni)
        mp_gemm_kernel<false, false><<<blocks((long long)(rows / 16) * (ni / 8) * 32, 128), 128, 0, st>>>(
            rows, ni, no, W.dZb, no, net.wb + mp_wofs(l), ni, dX, ni);
    }
}

// forward + backward of the mean squared error on graph g (targets g.target):
// gradients into gW (kMpNW), gb (kMpNB), loss into *loss (device)
static int mp_backward(MpnnNet &net, const MpGraph &g, MpWork &W, float *gW, float *gb, float *loss,
                       cudaStream_t st)
{
    if (int rc = mp_forward(net, g, W, st)) return rc;
    const int N = pad16(g.n_nodes), E = pad16(g.n_mp), B = pad16(g.n_band);
    const int r0 = 2 * kMpSteps + 1;
    const unsigned nbk = blocks((long long)B * kMpOut, 256);
    mp_mse_kernel<<<nbk, 256, 0, st>>>(W.Yf, g.target, net.dnorm + 2 * kNodeFeat + 2 * kEdgeFeat, g.n_band, B, W.dY,
                                       W.part);
    mp_sum_kernel<<<1, 32, 0, st>>>(W.part, (int)nbk, loss);
    // readout
    dense_back(net, r0 + 2, W.A1, B, W.dY, W, gW, gb, W.dX, st);
    mp_act_grad_kernel<<<blocks((long long)B * kMpW, 256), 256, 0, st>>>(W.dX, kMpW, W.Z1, W.dZ, B, kMpW, 1);
    dense_back(net, r0 + 1, W.A0, B, W.dZ, W, gW, gb, W.dX, st);
    mp_act_grad_kernel<<<blocks((long long)B * kMpW, 256), 256, 0, st>>>(W.dX, kMpW, W.Z0, W.dZ, B, kMpW, 1);
    dense_back(net, r0, W.Xr, B, W.dZ, W, gW, gb, W.dX, st);
    mp_readout_scatter_kernel<<<blocks((long long)N * kMpW, 256), 256, 0, st>>>(W.dX, g.band_off, g.band_rev,
                                                                                 g.n_nodes, W.dh);
    // the padding rows of both node-gradient buffers are zero (the node kernels write the real rows only;
    // the weight-gradient GEMMs sum over every row)
    if (N > g.n_nodes) {
        cudaMemsetAsync(W.dh + (long long)g.n_nodes * kMpW, 0, sizeof(float) * (N - g.n_nodes) * kMpW, st);
        cudaMemsetAsync(W.dh2 + (long long)g.n_nodes * kMpW, 0, sizeof(float) * (N - g.n_nodes) * kMpW, st);
    }
    // message-passing steps, last first
    for (int t = kMpSteps - 1; t >= 0; --t) {
        // h_{t+1} = h_t + silu(Zu): dZu = dh * silu'(Zu)
        mp_act_grad_kernel<<<blocks((long long)N * kMpW, 256), 256, 0, st>>>(W.dh, kMpW, W.Zu[t], W.dZ, N, kMpW, 1);
        dense_back(net, 2 + 2 * t, W.Xu[t], N, W.dZ, W, gW, gb, W.dX, st);  // dX = dXu (N x 128)
        if (E > g.n_mp) cudaMemsetAsync(W.dZ + (long long)g.n_mp * kMpW, 0, sizeof(float) * (E - g.n_mp) * kMpW, st);
        mp_msg_grad_kernel<<<blocks((long long)g.n_mp * kMpW, 256), 256, 0, st>>>(W.dX, g.mp_dst, g.mp_off, W.Zm[t],
                                                                                  g.n_mp, W.dZ);
        dense_back(net, 1 + 2 * t, W.Xm[t], E, W.dZ, W, gW, gb, W.dX2, st);  // dX2 = dXm (E x 80)
        mp_node_grad_kernel<<<blocks((long long)g.n_nodes * kMpW, 256), 256, 0, st>>>(W.dh, W.dX, W.dX2, g.mp_off,
                                                                                      g.mp_rev, g.n_nodes, W.dh2);
        std::swap(W.dh, W.dh2);
    }
    // embed: dZ = dh * silu'(Zemb)
    mp_act_grad_kernel<<<blocks((long long)N * kMpW, 256), 256, 0, st>>>(W.dh, kMpW, W.Zemb, W.dZ, N, kMpW, 1);
    dense_back(net, 0, W.X0, N, W.dZ, W, gW, gb, nullptr, st);
    RMW_CHECK_LAUNCH("message-passing backward");
    return RMW_OK;
}

}  // namespace rmw

// ---------------------------------------------------------------------------
// C ABI
using rmw::MpGraph;
using rmw::MpnnNet;

static MpGraph graph_of(const rmw_graph &h)
{
    MpGraph g;
    g.n_nodes = h.n_nodes;
    g.n_mp = h.n_mp;
    g.n_band = h.n_band;
    g.node_feat = h.node_feat;
    g.mp_src = h.mp_src;
    g.mp_dst = h.mp_dst;
    g.mp_off = h.mp_off;
    g.mp_rev = h.mp_rev;
    g.mp_feat = h.mp_feat;
    g.band_i = h.band_i;
    g.band_j = h.band_j;
    g.band_off = h.band_off;
    g.band_rev = h.band_rev;
    g.band_feat = h.band_feat;
    g.target = h.target;
    return g;
}

static int check_graph(const rmw_graph *g, bool need_target)
{
    if (!g) return rmw::fail(RMW_ERR_ARG, "null graph");
    if (g->n_nodes < 1 || g->n_mp < 0 || g->n_band < 1) return rmw::fail(RMW_ERR_ARG, "graph needs nodes and band edges");
    if (!g->node_feat || !g->mp_off || !g->band_i || !g->band_j || !g->band_off || !g->band_feat ||
        (g->n_mp > 0 && (!g->mp_src || !g->mp_dst || !g->mp_feat)))
        return rmw::fail(RMW_ERR_ARG, "graph arrays missing");
    if (need_target && (!g->target || !g->band_rev || (g->n_mp > 0 && !g->mp_rev)))
        return rmw::fail(RMW_ERR_ARG, "training graphs need targets and reverse edges");
    return RMW_OK;
}

extern "C" {

int rmw_nearfield_create(void **net_out, double body_radius, double cutoff, unsigned long long seed)
{
    if (!net_out) return rmw::fail(RMW_ERR_ARG, "null argument");
    if (!(body_radius > 0) || !(cutoff > 0)) return rmw::fail(RMW_ERR_ARG, "radius and cutoff must be positive");
    MpnnNet *N = new MpnnNet();
    N->radius = body_radius;
    N->cutoff = cutoff;
    N->mp_cutoff = 3.0 * body_radius;
    cudaGetDevice(&N->device);
    // He-style uniform initialisation from a fixed-seed generator (host, deterministic);
    // weights on zero-padded inputs or on unused outputs are zero
    std::vector<float> w(rmw::kMpNW, 0.f), b(rmw::kMpNB, 0.f);
    unsigned long long x = seed ? seed : 1;
    auto uni = [&]() {
        x ^= x << 13; x ^= x >> 7; x ^= x << 17;
        return (double)(x >> 11) / 9007199254740992.0;
    };
    for (int l = 0; l < rmw::kMpLayers; ++l) {
        const int ni = rmw::mp_layer_in(l), no = rmw::mp_layer_out(l);
        auto live_in = [&](int i) {
            if (l == 0) return i < rmw::kNodeFeat;
            if (ni == rmw::kMpW + rmw::kMpIn) return i < rmw::kMpW + rmw::kEdgeFeat;
            if (ni == 2 * rmw::kMpW + rmw::kMpIn) return i < 2 * rmw::kMpW + rmw::kEdgeFeat;
            return true;
        };
        int fan = 0;
        for (int i = 0; i < ni; ++i) fan += live_in(i);
        const bool last = l == rmw::kMpLayers - 1;
        const bool upd = l >= 1 && l <= 2 * rmw::kMpSteps && (l - 1) % 2 == 1;
        const double sc = std::sqrt(6.0 / fan) * (last ? 0.25 : (upd ? 0.5 : 1.0));
        for (int o = 0; o < no; ++o)
            for (int i = 0; i < ni; ++i) {
                const bool live = live_in(i) && (!last || o < rmw::kMpTarget);
                w[rmw::mp_wofs(l) + o * ni + i] = live ? (float)((2.0 * uni() - 1.0) * sc) : 0.0f;
            }
    }
    for (int i = 0; i < rmw::kMpNorm; ++i) N->norm[i] = 1.f;
    for (int i = 0; i < rmw::kNodeFeat; ++i) N->norm[i] = 0.f;
    for (int i = 0; i < rmw::kEdgeFeat; ++i) N->norm[2 * rmw::kNodeFeat + i] = 0.f;
    cudaError_t e = cudaSuccess;
    auto chk = [&](cudaError_t c) { if (e == cudaSuccess) e = c; };
    chk(cudaMalloc(&N->w, sizeof(float) * rmw::kMpNW));
    chk(cudaMalloc(&N->b, sizeof(float) * rmw::kMpNB));
    chk(cudaMalloc(&N->wb, sizeof(__nv_bfloat16) * rmw::kMpNW));
    chk(cudaMalloc(&N->adam, sizeof(float) * 2 * (rmw::kMpNW + rmw::kMpNB)));
    chk(cudaMalloc(&N->dnorm, sizeof(float) * rmw::kMpNorm));
    if (e == cudaSuccess) {
        std::vector<__nv_bfloat16> wb(rmw::kMpNW);
        for (int i = 0; i < rmw::kMpNW; ++i) wb[i] = __float2bfloat16_rn(w[i]);
        chk(cudaMemcpy(N->w, w.data(), sizeof(float) * rmw::kMpNW, cudaMemcpyHostToDevice));
        chk(cudaMemcpy(N->b, b.data(), sizeof(float) * rmw::kMpNB, cudaMemcpyHostToDevice));
        chk(cudaMemcpy(N->wb, wb.data(), sizeof(__nv_bfloat16) * rmw::kMpNW, cudaMemcpyHostToDevice));
        chk(cudaMemset(N->adam, 0, sizeof(float) * 2 * (rmw::kMpNW + rmw::kMpNB)));
        chk(cudaMemcpy(N->dnorm, N->norm, sizeof(float) * rmw::kMpNorm, cudaMemcpyHostToDevice));
    }
    if (e != cudaSuccess) {
        cudaFree(N->w); cudaFree(N->b); cudaFree(N->wb); cudaFree(N->adam); cudaFree(N->dnorm);
        delete N;
        return rmw::cuda_fail(e, "rmw_nearfield_create");
    }
    *net_out = N;
    return RMW_OK;
}

int rmw_nearfield_destroy(void *net)
{
    if (!net) return RMW_OK;
    MpnnNet *N = (MpnnNet *)net;
    cudaFree(N->w); cudaFree(N->b); cudaFree(N->wb); cudaFree(N->adam); cudaFree(N->dnorm);
    delete N;
    return RMW_OK;
}

int rmw_nearfield_sizes(int *n_weights, int *n_biases, int *n_norm, int *width, int *n_out, int *n_target)
{
    if (n_weights) *n_weights = rmw::kMpNW;
    if (n_biases) *n_biases = rmw::kMpNB;
    if (n_norm) *n_norm = rmw::kMpNorm;
    if (width) *width = rmw::kMpW;
    if (n_out) *n_out = rmw::kMpOut;
    if (n_target) *n_target = rmw::kMpTarget;
    return RMW_OK;
}

int rmw_nearfield_set_cutoffs(void *net, double mp_cutoff, double cutoff)
{
    if (!net) return rmw::fail(RMW_ERR_ARG, "null network");
    if (!(mp_cutoff > 0) || !(cutoff > 0)) return rmw::fail(RMW_ERR_ARG, "cutoffs must be positive");
    MpnnNet *N = (MpnnNet *)net;
    N->mp_cutoff = mp_cutoff;
    N->cutoff = cutoff;
    return RMW_OK;
}

int rmw_nearfield_get(void *net, float *w_host, float *b_host, float *norm_host)
{
    if (!net) return rmw::fail(RMW_ERR_ARG, "null network");
    MpnnNet *N = (MpnnNet *)net;
    if (w_host) RMW_CUDA(cudaMemcpy(w_host, N->w, sizeof(float) * rmw::kMpNW, cudaMemcpyDeviceToHost));
    if (b_host) RMW_CUDA(cudaMemcpy(b_host, N->b, sizeof(float) * rmw::kMpNB, cudaMemcpyDeviceToHost));
    if (norm_host) std::memcpy(norm_host, N->norm, sizeof(float) * rmw::kMpNorm);
    return RMW_OK;
}

int rmw_nearfield_set(void *net, const float *w_host, const float *b_host, const float *norm_host)
{
    if (!net) return rmw::fail(RMW_ERR_ARG, "null network");
    MpnnNet *N = (MpnnNet *)net;
    if (w_host) {
        std::vector<__nv_bfloat16> wb(rmw::kMpNW);
        for (int i = 0; i < rmw::kMpNW; ++i) wb[i] = __float2bfloat16_rn(w_host[i]);
        RMW_CUDA(cudaMemcpy(N->w, w_host, sizeof(float) * rmw::kMpNW, cudaMemcpyHostToDevice));
        RMW_CUDA(cudaMemcpy(N->wb, wb.data(), sizeof(__nv_bfloat16) * rmw::kMpNW, cudaMemcpyHostToDevice));
    }
    if (b_host) RMW_CUDA(cudaMemcpy(N->b, b_host, sizeof(float) * rmw::kMpNB, cudaMemcpyHostToDevice));
    if (norm_host) {
        std::memcpy(N->norm, norm_host, sizeof(float) * rmw::kMpNorm);
        RMW_CUDA(cudaMemcpy(N->dnorm, N->norm, sizeof(float) * rmw::kMpNorm, cudaMemcpyHostToDevice));
    }
    return RMW_OK;
}

int rmw_nearfield_forward(void *net, const rmw_graph *graph, float *out, void *stream)
{
    if (!net || !out) return rmw::fail(RMW_ERR_ARG, "null argument");
    if (int rc = check_graph(graph, false)) return rc;
    MpnnNet *N = (MpnnNet *)net;
    cudaStream_t st = rmw::as_stream(stream);
    const MpGraph g = graph_of(*graph);
    rmw::MpWork *W = nullptr;
    if (int rc = rmw::mp_work_create(&W, g.n_nodes, g.n_mp, g.n_band, st)) return rc;
    int rc = rmw::mp_forward(*N, g, *W, st);
    if (rc == RMW_OK)
        rc = cudaMemcpy2DAsync(out, sizeof(float) * rmw::kMpTarget, W->Yf, sizeof(float) * rmw::kMpOut,
                               sizeof(float) * rmw::kMpTarget, g.n_band, cudaMemcpyDeviceToDevice, st) == cudaSuccess
                 ? RMW_OK
                 : rmw::fail(RMW_ERR_CUDA, "copy of the network outputs");
    rmw::mp_work_destroy(W);
    if (cudaStreamSynchronize(st) != cudaSuccess && rc == RMW_OK) rc = rmw::fail(RMW_ERR_CUDA, "forward");
    return rc;
}

int rmw_nearfield_grad(void *net, const rmw_graph *graph, float *gW_host, float *gb_host, float *loss_host)
{
    if (!net || !gW_host || !gb_host || !loss_host) return rmw::fail(RMW_ERR_ARG, "null argument");
    if (int rc = check_graph(graph, true)) return rc;
    MpnnNet *N = (MpnnNet *)net;
    cudaStream_t st = 0;
    const MpGraph g = graph_of(*graph);
    rmw::MpWork *W = nullptr;
    if (int rc = rmw::mp_work_create(&W, g.n_nodes, g.n_mp, g.n_band, st)) return rc;
    float *buf = nullptr;
    RMW_CUDA(cudaMalloc(&buf, sizeof(float) * (rmw::kMpNW + rmw::kMpNB + 1)));
    int rc = rmw::mp_backward(*N, g, *W, buf, buf + rmw::kMpNW, buf + rmw::kMpNW + rmw::kMpNB, st);
    if (rc == RMW_OK) {
        RMW_CUDA(cudaMemcpy(gW_host, buf, sizeof(float) * rmw::kMpNW, cudaMemcpyDeviceToHost));
        RMW_CUDA(cudaMemcpy(gb_host, buf + rmw::kMpNW, sizeof(float) * rmw::kMpNB, cudaMemcpyDeviceToHost));
        RMW_CUDA(cudaMemcpy(loss_host, buf + rmw::kMpNW + rmw::kMpNB, sizeof(float), cudaMemcpyDeviceToHost));
    }
    cudaFree(buf);
    rmw::mp_work_destroy(W);
    cudaDeviceSynchronize();
    return rc;
}

// Adam over the graphs (one graph per step, in order, cycling); sets the
// normalisation from the graphs' features and targets first.
int rmw_nearfield_train(void *net, const rmw_graph *graphs, int n_graphs, int steps, float lr,
                        float *loss_host, void *stream)
{
    if (!net || !graphs || n_graphs < 1 || steps < 1) return rmw::fail(RMW_ERR_ARG, "bad argument");
    for (int k = 0; k < n_graphs; ++k)
        if (int rc = check_graph(graphs + k, true)) return rc;
    MpnnNet *N = (MpnnNet *)net;
    cudaStream_t st = rmw::as_stream(stream);
    // normalisation from the data: feature mean / standard deviation, per-output
    // target RMS floored at 5% of the largest (outputs that vanish for a sphere
    // by the pair's mirror symmetry carry only orientation noise)
    std::vector<double> s1(rmw::kNodeFeat + rmw::kEdgeFeat, 0.0), s2(s1.size(), 0.0), tq(rmw::kMpTarget, 0.0);
    double cn = 0, ce = 0, cb = 0;
    int maxn = 1, maxe = 1, maxb = 1;
    for (int k = 0; k < n_graphs; ++k) {
        const rmw_graph &g = graphs[k];
        maxn = std::max(maxn, g.n_nodes);
        maxe = std::max(maxe, g.n_mp);
        maxb = std::max(maxb, g.n_band);
        std::vector<float> nf((size_t)g.n_nodes * rmw::kNodeFeat), ef((size_t)g.n_band * rmw::kEdgeFeat),
            tg((size_t)g.n_band * rmw::kMpTarget), mf((size_t)g.n_mp * rmw::kEdgeFeat);
        RMW_CUDA(cudaMemcpyAsync(nf.data(), g.node_feat, sizeof(float) * nf.size(), cudaMemcpyDeviceToHost, st));
        RMW_CUDA(cudaMemcpyAsync(ef.data(), g.band_feat, sizeof(float) * ef.size(), cudaMemcpyDeviceToHost, st));
        RMW_CUDA(cudaMemcpyAsync(tg.data(), g.target, sizeof(float) * tg.size(), cudaMemcpyDeviceToHost, st));
        if (g.n_mp) RMW_CUDA(cudaMemcpyAsync(mf.data(), g.mp_feat, sizeof(float) * mf.size(), cudaMemcpyDeviceToHost, st));
        RMW_CUDA(cudaStreamSynchronize(st));
        for (int i = 0; i < g.n_nodes; ++i)
            for (int f = 0; f < rmw::kNodeFeat; ++f) {
                s1[f] += nf[(size_t)i * rmw::kNodeFeat + f];
                s2[f] += (double)nf[(size_t)i * rmw::kNodeFeat + f] * nf[(size_t)i * rmw::kNodeFeat + f];
            }
        cn += g.n_nodes;
        for (int e = 0; e < g.n_band; ++e) {
            for (int f = 0; f < rmw::kEdgeFeat; ++f) {
                const double v = ef[(size_t)e * rmw::kEdgeFeat + f];
                s1[rmw::kNodeFeat + f] += v;
                s2[rmw::kNodeFeat + f] += v * v;
            }
            for (int o = 0; o < rmw::kMpTarget; ++o)
                tq[o] += (double)tg[(size_t)e * rmw::kMpTarget + o] * tg[(size_t)e * rmw::kMpTarget + o];
        }
        for (int e = 0; e < g.n_mp; ++e)
            for (int f = 0; f < rmw::kEdgeFeat; ++f) {
                const double v = mf[(size_t)e * rmw::kEdgeFeat + f];
                s1[rmw::kNodeFeat + f] += v;
                s2[rmw::kNodeFeat + f] += v * v;
            }
        ce += g.n_band + g.n_mp;
        cb += g.n_band;
    }
    float norm[rmw::kMpNorm];
    for (int f = 0; f < rmw::kNodeFeat; ++f) {
        const double m = s1[f] / cn, v = std::max(s2[f] / cn - m * m, 0.0);
        norm[f] = (float)m;
        norm[rmw::kNodeFeat + f] = (float)std::max(std::sqrt(v), 1e-3);
    }
    for (int f = 0; f < rmw::kEdgeFeat; ++f) {
        const double m = s1[rmw::kNodeFeat + f] / ce, v = std::max(s2[rmw::kNodeFeat + f] / ce - m * m, 0.0);
        norm[2 * rmw::kNodeFeat + f] = (float)m;
        norm[2 * rmw::kNodeFeat + rmw::kEdgeFeat + f] = (float)std::max(std::sqrt(v), 1e-3);
    }
    double tmax = 0.0;
    for (int o = 0; o < rmw::kMpTarget; ++o) tmax = std::max(tmax, std::sqrt(tq[o] / cb));
    for (int o = 0; o < rmw::kMpTarget; ++o)
        norm[2 * rmw::kNodeFeat + 2 * rmw::kEdgeFeat + o] =
            (float)std::max(std::sqrt(tq[o] / cb), std::max(0.05 * tmax, 1e-30));
    if (int rc = rmw_nearfield_set(net, nullptr, nullptr, norm)) return rc;
    rmw::MpWork *W = nullptr;
    if (int rc = rmw::mp_work_create(&W, maxn, maxe, maxb, st)) return rc;
    float *buf = nullptr;
    if (rmw::dmalloc_async((void **)&buf, sizeof(float) * (rmw::kMpNW + rmw::kMpNB + steps), st) != cudaSuccess) {
        rmw::mp_work_destroy(W);
        return rmw::fail(RMW_ERR_ALLOC, "training buffers");
    }
    float *gW = buf, *gb = buf + rmw::kMpNW, *loss = gb + rmw::kMpNB;
    const float b1 = 0.9f, b2 = 0.999f;
    float *mW = N->adam, *vW = N->adam + rmw::kMpNW, *mB = N->adam + 2 * rmw::kMpNW, *vB = mB + rmw::kMpNB;
    int rc = RMW_OK;
    for (int t = 0; t < steps && rc == RMW_OK; ++t) {
        rc = rmw::mp_backward(*N, graph_of(graphs[t % n_graphs]), *W, gW, gb, loss + t, st);
        if (rc) break;
        const float c1 = 1.f - std::pow(b1, (float)(t + 1)), c2 = 1.f - std::pow(b2, (float)(t + 1));
        rmw::mp_adam_kernel<<<(rmw::kMpNW + 255) / 256, 256, 0, st>>>(N->w, gW, mW, vW, N->wb, rmw::kMpNW, lr, b1,
                                                                     b2, c1, c2, 1e-8f);
        rmw::mp_adam_kernel<<<(rmw::kMpNB + 255) / 256, 256, 0, st>>>(N->b, gb, mB, vB, nullptr, rmw::kMpNB, lr, b1,
                                                                     b2, c1, c2, 1e-8f);
    }
    cudaError_t e = cudaGetLastError();
    if (rc == RMW_OK && e != cudaSuccess) rc = rmw::cuda_fail(e, "near-field training");
    if (rc == RMW_OK && loss_host)
        if (cudaMemcpyAsync(loss_host, loss, sizeof(float) * steps, cudaMemcpyDeviceToHost, st) != cudaSuccess)
            rc = rmw::fail(RMW_ERR_CUDA, "loss copy");
    cudaFreeAsync(buf, st);
    rmw::mp_work_destroy(W);
    if (cudaStreamSynchronize(st) != cudaSuccess && rc == RMW_OK) rc = rmw::fail(RMW_ERR_CUDA, "training");
    return rc;
}

}  // extern "C"
