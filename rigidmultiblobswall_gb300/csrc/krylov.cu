// Krylov solvers of the rigid mobility problem on the GPU.
//
// GMRES: right-preconditioned restarted GMRES, the algorithm of
// general_application_utils.py:514-635 (solve A P^-1 y = b, x = P^-1 y) on top
// of scipy's gmres (restart m, zero initial guess, relative tolerance on the
// 2-norm of the residual, atol = 0).  All vector work runs on the device:
// Arnoldi with classical Gram-Schmidt plus one reorthogonalisation pass (CGS2:
// two dot-product passes and two update passes over the basis per step).
// The small (m+1) x m Hessenberg least-squares problem is solved on the host in
// FP64 with Givens rotations, as scipy does; it needs the step's m+2 dot
// products, which come back with the per-step convergence check.
//
// Mixed precision: the inner GMRES applies the FP32-pair operator; an outer
// iterative-refinement loop recomputes the residual with the FP64-accurate
// operator and stops on that residual, so the returned solution meets the
// same relative-residual tolerance as a plain FP64 solve.  Once the residual
// is small the loop updates it by the recurrence r <- r - A32 d instead
// (refine_by_recurrence in rigid.cuh).
//
// Lanczos: stochastic_forcing/stochastic_forcing.py:112-264 (Ando et al. 2012):
// three-term recurrence, one full reorthogonalisation pass against every
// previous basis vector per step (no renormalisation afterwards, as in the
// reference), the noise factor*|z|*V^T Q sqrt(max(L,0)) Q^T e1 from the
// eigen-decomposition of the tridiagonal matrix (implicit QL, FP64 on the
// host), and convergence on the relative change of the noise between steps,
// measured on the coefficient vectors (the basis rows are orthonormal).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "graph_op.cuh"
#include "krylov_device.cuh"
#include "rigid.cuh"
#include "wall_pair.cuh"

namespace rmw {

constexpr int kVecThreads = 256;
constexpr int kElemsPerThread = 4;
constexpr int kChunk = 128;  // basis vectors per dot/update pass (shared coefficient array size)

// ---------------------------------------------------------------------------
// vector kernels
// partial[q * nblk + blk] = sum over the block's chunk of V_q[i] * w[i]  (q < k)
__global__ void dots_partial_kernel(const double *__restrict__ V, long long ldv, int k,
                                    const double *__restrict__ w, long long n, double *__restrict__ partial)
{
    extern __shared__ double red[];  // k * nwarps
    const int nw = blockDim.x / 32, wid = threadIdx.x / 32, lane = threadIdx.x & 31;
    const long long base = (long long)blockIdx.x * blockDim.x * kElemsPerThread + threadIdx.x;
    double wv[kElemsPerThread];
#pragma unroll
    for (int e = 0; e < kElemsPerThread; ++e) {
        const long long i = base + (long long)e * blockDim.x;
        wv[e] = (i < n) ? w[i] : 0.0;
    }
    for (int q = 0; q < k; ++q) {
        const double *Vq = V + (long long)q * ldv;
        double acc = 0.0;
#pragma unroll
        for (int e = 0; e < kElemsPerThread; ++e) {
            const long long i = base + (long long)e * blockDim.x;
            if (i < n) acc += Vq[i] * wv[e];
        }
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) red[q * nw + wid] = acc;
    }
    __syncthreads();
    for (int q = threadIdx.x; q < k; q += blockDim.x) {
        double s = 0.0;
        for (int j = 0; j < nw; ++j) s += red[q * nw + j];
        partial[(long long)q * gridDim.x + blockIdx.x] = s;
    }
}

// out[q] (+)= sum_b partial[q * nblk + b], fixed order; one warp per q
__global__ void reduce_partial_kernel(const double *__restrict__ partial, int nblk, int k, double *__restrict__ out,
                                      int accumulate)
{
    const int q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (q >= k) return;
    double s = 0.0;
    for (int b = lane; b < nblk; b += 32) s += partial[(long long)q * nblk + b];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) out[q] = accumulate ? out[q] + s : s;
}

// w[i] -= sum_q h[q] V_q[i]; optional partial sums of w[i]^2 (per block)
__global__ void update_kernel(const double *__restrict__ V, long long ldv, int k, const double *__restrict__ h,
                              double *__restrict__ w, long long n, double *__restrict__ norm_partial)
{
    __shared__ double hs[kChunk];
    __shared__ double red[32];
    for (int q = threadIdx.x; q < k; q += blockDim.x) hs[q] = h[q];
    __syncthreads();
    const long long base = (long long)blockIdx.x * blockDim.x * kElemsPerThread + threadIdx.x;
    double nrm = 0.0;
#pragma unroll
    for (int e = 0; e < kElemsPerThread; ++e) {
        const long long i = base + (long long)e * blockDim.x;
        if (i < n) {
            double x = w[i];
            for (int q = 0; q < k; ++q) x -= hs[q] * V[(long long)q * ldv + i];
            w[i] = x;
            nrm += x * x;
        }
    }
    if (norm_partial) {
        const int lane = threadIdx.x & 31, wid = threadIdx.x / 32;
        for (int o = 16; o > 0; o >>= 1) nrm += __shfl_xor_sync(0xffffffffu, nrm, o);
        if (lane == 0) red[wid] = nrm;
        __syncthreads();
        if (threadIdx.x == 0) {
            double s = 0.0;
            for (int j = 0; j < (int)blockDim.x / 32; ++j) s += red[j];
            norm_partial[blockIdx.x] = s;
        }
    }
}

// y[i] = alpha * x[i]   with alpha = num / sqrt(*den) or num if den == null
__global__ void scale_kernel(const double *__restrict__ x, double *__restrict__ y, long long n, double num,
                             const double *__restrict__ den_sq)
{
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double alpha = num;
    if (den_sq) {
        const double d = sqrt(*den_sq);
        alpha = (d > 0.0) ? num / d : 0.0;
    }
    y[i] = alpha * x[i];
}

// y[i] = a*x[i] + b*y[i]
__global__ void axpby_kernel(const double *__restrict__ x, double *__restrict__ y, long long n, double a, double b)
{
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = a * x[i] + b * y[i];
}

// out[i] (+)= sum_q c[q] V_q[i]
__global__ void combine_kernel(const double *__restrict__ V, long long ldv, int k, const double *__restrict__ c,
                               double *__restrict__ out, long long n, int accumulate)
{
    __shared__ double cs[kChunk];
    for (int q = threadIdx.x; q < k; q += blockDim.x) cs[q] = c[q];
    __syncthreads();
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double s = 0.0;
    for (int q = 0; q < k; ++q) s += cs[q] * V[(long long)q * ldv + i];
    out[i] = accumulate ? out[i] + s : s;
}

// ---------------------------------------------------------------------------
// host helpers
struct VecOps {
    cudaStream_t st;
    double *partial = nullptr;  // kmax * nblk
    double *dsc = nullptr;      // device scalars / small vectors (>= 2*kmax + 8)
    double *hpin = nullptr;     // pinned host mirror of dsc
    long long n = 0;
    int nblk = 0, kmax = 0;

    int blocks() const { return nblk; }

    // dsc[off .. off+k) = V[0..k)^T w   (basis processed in chunks of kChunk vectors)
    int dots(const double *V, long long ldv, int k, const double *w, int off)
    {
        for (int q0 = 0; q0 < k; q0 += kChunk) {
            const int kc = std::min(kChunk, k - q0);
            const size_t sm = sizeof(double) * kc * (kVecThreads / 32);
            dots_partial_kernel<<<nblk, kVecThreads, sm, st>>>(V + (long long)q0 * ldv, ldv, kc, w, n, partial);
            reduce_partial_kernel<<<(kc * 32 + 255) / 256, 256, 0, st>>>(partial, nblk, kc, dsc + off + q0, 0);
        }
        RMW_CHECK_LAUNCH("dots");
        return RMW_OK;
    }
    // w -= V h (h at dsc+hoff); if nrm_off >= 0, dsc[nrm_off] = |w|^2
    int update(const double *V, long long ldv, int k, int hoff, double *w, int nrm_off)
    {
        for (int q0 = 0; q0 < k; q0 += kChunk) {
            const int kc = std::min(kChunk, k - q0);
            const bool last = q0 + kc >= k;
            update_kernel<<<nblk, kVecThreads, 0, st>>>(V + (long long)q0 * ldv, ldv, kc, dsc + hoff + q0, w, n,
                                                        (last && nrm_off >= 0) ? partial : nullptr);
        }
        if (nrm_off >= 0) reduce_partial_kernel<<<1, 32, 0, st>>>(partial, nblk, 1, dsc + nrm_off, 0);
        RMW_CHECK_LAUNCH("update");
        return RMW_OK;
    }
    int norm2(const double *w, int off)
    {
        dots_partial_kernel<<<nblk, kVecThreads, sizeof(double) * (kVecThreads / 32), st>>>(w, 0, 1, w, n, partial);
        reduce_partial_kernel<<<1, 32, 0, st>>>(partial, nblk, 1, dsc + off, 0);
        RMW_CHECK_LAUNCH("norm");
        return RMW_OK;
    }
    int fetch(int off, int count)
    {
        RMW_CUDA(cudaMemcpyAsync(hpin + off, dsc + off, sizeof(double) * count, cudaMemcpyDeviceToHost, st));
        RMW_CUDA(cudaStreamSynchronize(st));
        return RMW_OK;
    }
    int put(int off, const double *src, int count)
    {
        std::memcpy(hpin + off, src, sizeof(double) * count);
        RMW_CUDA(cudaMemcpyAsync(dsc + off, hpin + off, sizeof(double) * count, cudaMemcpyHostToDevice, st));
        return RMW_OK;
    }
    int scale(const double *x, double *y, double num, const double *den_sq)
    {
        scale_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(x, y, n, num, den_sq);
        RMW_CHECK_LAUNCH("scale");
        return RMW_OK;
    }
    int axpby(const double *x, double *y, double a, double b)
    {
        axpby_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(x, y, n, a, b);
        RMW_CHECK_LAUNCH("axpby");
        return RMW_OK;
    }
    // out = V[0..k) c  (c at dsc+coff)
    int combine(const double *V, long long ldv, int k, int coff, double *out)
    {
        for (int q0 = 0; q0 < k; q0 += kChunk) {
            const int kc = std::min(kChunk, k - q0);
            combine_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(V + (long long)q0 * ldv, ldv, kc,
                                                                        dsc + coff + q0, out, n, q0 > 0);
        }
        RMW_CHECK_LAUNCH("combine");
        return RMW_OK;
    }
};

// Per-solve workspace carved out of one stream-ordered allocation (freed when
// the solve returns), so nested or concurrent solves never share memory.
struct KrylovWork {
    double *V, *w, *x, *r, *t1, *t2;
    VecOps ops;
    void *base = nullptr;
    cudaStream_t st = 0;
    ~KrylovWork()
    {
        if (base) cudaFreeAsync(base, st);
    }
};

static int make_work(long long n, int kmax, cudaStream_t st, KrylovWork &K, int nbasis = -1)
{
    if (nbasis < 0) nbasis = kmax + 1;
    const int nblk = (int)std::max<long long>(1, (n + (long long)kVecThreads * kElemsPerThread - 1) /
                                                    ((long long)kVecThreads * kElemsPerThread));
    const long long ldv = ((n + 31) / 32) * 32;
    const size_t doubles = (size_t)ldv * nbasis + 5 * (size_t)ldv + (size_t)nblk * (kChunk + 2) + 4 * (kmax + 8);
    void *p = nullptr;
    RMW_CUDA(rmw::dmalloc_async(&p, sizeof(double) * doubles, st));
    K.base = p;
    K.st = st;
    double *d = (double *)p;
    K.V = d; d += (size_t)ldv * nbasis;
    K.w = d; d += ldv;
    K.x = d; d += ldv;
    K.r = d; d += ldv;
    K.t1 = d; d += ldv;
    K.t2 = d; d += ldv;
    K.ops.partial = d; d += (size_t)nblk * (kChunk + 2);
    K.ops.dsc = d;
    K.ops.st = st;
    K.ops.n = n;
    K.ops.nblk = nblk;
    K.ops.kmax = kmax;
    static thread_local double *pin = nullptr;
    static thread_local size_t pin_n = 0;
    const size_t need = 4 * (size_t)(kmax + 8);
    if (pin_n < need) {
        if (pin) cudaFreeHost(pin);
        RMW_CUDA(cudaHostAlloc(&pin, sizeof(double) * need, cudaHostAllocDefault));
        pin_n = need;
    }
    K.ops.hpin = pin;
    return RMW_OK;
}

static inline long long ldv_of(long long n) { return ((n + 31) / 32) * 32; }

// ---------------------------------------------------------------------------
// GMRES (right preconditioned).  op(x, y): y = A x ; pc(x, y): y = P^-1 x ;
// pcop(x, y): y = A P^-1 x, the Arnoldi step's operator (given separately so
// that the caller can fuse it and replay it as a CUDA graph).
template <typename Op, typename Pc, typename PcOp>
static int gmres_right(Op op, Pc pc, PcOp pcop, const double *b, double *x_out, long long n, double tol, int restart,
                       int maxiter, cudaStream_t st, int *iters_out, double *relres_out, std::vector<double> *hist)
{
    restart = std::max(1, std::min(restart, 120));
    KrylovWork K;
    if (int rc = make_work(n, restart + 2, st, K)) return rc;
    VecOps &O = K.ops;
    const long long ldv = ldv_of(n);
    const int SC = 2 * (restart + 2);  // scalar area offset inside dsc (h1 at 0, h2 at restart+2)
    // |b|
    if (int rc = O.norm2(b, SC)) return rc;
    if (int rc = O.fetch(SC, 1)) return rc;
    const double bnorm = std::sqrt(O.hpin[SC]);
    RMW_CUDA(cudaMemsetAsync(K.x, 0, sizeof(double) * n, st));
    int iters = 0;
    if (!(bnorm > 0.0)) {
        RMW_CUDA(cudaMemcpyAsync(x_out, K.x, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
        if (iters_out) *iters_out = 0;
        if (relres_out) *relres_out = 0.0;
        if (!std::isfinite(bnorm)) return fail(RMW_ERR_NONFINITE, "right-hand side is not finite");
        return RMW_OK;
    }
    const double tol_abs = tol * bnorm;
    RMW_CUDA(cudaMemcpyAsync(K.r, b, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
    double beta = bnorm;
    std::vector<double> H((size_t)(restart + 1) * restart), cs(restart), sn(restart), g(restart + 1);
    int status = RMW_ERR_NOT_CONVERGED;
    double res_true = beta;
    while (true) {
        // V_0 = r / beta
        if (int rc = O.scale(K.r, K.V, 1.0 / beta, nullptr)) return rc;
        std::fill(g.begin(), g.end(), 0.0);
        g[0] = beta;
        int jdone = 0;
        bool inner_conv = false, breakdown = false;
        for (int j = 0; j < restart; ++j) {
            double *Vj = K.V + (long long)j * ldv;
            double *Vn = K.V + (long long)(j + 1) * ldv;
            {
                void *otok = nullptr;
                if (int rc = trace_begin(TRACE_OPERATOR, st, &otok)) return rc;
                if (int rc = pcop(Vj, K.w)) return rc;
                if (int rc = trace_end(otok, st)) return rc;
            }
            // CGS2 against V_0..V_j; algorithmic bytes: 2 x (dots (j+2) n + update (j+3) n) + scale 2 n
            void *tok = nullptr;
            if (int rc = trace_begin(TRACE_KRYLOV, st, &tok)) return rc;
            if (int rc = O.dots(K.V, ldv, j + 1, K.w, 0)) return rc;
            if (int rc = O.update(K.V, ldv, j + 1, 0, K.w, -1)) return rc;
            if (int rc = O.dots(K.V, ldv, j + 1, K.w, restart + 2)) return rc;
            if (int rc = O.update(K.V, ldv, j + 1, restart + 2, K.w, SC + 1)) return rc;
            if (int rc = O.scale(K.w, Vn, 1.0, O.dsc + SC + 1)) return rc;
            if (int rc = trace_end(tok, st)) return rc;
            if (tok) trace_bytes(TRACE_KRYLOV, 8.0 * (4.0 * j + 12.0) * (double)n);
            if (int rc = O.fetch(0, SC + 2)) return rc;
            double *h = &H[(size_t)j * (restart + 1)];
            for (int q = 0; q <= j; ++q) h[q] = O.hpin[q] + O.hpin[restart + 2 + q];
            h[j + 1] = std::sqrt(O.hpin[SC + 1]);
            if (!std::isfinite(h[j + 1])) return fail(RMW_ERR_BREAKDOWN, "GMRES: non-finite Arnoldi vector");
            // apply previous rotations and make the new one
            for (int q = 0; q < j; ++q) {
                const double t = cs[q] * h[q] + sn[q] * h[q + 1];
                h[q + 1] = -sn[q] * h[q] + cs[q] * h[q + 1];
                h[q] = t;
            }
            const double den = std::hypot(h[j], h[j + 1]);
            if (den == 0.0) { cs[j] = 1.0; sn[j] = 0.0; }
            else { cs[j] = h[j] / den; sn[j] = h[j + 1] / den; }
            h[j] = cs[j] * h[j] + sn[j] * h[j + 1];
            h[j + 1] = 0.0;
            g[j + 1] = -sn[j] * g[j];
            g[j] = cs[j] * g[j];
            ++iters;
            jdone = j + 1;
            const double res = std::fabs(g[j + 1]);
            if (hist) hist->push_back(res / bnorm);
            if (res <= tol_abs) { inner_conv = true; break; }
            if (std::sqrt(O.hpin[SC + 1]) == 0.0) { breakdown = true; break; }
            if (iters >= maxiter) break;
        }
        // y = R^-1 g (back substitution), dy = V y, dx = P^-1 dy, x += dx
        std::vector<double> y(jdone);
        for (int q = jdone - 1; q >= 0; --q) {
            double s = g[q];
            for (int c = q + 1; c < jdone; ++c) s -= H[(size_t)c * (restart + 1) + q] * y[c];
            const double d = H[(size_t)q * (restart + 1) + q];
            y[q] = (d != 0.0) ? s / d : 0.0;
        }
        if (int rc = O.put(SC + 4, y.data(), jdone)) return rc;
        if (int rc = O.combine(K.V, ldv, jdone, SC + 4, K.t1)) return rc;
        if (int rc = pc(K.t1, K.t2)) return rc;
        if (int rc = O.axpby(K.t2, K.x, 1.0, 1.0)) return rc;
        // true residual r = b - A x
        if (int rc = op(K.x, K.r)) return rc;
        if (int rc = O.axpby(b, K.r, 1.0, -1.0)) return rc;
        if (int rc = O.norm2(K.r, SC + 2)) return rc;
        if (int rc = O.fetch(SC + 2, 1)) return rc;
        beta = std::sqrt(O.hpin[SC + 2]);
        res_true = beta;
        if (!std::isfinite(beta)) return fail(RMW_ERR_BREAKDOWN, "GMRES: non-finite residual");
        if (beta <= tol_abs) { status = RMW_OK; break; }
        if (iters >= maxiter) { status = RMW_ERR_NOT_CONVERGED; break; }
        if (breakdown && !inner_conv) { status = RMW_ERR_BREAKDOWN; break; }
    }
    RMW_CUDA(cudaMemcpyAsync(x_out, K.x, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
    RMW_CUDA(cudaStreamSynchronize(st));
    if (iters_out) *iters_out = iters;
    if (relres_out) *relres_out = res_true / bnorm;
    if (status == RMW_ERR_NOT_CONVERGED) set_error("GMRES reached maxiter without converging");
    if (status == RMW_ERR_BREAKDOWN) set_error("GMRES breakdown");
    return status;
}

// ---------------------------------------------------------------------------
// symmetric tridiagonal eigen-decomposition (implicit QL with Wilkinson-type
// shifts, the classical algorithm of Bowdler, Martin, Reinsch & Wilkinson).
// d: diagonal (k), e: sub-diagonal (k-1); on exit d = eigenvalues and z (k x k,
// column-major: z[i + k*j] = component i of eigenvector j).
static bool tridiag_eigen(std::vector<double> &d, std::vector<double> e, std::vector<double> &z)
{
    const int k = (int)d.size();
    z.assign((size_t)k * k, 0.0);
    for (int i = 0; i < k; ++i) z[i + (size_t)k * i] = 1.0;
    e.resize(k, 0.0);
    for (int l = 0; l < k; ++l) {
        int iter = 0;
        int m;
        do {
            for (m = l; m < k - 1; ++m) {
                const double dd = std::fabs(d[m]) + std::fabs(d[m + 1]);
                if (std::fabs(e[m]) <= 1e-16 * dd) break;
            }
            if (m != l) {
                if (++iter > 60) return false;
                double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
                double r = std::hypot(g, 1.0);
                g = d[m] - d[l] + e[l] / (g + (g >= 0 ? std::fabs(r) : -std::fabs(r)));
                double s = 1.0, c = 1.0, p = 0.0;
                int i;
                for (i = m - 1; i >= l; --i) {
                    double f = s * e[i], b = c * e[i];
                    r = std::hypot(f, g);
                    e[i + 1] = r;
                    if (r == 0.0) {
                        d[i + 1] -= p;
                        e[m] = 0.0;
                        break;
                    }
                    s = f / r;
                    c = g / r;
                    g = d[i + 1] - p;
                    r = (d[i] - g) * s + 2.0 * c * b;
                    p = s * r;
                    d[i + 1] = g + p;
                    g = c * r - b;
                    for (int q = 0; q < k; ++q) {
                        f = z[q + (size_t)k * (i + 1)];
                        z[q + (size_t)k * (i + 1)] = s * z[q + (size_t)k * i] + c * f;
                        z[q + (size_t)k * i] = c * z[q + (size_t)k * i] - s * f;
                    }
                }
                if (r == 0.0 && i >= l) continue;
                d[l] -= p;
                e[l] = g;
                e[m] = 0.0;
            }
        } while (m != l);
    }
    return true;
}

bool tridiag_eigen_host(std::vector<double> &d, std::vector<double> e, std::vector<double> &z)
{
    return tridiag_eigen(d, std::move(e), z);
}

// Lanczos noise = factor * M^(1/2) z (op: y = M x).  z and noise are device vectors.
template <typename Op>
static int lanczos(Op op, const double *z, double *noise, long long n, double factor, double tol, int max_iter,
                   cudaStream_t st, int *iters_out)
{
    const int kcap = std::max(2, std::min(max_iter + 1, 1000));
    KrylovWork K;
    if (int rc = make_work(n, kcap + 1, st, K, 0)) return rc;
    VecOps &O = K.ops;
    const long long ldv = ldv_of(n);
    // The basis grows on demand (stream-ordered allocations, doubling).
    int vcap = std::min(kcap + 1, 32);
    double *Vb = nullptr;
    RMW_CUDA(rmw::dmalloc_async(&Vb, sizeof(double) * ldv * vcap, st));
    K.V = Vb;
    struct Guard {
        double **p;
        cudaStream_t s;
        ~Guard() { if (*p) cudaFreeAsync(*p, s); }
    } guard{&K.V, st};
    const int SC = 2 * (kcap + 3);
    if (factor == 0.0) {
        RMW_CUDA(cudaMemsetAsync(noise, 0, sizeof(double) * n, st));
        if (iters_out) *iters_out = 0;
        return RMW_OK;
    }
    if (int rc = O.norm2(z, SC)) return rc;
    if (int rc = O.fetch(SC, 1)) return rc;
    const double znorm = std::sqrt(O.hpin[SC]);
    if (!(znorm > 0.0) || !std::isfinite(znorm)) return fail(RMW_ERR_NONFINITE, "Lanczos: |z| is zero or not finite");
    if (int rc = O.scale(z, K.V, 1.0 / znorm, nullptr)) return rc;
    std::vector<double> hd, hs, c, c_old, zq, ev;
    int it_final = max_iter;
    bool done = false;
    for (int i = 0; i <= max_iter && i < kcap; ++i) {
        double *Vi = K.V + (long long)i * ldv;
        {
            void *otok = nullptr;
            if (int rc = trace_begin(TRACE_OPERATOR, st, &otok)) return rc;
            if (int rc = op(Vi, K.w)) return rc;
            if (int rc = trace_end(otok, st)) return rc;
        }
        // w -= hs[i-1] V_{i-1}; hd[i] = <w, V_i>; w -= hd[i] V_i; hs[i] = |w|
        if (i > 0) {
            const double a = -hs[i - 1];
            if (int rc = O.axpby(K.V + (long long)(i - 1) * ldv, K.w, a, 1.0)) return rc;
        }
        if (int rc = O.dots(Vi, ldv, 1, K.w, 0)) return rc;
        if (int rc = O.fetch(0, 1)) return rc;
        hd.push_back(O.hpin[0]);
        if (int rc = O.axpby(Vi, K.w, -hd[i], 1.0)) return rc;
        if (int rc = O.norm2(K.w, SC + 1)) return rc;
        if (int rc = O.fetch(SC + 1, 1)) return rc;
        const double wn = std::sqrt(O.hpin[SC + 1]);
        if (!std::isfinite(wn) || !std::isfinite(hd[i])) return fail(RMW_ERR_BREAKDOWN, "Lanczos: non-finite value");
        hs.push_back(wn);
        if (wn > 0.0) {
            if (int rc = O.scale(K.w, K.w, 1.0 / wn, nullptr)) return rc;
        } else {
            // the reference sets w[0] = 1 on an exact breakdown
            const double one = 1.0;
            RMW_CUDA(cudaMemcpyAsync(K.w, &one, sizeof(double), cudaMemcpyHostToDevice, st));
        }
        // eigen-decomposition of the (i+1) x (i+1) tridiagonal matrix
        std::vector<double> dd(hd), ee(hs.begin(), hs.begin() + i);
        if (!tridiag_eigen(dd, ee, zq)) return fail(RMW_ERR_BREAKDOWN, "Lanczos: tridiagonal eigensolver failed");
        const int k = i + 1;
        c.assign(k, 0.0);
        for (int j = 0; j < k; ++j) {
            const double lam = dd[j] > 0 ? std::sqrt(dd[j]) : 0.0;
            const double w1 = zq[0 + (size_t)k * j] * lam * znorm * factor;  // (Q^T e1)_j * sqrt(l_j)
            for (int q = 0; q < k; ++q) c[q] += zq[q + (size_t)k * j] * w1;
        }
        // reorthogonalise w against V_0..V_i (one pass, as the reference) -> V_{i+1}
        if (int rc = O.dots(K.V, ldv, k, K.w, 0)) return rc;
        if (int rc = O.update(K.V, ldv, k, 0, K.w, -1)) return rc;
        if (i + 2 > vcap) {
            const int ncap = std::min(kcap + 1, 2 * vcap);
            double *nv = nullptr;
            RMW_CUDA(rmw::dmalloc_async(&nv, sizeof(double) * ldv * ncap, st));
            RMW_CUDA(cudaMemcpyAsync(nv, K.V, sizeof(double) * ldv * vcap, cudaMemcpyDeviceToDevice, st));
            RMW_CUDA(cudaFreeAsync(K.V, st));
            K.V = nv;
            vcap = ncap;
        }
        RMW_CUDA(cudaMemcpyAsync(K.V + (long long)(i + 1) * ldv, K.w, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
        if (i > 0) {
            double dn = 0.0, on = 0.0;
            for (int q = 0; q < k; ++q) {
                const double co = (q < (int)c_old.size()) ? c_old[q] : 0.0;
                dn += (c[q] - co) * (c[q] - co);
                on += co * co;
            }
            dn = std::sqrt(dn);
            on = std::sqrt(on);
            if (dn / std::max(on, 2.220446049250313e-16) < tol) {
                it_final = i;
                done = true;
            }
        }
        c_old = c;
        if (done) break;
    }
    // noise = V^T c
    const int k = (int)c.size();
    if (int rc = O.put(SC + 4, c.data(), k)) return rc;
    if (int rc = O.combine(K.V, ldv, k, SC + 4, noise)) return rc;
    RMW_CUDA(cudaStreamSynchronize(st));
    if (iters_out) *iters_out = it_final;
    return RMW_OK;
}

// y = x / d
__global__ void div_scalar_kernel(const double *__restrict__ x, double *__restrict__ y, long long n, double d)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = x[i] / d;
}

}  // namespace rmw

// ---------------------------------------------------------------------------
// C ABI
using rmw::RigidSystem;

extern "C" {

static int rigid_solve_impl(void *sys, const double *rhs, double *sol, double tol, int restart, int maxiter,
                            int mode, int *iters_host, double *relres_host);

int rmw_rigid_solve(void *sys, const double *rhs, double *sol, double tol, int restart, int maxiter, int mode,
                    int *iters_host, double *relres_host)
{
    if (!sys) return rmw::fail(RMW_ERR_ARG, "null argument");
    RigidSystem &S = *(RigidSystem *)sys;
    void *tok = nullptr;
    if (int rc = rmw::trace_begin(rmw::TRACE_SOLVE, S.st, &tok)) return rc;
    const int rc = rigid_solve_impl(sys, rhs, sol, tol, restart, maxiter, mode, iters_host, relres_host);
    if (int rc2 = rmw::trace_end(tok, S.st)) return rc2;
    return rc;
}

int rmw_rigid_solve_scaled(void *sys, const double *rhs, double *sol, double tol, int restart, int maxiter, int mode,
                           int *iters_host, double *relres_host)
{
    if (!sys || !rhs || !sol) return rmw::fail(RMW_ERR_ARG, "null argument");
    RigidSystem &S = *(RigidSystem *)sys;
    const long long n = S.sys_size();
    const int nblk = (int)((n + 1023) / 1024);
    double *buf = nullptr;  // the scaled rhs, the norm's block partials and its square
    RMW_CUDA(rmw::dmalloc_async(&buf, sizeof(double) * (n + nblk + 1), S.st));
    struct FreeB {
        double *p;
        cudaStream_t s;
        ~FreeB() { cudaFreeAsync(p, s); }
    } free_b{buf, S.st};
    double *bs = buf, *part = buf + n, *nrm2 = part + nblk;
    rmw::dots_partial_kernel<<<nblk, 256, sizeof(double) * 8, S.st>>>(rhs, 0, 1, rhs, n, part);
    rmw::reduce_partial_kernel<<<1, 32, 0, S.st>>>(part, nblk, 1, nrm2, 0);
    double h = 0.0;
    RMW_CUDA(cudaMemcpyAsync(&h, nrm2, sizeof(double), cudaMemcpyDeviceToHost, S.st));
    RMW_CUDA(cudaStreamSynchronize(S.st));
    const double nrm = std::sqrt(h);
    if (!std::isfinite(nrm)) return rmw::fail(RMW_ERR_NONFINITE, "right-hand side is not finite");
    if (nrm == 0.0) {
        RMW_CUDA(cudaMemsetAsync(sol, 0, sizeof(double) * n, S.st));
        RMW_CUDA(cudaStreamSynchronize(S.st));
        if (iters_host) *iters_host = 0;
        if (relres_host) *relres_host = 0.0;
        return RMW_OK;
    }
    const unsigned g = (unsigned)((n + 255) / 256);
    rmw::div_scalar_kernel<<<g, 256, 0, S.st>>>(rhs, bs, n, nrm);
    const int rc = rmw_rigid_solve(sys, bs, sol, tol, restart, maxiter, mode, iters_host, relres_host);
    if (rc != RMW_OK && rc != RMW_ERR_NOT_CONVERGED) return rc;
    rmw::axpby_kernel<<<g, 256, 0, S.st>>>(sol, sol, n, 0.0, nrm);
    RMW_CHECK_LAUNCH("rmw_rigid_solve_scaled");
    return rc;
}

static int rigid_solve_impl(void *sys, const double *rhs, double *sol, double tol, int restart, int maxiter,
                            int mode, int *iters_host, double *relres_host)
{
    if (!sys || !rhs || !sol) return rmw::fail(RMW_ERR_ARG, "null argument");
    if (!(tol > 0)) return rmw::fail(RMW_ERR_ARG, "tolerance must be positive");
    if (mode != RMW_MODE_FP64 && mode != RMW_MODE_MIXED && mode != RMW_MODE_DF64)
        return rmw::fail(RMW_ERR_ARG, "unknown precision mode");
    RigidSystem &S = *(RigidSystem *)sys;
    // an FP32-factorised preconditioner serves the mixed solves only
    if (!S.pc_ready || (S.pc_fp32 && mode != RMW_MODE_MIXED)) {
        if (int rc = rmw_rigid_build_pc_mode(sys, 0, mode)) return rc;
    }
    const long long n = S.sys_size();
    // the mixed solves apply the preconditioner in FP32 (their refinement
    // residual is FP64-accurate); its FP32 copies are made before any capture
    if (mode == RMW_MODE_MIXED)
        if (int rc = rmw::rigid_pc_prepare_f32(S)) return rc;
    auto pc = [&](const double *x, double *y) {
        return mode == RMW_MODE_MIXED ? rmw::rigid_apply_pc_mixed(S, x, y) : rmw::rigid_apply_pc(S, x, y);
    };
    // A P^-1 fused through a private buffer and replayed as one CUDA graph
    double *pbuf = nullptr;
    RMW_CUDA(rmw::dmalloc_async(&pbuf, sizeof(double) * n, S.st));
    struct FreeP {
        double *p;
        cudaStream_t s;
        ~FreeP() { cudaFreeAsync(p, s); }
    } free_p{pbuf, S.st};
    auto fused = [&](int m) {
        return [&, m](const double *x, double *y) -> int {
            if (int rc = pc(x, pbuf)) return rc;
            return rmw::rigid_apply(S, pbuf, y, m);
        };
    };
    auto gop = rmw::make_graph_op(fused(mode == RMW_MODE_MIXED ? RMW_MODE_MIXED : mode), &S.st, n, n);
    auto pcop = [&](const double *x, double *y) -> int { return gop(x, y); };
    // device-resident restart cycles (fused CGS2 + Givens step kernel, one
    // graph launch per cycle) unless switched off or unavailable
    const bool dev = rmw::krylov_device_enabled() && rmw::krylov_device_available();
    auto fop = fused(mode == RMW_MODE_MIXED ? RMW_MODE_MIXED : mode);
    rmw::GmresDevice<decltype(fop)> E(fop, &S.st);
    if (dev) {
        if (int rc = E.init({0, n}, restart, 0)) return rc;
    }
    // one GMRES solve of A x = b to tol (x from 0) on operator A = opA
    auto gmres = [&](auto opA, const double *b, double *x, double tl, int mi, int *it, double *rr,
                     bool trust = false) -> int {
        if (!dev) return rmw::gmres_right(opA, pc, pcop, b, x, n, tl, restart, mi, S.st, it, rr, nullptr);
        std::vector<int> its, stt;
        std::vector<double> rrs;
        if (int rc = E.solve(opA, pc, b, x, {tl}, mi, its, rrs, stt, nullptr, trust)) return rc;
        *it = its[0];
        *rr = rrs[0];
        if (stt[0] == RMW_ERR_NOT_CONVERGED) rmw::set_error("GMRES reached maxiter without converging");
        if (stt[0] == RMW_ERR_BREAKDOWN) rmw::set_error("GMRES breakdown");
        return stt[0];
    };
    if (mode == RMW_MODE_FP64 || mode == RMW_MODE_DF64) {
        auto op = [&](const double *x, double *y) { return rmw::rigid_apply(S, x, y, mode); };
        int it = 0;
        double rr = 0.0;
        const int rc = gmres(op, rhs, sol, tol, maxiter, &it, &rr);
        if (iters_host) *iters_host = it;
        if (relres_host) *relres_host = rr;
        return rc;
    }
    // mixed: inner GMRES on the FP32-pair operator; the refinement residual
    // b - A x uses the FP64-accurate double-float operator (<= 1e-12 against
    // FP64), or the recurrence r - A32 d once it is small enough
    auto op32 = [&](const double *x, double *y) { return rmw::rigid_apply(S, x, y, RMW_MODE_MIXED); };
    // x, r, d, A32 d, then the norm's block partials and result
    const int nblk = (int)((n + 1023) / 1024);
    double *buf = nullptr;
    RMW_CUDA(rmw::dmalloc_async(&buf, sizeof(double) * (4 * n + nblk + 1), S.st));
    double *x = buf, *r = buf + n, *d = buf + 2 * n, *ad = buf + 3 * n;
    double *part = buf + 4 * n, *nrm2 = part + nblk;
    RMW_CUDA(cudaMemsetAsync(x, 0, sizeof(double) * n, S.st));
    RMW_CUDA(cudaMemcpyAsync(r, rhs, sizeof(double) * n, cudaMemcpyDeviceToDevice, S.st));
    // |v| through the dots kernels (block partials, then one fixed-order sum)
    auto norm = [&](const double *v, double *out) -> int {
        rmw::dots_partial_kernel<<<nblk, 256, sizeof(double) * 8, S.st>>>(v, 0, 1, v, n, part);
        rmw::reduce_partial_kernel<<<1, 32, 0, S.st>>>(part, nblk, 1, nrm2, 0);
        double h = 0.0;
        RMW_CUDA(cudaMemcpyAsync(&h, nrm2, sizeof(double), cudaMemcpyDeviceToHost, S.st));
        RMW_CUDA(cudaStreamSynchronize(S.st));
        *out = std::sqrt(h);
        return RMW_OK;
    };
    double bnorm = 0.0;
    if (int rc = norm(rhs, &bnorm)) return rc;
    int total = 0;
    double relres = 0.0;
    int status = RMW_ERR_NOT_CONVERGED;
    const double inner_tol = 1e-5;
    // With the device engine the inner solves skip their closing FP32 residual
    // when the outer loop recomputes b - A x anyway, and hand it over as the
    // next residual when the outer loop takes the recurrence r - A32 d (the
    // same vector): one FP32-pair operator application less per refinement.
    // The first residual is b itself, whose norm is known.
    bool carried = true;
    double rnorm_next = bnorm;
    for (int outer = 0; outer < 8 && bnorm > 0.0; ++outer) {
        double rnorm = rnorm_next;
        if (!carried)
            if (int rc = norm(r, &rnorm)) return rc;
        relres = rnorm / bnorm;
        if (relres <= tol) { status = RMW_OK; break; }
        const double itol = std::max(inner_tol, 0.5 * tol * bnorm / rnorm);
        const bool recur = rmw::refine_by_recurrence(relres, tol);
        int it = 0;
        double rr = 0.0;
        int rc = gmres(op32, r, d, itol, std::max(1, maxiter - total), &it, &rr, dev && !recur);
        total += it;
        if (rc != RMW_OK && rc != RMW_ERR_NOT_CONVERGED) return rc;
        rmw::axpby_kernel<<<(unsigned)((n + 255) / 256), 256, 0, S.st>>>(d, x, n, 1.0, 1.0);
        void *rtok = nullptr;
        if (int rc2 = rmw::trace_begin(rmw::TRACE_REFINE, S.st, &rtok)) return rc2;
        carried = false;
        if (recur && dev) {
            // r - A32 d is the inner solve's closing residual
            RMW_CUDA(cudaMemcpyAsync(r, E.K.r, sizeof(double) * n, cudaMemcpyDeviceToDevice, S.st));
            carried = true;
            rnorm_next = rr * rnorm;
        } else if (recur) {
            // r = r - A32 d
            if (int rc2 = rmw::rigid_apply(S, d, ad, RMW_MODE_MIXED)) return rc2;
            rmw::axpby_kernel<<<(unsigned)((n + 255) / 256), 256, 0, S.st>>>(ad, r, n, -1.0, 1.0);
        } else {
            // r = b - A x with the FP64-accurate operator
            if (int rc2 = rmw::rigid_apply(S, x, r, RMW_MODE_DF64)) return rc2;
            rmw::axpby_kernel<<<(unsigned)((n + 255) / 256), 256, 0, S.st>>>(rhs, r, n, 1.0, -1.0);
        }
        if (int rc2 = rmw::trace_end(rtok, S.st)) return rc2;
        if (total >= maxiter) {
            if (int rc3 = norm(r, &rnorm)) return rc3;
            carried = false;
            relres = rnorm / bnorm;
            status = (relres <= tol) ? RMW_OK : RMW_ERR_NOT_CONVERGED;
            break;
        }
    }
    if (bnorm == 0.0) status = RMW_OK;
    RMW_CUDA(cudaMemcpyAsync(sol, x, sizeof(double) * n, cudaMemcpyDeviceToDevice, S.st));
    RMW_CUDA(cudaFreeAsync(buf, S.st));
    RMW_CUDA(cudaStreamSynchronize(S.st));
    if (iters_host) *iters_host = total;
    if (relres_host) *relres_host = relres;
    if (status != RMW_OK) rmw::set_error("mixed-precision refinement did not reach the tolerance");
    return status;
}

int rmw_rigid_lanczos(void *sys, const double *z, double *noise, double factor, double tol, int max_iter, int mode,
                      int *iters_host)
{
    if (!sys || !z || !noise) return rmw::fail(RMW_ERR_ARG, "null argument");
    if (max_iter < 1) return rmw::fail(RMW_ERR_ARG, "max_iter must be >= 1");
    RigidSystem &S = *(RigidSystem *)sys;
    if (!S.stoch_ready || (S.pc_fp32 && mode != RMW_MODE_MIXED)) {
        if (int rc = rmw_rigid_build_pc_mode(sys, 1, mode)) return rc;
    }
    auto op_direct = [&](const double *x, double *y) { return rmw::rigid_mobility_pc(S, x, y, mode); };
    const long long n = 3LL * S.n;
    auto gop = rmw::make_graph_op(op_direct, &S.st, n, n);  // one graph per application
    auto op = [&](const double *x, double *y) -> int { return gop(x, y); };
    double *tmp = nullptr;
    RMW_CUDA(rmw::dmalloc_async(&tmp, sizeof(double) * n, S.st));
    int rc = RMW_OK;
    if (rmw::krylov_device_enabled() && rmw::krylov_device_available()) {
        // device-resident iterations (fused step kernel, one graph launch per call)
        rmw::LanczosDevice<decltype(op_direct)> D(op_direct, &S.st);
        std::vector<int> its;
        rc = D.run(z, tmp, factor, tol, max_iter, std::max(2, std::min(max_iter + 1, 1000)), {0, n}, its,
                   rmw::LzMask(), true);
        if (rc == RMW_OK && iters_host) *iters_host = its[0];
    } else {
        rc = rmw::lanczos(op, z, tmp, n, factor, tol, max_iter, S.st, iters_host);
    }
    if (rc == RMW_OK) rc = rmw::rigid_P_inv_mult(S, tmp, noise);
    RMW_CUDA(cudaFreeAsync(tmp, S.st));
    RMW_CUDA(cudaStreamSynchronize(S.st));
    return rc;
}

// Generic right-preconditioned GMRES with caller-supplied operators.
int rmw_gmres(int64_t n, rmw_operator_fn op, void *op_ctx, rmw_operator_fn pc, void *pc_ctx, const double *b,
              double *x, double tol, int restart, int maxiter, void *stream, int *iters_host, double *relres_host,
              double *history_host, int history_cap)
{
    if (!op || !b || !x) return rmw::fail(RMW_ERR_ARG, "null argument");
    if (n <= 0) return rmw::fail(RMW_ERR_ARG, "n must be positive");
    if (!(tol > 0)) return rmw::fail(RMW_ERR_ARG, "tolerance must be positive");
    cudaStream_t st = rmw::as_stream(stream);
    auto A = [&](const double *xx, double *yy) -> int {
        int rc = op(op_ctx, xx, yy);
        return rc ? rmw::fail(rc, "operator callback failed") : RMW_OK;
    };
    auto P = [&](const double *xx, double *yy) -> int {
        if (!pc) {
            RMW_CUDA(cudaMemcpyAsync(yy, xx, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
            return RMW_OK;
        }
        int rc = pc(pc_ctx, xx, yy);
        return rc ? rmw::fail(rc, "preconditioner callback failed") : RMW_OK;
    };
    double *tmp = nullptr;
    RMW_CUDA(rmw::dmalloc_async(&tmp, sizeof(double) * n, st));
    auto AP = [&](const double *xx, double *yy) -> int {
        if (int rc = P(xx, tmp)) return rc;
        return A(tmp, yy);
    };
    std::vector<double> hist;
    int rc = rmw::gmres_right(A, P, AP, b, x, n, tol, restart, maxiter, st, iters_host, relres_host, &hist);
    cudaFreeAsync(tmp, st);
    if (history_host)
        for (int i = 0; i < (int)hist.size() && i < history_cap; ++i) history_host[i] = hist[i];
    return rc;
}

// Generic Lanczos noise = factor * M^(1/2) z with a caller-supplied operator.
int rmw_lanczos(int64_t n, rmw_operator_fn op, void *op_ctx, const double *z, double *noise, double factor,
                double tol, int max_iter, void *stream, int *iters_host)
{
    if (!op || !z || !noise) return rmw::fail(RMW_ERR_ARG, "null argument");
    if (n <= 0 || max_iter < 1) return rmw::fail(RMW_ERR_ARG, "n and max_iter must be positive");
    auto A = [&](const double *xx, double *yy) -> int {
        int rc = op(op_ctx, xx, yy);
        return rc ? rmw::fail(rc, "operator callback failed") : RMW_OK;
    };
    return rmw::lanczos(A, z, noise, n, factor, tol, max_iter, rmw::as_stream(stream), iters_host);
}

// Lanczos on the plain (unpreconditioned) wall mobility of n free blobs.
int rmw_wall_lanczos(const double *r, const double *z, double *noise, int64_t n, double eta, double a,
                     const double *L_host, double factor, double tol, int max_iter, int mode, void *stream,
                     int *iters_host)
{
    if (!r || !z || !noise) return rmw::fail(RMW_ERR_ARG, "null argument");
    if (n <= 0) return rmw::fail(RMW_ERR_ARG, "n must be positive");
    cudaStream_t st = rmw::as_stream(stream);
    auto op = [&](const double *x, double *y) {
        return rmw::wall_product(RMW_UF, r, x, y, n, eta, a, L_host, mode, st);
    };
    if (rmw::krylov_device_enabled() && rmw::krylov_device_available()) {
        auto op_dev = [&](const double *x, double *y) {  // on the engine's stream (redirected while capturing)
            return rmw::wall_product(RMW_UF, r, x, y, n, eta, a, L_host, mode, st);
        };
        rmw::LanczosDevice<decltype(op_dev)> D(op_dev, &st);
        std::vector<int> its;
        const int rc = D.run(z, noise, factor, tol, max_iter, std::max(2, std::min(max_iter + 1, 1000)),
                             {0, 3 * (long long)n}, its, rmw::LzMask(), true);
        if (rc == RMW_OK && iters_host) *iters_host = its[0];
        return rc;
    }
    return rmw::lanczos(op, z, noise, 3 * n, factor, tol, max_iter, st, iters_host);
}

}  // extern "C"

namespace rmw {
int wall_force_torque(const double *r, const double *F, const double *T, double *U, double *W, int64_t n,
                      double eta, double a, const double *L, int mode, cudaStream_t st);
}

extern "C" {

// Rollers with a prescribed angular velocity
// (quaternion_integrator/quaternion_integrator_rollers.py:905-983): the torques
// solve M_WT torque = omega - M_WF force by unpreconditioned GMRES from zero
// (relative tolerance, restart), then velocity = M_UF force + M_UT torque.
// wall = 1: single-wall products; 0: free space.  Device arrays of 3n doubles.
int rmw_rollers_velocity_and_torque(const double *r, const double *force, const double *omega, double *velocity,
                                    double *torque, int64_t n, double eta, double a, const double *L_host, int wall,
                                    double tol, int restart, int maxiter, int mode, void *stream, int *iters_host,
                                    double *relres_host)
{
    if (!r || !force || !omega || !velocity || !torque) return rmw::fail(RMW_ERR_ARG, "null argument");
    if (n <= 0 || n > (int64_t(1) << 28)) return rmw::fail(RMW_ERR_ARG, "number of rollers out of range [1, 2^28]");
    if (!(tol > 0) || maxiter < 1) return rmw::fail(RMW_ERR_ARG, "tolerance and maxiter must be positive");
    if (!(eta > 0) || !(a > 0)) return rmw::fail(RMW_ERR_ARG, "viscosity and radius must be positive");
    if (mode != RMW_MODE_FP64 && mode != RMW_MODE_MIXED && mode != RMW_MODE_DF64)
        return rmw::fail(RMW_ERR_ARG, "unknown precision mode");
    cudaStream_t st = rmw::as_stream(stream);
    const long long m = 3 * (long long)n;
    auto product = [&](int kind, const double *x, double *y) -> int {
        return wall ? rmw::wall_product(kind, r, x, y, n, eta, a, L_host, mode, st)
                    : rmw::nowall_product(kind, r, x, y, n, eta, a, L_host, mode, st);
    };
    double *rhs = nullptr;
    RMW_CUDA(rmw::dmalloc_async(&rhs, sizeof(double) * 2 * m, st));
    double *tmp = rhs + m;
    struct Free {
        double *p;
        cudaStream_t s;
        ~Free() { cudaFreeAsync(p, s); }
    } free_rhs{rhs, st};
    // rhs = omega - M_WF force
    if (int rc = product(RMW_WF, force, rhs)) return rc;
    rmw::axpby_kernel<<<(unsigned)((m + 255) / 256), 256, 0, st>>>(omega, rhs, m, 1.0, -1.0);
    RMW_CHECK_LAUNCH("rollers right-hand side");
    auto op = [&](const double *x, double *y) -> int { return product(RMW_WT, x, y); };
    auto pc = [&](const double *x, double *y) -> int {
        RMW_CUDA(cudaMemcpyAsync(y, x, sizeof(double) * m, cudaMemcpyDeviceToDevice, st));
        return RMW_OK;
    };
    const int status =
        rmw::gmres_right(op, pc, op, rhs, torque, m, tol, restart, maxiter, st, iters_host, relres_host, nullptr);
    if (status != RMW_OK && status != RMW_ERR_NOT_CONVERGED) return status;
    // velocity = M_UF force + M_UT torque
    if (wall) {
        if (int rc = rmw::wall_force_torque(r, force, torque, velocity, nullptr, n, eta, a, L_host, mode, st))
            return rc;
    } else {
        if (int rc = product(RMW_UF, force, velocity)) return rc;
        if (int rc = product(RMW_UT, torque, tmp)) return rc;
        rmw::axpby_kernel<<<(unsigned)((m + 255) / 256), 256, 0, st>>>(tmp, velocity, m, 1.0, 1.0);
        RMW_CHECK_LAUNCH("rollers velocity");
    }
    RMW_CUDA(cudaStreamSynchronize(st));
    if (status != RMW_OK) rmw::set_error("rollers torque solve did not reach the tolerance");
    return status;
}

}  // extern "C"
