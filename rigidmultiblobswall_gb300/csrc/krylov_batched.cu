// Batched Krylov solves of many independent rigid suspensions on one GPU.
//
// The suspensions live in one rigid handle (bodies concatenated) whose pair
// product is segmented by suspension (rmw_rigid_set_suspensions), so the
// operator is block-diagonal over suspensions.  Each suspension runs its own
// right-preconditioned restarted GMRES - its own Krylov basis, Hessenberg
// matrix, Givens rotations, tolerance and iteration count - but all advance
// in lockstep: one operator application, one preconditioner application and
// one set of segmented Gram-Schmidt kernels per step serve every suspension.
// Krylov vectors use an instance-major layout (suspension k's [lambda_k; U_k]
// contiguous), so every per-suspension reduction is over a contiguous segment;
// gather/scatter kernels map to and from the operator's [lambda; U] layout.
// A suspension that has converged is frozen by zeroing its segment: the
// operator maps zero to zero, so it costs no further attention.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "graph_op.cuh"
#include "krylov_device.cuh"
#include "rigid.cuh"
#include "wall_pair.cuh"

namespace rmw {

constexpr int kSegThreads = 256;
constexpr int kSegElems = 4;  // elements per thread per job
constexpr int kSegChunk = 64; // basis vectors per pass (shared coefficient array)

struct VecJob {
    int seg;
    long long b, e;
};

__global__ void seg_dots_kernel(const double *__restrict__ V, long long ldv, int k, const double *__restrict__ w,
                                const VecJob *__restrict__ jobs, double *__restrict__ partial)
{
    __shared__ double red[kSegChunk * (kSegThreads / 32)];
    const VecJob jb = jobs[blockIdx.x];
    const int nw = blockDim.x / 32, wid = threadIdx.x / 32, lane = threadIdx.x & 31;
    double wv[kSegElems];
#pragma unroll
    for (int e = 0; e < kSegElems; ++e) {
        const long long i = jb.b + threadIdx.x + (long long)e * blockDim.x;
        wv[e] = (i < jb.e) ? w[i] : 0.0;
    }
    for (int q = 0; q < k; ++q) {
        const double *Vq = V + (long long)q * ldv;
        double acc = 0.0;
#pragma unroll
        for (int e = 0; e < kSegElems; ++e) {
            const long long i = jb.b + threadIdx.x + (long long)e * blockDim.x;
            if (i < jb.e) acc += Vq[i] * wv[e];
        }
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) red[q * nw + wid] = acc;
    }
    __syncthreads();
    for (int q = threadIdx.x; q < k; q += blockDim.x) {
        double s = 0.0;
        for (int j = 0; j < nw; ++j) s += red[q * nw + j];
        partial[(long long)blockIdx.x * k + q] = s;
    }
}

// out[seg * stride + off + q] = sum over the segment's jobs of partial[job * k + q]
__global__ void seg_reduce_kernel(const double *__restrict__ partial, int k, const int *__restrict__ job_off,
                                  int nseg, double *__restrict__ out, int stride, int off)
{
    const int wq = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (wq >= nseg * k) return;
    const int seg = wq / k, q = wq % k;
    double s = 0.0;
    for (int j = job_off[seg] + lane; j < job_off[seg + 1]; j += 32) s += partial[(long long)j * k + q];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) out[(long long)seg * stride + off + q] = s;
}

// w -= V H[seg] (coefficients at H[seg*stride + off + q]); optional per-job |w|^2
__global__ void seg_update_kernel(const double *__restrict__ V, long long ldv, int k, const double *__restrict__ H,
                                  int stride, int off, double *__restrict__ w, const VecJob *__restrict__ jobs,
                                  double *__restrict__ norm_partial)
{
    __shared__ double hs[kSegChunk];
    __shared__ double red[32];
    const VecJob jb = jobs[blockIdx.x];
    for (int q = threadIdx.x; q < k; q += blockDim.x) hs[q] = H[(long long)jb.seg * stride + off + q];
    __syncthreads();
    double nrm = 0.0;
#pragma unroll
    for (int e = 0; e < kSegElems; ++e) {
        const long long i = jb.b + threadIdx.x + (long long)e * blockDim.x;
        if (i < jb.e) {
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

// y = x * f(S[seg*stride + off]) with f = identity (inv_sqrt = 0) or 1/sqrt (0 for 0)
__global__ void seg_scale_kernel(const double *__restrict__ x, double *__restrict__ y,
                                 const VecJob *__restrict__ jobs, const double *__restrict__ S, int stride, int off,
                                 int inv_sqrt)
{
    const VecJob jb = jobs[blockIdx.x];
    double a = S[(long long)jb.seg * stride + off];
    if (inv_sqrt) a = (a > 0.0) ? 1.0 / sqrt(a) : 0.0;
#pragma unroll
    for (int e = 0; e < kSegElems; ++e) {
        const long long i = jb.b + threadIdx.x + (long long)e * blockDim.x;
        if (i < jb.e) y[i] = a * x[i];
    }
}

// out (+)= V C[seg]
__global__ void seg_combine_kernel(const double *__restrict__ V, long long ldv, int k, const double *__restrict__ C,
                                   int stride, int off, double *__restrict__ out, const VecJob *__restrict__ jobs,
                                   int accumulate)
{
    __shared__ double cs[kSegChunk];
    const VecJob jb = jobs[blockIdx.x];
    for (int q = threadIdx.x; q < k; q += blockDim.x) cs[q] = C[(long long)jb.seg * stride + off + q];
    __syncthreads();
#pragma unroll
    for (int e = 0; e < kSegElems; ++e) {
        const long long i = jb.b + threadIdx.x + (long long)e * blockDim.x;
        if (i < jb.e) {
            double s = 0.0;
            for (int q = 0; q < k; ++q) s += cs[q] * V[(long long)q * ldv + i];
            out[i] = accumulate ? out[i] + s : s;
        }
    }
}

__global__ void permute_kernel(const double *__restrict__ x, double *__restrict__ y, const long long *__restrict__ idx,
                               long long n, int scatter)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (scatter) y[idx[i]] = x[i];
    else y[i] = x[idx[i]];
}

__global__ void axpby_batched_kernel(const double *__restrict__ x, double *__restrict__ y, long long n, double a,
                                     double b)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = a * x[i] + b * y[i];
}

// ---------------------------------------------------------------------------
// host side: segmented vector operations on instance-major vectors
struct SegOps {
    cudaStream_t st = 0;
    long long n = 0;
    int nseg = 0, njobs = 0, stride = 0;
    VecJob *jobs = nullptr;      // device
    int *job_off = nullptr;      // device, nseg + 1
    double *partial = nullptr;   // device, njobs * kSegChunk
    double *S = nullptr;         // device scalars, nseg * stride
    double *Sh = nullptr;        // pinned host mirror
    void *base = nullptr;

    int init(const std::vector<long long> &off, int stride_, cudaStream_t s)
    {
        st = s;
        nseg = (int)off.size() - 1;
        n = off.back();
        stride = stride_;
        std::vector<VecJob> jb;
        std::vector<int> jo(nseg + 1, 0);
        const long long per = (long long)kSegThreads * kSegElems;
        for (int k = 0; k < nseg; ++k) {
            jo[k] = (int)jb.size();
            for (long long b = off[k]; b < off[k + 1]; b += per) jb.push_back({k, b, std::min(off[k + 1], b + per)});
        }
        jo[nseg] = (int)jb.size();
        njobs = (int)jb.size();
        const size_t bytes = sizeof(VecJob) * std::max(1, njobs) + sizeof(int) * (nseg + 1) + 64 +
                             sizeof(double) * ((size_t)std::max(1, njobs) * kSegChunk + (size_t)nseg * stride);
        RMW_CUDA(rmw::dmalloc_async(&base, bytes + 256, st));
        char *p = (char *)base;
        jobs = (VecJob *)p;
        p += ((sizeof(VecJob) * std::max(1, njobs) + 15) / 16) * 16;
        job_off = (int *)p;
        p += ((sizeof(int) * (nseg + 1) + 15) / 16) * 16;
        partial = (double *)p;
        p += sizeof(double) * (size_t)std::max(1, njobs) * kSegChunk;
        S = (double *)p;
        if (njobs) RMW_CUDA(cudaMemcpyAsync(jobs, jb.data(), sizeof(VecJob) * njobs, cudaMemcpyHostToDevice, st));
        RMW_CUDA(cudaMemcpyAsync(job_off, jo.data(), sizeof(int) * (nseg + 1), cudaMemcpyHostToDevice, st));
        RMW_CUDA(cudaHostAlloc(&Sh, sizeof(double) * (size_t)nseg * stride, cudaHostAllocDefault));
        RMW_CUDA(cudaMemsetAsync(S, 0, sizeof(double) * (size_t)nseg * stride, st));
        RMW_CUDA(cudaStreamSynchronize(st));
        return RMW_OK;
    }
    ~SegOps()
    {
        if (base) cudaFreeAsync(base, st);
        if (Sh) {
            cudaStreamSynchronize(st);
            cudaFreeHost(Sh);
        }
    }
    int dots(const double *V, long long ldv, int k, const double *w, int off)
    {
        if (njobs == 0) return RMW_OK;
        for (int q0 = 0; q0 < k; q0 += kSegChunk) {
            const int kc = std::min(kSegChunk, k - q0);
            seg_dots_kernel<<<njobs, kSegThreads, 0, st>>>(V + (long long)q0 * ldv, ldv, kc, w, jobs, partial);
            seg_reduce_kernel<<<(nseg * kc * 32 + 255) / 256, 256, 0, st>>>(partial, kc, job_off, nseg, S, stride,
                                                                             off + q0);
        }
        RMW_CHECK_LAUNCH("segmented dots");
        return RMW_OK;
    }
    int update(const double *V, long long ldv, int k, int hoff, double *w, int nrm_off)
    {
        if (njobs == 0) return RMW_OK;
        for (int q0 = 0; q0 < k; q0 += kSegChunk) {
            const int kc = std::min(kSegChunk, k - q0);
            const bool last = q0 + kc >= k;
            seg_update_kernel<<<njobs, kSegThreads, 0, st>>>(V + (long long)q0 * ldv, ldv, kc, S, stride, hoff + q0,
                                                             w, jobs, (last && nrm_off >= 0) ? partial : nullptr);
        }
        if (nrm_off >= 0)
            seg_reduce_kernel<<<(nseg * 32 + 255) / 256, 256, 0, st>>>(partial, 1, job_off, nseg, S, stride, nrm_off);
        RMW_CHECK_LAUNCH("segmented update");
        return RMW_OK;
    }
    int norm2(const double *w, int off)
    {
        if (njobs == 0) return RMW_OK;
        seg_dots_kernel<<<njobs, kSegThreads, 0, st>>>(w, 0, 1, w, jobs, partial);
        seg_reduce_kernel<<<(nseg * 32 + 255) / 256, 256, 0, st>>>(partial, 1, job_off, nseg, S, stride, off);
        RMW_CHECK_LAUNCH("segmented norm");
        return RMW_OK;
    }
    int scale(const double *x, double *y, int off, bool inv_sqrt)
    {
        if (njobs == 0) return RMW_OK;
        seg_scale_kernel<<<njobs, kSegThreads, 0, st>>>(x, y, jobs, S, stride, off, inv_sqrt ? 1 : 0);
        RMW_CHECK_LAUNCH("segmented scale");
        return RMW_OK;
    }
    int combine(const double *V, long long ldv, int k, int coff, double *out)
    {
        if (njobs == 0) return RMW_OK;
        if (k == 0) {
            RMW_CUDA(cudaMemsetAsync(out, 0, sizeof(double) * n, st));
            return RMW_OK;
        }
        for (int q0 = 0; q0 < k; q0 += kSegChunk) {
            const int kc = std::min(kSegChunk, k - q0);
            seg_combine_kernel<<<njobs, kSegThreads, 0, st>>>(V + (long long)q0 * ldv, ldv, kc, S, stride, coff + q0,
                                                              out, jobs, q0 > 0);
        }
        RMW_CHECK_LAUNCH("segmented combine");
        return RMW_OK;
    }
    int fetch()
    {
        RMW_CUDA(cudaMemcpyAsync(Sh, S, sizeof(double) * (size_t)nseg * stride, cudaMemcpyDeviceToHost, st));
        RMW_CUDA(cudaStreamSynchronize(st));
        return RMW_OK;
    }
    int put()
    {
        RMW_CUDA(cudaMemcpyAsync(S, Sh, sizeof(double) * (size_t)nseg * stride, cudaMemcpyHostToDevice, st));
        return RMW_OK;
    }
    double &h(int seg, int off) { return Sh[(size_t)seg * stride + off]; }
    int axpby(const double *x, double *y, double a, double b)
    {
        axpby_batched_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(x, y, n, a, b);
        RMW_CHECK_LAUNCH("axpby");
        return RMW_OK;
    }
};

// Batched right-preconditioned restarted GMRES (zero initial guess).
// op/pc act on instance-major vectors.  tol_abs[k] is suspension k's absolute
// residual target; a suspension whose b segment is zero is solved by x = 0.
// pcop(x, y) = op(pc(x)): the Arnoldi step's operator, given separately so that
// the caller can fuse and graph-capture it
template <typename Op, typename Pc, typename PcOp>
static int gmres_batched(Op op, Pc pc, PcOp pcop, const double *b, double *x_out, const std::vector<long long> &off,
                         const std::vector<double> &tol_rel, int restart, int maxiter, cudaStream_t st,
                         std::vector<int> &iters, std::vector<double> &relres, std::vector<int> &status)
{
    restart = std::max(1, std::min(restart, 60));
    const int nseg = (int)off.size() - 1;
    const long long n = off.back();
    const long long ldv = ((n + 31) / 32) * 32;
    const int R = restart;
    const int H1 = 0, H2 = R + 2, NW = 2 * R + 4, NR = 2 * R + 5, NB = 2 * R + 6, AL = 2 * R + 7, YC = 2 * R + 8;
    const int stride = 3 * R + 16;
    SegOps O;
    if (int rc = O.init(off, stride, st)) return rc;
    double *buf = nullptr;
    RMW_CUDA(rmw::dmalloc_async(&buf, sizeof(double) * ldv * (R + 6), st));
    struct Free {
        double *p;
        cudaStream_t s;
        ~Free() { cudaFreeAsync(p, s); }
    } fr{buf, st};
    double *V = buf, *w = V + ldv * (R + 1), *x = w + ldv, *r = x + ldv, *t1 = r + ldv, *t2 = t1 + ldv;
    iters.assign(nseg, 0);
    relres.assign(nseg, 0.0);
    status.assign(nseg, RMW_ERR_NOT_CONVERGED);
    RMW_CUDA(cudaMemsetAsync(x, 0, sizeof(double) * n, st));
    RMW_CUDA(cudaMemcpyAsync(r, b, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
    if (int rc = O.norm2(b, NB)) return rc;
    if (int rc = O.fetch()) return rc;
    std::vector<double> bnorm(nseg), tol_abs(nseg), beta(nseg);
    std::vector<char> active(nseg);
    int n_active = 0;
    for (int k = 0; k < nseg; ++k) {
        bnorm[k] = std::sqrt(O.h(k, NB));
        if (!std::isfinite(bnorm[k])) return fail(RMW_ERR_NONFINITE, "batched GMRES: right-hand side not finite");
        tol_abs[k] = tol_rel[k] * bnorm[k];
        beta[k] = bnorm[k];
        active[k] = bnorm[k] > 0.0;
        if (!active[k]) status[k] = RMW_OK;
        n_active += active[k];
    }
    std::vector<double> H((size_t)nseg * (R + 1) * R), cs((size_t)nseg * R), sn((size_t)nseg * R),
        g((size_t)nseg * (R + 1));
    std::vector<int> jdone(nseg);
    std::vector<char> done_cycle(nseg);
    while (n_active > 0) {
        for (int k = 0; k < nseg; ++k) O.h(k, AL) = active[k] ? 1.0 / beta[k] : 0.0;
        if (int rc = O.put()) return rc;
        if (int rc = O.scale(r, V, AL, false)) return rc;  // frozen segments become zero
        for (int k = 0; k < nseg; ++k) {
            std::fill(&g[(size_t)k * (R + 1)], &g[(size_t)k * (R + 1)] + R + 1, 0.0);
            g[(size_t)k * (R + 1)] = beta[k];
            jdone[k] = 0;
            done_cycle[k] = !active[k];
        }
        int jmax = 0;
        for (int j = 0; j < R; ++j) {
            double *Vj = V + (long long)j * ldv, *Vn = V + (long long)(j + 1) * ldv;
            if (int rc = pcop(Vj, w)) return rc;
            // CGS2 per segment; algorithmic bytes as in the single-system GMRES
            void *tok = nullptr;
            if (int rc = trace_begin(TRACE_KRYLOV, st, &tok)) return rc;
            if (int rc = O.dots(V, ldv, j + 1, w, H1)) return rc;
            if (int rc = O.update(V, ldv, j + 1, H1, w, -1)) return rc;
            if (int rc = O.dots(V, ldv, j + 1, w, H2)) return rc;
            if (int rc = O.update(V, ldv, j + 1, H2, w, NW)) return rc;
            if (int rc = O.scale(w, Vn, NW, true)) return rc;
            if (int rc = trace_end(tok, st)) return rc;
            if (tok) trace_bytes(TRACE_KRYLOV, 8.0 * (4.0 * j + 12.0) * (double)n);
            if (int rc = O.fetch()) return rc;
            jmax = j + 1;
            int still = 0;
            for (int k = 0; k < nseg; ++k) {
                if (done_cycle[k]) continue;
                double *hc = &H[((size_t)k * R + j) * (R + 1)];
                for (int q = 0; q <= j; ++q) hc[q] = O.h(k, H1 + q) + O.h(k, H2 + q);
                hc[j + 1] = std::sqrt(O.h(k, NW));
                if (!std::isfinite(hc[j + 1])) return fail(RMW_ERR_BREAKDOWN, "batched GMRES: non-finite vector");
                double *c = &cs[(size_t)k * R], *sv = &sn[(size_t)k * R], *gk = &g[(size_t)k * (R + 1)];
                for (int q = 0; q < j; ++q) {
                    const double t = c[q] * hc[q] + sv[q] * hc[q + 1];
                    hc[q + 1] = -sv[q] * hc[q] + c[q] * hc[q + 1];
                    hc[q] = t;
                }
                const double den = std::hypot(hc[j], hc[j + 1]);
                c[j] = (den == 0.0) ? 1.0 : hc[j] / den;
                sv[j] = (den == 0.0) ? 0.0 : hc[j + 1] / den;
                hc[j] = c[j] * hc[j] + sv[j] * hc[j + 1];
                hc[j + 1] = 0.0;
                gk[j + 1] = -sv[j] * gk[j];
                gk[j] = c[j] * gk[j];
                ++iters[k];
                jdone[k] = j + 1;
                const bool breakdown = std::sqrt(O.h(k, NW)) == 0.0;
                if (std::fabs(gk[j + 1]) <= tol_abs[k] || iters[k] >= maxiter || breakdown) done_cycle[k] = 1;
                else ++still;
            }
            if (still == 0) break;
        }
        // per-suspension back substitution; y into the scalar area
        for (int k = 0; k < nseg; ++k) {
            for (int q = 0; q < R; ++q) O.h(k, YC + q) = 0.0;
            if (!active[k]) continue;
            const int jd = jdone[k];
            const double *gk = &g[(size_t)k * (R + 1)];
            for (int q = jd - 1; q >= 0; --q) {
                double sacc = gk[q];
                for (int c = q + 1; c < jd; ++c) sacc -= H[((size_t)k * R + c) * (R + 1) + q] * O.h(k, YC + c);
                const double d = H[((size_t)k * R + q) * (R + 1) + q];
                O.h(k, YC + q) = (d != 0.0) ? sacc / d : 0.0;
            }
        }
        if (int rc = O.put()) return rc;
        if (int rc = O.combine(V, ldv, jmax, YC, t1)) return rc;
        if (int rc = pc(t1, t2)) return rc;
        if (int rc = O.axpby(t2, x, 1.0, 1.0)) return rc;
        if (int rc = op(x, r)) return rc;
        if (int rc = O.axpby(b, r, 1.0, -1.0)) return rc;
        if (int rc = O.norm2(r, NR)) return rc;
        if (int rc = O.fetch()) return rc;
        n_active = 0;
        for (int k = 0; k < nseg; ++k) {
            if (!active[k]) continue;
            beta[k] = std::sqrt(O.h(k, NR));
            relres[k] = beta[k] / bnorm[k];
            if (!std::isfinite(beta[k])) return fail(RMW_ERR_BREAKDOWN, "batched GMRES: non-finite residual");
            if (beta[k] <= tol_abs[k]) {
                status[k] = RMW_OK;
                active[k] = 0;
            } else if (iters[k] >= maxiter) {
                status[k] = RMW_ERR_NOT_CONVERGED;
                active[k] = 0;
            } else {
                ++n_active;
            }
        }
    }
    RMW_CUDA(cudaMemcpyAsync(x_out, x, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
    RMW_CUDA(cudaStreamSynchronize(st));
    return RMW_OK;
}

// implicit-QL eigen-decomposition of a symmetric tridiagonal matrix (krylov.cu)
bool tridiag_eigen_host(std::vector<double> &d, std::vector<double> e, std::vector<double> &z);

// Lockstep Lanczos over independent segments (one per suspension and right-
// hand side): each segment has its own recurrence, tridiagonal matrix,
// eigen-decomposition and convergence test (stochastic_forcing.py:112-264),
// the operator is applied to all of them at once.  Converged segments are
// frozen by zeroing their part of the next basis vector.
// before_op(active) runs before every operator application with the
// segments' current active flags (converged segments are 0).
template <typename Op, typename Pre>
static int lanczos_batched(Op op, const double *z, double *noise, const std::vector<long long> &off, double factor,
                           double tol, int max_iter, cudaStream_t st, std::vector<int> &iters, Pre before_op)
{
    const int nseg = (int)off.size() - 1;
    const long long n = off.back();
    const long long ldv = ((n + 31) / 32) * 32;
    const int kcap = std::max(2, std::min(max_iter + 1, 96));
    const int HD = 0, HS = 1, ZN = 2, CF = 8;  // per-segment scalars; CF: coefficients (kcap)
    const int stride = CF + 2 * kcap + 8;
    SegOps O;
    if (int rc = O.init(off, stride, st)) return rc;
    int vcap = std::min(kcap + 1, 16);
    double *V = nullptr, *w = nullptr;
    RMW_CUDA(rmw::dmalloc_async(&w, sizeof(double) * ldv, st));
    RMW_CUDA(rmw::dmalloc_async(&V, sizeof(double) * ldv * vcap, st));
    struct Free {
        double **a, **b;
        cudaStream_t s;
        ~Free() { if (*a) cudaFreeAsync(*a, s); if (*b) cudaFreeAsync(*b, s); }
    } fr{&V, &w, st};
    if (int rc = O.norm2(z, ZN)) return rc;
    if (int rc = O.fetch()) return rc;
    std::vector<double> zn(nseg);
    std::vector<char> active(nseg, 0);
    iters.assign(nseg, max_iter);
    for (int k = 0; k < nseg; ++k) {
        zn[k] = std::sqrt(O.h(k, ZN));
        if (!std::isfinite(zn[k])) return fail(RMW_ERR_NONFINITE, "batched Lanczos: z not finite");
        active[k] = zn[k] > 0.0 && factor != 0.0;
        if (!active[k]) iters[k] = 0;
        O.h(k, HD) = active[k] ? 1.0 / zn[k] : 0.0;
        for (int q = 0; q < kcap; ++q) O.h(k, CF + q) = 0.0;
    }
    if (int rc = O.put()) return rc;
    if (int rc = O.scale(z, V, HD, false)) return rc;
    std::vector<std::vector<double>> hd(nseg), hs(nseg), cold(nseg), cfin(nseg);
    int kmax_used = 1;
    for (int i = 0; i <= max_iter && i < kcap; ++i) {
        int n_active = 0;
        for (int k = 0; k < nseg; ++k) n_active += active[k];
        if (!n_active) break;
        double *Vi = V + (long long)i * ldv;
        if (int rc = before_op(active)) return rc;
        if (int rc = op(Vi, w)) return rc;
        if (i > 0) {  // w -= hs[i-1] V_{i-1}
            if (int rc = O.fetch()) return rc;
            for (int k = 0; k < nseg; ++k) O.h(k, HS) = active[k] ? hs[k][i - 1] : 0.0;
            if (int rc = O.put()) return rc;
            if (int rc = O.update(V + (long long)(i - 1) * ldv, ldv, 1, HS, w, -1)) return rc;
        }
        if (int rc = O.dots(Vi, ldv, 1, w, HD)) return rc;        // hd = <w, V_i>
        if (int rc = O.update(Vi, ldv, 1, HD, w, ZN)) return rc;  // w -= hd V_i ; |w|^2
        if (int rc = O.scale(w, w, ZN, true)) return rc;          // w /= |w|
        if (int rc = O.fetch()) return rc;
        for (int k = 0; k < nseg; ++k) {
            if (!active[k]) continue;
            hd[k].push_back(O.h(k, HD));
            const double wn = std::sqrt(O.h(k, ZN));
            hs[k].push_back(wn);
            if (!std::isfinite(wn) || !std::isfinite(hd[k].back()))
                return fail(RMW_ERR_BREAKDOWN, "batched Lanczos: non-finite value");
            std::vector<double> dd(hd[k]), ee(hs[k].begin(), hs[k].begin() + i), zq;
            if (!tridiag_eigen_host(dd, ee, zq)) return fail(RMW_ERR_BREAKDOWN, "batched Lanczos: eigensolver");
            const int kk = i + 1;
            std::vector<double> c(kk, 0.0);
            for (int j = 0; j < kk; ++j) {
                const double lam = dd[j] > 0 ? std::sqrt(dd[j]) : 0.0;
                const double w1 = zq[(size_t)kk * j] * lam * zn[k] * factor;
                for (int q = 0; q < kk; ++q) c[q] += zq[q + (size_t)kk * j] * w1;
            }
            bool conv = false;
            if (i > 0) {
                double dn = 0.0, on = 0.0;
                for (int q = 0; q < kk; ++q) {
                    const double co = q < (int)cold[k].size() ? cold[k][q] : 0.0;
                    dn += (c[q] - co) * (c[q] - co);
                    on += co * co;
                }
                conv = std::sqrt(dn) / std::max(std::sqrt(on), 2.220446049250313e-16) < tol;
            }
            cold[k] = c;
            cfin[k] = c;
            if (conv || wn == 0.0) {
                iters[k] = i;
                active[k] = 0;
            }
        }
        kmax_used = i + 1;
        // reorthogonalise w against V_0..V_i (one pass) -> V_{i+1}; frozen segments get zeros
        if (int rc = O.dots(V, ldv, i + 1, w, CF + kcap)) return rc;
        if (int rc = O.update(V, ldv, i + 1, CF + kcap, w, -1)) return rc;
        if (i + 2 > vcap) {
            const int ncap = std::min(kcap + 1, 2 * vcap);
            double *nv = nullptr;
            RMW_CUDA(rmw::dmalloc_async(&nv, sizeof(double) * ldv * ncap, st));
            RMW_CUDA(cudaMemcpyAsync(nv, V, sizeof(double) * ldv * vcap, cudaMemcpyDeviceToDevice, st));
            RMW_CUDA(cudaFreeAsync(V, st));
            V = nv;
            vcap = ncap;
        }
        if (int rc = O.fetch()) return rc;
        for (int k = 0; k < nseg; ++k) O.h(k, HD) = active[k] ? 1.0 : 0.0;
        if (int rc = O.put()) return rc;
        if (int rc = O.scale(w, V + (long long)(i + 1) * ldv, HD, false)) return rc;
    }
    // noise = V c per segment
    if (int rc = O.fetch()) return rc;
    for (int k = 0; k < nseg; ++k)
        for (int q = 0; q < kcap; ++q) O.h(k, CF + q) = q < (int)cfin[k].size() ? cfin[k][q] : 0.0;
    if (int rc = O.put()) return rc;
    if (int rc = O.combine(V, ldv, kmax_used, CF, noise)) return rc;
    RMW_CUDA(cudaStreamSynchronize(st));
    return RMW_OK;
}

}  // namespace rmw

// ---------------------------------------------------------------------------
// C ABI
using rmw::RigidSystem;

extern "C" {

int rmw_rigid_set_suspensions(void *sys, int64_t n_suspensions, const int64_t *body_offsets_host)
{
    if (!sys || !body_offsets_host) return rmw::fail(RMW_ERR_ARG, "null argument");
    RigidSystem &S = *(RigidSystem *)sys;
    if (!S.wall) return rmw::fail(RMW_ERR_ARG, "batched suspensions are available with the wall only");
    if (n_suspensions <= 0 || body_offsets_host[0] != 0 || body_offsets_host[n_suspensions] != S.nb)
        return rmw::fail(RMW_ERR_ARG, "body offsets must run from 0 to the number of bodies");
    std::vector<long long> boff(n_suspensions + 1), blob_off(n_suspensions + 1), sys_off(n_suspensions + 1);
    for (int64_t k = 0; k <= n_suspensions; ++k) {
        boff[k] = body_offsets_host[k];
        if (k > 0 && boff[k] < boff[k - 1]) return rmw::fail(RMW_ERR_ARG, "body offsets must not decrease");
        blob_off[k] = S.boff_h[boff[k]];
    }
    if (S.batch) {
        rmw::wall_batch_free(*S.batch);
        delete S.batch;
        S.batch = nullptr;
    }
    S.batch = new rmw::WallBatch();
    if (int rc = rmw::wall_batch_build(*S.batch, blob_off.data(), (int)n_suspensions)) {
        delete S.batch;
        S.batch = nullptr;
        return rc;
    }
    // instance-major permutation: suspension k's [lambda_k; U_k] contiguous
    S.susp_body_off = boff;
    S.susp_off.assign(n_suspensions + 1, 0);
    std::vector<long long> perm((size_t)S.sys_size());
    long long pos = 0;
    for (int64_t k = 0; k < n_suspensions; ++k) {
        S.susp_off[k] = pos;
        for (long long t = 3 * blob_off[k]; t < 3 * blob_off[k + 1]; ++t) perm[pos++] = t;
        for (long long t = 3LL * S.n + 6 * boff[k]; t < 3LL * S.n + 6 * boff[k + 1]; ++t) perm[pos++] = t;
    }
    S.susp_off[n_suspensions] = pos;
    if (S.perm) cudaFree(S.perm);
    RMW_CUDA(cudaMalloc(&S.perm, sizeof(long long) * perm.size()));
    RMW_CUDA(cudaMemcpy(S.perm, perm.data(), sizeof(long long) * perm.size(), cudaMemcpyHostToDevice));
    return RMW_OK;
}

// Solve every suspension of the handle to its own relative residual tol
// (x = 0 start).  rhs and sol use the handle's [lambda; U] layout.
int rmw_rigid_solve_batched(void *sys, const double *rhs, double *sol, double tol, int restart, int maxiter, int mode,
                            int *iters_host, double *relres_host, int *status_host)
{
    if (!sys || !rhs || !sol) return rmw::fail(RMW_ERR_ARG, "null argument");
    RigidSystem &S = *(RigidSystem *)sys;
    if (!S.batch || !S.perm) return rmw::fail(RMW_ERR_ARG, "call rmw_rigid_set_suspensions first");
    if (!(tol > 0)) return rmw::fail(RMW_ERR_ARG, "tolerance must be positive");
    if (mode != RMW_MODE_FP64 && mode != RMW_MODE_MIXED && mode != RMW_MODE_DF64)
        return rmw::fail(RMW_ERR_ARG, "unknown precision mode");
    // an FP32-factorised preconditioner serves the mixed solves only
    if (!S.pc_ready || (S.pc_fp32 && mode != RMW_MODE_MIXED)) {
        if (int rc = rmw_rigid_build_pc_mode(sys, 0, mode)) return rc;
    }
    const int nseg = (int)S.susp_off.size() - 1;
    const long long n = S.sys_size();
    cudaStream_t st = S.st;
    double *buf = nullptr;
    RMW_CUDA(rmw::dmalloc_async(&buf, sizeof(double) * n * 7, st));
    double *gx = buf, *gy = buf + n, *bim = buf + 2 * n, *xim = buf + 3 * n, *rim = buf + 4 * n, *dim = buf + 5 * n;
    double *adim = buf + 6 * n;  // A32 d of the residual recurrence
    const unsigned pg = (unsigned)((n + 255) / 256);
    // S.st, not st: inside a graph capture the handle's stream is redirected
    auto to_global = [&](const double *xi, double *xg) { rmw::permute_kernel<<<pg, 256, 0, S.st>>>(xi, xg, S.perm, n, 1); };
    auto to_im = [&](const double *xg, double *xi) { rmw::permute_kernel<<<pg, 256, 0, S.st>>>(xg, xi, S.perm, n, 0); };
    auto op_mode = [&](int m) {
        return [&, m](const double *xi, double *yi) -> int {
            to_global(xi, gx);
            if (int rc = rmw::rigid_apply(S, gx, gy, m)) return rc;
            to_im(gy, yi);
            return RMW_OK;
        };
    };
    // the mixed solves apply the preconditioner in FP32 (see rigid_solve_impl)
    if (mode == RMW_MODE_MIXED) {
        if (int rc0 = rmw::rigid_pc_prepare_f32(S)) {
            cudaFreeAsync(buf, st);
            return rc0;
        }
    }
    auto apply_pc = [&](const double *x, double *y) {
        return mode == RMW_MODE_MIXED ? rmw::rigid_apply_pc_mixed(S, x, y) : rmw::rigid_apply_pc(S, x, y);
    };
    auto pc = [&](const double *xi, double *yi) -> int {
        to_global(xi, gx);
        if (int rc = apply_pc(gx, gy)) return rc;
        to_im(gy, yi);
        return RMW_OK;
    };
    // the Arnoldi operator A P^-1 over all suspensions, fused (no permutation
    // between the two) and replayed as one CUDA graph per application
    auto pcop_mode = [&](int m) {
        return [&, m](const double *xi, double *yi) -> int {
            to_global(xi, gx);
            if (int rc = apply_pc(gx, gy)) return rc;
            if (int rc = rmw::rigid_apply(S, gy, gx, m)) return rc;
            to_im(gx, yi);
            return RMW_OK;
        };
    };
    auto gop = rmw::make_graph_op(pcop_mode(mode == RMW_MODE_MIXED ? RMW_MODE_MIXED : mode), &S.st, n, n);
    auto pcop = [&](const double *xi, double *yi) -> int { return gop(xi, yi); };
    // device-resident restart cycles over all suspensions (one segment each)
    // unless switched off or unavailable
    const bool dev = rmw::krylov_device_enabled() && rmw::krylov_device_available();
    auto fop = pcop_mode(mode == RMW_MODE_MIXED ? RMW_MODE_MIXED : mode);
    rmw::GmresDevice<decltype(fop)> E(fop, &S.st);
    if (dev) {
        if (int rc0 = E.init(S.susp_off, std::min(restart, 60), 0)) {
            cudaFreeAsync(buf, st);
            return rc0;
        }
    }
    auto batched = [&](auto opA, const double *b, double *x, const std::vector<double> &tl, int mi,
                       std::vector<int> &its, std::vector<double> &rrs, std::vector<int> &sts) -> int {
        if (!dev) return rmw::gmres_batched(opA, pc, pcop, b, x, S.susp_off, tl, restart, mi, st, its, rrs, sts);
        return E.solve(opA, pc, b, x, tl, mi, its, rrs, sts);
    };
    to_im(rhs, bim);
    std::vector<int> it, stt, tot(nseg, 0);
    std::vector<double> rr;
    int rc = RMW_OK;
    if (mode != RMW_MODE_MIXED) {
        std::vector<double> tolv(nseg, tol);
        rc = batched(op_mode(mode), bim, xim, tolv, maxiter, it, rr, stt);
        tot = it;
    } else {
        // per-suspension iterative refinement: inner GMRES on the FP32-pair
        // operator, residual with the FP64-accurate double-float operator, or
        // by the recurrence r - A32 d once every pending suspension's residual
        // is small enough (refine_by_recurrence)
        RMW_CUDA(cudaMemsetAsync(xim, 0, sizeof(double) * n, st));
        RMW_CUDA(cudaMemcpyAsync(rim, bim, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
        rmw::SegOps O;
        if ((rc = O.init(S.susp_off, 4, st))) goto done;
        if ((rc = O.norm2(bim, 0))) goto done;
        if ((rc = O.fetch())) goto done;
        {
            std::vector<double> bn(nseg);
            for (int k = 0; k < nseg; ++k) bn[k] = std::sqrt(O.h(k, 0));
            rr.assign(nseg, 0.0);
            stt.assign(nseg, RMW_ERR_NOT_CONVERGED);
            std::vector<char> finished(nseg, 0);
            for (int outer = 0; outer < 8; ++outer) {
                if ((rc = O.norm2(rim, 1))) goto done;
                if ((rc = O.fetch())) goto done;
                std::vector<double> itol(nseg, 1.0);
                int pending = 0;
                bool recurrence = true;
                for (int k = 0; k < nseg; ++k) {
                    if (finished[k]) {  // residual, status and count stay as they were
                        O.h(k, 2) = 0.0;
                        continue;
                    }
                    const double rn = std::sqrt(O.h(k, 1));
                    rr[k] = bn[k] > 0 ? rn / bn[k] : 0.0;
                    const bool ok = rr[k] <= tol;
                    if (ok) stt[k] = RMW_OK;
                    const bool stop = ok || tot[k] >= maxiter;
                    finished[k] = stop;
                    O.h(k, 2) = stop ? 0.0 : 1.0;  // freeze finished suspensions (zero their residual)
                    itol[k] = stop ? 1.0 : std::max(1e-5, 0.5 * tol * bn[k] / std::max(rn, 1e-300));
                    pending += !stop;
                    if (!stop) recurrence = recurrence && rmw::refine_by_recurrence(rr[k], tol);
                }
                if (!pending) break;
                if ((rc = O.put())) goto done;
                if ((rc = O.scale(rim, rim, 2, false))) goto done;
                std::vector<double> rri;
                std::vector<int> si;
                rc = batched(op_mode(RMW_MODE_MIXED), rim, dim, itol, std::max(1, maxiter), it, rri, si);
                if (rc) goto done;
                for (int k = 0; k < nseg; ++k) tot[k] += it[k];
                if ((rc = O.axpby(dim, xim, 1.0, 1.0))) goto done;
                if (recurrence) {
                    // finished suspensions have r = 0 and d = 0 here and keep r = 0
                    if ((rc = op_mode(RMW_MODE_MIXED)(dim, adim))) goto done;
                    if ((rc = O.axpby(adim, rim, -1.0, 1.0))) goto done;
                } else {
                    if ((rc = op_mode(RMW_MODE_DF64)(xim, rim))) goto done;
                    if ((rc = O.axpby(bim, rim, 1.0, -1.0))) goto done;
                }
            }
        }
    }
    to_global(xim, sol);
done:
    cudaFreeAsync(buf, st);
    cudaStreamSynchronize(st);
    if (rc) return rc;
    int worst = RMW_OK;
    for (int k = 0; k < nseg; ++k) {
        if (iters_host) iters_host[k] = tot[k];
        if (relres_host) relres_host[k] = rr[k];
        if (status_host) status_host[k] = stt[k];
        if (stt[k] != RMW_OK) worst = stt[k];
    }
    if (worst != RMW_OK) rmw::set_error("some suspensions did not reach the tolerance");
    return worst;
}

// Lanczos noise for nrhs right-hand sides of every suspension of the handle:
// noise_q = factor * L (L^-1 M L^-T)^(1/2) z_q restricted to each suspension,
// i.e. stochastic_forcing_lanczos with the det_stoch preconditioner, run for
// every (suspension, right-hand side) pair in lockstep.  Z and noise hold nrhs
// rows of 3N doubles; iters_host receives nrhs * n_suspensions counts
// (row-major by right-hand side).
int rmw_rigid_lanczos_batched(void *sys, const double *Z, double *noise, int nrhs, double factor, double tol,
                              int max_iter, int mode, int *iters_host)
{
    if (!sys || !Z || !noise) return rmw::fail(RMW_ERR_ARG, "null argument");
    if (nrhs < 1 || max_iter < 1) return rmw::fail(RMW_ERR_ARG, "nrhs and max_iter must be positive");
    RigidSystem &S = *(RigidSystem *)sys;
    if (!S.batch) return rmw::fail(RMW_ERR_ARG, "call rmw_rigid_set_suspensions first");
    if (!S.stoch_ready || (S.pc_fp32 && mode != RMW_MODE_MIXED)) {
        if (int rc = rmw_rigid_build_pc_mode(sys, 1, mode)) return rc;
    }
    const int nsusp = (int)S.susp_body_off.size() - 1;
    const long long N3 = 3LL * S.n;
    std::vector<long long> off((size_t)nrhs * nsusp + 1);
    for (int q = 0; q < nrhs; ++q)
        for (int k = 0; k < nsusp; ++k) off[(size_t)q * nsusp + k] = q * N3 + 3LL * S.batch->off[k];
    off[(size_t)nrhs * nsusp] = (long long)nrhs * N3;
    double *buf = nullptr;
    RMW_CUDA(rmw::dmalloc_async(&buf, sizeof(double) * 2 * nrhs * N3, S.st));
    double *tmp = buf, *raw = buf + nrhs * N3;
    // mixed precision: the multi-vector product skips suspensions whose
    // segments of a pass of 8 right-hand sides have all converged (their rows
    // are zero anyway), through one byte per (pass, suspension)
    const bool mask = (mode == RMW_MODE_MIXED) && S.wall;
    const int npass = (nrhs + rmw::kMultiPass - 1) / rmw::kMultiPass;
    unsigned char *d_act = nullptr;
    static thread_local unsigned char *h_act = nullptr;
    static thread_local size_t h_cap = 0;
    const size_t nact = (size_t)npass * nsusp;
    if (mask) {
        RMW_CUDA(rmw::dmalloc_async(&d_act, nact, S.st));
        if (h_cap < nact) {
            if (h_act) cudaFreeHost(h_act);
            RMW_CUDA(cudaHostAlloc(&h_act, nact, cudaHostAllocDefault));
            h_cap = nact;
        }
    }
    auto op_direct = [&](const double *x, double *y) {
        return rmw::rigid_mobility_pc_multi(S, x, y, nrhs, mode, tmp, d_act);
    };
    auto gop = rmw::make_graph_op(op_direct, &S.st, nrhs * N3, nrhs * N3);  // one graph per application
    auto op = [&](const double *x, double *y) -> int { return gop(x, y); };
    auto before_op = [&](const std::vector<char> &act) -> int {
        if (!mask) return RMW_OK;
        for (int p = 0; p < npass; ++p)
            for (int k = 0; k < nsusp; ++k) {
                unsigned char any = 0;
                for (int q = rmw::kMultiPass * p; q < std::min(nrhs, rmw::kMultiPass * (p + 1)); ++q)
                    any |= act[(size_t)q * nsusp + k] ? 1 : 0;
                h_act[(size_t)p * nsusp + k] = any;
            }
        RMW_CUDA(cudaMemcpyAsync(d_act, h_act, nact, cudaMemcpyHostToDevice, S.st));
        return RMW_OK;
    };
    std::vector<int> it;
    int rc = RMW_OK;
    if (rmw::krylov_device_enabled() && rmw::krylov_device_available()) {
        // device-resident lockstep iterations: the step kernel updates the
        // (pass, suspension) activity bytes of the multi-vector product itself
        rmw::LanczosDevice<decltype(op_direct)> D(op_direct, &S.st);
        rmw::LzMask mk;
        if (mask) {
            mk.mask = d_act;
            mk.nsusp = nsusp;
            mk.nrhs = nrhs;
            mk.pass = rmw::kMultiPass;
        }
        rc = D.run(Z, raw, factor, tol, max_iter, std::max(2, std::min(max_iter + 1, 96)), off, it, mk);
    } else {
        rc = rmw::lanczos_batched(op, Z, raw, off, factor, tol, max_iter, S.st, it, before_op);
    }
    if (d_act) cudaFreeAsync(d_act, S.st);
    if (rc == RMW_OK) rc = rmw::rigid_P_inv_mult_multi(S, raw, noise, nrhs, mode);
    cudaFreeAsync(buf, S.st);
    cudaStreamSynchronize(S.st);
    if (rc) return rc;
    if (iters_host)
        for (size_t k = 0; k < it.size(); ++k) iters_host[k] = it[k];
    return RMW_OK;
}

}  // extern "C"
