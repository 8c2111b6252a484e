// Kernels and buffers of the device-resident GMRES engine (krylov_device.cuh).
#include <atomic>
#include <cstring>

#include "krylov_device.cuh"

namespace rmw {

// spins of a grid barrier before it gives up (about 0.3 s with the 64 ns sleeps)
constexpr unsigned kBarrierSpins = 1u << 22;
// tridiagonal matrices up to this size are diagonalised in shared memory
constexpr int kLzShared = 256;

// ---------------------------------------------------------------------------
// device helpers

__device__ __forceinline__ double warp_sum(double v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Sum of eight values over the warp, transposed across the lanes: 9 shuffles
// and 9 adds instead of 40 + 40.  Lane l ends with the sum of value
// u(l) = 4 b4 + 2 b3 + b2 (b_i the bits of l; the four lanes of a group hold
// the same sum); the order of the adds is fixed.
__device__ __forceinline__ double warp_sum8(const double a[8], int lane)
{
    const bool h4 = lane & 16, h3 = lane & 8, h2 = lane & 4;
    double b[4], c[2];
#pragma unroll
    for (int i = 0; i < 4; ++i)
        b[i] = (h4 ? a[i + 4] : a[i]) + __shfl_xor_sync(0xffffffffu, h4 ? a[i] : a[i + 4], 16);
#pragma unroll
    for (int i = 0; i < 2; ++i)
        c[i] = (h3 ? b[i + 2] : b[i]) + __shfl_xor_sync(0xffffffffu, h3 ? b[i] : b[i + 2], 8);
    double d = (h2 ? c[1] : c[0]) + __shfl_xor_sync(0xffffffffu, h2 ? c[0] : c[1], 4);
    d += __shfl_xor_sync(0xffffffffu, d, 2);
    d += __shfl_xor_sync(0xffffffffu, d, 1);
    return d;
}

// Grid barrier of a cooperative launch: generation counter, bounded spin.
__device__ void grid_barrier(GridBar *b)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned *vgen = &b->gen;
        const unsigned gen = *vgen;
        __threadfence();
        const unsigned arrived = atomicAdd(&b->count, 1u);
        if (arrived == gridDim.x - 1) {
            atomicExch(&b->count, 0u);
            __threadfence();
            atomicAdd(&b->gen, 1u);
        } else {
            unsigned spins = 0;
            while (*vgen == gen) {
                if (++spins > kBarrierSpins) {
                    atomicExch(&b->err, 1);
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
    }
    __syncthreads();
}

// hs[q] = sum over jobs [j0, j1) of part[job * KP + q], q < k, in a fixed
// order (lanes over jobs, then a butterfly): every CTA gets identical values.
__device__ void reduce_segment(const double *part, int KP, int j0, int j1, int k, double *hs)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int q = wid; q < k; q += nw) {
        double s = 0.0;
        for (int jb = j0 + lane; jb < j1; jb += 32) s += __ldcg(part + (long long)jb * KP + q);
        s = warp_sum(s);
        if (lane == 0) hs[q] = s;
    }
    __syncthreads();
}

// part[job * KP + q] = sum_{i in job} V_q[i] w[i], q < k (red: k x 32 shared
// doubles); eight basis vectors per pass over the job, so that each thread has
// several independent loads in flight.  w[i] comes from wval(i, first): first
// is true on the first pass over the job, where wval may also form w[i] and
// store it (each thread reads back only the entries it stored).
template <typename WVal>
__device__ void job_dots_w(const double *__restrict__ V, long long ldv, int k, const KJob jb, double *part, int KP,
                           int job, double *red, WVal wval)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int q0 = 0; q0 < k; q0 += 8) {
        const int nq = min(8, k - q0);
        const double *V0 = V + (long long)q0 * ldv;
        double a[8] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
        for (long long i = jb.b + threadIdx.x; i < jb.e; i += blockDim.x) {
            const double wi = wval(i, q0 == 0);
#pragma unroll
            for (int u = 0; u < 8; ++u)
                if (u < nq) a[u] = fma(V0[(long long)u * ldv + i], wi, a[u]);
        }
        const double sum = warp_sum8(a, lane);
        const int u = ((lane >> 4) & 1) * 4 + ((lane >> 3) & 1) * 2 + ((lane >> 2) & 1);
        if ((lane & 3) == 0 && u < nq) red[(q0 + u) * 32 + wid] = sum;
    }
    __syncthreads();
    for (int q = threadIdx.x; q < k; q += blockDim.x) {
        double s = 0.0;
        for (int u = 0; u < nw; ++u) s += red[q * 32 + u];
        part[(long long)job * KP + q] = s;
    }
    __syncthreads();
}

__device__ void job_dots(const double *__restrict__ V, long long ldv, int k, const double *w, const KJob jb,
                         double *part, int KP, int job, double *red)
{
    job_dots_w(V, ldv, k, jb, part, KP, job, red, [w](long long i, bool) { return w[i]; });
}

// w[i] -= sum_q hs[q] V_q[i] over the job, the new w[i] also stored to c1 and
// c2 when given; returns this thread's sum of the new w[i]^2
__device__ double job_update(const double *__restrict__ V, long long ldv, int k, const double *hs, double *w,
                             const KJob jb, double *c1 = nullptr, double *c2 = nullptr)
{
    double nrm = 0.0;
    for (long long i = jb.b + threadIdx.x; i < jb.e; i += blockDim.x) {
        double x = w[i];
#pragma unroll 8
        for (int q = 0; q < k; ++q) x = fma(-hs[q], V[(long long)q * ldv + i], x);
        w[i] = x;
        if (c1) {
            c1[i] = x;
            c2[i] = x;
        }
        nrm = fma(x, x, nrm);
    }
    return nrm;
}

// block sum of one value per thread (fixed order) into part[job * KP]
__device__ void job_norm_partial(double v, double *part, int KP, int job, double *red)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    v = warp_sum(v);
    if (lane == 0) red[wid] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int u = 0; u < nw; ++u) s += red[u];
        part[(long long)job * KP] = s;
    }
    __syncthreads();
}

struct StepArgs {
    double *V;
    long long ldv;
    double *w, *xin;
    const KJob *jobs;
    const int *sjob, *bjob;
    double *partA, *partB, *partC;
    int KP, R, hcap;
    double *H, *cs, *sn, *g, *hc1, *hc2, *hist, *gres;
    const double *tol_abs;
    int *iters, *jdone, *cyc, *flags;
    KState *st;
    unsigned long long cond;
    int use_cond;
};

// One Arnoldi step of every segment: CGS2 against V_0..V_j, V_{j+1} = w/|w|
// (also written to xin, the operator's next input), the Givens update of the
// Hessenberg column and the stopping test.  Cooperative launch, one CTA per
// SM at most; CTA b works on the jobs [bjob[b], bjob[b+1]).
__global__ void __launch_bounds__(kKdThreads, 1) arnoldi_step_kernel(StepArgs A)
{
    __shared__ double red[kKdMaxBasis * 32];
    __shared__ double hs[kKdMaxBasis];
    const int j = *(volatile int *)&A.st->j;
    const int k = j + 1;
    const int jb0 = A.bjob[blockIdx.x], jb1 = A.bjob[blockIdx.x + 1];
    // pass 1: partial dots V^T w
    for (int job = jb0; job < jb1; ++job) job_dots(A.V, A.ldv, k, A.w, A.jobs[job], A.partA, A.KP, job, red);
    grid_barrier(&A.st->bar);
    // pass 2: w -= V h1, partial dots V^T w again
    for (int job = jb0; job < jb1; ++job) {
        const KJob jb = A.jobs[job];
        reduce_segment(A.partA, A.KP, A.sjob[jb.seg], A.sjob[jb.seg + 1], k, hs);
        if (job == A.sjob[jb.seg])
            for (int q = threadIdx.x; q < k; q += blockDim.x) A.hc1[(long long)jb.seg * A.KP + q] = hs[q];
        job_update(A.V, A.ldv, k, hs, A.w, jb);
        __syncthreads();
        job_dots(A.V, A.ldv, k, A.w, jb, A.partB, A.KP, job, red);
    }
    grid_barrier(&A.st->bar);
    // pass 3: w -= V h2, partial |w|^2
    for (int job = jb0; job < jb1; ++job) {
        const KJob jb = A.jobs[job];
        reduce_segment(A.partB, A.KP, A.sjob[jb.seg], A.sjob[jb.seg + 1], k, hs);
        if (job == A.sjob[jb.seg])
            for (int q = threadIdx.x; q < k; q += blockDim.x) A.hc2[(long long)jb.seg * A.KP + q] = hs[q];
        const double nrm = job_update(A.V, A.ldv, k, hs, A.w, jb);
        __syncthreads();
        job_norm_partial(nrm, A.partC, A.KP, job, red);
    }
    grid_barrier(&A.st->bar);
    // pass 4: V_{j+1} = w / |w| (zero vector for |w| = 0); Givens by the CTA owning the segment's first job
    for (int job = jb0; job < jb1; ++job) {
        const KJob jb = A.jobs[job];
        reduce_segment(A.partC, A.KP, A.sjob[jb.seg], A.sjob[jb.seg + 1], 1, hs);
        const double nw = hs[0];
        const double inv = (nw > 0.0) ? 1.0 / sqrt(nw) : 0.0;
        double *Vn = A.V + (long long)(j + 1) * A.ldv;
        for (long long i = jb.b + threadIdx.x; i < jb.e; i += blockDim.x) {
            const double v = A.w[i] * inv;
            Vn[i] = v;
            A.xin[i] = v;
        }
        if (job == A.sjob[jb.seg]) {  // uniform over the CTA: it owns this segment's Givens update
            const int s = jb.seg, R = A.R;
            double *col = red, *cq = red + kKdMaxBasis + 2, *sq = cq + kKdMaxBasis;  // shared scratch
            double *h = A.H + ((long long)s * R + j) * (R + 1);
            double *c = A.cs + (long long)s * R, *sv = A.sn + (long long)s * R, *gs = A.g + (long long)s * (R + 1);
            const bool run = A.cyc[s] != 0;
            for (int q = threadIdx.x; q <= j; q += blockDim.x)
                col[q] = A.hc1[(long long)s * A.KP + q] + A.hc2[(long long)s * A.KP + q];
            for (int q = threadIdx.x; q < j; q += blockDim.x) {
                cq[q] = c[q];
                sq[q] = sv[q];
            }
            __syncthreads();
            if (threadIdx.x == 0 && run) {
                const double hn = sqrt(nw);
                col[j + 1] = hn;
                int stop = 0;
                if (!isfinite(hn)) {
                    A.flags[s] |= 2;  // non-finite Arnoldi vector
                    stop = 1;
                } else {
                    for (int q = 0; q < j; ++q) {
                        const double t = cq[q] * col[q] + sq[q] * col[q + 1];
                        col[q + 1] = -sq[q] * col[q] + cq[q] * col[q + 1];
                        col[q] = t;
                    }
                    const double den = hypot(col[j], col[j + 1]);
                    const double cj = (den == 0.0) ? 1.0 : col[j] / den;
                    const double sj = (den == 0.0) ? 0.0 : col[j + 1] / den;
                    c[j] = cj;
                    sv[j] = sj;
                    col[j] = cj * col[j] + sj * col[j + 1];
                    col[j + 1] = 0.0;
                    const double gj = gs[j];
                    gs[j + 1] = -sj * gj;
                    gs[j] = cj * gj;
                    const int it = ++A.iters[s];
                    A.jdone[s] = j + 1;
                    const double res = fabs(sj * gj);
                    if (A.hist && it <= A.hcap) A.hist[(long long)s * A.hcap + it - 1] = res;
                    const bool conv = res <= A.tol_abs[s];
                    A.gres[s] = res;
                    if (conv) A.flags[s] |= 4;                 // the estimate met the tolerance
                    if (hn == 0.0 && !conv) A.flags[s] |= 1;  // breakdown without convergence
                    stop = conv || hn == 0.0 || it >= A.st->maxiter;
                }
                if (stop) A.cyc[s] = 0;
                else atomicAdd(&A.st->active, 1);
            }
            __syncthreads();
            if (run)
                for (int q = threadIdx.x; q <= j + 1; q += blockDim.x) h[q] = col[q];
        }
        __syncthreads();
    }
    // the last CTA to finish advances the step and sets the loop condition
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned prev = atomicAdd(&A.st->bar.done, 1u);
        if (prev == gridDim.x - 1) {
            __threadfence();
            const int act = atomicAdd(&A.st->active, 0);
            const int jn = j + 1;
            const int more = (act > 0 && jn < A.R && !*(volatile int *)&A.st->bar.err) ? 1 : 0;
            A.st->j = jn;
            A.st->active = 0;
            A.st->more = more;
            atomicExch(&A.st->bar.done, 0u);
            __threadfence();
            if (A.use_cond) cudaGraphSetConditional((cudaGraphConditionalHandle)A.cond, (unsigned)more);
        }
    }
}

// per-job |v|^2 partials (one CTA per job)
__global__ void seg_norm_partial_kernel(const double *__restrict__ v, const KJob *__restrict__ jobs,
                                        double *__restrict__ part)
{
    __shared__ double red[32];
    const KJob jb = jobs[blockIdx.x];
    double s = 0.0;
    for (long long i = jb.b + threadIdx.x; i < jb.e; i += blockDim.x) s = fma(v[i], v[i], s);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    s = warp_sum(s);
    if (lane == 0) red[wid] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int u = 0; u < nw; ++u) t += red[u];
        part[blockIdx.x] = t;
    }
}

// nrm[s] = sum of the segment's job partials (one warp per segment)
__global__ void seg_norm_reduce_kernel(const double *__restrict__ part, const int *__restrict__ sjob, int nseg,
                                       double *__restrict__ nrm)
{
    const int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (s >= nseg) return;
    double t = 0.0;
    for (int jb = sjob[s] + lane; jb < sjob[s + 1]; jb += 32) t += part[jb];
    t = warp_sum(t);
    if (lane == 0) nrm[s] = t;
}

// V_0 = alpha_seg r, xin = V_0 (one CTA per job)
__global__ void cycle_begin_kernel(const double *__restrict__ r, double *__restrict__ V0, double *__restrict__ xin,
                                   const KJob *__restrict__ jobs, const double *__restrict__ alpha)
{
    const KJob jb = jobs[blockIdx.x];
    const double a = alpha[jb.seg];
    for (long long i = jb.b + threadIdx.x; i < jb.e; i += blockDim.x) {
        const double v = a * r[i];
        V0[i] = v;
        xin[i] = v;
    }
}

// per-segment cycle state: g = (beta, 0, ...), cycle flag, step counters
__global__ void cycle_state_kernel(const double *__restrict__ beta, const double *__restrict__ cycf, int nseg, int R,
                                   double *__restrict__ g, int *__restrict__ cyc, int *__restrict__ jdone,
                                   KState *__restrict__ st)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < nseg) {
        double *gs = g + (long long)s * (R + 1);
        gs[0] = beta[s];
        for (int q = 1; q <= R; ++q) gs[q] = 0.0;
        cyc[s] = cycf[s] != 0.0;
        jdone[s] = 0;
    }
    if (s == 0) {
        st->j = 0;
        st->active = 0;
        st->bar.done = 0;
        st->more = 1;
    }
}

// y = R^-1 g per segment (back substitution; zero beyond the steps done)
__global__ void backsub_kernel(const double *__restrict__ H, const double *__restrict__ g,
                               const int *__restrict__ jdone, int nseg, int R, int KP, double *__restrict__ y)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nseg) return;
    const int jd = jdone[s];
    double *ys = y + (long long)s * KP;
    const double *Hs = H + (long long)s * R * (R + 1);
    const double *gs = g + (long long)s * (R + 1);
    for (int q = jd; q < KP; ++q) ys[q] = 0.0;
    for (int q = jd - 1; q >= 0; --q) {
        double acc = gs[q];
        for (int c = q + 1; c < jd; ++c) acc -= Hs[(long long)c * (R + 1) + q] * ys[c];
        const double d = Hs[(long long)q * (R + 1) + q];
        ys[q] = (d != 0.0) ? acc / d : 0.0;
    }
}

// out = V_{0..k} y_seg (one CTA per job)
__global__ void seg_combine_kernel_dev(const double *__restrict__ V, long long ldv, int k,
                                       const double *__restrict__ y, int KP, const KJob *__restrict__ jobs,
                                       double *__restrict__ out)
{
    __shared__ double ys[kKdMaxBasis];
    const KJob jb = jobs[blockIdx.x];
    for (int q = threadIdx.x; q < k; q += blockDim.x) ys[q] = y[(long long)jb.seg * KP + q];
    __syncthreads();
    for (long long i = jb.b + threadIdx.x; i < jb.e; i += blockDim.x) {
        double s = 0.0;
        for (int q = 0; q < k; ++q) s = fma(ys[q], V[(long long)q * ldv + i], s);
        out[i] = s;
    }
}

__global__ void kd_axpby_kernel(const double *__restrict__ x, double *__restrict__ y, long long n, double a,
                                double b)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = a * x[i] + b * y[i];
}

// ---------------------------------------------------------------------------
// Lanczos

// Symmetric tridiagonal eigen-decomposition by implicit QL (the classical
// algorithm of Bowdler, Martin, Reinsch and Wilkinson, as the host routine of
// the library), run by one warp: every lane carries the scalar recurrence
// (identical values, so each lane reads back its own writes of d and e) and
// lane l applies the rotations to rows l, l+32, ... of z (k x k,
// column-major).  On exit d holds the eigenvalues.
__device__ bool tridiag_eigen_warp(double *d, double *e, double *z, int k, int lane)
{
    for (int q = lane; q < k; q += 32)
        for (int c = 0; c < k; ++c) z[q + (long long)k * c] = (q == c) ? 1.0 : 0.0;
    e[k - 1] = 0.0;
    for (int l = 0; l < k; ++l) {
        int iter = 0, m;
        do {
            for (m = l; m < k - 1; ++m) {
                const double dd = fabs(d[m]) + fabs(d[m + 1]);
                if (fabs(e[m]) <= 1e-16 * dd) break;
            }
            if (m != l) {
                if (++iter > 60) return false;
                double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
                double r = hypot(g, 1.0);
                g = d[m] - d[l] + e[l] / (g + (g >= 0 ? fabs(r) : -fabs(r)));
                double s = 1.0, c = 1.0, p = 0.0;
                int i;
                for (i = m - 1; i >= l; --i) {
                    const double f = s * e[i], b = c * e[i];
                    r = hypot(f, g);
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
                    for (int q = lane; q < k; q += 32) {
                        double *z1 = z + q + (long long)k * (i + 1), *z0 = z + q + (long long)k * i;
                        const double t = *z1;
                        *z1 = s * *z0 + c * t;
                        *z0 = c * *z0 - s * t;
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

struct LzArgs {
    double *w, *xin;
    const KJob *jobs;
    const int *sjob, *bjob;
    double *partA, *partB, *partC;
    int KP, kcap;
    double *hd, *hs, *c, *cold, *dt, *et, *z;  // per segment: kcap (z: kcap^2)
    const double *zn;                          // |z_s|
    double factor, tol;
    int *iters, *cyc, *kfin, *flags;
    LzState *st;
    unsigned char *mask;  // optional (pass, suspension) activity bytes of the next operator application
    int nsusp, nrhs, pass;
    unsigned long long cond;
    int use_cond;
};

// One Lanczos iteration i of every segment (stochastic_forcing.py:112-264):
// w -= hs[i-1] V_{i-1}; hd[i] = <w, V_i>; w -= hd[i] V_i; hs[i] = |w|;
// w /= hs[i]; one classical reorthogonalisation pass against V_0..V_i;
// V_{i+1} = w (also the operator's next input).  The CTA owning a segment's
// first job then diagonalises the (i+1) x (i+1) tridiagonal matrix with one
// warp, forms the coefficients c of the noise |z| factor V^T Q sqrt(L) Q^T e1
// and applies the stopping test |c - c_old| < tol |c_old|.  A segment that
// stopped at the previous iteration is frozen (its w and next vector zero).
__global__ void __launch_bounds__(kKdThreads, 3) lanczos_step_kernel(LzArgs A)
{
    __shared__ double red[kKdMaxBasis * 32];
    __shared__ double hsh[kKdMaxBasis];
    __shared__ double tdg[kLzShared], tsd[kLzShared];  // the owner warp's tridiagonal matrix
    __shared__ int actv[8];
    const int i = *(volatile int *)&A.st->i;
    const int k = i + 1;
    double *const V = *(double *volatile *)&A.st->V;
    const long long ldv = A.st->ldv;
    const int jb0 = A.bjob[blockIdx.x], jb1 = A.bjob[blockIdx.x + 1];
    // frozen segments: read once, before any owner can change them (owners write after the last barrier)
    for (int job = jb0; job < jb1 && job - jb0 < 8; ++job)
        if (threadIdx.x == 0) actv[job - jb0] = A.cyc[A.jobs[job].seg];
    __syncthreads();
    // pass 1: w -= hs[i-1] V_{i-1} (frozen: w = 0) and, in the same pass, partial <w, V_i>
    for (int job = jb0; job < jb1; ++job) {
        const KJob jb = A.jobs[job];
        const bool on = (job - jb0 < 8) ? actv[job - jb0] != 0 : A.cyc[jb.seg] != 0;
        const double hp = (i > 0) ? A.hs[(long long)jb.seg * A.kcap + i - 1] : 0.0;
        const double *Vp = V + (long long)(i > 0 ? i - 1 : 0) * ldv;
        double *w = A.w;
        job_dots_w(V + (long long)i * ldv, ldv, 1, jb, A.partA, A.KP, job, red, [=](long long e, bool) {
            const double x = on ? ((i > 0) ? fma(-hp, Vp[e], w[e]) : w[e]) : 0.0;
            w[e] = x;
            return x;
        });
    }
    grid_barrier(&A.st->bar);
    // pass 2: hd = <w, V_i>; w -= hd V_i; partial |w|^2
    for (int job = jb0; job < jb1; ++job) {
        const KJob jb = A.jobs[job];
        reduce_segment(A.partA, A.KP, A.sjob[jb.seg], A.sjob[jb.seg + 1], 1, hsh);
        const double nrm = job_update(V + (long long)i * ldv, ldv, 1, hsh, A.w, jb);
        if (job == A.sjob[jb.seg] && threadIdx.x == 0) A.dt[(long long)jb.seg * A.kcap] = hsh[0];  // hd[i], kept below
        __syncthreads();
        job_norm_partial(nrm, A.partC, A.KP, job, red);
    }
    grid_barrier(&A.st->bar);
    // pass 3: hs = |w|; w /= hs (0 on an exact breakdown) during the first pass of the partial
    // reorthogonalisation dots V_q^T w
    for (int job = jb0; job < jb1; ++job) {
        const KJob jb = A.jobs[job];
        reduce_segment(A.partC, A.KP, A.sjob[jb.seg], A.sjob[jb.seg + 1], 1, hsh);
        const double wn = sqrt(hsh[0]);
        const double inv = (wn > 0.0) ? 1.0 / wn : 0.0;
        if (job == A.sjob[jb.seg] && threadIdx.x == 0) A.et[(long long)jb.seg * A.kcap] = wn;
        __syncthreads();
        double *w = A.w;
        for (int q0 = 0; q0 < k; q0 += kKdMaxBasis)
            job_dots_w(V + (long long)q0 * ldv, ldv, min(kKdMaxBasis, k - q0), jb, A.partB + q0, A.KP, job, red,
                       [=](long long e, bool first) {
                           if (q0 == 0 && first) {
                               const double x = w[e] * inv;
                               w[e] = x;
                               return x;
                           }
                           return w[e];
                       });
    }
    grid_barrier(&A.st->bar);
    // pass 4: w -= V h; V_{i+1} = w; owners: tridiagonal eigen-problem, coefficients, stopping test
    for (int job = jb0; job < jb1; ++job) {
        const KJob jb = A.jobs[job];
        double *Vn = V + (long long)(i + 1) * ldv;
        for (int q0 = 0; q0 < k; q0 += kKdMaxBasis) {
            const int kc = min(kKdMaxBasis, k - q0);
            reduce_segment(A.partB + q0, A.KP, A.sjob[jb.seg], A.sjob[jb.seg + 1], kc, hsh);
            // the last group's pass also writes V_{i+1} and the operator's next input
            const bool last = q0 + kc >= k;
            job_update(V + (long long)q0 * ldv, ldv, kc, hsh, A.w, jb, last ? Vn : nullptr, last ? A.xin : nullptr);
            __syncthreads();
        }
        const int s = jb.seg;
        if (job == A.sjob[s] && A.cyc[s] && threadIdx.x < 32) {
            const int lane = threadIdx.x;
            const long long so = (long long)s * A.kcap;
            const double hdi = A.dt[so], wn = A.et[so];
            if (lane == 0) {
                A.hd[so + i] = hdi;
                A.hs[so + i] = wn;
            }
            __syncwarp();
            const bool host_checks = A.st->host != 0;  // the host checks convergence from here on
            int stop = 0;
            if (host_checks) {
            } else if (!isfinite(wn) || !isfinite(hdi)) {
                if (lane == 0) A.flags[s] |= 2;
                stop = 1;
            } else {
                // the eigen-problem in shared memory while it fits (the global copies otherwise): its
                // recurrence is a long chain of dependent accesses
                double *d = (k <= kLzShared) ? tdg : A.dt + so, *ee = (k <= kLzShared) ? tsd : A.et + so;
                double *zz = (k * k <= kKdMaxBasis * 32) ? red : A.z + (long long)s * A.kcap * A.kcap;
                for (int q = lane; q < k; q += 32) {
                    d[q] = A.hd[so + q];
                    ee[q] = (q < i) ? A.hs[so + q] : 0.0;
                }
                __syncwarp();
                const bool ok = tridiag_eigen_warp(d, ee, zz, k, lane);
                __syncwarp();
                if (!ok) {
                    if (lane == 0) A.flags[s] |= 4;
                    stop = 1;
                } else {
                    double *cc = A.c + so, *co = A.cold + so;
                    const double sc = A.zn[s] * A.factor;
                    double dn = 0.0, on = 0.0;
                    for (int q = lane; q < k; q += 32) {
                        double acc = 0.0;
                        for (int jj = 0; jj < k; ++jj) {
                            const double lam = d[jj] > 0.0 ? sqrt(d[jj]) : 0.0;
                            acc += zz[q + (long long)k * jj] * (zz[(long long)k * jj] * lam * sc);
                        }
                        const double old = (q < i) ? co[q] : 0.0;
                        dn += (acc - old) * (acc - old);
                        on += old * old;
                        cc[q] = acc;
                    }
                    dn = warp_sum(dn);
                    on = warp_sum(on);
                    __syncwarp();
                    for (int q = lane; q < k; q += 32) co[q] = cc[q];
                    const bool conv = i > 0 && sqrt(dn) / fmax(sqrt(on), 2.220446049250313e-16) < A.tol;
                    stop = conv || wn == 0.0;
                    if (lane == 0) {
                        A.kfin[s] = k;
                        if (stop) A.iters[s] = i;
                    }
                }
            }
            if (lane == 0 && !host_checks) {
                if (stop) A.cyc[s] = 0;
                else atomicAdd(&A.st->active, 1);
            }
        }
        __syncthreads();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned prev = atomicAdd(&A.st->bar.done, 1u);
        if (prev == gridDim.x - 1) {
            __threadfence();
            const int act = atomicAdd(&A.st->active, 0);
            const int in = i + 1;
            // stop when no segment is left, past max_iter, when the basis is full (the host grows it) or
            // when the tridiagonal matrix gets too large for the device eigen-solve (the host goes on)
            const int more = (act > 0 && in <= A.st->max_iter && in + 1 < A.st->vcap && in < A.st->dev_k &&
                              !*(volatile int *)&A.st->bar.err) ? 1 : 0;
            A.st->i = in;
            A.st->active = 0;
            A.st->more = more;
            A.st->live = act;
            if (A.mask) {
                const int npass = (A.nrhs + A.pass - 1) / A.pass;
                for (int p = 0; p < npass; ++p)
                    for (int u = 0; u < A.nsusp; ++u) {
                        unsigned char any = 0;
                        for (int q = p * A.pass; q < min(A.nrhs, (p + 1) * A.pass); ++q)
                            any |= A.cyc[(long long)q * A.nsusp + u] ? 1 : 0;
                        A.mask[(long long)p * A.nsusp + u] = any;
                    }
            }
            atomicExch(&A.st->bar.done, 0u);
            __threadfence();
            if (A.use_cond) cudaGraphSetConditional((cudaGraphConditionalHandle)A.cond, (unsigned)more);
        }
    }
}

// out = V c_s per segment (first kfin[s] basis vectors; one CTA per job)
__global__ void lz_combine_kernel(const LzState *__restrict__ st, const double *__restrict__ c,
                                  const int *__restrict__ kfin, int kcap, const KJob *__restrict__ jobs,
                                  double *__restrict__ out)
{
    __shared__ double cs[256];
    const KJob jb = jobs[blockIdx.x];
    const double *V = st->V;
    const long long ldv = st->ldv;
    const int k = kfin[jb.seg];
    for (long long e = jb.b + threadIdx.x; e < jb.e; e += blockDim.x) out[e] = 0.0;
    for (int q0 = 0; q0 < k; q0 += 256) {
        const int kc = min(256, k - q0);
        __syncthreads();
        for (int q = threadIdx.x; q < kc; q += blockDim.x) cs[q] = c[(long long)jb.seg * kcap + q0 + q];
        __syncthreads();
        for (long long e = jb.b + threadIdx.x; e < jb.e; e += blockDim.x) {
            double s = out[e];
            for (int q = 0; q < kc; ++q) s = fma(cs[q], V[(long long)(q0 + q) * ldv + e], s);
            out[e] = s;
        }
    }
}

// V_0 = z / |z_s| (0 for a segment that does not run), xin = V_0
__global__ void lz_begin_kernel(const double *__restrict__ z, const double *__restrict__ zn,
                                const int *__restrict__ cyc, const KJob *__restrict__ jobs, LzState *st,
                                double *__restrict__ xin)
{
    const KJob jb = jobs[blockIdx.x];
    const double a = cyc[jb.seg] ? 1.0 / zn[jb.seg] : 0.0;
    double *V0 = st->V;
    for (long long e = jb.b + threadIdx.x; e < jb.e; e += blockDim.x) {
        const double v = a * z[e];
        V0[e] = v;
        xin[e] = v;
    }
}

// ---------------------------------------------------------------------------
// host side

static std::atomic<bool> g_device_krylov{true};

bool krylov_device_enabled() { return g_device_krylov.load(); }

bool krylov_device_available()
{
    // per device, determined once: 1 available, 2 not
    static std::atomic<int> known[64];
    int dev = 0, coop = 0, nb = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return false;
    if (dev >= 0 && dev < 64)
        if (const int k = known[dev].load()) return k == 1;
    bool ok = cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) == cudaSuccess && coop;
    if (ok && (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, arnoldi_step_kernel, kKdThreads, 0) != cudaSuccess ||
               nb < 1)) {
        cudaGetLastError();
        ok = false;
    }
    if (dev >= 0 && dev < 64) known[dev].store(ok ? 1 : 2);
    return ok;
}

// CTAs the cooperative step kernels may use: as many per SM as both kernels
// keep resident (registers, shared memory), at most 4
static int kd_max_ctas()
{
    // per device, computed once
    static std::atomic<int> cached[64];
    int dev = 0, sms = 1, a = 1, l = 1;
    if (cudaGetDevice(&dev) != cudaSuccess) return 1;
    if (dev >= 0 && dev < 64)
        if (const int c = cached[dev].load()) return c;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, arnoldi_step_kernel, kKdThreads, 0) != cudaSuccess) a = 1;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&l, lanczos_step_kernel, kKdThreads, 0) != cudaSuccess) l = 1;
    cudaGetLastError();
    const int c = sms * std::max(1, std::min(4, std::min(a, l)));
    if (dev >= 0 && dev < 64) cached[dev].store(c);
    return c;
}

KrylovDev::~KrylovDev()
{
    if (base) cudaFreeAsync(base, st);
    if (pinned) {
        cudaStreamSynchronize(st);  // no copy still uses the host block
        pinned_give(pinned);
    }
}

// Copies the job tables to the device through the tail of the engine's pinned
// block (truly asynchronous copies: a copy from pageable memory waits for the
// stream first).
static int kd_upload_jobs(char *hp, const std::vector<KJob> &jb, const std::vector<int> &sj,
                          const std::vector<int> &bj, KJob *jobs, int *sjob, int *bjob, cudaStream_t st)
{
    const size_t b0 = sizeof(KJob) * jb.size(), b1 = sizeof(int) * sj.size(), b2 = sizeof(int) * bj.size();
    if (b0) std::memcpy(hp, jb.data(), b0);
    std::memcpy(hp + b0, sj.data(), b1);
    std::memcpy(hp + b0 + b1, bj.data(), b2);
    if (b0) RMW_CUDA(cudaMemcpyAsync(jobs, hp, b0, cudaMemcpyHostToDevice, st));
    RMW_CUDA(cudaMemcpyAsync(sjob, hp + b0, b1, cudaMemcpyHostToDevice, st));
    RMW_CUDA(cudaMemcpyAsync(bjob, hp + b0 + b1, b2, cudaMemcpyHostToDevice, st));
    return RMW_OK;
}

static size_t kd_jobs_bytes(size_t njobs, size_t nseg, size_t nblk)
{
    return sizeof(KJob) * njobs + sizeof(int) * (nseg + 1) + sizeof(int) * (nblk + 1);
}

int kd_build_jobs(const std::vector<long long> &off, int nblk_max, std::vector<KJob> &jb, std::vector<int> &sj,
                  std::vector<int> &bj)
{
    const int nseg = (int)off.size() - 1;
    const long long n = off.back();
    // at most nblk_max CTAs (the co-resident count), at least kKdThreads elements per CTA
    const int nblk = (int)std::max<long long>(1, std::min<long long>(nblk_max, (n + kKdThreads - 1) / kKdThreads));
    long long per = (n + nblk - 1) / nblk;
    per = ((per + 31) / 32) * 32;
    jb.clear();
    sj.assign(nseg + 1, 0);
    bj.assign(nblk + 1, 0);
    int sg = 0;
    for (int b = 0; b < nblk; ++b) {
        bj[b] = (int)jb.size();
        const long long lo = std::min(n, (long long)b * per), hi = std::min(n, lo + per);
        long long p = lo;
        while (p < hi) {
            while (sg < nseg && off[sg + 1] <= p) ++sg;
            const long long e = std::min(hi, off[sg + 1]);
            jb.push_back({sg, b, p, e});
            p = e;
        }
    }
    bj[nblk] = (int)jb.size();
    // first job of every segment (empty segments own no job: [x, x))
    const int njobs = (int)jb.size();
    int q = 0;
    for (int t = 0; t < nseg; ++t) {
        while (q < njobs && jb[q].seg < t) ++q;
        sj[t] = q;
    }
    sj[nseg] = njobs;
    return nblk;
}

int KrylovDev::init(const std::vector<long long> &seg_off, int restart, int hist_cap, cudaStream_t s)
{
    st = s;
    off = seg_off;
    nseg = (int)off.size() - 1;
    n = off.back();
    R = std::max(1, std::min(restart, kKdMaxBasis - 8));
    KP = R + 2;
    hcap = hist_cap;
    ldv = ((n + 31) / 32) * 32;
    std::vector<KJob> jb;
    std::vector<int> sj, bj;
    nblk = kd_build_jobs(off, kd_max_ctas(), jb, sj, bj);
    njobs = (int)jb.size();
    const size_t nj = (size_t)std::max(1, njobs), ns = (size_t)nseg;
    auto al = [](size_t b) { return (b + 255) / 256 * 256; };
    size_t bytes = al(sizeof(double) * (size_t)ldv * (R + 1)) + 6 * al(sizeof(double) * (size_t)ldv) +
                   al(sizeof(KJob) * nj) + al(sizeof(int) * (ns + 1)) + al(sizeof(int) * (nblk + 1)) +
                   3 * al(sizeof(double) * nj * KP) + al(sizeof(double) * ns * R * (R + 1)) +
                   2 * al(sizeof(double) * ns * R) + al(sizeof(double) * ns * (R + 1)) +
                   2 * al(sizeof(double) * ns * KP) + 4 * al(sizeof(double) * ns) + al(sizeof(double) * ns * KP) +
                   al(sizeof(double) * ns * std::max(1, hcap)) + 4 * al(sizeof(int) * ns) + al(sizeof(KState));
    RMW_CUDA(rmw::dmalloc_async(&base, bytes, st));
    char *p = (char *)base;
    auto take = [&](size_t b) {
        char *q = p;
        p += al(b);
        return (void *)q;
    };
    V = (double *)take(sizeof(double) * (size_t)ldv * (R + 1));
    w = (double *)take(sizeof(double) * ldv);
    xin = (double *)take(sizeof(double) * ldv);
    x = (double *)take(sizeof(double) * ldv);
    r = (double *)take(sizeof(double) * ldv);
    t1 = (double *)take(sizeof(double) * ldv);
    t2 = (double *)take(sizeof(double) * ldv);
    jobs = (KJob *)take(sizeof(KJob) * nj);
    sjob = (int *)take(sizeof(int) * (ns + 1));
    bjob = (int *)take(sizeof(int) * (nblk + 1));
    partA = (double *)take(sizeof(double) * nj * KP);
    partB = (double *)take(sizeof(double) * nj * KP);
    partC = (double *)take(sizeof(double) * nj * KP);
    H = (double *)take(sizeof(double) * ns * R * (R + 1));
    cs = (double *)take(sizeof(double) * ns * R);
    sn = (double *)take(sizeof(double) * ns * R);
    g = (double *)take(sizeof(double) * ns * (R + 1));
    hc1 = (double *)take(sizeof(double) * ns * KP);
    hc2 = (double *)take(sizeof(double) * ns * KP);
    tol_abs = (double *)take(sizeof(double) * ns);
    alpha = (double *)take(sizeof(double) * ns);
    nrm = (double *)take(sizeof(double) * ns);
    gres = (double *)take(sizeof(double) * ns);
    y = (double *)take(sizeof(double) * ns * KP);
    hist = (double *)take(sizeof(double) * ns * std::max(1, hcap));
    // iters, jdone, cyc and flags back to back (one copy reads all four)
    iters = (int *)take(sizeof(int) * 4 * ns);
    jdone = iters + ns;
    cyc = iters + 2 * ns;
    flags = iters + 3 * ns;
    state = (KState *)take(sizeof(KState));
    // pinned host scalars: alpha, beta, cycle flags, tolerances (ns doubles each), maxiter, the loop
    // flag, the state, and four ns-int arrays (iters, jdone, cyc, flags) from 4 ns + 2 + 4 doubles on;
    // then the job tables on their way to the device
    const size_t scal = sizeof(double) * (8 * ns + 16);
    void *hp = nullptr;
    if (int rc = pinned_take(scal + kd_jobs_bytes(jb.size(), ns, nblk), &hp)) return rc;
    pinned = (double *)hp;
    if (int rc = kd_upload_jobs((char *)hp + scal, jb, sj, bj, jobs, sjob, bjob, st)) return rc;
    RMW_CUDA(cudaMemsetAsync(V, 0, sizeof(double) * (size_t)ldv * (R + 1), st));
    RMW_CUDA(cudaMemsetAsync(w, 0, sizeof(double) * 6 * (size_t)ldv, st));
    RMW_CUDA(cudaMemsetAsync(iters, 0, sizeof(int) * ns, st));
    RMW_CUDA(cudaMemsetAsync(flags, 0, sizeof(int) * ns, st));
    RMW_CUDA(cudaMemsetAsync(state, 0, sizeof(KState), st));
    return RMW_OK;
}

// ---- Lanczos buffers ------------------------------------------------------
LanczosDev::~LanczosDev()
{
    if (V) cudaFreeAsync(V, st);
    if (base) cudaFreeAsync(base, st);
    if (pinned) {
        cudaStreamSynchronize(st);  // no copy still uses the host block
        pinned_give(pinned);
    }
}

int LanczosDev::init(const std::vector<long long> &seg_off, int kcap_, cudaStream_t s)
{
    st = s;
    nseg = (int)seg_off.size() - 1;
    n = seg_off.back();
    kcap = std::max(2, kcap_);
    KP = kcap + 2;
    ldv = ((n + 31) / 32) * 32;
    std::vector<KJob> jb;
    std::vector<int> sj, bj;
    nblk = kd_build_jobs(seg_off, kd_max_ctas(), jb, sj, bj);
    njobs = (int)jb.size();
    const size_t nj = (size_t)std::max(1, njobs), ns = (size_t)nseg, kc = (size_t)kcap;
    auto al = [](size_t b) { return (b + 255) / 256 * 256; };
    const size_t bytes = 2 * al(sizeof(double) * ldv) + al(sizeof(KJob) * nj) + al(sizeof(int) * (ns + 1)) +
                         al(sizeof(int) * (nblk + 1)) + 3 * al(sizeof(double) * nj * KP) + al(sizeof(double) * ns) +
                         6 * al(sizeof(double) * ns * kc) + al(sizeof(double) * ns * kc * kc) +
                         4 * al(sizeof(int) * ns) + al(sizeof(LzState));
    RMW_CUDA(rmw::dmalloc_async(&base, bytes, st));
    char *p = (char *)base;
    auto take = [&](size_t b) {
        char *q = p;
        p += al(b);
        return (void *)q;
    };
    w = (double *)take(sizeof(double) * ldv);
    xin = (double *)take(sizeof(double) * ldv);
    jobs = (KJob *)take(sizeof(KJob) * nj);
    sjob = (int *)take(sizeof(int) * (ns + 1));
    bjob = (int *)take(sizeof(int) * (nblk + 1));
    partA = (double *)take(sizeof(double) * nj * KP);
    partB = (double *)take(sizeof(double) * nj * KP);
    partC = (double *)take(sizeof(double) * nj * KP);
    zn = (double *)take(sizeof(double) * ns);
    hd = (double *)take(sizeof(double) * ns * kc);
    hs = (double *)take(sizeof(double) * ns * kc);
    c = (double *)take(sizeof(double) * ns * kc);
    cold = (double *)take(sizeof(double) * ns * kc);
    dt = (double *)take(sizeof(double) * ns * kc);
    et = (double *)take(sizeof(double) * ns * kc);
    z = (double *)take(sizeof(double) * ns * kc * kc);
    iters = (int *)take(sizeof(int) * ns);
    cyc = (int *)take(sizeof(int) * ns);
    kfin = (int *)take(sizeof(int) * ns);
    flags = (int *)take(sizeof(int) * ns);
    state = (LzState *)take(sizeof(LzState));
    // pinned host scalars (2 ns + 16 doubles, four ns-int arrays, the state), then the job tables
    const size_t scal = sizeof(double) * (2 * ns + 16) + sizeof(int) * 4 * ns + sizeof(LzState);
    const size_t scal_al = (scal + 15) / 16 * 16;
    if (int rc = pinned_take(scal_al + kd_jobs_bytes(jb.size(), ns, nblk), &pinned)) return rc;
    if (int rc = kd_upload_jobs((char *)pinned + scal_al, jb, sj, bj, jobs, sjob, bjob, st)) return rc;
    RMW_CUDA(cudaMemsetAsync(w, 0, sizeof(double) * 2 * ldv, st));
    RMW_CUDA(cudaMemsetAsync(state, 0, sizeof(LzState), st));
    RMW_CUDA(cudaMemsetAsync(flags, 0, sizeof(int) * ns, st));
    RMW_CUDA(cudaMemsetAsync(c, 0, sizeof(double) * ns * kc, st));
    return grow(std::min(kcap + 1, 32));
}

int LanczosDev::grow(int want)
{
    want = std::min(want, kcap + 1);
    if (want <= vcap) return RMW_OK;
    double *nv = nullptr;
    RMW_CUDA(rmw::dmalloc_async(&nv, sizeof(double) * (size_t)ldv * want, st));
    if (V) {
        RMW_CUDA(cudaMemcpyAsync(nv, V, sizeof(double) * (size_t)ldv * vcap, cudaMemcpyDeviceToDevice, st));
        RMW_CUDA(cudaFreeAsync(V, st));
    }
    V = nv;
    vcap = want;
    // the step kernels read the basis pointer and its room from the state
    LzState *h = (LzState *)((char *)pinned + sizeof(double) * (2 * nseg + 16) + sizeof(int) * 4 * nseg);
    RMW_CUDA(cudaMemcpyAsync(h, state, sizeof(LzState), cudaMemcpyDeviceToHost, st));
    RMW_CUDA(cudaStreamSynchronize(st));
    h->V = V;
    h->vcap = vcap;
    h->ldv = ldv;
    RMW_CUDA(cudaMemcpyAsync(state, h, sizeof(LzState), cudaMemcpyHostToDevice, st));
    RMW_CUDA(cudaStreamSynchronize(st));
    return RMW_OK;
}

__global__ void lz_init_kernel(const double *__restrict__ nrm, int nseg, double factor, int max_iter,
                               double *__restrict__ zn, int *__restrict__ cyc, int *__restrict__ iters,
                               int *__restrict__ kfin, LzState *st)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < nseg) {
        const double z = sqrt(nrm[s]);
        zn[s] = z;
        const int on = (z > 0.0 && isfinite(z) && factor != 0.0) ? 1 : 0;
        cyc[s] = on;
        iters[s] = on ? max_iter : 0;
        kfin[s] = 0;
    }
    if (s == 0) {
        st->i = 0;
        st->active = 0;
        st->more = 1;
        st->live = 0;
        st->max_iter = max_iter;
        st->dev_k = kLzDeviceRows;
        st->host = 0;
        st->bar.done = 0;
    }
}

int lz_begin(LanczosDev &L, const double *z, double factor, int max_iter, std::vector<double> &zn_host,
             std::vector<int> &run)
{
    const int ns = L.nseg;
    if (L.njobs) {
        seg_norm_partial_kernel<<<L.njobs, 512, 0, L.st>>>(z, L.jobs, L.partC);
        seg_norm_reduce_kernel<<<(ns * 32 + 255) / 256, 256, 0, L.st>>>(L.partC, L.sjob, ns, L.partA);
    } else {
        RMW_CUDA(cudaMemsetAsync(L.partA, 0, sizeof(double) * ns, L.st));
    }
    lz_init_kernel<<<(ns + 127) / 128, 128, 0, L.st>>>(L.partA, ns, factor, max_iter, L.zn, L.cyc, L.iters, L.kfin,
                                                       L.state);
    if (L.njobs) lz_begin_kernel<<<L.njobs, 512, 0, L.st>>>(z, L.zn, L.cyc, L.jobs, L.state, L.xin);
    RMW_CHECK_LAUNCH("Lanczos start");
    double *h = (double *)L.pinned;
    int *hi = (int *)((char *)L.pinned + sizeof(double) * (2 * ns + 16));
    RMW_CUDA(cudaMemcpyAsync(h, L.zn, sizeof(double) * ns, cudaMemcpyDeviceToHost, L.st));
    RMW_CUDA(cudaMemcpyAsync(hi, L.cyc, sizeof(int) * ns, cudaMemcpyDeviceToHost, L.st));
    RMW_CUDA(cudaStreamSynchronize(L.st));
    zn_host.assign(h, h + ns);
    run.assign(hi, hi + ns);
    return RMW_OK;
}

int lz_step(LanczosDev &L, double factor, double tol, const LzMask &mk, unsigned long long cond, int use_cond,
            cudaStream_t st)
{
    LzArgs A;
    A.w = L.w;
    A.xin = L.xin;
    A.jobs = L.jobs;
    A.sjob = L.sjob;
    A.bjob = L.bjob;
    A.partA = L.partA;
    A.partB = L.partB;
    A.partC = L.partC;
    A.KP = L.KP;
    A.kcap = L.kcap;
    A.hd = L.hd;
    A.hs = L.hs;
    A.c = L.c;
    A.cold = L.cold;
    A.dt = L.dt;
    A.et = L.et;
    A.z = L.z;
    A.zn = L.zn;
    A.factor = factor;
    A.tol = tol;
    A.iters = L.iters;
    A.cyc = L.cyc;
    A.kfin = L.kfin;
    A.flags = L.flags;
    A.st = L.state;
    A.mask = mk.mask;
    A.nsusp = mk.nsusp;
    A.nrhs = mk.nrhs;
    A.pass = mk.pass;
    A.cond = cond;
    A.use_cond = use_cond;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)L.nblk);
    cfg.blockDim = dim3(kKdThreads);
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    RMW_CUDA(cudaLaunchKernelEx(&cfg, lanczos_step_kernel, A));
    return RMW_OK;
}

int lz_fetch_state(LanczosDev &L, LzState *host)
{
    LzState *h = (LzState *)((char *)L.pinned + sizeof(double) * (2 * L.nseg + 16) + sizeof(int) * 4 * L.nseg);
    RMW_CUDA(cudaMemcpyAsync(h, L.state, sizeof(LzState), cudaMemcpyDeviceToHost, L.st));
    RMW_CUDA(cudaStreamSynchronize(L.st));
    *host = *h;
    return RMW_OK;
}

int lz_finish(LanczosDev &L, double *noise, std::vector<int> &iters)
{
    const int ns = L.nseg;
    int *hi = (int *)((char *)L.pinned + sizeof(double) * (2 * ns + 16));
    RMW_CUDA(cudaMemcpyAsync(hi, L.flags, sizeof(int) * ns, cudaMemcpyDeviceToHost, L.st));
    RMW_CUDA(cudaStreamSynchronize(L.st));
    for (int s = 0; s < ns; ++s) {
        if (hi[s] & 2) return fail(RMW_ERR_BREAKDOWN, "Lanczos: non-finite value");
        if (hi[s] & 4) return fail(RMW_ERR_BREAKDOWN, "Lanczos: tridiagonal eigensolver failed");
    }
    if (L.njobs) lz_combine_kernel<<<L.njobs, 512, 0, L.st>>>(L.state, L.c, L.kfin, L.kcap, L.jobs, noise);
    RMW_CHECK_LAUNCH("Lanczos noise");
    RMW_CUDA(cudaMemcpyAsync(hi, L.iters, sizeof(int) * ns, cudaMemcpyDeviceToHost, L.st));
    RMW_CUDA(cudaStreamSynchronize(L.st));
    iters.assign(hi, hi + ns);
    return RMW_OK;
}

int kd_seg_norm2(KrylovDev &K, const double *v)
{
    if (K.njobs == 0) {
        RMW_CUDA(cudaMemsetAsync(K.nrm, 0, sizeof(double) * K.nseg, K.st));
        return RMW_OK;
    }
    seg_norm_partial_kernel<<<K.njobs, 512, 0, K.st>>>(v, K.jobs, K.partC);
    seg_norm_reduce_kernel<<<(K.nseg * 32 + 255) / 256, 256, 0, K.st>>>(K.partC, K.sjob, K.nseg, K.nrm);
    RMW_CHECK_LAUNCH("segment norms");
    return RMW_OK;
}

int kd_cycle_begin(KrylovDev &K, const std::vector<double> &alpha, const std::vector<double> &beta,
                   const std::vector<int> &cyc, int)
{
    const int ns = K.nseg;
    double *h = K.pinned;
    for (int s = 0; s < ns; ++s) {
        h[s] = alpha[s];
        h[ns + s] = beta[s];
        h[2 * ns + s] = cyc[s] ? 1.0 : 0.0;
    }
    // alpha, then beta and the flags in the two arrays after it (y is free here)
    RMW_CUDA(cudaMemcpyAsync(K.alpha, h, sizeof(double) * ns, cudaMemcpyHostToDevice, K.st));
    RMW_CUDA(cudaMemcpyAsync(K.y, h + ns, sizeof(double) * 2 * ns, cudaMemcpyHostToDevice, K.st));
    if (K.njobs) cycle_begin_kernel<<<K.njobs, 512, 0, K.st>>>(K.r, K.V, K.xin, K.jobs, K.alpha);
    cycle_state_kernel<<<(ns + 127) / 128, 128, 0, K.st>>>(K.y, K.y + ns, ns, K.R, K.g, K.cyc, K.jdone, K.state);
    RMW_CHECK_LAUNCH("cycle begin");
    return RMW_OK;
}

int kd_arnoldi_step(KrylovDev &K, unsigned long long cond, int use_cond, cudaStream_t st)
{
    StepArgs A;
    A.V = K.V;
    A.ldv = K.ldv;
    A.w = K.w;
    A.xin = K.xin;
    A.jobs = K.jobs;
    A.sjob = K.sjob;
    A.bjob = K.bjob;
    A.partA = K.partA;
    A.partB = K.partB;
    A.partC = K.partC;
    A.KP = K.KP;
    A.R = K.R;
    A.hcap = K.hcap;
    A.H = K.H;
    A.cs = K.cs;
    A.sn = K.sn;
    A.g = K.g;
    A.hc1 = K.hc1;
    A.hc2 = K.hc2;
    A.hist = K.hcap > 0 ? K.hist : nullptr;
    A.gres = K.gres;
    A.tol_abs = K.tol_abs;
    A.iters = K.iters;
    A.jdone = K.jdone;
    A.cyc = K.cyc;
    A.flags = K.flags;
    A.st = K.state;
    A.cond = cond;
    A.use_cond = use_cond;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)K.nblk);
    cfg.blockDim = dim3(kKdThreads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    RMW_CUDA(cudaLaunchKernelEx(&cfg, arnoldi_step_kernel, A));
    return RMW_OK;
}

int kd_cycle_solution(KrylovDev &K, int kmax)
{
    backsub_kernel<<<(K.nseg + 63) / 64, 64, 0, K.st>>>(K.H, K.g, K.jdone, K.nseg, K.R, K.KP, K.y);
    if (K.njobs) seg_combine_kernel_dev<<<K.njobs, 512, 0, K.st>>>(K.V, K.ldv, kmax, K.y, K.KP, K.jobs, K.t1);
    RMW_CHECK_LAUNCH("cycle solution");
    return RMW_OK;
}

int kd_axpby(KrylovDev &K, const double *x, double *y, double a, double b)
{
    kd_axpby_kernel<<<(unsigned)((K.n + 255) / 256), 256, 0, K.st>>>(x, y, K.n, a, b);
    RMW_CHECK_LAUNCH("axpby");
    return RMW_OK;
}

int kd_build_cycle_graph(cudaGraph_t *graph_out, cudaGraph_t *body_out, unsigned long long *cond_out)
{
    static_assert(sizeof(cudaGraphConditionalHandle) <= sizeof(unsigned long long), "handle size");
    cudaGraph_t g = nullptr;
    RMW_CUDA(cudaGraphCreate(&g, 0));
    cudaGraphConditionalHandle h;
    if (cudaError_t e = cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault)) {
        cudaGraphDestroy(g);
        return cuda_fail(e, "cudaGraphConditionalHandleCreate");
    }
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t node;
    if (cudaError_t e = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &cp)) {
        cudaGraphDestroy(g);
        return cuda_fail(e, "cudaGraphAddNode (while)");
    }
    *graph_out = g;
    *body_out = cp.conditional.phGraph_out[0];
    *cond_out = (unsigned long long)h;
    return RMW_OK;
}

int kd_set_solve_params(KrylovDev &K, const std::vector<double> &tol_abs, int maxiter)
{
    const int ns = K.nseg;
    double *h = K.pinned + 3 * ns;
    for (int s = 0; s < ns; ++s) h[s] = tol_abs[s];
    RMW_CUDA(cudaMemcpyAsync(K.tol_abs, h, sizeof(double) * ns, cudaMemcpyHostToDevice, K.st));
    int *mi = (int *)(K.pinned + 4 * ns);
    *mi = maxiter;
    RMW_CUDA(cudaMemcpyAsync(&K.state->maxiter, mi, sizeof(int), cudaMemcpyHostToDevice, K.st));
    RMW_CUDA(cudaMemsetAsync(K.iters, 0, sizeof(int) * ns, K.st));
    RMW_CUDA(cudaMemsetAsync(K.flags, 0, sizeof(int) * ns, K.st));
    RMW_CUDA(cudaMemsetAsync(K.hist, 0, sizeof(double) * ns * std::max(1, K.hcap), K.st));
    return RMW_OK;
}

int kd_fetch_cycle(KrylovDev &K, KState *state_host, int *ints_host)
{
    // iters, jdone, cyc and flags are four consecutive ns-int arrays
    char *h = (char *)(K.pinned + 4 * K.nseg + 2);
    RMW_CUDA(cudaMemcpyAsync(h, K.state, sizeof(KState), cudaMemcpyDeviceToHost, K.st));
    RMW_CUDA(cudaMemcpyAsync(ints_host, K.iters, sizeof(int) * 4 * K.nseg, cudaMemcpyDeviceToHost, K.st));
    RMW_CUDA(cudaStreamSynchronize(K.st));
    std::memcpy(state_host, h, sizeof(KState));
    return RMW_OK;
}

int kd_fetch_norms(KrylovDev &K, double *host)
{
    RMW_CUDA(cudaMemcpyAsync(host, K.nrm, sizeof(double) * K.nseg, cudaMemcpyDeviceToHost, K.st));
    RMW_CUDA(cudaStreamSynchronize(K.st));
    return RMW_OK;
}

int kd_fetch_more(KrylovDev &K, int *more)
{
    int *h = (int *)(K.pinned + 4 * K.nseg + 1);
    RMW_CUDA(cudaMemcpyAsync(h, &K.state->more, sizeof(int), cudaMemcpyDeviceToHost, K.st));
    RMW_CUDA(cudaStreamSynchronize(K.st));
    *more = *h;
    return RMW_OK;
}

}  // namespace rmw

extern "C" int rmw_use_device_krylov(int on)
{
    rmw::g_device_krylov.store(on != 0);
    return RMW_OK;
}
