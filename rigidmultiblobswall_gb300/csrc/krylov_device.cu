// Kernels and buffers of the device-resident GMRES engine (krylov_device.cuh).
#include <atomic>
#include <cstring>

#include "krylov_device.cuh"

namespace rmw {

// spins of a grid barrier before it gives up (about 0.3 s with the 64 ns sleeps)
constexpr unsigned kBarrierSpins = 1u << 22;

// ---------------------------------------------------------------------------
// device helpers

__device__ __forceinline__ double warp_sum(double v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Grid barrier of a cooperative launch: generation counter, bounded spin.
__device__ void grid_barrier(KState *st)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned *vgen = &st->bar_gen;
        const unsigned gen = *vgen;
        __threadfence();
        const unsigned arrived = atomicAdd(&st->bar_count, 1u);
        if (arrived == gridDim.x - 1) {
            atomicExch(&st->bar_count, 0u);
            __threadfence();
            atomicAdd(&st->bar_gen, 1u);
        } else {
            unsigned spins = 0;
            while (*vgen == gen) {
                if (++spins > kBarrierSpins) {
                    atomicExch(&st->err, 1);
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

// part[job * KP + q] = sum_{i in job} V_q[i] w[i], q < k (red: k x 32 shared doubles)
__device__ void job_dots(const double *__restrict__ V, long long ldv, int k, const double *w, const KJob jb,
                         double *part, int KP, int job, double *red)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int q0 = 0; q0 < k; q0 += 2) {
        const bool two = q0 + 1 < k;
        const double *V0 = V + (long long)q0 * ldv;
        const double *V1 = V0 + ldv;
        double a0 = 0.0, a1 = 0.0;
        for (long long i = jb.b + threadIdx.x; i < jb.e; i += blockDim.x) {
            const double wi = w[i];
            a0 = fma(V0[i], wi, a0);
            if (two) a1 = fma(V1[i], wi, a1);
        }
        a0 = warp_sum(a0);
        a1 = warp_sum(a1);
        if (lane == 0) {
            red[q0 * 32 + wid] = a0;
            if (two) red[(q0 + 1) * 32 + wid] = a1;
        }
    }
    __syncthreads();
    for (int q = threadIdx.x; q < k; q += blockDim.x) {
        double s = 0.0;
        for (int u = 0; u < nw; ++u) s += red[q * 32 + u];
        part[(long long)job * KP + q] = s;
    }
    __syncthreads();
}

// w[i] -= sum_q hs[q] V_q[i] over the job; returns this thread's sum of the new w[i]^2
__device__ double job_update(const double *__restrict__ V, long long ldv, int k, const double *hs, double *w,
                             const KJob jb)
{
    double nrm = 0.0;
    for (long long i = jb.b + threadIdx.x; i < jb.e; i += blockDim.x) {
        double x = w[i];
        for (int q = 0; q < k; ++q) x = fma(-hs[q], V[(long long)q * ldv + i], x);
        w[i] = x;
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
    double *H, *cs, *sn, *g, *hc1, *hc2, *hist;
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
    grid_barrier(A.st);
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
    grid_barrier(A.st);
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
    grid_barrier(A.st);
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
        if (job == A.sjob[jb.seg] && threadIdx.x == 0 && A.cyc[jb.seg]) {
            const int s = jb.seg, R = A.R;
            double *h = A.H + ((long long)s * R + j) * (R + 1);
            double *c = A.cs + (long long)s * R, *sv = A.sn + (long long)s * R, *gs = A.g + (long long)s * (R + 1);
            for (int q = 0; q <= j; ++q) h[q] = A.hc1[(long long)s * A.KP + q] + A.hc2[(long long)s * A.KP + q];
            const double hn = sqrt(nw);
            h[j + 1] = hn;
            int stop = 0;
            if (!isfinite(hn)) {
                A.flags[s] |= 2;  // non-finite Arnoldi vector
                stop = 1;
            } else {
                for (int q = 0; q < j; ++q) {
                    const double t = c[q] * h[q] + sv[q] * h[q + 1];
                    h[q + 1] = -sv[q] * h[q] + c[q] * h[q + 1];
                    h[q] = t;
                }
                const double den = hypot(h[j], h[j + 1]);
                c[j] = (den == 0.0) ? 1.0 : h[j] / den;
                sv[j] = (den == 0.0) ? 0.0 : h[j + 1] / den;
                h[j] = c[j] * h[j] + sv[j] * h[j + 1];
                h[j + 1] = 0.0;
                gs[j + 1] = -sv[j] * gs[j];
                gs[j] = c[j] * gs[j];
                const int it = ++A.iters[s];
                A.jdone[s] = j + 1;
                const double res = fabs(gs[j + 1]);
                if (A.hist && it <= A.hcap) A.hist[(long long)s * A.hcap + it - 1] = res;
                const bool conv = res <= A.tol_abs[s];
                if (hn == 0.0 && !conv) A.flags[s] |= 1;  // breakdown without convergence
                stop = conv || hn == 0.0 || it >= A.st->maxiter;
            }
            if (stop) A.cyc[s] = 0;
            else atomicAdd(&A.st->active, 1);
        }
        __syncthreads();
    }
    // the last CTA to finish advances the step and sets the loop condition
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned prev = atomicAdd(&A.st->done, 1u);
        if (prev == gridDim.x - 1) {
            __threadfence();
            const int act = atomicAdd(&A.st->active, 0);
            const int jn = j + 1;
            const int more = (act > 0 && jn < A.R && !*(volatile int *)&A.st->err) ? 1 : 0;
            A.st->j = jn;
            A.st->active = 0;
            A.st->more = more;
            atomicExch(&A.st->done, 0u);
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
        st->done = 0;
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
// host side

static std::atomic<bool> g_device_krylov{true};

bool krylov_device_enabled() { return g_device_krylov.load(); }

bool krylov_device_available()
{
    int dev = 0, coop = 0, nb = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return false;
    if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess || !coop) return false;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, arnoldi_step_kernel, kKdThreads, 0) != cudaSuccess ||
        nb < 1) {
        cudaGetLastError();
        return false;
    }
    return true;
}

KrylovDev::~KrylovDev()
{
    if (base) cudaFreeAsync(base, st);
    if (pinned) {
        cudaStreamSynchronize(st);
        cudaFreeHost(pinned);
    }
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
    int dev = 0, sms = 1;
    RMW_CUDA(cudaGetDevice(&dev));
    RMW_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    // one CTA per SM at most, at least 1024 elements per CTA
    nblk = (int)std::max<long long>(1, std::min<long long>(sms, (n + kKdThreads - 1) / kKdThreads));
    long long per = (n + nblk - 1) / nblk;
    per = ((per + 31) / 32) * 32;
    // jobs: intersections of CTA ranges with segments (both in element order)
    std::vector<KJob> jb;
    std::vector<int> sj(nseg + 1, 0), bj(nblk + 1, 0);
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
    njobs = (int)jb.size();
    // first job of every segment (empty segments own no job: [x, x))
    {
        int q = 0;
        for (int t = 0; t < nseg; ++t) {
            while (q < njobs && jb[q].seg < t) ++q;
            sj[t] = q;
        }
        sj[nseg] = njobs;
    }
    const size_t nj = (size_t)std::max(1, njobs), ns = (size_t)nseg;
    auto al = [](size_t b) { return (b + 255) / 256 * 256; };
    size_t bytes = al(sizeof(double) * (size_t)ldv * (R + 1)) + 6 * al(sizeof(double) * (size_t)ldv) +
                   al(sizeof(KJob) * nj) + al(sizeof(int) * (ns + 1)) + al(sizeof(int) * (nblk + 1)) +
                   3 * al(sizeof(double) * nj * KP) + al(sizeof(double) * ns * R * (R + 1)) +
                   2 * al(sizeof(double) * ns * R) + al(sizeof(double) * ns * (R + 1)) +
                   2 * al(sizeof(double) * ns * KP) + 3 * al(sizeof(double) * ns) + al(sizeof(double) * ns * KP) +
                   al(sizeof(double) * ns * std::max(1, hcap)) + 4 * al(sizeof(int) * ns) + al(sizeof(KState));
    RMW_CUDA(cudaMallocAsync(&base, bytes, st));
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
    y = (double *)take(sizeof(double) * ns * KP);
    hist = (double *)take(sizeof(double) * ns * std::max(1, hcap));
    iters = (int *)take(sizeof(int) * ns);
    jdone = (int *)take(sizeof(int) * ns);
    cyc = (int *)take(sizeof(int) * ns);
    flags = (int *)take(sizeof(int) * ns);
    state = (KState *)take(sizeof(KState));
    if (njobs) RMW_CUDA(cudaMemcpyAsync(jobs, jb.data(), sizeof(KJob) * njobs, cudaMemcpyHostToDevice, st));
    RMW_CUDA(cudaMemcpyAsync(sjob, sj.data(), sizeof(int) * (ns + 1), cudaMemcpyHostToDevice, st));
    RMW_CUDA(cudaMemcpyAsync(bjob, bj.data(), sizeof(int) * (nblk + 1), cudaMemcpyHostToDevice, st));
    RMW_CUDA(cudaMemsetAsync(V, 0, sizeof(double) * (size_t)ldv * (R + 1), st));
    RMW_CUDA(cudaMemsetAsync(w, 0, sizeof(double) * 6 * (size_t)ldv, st));
    RMW_CUDA(cudaMemsetAsync(iters, 0, sizeof(int) * ns, st));
    RMW_CUDA(cudaMemsetAsync(flags, 0, sizeof(int) * ns, st));
    RMW_CUDA(cudaMemsetAsync(state, 0, sizeof(KState), st));
    // pinned host scalars: alpha, beta, cycle flags, tolerances (ns doubles each), maxiter, the loop
    // flag, the state, and four ns-int arrays (iters, jdone, cyc, flags) from 4 ns + 2 + 4 doubles on
    RMW_CUDA(cudaHostAlloc(&pinned, sizeof(double) * (8 * ns + 16), cudaHostAllocDefault));
    // the copies above read host vectors that go out of scope
    RMW_CUDA(cudaStreamSynchronize(st));
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
