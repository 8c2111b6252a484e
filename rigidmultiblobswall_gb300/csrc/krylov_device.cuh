// Device-resident restarted GMRES over one or many independent segments.
//
// The algorithm is the right-preconditioned restarted GMRES of
// general_application_utils.py:514-635 (scipy's gmres with restart m, zero
// initial guess, relative tolerance on the residual 2-norm), run for every
// segment of the Krylov vectors at once - one segment for a single
// suspension, one per suspension for batched suspensions - each with its own
// Hessenberg matrix, Givens rotations, tolerance and iteration count.
//
// One Arnoldi step is two launches: the operator y = A P^-1 v (the caller's
// kernels) and arnoldi_step_kernel, a persistent cooperative kernel (as many
// CTAs as stay co-resident, up to 4 per SM) that does the whole classical
// Gram-Schmidt step with one
// reorthogonalisation (CGS2: two dot passes, two update passes, the norm and
// the scaling of the next basis vector, separated by grid barriers), applies
// the previous Givens rotations to the new Hessenberg column, forms the next
// rotation, updates the residual estimate and decides whether the cycle goes
// on.  Nothing returns to the host during a restart cycle: the operator and
// the step kernel are captured once into a CUDA graph whose while node
// repeats them until the step kernel clears the loop condition.  The host
// reads the state once per restart cycle (true residual and stopping test).
//
// Reductions are deterministic: every CTA reduces the per-job partial sums of
// its segments in the same fixed order, so all CTAs hold bit-identical
// coefficients without atomics.  Grid barriers spin on a generation counter
// with an iteration limit: a barrier that runs out (it cannot happen under a
// cooperative launch, which guarantees co-residency) sets an error flag that
// the host turns into RMW_ERR_CUDA after the cycle.
#pragma once
#include <algorithm>
#include <cmath>
#include <vector>

#include "rmw_common.cuh"

namespace rmw {

// threads of the fused step CTAs: the vector work is FP64-pipe bound on
// GB300 (two flops per 8-byte element against a 1:64 FP64 rate), so each
// thread takes several elements and the per-thread FP64 reduction overhead
// (warp trees per basis vector) stays small against the multiply-adds
constexpr int kKdThreads = 256;
constexpr int kKdMaxBasis = 128;  // basis vectors a step handles (restart <= 120)

// contiguous piece [b, e) of segment `seg`, processed by CTA `blk`
struct KJob {
    int seg, blk;
    long long b, e;
};

// grid barrier and last-CTA detection of one cooperative step kernel
struct GridBar {
    unsigned done;  // CTAs finished with the step (last-CTA detection)
    unsigned count;
    unsigned gen;
    int err;  // a grid barrier gave up waiting
};

// solver scalars shared by the GMRES step kernels of one solve
struct KState {
    GridBar bar;
    int j;        // Arnoldi step within the cycle
    int active;   // segments still iterating after the step (last CTA reads it)
    int more;     // the loop condition the last step set
    int maxiter;  // iteration limit per segment (the solve's)
};

// scalars of the Lanczos step kernels of one call
struct LzState {
    GridBar bar;
    int i;         // iteration
    int active;    // segments still iterating after the step (counted by the owners)
    int more;      // loop condition
    int live;      // segments still iterating after the last step
    int max_iter;  // the reference's max_iter
    int vcap;      // basis vectors V has room for
    int dev_k;     // the device checks convergence while i < dev_k; beyond, the host does
    int host;      // 1: the host checks convergence (the kernel only records the recurrence)
    long long ldv;
    double *V;     // the basis (grown by the host between graph launches)
};

// Tridiagonal matrices larger than this are diagonalised on the host: the
// implicit QL recurrence is a long chain of dependent FP64 operations, which
// GB300's FP64 pipe (1:64 of FP32) runs slower than a host core once the
// matrix has a dozen rows.
constexpr int kLzDeviceRows = 10;
bool tridiag_eigen_host(std::vector<double> &d, std::vector<double> e, std::vector<double> &z);

// Job table: CTA b of at most nblk_max CTAs gets a contiguous range of the n
// elements (a multiple of 32 long); jobs are the intersections of those ranges
// with the segments [off[s], off[s+1]).  Returns the CTA count.
int kd_build_jobs(const std::vector<long long> &off, int nblk_max, std::vector<KJob> &jobs, std::vector<int> &sjob,
                  std::vector<int> &bjob);

// device buffers and job tables of one device GMRES engine
struct KrylovDev {
    int nseg = 0, njobs = 0, nblk = 0, R = 0, KP = 0, hcap = 0;
    long long n = 0, ldv = 0;
    cudaStream_t st = 0;
    void *base = nullptr;
    double *pinned = nullptr;  // host mirror of the per-cycle scalars
    // vectors
    double *V = nullptr, *w = nullptr, *xin = nullptr, *x = nullptr, *r = nullptr, *t1 = nullptr, *t2 = nullptr;
    // jobs
    KJob *jobs = nullptr;
    int *sjob = nullptr;  // nseg + 1: jobs of segment s are [sjob[s], sjob[s+1])
    int *bjob = nullptr;  // nblk + 1: jobs of CTA b are [bjob[b], bjob[b+1])
    // partial sums
    double *partA = nullptr, *partB = nullptr, *partC = nullptr;
    // per-segment state
    double *H = nullptr, *cs = nullptr, *sn = nullptr, *g = nullptr, *hc1 = nullptr, *hc2 = nullptr;
    double *tol_abs = nullptr, *alpha = nullptr, *y = nullptr, *nrm = nullptr, *hist = nullptr;
    double *gres = nullptr;  // last residual estimate |g_{j+1}| per segment
    int *iters = nullptr, *jdone = nullptr, *cyc = nullptr, *flags = nullptr;
    KState *state = nullptr;
    // host copies of the job layout
    std::vector<long long> off;

    ~KrylovDev();
    int init(const std::vector<long long> &seg_off, int restart, int hist_cap, cudaStream_t s);
};

// true when this device can run the cooperative step kernel
bool krylov_device_available();
// library switch (rmw_use_device_krylov): device-resident cycles (1) or the
// host-driven Arnoldi loop (0)
bool krylov_device_enabled();

// per-segment |v|^2 into K.nrm (device)
int kd_seg_norm2(KrylovDev &K, const double *v);
// tolerances |b_s| tol_s, the iteration limit; clears the counters and flags
int kd_set_solve_params(KrylovDev &K, const std::vector<double> &tol_abs, int maxiter);
// start of a cycle: V_0 = alpha_s r, xin = V_0, g = (beta_s, 0, ...), cycle flags, step 0
int kd_cycle_begin(KrylovDev &K, const std::vector<double> &alpha, const std::vector<double> &beta,
                   const std::vector<int> &cyc, int unused = 0);
// one fused CGS2 + Givens step; use_cond != 0 sets the graph's loop condition `cond`
int kd_arnoldi_step(KrylovDev &K, unsigned long long cond, int use_cond, cudaStream_t st);
// end of a cycle: y = R^-1 g per segment, t1 = V y over the first kmax basis vectors
int kd_cycle_solution(KrylovDev &K, int kmax);
int kd_axpby(KrylovDev &K, const double *x, double *y, double a, double b);
// an empty graph holding one while node; body_out is the node's body graph
int kd_build_cycle_graph(cudaGraph_t *graph_out, cudaGraph_t *body_out, unsigned long long *cond_out);
// host reads (synchronous): the state and the iters / jdone / cyc / flags arrays; the norms; the loop flag
int kd_fetch_cycle(KrylovDev &K, KState *state_host, int *ints_host);
int kd_fetch_norms(KrylovDev &K, double *host);
int kd_fetch_more(KrylovDev &K, int *more);

// ---- Lanczos ---------------------------------------------------------------
struct LanczosDev {
    int nseg = 0, njobs = 0, nblk = 0, kcap = 0, KP = 0;
    long long n = 0, ldv = 0;
    cudaStream_t st = 0;
    void *base = nullptr;
    double *V = nullptr;  // basis (own allocation, grown by doubling)
    int vcap = 0;
    void *pinned = nullptr;
    double *w = nullptr, *xin = nullptr;
    KJob *jobs = nullptr;
    int *sjob = nullptr, *bjob = nullptr;
    double *partA = nullptr, *partB = nullptr, *partC = nullptr;
    double *zn = nullptr, *hd = nullptr, *hs = nullptr, *c = nullptr, *cold = nullptr, *dt = nullptr, *et = nullptr,
           *z = nullptr;
    int *iters = nullptr, *cyc = nullptr, *kfin = nullptr, *flags = nullptr;
    LzState *state = nullptr;
    ~LanczosDev();
    int init(const std::vector<long long> &seg_off, int kcap_, cudaStream_t s);
    int grow(int want);  // basis room for `want` vectors (copies the old ones)
};

struct LzMask {
    unsigned char *mask = nullptr;  // (pass, suspension) bytes the operator reads; null: none
    int nsusp = 0, nrhs = 0, pass = 8;
};

// start: |z_s| (host copy in zn_host), V_0 = z / |z_s| for the segments that
// run (zn > 0 and factor != 0), iteration counters, state
int lz_begin(LanczosDev &L, const double *z, double factor, int max_iter, std::vector<double> &zn_host,
             std::vector<int> &run);
int lz_step(LanczosDev &L, double factor, double tol, const LzMask &mk, unsigned long long cond, int use_cond,
            cudaStream_t st);
int lz_fetch_state(LanczosDev &L, LzState *host);
int lz_finish(LanczosDev &L, double *noise, std::vector<int> &iters);

bool graphs_enabled();
void graph_live(int delta);
void graph_count(bool captured);
int capture_stream(cudaStream_t home, cudaStream_t *out);

// Device-resident Lanczos (stochastic_forcing.py:112-264) over one or many
// segments: op(x, y) = y = M x on *sref.  Iterations run as a CUDA graph while
// node around [op(xin) -> w; lanczos_step_kernel]; the loop returns to the host
// only when every segment has stopped, after max_iter, or when the basis is
// full (the host doubles it and relaunches).
template <typename Op>
struct LanczosDevice {
    LanczosDev L;
    Op op;
    cudaStream_t *sref;
    cudaStream_t home;
    cudaStream_t priv = nullptr;
    cudaEvent_t ev = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    unsigned long long cond = 0;
    bool graph_failed = false;
    LzMask mk;
    double factor = 1.0, tol = 1e-3;
    std::vector<double> zn_;  // |z_s|

    LanczosDevice(Op f, cudaStream_t *s) : op(f), sref(s), home(*s) {}
    LanczosDevice(const LanczosDevice &) = delete;
    LanczosDevice &operator=(const LanczosDevice &) = delete;
    ~LanczosDevice()
    {
        if (exec) {
            cudaStreamSynchronize(home);
            cudaGraphExecDestroy(exec);
            graph_live(-1);
        }
        if (graph) cudaGraphDestroy(graph);
        if (ev) cudaEventDestroy(ev);
    }

    int capture_once()
    {
        cudaGraph_t g = nullptr, body = nullptr;
        if (int rc = kd_build_cycle_graph(&g, &body, &cond)) return rc;
        RMW_CUDA(cudaEventRecord(ev, home));
        RMW_CUDA(cudaStreamWaitEvent(priv, ev, 0));
        if (cudaStreamBeginCaptureToGraph(priv, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed) !=
            cudaSuccess) {
            cudaGraphDestroy(g);
            return RMW_ERR_CUDA;
        }
        *sref = priv;
        int rc = op(L.xin, L.w);
        *sref = home;
        if (rc == RMW_OK) rc = lz_step(L, factor, tol, mk, cond, 1, priv);
        cudaGraph_t cap = nullptr;
        const cudaError_t e = cudaStreamEndCapture(priv, &cap);
        if (rc != RMW_OK || e != cudaSuccess || cudaGraphInstantiate(&exec, g, 0) != cudaSuccess) {
            exec = nullptr;
            cudaGraphDestroy(g);
            cudaGetLastError();
            return RMW_ERR_CUDA;
        }
        graph = g;
        graph_live(+1);
        graph_count(true);
        return RMW_OK;
    }

    int build()
    {
        if (capture_stream(home, &priv) != RMW_OK || cudaEventCreateWithFlags(&ev, cudaEventDisableTiming))
            return RMW_ERR_CUDA;
        if (capture_once() == RMW_OK) return RMW_OK;
        // the operator grows its scratch on the capture stream once, then capture again
        RMW_CUDA(cudaEventRecord(ev, home));
        RMW_CUDA(cudaStreamWaitEvent(priv, ev, 0));
        *sref = priv;
        const int rc = op(L.xin, L.w);
        *sref = home;
        RMW_CUDA(cudaEventRecord(ev, priv));
        RMW_CUDA(cudaStreamWaitEvent(home, ev, 0));
        if (rc) return rc;
        return capture_once();
    }

    // iterations until the kernel clears the loop condition
    int run_loop()
    {
        if (graphs_enabled() && !graph_failed) {
            if (!exec && build() != RMW_OK) {
                cudaGetLastError();
                graph_failed = true;
            }
            if (exec) {
                void *tok = nullptr;
                if (int rc = trace_begin(TRACE_CYCLE, home, &tok)) return rc;
                RMW_CUDA(cudaGraphLaunch(exec, home));
                if (int rc = trace_end(tok, home)) return rc;
                graph_count(false);
                return RMW_OK;
            }
        }
        for (;;) {
            void *tok = nullptr;
            if (int rc = trace_begin(TRACE_OPERATOR, home, &tok)) return rc;
            if (int rc = op(L.xin, L.w)) return rc;
            if (int rc = trace_end(tok, home)) return rc;
            if (int rc = trace_begin(TRACE_KRYLOV, home, &tok)) return rc;
            if (int rc = lz_step(L, factor, tol, mk, 0, 0, home)) return rc;
            if (int rc = trace_end(tok, home)) return rc;
            LzState S;
            if (int rc = lz_fetch_state(L, &S)) return rc;
            if (!S.more) break;
        }
        return RMW_OK;
    }

    // Iterations from i0 on with the convergence test on the host: each step is
    // the operator and the step kernel in its recording mode, then one copy of
    // the new tridiagonal entries, the host's eigen-decompositions and
    // stopping tests, and the updated segment flags back to the device.
    int host_continuation(int i0, int max_iter)
    {
        const int ns = L.nseg, kc = L.kcap;
        std::vector<double> hd((size_t)ns * kc), hs((size_t)ns * kc), c((size_t)ns * kc), cold((size_t)ns * kc);
        std::vector<int> cyc(ns), iters(ns), kfin(ns);
        RMW_CUDA(cudaMemcpyAsync(hd.data(), L.hd, sizeof(double) * hd.size(), cudaMemcpyDeviceToHost, home));
        RMW_CUDA(cudaMemcpyAsync(hs.data(), L.hs, sizeof(double) * hs.size(), cudaMemcpyDeviceToHost, home));
        RMW_CUDA(cudaMemcpyAsync(cold.data(), L.cold, sizeof(double) * cold.size(), cudaMemcpyDeviceToHost, home));
        RMW_CUDA(cudaMemcpyAsync(cyc.data(), L.cyc, sizeof(int) * ns, cudaMemcpyDeviceToHost, home));
        RMW_CUDA(cudaMemcpyAsync(iters.data(), L.iters, sizeof(int) * ns, cudaMemcpyDeviceToHost, home));
        RMW_CUDA(cudaMemcpyAsync(kfin.data(), L.kfin, sizeof(int) * ns, cudaMemcpyDeviceToHost, home));
        RMW_CUDA(cudaStreamSynchronize(home));
        c = cold;
        const int one = 1;
        RMW_CUDA(cudaMemcpyAsync(&L.state->host, &one, sizeof(int), cudaMemcpyHostToDevice, home));
        std::vector<double> nd(2 * (size_t)ns), dd, ee, zq;
        std::vector<unsigned char> mask;
        for (int i = i0; i <= max_iter && i < kc; ++i) {
            int live = 0;
            for (int s = 0; s < ns; ++s) live += cyc[s];
            if (!live) break;
            if (i + 2 > L.vcap)
                if (int rc = L.grow(2 * L.vcap)) return rc;
            if (int rc = op(L.xin, L.w)) return rc;
            if (int rc = lz_step(L, factor, tol, mk, 0, 0, home)) return rc;
            // hd[s][i], hs[s][i] of every segment
            RMW_CUDA(cudaMemcpy2DAsync(nd.data(), sizeof(double), L.hd + i, sizeof(double) * kc, sizeof(double), ns,
                                       cudaMemcpyDeviceToHost, home));
            RMW_CUDA(cudaMemcpy2DAsync(nd.data() + ns, sizeof(double), L.hs + i, sizeof(double) * kc, sizeof(double),
                                       ns, cudaMemcpyDeviceToHost, home));
            RMW_CUDA(cudaStreamSynchronize(home));
            bool changed = false;
            const int k = i + 1;
            for (int s = 0; s < ns; ++s) {
                if (!cyc[s]) continue;
                const size_t so = (size_t)s * kc;
                hd[so + i] = nd[s];
                hs[so + i] = nd[ns + s];
                if (!std::isfinite(nd[s]) || !std::isfinite(nd[ns + s]))
                    return fail(RMW_ERR_BREAKDOWN, "Lanczos: non-finite value");
                dd.assign(hd.begin() + so, hd.begin() + so + k);
                ee.assign(hs.begin() + so, hs.begin() + so + i);
                if (!tridiag_eigen_host(dd, ee, zq)) return fail(RMW_ERR_BREAKDOWN, "Lanczos: tridiagonal eigensolver failed");
                double dn = 0.0, on = 0.0;
                for (int q = 0; q < k; ++q) {
                    double acc = 0.0;
                    for (int j = 0; j < k; ++j) {
                        const double lam = dd[j] > 0 ? std::sqrt(dd[j]) : 0.0;
                        acc += zq[q + (size_t)k * j] * (zq[(size_t)k * j] * lam * zn_[s] * factor);
                    }
                    const double old = q < i ? cold[so + q] : 0.0;
                    dn += (acc - old) * (acc - old);
                    on += old * old;
                    c[so + q] = acc;
                }
                for (int q = 0; q < k; ++q) cold[so + q] = c[so + q];
                kfin[s] = k;
                const bool conv = i > 0 && std::sqrt(dn) / std::max(std::sqrt(on), 2.220446049250313e-16) < tol;
                if (conv || nd[ns + s] == 0.0) {
                    iters[s] = i;
                    cyc[s] = 0;
                    changed = true;
                }
            }
            if (changed) {
                // freeze the stopped segments from the next step on (and their passes of the product)
                RMW_CUDA(cudaMemcpyAsync(L.cyc, cyc.data(), sizeof(int) * ns, cudaMemcpyHostToDevice, home));
                if (mk.mask) {
                    const int npass = (mk.nrhs + mk.pass - 1) / mk.pass;
                    mask.assign((size_t)npass * mk.nsusp, 0);
                    for (int p = 0; p < npass; ++p)
                        for (int u = 0; u < mk.nsusp; ++u)
                            for (int q = p * mk.pass; q < std::min(mk.nrhs, (p + 1) * mk.pass); ++q)
                                mask[(size_t)p * mk.nsusp + u] |= cyc[(size_t)q * mk.nsusp + u] ? 1 : 0;
                    RMW_CUDA(cudaMemcpyAsync(mk.mask, mask.data(), mask.size(), cudaMemcpyHostToDevice, home));
                }
                RMW_CUDA(cudaStreamSynchronize(home));
            }
        }
        RMW_CUDA(cudaMemcpyAsync(L.c, c.data(), sizeof(double) * c.size(), cudaMemcpyHostToDevice, home));
        RMW_CUDA(cudaMemcpyAsync(L.iters, iters.data(), sizeof(int) * ns, cudaMemcpyHostToDevice, home));
        RMW_CUDA(cudaMemcpyAsync(L.kfin, kfin.data(), sizeof(int) * ns, cudaMemcpyHostToDevice, home));
        RMW_CUDA(cudaStreamSynchronize(home));
        return RMW_OK;
    }

    // noise_s = factor M_s^(1/2) z_s per segment; iters per segment (the
    // reference's count: the index of the converged iteration, max_iter if none)
    // require_nonzero: a zero z is an error (the single-vector entry points), not a zero noise
    int run(const double *z, double *noise, double factor_, double tol_, int max_iter, int kcap,
            const std::vector<long long> &seg_off, std::vector<int> &iters, const LzMask &mask = LzMask(),
            bool require_nonzero = false)
    {
        factor = factor_;
        tol = tol_;
        mk = mask;
        if (int rc = L.init(seg_off, kcap, home)) return rc;
        std::vector<int> run;
        if (int rc = lz_begin(L, z, factor, max_iter, zn_, run)) return rc;
        std::vector<double> &zn = zn_;
        int n_run = 0;
        for (int s = 0; s < L.nseg; ++s) {
            if (!std::isfinite(zn[s]) || (require_nonzero && factor != 0.0 && !(zn[s] > 0.0)))
                return fail(RMW_ERR_NONFINITE, "Lanczos: |z| is zero or not finite");
            n_run += run[s];
        }
        if (mk.mask) {
            // the first operator application: every running segment
            const int npass = (mk.nrhs + mk.pass - 1) / mk.pass;
            std::vector<unsigned char> h((size_t)npass * mk.nsusp, 0);
            for (int p = 0; p < npass; ++p)
                for (int u = 0; u < mk.nsusp; ++u)
                    for (int q = p * mk.pass; q < std::min(mk.nrhs, (p + 1) * mk.pass); ++q)
                        h[(size_t)p * mk.nsusp + u] |= run[(size_t)q * mk.nsusp + u] ? 1 : 0;
            RMW_CUDA(cudaMemcpyAsync(mk.mask, h.data(), h.size(), cudaMemcpyHostToDevice, home));
            RMW_CUDA(cudaStreamSynchronize(home));
        }
        LzState S{};
        while (n_run > 0) {
            if (int rc = run_loop()) return rc;
            if (int rc = lz_fetch_state(L, &S)) return rc;
            if (S.bar.err) return fail(RMW_ERR_CUDA, "Lanczos: a grid barrier of the step kernel timed out");
            if (S.live > 0 && S.i <= max_iter && S.i < L.kcap && S.i < S.dev_k && S.i + 1 >= L.vcap) {
                if (int rc = L.grow(2 * L.vcap)) return rc;
                continue;
            }
            break;
        }
        if (n_run > 0 && S.live > 0 && S.i <= max_iter && S.i < L.kcap)
            if (int rc = host_continuation(S.i, max_iter)) return rc;
        if (n_run == 0) {
            RMW_CUDA(cudaMemsetAsync(noise, 0, sizeof(double) * L.n, home));
            iters.assign(L.nseg, 0);
            RMW_CUDA(cudaStreamSynchronize(home));
            return RMW_OK;
        }
        return lz_finish(L, noise, iters);
    }
};

// The engine: buffers, the captured cycle graph and the solve loop.
// pcop(x, y): y = A P^-1 x, launched on *sref (the engine redirects it to its
// capture stream while capturing).  op / pc of solve() run on *sref too.
template <typename PcOp>
struct GmresDevice {
    KrylovDev K;
    PcOp pcop;
    cudaStream_t *sref;
    cudaStream_t home;
    cudaStream_t priv = nullptr;
    cudaEvent_t ev = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    unsigned long long cond = 0;
    bool graph_failed = false;
    std::vector<int> ints;

    GmresDevice(PcOp f, cudaStream_t *s) : pcop(f), sref(s), home(*s) {}
    GmresDevice(const GmresDevice &) = delete;
    GmresDevice &operator=(const GmresDevice &) = delete;
    ~GmresDevice()
    {
        if (exec) {
            cudaStreamSynchronize(home);
            cudaGraphExecDestroy(exec);
            graph_live(-1);
        }
        if (graph) cudaGraphDestroy(graph);
        if (ev) cudaEventDestroy(ev);
    }

    int init(const std::vector<long long> &seg_off, int restart, int hist_cap)
    {
        return K.init(seg_off, restart, hist_cap, home);
    }

    int capture_once()
    {
        cudaGraph_t g = nullptr, body = nullptr;
        if (int rc = kd_build_cycle_graph(&g, &body, &cond)) return rc;
        RMW_CUDA(cudaEventRecord(ev, home));
        RMW_CUDA(cudaStreamWaitEvent(priv, ev, 0));
        if (cudaStreamBeginCaptureToGraph(priv, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed) !=
            cudaSuccess) {
            cudaGraphDestroy(g);
            return RMW_ERR_CUDA;
        }
        *sref = priv;
        int rc = pcop(K.xin, K.w);
        *sref = home;
        if (rc == RMW_OK) rc = kd_arnoldi_step(K, cond, 1, priv);
        cudaGraph_t cap = nullptr;
        const cudaError_t e = cudaStreamEndCapture(priv, &cap);
        if (rc != RMW_OK || e != cudaSuccess || cudaGraphInstantiate(&exec, g, 0) != cudaSuccess) {
            exec = nullptr;
            cudaGraphDestroy(g);
            cudaGetLastError();
            return RMW_ERR_CUDA;
        }
        graph = g;
        graph_live(+1);
        graph_count(true);
        return RMW_OK;
    }

    // Build the cycle graph: capture [pcop(xin) -> w; step] into the while
    // body on the private capture stream.  A first failure (an operator that
    // still had to grow its scratch on that stream) is retried once after one
    // direct application there.
    int build()
    {
        if (capture_stream(home, &priv) != RMW_OK || cudaEventCreateWithFlags(&ev, cudaEventDisableTiming))
            return RMW_ERR_CUDA;
        if (capture_once() == RMW_OK) return RMW_OK;
        RMW_CUDA(cudaEventRecord(ev, home));
        RMW_CUDA(cudaStreamWaitEvent(priv, ev, 0));
        *sref = priv;
        const int rc = pcop(K.xin, K.t2);
        *sref = home;
        RMW_CUDA(cudaEventRecord(ev, priv));
        RMW_CUDA(cudaStreamWaitEvent(home, ev, 0));
        if (rc) return rc;
        return capture_once();
    }

    // the Arnoldi steps of one restart cycle
    int run_steps()
    {
        if (graphs_enabled() && !graph_failed) {
            if (!exec && build() != RMW_OK) {
                cudaGetLastError();
                graph_failed = true;
            }
            if (exec) {
                void *tok = nullptr;
                if (int rc = trace_begin(TRACE_CYCLE, home, &tok)) return rc;
                RMW_CUDA(cudaGraphLaunch(exec, home));
                if (int rc = trace_end(tok, home)) return rc;
                graph_count(false);
                return RMW_OK;
            }
        }
        for (int j = 0; j < K.R; ++j) {
            void *tok = nullptr;
            if (int rc = trace_begin(TRACE_OPERATOR, home, &tok)) return rc;
            if (int rc = pcop(K.xin, K.w)) return rc;
            if (int rc = trace_end(tok, home)) return rc;
            if (int rc = trace_begin(TRACE_KRYLOV, home, &tok)) return rc;
            if (int rc = kd_arnoldi_step(K, 0, 0, home)) return rc;
            if (int rc = trace_end(tok, home)) return rc;
            if (tok) trace_bytes(TRACE_KRYLOV, 8.0 * (4.0 * j + 12.0) * (double)K.n);
            int more = 0;
            if (int rc = kd_fetch_more(K, &more)) return rc;
            if (!more) break;
        }
        return RMW_OK;
    }

    // x_s = A^-1 b_s per segment from x = 0, to |b_s - A x_s| <= tol_rel[s] |b_s|.
    // op(x, y): y = A x; pc(x, y): y = P^-1 x.  hist: per segment and step, the
    // residual estimate |g_{j+1}| / |b_s| (segment-major, hist_cap per segment).
    //
    // trust_estimate: when every running segment's Givens estimate met its
    // tolerance in a cycle, return without the closing true residual b - A x
    // (relres is then the estimate).  The inner solves of iterative refinement
    // use it: the outer loop recomputes the residual anyway.  Otherwise K.r
    // holds b - A x of the returned x (the inner solves of the residual
    // recurrence reuse it as their next residual).
    template <typename Op, typename Pc>
    int solve(Op op, Pc pc, const double *b, double *x_out, const std::vector<double> &tol_rel, int maxiter,
              std::vector<int> &iters, std::vector<double> &relres, std::vector<int> &status,
              std::vector<double> *hist = nullptr, bool trust_estimate = false)
    {
        const int ns = K.nseg;
        const long long n = K.n;
        cudaStream_t st = home;
        iters.assign(ns, 0);
        relres.assign(ns, 0.0);
        status.assign(ns, RMW_ERR_NOT_CONVERGED);
        std::vector<double> nr(ns), bnorm(ns), tol_abs(ns), beta(ns), alpha(ns);
        std::vector<int> act(ns, 0);
        ints.assign(4 * ns, 0);
        if (int rc = kd_seg_norm2(K, b)) return rc;
        if (int rc = kd_fetch_norms(K, nr.data())) return rc;
        int n_active = 0;
        for (int s = 0; s < ns; ++s) {
            bnorm[s] = std::sqrt(nr[s]);
            if (!std::isfinite(bnorm[s])) return fail(RMW_ERR_NONFINITE, "GMRES: right-hand side is not finite");
            tol_abs[s] = tol_rel[s] * bnorm[s];
            beta[s] = bnorm[s];
            act[s] = bnorm[s] > 0.0;
            if (!act[s]) status[s] = RMW_OK;
            n_active += act[s];
        }
        if (int rc = kd_set_solve_params(K, tol_abs, maxiter)) return rc;
        RMW_CUDA(cudaMemsetAsync(K.x, 0, sizeof(double) * n, st));
        RMW_CUDA(cudaMemcpyAsync(K.r, b, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
        while (n_active > 0) {
            for (int s = 0; s < ns; ++s) alpha[s] = act[s] ? 1.0 / beta[s] : 0.0;
            if (int rc = kd_cycle_begin(K, alpha, beta, act)) return rc;
            if (int rc = run_steps()) return rc;
            KState S;
            if (int rc = kd_fetch_cycle(K, &S, ints.data())) return rc;
            if (S.bar.err) return fail(RMW_ERR_CUDA, "GMRES: a grid barrier of the Arnoldi step timed out");
            for (int s = 0; s < ns; ++s)
                if (ints[3 * ns + s] & 2) return fail(RMW_ERR_BREAKDOWN, "GMRES: non-finite Arnoldi vector");
            // x += P^-1 V y
            if (int rc = kd_cycle_solution(K, S.j)) return rc;
            if (int rc = pc(K.t1, K.t2)) return rc;
            if (int rc = kd_axpby(K, K.t2, K.x, 1.0, 1.0)) return rc;
            if (trust_estimate) {
                bool all = true;
                for (int s = 0; s < ns; ++s) all = all && (!act[s] || (ints[3 * ns + s] & 4));
                if (all) {
                    std::vector<double> ge(ns);
                    RMW_CUDA(cudaMemcpyAsync(ge.data(), K.gres, sizeof(double) * ns, cudaMemcpyDeviceToHost, st));
                    RMW_CUDA(cudaStreamSynchronize(st));
                    for (int s = 0; s < ns; ++s) {
                        iters[s] = ints[s];
                        if (!act[s]) continue;
                        relres[s] = ge[s] / bnorm[s];
                        status[s] = RMW_OK;
                        act[s] = 0;
                    }
                    n_active = 0;
                    break;
                }
            }
            // r = b - A x
            if (int rc = op(K.x, K.r)) return rc;
            if (int rc = kd_axpby(K, b, K.r, 1.0, -1.0)) return rc;
            if (int rc = kd_seg_norm2(K, K.r)) return rc;
            if (int rc = kd_fetch_norms(K, nr.data())) return rc;
            RMW_CUDA(cudaMemsetAsync(K.flags, 0, sizeof(int) * ns, st));  // estimate flags are per cycle
            n_active = 0;
            for (int s = 0; s < ns; ++s) {
                iters[s] = ints[s];
                if (!act[s]) continue;
                beta[s] = std::sqrt(nr[s]);
                relres[s] = beta[s] / bnorm[s];
                if (!std::isfinite(beta[s])) return fail(RMW_ERR_BREAKDOWN, "GMRES: non-finite residual");
                if (beta[s] <= tol_abs[s]) {
                    status[s] = RMW_OK;
                    act[s] = 0;
                } else if (iters[s] >= maxiter) {
                    status[s] = RMW_ERR_NOT_CONVERGED;
                    act[s] = 0;
                } else if (ints[3 * ns + s] & 1) {
                    status[s] = RMW_ERR_BREAKDOWN;
                    act[s] = 0;
                } else {
                    ++n_active;
                }
            }
        }
        RMW_CUDA(cudaMemcpyAsync(x_out, K.x, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
        if (hist && K.hcap > 0) {
            hist->assign((size_t)ns * K.hcap, 0.0);
            RMW_CUDA(cudaMemcpyAsync(hist->data(), K.hist, sizeof(double) * ns * K.hcap, cudaMemcpyDeviceToHost, st));
        }
        RMW_CUDA(cudaStreamSynchronize(st));
        if (hist && K.hcap > 0)
            for (int s = 0; s < ns; ++s)
                for (int q = 0; q < K.hcap; ++q) (*hist)[(size_t)s * K.hcap + q] /= (bnorm[s] > 0 ? bnorm[s] : 1.0);
        return RMW_OK;
    }
};

}  // namespace rmw
