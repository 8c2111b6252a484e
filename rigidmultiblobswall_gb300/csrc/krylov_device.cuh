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
// kernels) and arnoldi_step_kernel, a persistent cooperative kernel (one CTA
// per SM at most) that does the whole classical Gram-Schmidt step with one
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

constexpr int kKdThreads = 1024;  // threads of the fused step CTAs
constexpr int kKdMaxBasis = 128;  // basis vectors a step handles (restart <= 120)

// contiguous piece [b, e) of segment `seg`, processed by CTA `blk`
struct KJob {
    int seg, blk;
    long long b, e;
};

// solver scalars shared by the step kernels of one solve
struct KState {
    int j;              // Arnoldi step within the cycle
    int active;         // segments still iterating after the step (last CTA reads it)
    unsigned done;      // CTAs finished with the step (last-CTA detection)
    unsigned bar_count;
    unsigned bar_gen;
    int err;            // a grid barrier gave up waiting
    int more;           // the loop condition the last step set
    int maxiter;        // iteration limit per segment (the solve's)
};

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

bool graphs_enabled();
void graph_live(int delta);
void graph_count(bool captured);
int capture_stream(cudaStream_t home, cudaStream_t *out);

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
    template <typename Op, typename Pc>
    int solve(Op op, Pc pc, const double *b, double *x_out, const std::vector<double> &tol_rel, int maxiter,
              std::vector<int> &iters, std::vector<double> &relres, std::vector<int> &status,
              std::vector<double> *hist = nullptr)
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
            if (S.err) return fail(RMW_ERR_CUDA, "GMRES: a grid barrier of the Arnoldi step timed out");
            for (int s = 0; s < ns; ++s)
                if (ints[3 * ns + s] & 2) return fail(RMW_ERR_BREAKDOWN, "GMRES: non-finite Arnoldi vector");
            // x += P^-1 V y
            if (int rc = kd_cycle_solution(K, S.j)) return rc;
            if (int rc = pc(K.t1, K.t2)) return rc;
            if (int rc = kd_axpby(K, K.t2, K.x, 1.0, 1.0)) return rc;
            // r = b - A x
            if (int rc = op(K.x, K.r)) return rc;
            if (int rc = kd_axpby(K, b, K.r, 1.0, -1.0)) return rc;
            if (int rc = kd_seg_norm2(K, K.r)) return rc;
            if (int rc = kd_fetch_norms(K, nr.data())) return rc;
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
