// A fixed linear operator y = F(x) on device vectors, replayed as one CUDA
// graph per application.
//
// The operator's launches go to the stream *sref (a handle's stream field).
// Because a handle may live on the legacy default stream, which cannot be
// captured, warm-up and capture run on a private non-blocking stream paired
// with the handle's stream (ordered against it with events): the first call
// runs F there directly (so that scratch buffers, kernel attributes and lazy
// tables exist for that stream), the second captures F on two private
// buffers, and every later call copies x in, launches the graph on the
// handle's stream and copies y out - one graph launch instead of the
// operator's dozen kernel launches.  If anything in capture or instantiation
// fails the operator keeps running directly.  F must launch the same work for
// every input, read the stream from *sref at each launch and allocate nothing
// once warmed up.
#pragma once
#include "rmw_common.cuh"

namespace rmw {

bool graphs_enabled();
void graph_count(bool captured);
// number of instantiated graphs alive (scratch buffers they may reference are
// not freed while it is positive)
void graph_live(int delta);
// the private capture stream paired with `home` on the current device
int capture_stream(cudaStream_t home, cudaStream_t *out);

template <typename F>
struct GraphOp {
    F f;
    cudaStream_t *sref;
    cudaStream_t home;
    cudaStream_t priv = nullptr;
    cudaEvent_t ev_a = nullptr, ev_b = nullptr;
    long long n_in, n_out;
    double *xin = nullptr, *yout = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int calls = 0;
    bool direct;

    GraphOp(F f_, cudaStream_t *s, long long nin, long long nout)
        : f(f_), sref(s), home(*s), n_in(nin), n_out(nout), direct(!graphs_enabled()) {}
    GraphOp(const GraphOp &) = delete;
    GraphOp &operator=(const GraphOp &) = delete;
    ~GraphOp()
    {
        if (exec) {
            cudaGraphExecDestroy(exec);
            graph_live(-1);
        }
        if (graph) cudaGraphDestroy(graph);
        if (xin) cudaFreeAsync(xin, home);
        if (yout) cudaFreeAsync(yout, home);
        if (ev_a) cudaEventDestroy(ev_a);
        if (ev_b) cudaEventDestroy(ev_b);
    }

    // run F on the private stream, ordered after and before the home stream's work
    int on_private(const double *x, double *y)
    {
        RMW_CUDA(cudaEventRecord(ev_a, home));
        RMW_CUDA(cudaStreamWaitEvent(priv, ev_a, 0));
        *sref = priv;
        const int rc = f(x, y);
        *sref = home;
        RMW_CUDA(cudaEventRecord(ev_b, priv));
        RMW_CUDA(cudaStreamWaitEvent(home, ev_b, 0));
        return rc;
    }

    int fall_back(const double *x, double *y)
    {
        cudaGetLastError();
        direct = true;
        return f(x, y);
    }

    int operator()(const double *x, double *y)
    {
        if (direct) return f(x, y);
        if (!priv) {
            if (capture_stream(home, &priv) != RMW_OK ||
                cudaEventCreateWithFlags(&ev_a, cudaEventDisableTiming) != cudaSuccess ||
                cudaEventCreateWithFlags(&ev_b, cudaEventDisableTiming) != cudaSuccess)
                return fall_back(x, y);
        }
        if (calls++ == 0) return on_private(x, y);
        if (!exec) {
            if (cudaMalloc(&xin, sizeof(double) * n_in) != cudaSuccess ||
                cudaMalloc(&yout, sizeof(double) * n_out) != cudaSuccess ||
                cudaMemset(xin, 0, sizeof(double) * n_in) != cudaSuccess)
                return fall_back(x, y);
            RMW_CUDA(cudaEventRecord(ev_a, home));
            RMW_CUDA(cudaStreamWaitEvent(priv, ev_a, 0));
            if (cudaStreamBeginCapture(priv, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return fall_back(x, y);
            *sref = priv;
            const int rc = f(xin, yout);
            *sref = home;
            cudaGraph_t g = nullptr;
            const cudaError_t e = cudaStreamEndCapture(priv, &g);
            if (rc != RMW_OK || e != cudaSuccess || !g || cudaGraphInstantiate(&exec, g, 0) != cudaSuccess) {
                if (g) cudaGraphDestroy(g);
                exec = nullptr;
                return fall_back(x, y);
            }
            graph = g;
            graph_live(+1);
            graph_count(true);
        }
        RMW_CUDA(cudaMemcpyAsync(xin, x, sizeof(double) * n_in, cudaMemcpyDeviceToDevice, home));
        RMW_CUDA(cudaGraphLaunch(exec, home));
        RMW_CUDA(cudaMemcpyAsync(y, yout, sizeof(double) * n_out, cudaMemcpyDeviceToDevice, home));
        graph_count(false);
        return RMW_OK;
    }
};

template <typename F>
GraphOp<F> make_graph_op(F f, cudaStream_t *stream_ref, long long n_in, long long n_out)
{
    return GraphOp<F>(f, stream_ref, n_in, n_out);
}

}  // namespace rmw
