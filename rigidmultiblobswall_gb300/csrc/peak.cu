// FMA-pipe throughput probe: the measured FP32 / FP64 vector peak that the
// pair kernels' roofline fractions are reported against (the pair products are
// bound by the FP32 or FP64 pipe, not by HBM or the tensor cores).
#include "rmw_common.cuh"

namespace rmw {

template <typename T, int CHAINS>
__global__ void __launch_bounds__(256) fma_probe_kernel(T *sink, int iters, T seed)
{
    T acc[CHAINS];
#pragma unroll
    for (int c = 0; c < CHAINS; ++c) acc[c] = seed + T(threadIdx.x + c);
    const T m = T(0.9999999), k = T(1e-7);
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int c = 0; c < CHAINS; ++c) acc[c] = fma(acc[c], m, k);
    }
    T s = T(0);
#pragma unroll
    for (int c = 0; c < CHAINS; ++c) s += acc[c];
    if (s == T(-12345.678)) sink[0] = s;  // never true; keeps the chains alive
}

template <typename T, int CHAINS>
static int run_probe(int iters, double *flops_per_s, cudaStream_t st)
{
    int dev = 0, sms = 0;
    RMW_CUDA(cudaGetDevice(&dev));
    RMW_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    T *sink = nullptr;
    RMW_CUDA(rmw::dmalloc_async((void **)&sink, sizeof(T), st));
    const int blocks = sms * 8, threads = 256;
    cudaEvent_t e0, e1;
    RMW_CUDA(cudaEventCreate(&e0));
    RMW_CUDA(cudaEventCreate(&e1));
    fma_probe_kernel<T, CHAINS><<<blocks, threads, 0, st>>>(sink, iters / 8, T(1));  // warm-up
    RMW_CUDA(cudaEventRecord(e0, st));
    fma_probe_kernel<T, CHAINS><<<blocks, threads, 0, st>>>(sink, iters, T(1));
    RMW_CUDA(cudaEventRecord(e1, st));
    RMW_CUDA(cudaEventSynchronize(e1));
    RMW_CHECK_LAUNCH("fma probe");
    float ms = 0.f;
    RMW_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    RMW_CUDA(cudaEventDestroy(e0));
    RMW_CUDA(cudaEventDestroy(e1));
    RMW_CUDA(cudaFreeAsync(sink, st));
    RMW_CUDA(cudaStreamSynchronize(st));
    const double flops = 2.0 * CHAINS * (double)iters * blocks * threads;
    *flops_per_s = flops / (ms * 1e-3);
    return RMW_OK;
}

}  // namespace rmw

extern "C" int rmw_fma_peak(int fp64, double *flops_per_s_host, void *stream)
{
    if (!flops_per_s_host) return rmw::fail(RMW_ERR_ARG, "null output pointer");
    cudaStream_t st = rmw::as_stream(stream);
    if (fp64) return rmw::run_probe<double, 8>(1 << 12, flops_per_s_host, st);
    return rmw::run_probe<float, 8>(1 << 17, flops_per_s_host, st);
}
