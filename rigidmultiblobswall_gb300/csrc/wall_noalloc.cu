// rmw_wall_product_noalloc: the wall-RPY product with its scratch memory in a
// fixed, statically sized device array instead of a buffer the library
// allocates.
//
// Who needs it: callers that cannot call cudaMalloc.  Typical cases are a host
// application whose device memory is owned by another allocator (a framework
// that reserves the whole GPU up front and forbids foreign allocations), code
// that must not change the process's device-memory footprint after start-up,
// and latency-sensitive loops that cannot afford the implicit device-wide
// synchronisation of cudaMalloc / cudaFree.  The standard entry points grow a
// per-stream scratch buffer with cudaMalloc on first use; this one never
// allocates: the caller passes inputs and outputs, and the scratch lives in
// g_noalloc_scratch below.
//
// Cost of that choice: every GPU that loads the library holds the array
// (kNoallocScratchBytes = 16 MiB) until the process exits, and the largest
// product it accepts is RMW_NOALLOC_MAX_BLOBS blobs.
#include <mutex>

#include "rmw_common.cuh"
#include "wall_pair.cuh"

namespace rmw {

// Packed sources (<= 64 B/blob) plus one chunk of partial sums (24 B/blob)
// for RMW_NOALLOC_MAX_BLOBS blobs, rounded up: 88 B * 180,000 < 16 MiB.
constexpr size_t kNoallocScratchBytes = size_t(16) << 20;
static_assert(size_t(88) * RMW_NOALLOC_MAX_BLOBS + 256 <= kNoallocScratchBytes, "scratch too small");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];

namespace {
constexpr int kMaxDev = 64;
std::mutex g_noalloc_mu;
void *g_noalloc_addr[kMaxDev] = {};  // device address of g_noalloc_scratch, per device
}  // namespace

// Device address of the array on the current device.  In host code the name
// g_noalloc_scratch is only a host-side stand-in, not a device address, so the
// address is looked up once per device, with that device current, and cached.
static int noalloc_scratch_address(void **ptr)
{
    int dev = 0;
    RMW_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDev) return fail(RMW_ERR_ARG, "device index out of range");
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
        g_noalloc_addr[dev] = p;
    }
    *ptr = g_noalloc_addr[dev];
    return RMW_OK;
}

}  // namespace rmw

extern "C" int rmw_wall_product_noalloc(int kind, const double *r, const double *v, double *out, int64_t n,
                                        double eta, double a, const double *L_host, int mode, void *stream)
{
    int rc = rmw::validate_product_args(kind, r, v, out, n, eta, a, mode);
    if (rc) return rc;
    if (n > RMW_NOALLOC_MAX_BLOBS)
        return rmw::fail(RMW_ERR_ARG, "rmw_wall_product_noalloc: n = " + std::to_string((long long)n) +
                                          " exceeds RMW_NOALLOC_MAX_BLOBS = " +
                                          std::to_string((long long)RMW_NOALLOC_MAX_BLOBS) +
                                          " (the static scratch holds 16 MiB); use rmw_wall_product");
    if (n == 0) return RMW_OK;
    void *ws = nullptr;
    rc = rmw::noalloc_scratch_address(&ws);
    if (rc) return rc;
    // Same source-chunk split as the standard entry point when it fits,
    // otherwise as many chunks as the fixed array holds (at least one).
    int nchunks = rmw::wall_default_chunks((int)n);
    while (nchunks > 1 && rmw::wall_scratch_bytes((int)n, mode, nchunks) > rmw::kNoallocScratchBytes) --nchunks;
    // Every scratch byte a call reads was written earlier in the same call
    // (pack writes all n records, the pair kernel writes every partial slot),
    // so the previous call's contents never leak into the result and nothing
    // needs clearing.
    return rmw::wall_product_with_scratch(kind, r, v, out, (int)n, eta, a, L_host, mode, rmw::as_stream(stream), ws,
                                          nchunks);
}
