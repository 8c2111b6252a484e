// Shared host/device helpers of the rmw_gb300 library (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string>

#include "../../include/rmw_gb300.h"

namespace rmw {

// ---- error reporting (thread-local message, status codes of rmw_gb300.h) --
void set_error(const std::string &msg);
int fail(int code, const std::string &msg);
int cuda_fail(cudaError_t e, const char *where);

#define RMW_CUDA(call)                                        \
    do {                                                      \
        cudaError_t e_ = (call);                              \
        if (e_ != cudaSuccess) return ::rmw::cuda_fail(e_, #call); \
    } while (0)

#define RMW_CHECK_LAUNCH(where)                               \
    do {                                                      \
        cudaError_t e_ = cudaGetLastError();                  \
        if (e_ != cudaSuccess) return ::rmw::cuda_fail(e_, where); \
    } while (0)

// ---- per-device scratch --------------------------------------------------
// A grow-only device buffer per (device, stream, slot).  Calls on the same
// device, stream and slot share it (they are ordered by the stream); a call that
// needs more frees the old buffer (cudaFree synchronises the device, so no
// kernel still reads it) and allocates anew.
enum ScratchSlot { SCRATCH_PAIR = 0, SCRATCH_HOST_STAGING = 1, SCRATCH_FT_TERM = 2, SCRATCH_SLOTS = 3 };
int scratch(ScratchSlot slot, size_t bytes, void **ptr, cudaStream_t st);
// frees the current device's scratch buffers (deferred while graphs are alive)
int scratch_release_all();
// requests above `bytes` fail with RMW_ERR_ALLOC without touching the device (0 = no cap)
void scratch_set_limit(size_t bytes);
size_t scratch_limit();

// Keeps up to 1 GiB of freed stream-ordered allocations (cudaMallocAsync) in
// the current device's default pool across synchronisations, once per device.
// The solves allocate and free their work vectors on every call; with the
// pool's default release threshold of 0 each synchronisation hands that memory
// back to the driver and the next call maps it again.  The setting belongs to
// this process's context and ends with it.
int pool_retain();

// cudaMallocAsync.  With the environment variable RMW_POISON_ALLOC set, the new
// memory is filled with 0xFF bytes on the same stream (NaN in every
// floating-point type, -1 in every integer type), so that a kernel reading
// memory nothing wrote shows in its results: a debug aid for the test suite.
cudaError_t dmalloc_async(void **p, size_t bytes, cudaStream_t st);
template <typename T>
cudaError_t dmalloc_async(T **p, size_t bytes, cudaStream_t st)
{
    return dmalloc_async((void **)p, bytes, st);
}

// Page-locked host blocks reused across calls: cudaHostAlloc and cudaFreeHost
// cost tens of microseconds each, and cudaFreeHost waits for the device.
// pinned_take hands out a block of at least `bytes` (a cached one when one is
// large enough); pinned_give returns it for reuse once no copy uses it.
int pinned_take(size_t bytes, void **p);
void pinned_give(void *p);

inline cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

// ---- kernel tracing -------------------------------------------------------
// When enabled (rmw_trace_enable), launchers bracket their dominant kernel with
// CUDA events on the launching stream; rmw_trace_read sums the durations.
// Classes: the pair kernel, the Krylov vector work, the preconditioner apply
// (direct launches; work replayed inside a CUDA graph is timed by the class of
// the graph launch), one Krylov operator application (A P^-1, the Lanczos
// operator: graph replay or direct launches), a mixed solve's refinement
// residual, the preconditioner build, whole solves (first to last launch,
// host gaps included), and device-resident GMRES restart cycles (one graph
// launch: every operator application and fused Arnoldi step of the cycle).
enum TraceKernel {
    TRACE_PAIR = 0,
    TRACE_KRYLOV = 1,
    TRACE_PC = 2,
    TRACE_OPERATOR = 3,
    TRACE_REFINE = 4,
    TRACE_PCBUILD = 5,
    TRACE_SOLVE = 6,
    TRACE_CYCLE = 7,
    TRACE_KINDS = 8
};
bool trace_on();
int trace_begin(TraceKernel k, cudaStream_t st, void **token);
int trace_end(void *token, cudaStream_t st);
// algorithmic bytes moved by traced work of one class (counted while tracing is on)
void trace_bytes(TraceKernel k, double bytes);

constexpr double kPi = 3.14159265358979323846;

// ---- compensated FP32 accumulation ----------------------------------------
// TwoSum (Knuth): s + e == a + b exactly.
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e)
{
    // _rn intrinsics: never contracted into an FMA, so the transformation stays exact
    s = __fadd_rn(a, b);
    float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// 1/sqrt(x) by the hardware approximation (relative error below 2^-22) with
// a subnormal input flushed to zero: the arguments here are squared
// distances in blob radii, never subnormal, so the approximation needs no
// subnormal-input fix-up around it.
__device__ __forceinline__ float rsqrt_approx(float x)
{
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// (hi, lo) += x, keeping lo as the running compensation.
__device__ __forceinline__ void comp_add(float &hi, float &lo, float x)
{
    float s, e;
    two_sum(hi, x, s, e);
    hi = s;
    lo = __fadd_rn(lo, e);
}

}  // namespace rmw
