// Error reporting and per-device scratch of the rmw_gb300 library.
#include <algorithm>
#include <cstdlib>
#include <cstdio>
#include <atomic>
#include <mutex>
#include <string>
#include <vector>
#include <map>
#include <tuple>

#include "rmw_common.cuh"

namespace rmw {

static thread_local std::string g_last_error;

void set_error(const std::string &msg) { g_last_error = msg; }

int fail(int code, const std::string &msg)
{
    set_error(msg);
    return code;
}

int cuda_fail(cudaError_t e, const char *where)
{
    std::string m = std::string(where) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
    set_error(m);
    return (e == cudaErrorMemoryAllocation) ? RMW_ERR_ALLOC : RMW_ERR_CUDA;
}

namespace {
struct ScratchBuf {
    void *ptr = nullptr;
    size_t bytes = 0;
};
std::mutex g_scratch_mu;
// keyed by (device, stream, slot): calls on different streams never share scratch
std::map<std::tuple<int, void *, int>, ScratchBuf> g_scratch;
}  // namespace

// Buffers replaced while a captured CUDA graph may still reference them are
// freed only when the last graph is gone.
static int g_live_graphs = 0;
static std::vector<std::pair<int, void *>> g_deferred;

void graph_live(int delta)
{
    std::vector<std::pair<int, void *>> release;
    {
        std::lock_guard<std::mutex> lock(g_scratch_mu);
        g_live_graphs += delta;
        if (g_live_graphs == 0) release.swap(g_deferred);
    }
    int cur = 0;
    cudaGetDevice(&cur);
    for (auto &d : release) {
        cudaSetDevice(d.first);
        cudaFree(d.second);  // waits for the device: no replay still uses it
    }
    if (!release.empty()) cudaSetDevice(cur);
}

// cap on one scratch buffer (rmw_set_scratch_limit); 0 = no cap
static std::atomic<size_t> g_scratch_limit{0};

static std::mutex g_pool_mu;
static std::vector<int> g_pool_devices;  // devices whose default pool retains memory

cudaError_t dmalloc_async(void **p, size_t bytes, cudaStream_t st)
{
    static const bool poison = [] {
        const char *v = std::getenv("RMW_POISON_ALLOC");
        return v && *v && *v != '0';
    }();
    const cudaError_t e = cudaMallocAsync(p, bytes, st);
    if (e != cudaSuccess || !poison || bytes == 0) return e;
    return cudaMemsetAsync(*p, 0xFF, bytes, st);
}

namespace {
struct PinnedBlock {
    void *p;
    size_t bytes;
};
std::mutex g_pinned_mu;
std::vector<PinnedBlock> g_pinned_free;               // blocks ready for reuse
std::map<void *, size_t> g_pinned_size;               // every block handed out, with its size
constexpr size_t kPinnedCached = 32;                  // free blocks kept at most
}  // namespace

int pinned_take(size_t bytes, void **p)
{
    *p = nullptr;
    std::lock_guard<std::mutex> lock(g_pinned_mu);
    int best = -1;
    for (int k = 0; k < (int)g_pinned_free.size(); ++k)
        if (g_pinned_free[k].bytes >= bytes && (best < 0 || g_pinned_free[k].bytes < g_pinned_free[best].bytes))
            best = k;
    if (best >= 0) {
        *p = g_pinned_free[best].p;
        g_pinned_free.erase(g_pinned_free.begin() + best);
        return RMW_OK;
    }
    const size_t want = (std::max<size_t>(bytes, 1) + 4095) / 4096 * 4096;
    RMW_CUDA(cudaHostAlloc(p, want, cudaHostAllocDefault));
    g_pinned_size[*p] = want;
    return RMW_OK;
}

void pinned_give(void *p)
{
    if (!p) return;
    std::lock_guard<std::mutex> lock(g_pinned_mu);
    auto it = g_pinned_size.find(p);
    if (it == g_pinned_size.end()) return;
    if (g_pinned_free.size() >= kPinnedCached) {
        // drop the smallest cached block
        int small = 0;
        for (int k = 1; k < (int)g_pinned_free.size(); ++k)
            if (g_pinned_free[k].bytes < g_pinned_free[small].bytes) small = k;
        if (g_pinned_free[small].bytes < it->second) {
            cudaFreeHost(g_pinned_free[small].p);
            g_pinned_size.erase(g_pinned_free[small].p);
            g_pinned_free[small] = {p, it->second};
        } else {
            cudaFreeHost(p);
            g_pinned_size.erase(it);
        }
        return;
    }
    g_pinned_free.push_back({p, it->second});
}

int pool_retain()
{
    int dev = 0;
    RMW_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(g_pool_mu);
    for (int d : g_pool_devices)
        if (d == dev) return RMW_OK;
    cudaMemPool_t pool;
    RMW_CUDA(cudaDeviceGetDefaultMemPool(&pool, dev));
    unsigned long long keep = 1ULL << 30;
    RMW_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
    g_pool_devices.push_back(dev);
    return RMW_OK;
}

int scratch(ScratchSlot slot, size_t bytes, void **ptr, cudaStream_t st)
{
    int dev = 0;
    RMW_CUDA(cudaGetDevice(&dev));
    const size_t cap = g_scratch_limit.load();
    if (cap && bytes > cap)
        return fail(RMW_ERR_ALLOC, "scratch request of " + std::to_string(bytes) + " bytes is above the limit of " +
                                       std::to_string(cap) + " bytes set by rmw_set_scratch_limit");
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    ScratchBuf &b = g_scratch[std::make_tuple(dev, (void *)st, (int)slot)];
    if (b.bytes < bytes) {
        if (b.ptr) {
            if (g_live_graphs > 0) {
                g_deferred.push_back({dev, b.ptr});
            } else {
                // cudaFree waits for all work on the device, so no kernel still uses the old buffer.
                RMW_CUDA(cudaFree(b.ptr));
            }
            b.ptr = nullptr;
            b.bytes = 0;
        }
        // headroom so that slowly growing sizes reallocate rarely (none above 1 GiB, and never past the cap)
        size_t want = bytes + (bytes >= ((size_t)1 << 30) ? 0 : bytes / 4) + 4096;
        if (cap && want > cap) want = bytes;
        RMW_CUDA(cudaMalloc(&b.ptr, want));
        b.bytes = want;
    }
    *ptr = b.ptr;
    return RMW_OK;
}

// Frees every scratch buffer of the current device that no live graph may use.
int scratch_release_all()
{
    int dev = 0;
    RMW_CUDA(cudaGetDevice(&dev));
    std::vector<void *> release;
    {
        std::lock_guard<std::mutex> lock(g_scratch_mu);
        for (auto it = g_scratch.begin(); it != g_scratch.end();) {
            if (std::get<0>(it->first) == dev && it->second.ptr) {
                if (g_live_graphs > 0) g_deferred.push_back({dev, it->second.ptr});
                else release.push_back(it->second.ptr);
                it = g_scratch.erase(it);
            } else {
                ++it;
            }
        }
    }
    for (void *p : release) RMW_CUDA(cudaFree(p));
    return RMW_OK;
}

void scratch_set_limit(size_t bytes) { g_scratch_limit.store(bytes); }
size_t scratch_limit() { return g_scratch_limit.load(); }

// ---- tracing ---------------------------------------------------------------
namespace {
struct TraceRec {
    int kind;
    cudaEvent_t e0, e1;
};
std::mutex g_trace_mu;
bool g_trace = false;
std::vector<TraceRec> g_trace_recs;
std::vector<cudaEvent_t> g_event_pool;  // reused events: no event creation on the launch path

cudaError_t pooled_event(cudaEvent_t *e)
{
    if (g_event_pool.empty()) {
        for (int k = 0; k < 64; ++k) {
            cudaEvent_t x;
            cudaError_t rc = cudaEventCreate(&x);
            if (rc != cudaSuccess) return rc;
            g_event_pool.push_back(x);
        }
    }
    *e = g_event_pool.back();
    g_event_pool.pop_back();
    return cudaSuccess;
}
}  // namespace

bool trace_on() { return g_trace; }

int trace_begin(TraceKernel k, cudaStream_t st, void **token)
{
    *token = nullptr;
    if (!g_trace) return RMW_OK;
    // work captured into a CUDA graph is not traced (its events would be
    // recorded once at capture, not at every replay)
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cap) == cudaSuccess && cap != cudaStreamCaptureStatusNone) return RMW_OK;
    TraceRec *r = new TraceRec{(int)k, nullptr, nullptr};
    {
        std::lock_guard<std::mutex> lock(g_trace_mu);
        RMW_CUDA(pooled_event(&r->e0));
        RMW_CUDA(pooled_event(&r->e1));
    }
    RMW_CUDA(cudaEventRecord(r->e0, st));
    *token = r;
    return RMW_OK;
}

static double g_trace_byte_count[TRACE_KINDS] = {};

void trace_bytes(TraceKernel k, double bytes)
{
    std::lock_guard<std::mutex> lock(g_trace_mu);
    if (g_trace) g_trace_byte_count[k] += bytes;
}

int trace_end(void *token, cudaStream_t st)
{
    if (!token) return RMW_OK;
    TraceRec *r = (TraceRec *)token;
    RMW_CUDA(cudaEventRecord(r->e1, st));
    std::lock_guard<std::mutex> lock(g_trace_mu);
    g_trace_recs.push_back(*r);
    delete r;
    return RMW_OK;
}

static std::atomic<bool> g_graphs{true};
static std::atomic<long long> g_graph_captures{0}, g_graph_replays{0};

bool graphs_enabled() { return g_graphs.load(); }

// one private non-blocking stream per (device, home stream), kept for the
// process lifetime so that its scratch buffers are reused across solves
static std::mutex g_capture_mu;
static std::map<std::pair<int, void *>, cudaStream_t> g_capture_streams;

int capture_stream(cudaStream_t home, cudaStream_t *out)
{
    int dev = 0;
    RMW_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(g_capture_mu);
    cudaStream_t &s = g_capture_streams[{dev, (void *)home}];
    if (!s) RMW_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    *out = s;
    return RMW_OK;
}
void graph_count(bool captured)
{
    if (captured) ++g_graph_captures;
    else ++g_graph_replays;
}

}  // namespace rmw

extern "C" {

int rmw_use_graphs(int on)
{
    rmw::g_graphs = (on != 0);
    return RMW_OK;
}

int rmw_graph_stats(int64_t *captures_host, int64_t *replays_host, int reset)
{
    if (captures_host) *captures_host = rmw::g_graph_captures.load();
    if (replays_host) *replays_host = rmw::g_graph_replays.load();
    if (reset) {
        rmw::g_graph_captures = 0;
        rmw::g_graph_replays = 0;
    }
    return RMW_OK;
}

int rmw_set_scratch_limit(int64_t bytes)
{
    if (bytes < 0) return rmw::fail(RMW_ERR_ARG, "scratch limit must be >= 0");
    rmw::scratch_set_limit((size_t)bytes);
    return RMW_OK;
}

int rmw_release_scratch(void) { return rmw::scratch_release_all(); }

int rmw_trace_enable(int on)
{
    std::lock_guard<std::mutex> lock(rmw::g_trace_mu);
    rmw::g_trace = (on != 0);
    return RMW_OK;
}

int rmw_trace_read(int kind, double *total_ms_host, int64_t *launches_host, int reset)
{
    if (!total_ms_host || !launches_host) return rmw::fail(RMW_ERR_ARG, "null output pointer");
    if (kind < 0 || kind >= rmw::TRACE_KINDS) return rmw::fail(RMW_ERR_ARG, "bad trace kind");
    std::lock_guard<std::mutex> lock(rmw::g_trace_mu);
    double tot = 0.0;
    int64_t cnt = 0;
    for (auto &r : rmw::g_trace_recs) {
        if (r.kind != kind) continue;
        RMW_CUDA(cudaEventSynchronize(r.e1));
        float ms = 0.f;
        RMW_CUDA(cudaEventElapsedTime(&ms, r.e0, r.e1));
        tot += ms;
        ++cnt;
    }
    *total_ms_host = tot;
    *launches_host = cnt;
    if (reset) {
        // only this class's records: the others stay readable
        std::vector<rmw::TraceRec> keep;
        for (auto &r : rmw::g_trace_recs) {
            if (r.kind == kind) {
                rmw::g_event_pool.push_back(r.e0);
                rmw::g_event_pool.push_back(r.e1);
            } else {
                keep.push_back(r);
            }
        }
        rmw::g_trace_recs.swap(keep);
    }
    return RMW_OK;
}


int rmw_trace_bytes(int kind, double *bytes_host, int reset)
{
    if (kind < 0 || kind >= rmw::TRACE_KINDS || !bytes_host) return rmw::fail(RMW_ERR_ARG, "bad trace kind or pointer");
    std::lock_guard<std::mutex> lock(rmw::g_trace_mu);
    *bytes_host = rmw::g_trace_byte_count[kind];
    if (reset) rmw::g_trace_byte_count[kind] = 0.0;
    return RMW_OK;
}

const char *rmw_last_error(void) { return rmw::g_last_error.c_str(); }

int rmw_version(void) { return 1; }

}  // extern "C"
