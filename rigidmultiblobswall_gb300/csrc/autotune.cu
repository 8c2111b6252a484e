// Launch-shape autotuner for the all-pairs product kernels.
//
// The tunable shape is the source split of the 2-D grid (target tiles x
// source chunks): more chunks fill the 152 SMs for small N, fewer chunks cut
// the partial-sum traffic of the finalize pass for large N.  For the df64
// and mixed UF products the symmetric kernel (each unordered pair once) is a
// further candidate.  rmw_wall_autotune
// times every admissible split on synthetic blobs of the requested size with
// CUDA events and caches the fastest per (device, kind, precision mode, size
// bucket); the standard product entry points and the rigid-body operators use
// the cached split for every N in that bucket, the built-in rule otherwise.
#include <algorithm>
#include <cmath>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "wall_pair.cuh"

namespace rmw {

namespace {

struct TuneKey {
    int dev, kind, mode, bucket;
    bool operator<(const TuneKey &o) const
    {
        return std::tie(dev, kind, mode, bucket) < std::tie(o.dev, o.kind, o.mode, o.bucket);
    }
};

std::mutex g_tune_mu;
std::map<TuneKey, int> g_tuned;

// quarter-octave size buckets
int bucket_of(int n) { return n <= 1 ? 0 : (int)std::floor(4.0 * std::log2((double)n)); }

// largest admissible split: every chunk keeps at least one 128-source tile
int max_chunks(int n) { return std::max(1, std::min(64, n / 128)); }

TuneKey key_of(int kind, int mode, int n)
{
    int dev = 0;
    cudaGetDevice(&dev);
    return TuneKey{dev, kind, mode, bucket_of(n)};
}

// blobs uniform in a box of side ~ 4a N^(1/3) (x, y) and heights in [1.5a, 9.5a],
// unit-scale vectors; a splitmix hash of (seed, index) drives every draw
__global__ void synth_blobs_kernel(double *r, double *v, int n, double a, unsigned long long seed)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double side = 4.0 * a * cbrt((double)n);
    double u[6];
    unsigned long long x = seed + 0x9E3779B97F4A7C15ULL * (unsigned long long)(i + 1);
    for (int k = 0; k < 6; ++k) {
        x += 0x9E3779B97F4A7C15ULL;
        unsigned long long z = x;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
        z ^= z >> 31;
        u[k] = (double)(z >> 11) * (1.0 / 9007199254740992.0);
    }
    r[3 * i] = side * u[0];
    r[3 * i + 1] = side * u[1];
    r[3 * i + 2] = a * (1.5 + 8.0 * u[2]);
    v[3 * i] = u[3] - 0.5;
    v[3 * i + 1] = u[4] - 0.5;
    v[3 * i + 2] = u[5] - 0.5;
}

}  // namespace

int wall_chunks(int kind, int mode, int n)
{
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tuned.find(key_of(kind, mode, n));
        if (it != g_tuned.end()) {
            if (it->second == kSymChunks) return kSymChunks;
            return std::max(1, std::min(it->second, max_chunks(n)));
        }
    }
    // untuned: the symmetric kernel from 4,096 blobs in FP64 and df64 and from
    // 8,192 in mixed precision (measured faster at every size from there; the
    // caller falls back where it does not apply)
    if ((mode != RMW_MODE_MIXED && n >= 4096) || (mode == RMW_MODE_MIXED && n >= 8192)) return kSymChunks;
    return wall_default_chunks(n);
}

}  // namespace rmw

extern "C" {

// Time every admissible source split of the `kind` product in `mode` on n
// synthetic blobs (reps timed launches each, after one warm-up), cache the
// fastest for n's size bucket on the current device and report it with its
// time and the built-in rule's.  Synchronous.
int rmw_wall_autotune(int kind, int mode, int64_t n, int reps, void *stream, int *best_nchunks, double *best_ms,
                      double *default_ms)
{
    if (int rc = rmw::validate_product_args(kind, (void *)1, (void *)1, (void *)1, n, 1.0, 1.0, mode)) return rc;
    if (n < 2) return rmw::fail(RMW_ERR_ARG, "autotuning needs at least two blobs");
    if (reps <= 0) reps = 3;
    cudaStream_t st = rmw::as_stream(stream);
    const int N = (int)n;
    std::vector<int> cand;
    for (int c : {1, 2, 3, 4, 6, 8, 12, 16, 24, 32, 48, 64})
        if (c <= rmw::max_chunks(N)) cand.push_back(c);
    const int def = rmw::wall_default_chunks(N);
    if (std::find(cand.begin(), cand.end(), def) == cand.end()) cand.push_back(def);
    const bool try_sym = rmw::wall_sym_applicable(kind, mode, N, nullptr);
    if (try_sym) cand.push_back(rmw::kSymChunks);
    const int cmax = std::max(*std::max_element(cand.begin(), cand.end()), try_sym ? rmw::wall_sym_slots(N) : 1);
    const size_t vec = sizeof(double) * 3 * (size_t)N;
    const size_t ws_bytes = rmw::wall_scratch_bytes(N, mode, cmax);
    // events first: nothing to release if their creation fails
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    RMW_CUDA(cudaEventCreate(&e0));
    if (cudaError_t e = cudaEventCreate(&e1)) {
        cudaEventDestroy(e0);
        return rmw::cuda_fail(e, "cudaEventCreate");
    }
    char *buf = nullptr;
    if (cudaError_t e = rmw::dmalloc_async((void **)&buf, 3 * vec + ws_bytes + 256, st)) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        return rmw::cuda_fail(e, "cudaMallocAsync (autotune buffers)");
    }
    double *r = (double *)buf, *v = (double *)(buf + vec), *out = (double *)(buf + 2 * vec);
    void *ws = (void *)(((uintptr_t)(buf + 3 * vec) + 255) & ~(uintptr_t)255);
    rmw::synth_blobs_kernel<<<(N + 255) / 256, 256, 0, st>>>(r, v, N, 1.0, 0x5EEDULL);
    int rc = RMW_OK, best = def;
    float tbest = 0.f, tdef = 0.f;
    auto run = [&](int c) {
        if (c == rmw::kSymChunks)
            return rmw::wall_product_sym_with_scratch(kind, r, v, out, N, 1.0, 1.0, mode, st, ws);
        return rmw::wall_product_with_scratch(kind, r, v, out, N, 1.0, 1.0, nullptr, mode, st, ws, c);
    };
    for (int c : cand) {
        rc = run(c);
        if (rc) break;
        cudaEventRecord(e0, st);
        for (int k = 0; k < reps && rc == RMW_OK; ++k) rc = run(c);
        cudaEventRecord(e1, st);
        if (rc) break;
        cudaError_t e = cudaEventSynchronize(e1);
        if (e != cudaSuccess) {
            rc = rmw::cuda_fail(e, "autotune timing");
            break;
        }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        ms /= (float)reps;
        if (c == def) tdef = ms;
        if (tbest == 0.f || ms < tbest) {
            tbest = ms;
            best = c;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFreeAsync(buf, st);
    if (rc) return rc;
    RMW_CUDA(cudaStreamSynchronize(st));
    {
        std::lock_guard<std::mutex> lk(rmw::g_tune_mu);
        rmw::g_tuned[rmw::key_of(kind, mode, N)] = best;
    }
    if (best_nchunks) *best_nchunks = best;
    if (best_ms) *best_ms = tbest;
    if (default_ms) *default_ms = tdef;
    return RMW_OK;
}

// Source split the product entry points use for (kind, mode, n) on the
// current device (-1: the symmetric kernel); *tuned = 1 when it comes from
// rmw_wall_autotune.
int rmw_wall_autotune_lookup(int kind, int mode, int64_t n, int *nchunks, int *tuned)
{
    if (n < 1 || n > (int64_t(1) << 28)) return rmw::fail(RMW_ERR_ARG, "number of blobs out of range");
    const int c = rmw::wall_chunks(kind, mode, (int)n);
    bool hit = false;
    {
        std::lock_guard<std::mutex> lk(rmw::g_tune_mu);
        hit = rmw::g_tuned.count(rmw::key_of(kind, mode, (int)n)) > 0;
    }
    if (nchunks) *nchunks = c;
    if (tuned) *tuned = hit ? 1 : 0;
    return RMW_OK;
}

// Pin the launch choice of (kind, mode, n's size bucket) on the current
// device: a source split in [1, 64], or -1 for the symmetric kernel (only
// where it applies).
int rmw_wall_autotune_set(int kind, int mode, int64_t n, int nchunks)
{
    if (int rc = rmw::validate_product_args(kind, (void *)1, (void *)1, (void *)1, n, 1.0, 1.0, mode)) return rc;
    if (n < 1) return rmw::fail(RMW_ERR_ARG, "number of blobs must be positive");
    if (nchunks == rmw::kSymChunks) {
        if (!rmw::wall_sym_applicable(kind, mode, (int)n, nullptr))
            return rmw::fail(RMW_ERR_ARG, "the symmetric kernel covers the non-periodic products of 256 or "
                                          "more blobs within its partial-sum budget");
    } else if (nchunks < 1 || nchunks > 64) {
        return rmw::fail(RMW_ERR_ARG, "source split must be in [1, 64] or -1");
    }
    std::lock_guard<std::mutex> lk(rmw::g_tune_mu);
    rmw::g_tuned[rmw::key_of(kind, mode, (int)n)] = nchunks;
    return RMW_OK;
}

// Forget every tuned shape (all devices).
int rmw_wall_autotune_clear(void)
{
    std::lock_guard<std::mutex> lk(rmw::g_tune_mu);
    rmw::g_tuned.clear();
    return RMW_OK;
}

}  // extern "C"
