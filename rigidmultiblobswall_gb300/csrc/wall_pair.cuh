// Internal interface of the wall-RPY product launcher (wall_pair.cu).
#pragma once
#include "rmw_common.cuh"

#include <vector>

namespace rmw {

// One CTA of a segmented (batched) product: targets [t0, t1) against sources
// [s0, s1) of the same suspension, partial sums into chunk slot `slot`.
struct TileJob {
    int t0, t1, s0, s1, slot, susp;
};

// One CTA of a segmented symmetric UF product: tile pair T <= S of the
// suspension whose blobs start at `base` (n of them), partial sums of that
// suspension at `pbase` (its nt slots of 3n doubles).
struct SymJob {
    long long pbase;
    int base, n, T, S;
};

// Segmented product layout for many independent suspensions of one blob
// array: suspension k owns blobs [off[k], off[k+1]) and only interacts with
// itself.  Built once (rmw_wall_batch_create) and reused by every product.
struct WallBatch {
    int n = 0;          // total blobs
    int ninst = 0;      // suspensions
    int njobs = 0;      // CTAs per product
    int max_slots = 1;  // chunk slots of the partial-sum buffer
    TileJob *jobs = nullptr;  // device
    int *blob_nch = nullptr;  // device: chunk count of each blob's suspension
    int *blob_susp = nullptr; // device: suspension of each blob
    // symmetric UF layout: per suspension nt = ceil(n / 128) tiles, nt (nt + 1) / 2 CTAs
    long long nsym = 0;             // CTAs
    long long sym_doubles = 0;      // partial-sum doubles (sum over suspensions of nt * 3n)
    SymJob *sym_jobs = nullptr;     // device
    long long *blob_pbase = nullptr;  // device: slot-0 entry of each blob's partial sums
    int *blob_pstride = nullptr;    // device: 3n of each blob's suspension (slot stride)
    int *blob_nslots = nullptr;     // device: nt of each blob's suspension
    std::vector<long long> off;
    int device = 0;
};
int wall_batch_build(WallBatch &B, const long long *off_host, int ninst);
void wall_batch_free(WallBatch &B);
// Tile pair (T, S), T <= S, of CTA b over the upper triangle of nt tiles (the
// symmetric kernels' grid): rows T = 0.. hold nt - T entries.
__device__ __forceinline__ void sym_tile_pair(long long b, int nt, int &T, int &S)
{
    // rows T = 0.. of the upper triangle hold nt - T entries; offset(T) = T nt - T (T - 1) / 2
    const double c = 2.0 * nt + 1.0;
    int t = (int)floor(0.5 * (c - sqrt(fmax(c * c - 8.0 * (double)b, 0.0))));
    t = max(0, min(nt - 1, t));
    auto off = [nt](long long tt) { return tt * nt - tt * (tt - 1) / 2; };
    while (t > 0 && off(t) > b) --t;
    while (t + 1 < nt && off(t + 1) <= b) ++t;
    T = t;
    S = t + (int)(b - off(t));
}

// Right-hand sides per pass of wall_uf_multi.
constexpr int kMultiPass = 16;
// M_UF applied to nrhs vectors in mixed precision (rows of V, stride ldv).
// With a batch and `active` (one byte per suspension and pass of kMultiPass
// vectors, pass-major), suspensions whose byte is 0 are skipped and get zero
// rows.
int wall_uf_multi(const double *r, const double *V, long long ldv, double *Y, long long ldy, int nrhs, int n,
                  double eta, double a, const WallBatch *B, cudaStream_t st, const unsigned char *active = nullptr);
int wall_product_batched(const WallBatch &B, int kind, const double *r, const double *v, double *out, double eta,
                         double a, int mode, cudaStream_t st);

// Source-chunk count of the built-in rule for n blobs.
int wall_default_chunks(int n);
// Symmetric product of any kind (each unordered pair once, applied both ways),
// df64 or mixed: selected when wall_chunks returns kSymChunks and
// wall_sym_applicable holds (df64 or mixed, not periodic, n >= 256, ntiles x
// 3n doubles of partial sums within wall_sym_partial_budget()).  Its scratch is
// wall_scratch_bytes(n, mode, wall_sym_slots(n)).
constexpr int kSymChunks = -1;
constexpr size_t kSymMaxPartialBytes = size_t(6) << 30;  // up to ~185,000 blobs (5.5 GB at 172,032)
// The partial-sum budget of the current device: kSymMaxPartialBytes, or an
// eighth of the device's memory if that is more (35 GB, ~430,000 blobs, on a
// 284 GB part).  A fixed property of the device, so the kernel choice for a
// given n does not depend on what else is allocated.
size_t wall_sym_partial_budget();
bool wall_sym_applicable(int kind, int mode, int n, const double *L);
int wall_sym_slots(int n);
// banded symmetric df64 product (above the partial-sum budget): tile rows per band, its scratch
int wall_sym_band_rows(int n);
size_t wall_sym_band_scratch_bytes(int n);
int wall_product_sym_with_scratch(int kind, const double *r, const double *v, double *out, int n, double eta,
                                  double a, int mode, cudaStream_t st, void *scratch_ptr);
// The symmetric free-space pair kernel of `kind` on records packed by the
// no-wall product (layouts of SrcD / SrcDF / SrcF, positions over a); writes
// wall_sym_slots(n) partial-sum slots of 3n doubles.
int nowall_sym_launch(int kind, int mode, const void *src, int n, double *partial, cudaStream_t st);
// Source-chunk count the standard entry points use: the autotuned choice of
// (kind, mode, n's size bucket) on the current device if there is one
// (autotune.cu; kSymChunks = the symmetric kernel), else the built-in rule.
int wall_chunks(int kind, int mode, int n);
// Scratch bytes needed for n blobs in `mode` split into `nchunks` source chunks:
// packed sources (64 B/blob FP64, 48 B/blob mixed, rounded up to 256 B) plus
// nchunks * 3n doubles of partial sums.
size_t wall_scratch_bytes(int n, int mode, int nchunks);
int validate_product_args(int kind, const void *r, const void *v, const void *out, int64_t n, double eta, double a,
                          int mode);
// Free-space (no-wall) RPY product (nowall.cu, rmw_nowall_product).
int nowall_product(int kind, const double *r, const double *v, double *out, int64_t n, double eta, double a,
                   const double *L, int mode, cudaStream_t st);
// Full product with the library's per-stream scratch (rmw_wall_product).
int wall_product(int kind, const double *r, const double *v, double *out, int64_t n, double eta, double a,
                 const double *L, int mode, cudaStream_t st);
// Launch pack + pair + finalize with caller-provided scratch (no allocation).
int wall_product_with_scratch(int kind, const double *r, const double *v, double *out, int n, double eta, double a,
                              const double *L, int mode, cudaStream_t st, void *scratch_ptr, int nchunks);

}  // namespace rmw
