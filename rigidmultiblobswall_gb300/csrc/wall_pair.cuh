// Internal interface of the wall-RPY product launcher (wall_pair.cu).
#pragma once
#include "rmw_common.cuh"

namespace rmw {

// Source-chunk count the standard entry points use for n blobs.
int wall_default_chunks(int n);
// Scratch bytes needed for n blobs in `mode` split into `nchunks` source chunks:
// packed sources (64 B/blob FP64, 48 B/blob mixed, rounded up to 256 B) plus
// nchunks * 3n doubles of partial sums.
size_t wall_scratch_bytes(int n, int mode, int nchunks);
int validate_product_args(int kind, const void *r, const void *v, const void *out, int64_t n, double eta, double a,
                          int mode);
// Full product with the library's per-stream scratch (rmw_wall_product).
int wall_product(int kind, const double *r, const double *v, double *out, int64_t n, double eta, double a,
                 const double *L, int mode, cudaStream_t st);
// Launch pack + pair + finalize with caller-provided scratch (no allocation).
int wall_product_with_scratch(int kind, const double *r, const double *v, double *out, int n, double eta, double a,
                              const double *L, int mode, cudaStream_t st, void *scratch_ptr, int nchunks);

}  // namespace rmw
