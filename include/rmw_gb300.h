/*
 * rmw_gb300 - C ABI of the GB300 (sm_103a) wall-corrected RPY blob mobility
 * library.  Plain pointers and sizes only; every array argument is a DEVICE
 * pointer unless its name ends in _host.  All calls are asynchronous on the
 * given CUDA stream (NULL = legacy default stream) unless documented otherwise,
 * and return an RMW_* status code; rmw_last_error() gives the message of the
 * last failure on the calling thread.
 *
 * Layouts follow the reference (RigidMultiblobsWall):
 *   positions r     (n,3) float64, row-major (x,y,z per blob)
 *   force / torque  (n,3) float64
 *   outputs         (n,3) float64, overwritten (never accumulated)
 *   periodic L      3 float64 on the HOST; L[k] > 0 makes dimension k
 *                   pseudo-periodic (minimum image + the +-1 neighbour boxes)
 */
#ifndef RMW_GB300_H
#define RMW_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------- */
#define RMW_OK 0
#define RMW_ERR_ARG 1           /* invalid argument (size, pointer, mode) */
#define RMW_ERR_CUDA 2          /* a CUDA runtime call failed */
#define RMW_ERR_NOT_CONVERGED 3 /* Krylov solver hit maxiter */
#define RMW_ERR_BREAKDOWN 4     /* Krylov breakdown / non-finite residual */
#define RMW_ERR_NONFINITE 5     /* NaN or Inf detected in an input or result */
#define RMW_ERR_ALLOC 6         /* device allocation failed */

/* ---- precision modes ------------------------------------------------- */
#define RMW_MODE_FP64 0  /* every pair in FP64 */
#define RMW_MODE_MIXED 1 /* FP32 pair evaluation (double-float positions),
                            compensated per-target accumulation, FP64 output */

/* ---- product kinds ---------------------------------------------------- */
#define RMW_UF 0 /* u = M_UF f  (1/(8 pi eta a))   */
#define RMW_UT 1 /* u = M_UT t  (1/(8 pi eta a^2)) */
#define RMW_WF 2 /* w = M_WF f  (1/(8 pi eta a^2)) */
#define RMW_WT 3 /* w = M_WT t  (1/(8 pi eta a^3)) */

const char *rmw_last_error(void);
int rmw_version(void);

/* Wall-regularised single-wall RPY products  out = B M(z_eff) B v  with
 * z_eff = max(z, a) and B = diag(min(z/a, 1)), exactly the operator the
 * reference's *_pycuda / *_numba wrappers compute.
 *
 * rmw_wall_uf replaces single_wall_mobility_trans_times_force_{pycuda,numba,cpp}
 *   (mobility/mobility.py:222-252, 1132-1163, 187-219; kernel
 *    mobility/mobility_pycuda.py:150-254)
 * rmw_wall_ut replaces single_wall_mobility_trans_times_torque_{pycuda,numba}
 *   (mobility/mobility.py:427-452, 1213-1233; mobility/mobility_pycuda.py:1516-1622)
 * rmw_wall_wf replaces single_wall_mobility_rot_times_force_{pycuda,numba}
 *   (mobility/mobility.py:300-325, 1273-1298; mobility/mobility_pycuda.py:926-1031)
 * rmw_wall_wt replaces single_wall_mobility_rot_times_torque_{pycuda,numba}
 *   (mobility/mobility.py:342-367, 1316-1341; mobility/mobility_pycuda.py:593-697)
 *
 * The library keeps a per-device scratch buffer (grown on demand). */
int rmw_wall_uf(const double *r, const double *v, double *out, int64_t n, double eta, double a,
                const double *L_host, int mode, void *stream);
int rmw_wall_ut(const double *r, const double *v, double *out, int64_t n, double eta, double a,
                const double *L_host, int mode, void *stream);
int rmw_wall_wf(const double *r, const double *v, double *out, int64_t n, double eta, double a,
                const double *L_host, int mode, void *stream);
int rmw_wall_wt(const double *r, const double *v, double *out, int64_t n, double eta, double a,
                const double *L_host, int mode, void *stream);

/* Generic form of the four entry points above (kind = RMW_UF..RMW_WT). */
int rmw_wall_product(int kind, const double *r, const double *v, double *out, int64_t n, double eta,
                     double a, const double *L_host, int mode, void *stream);

/* Host-buffer form: the drop-in for the reference's pycuda wrappers, which
 * copy host arrays to the device, launch, and copy the result back on every
 * call (mobility/mobility_pycuda.py:2235-2267).  Synchronous.  Pinned or
 * pageable host memory both work. */
int rmw_wall_product_host(int kind, const double *r_host, const double *v_host, double *out_host,
                          int64_t n, double eta, double a, const double *L_host, int mode);

/* Allocation-free variant of rmw_wall_product.  No counterpart in the
 * reference: it exists for callers that cannot call cudaMalloc - a host
 * application whose device memory belongs to another allocator (a framework
 * that reserves the whole GPU up front), code that must keep its device-memory
 * footprint fixed after start-up, or a latency-sensitive loop that cannot take
 * the implicit device-wide synchronisation of cudaMalloc/cudaFree.  Arguments
 * and result are those of rmw_wall_product (device pointers; the caller still
 * provides inputs and outputs).  The scratch is a file-scope device array of
 * 16 MiB that every GPU loading the library holds until process exit, so n is
 * limited to RMW_NOALLOC_MAX_BLOBS (larger n returns RMW_ERR_ARG).  The first
 * call on a device looks up the array's device address (cudaGetSymbolAddress,
 * with that device current) and caches it; make that first call before any
 * stream capture.  All calls share the one array: calls whose work overlaps on
 * the GPU (different streams, or several host threads) race on it and must be
 * serialised by the caller.  The function calls no cudaMalloc, cudaFree or
 * other allocating routine. */
#define RMW_NOALLOC_MAX_BLOBS 180000
int rmw_wall_product_noalloc(int kind, const double *r, const double *v, double *out, int64_t n, double eta,
                             double a, const double *L_host, int mode, void *stream);

/* Measured FMA-pipe throughput of the current device (FLOP/s, FMA = 2 flops)
 * for FP64 (fp64 != 0) or FP32: the denominator of the pair kernels' roofline
 * fraction.  Synchronous.  Library-only (no reference counterpart). */
int rmw_fma_peak(int fp64, double *flops_per_s_host, void *stream);

/* Kernel tracing (library-only, no reference counterpart; the reference's
 * only profiling is the wall-clock utils.timer, general_application_utils.py:486-511).
 * While enabled, each launch of a traced kernel is bracketed by CUDA events on
 * its launching stream.  rmw_trace_read sums the durations of one kernel class
 * (0 = pair kernel, 1 = Krylov vector kernels, 2 = preconditioner) and
 * optionally clears the records.  rmw_trace_read synchronises the events. */
int rmw_trace_enable(int on);
int rmw_trace_read(int kind, double *total_ms_host, int64_t *launches_host, int reset);

#ifdef __cplusplus
}
#endif
#endif /* RMW_GB300_H */
