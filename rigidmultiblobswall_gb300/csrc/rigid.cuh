// Rigid multiblob bodies on the GPU: state of one suspension and its
// operators (geometric matrix K, block-diagonal preconditioner, saddle-point
// operator).  Used by the C ABI in rigid.cu and the Krylov solvers in krylov.cu.
#pragma once
#include <vector>

#include "rmw_common.cuh"

namespace rmw {

struct WallBatch;

struct RigidSystem {
    int nb = 0;       // bodies
    int n = 0;        // blobs
    int max_m = 0;    // largest 3 * blobs-per-body
    double eta = 1.0, a = 1.0;
    double L[3] = {0, 0, 0};
    cudaStream_t st = 0;
    int device = 0;
    std::vector<int> boff_h;       // nb+1 blob offsets (host copy)
    std::vector<long long> moff_h; // nb+1 offsets of the per-body m x m matrices
    // device arrays (owned)
    int *boff = nullptr;           // nb+1
    int *blob_body = nullptr;      // n
    long long *moff = nullptr;     // nb+1
    double *r = nullptr;           // 3n blob positions
    double *xb = nullptr;          // 3nb body locations
    double *minv = nullptr;        // sum m^2 : inverse blob mobility per body
    double *minvK = nullptr;       // sum 6m  : M^-1 K per body (row-major m x 6)
    double *nmat = nullptr;        // 36 nb   : N = (K^T M^-1 K)^-1
    double *lfac = nullptr;        // sum m^2 : Cholesky factor L (lower), stochastic PC only
    double *linv = nullptr;        // sum m^2 : L^-1 (lower), stochastic PC only
    int *dstatus = nullptr;        // device status word
    double *tmp3n = nullptr;       // 3n scratch vector
    bool pc_ready = false, stoch_ready = false;
    bool pc_fp32 = false;  // body blocks factorised in FP32 (preconditioner of the mixed solves)
    // FP32 copies of minv, minvK, nmat for the mixed solves' FP32 apply
    // (rigid_apply_pc_mixed); filled from the FP64 arrays after each build
    float *minv32 = nullptr, *minvK32 = nullptr, *nmat32 = nullptr;
    float4 *blob32 = nullptr;  // n: blob offset from its body's centre and height, FP32
    bool pc32_ready = false;
    bool pc32_blocks = false;  // the build wrote minv32, minvK32, nmat32 itself (FP32 sweep build)
    float *linv32 = nullptr;   // FP32 copy of linv after an FP32 stochastic build (multi-vector L^-1 multiplies)
    bool linv32_ready = false;
    bool wall = true;  // false: free-space (no-wall) mobility (rmw_rigid_set_wall)
    // independent suspensions inside the handle (rmw_rigid_set_suspensions):
    // segmented pair products and the instance-major permutation
    WallBatch *batch = nullptr;
    std::vector<long long> susp_body_off;  // bodies of suspension k: [off[k], off[k+1])
    std::vector<long long> susp_off;       // instance-major offsets of the system vector
    long long *perm = nullptr;             // device: instance-major index -> [lambda; U] index
    // near-field augmented preconditioner (rmw_rigid_set_nearfield): CSR
    // neighbour lists by owner body of the exact blob-level pairs and of the
    // pairs whose 11x11 mode coupling the network predicts
    bool nf_on = false;
    int nf_ex_pairs = 0, nf_ln_pairs = 0;
    int *nf_off = nullptr;                          // 3 (nb+1): the three offset arrays (owned)
    int *nf_ex_off = nullptr, *nf_ln_off = nullptr;  // views into nf_off
    int *nf_mp_off = nullptr;                       // message-passing neighbours (view into nf_off)
    int *nf_ex_idx = nullptr, *nf_ln_idx = nullptr;
    int *nf_mp_idx = nullptr;
    int nf_mp_pairs = 0;
    size_t nf_cap_mp = 0;
    int *nf_cnt = nullptr;                          // 3 nb neighbour counts
    int2 *nf_range = nullptr;                       // nb: bodies of each body's suspension
    size_t nf_cap_ex = 0, nf_cap_ln = 0;            // capacities (entries) of the per-entry arrays
    double *nf_G = nullptr;    // 121 per learned entry (lab frame)
    double *nf_mom = nullptr;  // 11 mode moments per body
    float *nf_mom32 = nullptr;  // the same moments of the FP32 apply
    float *nf_lam32 = nullptr;  // 3n: damped blob forces b lambda of the FP32 apply
    float *nf_G32 = nullptr;    // FP32 copy of nf_G
    double *nf_v = nullptr;    // sys_size: near-field blob velocities, force rows zero
    double *nf_z = nullptr;    // sys_size: second block-diagonal solve
    double *nf_part = nullptr;  // max_m per exact entry: unscaled pair velocities

    long long sys_size() const { return 3LL * n + 6LL * nb; }
};

// y = A x with A = [[M, -K], [-K^T, 0]] (multi_bodies.py:424-471); mode = RMW_MODE_*.
int rigid_apply(RigidSystem &S, const double *x, double *y, int mode);
// y = P^-1 x (block-diagonal preconditioner, multi_bodies.py:825-861, or its
// near-field augmented form when one is attached).
int rigid_apply_pc(RigidSystem &S, const double *x, double *y);
// the block-diagonal form alone
int rigid_apply_pc_plain(RigidSystem &S, const double *x, double *y);
// The same operator (plain or near-field augmented) in FP32 arithmetic, for
// the mixed-precision solves, whose inner GMRES runs on FP32 pair products and
// whose refinement residual is FP64-accurate; the FP64 form for bodies too
// large for its shared-memory layout, and inside a stream capture before
// rigid_pc_prepare_f32 has run.
int rigid_apply_pc_mixed(RigidSystem &S, const double *x, double *y);
// FP32 copies of the built preconditioner (no-op when current); call before
// capturing rigid_apply_pc_mixed into a CUDA graph.
int rigid_pc_prepare_f32(RigidSystem &S);
// allocate the FP32 copies (no-op when present)
int alloc_pc32(RigidSystem &S);
// y = L^-1 M L^-T w on the blob space (det_stoch mobility_pc, multi_bodies.py:591-606).
int rigid_mobility_pc(RigidSystem &S, const double *w, double *y, int mode);
// y = L w (det_stoch P_inv_mult, multi_bodies.py:609-615).
int rigid_P_inv_mult(RigidSystem &S, const double *w, double *y);
// nvec vectors (stride 3N) at once; tmp holds nvec * 3N doubles.  Mixed mode
// uses the multi-right-hand-side pair kernel.
// active: optional per (pass of 8 vectors, suspension) bytes of the mixed
// multi-vector product (wall_uf_multi); 0 skips that suspension's rows.
int rigid_mobility_pc_multi(RigidSystem &S, const double *W, double *Y, int nvec, int mode, double *tmp,
                            const unsigned char *active = nullptr);
int rigid_P_inv_mult_multi(RigidSystem &S, const double *W, double *Y, int nvec, int mode = RMW_MODE_FP64);
// near-field augmented preconditioner apply, nearfield.cu
int nearfield_apply_pc(RigidSystem &S, const double *x, double *y);
// M v on the handle's blobs (segmented by suspension when suspensions are set).
int rigid_mobility(RigidSystem &S, const double *v, double *y, int mode);

// Iterative refinement x <- x + d after a residual r = b - A x computed with
// the FP64-accurate operator: the next residual is either recomputed the same
// way or updated as r - A32 d with the FP32-pair operator A32.  The update
// drifts from the true residual by (A - A32) d.  The FP32-pair products are
// within 1e-6 (relative 2-norm) of FP64 and d solves A32 d = r to the inner
// tolerance, so the drift is about 1e-6 |r| for a well-conditioned
// preconditioned system.  kRecurrenceDrift = 1e-5 takes ten times that as
// the bound, and the recurrence is used only while the bound stays below a
// tenth of the tolerance: |r| / |b| <= 1e4 tol (1e-4 at tol = 1e-8).  Below
// that the double-float product of a full refinement step (the dominant cost
// of a mixed solve next to the FP32 Krylov iterations) is replaced by one
// FP32-pair product.
constexpr double kRecurrenceDrift = 1e-5;
inline bool refine_by_recurrence(double relres, double tol) { return relres * kRecurrenceDrift <= 0.1 * tol; }

}  // namespace rmw
