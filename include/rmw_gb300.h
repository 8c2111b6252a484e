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
                            compensated per-target accumulation, FP64 output;
                            relative error <= 1e-6 against FP64 */
#define RMW_MODE_DF64 2  /* double-float (hi+lo FP32 pairs, ~48-bit) pair
                            evaluation on the FP32 pipe with FP64 accumulation;
                            relative error <= 1e-12 against FP64 */

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

/* Segmented products of many independent suspensions in one launch:
 * suspension k owns blobs [blob_offsets[k], blob_offsets[k+1]) of one (N,3)
 * array and interacts only with itself (block-diagonal mobility).  The batch
 * handle holds the CTA job table; no reference counterpart (the reference
 * loops over systems one call at a time). */
int rmw_wall_batch_create(void **handle, int64_t n_suspensions, const int64_t *blob_offsets_host);
int rmw_wall_batch_destroy(void *handle);
int rmw_wall_product_batched(void *handle, int kind, const double *r, const double *v, double *out, double eta,
                             double a, int mode, void *stream);

/* M_UF applied to nrhs vectors at once (V and Y: nrhs rows of 3n doubles),
 * mixed precision (<= 1e-6): each pair block is formed once and applied to
 * every vector of a pass (16 vectors per pass).  batch may be NULL or a rmw_wall_batch_create handle
 * (segmented).  Serves multi-right-hand-side Lanczos; no reference
 * counterpart. */
int rmw_wall_uf_multi(const double *r, const double *V, double *Y, int64_t n, int nrhs, double eta, double a,
                      void *batch, void *stream);

/* Host-buffer form: the drop-in for the reference's pycuda wrappers, which
 * copy host arrays to the device, launch, and copy the result back on every
 * call (mobility/mobility_pycuda.py:2235-2267).  Synchronous.  Pinned or
 * pageable host memory both work. */
int rmw_wall_product_host(int kind, const double *r_host, const double *v_host, double *out_host,
                          int64_t n, double eta, double a, const double *L_host, int mode);

/* Free-space (no-wall) RPY products out = M_kind v, kind = RMW_UF .. RMW_WT:
 * the reference's no_wall_mobility_{trans_times_force, trans_times_torque,
 * rot_times_force, rot_times_torque}_{pycuda,numba} (mobility/mobility.py:
 * 288-482, kernels mobility/mobility_numba.py:13-1190).  Positions are used
 * as given (no wall, no regularisation); periodic images, modes, device
 * pointers and errors as rmw_wall_product. */
int rmw_nowall_product(int kind, const double *r, const double *v, double *out, int64_t n, double eta, double a,
                       const double *L_host, int mode, void *stream);

/* Source-target translational products with per-blob radii: velocities
 * out (3 n_target) of target blobs of radii radius_target from forces
 * (3 n_source) on source blobs of radii radius_source, with the
 * unequal-sphere RPY pair block.  geometry:
 *   RMW_GEOM_NO_WALL       no_wall_mobility_trans_times_force_source_target_numba
 *                          (mobility/mobility.py:593-616, kernel
 *                          mobility/mobility_numba.py:1480-1572)
 *   RMW_GEOM_WALL          single_wall_mobility_trans_times_force_source_target_{numba,pycuda}
 *                          (mobility.py:494-590: heights shifted to max(z, radius),
 *                          forces and velocities damped by z / radius, image
 *                          system of mobility_numba.py:1573-1653)
 *   RMW_GEOM_FREE_SURFACE  free_surface_mobility_trans_times_force_source_target_numba
 *                          (mobility.py:1409-1429, mobility_numba.py:1941-2093)
 * Every radius must be positive.  Periodic images (L_host, may be NULL) and
 * precision modes as rmw_wall_product; device arrays; asynchronous. */
#define RMW_GEOM_NO_WALL 0
#define RMW_GEOM_WALL 1
#define RMW_GEOM_FREE_SURFACE 2
int rmw_source_target_product(int geometry, const double *source, const double *target, const double *force,
                              const double *radius_source, const double *radius_target, int64_t n_source,
                              int64_t n_target, double eta, const double *L_host, int mode, double *out,
                              void *stream);

/* Free-surface product out = M f of n blobs of radius a (the mirror image
 * with diag(1, 1, -1) instead of the wall's image system):
 * free_surface_mobility_trans_times_force_{numba,pycuda} (mobility/mobility.py:
 * 533-548, 1390-1406, kernel mobility/mobility_numba.py:1770-1938).  Periodic
 * images and modes as rmw_wall_product; device arrays; asynchronous. */
int rmw_free_surface_product(const double *r, const double *force, double *out, int64_t n, double eta, double a,
                             const double *L_host, int mode, void *stream);

/* Dense translational blob mobility M (row-major 3n x 3n, FP64) of n <= 65535
 * blobs: wall = 1 single_wall_fluid_mobility (mobility/mobility.py:1018-1116,
 * shifted heights and damping), wall = 0 rotne_prager_tensor
 * (mobility/mobility.py:967-1015).  Device arrays; asynchronous. */
int rmw_dense_mobility(int wall, const double *r, double *M, int64_t n, double eta, double a, void *stream);

/* Rollers driven at a prescribed angular velocity: the torques solve
 * M_WT torque = omega - M_WF force (unpreconditioned restarted GMRES from
 * zero to the relative tolerance tol), then velocity = M_UF force +
 * M_UT torque - QuaternionIntegratorRollers.compute_deterministic_velocity_and_torque
 * (quaternion_integrator/quaternion_integrator_rollers.py:905-983).  wall = 1
 * single-wall products, 0 free space; mode applies to every product.  Device
 * arrays of 3n doubles; synchronous; RMW_ERR_NOT_CONVERGED (results still
 * written) when maxiter is reached. */
int rmw_rollers_velocity_and_torque(const double *r, const double *force, const double *omega, double *velocity,
                                    double *torque, int64_t n, double eta, double a, const double *L_host, int wall,
                                    double tol, int restart, int maxiter, int mode, void *stream, int *iters_host,
                                    double *relres_host);

/* Blob forces (the mobility problem's right-hand side), device arrays of 3n
 * doubles; accumulate != 0 adds to f instead of overwriting it.
 * rmw_blob_blob_forces: soft repulsion of multi_bodies/forces_pycuda.py:40-118
 * (Python form multi_bodies/multi_bodies_functions.py:297-345), all pairs
 * (cutoff <= 0) or the pairs within `cutoff` (the neighbour-list variant of
 * multi_bodies/forces_numba.py:228-270 uses 2a + 30 b), minimum periodic
 * image (L_host may be NULL).
 * rmw_blob_external_forces: gravity and wall repulsion of
 * multi_bodies/multi_bodies_functions.py:153-189.  Body forces and torques
 * follow with rmw_rigid_KT_mult (the reduction of
 * force_torque_calculator_sort_by_bodies, multi_bodies_functions.py:411-445). */
int rmw_blob_blob_forces(const double *r, double *f, int64_t n, double repulsion_strength, double debye_length,
                         double blob_radius, double cutoff, const double *L_host, int accumulate, void *stream);
int rmw_blob_external_forces(const double *r, double *f, int64_t n, double blob_mass, double blob_radius, double g,
                             double repulsion_strength_wall, double debye_length_wall, int accumulate, void *stream);

/* Fused force-and-torque product: U = M_UF F + M_UT T and, if W != NULL,
 * W = M_WF F + M_WT T, in one pass over the pairs (the four blocks share
 * each pair's geometry).  U alone replaces
 * single_wall_mobility_trans_times_force_torque_pycuda (mobility/mobility.py:
 * 384-411, kernel mobility/mobility_pycuda.py:1266-1392); [U; W] replaces the
 * four products of Lub_Solver.Wall_Mobility_Mult (Lubrication/Lub_Solver.py:
 * 277-305).  Device arrays of 3n doubles; same regularisation, periodic
 * images, modes and errors as rmw_wall_product. */
int rmw_wall_force_torque(const double *r, const double *F, const double *T, double *U, double *W, int64_t n,
                          double eta, double a, const double *L_host, int mode, void *stream);

/* Launch-shape autotuner (no reference counterpart): times every admissible
 * source split of the all-pairs grid (and, where it applies, the symmetric
 * kernel, reported as nchunks = -1) on n synthetic blobs and caches the
 * fastest for (device, kind, mode, n's quarter-octave size bucket); the
 * product entry points above and the rigid-body operators then use it.
 * Synchronous.  best_ms / default_ms: mean time of the chosen split and of
 * the built-in rule's. */
int rmw_wall_autotune(int kind, int mode, int64_t n, int reps, void *stream, int *best_nchunks, double *best_ms,
                      double *default_ms);
int rmw_wall_autotune_lookup(int kind, int mode, int64_t n, int *nchunks, int *tuned);
/* Pin a choice instead of measuring: nchunks in [1, 64], or -1 for the
 * symmetric kernel of any block and precision mode (each unordered pair
 * evaluated once and applied both ways; non-periodic, n >= 256; its
 * deterministic partial sums take ceil(n/128) x 3n doubles, 5.5 GB at
 * 172,032 blobs, within an eighth of the device memory and at least 6 GiB:
 * about 430,000 blobs on a 284 GB device).  Without a tuned or pinned
 * choice the products use the symmetric kernel from 4,096 blobs in FP64 and
 * df64 and from 8,192 in mixed precision. */
int rmw_wall_autotune_set(int kind, int mode, int64_t n, int nchunks);
/* Library-only (no reference counterpart): how a product of (kind, mode, n)
 * runs on the current device - 0 the one-sided kernel, 1 the symmetric kernel
 * (each unordered pair once; ceil(n/128) x 3n doubles of partial sums), 2 the
 * symmetric df64 kernel band by band of tile rows, when those partial sums
 * exceed the budget (an eighth of the device memory, or the scratch cap):
 * about 3 x 128 doubles per blob and tile row of a band, bands summed in a
 * fixed order. */
int rmw_wall_product_route(int kind, int mode, int64_t n, const double *L_host, int *route_host);
int rmw_wall_autotune_clear(void);

/* CUDA graphs (no reference counterpart): the solvers' per-iteration
 * operators (A P^-1 of rmw_rigid_solve / rmw_rigid_solve_batched, the
 * preconditioned mobility of the Lanczos entry points) are captured once per
 * call and replayed as one graph launch per application.  on = 0 runs them
 * as plain launches.  Stats: graphs captured and replayed since the last
 * reset. */
int rmw_use_graphs(int on);
/* Device-resident GMRES (no reference counterpart; the reference's GMRES is
 * scipy's host loop, general_application_utils.py:514-635): the rigid solves
 * (rmw_rigid_solve, rmw_rigid_solve_batched) run each restart cycle on the
 * device - operator applications and a fused cooperative Arnoldi step kernel
 * (CGS2, Givens rotations, stopping test) repeated by a CUDA graph while node,
 * one host round trip per cycle.  on = 0 selects the host-driven loop (one
 * round trip per Arnoldi step).  Default on; devices without cooperative
 * launches use the host-driven loop. */
int rmw_use_device_krylov(int on);
int rmw_graph_stats(int64_t *captures_host, int64_t *replays_host, int reset);

/* ---- rigid multiblob bodies ------------------------------------------
 * A handle (opaque, void*) holds one suspension of rigid bodies: body b owns
 * blobs [blob_offsets[b], blob_offsets[b+1]) (the reference's bodies list in
 * order, multi_bodies/multi_bodies.py:194-204).  Vectors of the saddle-point
 * system are [lambda (3N); U (6 Nb)] with U_b = (velocity, angular velocity),
 * the layout of linear_operator_rigid (multi_bodies.py:424-471).  The handle
 * is bound to the stream it was created with; all device arrays are owned by
 * the caller except the handle's own copies. */

/* Create a handle (blob_offsets_host: n_bodies + 1 entries, starting at 0). */
int rmw_rigid_create(void **handle, int64_t n_bodies, const int64_t *blob_offsets_host, double eta, double a,
                     const double *L_host, void *stream);
int rmw_rigid_destroy(void *handle);
int rmw_rigid_sizes(void *handle, int64_t *n_blobs_host, int64_t *n_bodies_host);
/* Copy blob positions r (N,3) and body locations x (Nb,3) (device pointers)
 * into the handle; invalidates the preconditioner
 * (body/body.py:64-78 get_r_vectors gives r from location + orientation). */
int rmw_rigid_set_configuration(void *handle, const double *r_blobs, const double *x_bodies);
/* Block-diagonal preconditioner: per body the dense wall mobility, its
 * Cholesky factor, inverse and N = (K^T M^-1 K)^-1.  Replaces
 * build_block_diagonal_preconditioner (multi_bodies.py:752-903); with
 * stochastic != 0 also keeps L and L^-1, replacing
 * build_block_diagonal_preconditioners_det_stoch (multi_bodies.py:480-618).
 * Synchronous; RMW_ERR_NONFINITE if a body matrix is not positive definite. */
int rmw_rigid_build_pc(void *handle, int stochastic);
/* The same for the solves of one precision mode: RMW_MODE_MIXED factorises the
 * body blocks on the FP32 pipe (FP64 runs at 1/64 of its rate on GB300) - an
 * equally valid block-diagonal preconditioner, convergence still decided by the
 * FP64-accurate residual; a block that is not positive definite in FP32 makes
 * it fall back to FP64.  RMW_MODE_FP64 / RMW_MODE_DF64: rmw_rigid_build_pc.
 * Solves and Lanczos in FP64 or df64 rebuild an FP32-factorised one. */
int rmw_rigid_build_pc_mode(void *handle, int stochastic, int mode);
/* y = [[M, -K], [-K^T, 0]] x  (linear_operator_rigid, multi_bodies.py:424-471). */
int rmw_rigid_apply(void *handle, const double *x, double *y, int mode);
/* y = P^-1 x  (block_diagonal_preconditioner apply, multi_bodies.py:825-861). */
int rmw_rigid_apply_pc(void *handle, const double *x, double *y);
/* The same apply as the solves of one precision mode run it (same operator as
 * multi_bodies.py:825-861, plus the attached near-field augmentation): FP64 for
 * RMW_MODE_FP64 / RMW_MODE_DF64; FP32 arithmetic on FP32 copies of the body
 * blocks for RMW_MODE_MIXED (~1e-7 relative: the mixed solves refine with an
 * FP64-accurate residual, so their preconditioner needs no FP64 arithmetic). */
int rmw_rigid_apply_pc_mode(void *handle, const double *x, double *y, int mode);
/* y = L^-1 M L^-T w on the 3N blob space (det_stoch mobility_pc, multi_bodies.py:591-606). */
int rmw_rigid_mobility_pc(void *handle, const double *w, double *y, int mode);
/* y = L w  (det_stoch P_inv_mult, multi_bodies.py:609-615). */
int rmw_rigid_P_inv_mult(void *handle, const double *w, double *y);
/* out (3N) = K u (u: 6 Nb)  (K_matrix_vector_prod, multi_bodies.py:328-347). */
int rmw_rigid_K_mult(void *handle, const double *u, double *out);
/* out (6 Nb) = K^T lambda  (K_matrix_T_vector_prod, multi_bodies.py:350-371). */
int rmw_rigid_KT_mult(void *handle, const double *lambda, double *out);
/* Dense per-body wall mobility blocks, bodies concatenated (each 3n_b x 3n_b,
 * row-major): Body.calc_mobility_blobs with single_wall_fluid_mobility
 * (body/body.py:186-191, mobility/mobility.py:1018-1116). */
int rmw_rigid_body_mobility(void *handle, double *out);
/* r_out (N,3) = R(q_b) r_ref + x_b for every blob: r_ref (N,3) body-frame
 * blob coordinates, q (Nb,4) quaternions (s, p), x (Nb,3) locations
 * (Body.get_r_vectors, body/body.py:64-78; Quaternion.rotation_matrix,
 * quaternion_integrator/quaternion.py:42-51). */
int rmw_rigid_blob_positions(void *handle, const double *x_bodies, const double *q_bodies, const double *r_ref,
                             double *r_out);
/* Euler-Maruyama body update x_new = x + U dt, q_new = from_rotation(w dt) q
 * with velocities (Nb,6) = (U, w) per body
 * (quaternion_integrator_multi_bodies.py:308-312, quaternion.py:16-39). */
int rmw_rigid_euler_update(void *handle, const double *x_bodies, const double *q_bodies, const double *velocities,
                           double dt, double *x_new, double *q_new);
/* Number of blobs with z < zmin (the wall check of Body.check_function,
 * body/body.py:118-140).  Synchronous. */
int rmw_count_below(const double *r, int64_t n, double zmin, int *count_host, void *stream);
/* Right-preconditioned restarted GMRES on the saddle-point system with the
 * block-diagonal preconditioner (zero initial guess), stopping when the true
 * residual |b - A x| <= tol |b|: utils.gmres as called by
 * solve_mobility_problem (general_application_utils.py:514-635,
 * quaternion_integrator_multi_bodies.py:1441-1547).  mode RMW_MODE_FP64 or
 * RMW_MODE_DF64 selects the operator's pair arithmetic; RMW_MODE_MIXED runs the
 * inner GMRES on the FP32-pair operator inside iterative refinement whose
 * residual uses the FP64-accurate double-float operator.
 * Synchronous.  Returns RMW_ERR_NOT_CONVERGED after maxiter iterations (the
 * best iterate is still written to sol). */
int rmw_rigid_solve(void *handle, const double *rhs, double *sol, double tol, int restart, int maxiter, int mode,
                    int *iters_host, double *relres_host);
/* rmw_rigid_solve on the right-hand side scaled to unit norm, the solution
 * scaled back: solve_mobility_problem's normalisation
 * (quaternion_integrator_multi_bodies.py:1519-1537).  A zero rhs gives a zero
 * solution without GMRES.  Returns after the solve (the last scaling is queued
 * on the handle's stream); the codes are rmw_rigid_solve's. */
int rmw_rigid_solve_scaled(void *handle, const double *rhs, double *sol, double tol, int restart, int maxiter,
                           int mode, int *iters_host, double *relres_host);
/* noise = factor * L (L^-1 M L^-T)^(1/2) z by Lanczos: stochastic_forcing_lanczos
 * with mobility_mult = mobility_pc and L_mult = P_inv_mult
 * (stochastic_forcing/stochastic_forcing.py:112-264), z and noise 3N device
 * vectors.  Synchronous. */
int rmw_rigid_lanczos(void *handle, const double *z, double *noise, double factor, double tol, int max_iter,
                      int mode, int *iters_host);
/* noise = factor * M^(1/2) z for the wall mobility of n free blobs (Lanczos
 * without preconditioner).  Synchronous. */
int rmw_wall_lanczos(const double *r, const double *z, double *noise, int64_t n, double eta, double a,
                     const double *L_host, double factor, double tol, int max_iter, int mode, void *stream,
                     int *iters_host);

/* Wall (1, default) or free space (0) for every mobility of the handle: blob
 * products, the preconditioners' dense per-body blocks, solves and Lanczos.
 * Free space is the reference's *_no_wall implementations (mobility/mobility.py:
 * 288-482; dense rotne_prager_tensor, :967-1015), as selected by
 * mobility_blobs_implementation = 'python_no_wall' and
 * mobility_vector_prod_implementation = 'pycuda_no_wall'
 * (multi_bodies/multi_bodies.py:207-287).  Invalidates the preconditioners;
 * batched suspensions and the near-field preconditioner are wall-only. */
int rmw_rigid_set_wall(void *handle, int wall);

/* Declare that the handle's bodies form independent suspensions: suspension
 * k owns bodies [body_offsets[k], body_offsets[k+1]) and its blobs interact
 * only with each other (segmented pair products).  Enables the batched
 * solver.  No reference counterpart: the reference solves one suspension per
 * process. */
int rmw_rigid_set_suspensions(void *handle, int64_t n_suspensions, const int64_t *body_offsets_host);
/* Solve every suspension of the handle with its own right-preconditioned
 * restarted GMRES (own Krylov space, tolerance, iteration count) in lockstep:
 * one operator and preconditioner application per step for all suspensions.
 * rhs/sol use the [lambda; U] layout; iters/relres/status_host receive one
 * entry per suspension.  mode as rmw_rigid_solve (MIXED refines per
 * suspension).  Synchronous; returns RMW_OK when every suspension converged. */
int rmw_rigid_solve_batched(void *handle, const double *rhs, double *sol, double tol, int restart, int maxiter,
                            int mode, int *iters_host, double *relres_host, int *status_host);

/* Lanczos Brownian noise for nrhs right-hand sides of every suspension:
 * noise_q = factor * L (L^-1 M L^-T)^(1/2) z_q per suspension (the det_stoch
 * preconditioned stochastic_forcing_lanczos, stochastic_forcing.py:112-264),
 * all (suspension, right-hand side) recurrences in lockstep with one
 * multi-right-hand-side operator application per step.  Z, noise: nrhs rows
 * of 3N doubles.  iters_host: nrhs * n_suspensions entries.  The basis is
 * capped at 96 vectors.  Synchronous. */
int rmw_rigid_lanczos_batched(void *handle, const double *Z, double *noise, int nrhs, double factor, double tol,
                              int max_iter, int mode, int *iters_host);

/* ---- near-field augmented preconditioner (no reference counterpart) ----
 * The block-diagonal preconditioner (rmw_rigid_build_pc) drops every
 * inter-body blob block of M.  The augmented form adds the first Neumann term
 * of the near blocks: y = P0 x, v_i = sum_{j near i} M_ij lambda_j(y),
 * y <- y - P0 [v; 0].  Pairs closer than an exact cutoff use the blob-level
 * blocks; pairs in the learned band use the 11x11 coupling of the bodies'
 * low-order modes (3 translations, 3 rotations, 5 strains) that a
 * message-passing network predicts: body embeddings from (z/R, neighbour
 * count), three rounds of messages between bodies closer than the message
 * cutoff (3R by default), and a readout per learned pair from both
 * embeddings and the pair's (horizontal distance, z_i, z_j)/R; width 64,
 * SiLU, BF16 weights and activations, FP32 accumulation on the tensor cores
 * in the forward and the backward pass. */
/* 11x11 mode couplings G_01, G_10 (lab frame, row-major; 242 doubles per
 * sample) of every pair of handle bodies (2s, 2s+1); call after
 * rmw_rigid_build_pc.  Training data. */
int rmw_rigid_pair_coupling(void *handle, double *out);
/* The same coupling G_ij (lab frame, 121 doubles each) for n_pairs arbitrary
 * ordered pairs (pairs: 2 n_pairs ints on the device, (i, j) per pair) of the
 * handle's bodies: the targets of few-body training clusters.  Synchronous. */
int rmw_rigid_pair_coupling_list(void *handle, const int *pairs, int64_t n_pairs, double *out);

/* A graph for the message-passing network (device arrays, int32 indices).
 * Nodes are bodies; node_feat holds (z/R, degree/8) per node.  Message edges
 * (dst <- src) are sorted by dst with CSR offsets mp_off (n_nodes + 1) and
 * mp_rev[e] = the index of the reverse edge; band edges (i <- j), whose
 * coupling G_ij is predicted, are sorted by i with band_off and band_rev.
 * Edge features: (horizontal distance, z_dst, z_src)/R.  target: n_band x 121
 * couplings in each pair's frame (x axis along the horizontal separation),
 * training only; the reverse-edge arrays are needed for training only. */
typedef struct {
    int32_t n_nodes, n_mp, n_band;
    const float *node_feat;
    const int32_t *mp_src, *mp_dst, *mp_off, *mp_rev;
    const float *mp_feat;
    const int32_t *band_i, *band_j, *band_off, *band_rev;
    const float *band_feat;
    const float *target;
} rmw_graph;

int rmw_nearfield_create(void **net, double body_radius, double cutoff, unsigned long long seed);
int rmw_nearfield_destroy(void *net);
/* the message cutoff (default 3R) and the learned band's outer cutoff */
int rmw_nearfield_set_cutoffs(void *net, double mp_cutoff, double cutoff);
int rmw_nearfield_sizes(int *n_weights, int *n_biases, int *n_norm, int *width, int *n_out, int *n_target);
int rmw_nearfield_get(void *net, float *w_host, float *b_host, float *norm_host);
int rmw_nearfield_set(void *net, const float *w_host, const float *b_host, const float *norm_host);
/* forward pass on one graph: out (device) n_band x 121 normalised outputs
 * (multiply by the target scale of the normalisation block for G) */
int rmw_nearfield_forward(void *net, const rmw_graph *graph, float *out, void *stream);
/* gradients of the mean squared error on normalised targets (host outputs) */
int rmw_nearfield_grad(void *net, const rmw_graph *graph, float *gW_host, float *gb_host, float *loss_host);
/* Adam over the graphs (one per step, cycling), after setting the
 * normalisation from their features and targets.  Synchronous. */
int rmw_nearfield_train(void *net, const rmw_graph *graphs, int n_graphs, int steps, float lr, float *loss_host,
                        void *stream);
/* Switch a handle's preconditioner (after rmw_rigid_build_pc) to the
 * augmented form: exact couplings below exact_cutoff, learned ones from there
 * to the network's cutoff (net may be NULL).  net == NULL with exact_cutoff <= 0
 * restores the block-diagonal form.  n_pairs_host (optional): 2 entries,
 * ordered exact and learned pair counts.  Synchronous. */
int rmw_rigid_set_nearfield(void *handle, void *net, double exact_cutoff, int64_t *n_pairs_host);
/* The same with the learned band starting at max(learned_from, exact_cutoff):
 * learned_from = exact_cutoff = 0 learns every pair below the network's
 * cutoff; exact_cutoff = 0 < learned_from learns only the outer band. */
int rmw_rigid_set_nearfield_bands(void *handle, void *net, double exact_cutoff, double learned_from,
                                  int64_t *n_pairs_host);

/* ---- generic Krylov solvers with caller-supplied operators ------------
 * op(ctx, x, y) must write y = A x for device vectors of length n, enqueue its
 * work on the solver's stream (or finish it before returning) and return 0 on
 * success.  These serve the reference's generic entry points, whose operators
 * are arbitrary callables. */
typedef int (*rmw_operator_fn)(void *ctx, const double *x, double *y);
/* Right-preconditioned restarted GMRES (pc may be NULL: no preconditioner),
 * zero initial guess, stop on the true residual |b - A x| <= tol |b|:
 * general_application_utils.gmres (general_application_utils.py:514-635).
 * history_host (optional, history_cap entries) receives the relative residual
 * estimate of every iteration.  Synchronous. */
int rmw_gmres(int64_t n, rmw_operator_fn op, void *op_ctx, rmw_operator_fn pc, void *pc_ctx, const double *b,
              double *x, double tol, int restart, int maxiter, void *stream, int *iters_host, double *relres_host,
              double *history_host, int history_cap);
/* noise = factor * A^(1/2) z by Lanczos with one full reorthogonalisation
 * pass per step: stochastic_forcing_lanczos (stochastic_forcing.py:112-264)
 * without L_mult.  Synchronous. */
int rmw_lanczos(int64_t n, rmw_operator_fn op, void *op_ctx, const double *z, double *noise, double factor,
                double tol, int max_iter, void *stream, int *iters_host);

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

/* Scratch memory (library-only, no reference counterpart).  Products keep
 * their packed sources and partial sums in a device buffer per (device,
 * stream, purpose) that grows on demand and is kept until process exit or
 * rmw_release_scratch, so a process holds at most a few such buffers per
 * stream it calls the library on.  The symmetric pair kernels need
 * ceil(n/128) * 3n doubles of partial sums (21.7 MB at 10,752 blobs, 5.5 GB at
 * 172,032); buffers of 1 GiB and more are allocated without headroom.
 * rmw_set_scratch_limit caps one buffer at `bytes` (0 = no cap): a product
 * whose symmetric partial sums would exceed it runs the one-sided kernels,
 * whose scratch is a few hundred bytes per blob, and a request still above the
 * cap returns RMW_ERR_ALLOC.  rmw_release_scratch frees the current device's
 * buffers (after the device is idle); buffers a live CUDA graph may use are
 * freed when the last graph is destroyed. */
int rmw_set_scratch_limit(int64_t bytes);
int rmw_release_scratch(void);

/* Measured FMA-pipe throughput of the current device (FLOP/s, FMA = 2 flops)
 * for FP64 (fp64 != 0) or FP32: the denominator of the pair kernels' roofline
 * fraction.  Synchronous.  Library-only (no reference counterpart). */
int rmw_fma_peak(int fp64, double *flops_per_s_host, void *stream);

/* Kernel tracing (library-only, no reference counterpart; the reference's
 * only profiling is the wall-clock utils.timer, general_application_utils.py:486-511).
 * While enabled, each launch of a traced kernel is bracketed by CUDA events on
 * its launching stream.  rmw_trace_read sums the durations of one class
 * (0 = pair kernel, 1 = Krylov vector work, 2 = preconditioner apply - these
 * three for direct launches only -, 3 = one Krylov operator application
 * A P^-1 or the Lanczos operator, graph replay or direct, 4 = a mixed solve's
 * refinement residual, 5 = preconditioner build, 6 = whole solve calls, host
 * gaps included) and optionally clears that class's records.  rmw_trace_read
 * synchronises the events. */
int rmw_trace_enable(int on);
int rmw_trace_read(int kind, double *total_ms_host, int64_t *launches_host, int reset);
/* Algorithmic bytes the traced work of one class moved while tracing was on
 * (kind 1: the GMRES Arnoldi orthogonalisation, (4j + 12) n doubles at step j). */
int rmw_trace_bytes(int kind, double *bytes_host, int reset);

#ifdef __cplusplus
}
#endif
#endif /* RMW_GB300_H */
