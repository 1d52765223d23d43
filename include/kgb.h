/*
 * kgb.h -- C ABI of kripke_gb300, the GB300 (sm_103a) implementation of
 * Kripke's source-iteration hot path.
 *
 * One context = one GPU, one CUDA stream, and the device-resident fields of
 * one Kripke problem.  Fields are named exactly as in Kripke's DataStore and
 * move across the ABI in Kripke's own host layout: the concatenation of the
 * field's per-subdomain chunks, in chunk order, each chunk in the nesting
 * (DGZ..ZGD) given to kgb_setup.  On the device every field lives in one
 * GPU-chosen nesting (zone-major, direction fastest: "ZGD" over the whole
 * problem) and is transposed on upload and download.
 *
 * Every entry point returns a kgb_status (KGB_OK = 0) and never throws or
 * aborts; kgb_last_error() describes the most recent failure on a context.
 * All work is queued on the context's stream; only the calls that hand a
 * host value back (population, balance, solve, download, sync) wait for it.
 *
 * Reference interfaces replaced (paths relative to the Kripke source tree):
 *   Kripke::Kernel::LTimes          src/Kripke/Kernel.h:22   -> kgb_ltimes
 *   Kripke::Kernel::LPlusTimes      src/Kripke/Kernel.h:19   -> kgb_lplustimes
 *   Kripke::Kernel::scattering      src/Kripke/Kernel.h:28   -> kgb_scattering
 *   Kripke::Kernel::source          src/Kripke/Kernel.h:31   -> kgb_source
 *   Kripke::Kernel::sweepSubdomain  src/Kripke/Kernel.h:34   -> kgb_sweep_subdomain
 *   Kripke::Kernel::population      src/Kripke/Kernel.h:25   -> kgb_population
 *   Kripke::Kernel::kConst          src/Kripke/Kernel.h:37-55 -> kgb_field_fill
 *   Kripke::SweepSolver             src/Kripke/SweepSolver.h:20-22 -> kgb_sweep_solver
 *   Kripke::SteadyStateSolver       src/Kripke/SteadyStateSolver.h:18 -> kgb_solve
 *   Core::Field chunk storage       src/Kripke/Core/Field.h:53-104 -> kgb_field_upload/download
 *   Kripke::generateProblem         src/Kripke/Generate.h:20-21 -> kgb_generate
 *   Kripke::Core::Set sizes / PartitionSpace (one rank)
 *                                   src/Kripke/Core/Set.h:23-202, Core/PartitionSpace.h:35-88 -> kgb_setup
 */
#ifndef KGB_H
#define KGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum kgb_status {
  KGB_OK = 0,
  KGB_ERR_ARG = 1,      /* bad argument, size or name */
  KGB_ERR_CUDA = 2,     /* a CUDA runtime call failed */
  KGB_ERR_OOM = 3,      /* device or host allocation failed */
  KGB_ERR_TIMEOUT = 4,  /* a bounded device-side wait gave up */
  KGB_ERR_LAYOUT = 5,   /* unknown nesting */
  KGB_ERR_STATE = 6     /* call out of order (e.g. kernel before kgb_setup) */
} kgb_status;

/* Nestings, longest stride first (src/Kripke/ArchLayout.h:92-101). */
typedef enum kgb_layout {
  KGB_LAYOUT_DGZ = 0, KGB_LAYOUT_DZG = 1, KGB_LAYOUT_GDZ = 2,
  KGB_LAYOUT_GZD = 3, KGB_LAYOUT_ZDG = 4, KGB_LAYOUT_ZGD = 5
} kgb_layout;

/* Precision forms. */
typedef enum kgb_precision {
  KGB_FP64 = 0,   /* plain form: every kernel in FP64 (the drop-in) */
  KGB_MIXED = 1   /* FP32 state and sweep, FP32 GEMM-shaped kernels, FP64 reductions */
} kgb_precision;

typedef struct kgb_ctx kgb_ctx;

/* Problem shape: InputVariables sizes and the on-rank decomposition
 * (src/Kripke/InputVariables.h:18-49, Generate/Decomp.cpp:35-48). */
typedef struct kgb_dims {
  int32_t nx, ny, nz;            /* global zones */
  int32_t num_groups;
  int32_t num_directions;
  int32_t legendre_order;
  int32_t num_groupsets;         /* --gset */
  int32_t num_dirsets;           /* --dset */
  int32_t num_zonesets[3];       /* --zset */
  int32_t layout;                /* kgb_layout of the host-side chunks */
  int32_t precision;             /* kgb_precision */
} kgb_dims;

/* --- lifecycle --------------------------------------------------------- */
int kgb_ctx_create(int device, kgb_ctx **out);
int kgb_ctx_destroy(kgb_ctx *ctx);
const char *kgb_last_error(const kgb_ctx *ctx);
/* Library version string, e.g. "kripke_gb300 0.1 sm_103a". */
const char *kgb_version(void);

/* Allocates every device field for this shape (contents zero). */
int kgb_setup(kgb_ctx *ctx, const kgb_dims *dims);
/* Number of PQR subdomains (= gset * dset * zset_x * zset_y * zset_z). */
int kgb_num_subdomains(const kgb_ctx *ctx, int32_t *out);

/* --- problem generation (Kripke::generateProblem) ---------------------
 * InputVariables (src/Kripke/InputVariables.h:18-49) plus the generator
 * options of the benchmark problems.  kgb_generate calls kgb_setup with the
 * matching dims and uploads every input field the hot path reads, generated
 * as src/Kripke/Generate/{Quadrature,Space,Data,Energy}.cpp do. */
typedef struct kgb_input {
  int32_t nx, ny, nz;
  int32_t num_directions;
  int32_t num_groups;
  int32_t legendre_order;
  int32_t quad_num_polar;        /* 0: the reference's dummy S2 set (--quad N) */
  int32_t quad_num_azimuthal;    /* >0 with quad_num_polar: Gauss-Legendre product set */
  int32_t num_groupsets;
  int32_t num_dirsets;
  int32_t num_zonesets[3];
  int32_t layout;
  int32_t precision;
  int32_t num_material_subsamples;
  int32_t geometry;              /* 0: Kobayashi 3i (reference); 1: 100 cm cube, first duct leg only */
  int32_t scatter;               /* 0: diagonal P0 (reference); 1: seeded lower-triangular downscatter,
                                    columns summing to (sigs[m] / sigt[m]) * sigma_t(m, g') */
  int32_t perturb;               /* 1: seeded uniform +-20% per (material, group) on sigma_t, sigma_s */
  int32_t pad_;
  uint64_t seed;
  double sigt[3];
  double sigs[3];
} kgb_input;
/* The reference defaults (src/Kripke/InputVariables.cpp:17-47). */
void kgb_default_input(kgb_input *in);
int kgb_generate(kgb_ctx *ctx, const kgb_input *in);

/* --- fields (Core::Field chunks, Kripke DataStore names) ---------------
 * Names: psi rhs phi phi_out i_plane j_plane k_plane ell ell_plus sigt_zonal
 * data/sigs quadrature/{xcos,ycos,zcos,w,id,jd,kd} dx dy dz volume
 * zone_to_mixelem zone_to_num_mixelem mixelem_to_zone mixelem_to_material
 * mixelem_to_fraction moment_to_legendre.
 * Element type: int32 for the id/jd/kd, zone/mixelem/material and
 * moment_to_legendre maps, double for everything else.  nbytes must equal
 * the field's full size; kgb_field_bytes reports it (mixed-element fields are
 * sized by the uploaded zone_to_num_mixelem, so upload that map first). */
int kgb_field_bytes(kgb_ctx *ctx, const char *name, int64_t *nbytes);
int kgb_field_upload(kgb_ctx *ctx, const char *name, const void *host, int64_t nbytes);
int kgb_field_download(kgb_ctx *ctx, const char *name, void *host, int64_t nbytes);
/* Kripke::Kernel::kConst over every chunk of a state field. */
int kgb_field_fill(kgb_ctx *ctx, const char *name, double value);

/* --- the hot path (Kripke::Kernel::*) ----------------------------------
 * Same semantics as the reference: LTimes accumulates into phi, LPlusTimes
 * into rhs, scattering into phi_out, source adds the isotropic source of
 * material 0 to moment 0 of phi_out.  The caller zeroes targets with
 * kgb_field_fill exactly as SteadyStateSolver does. */
int kgb_ltimes(kgb_ctx *ctx);
int kgb_lplustimes(kgb_ctx *ctx);
int kgb_scattering(kgb_ctx *ctx);
int kgb_source(kgb_ctx *ctx, double source_strength);
/* Sweeps one subdomain: reads its incoming i/j/k planes and overwrites them
 * with the outgoing ones, like Kernel::sweepSubdomain. */
int kgb_sweep_subdomain(kgb_ctx *ctx, int32_t sdom_id);
/* SweepSolver over all subdomains: zeroes the planes, clears vacuum
 * boundaries, sweeps every subdomain in upwind order (all octants at once)
 * and hands planes to downwind zone sets.  With the option "block_jacobi" = 1
 * (--pmethod bj, src/Kripke/ParallelComm/BlockJacobiComm.cpp) every subdomain
 * is swept at once from the planes as they stood after the zeroing, i.e. from
 * zero inflow on every face, and no planes are handed on. */
int kgb_sweep_solver(kgb_ctx *ctx);
/* Kernel::population: sum over d,g,z of w(d) psi(d,g,z) volume(z), in FP64. */
int kgb_population(kgb_ctx *ctx, double *out);
/* FP64 particle balance after a sweep: out[0] emission (sum w rhs vol),
 * out[1] collision (sum w sigt psi vol), out[2] leakage through the domain
 * boundary, out[3] population, out[4] = out[0]-out[1]-out[2]. */
int kgb_balance(kgb_ctx *ctx, double out[5]);

/* SteadyStateSolver: niter source iterations from psi = 0.  part[i] gets the
 * particle count after iteration i (may be NULL).  source_strength is the
 * reference's 1.0 unless a caller scales the source. */
int kgb_solve(kgb_ctx *ctx, int32_t niter, double source_strength, double *part);
/* One source iteration on the current psi (no psi reset).  With part, the
 * particle count of the new psi is returned (and the call waits); without
 * it, a count is still formed on the device (one per iteration, as
 * SteadyStateSolver does): in FP64 that of the psi the iteration started from,
 * from the iteration's own moments; in the mixed form that of the new psi. */
int kgb_iterate(kgb_ctx *ctx, double source_strength, double *part);
/* Blocks until the context's stream is idle. */
int kgb_sync(kgb_ctx *ctx);
/* Run on a caller-owned CUDA stream (a cudaStream_t passed as a pointer)
 * instead of the context's own; NULL restores the context's stream. */
int kgb_set_stream(kgb_ctx *ctx, void *cuda_stream);
/* Tuning knobs: "sweep_tile_z" (tile depth in k, default 8); "sweep_tile_xy"
 * (tile footprint in i and j: 44, 42 or 22; default 22 in FP64, 42 in the
 * mixed form); "sweep_reciprocals"
 * (uniform mesh: 1 = tabulate 1/denominator per (sigt value, direction), the
 * FP64 default; 0 = divide in every cell, the mixed default); "moments_tensor"
 * (1 = LTimes and LPlusTimes on the tensor cores with exact digit products when
 * the shapes fit; 0 = SIMT kernels; default: tensor for FP64, SIMT for the
 * mixed form); "moments_tf32" (mixed form: 1 = LTimes and LPlusTimes may run
 * as split-TF32 tensor-core GEMMs -- each FP32 operand split exactly into three
 * TF32 pieces, six products, FP32 accumulation -- when moments <= 32 and there
 * are at least 32 directions, a multiple of 4 (LTimes) or of 16 up to 256
 * (LPlusTimes); ahead of "moments_tensor"; the default; 0 = off), with
 * "moments_tf32_lplustimes" (1 = LPlusTimes may, the default) and
 * "moments_tf32_ltimes" (1 = LTimes may; default 0: the tensor core's
 * accumulation truncates, and LTimes, whose directions weigh alike, would bias
 * phi towards zero by up to about one unit in the last place per iteration,
 * where LPlusTimes adds its dominant moment last);
 * "scattering_tensor" (1 = the single-material zones' scattering on the tensor
 * cores, exact digit products, when groups <= 64; the default in both forms);
 * "scattering_block" (mixed form: 1 = the single-material zones' scattering by
 * the zone-blocked FP32 kernel, bit for bit the SIMT kernel's sums, when
 * groups <= 64 and Legendre order <= 4; ahead of "scattering_tensor"; the
 * default; 0 = off);
 * "graph" (1 = kgb_solve replays a captured CUDA graph, the default);
 * "sweep_streams" (1 to 4: each sweep step launches its subdomains in that
 * many parts on as many streams, so one part's wave tail overlaps the others'
 * blocks; default 2);
 * "sweep_stream" (mixed form: 1 = the sweep runs on the streamed kernel --
 * each k-slice's rhs, sigt and entering faces copied into shared memory by
 * TMA boxes, slices ahead -- where a block of 128 or 96 chains holds whole
 * groups (4 to 32 directions per set, a multiple of 4; D and G multiples of 4;
 * footprints 44 and 42; the divide form; no fused prologue or epilogue); bit
 * for bit the per-step kernel's psi and planes; the default; 0 = off);
 * "sweep_stream_stages" (1 to 4 slices of operands in flight per block;
 * default 2);
 * "ltimes_stream" (mixed form: 1 = the solver's LTimes on the TMA-fed SIMT
 * kernel when directions are a multiple of 32 and 13 <= moments <= 32, bit for
 * bit the register-tiled kernel; the default; 0 = off) and
 * "ltimes_stream_stages" (2 to 4, default 2);
 * "ltimes_symmetric" (mixed form: 1 = where the 16 directions of each
 * octant are mirrored by the next octant's with L columns equal up to a sign
 * per moment -- Kripke's sets with 16 directions per octant -- the streamed
 * LTimes sums L(m,b)(psi(b) +- psi(b')) over octant pairs: half the
 * multiply-adds, summed in another order than the reference; the default;
 * 0 = off; read-only "ltimes_symmetric_active");
 * "block_jacobi" (0 = the sweep method, default; 1 = block Jacobi, used by
 * kgb_sweep_solver and so by every solve, iterate and adjoint call);
 * "fused_sweep" (mixed form, Legendre order <= 4: 1 = the solver loop forms
 * each cell's rhs inside the sweep from phi_out and ell_plus instead of
 * running LPlusTimes, with the SIMT kernel's arithmetic, so psi is unchanged;
 * rhs is then refreshed, as L+ phi_out, only when an entry point reads it --
 * download, kgb_lplustimes, the sweep entry points, kgb_balance, autotune);
 * "fused_ltimes" (mixed form, forward solves, (directions per set) x (groups
 * per set) a multiple of 128, without "fused_sweep": 1 = inside kgb_solve the
 * sweep of every iteration but the last also adds the next iteration's moments
 * phi = L psi -- per k-slice of a tile, each (zone, group, moment) takes the
 * sum over the subdomain's directions, added with FP32 reductions whose order
 * between subdomains is not fixed -- and the next iteration skips LTimes; phi
 * after the solve is still L of the psi the last iteration started from;
 * default 0);
 * "row_exponents" (1 = in FP64 with the tensor-core LTimes the solver loop's
 * sweep records the largest exponent of every (zone, group) row of psi, and
 * the next iteration's LTimes scales its digit split by it instead of reading
 * each row twice; that LTimes, or in the mixed form the register-tiled SIMT
 * LTimes, records phi's largest exponent per (zone, moment) for the
 * tensor-core scattering's gathered rows likewise; the
 * results are bit for bit those of 0; default 1; a fill of psi with 0
 * records zeros; any other write of psi -- upload, other fills,
 * kgb_sweep_subdomain, kgb_sweep_solver, the adjoint, a batched solve --
 * drops psi's record). */
int kgb_set_option(kgb_ctx *ctx, const char *key, int64_t value);
/* Current value of a knob: the keys above, plus "moments_tensor_ltimes",
 * "moments_tensor_lplustimes" and "scattering_tensor_active" (1 when that
 * kernel runs on the tensor cores), "sweep_reciprocals_active" (1 when the
 * sweep uses tabulated reciprocals), "graph_active" (1 when the last
 * kgb_solve replayed a graph), "fused_sweep_active" (1 when the last
 * iteration formed rhs inside the sweep), "moments_tf32_ltimes" and
 * "moments_tf32_lplustimes" (1 when that transform runs the TF32 kernel),
 * "fused_ltimes_active" (1 when
 * kgb_solve fuses the LTimes epilogue on this problem),
 * "psi_row_exponents_active" and
 * "phi_row_exponents_active" (1 when the solver loop records them on this
 * problem), "psi_row_exponents_valid" (1 when psi's record matches the
 * current psi) and "sweep_stream_active" (1 when the sweep runs on the
 * streamed kernel with the current tiles). */
int kgb_get_option(kgb_ctx *ctx, const char *key, int64_t *value);
/* Autotuner: times every sweep tile shape (footprint 4x4, 4x2, 2x2 x depth
 * 2, 4, 8, 16 zones; in the mixed form also the streamed kernel at 4x4 and 4x2,
 * depth up to 32) and both LTimes / LPlusTimes paths (tensor-core digit
 * products or SIMT) on this problem with CUDA events, keeps the fastest and
 * returns the sweep time (best_ms), footprint (as 44/42/22) and depth.  It
 * sweeps the current rhs and recomputes phi and rhs: psi, phi, rhs and the
 * planes are overwritten. */
int kgb_autotune(kgb_ctx *ctx, double *best_ms, int32_t *tile_xy, int32_t *tile_z);
/* Device time in milliseconds of the named kernel family accumulated since the
 * last reset ("sweep", "ltimes", "lplustimes", "scattering", "population");
 * timing is off unless kgb_set_timing(ctx, 1). */
int kgb_set_timing(kgb_ctx *ctx, int on);
int kgb_kernel_time(kgb_ctx *ctx, const char *family, double *ms, int64_t *launches);
int kgb_reset_timers(kgb_ctx *ctx);
/* Number of kernels this context has launched since it was created. */
int kgb_launch_count(kgb_ctx *ctx, int64_t *out);

/* --- converged solves, the adjoint and gradients ------------------------
 * No counterpart in the reference, whose SteadyStateSolver
 * (src/Kripke/SteadyStateSolver.cpp:24-115) runs a fixed iteration count;
 * these solve to a tolerance and differentiate a response at the fixed point.
 * Response: R = sum_z det(z) volume(z) sum_g siga(g,z) sum_d w(d) psi(d,g,z),
 * the absorption rate in a detector region, with siga(g,z) = sigt_zonal(g,z)
 * - sum over the zone's mix elements of fraction * sum_g' sigs(mat,0,g',g).
 * The adjoint iteration is the forward one with L and L+ exchanged, the
 * scattering transposed over groups and every direction swept in the
 * reversed orientation; its state lives beside psi, which it leaves alone
 * (phi, phi_out, rhs and the planes are scratch for either solve). */

/* The generator's material cross sections for `in` (kgb_generate uses the
 * same): sigt [3][G] per (material, group), and the scattering tables
 * sigs [3][L+1][G][G] indexed (material, Legendre order, destination group,
 * source group).  Either output may be NULL. */
int kgb_material_tables(const kgb_input *in, double *sigt, double *sigs);
/* Sets the cross sections from per-material tables: sigt [3][G] rebuilds
 * sigt_zonal through the uploaded mix elements (sum of fraction * sigma_t in
 * mix order, like the generator); sigs [3][L+1][G][G] replaces data/sigs.
 * NULL leaves that table unchanged. */
int kgb_set_materials(kgb_ctx *ctx, const double *sigt, const double *sigs);
/* Detector weights det(z), z = (k*ny + j)*nx + i over the whole mesh (n must
 * be nx*ny*nz); NULL = 1 everywhere (the default). */
int kgb_set_response(kgb_ctx *ctx, const double *det, int64_t n);
/* Source iterations from psi = 0 until moment 0 of successive iterates
 * satisfies max|phi_k - phi_(k-1)| <= tol * max|phi_k|, the change has made
 * no new minimum for 4 iterations (the rounding floor: near 1e-7 for the
 * mixed form's FP32 state), or max_iter iterations ran; tol < 0 runs exactly
 * max_iter iterations.  *iters and *change (either may be NULL) receive the
 * count and the last relative change (with tol < 0, *change is not measured);
 * *change > tol tells that tol was not reached, which is not an error. */
int kgb_solve_converged(kgb_ctx *ctx, double source_strength, double tol, int32_t max_iter, int32_t *iters,
                        double *change);
/* The adjoint source iteration for the response, from a zero state, with the
 * same stopping rule.  Needs ell(0,d) proportional to w(d) (true for the
 * reference's L); KGB_ERR_ARG otherwise. */
int kgb_adjoint_solve(kgb_ctx *ctx, double tol, int32_t max_iter, int32_t *iters, double *change);
/* R at the current psi. */
int kgb_response(kgb_ctx *ctx, double *response);
/* R and its gradients at the current psi and adjoint state: dsigt [3][G]
 * with respect to sigma_t of (material, group), dsigs [3][G] with respect to
 * the isotropic in-group scattering sigs(material, 0, g, g), dq with respect
 * to the source strength.  Exact for converged psi and adjoint; KGB_ERR_STATE
 * when no adjoint solve ran since the inputs last changed.  Outputs may be
 * NULL. */
int kgb_gradient(kgb_ctx *ctx, double *response, double *dsigt, double *dsigs, double *dq);
/* Unrolled (checkpoint) mode: R after exactly niter source iterations from
 * psi = 0 -- SteadyStateSolver's fixed count -- and its exact gradients, by
 * reverse mode through the iterations.  Forward iterates are checkpointed
 * every `stride` iterations (<= 0: ceil(sqrt(niter))) and recomputed one
 * segment at a time in the reverse pass, holding niter/stride + stride - 1
 * extra psi-sized buffers (stride 1 stores every iterate and recomputes
 * none).  Leaves psi at the niter-th iterate; the adjoint state is scratch. */
int kgb_gradient_unrolled(kgb_ctx *ctx, int32_t niter, double source_strength, int32_t stride, double *response,
                          double *dsigt, double *dsigs, double *dq);

/* --- batches of independent problems ---------------------------------
 * No counterpart in the reference (one problem per run).  A batch holds
 * independent problems of uneven sizes, each an ordinary context with one
 * zone set and Legendre order <= 4, all in the batch's precision, and
 * advances them together: one launch per kernel family for all problems,
 * the sweeps of all problems in ONE persistent cooperative launch, and a
 * whole solve captured once into a CUDA graph and replayed.  LTimes,
 * scattering and LPlusTimes run either as batched SIMT launches (the mixed
 * default) or as each problem's own kernels -- the tensor-core digit products
 * in FP64, the FP64 default -- on parallel branches of the graph.  Each
 * problem's results equal its own context's with the same sweep tiles (and
 * "moments_tensor" 0, "scattering_tensor" 0 when the batch runs its batched
 * SIMT kernels on FP64 problems). */
typedef struct kgb_batch kgb_batch;
int kgb_batch_create(int device, int32_t precision, kgb_batch **out);
int kgb_batch_destroy(kgb_batch *b);
const char *kgb_batch_last_error(const kgb_batch *b);
/* Generates a problem from `in` (precision taken from the batch); *index
 * receives its position. */
int kgb_batch_add(kgb_batch *b, const kgb_input *in, int32_t *index);
int kgb_batch_size(const kgb_batch *b, int32_t *n);
/* The problem's own context (owned by the batch): its fields can be read and
 * written, and its kernels run on their own, between batch solves. */
int kgb_batch_context(kgb_batch *b, int32_t index, kgb_ctx **ctx);
/* Knobs: "sweep_tile_xy" (44, 42, 22), "sweep_tile_z", "rows_per_item" (rows
 * of a moment / scattering work item), "graph" (1: capture solves, the
 * default), "per_problem_kernels" (1: each problem's own LTimes,
 * scattering and LPlusTimes kernels; 0: batched SIMT; -1: by precision, the
 * default), "per_problem_sweeps" (1: each problem's own sweeps -- its
 * per-step launches, the streamed FP32 sweep where it applies -- on parallel
 * graph branches, with the batch's tiles; 0: one persistent launch over all
 * problems; -1: by precision, the default; psi is bit for bit the same
 * either way), "branches" (1 to 8, default 8: the streams the problems' own
 * kernels are spread over, round-robin -- parallel branches of the graph;
 * the results do not depend on it), "barrier_wait_ns" (how long a grid-barrier wait of the persistent
 * sweep waits before it gives up; default 2e9; a solve whose wait gave up
 * returns KGB_ERR_TIMEOUT with its results undefined, and the batch stays
 * usable).  Read-only:
 * "graph_active" (the last solve replayed a graph),
 * "sweep_grid" (blocks of the persistent sweep), "sweep_steps",
 * "kernels_per_iteration". */
int kgb_batch_set_option(kgb_batch *b, const char *key, int64_t value);
int kgb_batch_get_option(kgb_batch *b, const char *key, int64_t *value);
/* Times every sweep tile shape (4x4, 4x2, 2x2 x depth 2, 4, 8, 16) in both
 * sweep modes (unless "per_problem_sweeps" was set), row item size (256,
 * 1024, 4096) and, unless "per_problem_kernels" was set, both transform modes
 * on the batch and keeps the fastest; overwrites the problems' state. */
int kgb_batch_autotune(kgb_batch *b, double *best_ms);
/* niter source iterations from psi = 0 for every problem (SteadyStateSolver
 * each); part (may be NULL) receives the particle counts [niter][n]. */
int kgb_batch_solve(kgb_batch *b, int32_t niter, double source_strength, double *part);
/* Device time (ms) of each phase of one iteration run launch by launch:
 * ms[0] LTimes, [1] scattering + source, [2] LPlusTimes, [3] persistent sweep,
 * [4] population; advances the problems' state by two iterations. */
int kgb_batch_profile(kgb_batch *b, double ms[5]);
/* Kernels the batch has launched (graph replays included). */
int kgb_batch_launch_count(kgb_batch *b, int64_t *out);

/* Allocation-free population edit.  No counterpart in the reference: it
 * exists for callers that cannot allocate device memory at the point they
 * need the particle count -- frameworks that own all device memory through
 * their own pool allocator, latency-bound loops that cannot afford an
 * allocation's implicit synchronisation.  Same
 * sum as kgb_population, over caller-owned device arrays: psi in the device
 * nesting [zone][group][direction] (FP64), w [directions], volume [zones];
 * *out (device memory) receives the FP64 result.  Allocates nothing: its
 * scratch is a static 128 KiB device array, which limits zones*groups to
 * 33,554,432 rows (larger sizes return KGB_ERR_ARG).  Launches on `stream`
 * (a cudaStream_t, NULL = legacy default stream) on the current device; the
 * first call on each device looks up the scratch address and should come
 * before any stream capture; a cudaDeviceReset invalidates that address, so
 * do not call it on a device after resetting it.  Calls share the scratch and
 * it keeps the last call's contents: calls that overlap on the GPU race, so
 * issue them on one stream.  err/err_len (optional) receive a message on
 * failure. */
int kgb_population_noalloc(const double *psi, const double *w, const double *volume, int64_t zones,
                           int32_t groups, int32_t directions, double *out, void *stream, char *err,
                           int32_t err_len);

#ifdef __cplusplus
}
#endif
#endif
