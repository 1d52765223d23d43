// kgb_internal.h -- device data model and kernel launchers of kripke_gb300.
//
// Device nesting (chosen for the GPU, independent of the host nesting):
//   psi, rhs       [Z][G][D]   zone-major over the whole problem, direction fastest
//   phi, phi_out   [Z][G][M]   moment fastest
//   sigt_zonal     [Z][G]
//   planes         per subdomain chunk: i_plane [nzs][nys][Gs][Ds],
//                  j_plane [nzs][nxs][Gs][Ds], k_plane [nys][nxs][Gs][Ds]
// with Z = global zone index (k*ny + j)*nx + i.  A subdomain's (group,
// direction) pairs are "chains" c = g_local*Ds + d_local; chains are the
// fastest index everywhere the sweep touches memory, so one warp reads and
// writes contiguous runs.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/kgb.h"

namespace kgb {

// Per-subdomain sweep descriptor (device copy).
struct SdomDesc {
  int p, q, xs, ys, zs;   // coordinates in (P, Q, Rx, Ry, Rz)
  int glo, dlo;           // first global group / direction
  int io, jo, ko;         // zone-set origin in global zones
  int id, jd, kd;         // traversal of the subdomain's first direction
  int64_t ip, jp, kp;     // element offsets of its plane chunks
};

template <typename T>
struct SweepArgs {
  const T *rhs;
  T *psi;
  const T *sigt;
  T *iplane, *jplane, *kplane;
  const T *cx, *cy, *cz;      // 2*cos/delta per (direction, zone index): [D][nx], [D][ny], [D][nz]
  const SdomDesc *sdoms;
  const int *wave;            // subdomains swept by this launch
  const int4 *tiles;          // oriented tile coordinates of every step, concatenated
  int tile_off;               // first tile of this step
  int nx, ny, nz, G, D, Gs, Ds, nxs, nys, nzs;
  int tz;                     // tile depth in k
  int tx, ty;                 // tile footprint in i and j: 4x4, 4x2 or 2x2
  int flip;                   // 1: sweep every direction in the reversed orientation (adjoint)
  // tabulated reciprocals (uniform mesh): 1/((cx+cy+cz)[d] + sigt) per (sigt class, direction)
  const uint16_t *cls;        // [Z][G] class of sigt_zonal, or null: divide per cell
  const T *inv;               // [nclass][D]
  // fused population: per-block partial sums of w(d)*psi*volume(z), or null
  double *pop;                // slot = ((tile index)*nsdom + sdom)*gridDim.x + blockIdx.x
  int nsdom;
  const double *w;            // [D]
  const double *vol;          // [Z]; unused when vol_uniform > 0
  double vol_uniform;
  // fused LPlusTimes prologue (mixed form): rhs(z,g,d) = sum_m ellp[d][m] * phiout[z][g][m]
  // formed per cell instead of read, or null: read rhs
  const T *phiout;            // [Z][G][M]
  const T *ellp;              // [D][M]
  int M;
  // fused LTimes epilogue (mixed form): phiacc(z,g,m) += sum over this subdomain's
  // directions of ell[d][m] * psi(z,g,d), added per (zone, group, moment) after each
  // k-slice of a tile (FP32 reductions; phiacc zeroed before the sweep), or null
  T *phiacc;                  // [Z][G][M]
  const T *ell;               // [D][M]
  // row exponents for the next LTimes (FP64): rowexp[z*G + g] = max over the
  // row's swept psi of the biased exponent (atomic max, zeroed before the
  // sweep), or null.  rexp_w lanes share a group (a power of two <= 32 that
  // divides Ds, or 32 when 32 divides Ds).
  int *rowexp;
  int rexp_w;
  // streamed FP32 sweep (sweep_stream.cu): stages of slice operands in flight
  // (0: the per-step kernel of sweep.cu), and the word a bounded wait that
  // gives up sets
  int stream_ns;
  int *err;
};

// Largest moment count (Legendre order 4) of the fused LPlusTimes prologue.
constexpr int kFuseMaxM = 25;

// Sweep tiles: footprint in i and j is a compile-time instance (4x4, 4x2 or
// 2x2), depth in k is runtime.
constexpr int kSweepThreads = 128;

template <typename T>
void launch_sweep_step(const SweepArgs<T> &a, int ntiles, int nwave, cudaStream_t s);

// Streamed FP32 sweep (sweep_stream.cu): each block's rhs, sigt and entering
// faces of a whole k-slice of its tile arrive in shared memory by TMA box
// copies, slices ahead.  It applies to the divide form (no reciprocal tables,
// fused prologue or epilogue) when a block's 128 chains are whole groups whose
// operand boxes meet TMA's 16-byte rules: a multiple of 4 directions per set
// (at most 32), blocks of GB whole groups (GB a multiple of 4 dividing the
// group set, GB x Ds = 128 or 96 chains), D and G multiples of 4.  Tile footprints 4x4 and 4x2 (8x4 needs 150+ registers a
// thread for its k faces).
constexpr int kStreamMaxStages = 4;
int stream_block_chains(int Ds, int Gs);  // chains per block, 0: not streamable
bool sweep_stream_applies(int D, int G, int Ds, int Gs, int tx, int ty);
// launches one hyperplane step (a.stream_ns stages); false when a tensor map
// cannot be encoded (nothing launched)
bool launch_sweep_step_stream(const SweepArgs<float> &a, int ntiles, int nwave, cudaStream_t s);

// Classes of the distinct sigt values for the sweep's reciprocal tables, on the
// device: class_insert records every distinct bit pattern of sig in an
// open-addressing table of 2^kClassTableBits 64-bit keys (kClassEmpty = free;
// *overflow is set when a value cannot be recorded), class_lookup gives each
// element the index of its value in the sorted distinct values.
constexpr int kClassTableBits = 17;
constexpr unsigned long long kClassEmpty = ~0ull;
template <typename T>
void launch_class_insert(const T *sig, int64_t n, unsigned long long *table, int *overflow, cudaStream_t s);
template <typename T>
void launch_class_lookup(const T *sig, int64_t n, const T *uniq, int ncls, uint16_t *cls, cudaStream_t s);

template <typename T>
void launch_ltimes(const T *psi, T *phi, const T *ell_dm, int64_t rows, int D, int M, bool accumulate, cudaStream_t s);
template <typename T>
void launch_lplustimes(const T *phi_out, T *rhs, const T *ellp_dm, int64_t rows, int D, int M, bool accumulate, cudaStream_t s);
// FP32 LTimes (phi = L psi, not accumulated) through the register-tiled kernel,
// recording phi's largest biased exponent per (zone, moment) over the zone's
// groups into outexp[zone * M + m] (atomic max; zeroed by the caller), reduced
// over runs of rexp_w lanes (32, or the group count G when that is a power of
// two below 32).  Returns false, launching nothing, when the tiled kernel does
// not apply (ltimes_tiled_applies).
bool ltimes_tiled_applies(int D, int M);

// Split-TF32 tensor-core LTimes / LPlusTimes of the mixed form (tf32_moments.cu):
// phi (rhs) = or += L psi (L+ phi_out) over rows (zone, group) of the device
// nesting.  phi and phi_out must be allocated for tf32_padded_rows(rows)
// rows.  bimg: the B image built by tf32_build_b.  Nonzero return: not launched.
bool tf32_ltimes_applies(int D, int M);
bool tf32_lplustimes_applies(int D, int M);
int64_t tf32_padded_rows(int64_t rows);
void tf32_build_b(const float *b, int K, int N, int kpad, int npad, std::vector<float> &img);
int launch_tf32_ltimes(const float *psi, float *phi, int64_t rows, int D, int M, const float *bimg, bool accumulate,
                       int *err, int nsm, cudaStream_t s);
int launch_tf32_lplustimes(const float *phi_out, float *rhs, int64_t rows, int D, int M, const float *bimg,
                           bool accumulate, int *err, int nsm, cudaStream_t s);
bool launch_ltimes_record(const float *psi, float *phi, const float *ell_dm, int64_t rows, int D, int M,
                          int *outexp, int rexp_w, int G, cudaStream_t s);
// FP32 LTimes phi = L psi (not accumulated) on the TMA-fed SIMT kernel
// (ltimes_stream.cu): directions a multiple of 32, 13 <= M <= 32, ns = 2..4
// shared-memory stages; bit for bit the register-tiled kernel.  sym (device, or
// null): the octant-pair table of L (ltimes_sym_table), which halves the
// multiply-adds and sums in another order.  Nonzero return: not launched.
bool ltimes_stream_applies(int D, int M);
int launch_ltimes_stream(const float *psi, float *phi, const float *ell_dm, int64_t rows, int D, int M, int ns,
                         const int *sym, int *err, int nsm, cudaStream_t s);
// The octant-pair table of a [D][M] L for launch_ltimes_stream, or false when L
// has no such structure: per 32-direction chunk the partner column (16..31) of
// each of its first 16 directions, whose L column is the direction's times a
// sign that depends on the moment only; then the moment of each of 32 slots
// (slots 0-15 the moments of sign +1, 16-31 those of sign -1, ascending; -1
// empty).  D/2 + 32 entries.
bool ltimes_sym_table(const double *L, int D, int M, std::vector<int> &table);

struct ScatterArgsBase {
  int64_t Z;                  // zones (rows = Z * destination groups); with zlist, the list's length
  const int *zlist;           // zones to update, or null: every zone
  int G, M, L;
  const int *zmix_start, *zmix_count, *mix_mat;
  const double *mix_frac;
  const int *gp_lo, *gp_hi;   // nonzero source-group range per destination group
  int src_glo, src_ghi;       // source groups [lo, hi) taken (group-set pairs)
  int dst_glo, dst_ghi;       // destination groups updated
};
template <typename T>
void launch_scattering(const T *phi, T *phi_out, const T *sigsT, const ScatterArgsBase &a, bool accumulate, cudaStream_t s);
template <typename T>
void launch_source(T *phi_out, int64_t nmix, const int *mix_zone, const int *mix_mat, const double *mix_frac,
                   int G, int M, double strength, cudaStream_t s);
// Zone-blocked FP32 scattering of the single-material zones (scatter.cu): zl
// holds every material's pure zones, material m's at [off[m], off[m+1]).
struct ScatterBlockPlan {
  int64_t off[4];
  int64_t nitems[3];  // work items (runs of zpc zones) per material
  int64_t items;
  int G, zpc;
  const int *gp_lo, *gp_hi;
};
// Groups a multiple of 4 take the staged form (scatter_zone_kernel): zone blocks
// arrive by bulk copies, each thread keeps a 4-group x (L+1)^2 register tile.
struct ScatterZonePlan {
  int64_t off[4];
  int G, zpi;            // groups; zones per item of one 128-thread group
  int nh, qw, zw;        // a zone's quads in nh parts of qw (<= 8); zw zones per warp
  uint32_t slot;         // floats between staged zone blocks
  const int *gp_lo, *gp_hi;
  int *err;              // raised when a copy's bounded wait gives up
};
bool scatter_block_applies(int G, int L);
size_t scatter_block_smem(int G, int L);
// err: the context's device error word (the staged form's bounded waits)
void launch_scatter_block(const float *phi, float *phi_out, const float *sigsT, const int *zl, const int64_t off[4],
                          int G, int L, const int *gp_lo, const int *gp_hi, bool accumulate, int *err, int nsm,
                          cudaStream_t s);

// Tensor-core row products C[r][n] (+)= sum_k A[r][k] B[k][n] (tc_moments.cu).
template <typename T>
struct TcArgs {
  const T *A;            // [rows][lda]
  T *C;                  // [rows][ldc]
  int64_t rows;
  int lda, ldc;
  int K, kpad, N;        // real K, K padded to a multiple of 32, real N
  int nhalf;             // N blocks (1 for LTimes; LPlusTimes splits N)
  const uint16_t *bimg;  // digit image of B, built by tc_build_b
  const int *bexp;       // per-column exponent of B
  int *err;              // set to 1 when a bounded wait gives up
  bool accumulate;
  int nsm;
  // gathered rows (launch_tc_gather): row r = zone zl[r / nm], moment m0 + r % nm;
  // A and C elements at zone * zstride + moment + k * ks
  const int *zl;
  int nm, m0, ks;
  int64_t zstride;
  int stages;            // A stages in shared memory: 2 (default, 0) or 1 (one K chunk per tile only)
  int stage_out;         // 1: outputs of contiguous rows are staged in shared memory for wide stores
  // per-row bound of the biased exponents of A (max over the row, 0 for a zero
  // row), written by the kernel that produced A; null: the kernel finds it.
  // Row r's entry is rowexp[r]; gathered rows: rowexp[zone * ks + moment].
  const int *rowexp;
  // record of C's exponents for a gathered consumer (FP64, staged outputs):
  // outexp[(r / outexp_rows) * N + n] = max biased exponent of column n over
  // the outexp_rows consecutive rows of r's zone (atomic max; zeroed by the
  // caller), reduced over runs of outexp_w lanes (32, or outexp_rows when that
  // is a power of two below 32); null: none
  int *outexp;
  int outexp_w, outexp_rows;
};
// Digits per operand of the exact tensor-core products: 7 balanced 8-bit digits
// (54 bits) for FP64, 4 (30 bits) for the FP32 of the mixed form.
template <typename T>
constexpr int tcDigits() {
  return sizeof(T) == 8 ? 7 : 4;
}
template <typename T>
void tc_build_b(const double *b, int K, int N, int kpad, int S, int NB, int nhalf, std::vector<uint16_t> &img,
                std::vector<int> &texp);
template <typename T>
void launch_tc_rows(const TcArgs<T> &a, cudaStream_t s);
template <typename T>
void launch_tc_gather(const TcArgs<T> &a, cudaStream_t s);

// FP64 reductions, two passes with a fixed order: per-block partials then one block.
template <typename T>
void launch_population(const T *psi, const double *w, const double *vol, int64_t rows, int G, int D,
                       double *partials, int nblocks, double *out, cudaStream_t s);
template <typename T>
void launch_population_moments(const T *phi, int M, const double *vol, int64_t rows, int G, double scale,
                               double *partials, int nblocks, double *out, cudaStream_t s);
template <typename T>
void launch_balance_terms(const T *psi, const T *rhs, const T *sigt, const double *w, const double *vol,
                          int64_t rows, int G, int D, double *partials, int nblocks, double *out2, cudaStream_t s);
template <typename T>
void launch_leakage(const T *plane, int64_t nelem, int Gs, int Ds, int dlo, int na, const double *w,
                    const double *cosv, const double *wa, const double *wb, double *partials, int nblocks,
                    double *out, cudaStream_t s);

// One block sums n partials in a fixed order into *out.
void launch_sum_partials(const double *partials, int64_t n, double *out, cudaStream_t s);

// Layout transfer between a host-nested chunk and the device nesting.
struct XposeDesc {
  int nd;                 // logical dims (<= 4)
  int64_t n[4];           // logical sizes
  int64_t hs[4];          // host strides (elements)
  int64_t os[4];          // device strides (elements); the zone dim uses os for the global zone
  int zdim;               // logical dim that is a zone index (-1: none)
  int nxs, nys;           // zone-set shape for local->global zone mapping
  int io, jo, ko, nx, ny; // zone-set origin and global shape
  int iter[4];            // iteration order, fastest last (matches the device-fastest dim)
  int64_t obase;
};
template <typename Td>
void launch_upload_xpose(const double *staging, Td *dev, const XposeDesc &x, cudaStream_t s);
template <typename Td>
void launch_download_xpose(const Td *dev, double *staging, const XposeDesc &x, cudaStream_t s);
template <typename T>
void launch_fill(T *p, int64_t n, double v, cudaStream_t s);

// Batched problems (batch.cu): one launch per kernel family covers many
// independent problems.  Work items of the row kernels are row ranges of one
// problem each.
struct BatchRows {
  int inst;
  int pad_;
  int64_t r0, r1;
};
template <typename T>
struct BatchMom {      // LTimes: src psi, dst phi, mat ell; LPlusTimes: src phi_out, dst rhs, mat ell_plus
  const T *src;
  T *dst;
  const T *mat;        // [D][M]
  int D, M;
};
template <typename T>
struct BatchScat {
  const T *phi;
  T *phi_out;
  const T *sigsT;
  ScatterArgsBase a;
  double q;            // source strength of material 0 (Kernel::source, fused)
};
int moment_class(int M);
template <typename T>
void launch_batch_moments(const BatchMom<T> *inst, const BatchRows *items, int nitems, int M, int Dmax, bool plus,
                          bool vec, int grid, cudaStream_t s);
template <typename T>
void launch_batch_scattering(const BatchScat<T> *inst, const BatchRows *items, int nitems, int L, int grid,
                             cudaStream_t s);
// Persistent batched sweep: zero every plane, then every global hyperplane
// step of every problem, separated by a bounded grid barrier; launched
// cooperatively so all blocks are resident.
struct BatchZero {
  int inst, plane;
  int64_t begin, end;  // element range of the problem's plane array
};
struct BatchSweepPlan {
  const int4 *items;      // (problem, subdomain, tile, chain block), grouped by global step
  const int *step_off;    // [nsteps + 1]
  int nsteps;
  const BatchZero *zero;  // plane zeroing ranges
  int nzero;
  unsigned int *bar;      // [2] grid barrier: arrivals, generation (zero before a launch)
  int *err;               // set when a barrier wait gives up
  unsigned long long wait_ns;  // a barrier wait gives up after this long (globaltimer ns)
};
template <typename T>
int batch_sweep_grid(int tx, int ty, int nsm);
template <typename T>
cudaError_t launch_batch_sweep(const SweepArgs<T> *inst, const BatchSweepPlan &p, int tx, int ty, int grid,
                               cudaStream_t s);
// per-problem fixed-order sums of the fused population partials: out[i] = sum of slots[i][0 .. n[i])
void launch_batch_pop_finish(const double *const *slots, const int64_t *n, int ninst, double *out, cudaStream_t s);

// Device view of one prepared context (kgb_solver.cu), for the batched driver.
struct InstanceView {
  int prec;
  int64_t Z;
  int G, D, M, L, Gs, Ds, nx, ny, nz, nsdom, zonesets[3];
  void *psi, *rhs, *phi, *phi_out, *sigt, *plane[3];
  int64_t plane_chunk[3];
  void *ell, *ellp, *sigsT, *cx, *cy, *cz;
  const double *w, *vol, *mix_frac;
  const int *zmix_start, *zmix_count, *mix_mat, *gp_lo, *gp_hi;
  const SdomDesc *sdoms;
  double vol_uniform;
  const uint16_t *cls;  // tabulated sweep reciprocals, or null (divide per cell)
  const void *inv;      // [nclass][D] in the context's precision
  uint64_t gen;         // the context's table generation: changes whenever a table, tile list or kernel choice changes
  int *psi_exp;         // psi's row-exponent record for the problem's tensor-core LTimes, or null
  int psi_exp_w;        // lanes of one group in the sweep's chain order (rexp_w)
};
int instance_view(kgb_ctx *ctx, InstanceView *v);
// One of the context's own iteration kernels, launched on stream s with the
// kernels the context chooses (tensor-core or SIMT): LTimes (phi = L psi),
// LPlusTimes (rhs = L+ phi_out), or scattering then source (phi_out = S phi + q).
// psi_exp (LTimes): psi's row exponents as the batched sweep recorded them, or null.
// Sweep: the problem's own sweep of every octant (its tiles and kernels, the
// streamed FP32 sweep where it applies) with the population of the new psi
// summed into *pop; with psi_exp (FP64), psi's row exponents are recorded there.
enum class InstanceOp { LTimes, Scatter, LPlusTimes, Sweep };
int instance_op(kgb_ctx *ctx, InstanceOp op, double q, cudaStream_t s, const int *psi_exp = nullptr,
                double *pop = nullptr);
int instance_tiles(kgb_ctx *ctx, int tx, int ty, int tz);  // sets the problem's sweep tiles
int64_t instance_sweep_launches(const kgb_ctx *ctx);       // kernels one Sweep op launches
// Reports (KGB_ERR_TIMEOUT) and clears a bounded wait of one of the context's
// tensor-core kernels that gave up; the caller has synchronised the streams
// those kernels ran on.
int instance_check(kgb_ctx *ctx);

// Response, adjoint source and gradients (adjoint.cu).
struct MixArgs {
  int64_t Z;
  int G, nx, ny;
  const int *zmix_start, *zmix_count, *mix_mat;
  const double *mix_frac;
  const double *colsum;       // [3][G]: sum over destinations of the P0 scattering of source group g
  const double *det, *vol;    // detector weights and zone volumes [Z]
  const double *dx, *dy, *dz; // mesh spacing (cell volume dx*dy*dz scales the adjoint state)
};
template <typename T>
void launch_adjoint_source(T *phi_out, int M, const T *sigt, const MixArgs &a, double inv_c0, cudaStream_t s);
template <typename T>
void launch_response(const T *psi, const T *psi0, const T *lam, int D, const double *w, const double *ell0,
                     const double *ellp0, const T *sigt, const MixArgs &a, double *partials, int nblocks_z,
                     double *out, cudaStream_t s);
template <typename T>
void launch_change_norm(const T *phi, int M, double *prev, int64_t rows, unsigned long long *out, cudaStream_t s);
template <typename T>
void launch_material_sigt(T *sigt, const double *sigt_mat, const MixArgs &a, cudaStream_t s);

}  // namespace kgb
