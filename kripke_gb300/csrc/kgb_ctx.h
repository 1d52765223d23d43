// kgb_ctx.h -- the context behind the C ABI (include/kgb.h), shared by its
// translation units: kgb_context.cu (context, fields, derived tables, plans),
// kgb_solver.cu (kernel drivers, the source-iteration loop, solves, the kernel
// entry points), kgb_adjoint_api.cu (converged solves, the adjoint, response
// and gradients) and kgb_options.cu (options, autotuner, timers).
//
// A context owns one GPU problem: the device fields of one Kripke problem in
// the device nesting (kgb_internal.h), the host copies of the small inputs, the
// sweep schedule, and the source-iteration loop.  Kernels live in sweep.cu,
// moments.cu, tc_moments.cu, tf32_moments.cu, scatter.cu, reduce.cu, xpose.cu,
// adjoint.cu and batch.cu.
//
// Host-side conventions mirrored from the reference (paths relative to the
// Kripke source tree):
//   nesting strides ......... VarTypes.h:67-101 + Core/VarLayout.h:118-170 (the
//                             field's index types sorted by their position in
//                             the nesting's order list; ties keep argument order)
//   subdomain numbering ..... Core/PartitionSpace.cpp:82-92,246-273 (row-major
//                             over P, Q, Rx, Ry, Rz; spaces project coordinates out)
//   chunk of a field ........ Core/DomainVar.cpp:15-39 (one chunk per subdomain
//                             of the field's space, in space-index order)
//   zone numbering .......... Generate/Space.cpp:92-93 (zone = (k*nj + j)*ni + i)
//   sweep scheduling ........ SweepSolver.cpp:23-87, ParallelComm.cpp:61-185
//   iteration ............... SteadyStateSolver.cpp:39-108
#pragma once

//   iteration ............... SteadyStateSolver.cpp:39-108
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <map>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "kgb_internal.h"
#include "kgb_layout.h"


namespace kgb {
namespace api {


enum Kind { K_FLUX, K_MOM, K_PLANE, K_SIGT, K_ELL, K_ELLP, K_SIGS, K_QD, K_QI, K_DXYZ, K_VOL, K_ZI, K_MI, K_MD, K_M2L };

struct FieldInfo {
  const char *name;
  Kind kind;
  int which;
};

inline constexpr FieldInfo kFields[] = {
    {"psi", K_FLUX, 0}, {"rhs", K_FLUX, 1}, {"phi", K_MOM, 0}, {"phi_out", K_MOM, 1},
    {"i_plane", K_PLANE, 0}, {"j_plane", K_PLANE, 1}, {"k_plane", K_PLANE, 2},
    {"sigt_zonal", K_SIGT, 0}, {"ell", K_ELL, 0}, {"ell_plus", K_ELLP, 0}, {"data/sigs", K_SIGS, 0},
    {"quadrature/xcos", K_QD, 0}, {"quadrature/ycos", K_QD, 1}, {"quadrature/zcos", K_QD, 2},
    {"quadrature/w", K_QD, 3}, {"quadrature/id", K_QI, 0}, {"quadrature/jd", K_QI, 1},
    {"quadrature/kd", K_QI, 2}, {"dx", K_DXYZ, 0}, {"dy", K_DXYZ, 1}, {"dz", K_DXYZ, 2},
    {"volume", K_VOL, 0}, {"zone_to_mixelem", K_ZI, 0}, {"zone_to_num_mixelem", K_ZI, 1},
    {"mixelem_to_zone", K_MI, 0}, {"mixelem_to_material", K_MI, 1}, {"mixelem_to_fraction", K_MD, 0},
    {"moment_to_legendre", K_M2L, 0},
};

inline const FieldInfo *findField(const char *name) {
  if (!name) return nullptr;
  for (const auto &f : kFields)
    if (!std::strcmp(f.name, name)) return &f;
  return nullptr;
}

// One chunk of a field in Kripke's host layout.
struct ChunkGeom {
  int nd;
  Idx types[4];
  int64_t dims[4];
  Space space;
};

struct TimerFam {
  double ms = 0.0;
  int64_t launches = 0;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pending;
};


}  // namespace api
}  // namespace kgb

using namespace kgb;
using namespace kgb::api;

struct kgb_ctx {
  int device = 0;
  cudaStream_t own_stream = nullptr;
  // further streams for parts of each sweep step's subdomains: the parts' step
  // launches overlap, so one part's wave tail runs beside the others' blocks
  static constexpr int kMaxSweepStreams = 4;
  cudaStream_t aux[kMaxSweepStreams - 1] = {};
  cudaEvent_t fork_ev = nullptr, join_ev[kMaxSweepStreams - 1] = {};
  int sweep_streams = 2, max_streams = kMaxSweepStreams;
  cudaStream_t stream = nullptr;
  std::string err;
  bool ready = false;
  kgb_dims dims{};
  Decomp dc;
  int G = 0, D = 0, M = 0, L = 0, Gs = 0, Ds = 0;
  int nx = 0, ny = 0, nz = 0, nxs = 0, nys = 0, nzs = 0;
  int64_t Z = 0, Zs = 0;
  int prec = KGB_FP64;
  size_t tsz = 8;
  int tz = 4;
  int tx = 4, ty = 4;  // sweep tile footprint
  bool tiles_set = false;  // the caller chose the tile shape: setup keeps it
  // FP32 sweeps on the streamed kernel (sweep_stream.cu) where it applies, with
  // stream_ns k-slices of operands in flight per block
  bool allow_stream = true;
  int stream_ns = 2;
  // mixed LTimes on the TMA-fed SIMT kernel (ltimes_stream.cu), lt_stream_ns stages
  bool allow_lt_stream = true;
  int lt_stream_ns = 2;
  // its octant-pair form (ltimes_sym_table): the device table of the L in use (forward: ell;
  // swapped with lt_sym_adj, ell_plus's, while the adjoint is installed), null when L has no
  // such structure
  bool allow_lt_sym = true;
  int *lt_sym = nullptr, *lt_sym_adj = nullptr;

  // device state (element type T = double or float by precision)
  void *psi = nullptr, *rhs = nullptr, *phi = nullptr, *phi_out = nullptr, *sigt = nullptr;
  void *plane[3] = {nullptr, nullptr, nullptr};
  int64_t plane_chunk[3] = {0, 0, 0};
  void *ell = nullptr, *ellp = nullptr, *sigsT = nullptr, *cx = nullptr, *cy = nullptr, *cz = nullptr;
  double *w_d = nullptr, *cos_d[3] = {nullptr, nullptr, nullptr}, *vol_d = nullptr, *dxyz_d[3] = {nullptr, nullptr, nullptr};
  int *zmix_start = nullptr, *zmix_count = nullptr, *mix_mat = nullptr, *mix_zone = nullptr;
  double *mix_frac = nullptr;
  int64_t nmix = 0, nmix_cap = 0;
  int *gp_lo = nullptr, *gp_hi = nullptr;
  SdomDesc *sdoms_d = nullptr;
  int *ident_d = nullptr, *levels_d = nullptr;
  int4 *tiles_d = nullptr;
  double *partials = nullptr;
  int npart = 0;
  double *results = nullptr;   // small device result slots
  double *parts_dev = nullptr; // per-iteration population
  int parts_cap = 0;
  double *staging = nullptr;
  size_t staging_bytes = 0;

  // host copies of the small inputs (global indexing)
  std::vector<double> q[4];          // xcos, ycos, zcos, w  [D]
  std::vector<int> qi[3];            // id, jd, kd           [D]
  std::vector<double> dxyz[3];       // dx [nx], dy [ny], dz [nz]
  std::vector<double> ell_h, ellp_h; // [D][M]
  std::vector<double> sigs_h;        // [3][L+1][G][G]
  std::vector<double> vol_h;         // [Z]
  std::vector<std::vector<int>> zmap[2];  // per R chunk: zone_to_mixelem, zone_to_num_mixelem
  std::vector<std::vector<int>> mimap[2]; // per R chunk: mixelem_to_zone, mixelem_to_material
  std::vector<std::vector<double>> mfrac; // per R chunk
  std::vector<int> m2l;
  bool have[32] = {};
  bool dirty_quad = true, dirty_geom = true, dirty_ell = true, dirty_sigs = true, dirty_mix = true, dirty_vol = true;

  // sweep schedule
  std::vector<SdomDesc> sdoms_h;
  std::vector<int> tile_off;  // step -> first tile, size nsteps+1
  int nsteps = 0;
  std::vector<int> level_off;  // wave level -> offset into levels_d
  std::vector<int> level_sdoms;

  bool timing = false;
  std::map<std::string, TimerFam> fams;
  int64_t launches = 0;  // kernels launched by this context

  // tabulated sweep reciprocals (FP64, uniform mesh)
  bool dirty_sigt = true;
  bool use_recip = false;
  bool allow_recip = true;
  uint16_t *cls_d = nullptr;
  void *inv_d = nullptr;  // double (FP64) or float (mixed)
  int64_t ncls = 0;
  // tensor-core moment transforms (tc_moments.cu)
  bool allow_tc = true;
  bool tc_lt = false, tc_lp = false;        // LTimes / LPlusTimes planned for the tensor cores
  bool use_tc_lt = true, use_tc_lp = true;  // autotuner's choice between tensor and SIMT paths
  uint16_t *tc_lt_img = nullptr, *tc_lp_img = nullptr;
  int *tc_lt_exp = nullptr, *tc_lp_exp = nullptr;
  int tc_lt_kpad = 0, tc_lp_nhalf = 0;
  int tc_lp_stages = 2, tc_lp_stage_out = 1;
  // split-TF32 tensor-core LTimes / LPlusTimes of the mixed form (tf32_moments.cu): B images
  // of the forward operators and of the adjoint's (exchanged by AdjointView)
  bool allow_tf32 = true;                          // option "moments_tf32"
  // per transform (options "moments_tf32_ltimes", "moments_tf32_lplustimes"): the TF32 LTimes'
  // truncating accumulations bias phi, so it is opt-in; LPlusTimes' leading moment comes last
  bool allow_tf32_lt = false, allow_tf32_lp = true;
  bool use_tf32_lt = false, use_tf32_lp = true;    // autotuner's choice
  float *tf32_lt_img = nullptr, *tf32_lp_img = nullptr;
  float *tf32_lt_img_adj = nullptr, *tf32_lp_img_adj = nullptr;
  // row exponents of psi for the tensor-core LTimes (FP64), written by the solver's sweep:
  // while psi_exp_valid, psi_exp[z*G + g] is the largest biased exponent in psi's row (z, g)
  int *psi_exp = nullptr;
  bool psi_exp_valid = false;
  bool allow_row_exp = true;  // option "row_exponents"
  // phi's exponents per (zone, moment) over the groups, recorded by the tensor-core
  // LTimes for the tensor-core scattering that follows it in the same iteration
  int *phi_exp = nullptr;
  int *err_d = nullptr;                     // set by kernels whose bounded waits gave up
  int nsm = 0;
  // fused population partials, one per (tile, subdomain, chain block)
  double *pop_slots = nullptr;
  int64_t npop_slots = 0;
  int64_t npop_used = 0;  // partials the last sweep wrote (its kernel's chain blocks)
  double vol_uniform = 0.0;
  double pop_scale = 0.0;  // w(d) / ell(0,d) when L's moment-0 row is proportional to w, else 0

  // converged solves, the adjoint source iteration and gradients (adjoint.cu)
  void *lam = nullptr;          // adjoint state divided by the cell volume, device nesting [Z][G][D]
  double *phi_prev = nullptr;   // moment 0 of the previous iterate [Z][G] (convergence test)
  void *sigsT_adj = nullptr;    // tables of S^T: [mat][l][g'][g] = sigs(mat, l, g', g)
  int *gp_lo_adj = nullptr, *gp_hi_adj = nullptr;
  double *colsum_d = nullptr;   // [3][G]: sum over destinations g' of sigs(mat, 0, g', g)
  double *e0_d = nullptr;       // [2][D]: ell(0, d), ell_plus(d, 0)
  double *det_d = nullptr;      // detector weights [Z]
  unsigned long long *norm_d = nullptr;  // max|change|, max|value| as ordered bit patterns
  double *resp_part = nullptr, *resp_d = nullptr;
  int resp_nb = 0;
  bool tc_lt_adj = false, tc_lp_adj = false;
  uint16_t *tc_lt_img_adj = nullptr, *tc_lp_img_adj = nullptr;
  int *tc_lt_exp_adj = nullptr, *tc_lp_exp_adj = nullptr;
  int tc_lt_kpad_adj = 0, tc_lp_nhalf_adj = 0;
  double inv_c0 = 0.0;          // w(d) / ell(0, d), or 0 when ell(0, .) is not proportional to w
  bool adj_stale = true;        // adjoint tables must be rebuilt from the host inputs
  bool have_lam = false;        // an adjoint solve has filled lam
  int flip = 0;                 // 1 while the adjoint operators are installed

  // tensor-core scattering of single-material zones: digit images of every
  // (material, order) matrix (transposed for the forward operator, as is for
  // the adjoint), the zones of each material, and the other zones (SIMT)
  bool tc_sc = false, use_tc_sc = true, allow_tc_sc = true, dirty_tcsc = true;
  bool tcsc_img_stale = true;  // the scattering's digit images predate sigs (zone lists aside)
  // zone-blocked FP32 scattering of the single-material zones (mixed form, scatter.cu)
  bool allow_blk_sc = true, use_blk_sc = true;
  uint16_t *tc_sc_img = nullptr, *tc_sc_img_adj = nullptr;
  int *tc_sc_exp = nullptr, *tc_sc_exp_adj = nullptr;
  int tc_sc_kpad = 0;
  int *pure_z = nullptr, *mixed_z = nullptr;
  int64_t pure_off[4] = {0, 0, 0, 0};
  int64_t nmixed_z = 0;

  // captured solves (kgb_solve): valid while gen, bumped whenever a table,
  // tile list or kernel choice a capture baked in may have changed, is unchanged
  uint64_t gen = 0;
  struct SolveGraph {
    int niter;
    double q;
    uint64_t gen;
    cudaStream_t stream;
    cudaGraph_t g;
    cudaGraphExec_t x;
    int64_t launches;
  };
  std::vector<SolveGraph> solve_graphs;
  bool use_graph = true, graph_active = false;
  bool block_jacobi = false;  // --pmethod bj: every zone set swept at once from zeroed planes
  // mixed form: the solver loop forms rhs inside the sweep (no LPlusTimes launch);
  // rhs then holds an older value until an entry point that reads it refreshes it
  bool fuse_sweep = false, fuse_active = false, rhs_stale = false;
  // fused LTimes epilogue (option fused_ltimes): inside one solve, the sweep of every
  // iteration but the last adds L psi into phi, and the next iteration skips LTimes
  bool fuse_lt = false, phi_fused = false;
};

namespace kgb {
namespace api {


inline int fail(kgb_ctx *c, int code, const std::string &msg) {
  if (c) c->err = msg;
  return code;
}

#define CK(call)                                                                                  \
  do {                                                                                            \
    cudaError_t e_ = (call);                                                                      \
    if (e_ != cudaSuccess) return fail(ctx, KGB_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

#define CKL() CK(cudaGetLastError())
// record `n` kernel launches, then check the launch status
#define CKN(n)              \
  do {                      \
    ctx->launches += (n);   \
    CKL();                  \
  } while (0)

inline int fieldIndex(const FieldInfo *f) { return (int)(f - kFields); }

template <typename T>
T *as(void *p) {
  return reinterpret_cast<T *>(p);
}

template <typename T>
int dmalloc(kgb_ctx *ctx, T **p, size_t n) {
  cudaError_t e = cudaMalloc((void **)p, std::max<size_t>(n, 1) * sizeof(T));
  if (e != cudaSuccess) return fail(ctx, KGB_ERR_OOM, "device allocation failed");
  return KGB_OK;
}

// ---------------------------------------------------------------------------
// Timers (CUDA events on the context's stream)
// ---------------------------------------------------------------------------
// One kernel family's launches: an NVTX range on the calling thread (named
// "kgb:<family>", visible to Nsight Systems and any NVTX tool; a no-op without
// one) and, while timing is on, CUDA events on the context's stream.
struct FamScope {
  kgb_ctx *c;
  TimerFam *fam = nullptr;
  cudaEvent_t b = nullptr;
  FamScope(kgb_ctx *ctx, const char *name) : c(ctx) {
    char label[48];
    std::snprintf(label, sizeof label, "kgb:%s", name);
    nvtxRangePushA(label);
    if (!c->timing) return;
    fam = &c->fams[name];
    cudaEventCreate(&b);
    cudaEventRecord(b, c->stream);
  }
  ~FamScope() {
    nvtxRangePop();
    if (!fam) return;
    cudaEvent_t e;
    cudaEventCreate(&e);
    cudaEventRecord(e, c->stream);
    fam->pending.push_back({b, e});
    fam->launches++;
  }
};

template <typename T>
int uploadVec(kgb_ctx *ctx, void *dst, const std::vector<double> &src) {
  std::vector<T> tmp(src.begin(), src.end());
  CK(cudaMemcpyAsync(dst, tmp.data(), tmp.size() * sizeof(T), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));  // tmp goes out of scope
  return KGB_OK;
}

// Tensor-core digit images of the LTimes / LPlusTimes operators read from the [D][M] host tables
// lt_src / lp_src (kgb_context.cu; instantiated for double and float).
template <typename T>
int planTensorMomentsFrom(kgb_ctx *ctx, const std::vector<double> &lt_src, const std::vector<double> &lp_src,
                          bool *lt_ok, uint16_t **lt_img, int **lt_exp, int *lt_kpad, bool *lp_ok, uint16_t **lp_img,
                          int **lp_exp, int *lp_nhalf);

// ---- shared between the context's translation units ----
ChunkGeom chunkGeom(const kgb_ctx *c, const FieldInfo *f, int ch);
bool isIntKind(Kind k);
int64_t chunkElems(const ChunkGeom &g);
int numChunks(const kgb_ctx *c, const FieldInfo *f);
int64_t fieldBytes(const kgb_ctx *c, const FieldInfo *f);
int ensureStaging(kgb_ctx *ctx, size_t bytes);
XposeDesc chunkXpose(const kgb_ctx *c, const FieldInfo *f, int ch);
bool deviceKind(Kind k);
void *deviceArray(kgb_ctx *c, const FieldInfo *f);
int64_t deviceElems(const kgb_ctx *c, const FieldInfo *f);
int dalloc(kgb_ctx *ctx, void **p, size_t bytes);
void dropSolveGraphs(kgb_ctx *c);
void freeAll(kgb_ctx *c);
int need(kgb_ctx *ctx, std::initializer_list<const char *> names);
int buildReciprocals(kgb_ctx *ctx);
int planTf32From(kgb_ctx *ctx, const std::vector<double> &lt_src, const std::vector<double> &lp_src, float **lt_img,
                 float **lp_img);
int planLtSym(kgb_ctx *ctx, const std::vector<double> &lt_src, int **table);
bool ltSymActive(const kgb_ctx *ctx);
bool tf32LtActive(const kgb_ctx *ctx);
bool tf32LpActive(const kgb_ctx *ctx);
void updatePopScale(kgb_ctx *ctx);
int prepare(kgb_ctx *ctx);
int buildTiles(kgb_ctx *ctx);
int psiExpWidth(const kgb_ctx *ctx);
bool psiExpUsable(const kgb_ctx *ctx);
int phiExpWidth(const kgb_ctx *ctx);
bool phiExpUsable(const kgb_ctx *ctx);
int sweepWaveAny(kgb_ctx *ctx, const int *wave_dev, int nwave, bool fused_pop = false, bool fused_rhs = false,
                 int *rowexp = nullptr, bool fused_lt = false);
int fillField(kgb_ctx *ctx, const FieldInfo *f, double v);
int sweepSolver(kgb_ctx *ctx, bool fused_pop = false, bool fused_rhs = false, int *rowexp = nullptr,
                bool fused_lt = false);
bool fusedLtUsable(const kgb_ctx *ctx);
bool streamUsable(const kgb_ctx *ctx);
ScatterArgsBase scatterArgs(kgb_ctx *ctx);
int doLTimes(kgb_ctx *ctx, bool acc, const int *rowexp = nullptr, int *outexp = nullptr);
int doLPlusTimes(kgb_ctx *ctx, bool acc);
int ensureRhs(kgb_ctx *ctx);
bool blockScatterActive(const kgb_ctx *ctx);
int doScattering(kgb_ctx *ctx, bool acc, const int *rowexp = nullptr);
int doSource(kgb_ctx *ctx, double q);
int doPopulation(kgb_ctx *ctx, double *out);
int checkDeviceError(kgb_ctx *ctx);
// lt_next: the sweep also adds L psi into phi for the next iteration of the same solve
int iterateDevice(kgb_ctx *ctx, double q, double *part_slot, double *prev_slot = nullptr, bool lt_next = false);
bool lagPopulation(const kgb_ctx *ctx);
int resetPsiExp(kgb_ctx *ctx);
int solveIterations(kgb_ctx *ctx, int niter, double q);
int solveGraph(kgb_ctx *ctx, int niter, double q, const kgb_ctx::SolveGraph **out);
MixArgs mixArgs(const kgb_ctx *ctx);
int ensureResponseBuffers(kgb_ctx *ctx);
int prepareAdjoint(kgb_ctx *ctx);
int doAdjointSource(kgb_ctx *ctx);
int convergeLoop(kgb_ctx *ctx, bool adjoint, double q, double tol, int max_iter, int32_t *iters, double *change);
int responseTermsOf(kgb_ctx *ctx, const void *psi, const void *psi0, const void *lam, std::vector<double> &out);
int forwardStep(kgb_ctx *ctx, void *in, void *out, double q);
int reverseStep(kgb_ctx *ctx, bool first);

}  // namespace api
}  // namespace kgb
