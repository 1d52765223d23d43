// kgb_api.cu -- the C ABI of kripke_gb300 (include/kgb.h).
//
// Owns one GPU context: the device fields of one Kripke problem in the
// device nesting (kgb_internal.h), the host copies of the small inputs, the
// sweep schedule, and the source-iteration loop.  Kernels live in sweep.cu,
// moments.cu, scatter.cu, reduce.cu and xpose.cu.
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

using namespace kgb;

namespace {

enum Kind { K_FLUX, K_MOM, K_PLANE, K_SIGT, K_ELL, K_ELLP, K_SIGS, K_QD, K_QI, K_DXYZ, K_VOL, K_ZI, K_MI, K_MD, K_M2L };

struct FieldInfo {
  const char *name;
  Kind kind;
  int which;
};

const FieldInfo kFields[] = {
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

const FieldInfo *findField(const char *name) {
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

}  // namespace

struct kgb_ctx {
  int device = 0;
  cudaStream_t own_stream = nullptr;
  // further streams for parts of each sweep step's subdomains: the parts' step
  // launches overlap, so one part's wave tail runs beside the others' blocks
  static constexpr int kMaxSweepStreams = 4;
  cudaStream_t aux[kMaxSweepStreams - 1] = {};
  cudaEvent_t fork_ev = nullptr, join_ev[kMaxSweepStreams - 1] = {};
  int sweep_streams = 2, max_streams = kMaxSweepStreams;
  bool sweep_l2_hints = false;  // option sweep_l2_hints
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
  bool use_tf32_lt = true, use_tf32_lp = true;     // autotuner's choice
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
};

namespace {

int fail(kgb_ctx *c, int code, const std::string &msg) {
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

int fieldIndex(const FieldInfo *f) { return (int)(f - kFields); }

// Host-layout geometry of chunk `ch` of a field.
ChunkGeom chunkGeom(const kgb_ctx *c, const FieldInfo *f, int ch) {
  ChunkGeom g{};
  switch (f->kind) {
    case K_FLUX: g = {3, {I_DIR, I_GRP, I_ZONE}, {c->Ds, c->Gs, c->Zs}, S_PQR}; break;
    case K_MOM: g = {3, {I_MOM, I_GRP, I_ZONE}, {c->M, c->Gs, c->Zs}, S_PR}; break;
    case K_PLANE:
      if (f->which == 0) g = {4, {I_DIR, I_GRP, I_ZJ, I_ZK}, {c->Ds, c->Gs, c->nys, c->nzs}, S_PQR};
      else if (f->which == 1) g = {4, {I_DIR, I_GRP, I_ZI, I_ZK}, {c->Ds, c->Gs, c->nxs, c->nzs}, S_PQR};
      else g = {4, {I_DIR, I_GRP, I_ZI, I_ZJ}, {c->Ds, c->Gs, c->nxs, c->nys}, S_PQR};
      break;
    case K_SIGT: g = {2, {I_GRP, I_ZONE}, {c->Gs, c->Zs}, S_PR}; break;
    case K_ELL: g = {2, {I_MOM, I_DIR}, {c->M, c->Ds}, S_Q}; break;
    case K_ELLP: g = {2, {I_DIR, I_MOM}, {c->Ds, c->M}, S_Q}; break;
    case K_SIGS: g = {4, {I_MAT, I_LEG, I_GGRP, I_GGRP}, {3, c->L + 1, c->G, c->G}, S_NULL}; break;
    case K_QD:
    case K_QI: g = {1, {I_DIR}, {c->Ds}, S_Q}; break;
    case K_DXYZ:
      if (f->which == 0) g = {1, {I_ZI}, {c->nxs}, S_RX};
      else if (f->which == 1) g = {1, {I_ZJ}, {c->nys}, S_RY};
      else g = {1, {I_ZK}, {c->nzs}, S_RZ};
      break;
    case K_VOL:
    case K_ZI: g = {1, {I_ZONE}, {c->Zs}, S_R}; break;
    case K_MI:
    case K_MD: {
      int64_t n = 0;
      if (ch < (int)c->zmap[1].size())
        for (int v : c->zmap[1][ch]) n += v;
      g = {1, {I_MIX}, {n}, S_R};
      break;
    }
    case K_M2L: g = {1, {I_MOM}, {c->M}, S_NULL}; break;
  }
  return g;
}

bool isIntKind(Kind k) { return k == K_QI || k == K_ZI || k == K_MI || k == K_M2L; }

int64_t chunkElems(const ChunkGeom &g) {
  int64_t n = 1;
  for (int k = 0; k < g.nd; ++k) n *= g.dims[k];
  return n;
}

int numChunks(const kgb_ctx *c, const FieldInfo *f) { return c->dc.chunks(chunkGeom(c, f, 0).space); }

int64_t fieldBytes(const kgb_ctx *c, const FieldInfo *f) {
  int64_t n = 0;
  const int nch = numChunks(c, f);
  for (int ch = 0; ch < nch; ++ch) n += chunkElems(chunkGeom(c, f, ch));
  return n * (isIntKind(f->kind) ? 4 : 8);
}

template <typename T>
T *as(void *p) {
  return reinterpret_cast<T *>(p);
}

int ensureStaging(kgb_ctx *ctx, size_t bytes) {
  if (bytes <= ctx->staging_bytes) return KGB_OK;
  if (ctx->staging) cudaFree(ctx->staging);
  ctx->staging = nullptr;
  ctx->staging_bytes = 0;
  cudaError_t e = cudaMalloc(&ctx->staging, bytes);
  if (e != cudaSuccess) return fail(ctx, KGB_ERR_OOM, "staging allocation failed");
  ctx->staging_bytes = bytes;
  return KGB_OK;
}

// Device descriptor of one chunk of a device-transposed field.
XposeDesc chunkXpose(const kgb_ctx *c, const FieldInfo *f, int ch) {
  ChunkGeom g = chunkGeom(c, f, ch);
  XposeDesc x{};
  x.nd = g.nd;
  for (int k = 0; k < g.nd; ++k) x.n[k] = g.dims[k];
  nestStrides(c->dims.layout, g.nd, g.types, g.dims, x.hs);
  int co[5];
  c->dc.chunkCoord(g.space, ch, co);
  const int glo = co[0] * c->Gs, dlo = co[1] * c->Ds;
  x.nxs = c->nxs;
  x.nys = c->nys;
  x.io = co[2] * c->nxs;
  x.jo = co[3] * c->nys;
  x.ko = co[4] * c->nzs;
  x.nx = c->nx;
  x.ny = c->ny;
  x.zdim = -1;
  switch (f->kind) {
    case K_FLUX:  // (d, g, z) -> ((zg*G + glo+g)*D + dlo+d)
      x.os[0] = 1; x.os[1] = c->D; x.os[2] = (int64_t)c->G * c->D; x.zdim = 2;
      x.obase = (int64_t)glo * c->D + dlo;
      x.iter[0] = 2; x.iter[1] = 1; x.iter[2] = 0;
      break;
    case K_MOM:  // (m, g, z) -> ((zg*G + glo+g)*M + m)
      x.os[0] = 1; x.os[1] = c->M; x.os[2] = (int64_t)c->G * c->M; x.zdim = 2;
      x.obase = (int64_t)glo * c->M;
      x.iter[0] = 2; x.iter[1] = 1; x.iter[2] = 0;
      break;
    case K_SIGT:  // (g, z) -> zg*G + glo+g
      x.os[0] = 1; x.os[1] = c->G; x.zdim = 1;
      x.obase = glo;
      x.iter[0] = 1; x.iter[1] = 0;
      break;
    case K_PLANE: {  // (d, g, a, b) -> ((b*na + a)*Gs + g)*Ds + d within the subdomain's chunk
      const int64_t na = g.dims[2];
      x.os[0] = 1; x.os[1] = c->Ds; x.os[2] = (int64_t)c->Gs * c->Ds; x.os[3] = na * c->Gs * c->Ds;
      x.obase = (int64_t)ch * c->plane_chunk[f->which];
      x.iter[0] = 3; x.iter[1] = 2; x.iter[2] = 1; x.iter[3] = 0;
      break;
    }
    default: break;
  }
  return x;
}

bool deviceKind(Kind k) { return k == K_FLUX || k == K_MOM || k == K_PLANE || k == K_SIGT; }

void *deviceArray(kgb_ctx *c, const FieldInfo *f) {
  switch (f->kind) {
    case K_FLUX: return f->which == 0 ? c->psi : c->rhs;
    case K_MOM: return f->which == 0 ? c->phi : c->phi_out;
    case K_PLANE: return c->plane[f->which];
    case K_SIGT: return c->sigt;
    default: return nullptr;
  }
}

int64_t deviceElems(const kgb_ctx *c, const FieldInfo *f) {
  switch (f->kind) {
    case K_FLUX: return c->Z * c->G * c->D;
    case K_MOM: return c->Z * c->G * c->M;
    case K_PLANE: return c->plane_chunk[f->which] * c->dc.num();
    case K_SIGT: return c->Z * c->G;
    default: return 0;
  }
}

template <typename T>
int dmalloc(kgb_ctx *ctx, T **p, size_t n) {
  cudaError_t e = cudaMalloc((void **)p, std::max<size_t>(n, 1) * sizeof(T));
  if (e != cudaSuccess) return fail(ctx, KGB_ERR_OOM, "device allocation failed");
  return KGB_OK;
}

int dalloc(kgb_ctx *ctx, void **p, size_t bytes) {
  cudaError_t e = cudaMalloc(p, std::max<size_t>(bytes, 1));
  if (e != cudaSuccess) return fail(ctx, KGB_ERR_OOM, "device allocation failed (" + std::to_string(bytes) + " bytes)");
  e = cudaMemsetAsync(*p, 0, std::max<size_t>(bytes, 1), ctx->stream);
  if (e != cudaSuccess) return fail(ctx, KGB_ERR_CUDA, "memset failed");
  return KGB_OK;
}

void dropSolveGraphs(kgb_ctx *c) {
  for (auto &e : c->solve_graphs) {
    cudaGraphExecDestroy(e.x);
    cudaGraphDestroy(e.g);
  }
  c->solve_graphs.clear();
}

void freeAll(kgb_ctx *c) {
  dropSolveGraphs(c);
  ++c->gen;
  void *ptrs[] = {c->psi, c->rhs, c->phi, c->phi_out, c->sigt, c->plane[0], c->plane[1], c->plane[2], c->ell, c->ellp,
                  c->sigsT, c->cx, c->cy, c->cz, c->w_d, c->cos_d[0], c->cos_d[1], c->cos_d[2], c->vol_d,
                  c->dxyz_d[0], c->dxyz_d[1], c->dxyz_d[2], c->zmix_start, c->zmix_count, c->mix_mat, c->mix_zone,
                  c->mix_frac, c->gp_lo, c->gp_hi, c->sdoms_d, c->ident_d, c->levels_d, c->tiles_d, c->partials,
                  c->results, c->parts_dev, c->staging, c->cls_d, c->inv_d, c->pop_slots, c->tc_lt_img,
                  c->tc_lp_img, c->tc_lt_exp, c->tc_lp_exp, c->err_d, c->lam, c->phi_prev, c->sigsT_adj,
                  c->gp_lo_adj, c->gp_hi_adj, c->colsum_d, c->e0_d, c->det_d, c->norm_d, c->resp_part, c->resp_d,
                  c->tc_lt_img_adj, c->tc_lp_img_adj, c->tc_lt_exp_adj, c->tc_lp_exp_adj, c->tc_sc_img,
                  c->tc_sc_img_adj, c->tc_sc_exp, c->tc_sc_exp_adj, c->pure_z,  // mixed_z lies inside pure_z
                  c->psi_exp, c->phi_exp, c->tf32_lt_img, c->tf32_lp_img, c->tf32_lt_img_adj, c->tf32_lp_img_adj};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  c->psi = c->rhs = c->phi = c->phi_out = c->sigt = nullptr;
  c->psi_exp = c->phi_exp = nullptr;
  c->psi_exp_valid = false;
  c->tf32_lt_img = c->tf32_lp_img = c->tf32_lt_img_adj = c->tf32_lp_img_adj = nullptr;
  c->plane[0] = c->plane[1] = c->plane[2] = nullptr;
  c->ell = c->ellp = c->sigsT = c->cx = c->cy = c->cz = nullptr;
  c->w_d = c->vol_d = nullptr;
  for (int k = 0; k < 3; ++k) c->cos_d[k] = c->dxyz_d[k] = nullptr;
  c->zmix_start = c->zmix_count = c->mix_mat = c->mix_zone = nullptr;
  c->mix_frac = nullptr;
  c->gp_lo = c->gp_hi = nullptr;
  c->sdoms_d = nullptr;
  c->ident_d = c->levels_d = nullptr;
  c->tiles_d = nullptr;
  c->partials = c->results = c->parts_dev = c->staging = nullptr;
  c->cls_d = nullptr;
  c->inv_d = nullptr;
  c->pop_slots = nullptr;
  c->tc_lt_img = c->tc_lp_img = nullptr;
  c->tc_lt_exp = c->tc_lp_exp = nullptr;
  c->tc_lt = c->tc_lp = false;
  c->err_d = nullptr;
  c->lam = c->sigsT_adj = nullptr;
  c->phi_prev = c->colsum_d = c->e0_d = c->det_d = c->resp_part = c->resp_d = nullptr;
  c->gp_lo_adj = c->gp_hi_adj = nullptr;
  c->norm_d = nullptr;
  c->tc_lt_img_adj = c->tc_lp_img_adj = nullptr;
  c->tc_lt_exp_adj = c->tc_lp_exp_adj = nullptr;
  c->tc_lt_adj = c->tc_lp_adj = false;
  c->tc_sc_img = c->tc_sc_img_adj = nullptr;
  c->tc_sc_exp = c->tc_sc_exp_adj = nullptr;
  c->pure_z = c->mixed_z = nullptr;
  c->tc_sc = false;
  c->dirty_tcsc = true;
  c->nmixed_z = 0;
  c->resp_nb = 0;
  c->adj_stale = true;
  c->have_lam = false;
  c->flip = 0;
  c->npop_slots = 0;
  c->use_recip = false;
  c->staging_bytes = 0;
  c->nmix_cap = 0;
  c->parts_cap = 0;
  c->ready = false;
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

// ---------------------------------------------------------------------------
// Derived device tables (built lazily when inputs change)
// ---------------------------------------------------------------------------
template <typename T>
int uploadVec(kgb_ctx *ctx, void *dst, const std::vector<double> &src) {
  std::vector<T> tmp(src.begin(), src.end());
  CK(cudaMemcpyAsync(dst, tmp.data(), tmp.size() * sizeof(T), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));  // tmp goes out of scope
  return KGB_OK;
}

int need(kgb_ctx *ctx, std::initializer_list<const char *> names) {
  for (const char *n : names) {
    const FieldInfo *f = findField(n);
    if (!ctx->have[fieldIndex(f)]) return fail(ctx, KGB_ERR_STATE, std::string("input field '") + n + "' has not been uploaded");
  }
  return KGB_OK;
}

// Tabulated sweep reciprocals.  On a uniform mesh the per-cell denominator
// ((2mu/dx + 2eta/dy) + 2xi/dz) + sigt depends on the direction and on the
// zone's sigt value alone; the distinct sigt values are few (mixtures of three
// materials), so 1/den is tabulated per (class, direction) and each (zone,
// group) stores its class.  The denominator is formed exactly as the sweep
// forms it, in the sweep's precision (FP64, or FP32 in the mixed form), and
// rounded once to its reciprocal.  Falls back to a per-cell divide when the
// mesh is not uniform or the classes do not fit 16 bits.
template <typename T>
int buildReciprocalsT(kgb_ctx *ctx) {
  for (int k = 0; k < 3; ++k)
    for (double v : ctx->dxyz[k])
      if (v != ctx->dxyz[k][0]) return KGB_OK;
  const int64_t n = ctx->Z * ctx->G;
  // distinct sigt values found on the device (hash table of bit patterns), sorted here
  const size_t nslot = (size_t)1 << kClassTableBits;
  unsigned long long *table = nullptr;
  int *ovf = nullptr;
  int rc;
  if ((rc = dmalloc(ctx, &table, nslot)) || (rc = dmalloc(ctx, &ovf, 1))) {
    cudaFree(table);
    return rc;
  }
  struct Free {
    void *a, *b;
    ~Free() { cudaFree(a); cudaFree(b); }
  } guard{table, ovf};
  std::vector<unsigned long long> keys(nslot);
  int overflow = 0;
  CK(cudaMemsetAsync(table, 0xFF, nslot * sizeof(unsigned long long), ctx->stream));
  CK(cudaMemsetAsync(ovf, 0, sizeof(int), ctx->stream));
  launch_class_insert<T>(as<T>(ctx->sigt), n, table, ovf, ctx->stream);
  CKN(1);
  CK(cudaMemcpyAsync(keys.data(), table, nslot * sizeof(unsigned long long), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(&overflow, ovf, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if (overflow) return KGB_OK;  // not tabulated: the sweep divides per cell
  std::vector<T> uniq;
  for (unsigned long long k : keys) {
    if (k == kClassEmpty) continue;
    T v;
    if constexpr (sizeof(T) == 8) std::memcpy(&v, &k, 8);
    else {
      const uint32_t b = (uint32_t)k;
      std::memcpy(&v, &b, 4);
    }
    uniq.push_back(v);
  }
  std::sort(uniq.begin(), uniq.end());
  uniq.erase(std::unique(uniq.begin(), uniq.end()), uniq.end());
  const int64_t ncls = (int64_t)uniq.size();
  if (ncls == 0 || ncls > 65535 || ncls * ctx->D > (int64_t)16 << 20) return KGB_OK;
  std::vector<T> inv((size_t)ncls * ctx->D);
  for (int64_t c = 0; c < ncls; ++c)
    for (int d = 0; d < ctx->D; ++d) {
      // the coefficient tables hold 2*cos/delta rounded to T
      const T cx = (T)(2.0 * ctx->q[0][d] / ctx->dxyz[0][0]);
      const T cy = (T)(2.0 * ctx->q[1][d] / ctx->dxyz[1][0]);
      const T cz = (T)(2.0 * ctx->q[2][d] / ctx->dxyz[2][0]);
      const T den = ((cx + cy) + cz) + uniq[c];
      inv[(size_t)c * ctx->D + d] = T(1) / den;
    }
  if (ctx->cls_d) cudaFree(ctx->cls_d);
  if (ctx->inv_d) cudaFree(ctx->inv_d);
  ctx->cls_d = nullptr;
  ctx->inv_d = nullptr;
  T *inv_d = nullptr, *uniq_d = nullptr;
  if ((rc = dmalloc(ctx, &ctx->cls_d, n)) || (rc = dmalloc(ctx, &inv_d, inv.size()))) return rc;
  ctx->inv_d = inv_d;
  if ((rc = dmalloc(ctx, &uniq_d, uniq.size()))) return rc;
  struct FreeU {
    void *a;
    ~FreeU() { cudaFree(a); }
  } guard_u{uniq_d};
  CK(cudaMemcpyAsync(uniq_d, uniq.data(), uniq.size() * sizeof(T), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(inv_d, inv.data(), inv.size() * sizeof(T), cudaMemcpyHostToDevice, ctx->stream));
  launch_class_lookup<T>(as<T>(ctx->sigt), n, uniq_d, (int)ncls, ctx->cls_d, ctx->stream);
  CKN(1);
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->ncls = ncls;
  ctx->use_recip = true;
  return KGB_OK;
}

int buildReciprocals(kgb_ctx *ctx) {
  ctx->use_recip = false;
  if (!ctx->allow_recip) return KGB_OK;
  return ctx->prec == KGB_FP64 ? buildReciprocalsT<double>(ctx) : buildReciprocalsT<float>(ctx);
}

// Plan the tensor-core LTimes / LPlusTimes: digit images of L and L+ and the
// shapes the kernel supports (exact diagonal sums need K <= 128 directions per
// launch in FP64 and <= 256 in the mixed form; moments fit one 32-wide K chunk).
// lt_src / lp_src: the [D][M] host tables the LTimes / LPlusTimes operators
// read (ell and ell_plus for the forward iteration, exchanged for the adjoint).
template <typename T>
int planTensorMomentsFrom(kgb_ctx *ctx, const std::vector<double> &lt_src, const std::vector<double> &lp_src,
                          bool *lt_ok, uint16_t **lt_img, int **lt_exp, int *lt_kpad, bool *lp_ok, uint16_t **lp_img,
                          int **lp_exp, int *lp_nhalf) {
  *lt_ok = *lp_ok = false;
  if (!ctx->allow_tc) return KGB_OK;
  const int S = tcDigits<T>();
  const int D = ctx->D, M = ctx->M;
  auto upload = [&](uint16_t **img_d, int **exp_d, const std::vector<uint16_t> &img, const std::vector<int> &ex) {
    if (*img_d) cudaFree(*img_d);
    if (*exp_d) cudaFree(*exp_d);
    *img_d = nullptr;
    *exp_d = nullptr;
    int r;
    if ((r = dmalloc(ctx, img_d, img.size())) || (r = dmalloc(ctx, exp_d, ex.size()))) return r;
    if (cudaMemcpyAsync(*img_d, img.data(), img.size() * 2, cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess ||
        cudaMemcpyAsync(*exp_d, ex.data(), ex.size() * 4, cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess ||
        cudaStreamSynchronize(ctx->stream) != cudaSuccess)
      return fail(ctx, KGB_ERR_CUDA, "tensor plan upload failed");
    return (int)KGB_OK;
  };
  std::vector<uint16_t> img;
  std::vector<int> ex;
  int rc;
  // LTimes: B[d][m] = ell(m,d), K = D, N = M (one 32-wide block).  Exact diagonal
  // sums (at most S digit pairs of magnitude 128^2 per direction, below 2^24) hold
  // for at most 128 directions, so larger D runs in K chunks of equal width kc (a
  // multiple of 32), each with its own digit image, the chunk results added in the
  // output precision.  *lt_kpad = kc.
  if (M <= 32) {
    const int kmax = 128;
    static_assert(tcDigits<double>() * 128 * 128 * 128 < (1 << 24), "exact FP32 diagonal sums");
    const int nk = (D + kmax - 1) / kmax;
    const int kc = ((D + nk - 1) / nk + 31) / 32 * 32;
    std::vector<uint16_t> all;
    std::vector<int> allex;
    for (int k0 = 0; k0 < D; k0 += kc) {
      tc_build_b<T>(lt_src.data() + (size_t)k0 * M, std::min(kc, D - k0), M, kc, S, 32, 1, img, ex);
      all.insert(all.end(), img.begin(), img.end());
      allex.insert(allex.end(), ex.begin(), ex.end());
    }
    if ((rc = upload(lt_img, lt_exp, all, allex))) return rc;
    *lt_kpad = kc;
    *lt_ok = true;
  }
  // LPlusTimes: B[m][d] = ell_plus(d,m), K = M (one chunk), N = D in blocks of NB = 32;
  // the B image and two A stages must fit the 227 KB of shared memory
  if (M <= 32) {
    const int NB = 32;
    const int nhalf = (D + NB - 1) / NB;
    const size_t stage = (size_t)S * 32 * 128 * 2;
    const size_t smem1 = 1024 + (size_t)nhalf * 32 * S * NB * 2 + stage + 4 * nhalf * NB;
    // + the kernel's static shared memory; the output staging of 16 warps (32 rows x 5
    // values each) when it fits, then a second A stage when that fits too (overlap across tiles)
    const size_t lim = 227 * 1024 - 4096, stg = 16 * 32 * 5 * sizeof(T);
    ctx->tc_lp_stage_out = smem1 + stg <= lim ? 1 : 0;
    ctx->tc_lp_stages = smem1 + stage + (ctx->tc_lp_stage_out ? stg : 0) <= lim ? 2 : 1;
    if (smem1 <= lim) {
      std::vector<double> bt((size_t)M * D);
      for (int d = 0; d < D; ++d)
        for (int m = 0; m < M; ++m) bt[(size_t)m * D + d] = lp_src[(size_t)d * M + m];
      tc_build_b<T>(bt.data(), M, D, 32, S, NB, nhalf, img, ex);
      if ((rc = upload(lp_img, lp_exp, img, ex))) return rc;
      *lp_nhalf = nhalf;
      *lp_ok = true;
    }
  }
  return KGB_OK;
}

// Split-TF32 plan of the mixed form: TF32 hi/lo images of L (K = directions,
// N = moments padded to 16 or 32) and of L+ (K = moments padded to 32, N =
// directions) from the [D][M] host tables the two operators read.
int planTf32From(kgb_ctx *ctx, const std::vector<double> &lt_src, const std::vector<double> &lp_src, float **lt_img,
                 float **lp_img) {
  for (float **p : {lt_img, lp_img}) {
    if (*p) cudaFree(*p);
    *p = nullptr;
  }
  if (ctx->prec != KGB_MIXED || !ctx->allow_tf32) return KGB_OK;
  const int D = ctx->D, M = ctx->M;
  auto upload = [&](float **dst, const std::vector<float> &img) -> int {
    int r;
    if ((r = dmalloc(ctx, dst, img.size()))) return r;
    if (cudaMemcpyAsync(*dst, img.data(), img.size() * sizeof(float), cudaMemcpyHostToDevice, ctx->stream) !=
            cudaSuccess ||
        cudaStreamSynchronize(ctx->stream) != cudaSuccess)
      return fail(ctx, KGB_ERR_CUDA, "TF32 plan upload failed");
    return (int)KGB_OK;
  };
  std::vector<float> b, img;
  int rc;
  if (tf32_ltimes_applies(D, M)) {
    b.assign((size_t)D * M, 0.0f);  // B[d][m] = L(m, d), stored [D][M]
    for (size_t i = 0; i < b.size(); ++i) b[i] = (float)lt_src[i];
    tf32_build_b(b.data(), D, M, (D + 31) / 32 * 32, M <= 16 ? 16 : 32, img);
    if ((rc = upload(lt_img, img))) return rc;
  }
  if (tf32_lplustimes_applies(D, M)) {
    b.assign((size_t)M * D, 0.0f);  // B[m][d] = L+(d, m)
    for (int d = 0; d < D; ++d)
      for (int m = 0; m < M; ++m) b[(size_t)m * D + d] = (float)lp_src[(size_t)d * M + m];
    tf32_build_b(b.data(), M, D, 32, D, img);
    if ((rc = upload(lp_img, img))) return rc;
  }
  return KGB_OK;
}

bool tf32LtActive(const kgb_ctx *ctx) {
  return ctx->prec == KGB_MIXED && ctx->allow_tf32 && ctx->use_tf32_lt && ctx->tf32_lt_img != nullptr;
}
bool tf32LpActive(const kgb_ctx *ctx) {
  return ctx->prec == KGB_MIXED && ctx->allow_tf32 && ctx->use_tf32_lp && ctx->tf32_lp_img != nullptr;
}

template <typename T>
int planTensorMoments(kgb_ctx *ctx) {
  return planTensorMomentsFrom<T>(ctx, ctx->ell_h, ctx->ellp_h, &ctx->tc_lt, &ctx->tc_lt_img, &ctx->tc_lt_exp,
                                  &ctx->tc_lt_kpad, &ctx->tc_lp, &ctx->tc_lp_img, &ctx->tc_lp_exp, &ctx->tc_lp_nhalf);
}

// Tensor-core scattering plan: the single-material zones of each material take
// phi_out(z, ., m) = S(mat, l(m)) phi(z, ., m) as tcgen05 row products over
// (zone, moment) rows with the exact digit products of the moment transforms
// (K = N = groups <= 64); zones with several materials keep the SIMT kernel.
template <typename T>
int planTensorScatter(kgb_ctx *ctx) {
  ctx->tc_sc = false;
  const int G = ctx->G, L1 = ctx->L + 1, S = tcDigits<T>(), NB = 32;
  if (!ctx->allow_tc_sc || G > 64) return KGB_OK;
  // zone lists from the device mixing tables
  std::vector<int> zs(ctx->Z), zc(ctx->Z), mm(std::max<int64_t>(ctx->nmix, 1));
  std::vector<double> mf(std::max<int64_t>(ctx->nmix, 1));
  CK(cudaMemcpyAsync(zs.data(), ctx->zmix_start, ctx->Z * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(zc.data(), ctx->zmix_count, ctx->Z * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  if (ctx->nmix > 0) {
    CK(cudaMemcpyAsync(mm.data(), ctx->mix_mat, ctx->nmix * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(mf.data(), ctx->mix_frac, ctx->nmix * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  }
  CK(cudaStreamSynchronize(ctx->stream));
  std::vector<int> pure[3], mixed;
  for (int64_t z = 0; z < ctx->Z; ++z) {
    if (zc[z] == 1 && mf[zs[z]] == 1.0) pure[mm[zs[z]]].push_back((int)z);
    else mixed.push_back((int)z);
  }
  std::vector<int> lists;
  for (int m = 0; m < 3; ++m) {
    ctx->pure_off[m] = (int64_t)lists.size();
    lists.insert(lists.end(), pure[m].begin(), pure[m].end());
  }
  ctx->pure_off[3] = (int64_t)lists.size();
  ctx->nmixed_z = (int64_t)mixed.size();
  lists.insert(lists.end(), mixed.begin(), mixed.end());
  if (ctx->pure_z) cudaFree(ctx->pure_z);
  ctx->pure_z = ctx->mixed_z = nullptr;
  int rc;
  if ((rc = dmalloc(ctx, &ctx->pure_z, lists.size()))) return rc;
  ctx->mixed_z = ctx->pure_z + ctx->pure_off[3];
  CK(cudaMemcpyAsync(ctx->pure_z, lists.data(), lists.size() * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
  // digit images (N blocks of 32 columns): forward B[k][n] = S(n <- k), adjoint B[k][n] = S(k <- n)
  const int kpad = (G + 31) / 32 * 32, nbk = (G + 31) / 32;
  std::vector<double> b((size_t)G * G);
  std::vector<uint16_t> img, all;
  std::vector<int> ex, allex;
  for (int adj = 0; adj < 2; ++adj) {
    all.clear();
    allex.clear();
    for (int m = 0; m < 3; ++m)
      for (int l = 0; l < L1; ++l) {
        const double *sm = ctx->sigs_h.data() + ((size_t)m * L1 + l) * G * G;
        for (int k = 0; k < G; ++k)
          for (int n = 0; n < G; ++n) b[(size_t)k * G + n] = adj ? sm[(size_t)k * G + n] : sm[(size_t)n * G + k];
        tc_build_b<T>(b.data(), G, G, kpad, S, NB, nbk, img, ex);
        all.insert(all.end(), img.begin(), img.end());
        allex.insert(allex.end(), ex.begin(), ex.end());
      }
    uint16_t *&dimg = adj ? ctx->tc_sc_img_adj : ctx->tc_sc_img;
    int *&dexp = adj ? ctx->tc_sc_exp_adj : ctx->tc_sc_exp;
    if (dimg) cudaFree(dimg);
    if (dexp) cudaFree(dexp);
    dimg = nullptr;
    dexp = nullptr;
    if ((rc = dmalloc(ctx, &dimg, all.size())) || (rc = dmalloc(ctx, &dexp, allex.size()))) return rc;
    CK(cudaMemcpyAsync(dimg, all.data(), all.size() * sizeof(uint16_t), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(dexp, allex.data(), allex.size() * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));  // the host vectors are reused
  }
  ctx->tc_sc_kpad = kpad;
  ctx->tc_sc = true;
  return KGB_OK;
}

// w(d) / ell(0,d) when it is the same for every direction (Kripke's L: ell(0,d) =
// w(d) Y_00 / sqrt(4 pi)), else 0: the particle count then comes from psi.
void updatePopScale(kgb_ctx *ctx) {
  const std::vector<double> &w = ctx->q[3];
  const double e0 = ctx->ell_h[0];
  double s = e0 != 0.0 ? w[0] / e0 : 0.0;
  for (int d = 0; d < ctx->D && s != 0.0; ++d) {
    const double e = ctx->ell_h[(size_t)d * ctx->M];
    if (!(std::fabs(w[d] - s * e) <= 1e-14 * std::fabs(w[d]))) s = 0.0;
  }
  ctx->pop_scale = s;
}

template <typename T>
int prepareT(kgb_ctx *ctx) {
  int rc;
  const bool popscale_stale = ctx->dirty_quad || ctx->dirty_ell;
  if (ctx->dirty_quad) {
    if ((rc = need(ctx, {"quadrature/xcos", "quadrature/ycos", "quadrature/zcos", "quadrature/w", "quadrature/id",
                         "quadrature/jd", "quadrature/kd"})))
      return rc;
    CK(cudaMemcpyAsync(ctx->w_d, ctx->q[3].data(), ctx->D * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    for (int k = 0; k < 3; ++k)
      CK(cudaMemcpyAsync(ctx->cos_d[k], ctx->q[k].data(), ctx->D * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    // sweep descriptors: every direction of a subdomain follows its first direction's traversal
    ctx->sdoms_h.resize(ctx->dc.num());
    for (int s = 0; s < ctx->dc.num(); ++s) {
      int co[5];
      ctx->dc.coord(s, co);
      SdomDesc &d = ctx->sdoms_h[s];
      d.p = co[0]; d.q = co[1]; d.xs = co[2]; d.ys = co[3]; d.zs = co[4];
      d.glo = co[0] * ctx->Gs;
      d.dlo = co[1] * ctx->Ds;
      d.io = co[2] * ctx->nxs; d.jo = co[3] * ctx->nys; d.ko = co[4] * ctx->nzs;
      d.id = ctx->qi[0][d.dlo]; d.jd = ctx->qi[1][d.dlo]; d.kd = ctx->qi[2][d.dlo];
      d.ip = (int64_t)s * ctx->plane_chunk[0];
      d.jp = (int64_t)s * ctx->plane_chunk[1];
      d.kp = (int64_t)s * ctx->plane_chunk[2];
    }
    CK(cudaMemcpyAsync(ctx->sdoms_d, ctx->sdoms_h.data(), ctx->sdoms_h.size() * sizeof(SdomDesc), cudaMemcpyHostToDevice, ctx->stream));
    // zone-set waves in upwind order (level = oriented zone-set coordinate sum)
    const int S[3] = {ctx->dc.Sx, ctx->dc.Sy, ctx->dc.Sz};
    int nlev = S[0] + S[1] + S[2] - 2;
    std::vector<std::vector<int>> lv(nlev);
    for (int s = 0; s < ctx->dc.num(); ++s) {
      const SdomDesc &d = ctx->sdoms_h[s];
      int ox = d.id > 0 ? d.xs : S[0] - 1 - d.xs;
      int oy = d.jd > 0 ? d.ys : S[1] - 1 - d.ys;
      int oz = d.kd > 0 ? d.zs : S[2] - 1 - d.zs;
      lv[ox + oy + oz].push_back(s);
    }
    ctx->level_off.assign(1, 0);
    ctx->level_sdoms.clear();
    for (auto &v : lv) {
      for (int s : v) ctx->level_sdoms.push_back(s);
      ctx->level_off.push_back((int)ctx->level_sdoms.size());
    }
    CK(cudaMemcpyAsync(ctx->levels_d, ctx->level_sdoms.data(), ctx->level_sdoms.size() * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    ctx->dirty_quad = false;
    ++ctx->gen;
    ctx->dirty_geom = true;
    ctx->adj_stale = true;
  }
  if (ctx->dirty_geom) {
    if ((rc = need(ctx, {"dx", "dy", "dz"}))) return rc;
    const int n[3] = {ctx->nx, ctx->ny, ctx->nz};
    void *dst[3] = {ctx->cx, ctx->cy, ctx->cz};
    for (int k = 0; k < 3; ++k) {
      // 2*cos/delta exactly as the reference forms it per cell (SweepSubdomain.cpp:174-176)
      std::vector<double> t((size_t)ctx->D * n[k]);
      for (int d = 0; d < ctx->D; ++d)
        for (int i = 0; i < n[k]; ++i) t[(size_t)d * n[k] + i] = 2.0 * ctx->q[k][d] / ctx->dxyz[k][i];
      if ((rc = uploadVec<T>(ctx, dst[k], t))) return rc;
      CK(cudaMemcpyAsync(ctx->dxyz_d[k], ctx->dxyz[k].data(), n[k] * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    }
    CK(cudaStreamSynchronize(ctx->stream));
    ctx->dirty_geom = false;
    ++ctx->gen;
    ctx->dirty_sigt = true;  // the tabulated reciprocals depend on 2*cos/delta
  }
  if (ctx->dirty_ell) {
    if ((rc = need(ctx, {"ell", "ell_plus"}))) return rc;
    if ((rc = uploadVec<T>(ctx, ctx->ell, ctx->ell_h))) return rc;
    if ((rc = uploadVec<T>(ctx, ctx->ellp, ctx->ellp_h))) return rc;
    if ((rc = planTensorMoments<T>(ctx))) return rc;
    if ((rc = planTf32From(ctx, ctx->ell_h, ctx->ellp_h, &ctx->tf32_lt_img, &ctx->tf32_lp_img))) return rc;
    ctx->dirty_ell = false;
    ++ctx->gen;
    ctx->adj_stale = true;
  }
  if (ctx->dirty_sigs) {
    if ((rc = need(ctx, {"data/sigs"}))) return rc;
    const int G = ctx->G, L1 = ctx->L + 1;
    std::vector<double> t((size_t)3 * L1 * G * G);
    std::vector<int> lo(G, G), hi(G, -1);
    for (int m = 0; m < 3; ++m)
      for (int l = 0; l < L1; ++l)
        for (int g = 0; g < G; ++g)
          for (int gp = 0; gp < G; ++gp) {
            double v = ctx->sigs_h[(((size_t)m * L1 + l) * G + g) * G + gp];
            t[(((size_t)m * L1 + l) * G + gp) * G + g] = v;
            if (v != 0.0) {
              lo[g] = std::min(lo[g], gp);
              hi[g] = std::max(hi[g], gp);
            }
          }
    if ((rc = uploadVec<T>(ctx, ctx->sigsT, t))) return rc;
    CK(cudaMemcpyAsync(ctx->gp_lo, lo.data(), G * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->gp_hi, hi.data(), G * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    ctx->dirty_sigs = false;
    ctx->dirty_tcsc = true;
    ++ctx->gen;
    ctx->adj_stale = true;
  }
  if (ctx->dirty_vol) {
    if ((rc = need(ctx, {"volume"}))) return rc;
    CK(cudaMemcpyAsync(ctx->vol_d, ctx->vol_h.data(), ctx->Z * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    ctx->vol_uniform = ctx->vol_h[0];
    for (double v : ctx->vol_h)
      if (v != ctx->vol_uniform || !(v > 0.0)) { ctx->vol_uniform = 0.0; break; }
    ctx->dirty_vol = false;
    ++ctx->gen;
  }
  if (ctx->dirty_mix) {
    if ((rc = need(ctx, {"zone_to_mixelem", "zone_to_num_mixelem", "mixelem_to_zone", "mixelem_to_material",
                         "mixelem_to_fraction"})))
      return rc;
    const int nr = ctx->dc.chunks(S_R);
    int64_t total = 0;
    for (int r = 0; r < nr; ++r) total += (int64_t)ctx->mfrac[r].size();
    if (total > ctx->nmix_cap) {
      for (void *p : {(void *)ctx->mix_mat, (void *)ctx->mix_zone, (void *)ctx->mix_frac})
        if (p) cudaFree(p);
      ctx->mix_mat = ctx->mix_zone = nullptr;
      ctx->mix_frac = nullptr;
      if ((rc = dmalloc(ctx, &ctx->mix_mat, total)) || (rc = dmalloc(ctx, &ctx->mix_zone, total)) ||
          (rc = dmalloc(ctx, &ctx->mix_frac, total)))
        return rc;
      ctx->nmix_cap = total;
    }
    std::vector<int> zstart(ctx->Z, 0), zcount(ctx->Z, 0), mmat(total), mzone(total);
    std::vector<double> mfr(total);
    int64_t off = 0;
    for (int r = 0; r < nr; ++r) {
      int co[5];
      ctx->dc.chunkCoord(S_R, r, co);
      const int io = co[2] * ctx->nxs, jo = co[3] * ctx->nys, ko = co[4] * ctx->nzs;
      auto glob = [&](int64_t zl) {
        int64_t i = zl % ctx->nxs, j = (zl / ctx->nxs) % ctx->nys, k = zl / ((int64_t)ctx->nxs * ctx->nys);
        return ((k + ko) * ctx->ny + (j + jo)) * ctx->nx + (i + io);
      };
      const int64_t nm = (int64_t)ctx->mfrac[r].size();
      for (int64_t zl = 0; zl < ctx->Zs; ++zl) {
        const int64_t zg = glob(zl);
        const int st = ctx->zmap[0][r][zl], cn = ctx->zmap[1][r][zl];
        if (st < 0 || cn < 0 || st + cn > nm) return fail(ctx, KGB_ERR_ARG, "zone_to_mixelem out of range");
        zstart[zg] = (int)(off + st);
        zcount[zg] = cn;
      }
      for (int64_t m = 0; m < nm; ++m) {
        const int zl = ctx->mimap[0][r][m], mat = ctx->mimap[1][r][m];
        if (zl < 0 || zl >= ctx->Zs || mat < 0 || mat > 2) return fail(ctx, KGB_ERR_ARG, "mixelem map out of range");
        mzone[off + m] = (int)glob(zl);
        mmat[off + m] = mat;
        mfr[off + m] = ctx->mfrac[r][m];
      }
      off += nm;
    }
    ctx->nmix = total;
    CK(cudaMemcpyAsync(ctx->zmix_start, zstart.data(), ctx->Z * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->zmix_count, zcount.data(), ctx->Z * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->mix_mat, mmat.data(), total * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->mix_zone, mzone.data(), total * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->mix_frac, mfr.data(), total * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    ctx->dirty_mix = false;
    ctx->dirty_tcsc = true;
    ++ctx->gen;
  }
  if (popscale_stale) updatePopScale(ctx);
  if (ctx->dirty_tcsc) {
    if ((rc = planTensorScatter<T>(ctx))) return rc;
    ctx->dirty_tcsc = false;
    ++ctx->gen;
  }
  if (ctx->dirty_sigt) {
    if ((rc = need(ctx, {"sigt_zonal"}))) return rc;
    if ((rc = buildReciprocals(ctx))) return rc;
    ctx->dirty_sigt = false;
    ++ctx->gen;
  }
  if (sizeof(T) == 8 && !ctx->psi_exp) {
    if ((rc = dmalloc(ctx, &ctx->psi_exp, (size_t)(ctx->Z * ctx->G)))) return rc;
    ctx->psi_exp_valid = false;
  }
  if (!ctx->phi_exp && (rc = dmalloc(ctx, &ctx->phi_exp, (size_t)(ctx->Z * ctx->M)))) return rc;
  return KGB_OK;
}

int prepare(kgb_ctx *ctx) {
  if (!ctx) return KGB_ERR_ARG;
  if (!ctx->ready) return fail(ctx, KGB_ERR_STATE, "kgb_setup has not been called");
  CK(cudaSetDevice(ctx->device));
  return ctx->prec == KGB_FP64 ? prepareT<double>(ctx) : prepareT<float>(ctx);
}

int buildTiles(kgb_ctx *ctx) {
  ++ctx->gen;
  const int ntx = (ctx->nxs + ctx->tx - 1) / ctx->tx;
  const int nty = (ctx->nys + ctx->ty - 1) / ctx->ty;
  const int ntz = (ctx->nzs + ctx->tz - 1) / ctx->tz;
  ctx->nsteps = ntx + nty + ntz - 2;
  std::vector<int4> tiles;
  ctx->tile_off.assign(1, 0);
  for (int s = 0; s < ctx->nsteps; ++s) {
    for (int c = 0; c < ntz; ++c)
      for (int b = 0; b < nty; ++b) {
        int a = s - b - c;
        if (a >= 0 && a < ntx) tiles.push_back(make_int4(a, b, c, 0));
      }
    ctx->tile_off.push_back((int)tiles.size());
  }
  if (ctx->tiles_d) cudaFree(ctx->tiles_d);
  ctx->tiles_d = nullptr;
  int rc = dmalloc(ctx, &ctx->tiles_d, tiles.size());
  if (rc) return rc;
  const int64_t nchain = (int64_t)ctx->Gs * ctx->Ds;
  const int64_t nslots = (int64_t)tiles.size() * ctx->dc.num() * ((nchain + kSweepThreads - 1) / kSweepThreads);
  if (ctx->pop_slots) cudaFree(ctx->pop_slots);
  ctx->pop_slots = nullptr;
  if ((rc = dmalloc(ctx, &ctx->pop_slots, nslots))) return rc;
  ctx->npop_slots = nslots;
  CK(cudaMemcpyAsync(ctx->tiles_d, tiles.data(), tiles.size() * sizeof(int4), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return KGB_OK;
}

// ---------------------------------------------------------------------------
// Kernel drivers
// ---------------------------------------------------------------------------
// Lanes of one group in the sweep's chain order (chains run over a direction
// set's directions fastest), for the sweep's row-exponent reduction; 0 when a
// warp's groups are not aligned runs of a power-of-two length.
int psiExpWidth(const kgb_ctx *ctx) {
  const int ds = ctx->Ds;
  if (ds % 32 == 0) return 32;
  return (ds > 0 && ds < 32 && (ds & (ds - 1)) == 0) ? ds : 0;
}

// The solver's sweep records psi's row exponents for the next tensor-core
// LTimes (FP64, every direction in one K chunk), which then skips its own pass
// over each row.
bool psiExpUsable(const kgb_ctx *ctx) {
  return ctx->prec == KGB_FP64 && ctx->allow_row_exp && ctx->psi_exp && ctx->tc_lt && ctx->use_tc_lt &&
         ctx->D <= ctx->tc_lt_kpad && psiExpWidth(ctx) > 0;
}

// Lanes of one zone in the tensor-core LTimes' epilogue (one lane per (zone,
// group) row): 32 when the group count is a multiple of 32, the group count
// when it is a smaller power of two, else 0.
int phiExpWidth(const kgb_ctx *ctx) {
  const int g = ctx->G;
  if (g % 32 == 0) return 32;
  return (g > 0 && g < 32 && (g & (g - 1)) == 0) ? g : 0;
}

// LTimes records phi's exponents per (zone, moment) for the tensor-core
// scattering of the same iteration, which then skips its own pass over each
// gathered row: the tensor-core LTimes in FP64 (one K chunk), the
// register-tiled SIMT LTimes in the mixed form.
bool phiExpUsable(const kgb_ctx *ctx) {
  if (!ctx->allow_row_exp || !ctx->phi_exp || !ctx->tc_sc || !ctx->use_tc_sc || phiExpWidth(ctx) == 0) return false;
  const bool tensor = ctx->tc_lt && ctx->use_tc_lt;
  if (ctx->prec == KGB_FP64) return tensor && ctx->D <= ctx->tc_lt_kpad;
  return !tensor && !tf32LtActive(ctx) && ltimes_tiled_applies(ctx->D, ctx->M);
}

// rowexp: record psi's row exponents there (the caller zeroed it); null: psi
// changes without them, so the recorded ones no longer hold.
template <typename T>
int sweepWave(kgb_ctx *ctx, const int *wave_dev, int nwave, bool fused_pop, bool fused_rhs, int *rowexp) {
  SweepArgs<T> a{};
  if (rowexp) {
    a.rowexp = rowexp;
    a.rexp_w = psiExpWidth(ctx);
  } else {
    ctx->psi_exp_valid = false;
  }
  if (fused_rhs) {
    a.phiout = as<T>(ctx->phi_out);
    a.ellp = as<T>(ctx->ellp);
    a.M = ctx->M;
  }
  a.rhs = as<T>(ctx->rhs);
  a.psi = as<T>(ctx->psi);
  a.sigt = as<T>(ctx->sigt);
  a.l2hints = ctx->sweep_l2_hints ? 1 : 0;
  a.iplane = as<T>(ctx->plane[0]);
  a.jplane = as<T>(ctx->plane[1]);
  a.kplane = as<T>(ctx->plane[2]);
  a.cx = as<T>(ctx->cx);
  a.cy = as<T>(ctx->cy);
  a.cz = as<T>(ctx->cz);
  a.sdoms = ctx->sdoms_d;
  a.wave = wave_dev;
  a.tiles = ctx->tiles_d;
  a.nx = ctx->nx; a.ny = ctx->ny; a.nz = ctx->nz;
  a.G = ctx->G; a.D = ctx->D; a.Gs = ctx->Gs; a.Ds = ctx->Ds;
  a.nxs = ctx->nxs; a.nys = ctx->nys; a.nzs = ctx->nzs;
  a.tz = ctx->tz;
  a.tx = ctx->tx;
  a.ty = ctx->ty;
  a.flip = ctx->flip;
  if (ctx->use_recip) {
    a.cls = ctx->cls_d;
    a.inv = as<T>(ctx->inv_d);
  }
  if (fused_pop) {
    a.pop = ctx->pop_slots;
    a.nsdom = ctx->dc.num();
    a.w = ctx->w_d;
    a.vol = ctx->vol_d;
    a.vol_uniform = ctx->vol_uniform;
  }
  FamScope fs(ctx, "sweep");
  // parts of the wave's subdomain list, one per stream
  const int np = std::max(1, std::min(ctx->sweep_streams, nwave));
  SweepArgs<T> part[kgb_ctx::kMaxSweepStreams];
  int pn[kgb_ctx::kMaxSweepStreams];
  for (int i = 0, off = 0; i < np; ++i) {
    pn[i] = nwave / np + (i < nwave % np ? 1 : 0);
    part[i] = a;
    part[i].wave = wave_dev + off;
    off += pn[i];
  }
  auto streamOf = [&](int i) { return i == 0 ? ctx->stream : ctx->aux[i - 1]; };
  if (np > 1) {
    CK(cudaEventRecord(ctx->fork_ev, ctx->stream));
    for (int i = 1; i < np; ++i) CK(cudaStreamWaitEvent(ctx->aux[i - 1], ctx->fork_ev, 0));
  }
  for (int s = 0; s < ctx->nsteps; ++s) {
    const int nt = ctx->tile_off[s + 1] - ctx->tile_off[s];
    if (nt == 0) continue;
    for (int i = 0; i < np; ++i) {
      part[i].tile_off = ctx->tile_off[s];
      launch_sweep_step<T>(part[i], nt, pn[i], streamOf(i));
      CKN(1);
    }
  }
  for (int i = 1; i < np; ++i) {
    CK(cudaEventRecord(ctx->join_ev[i - 1], ctx->aux[i - 1]));
    CK(cudaStreamWaitEvent(ctx->stream, ctx->join_ev[i - 1], 0));
  }
  return KGB_OK;
}

int sweepWaveAny(kgb_ctx *ctx, const int *wave_dev, int nwave, bool fused_pop = false, bool fused_rhs = false,
                 int *rowexp = nullptr) {
  return ctx->prec == KGB_FP64 ? sweepWave<double>(ctx, wave_dev, nwave, fused_pop, fused_rhs, rowexp)
                               : sweepWave<float>(ctx, wave_dev, nwave, fused_pop, fused_rhs, nullptr);
}

int fillField(kgb_ctx *ctx, const FieldInfo *f, double v) {
  ctx->psi_exp_valid = false;
  void *p = deviceArray(ctx, f);
  const int64_t n = deviceElems(ctx, f);
  if (!p) return fail(ctx, KGB_ERR_ARG, std::string("field '") + f->name + "' cannot be filled");
  if (v == 0.0) {
    CK(cudaMemsetAsync(p, 0, n * ctx->tsz, ctx->stream));
    // psi = 0 (Kripke's kConst(psi, 0) before a solve): its row exponents are 0
    if (p == ctx->psi && psiExpUsable(ctx)) {
      CK(cudaMemsetAsync(ctx->psi_exp, 0, ctx->Z * ctx->G * sizeof(int), ctx->stream));
      ctx->psi_exp_valid = true;
    }
  } else if (ctx->prec == KGB_FP64) {
    launch_fill<double>(as<double>(p), n, v, ctx->stream);
    CKN(1);
  } else {
    launch_fill<float>(as<float>(p), n, v, ctx->stream);
    CKN(1);
  }
  return KGB_OK;
}

// rowexp (FP64, optional): zeroed here and filled with psi's row exponents.
int sweepSolver(kgb_ctx *ctx, bool fused_pop = false, bool fused_rhs = false, int *rowexp = nullptr) {
  for (int k = 0; k < 3; ++k) CK(cudaMemsetAsync(ctx->plane[k], 0, ctx->plane_chunk[k] * ctx->dc.num() * ctx->tsz, ctx->stream));
  if (rowexp) CK(cudaMemsetAsync(rowexp, 0, ctx->Z * ctx->G * sizeof(int), ctx->stream));
  // Block Jacobi (BlockJacobiComm.cpp:46-98 with SweepSolver.cpp:28-30): the
  // planes every subdomain receives are the ones saved right after the zeroing
  // above, so no subdomain waits on another and none hands its outgoing planes
  // on.  One launch sweeps all of them, each from zero inflow on every face.
  if (ctx->block_jacobi) return sweepWaveAny(ctx, ctx->levels_d, ctx->dc.num(), fused_pop, fused_rhs, rowexp);
  const int nlev = (int)ctx->level_off.size() - 1;
  const int S[3] = {ctx->dc.Sx, ctx->dc.Sy, ctx->dc.Sz};
  // the reversed (adjoint) orientation visits the zone-set levels last to first
  const int sgn = ctx->flip ? -1 : 1;
  for (int step = 0; step < nlev; ++step) {
    const int lv = ctx->flip ? nlev - 1 - step : step;
    const int b = ctx->level_off[lv], e = ctx->level_off[lv + 1];
    if (e == b) continue;
    int rc = sweepWaveAny(ctx, ctx->levels_d + b, e - b, fused_pop, fused_rhs, rowexp);
    if (rc) return rc;
    // hand the outgoing planes to downwind zone sets (ParallelComm.cpp:146-162)
    for (int x = b; x < e; ++x) {
      const int s = ctx->level_sdoms[x];
      const SdomDesc &d = ctx->sdoms_h[s];
      int co[5] = {d.p, d.q, d.xs, d.ys, d.zs};
      const int dirv[3] = {sgn * d.id, sgn * d.jd, sgn * d.kd};
      for (int dim = 0; dim < 3; ++dim) {
        int dn[5] = {co[0], co[1], co[2], co[3], co[4]};
        dn[2 + dim] += dirv[dim];
        if (dn[2 + dim] < 0 || dn[2 + dim] >= S[dim]) continue;
        const int t = ctx->dc.sdomOf(dn);
        const size_t bytes = ctx->plane_chunk[dim] * ctx->tsz;
        char *base = (char *)ctx->plane[dim];
        CK(cudaMemcpyAsync(base + (size_t)t * bytes, base + (size_t)s * bytes, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
      }
    }
  }
  return KGB_OK;
}

ScatterArgsBase scatterArgs(kgb_ctx *ctx) {
  ScatterArgsBase a{};
  a.Z = ctx->Z;
  a.G = ctx->G;
  a.M = ctx->M;
  a.L = ctx->L;
  a.zmix_start = ctx->zmix_start;
  a.zmix_count = ctx->zmix_count;
  a.mix_mat = ctx->mix_mat;
  a.mix_frac = ctx->mix_frac;
  a.gp_lo = ctx->gp_lo;
  a.gp_hi = ctx->gp_hi;
  a.src_glo = 0;
  a.src_ghi = ctx->G;
  a.dst_glo = 0;
  a.dst_ghi = ctx->G;
  return a;
}

template <typename T>
void tcRows(kgb_ctx *ctx, const T *A, T *C, int lda, int ldc, int K, int kpad, int N, int nhalf, const uint16_t *img,
            const int *ex, bool acc, bool multi_n, const int *rowexp = nullptr, int *outexp = nullptr) {
  TcArgs<T> a{};
  a.rowexp = rowexp;
  if (outexp) {  // LTimes only: its outputs are staged
    a.outexp = outexp;
    a.outexp_w = phiExpWidth(ctx);
    a.outexp_rows = ctx->G;
  }
  a.A = A;
  a.C = C;
  a.rows = ctx->Z * ctx->G;
  a.lda = lda;
  a.ldc = ldc;
  a.K = K;
  a.kpad = kpad;
  a.N = N;
  a.nhalf = nhalf;
  a.bimg = img;
  a.bexp = ex;
  a.err = ctx->err_d;
  a.accumulate = acc;
  a.nsm = ctx->nsm;
  a.stages = multi_n ? ctx->tc_lp_stages : 2;
  a.stage_out = multi_n ? ctx->tc_lp_stage_out : 1;  // LTimes' B image is at most 64 KB: staging fits
  launch_tc_rows<T>(a, ctx->stream);
}

// rowexp: psi's row exponents recorded by the sweep that wrote it (FP64 tensor
// path with one K chunk), or null.  outexp: zeroed and filled with phi's
// exponents per (zone, moment) for the tensor-core scattering, or null.
int doLTimes(kgb_ctx *ctx, bool acc, const int *rowexp = nullptr, int *outexp = nullptr) {
  FamScope fs(ctx, "ltimes");
  const int64_t rows = ctx->Z * ctx->G;
  if (!outexp && tf32LtActive(ctx)) {  // mixed form: split-TF32 tensor cores
    if (launch_tf32_ltimes(as<float>(ctx->psi), as<float>(ctx->phi), rows, ctx->D, ctx->M, ctx->tf32_lt_img, acc,
                           ctx->err_d, ctx->nsm, ctx->stream))
      return fail(ctx, KGB_ERR_CUDA, "split-TF32 LTimes launch failed");
    CKN(1);
    return KGB_OK;
  }
  if (ctx->tc_lt && ctx->use_tc_lt) {
    // one launch per K chunk of kc directions (one chunk up to 128 FP64 / 256 FP32 directions)
    const int kc = ctx->tc_lt_kpad, S = ctx->prec == KGB_FP64 ? tcDigits<double>() : tcDigits<float>();
    for (int k0 = 0, c = 0; k0 < ctx->D; k0 += kc, ++c) {
      const int K = std::min(kc, ctx->D - k0);
      const uint16_t *img = ctx->tc_lt_img + (size_t)c * kc * S * 32;
      const int *ex = ctx->tc_lt_exp + (size_t)c * 32;
      if (ctx->prec == KGB_FP64) {
        const bool one = ctx->D <= kc && !acc;  // the records hold for a whole, fresh phi only
        if (outexp && !one) return fail(ctx, KGB_ERR_STATE, "phi exponent record needs one fresh LTimes launch");
        if (outexp) CK(cudaMemsetAsync(outexp, 0, ctx->Z * ctx->M * sizeof(int), ctx->stream));
        tcRows<double>(ctx, as<double>(ctx->psi) + k0, as<double>(ctx->phi), ctx->D, ctx->M, K, kc, ctx->M, 1, img,
                       ex, acc || c > 0, false, one ? rowexp : nullptr, outexp);
      } else {
        if (outexp) return fail(ctx, KGB_ERR_STATE, "phi exponent record: not on the FP32 tensor-core LTimes");
        tcRows<float>(ctx, as<float>(ctx->psi) + k0, as<float>(ctx->phi), ctx->D, ctx->M, K, kc, ctx->M, 1, img, ex,
                      acc || c > 0, false);
      }
      CKN(1);
    }
    return KGB_OK;
  }
  if (outexp) {  // mixed form: the register-tiled SIMT LTimes records phi's exponents
    if (ctx->prec != KGB_MIXED || acc) return fail(ctx, KGB_ERR_STATE, "phi exponent record needs a fresh LTimes");
    CK(cudaMemsetAsync(outexp, 0, ctx->Z * ctx->M * sizeof(int), ctx->stream));
    if (!launch_ltimes_record(as<float>(ctx->psi), as<float>(ctx->phi), as<float>(ctx->ell), rows, ctx->D, ctx->M,
                              outexp, phiExpWidth(ctx), ctx->G, ctx->stream))
      return fail(ctx, KGB_ERR_STATE, "phi exponent record needs the tiled LTimes");
    CKN(1);
    return KGB_OK;
  }
  if (ctx->prec == KGB_FP64)
    launch_ltimes<double>(as<double>(ctx->psi), as<double>(ctx->phi), as<double>(ctx->ell), rows, ctx->D, ctx->M, acc, ctx->stream);
  else
    launch_ltimes<float>(as<float>(ctx->psi), as<float>(ctx->phi), as<float>(ctx->ell), rows, ctx->D, ctx->M, acc, ctx->stream);
  CKN((ctx->M + 31) / 32);
  return KGB_OK;
}

int doLPlusTimes(kgb_ctx *ctx, bool acc) {
  FamScope fs(ctx, "lplustimes");
  ctx->rhs_stale = false;
  const int64_t rows = ctx->Z * ctx->G;
  if (tf32LpActive(ctx)) {  // mixed form: split-TF32 tensor cores
    if (launch_tf32_lplustimes(as<float>(ctx->phi_out), as<float>(ctx->rhs), rows, ctx->D, ctx->M,
                               ctx->tf32_lp_img, acc, ctx->err_d, ctx->nsm, ctx->stream))
      return fail(ctx, KGB_ERR_CUDA, "split-TF32 LPlusTimes launch failed");
    CKN(1);
    return KGB_OK;
  }
  if (ctx->tc_lp && ctx->use_tc_lp) {
    if (ctx->prec == KGB_FP64)
      tcRows<double>(ctx, as<double>(ctx->phi_out), as<double>(ctx->rhs), ctx->M, ctx->D, ctx->M, 32, ctx->D,
                     ctx->tc_lp_nhalf, ctx->tc_lp_img, ctx->tc_lp_exp, acc, true);
    else
      tcRows<float>(ctx, as<float>(ctx->phi_out), as<float>(ctx->rhs), ctx->M, ctx->D, ctx->M, 32, ctx->D,
                    ctx->tc_lp_nhalf, ctx->tc_lp_img, ctx->tc_lp_exp, acc, true);
    CKN(1);
    return KGB_OK;
  }
  if (ctx->prec == KGB_FP64)
    launch_lplustimes<double>(as<double>(ctx->phi_out), as<double>(ctx->rhs), as<double>(ctx->ellp), rows, ctx->D, ctx->M, acc, ctx->stream);
  else
    launch_lplustimes<float>(as<float>(ctx->phi_out), as<float>(ctx->rhs), as<float>(ctx->ellp), rows, ctx->D, ctx->M, acc, ctx->stream);
  CKN(1);
  return KGB_OK;
}

// rhs as the last iteration swept it (L+ phi_out), for entry points that read
// rhs after a solver loop with the fused sweep.
int ensureRhs(kgb_ctx *ctx) {
  if (!ctx->rhs_stale) return KGB_OK;
  int rc = prepare(ctx);
  if (rc) return rc;
  // with the SIMT kernel's arithmetic, as the fused sweep formed it
  const bool tf32 = ctx->use_tf32_lp;
  ctx->use_tf32_lp = false;
  rc = doLPlusTimes(ctx, false);
  ctx->use_tf32_lp = tf32;
  return rc;
}

template <typename T>
int scatterTensor(kgb_ctx *ctx, bool acc, const int *rowexp) {
  const int G = ctx->G, L1 = ctx->L + 1, S = tcDigits<T>(), kpad = ctx->tc_sc_kpad;
  // the (material, order) launches write disjoint outputs: alternate them over two
  // streams so each launch's tail overlaps the next one's tiles
  const bool two = ctx->sweep_streams > 1 && ctx->aux[0] != nullptr;
  if (two) {
    CK(cudaEventRecord(ctx->fork_ev, ctx->stream));
    CK(cudaStreamWaitEvent(ctx->aux[0], ctx->fork_ev, 0));
  }
  int nl = 0;
  for (int m = 0; m < 3; ++m) {
    const int64_t nz = ctx->pure_off[m + 1] - ctx->pure_off[m];
    if (nz == 0) continue;
    for (int l = 0; l < L1; ++l) {
      TcArgs<T> a{};
      a.A = as<T>(ctx->phi);
      a.C = as<T>(ctx->phi_out);
      a.rows = nz * (2 * l + 1);
      a.K = G;
      a.kpad = kpad;
      a.N = G;
      const int nbk = (G + 31) / 32;  // N blocks of 32 columns
      a.nhalf = nbk;
      a.bimg = ctx->tc_sc_img + ((size_t)m * L1 + l) * nbk * kpad * S * 32;
      a.bexp = ctx->tc_sc_exp + ((size_t)m * L1 + l) * nbk * 32;
      a.err = ctx->err_d;
      a.accumulate = acc;
      a.nsm = ctx->nsm;
      a.zl = ctx->pure_z + ctx->pure_off[m];
      a.nm = 2 * l + 1;
      a.m0 = l * l;
      a.ks = ctx->M;
      a.zstride = (int64_t)G * ctx->M;
      a.stages = 2;  // both K chunks of a tile stay resident across its N blocks
      a.rowexp = rowexp;
      launch_tc_gather<T>(a, two && (nl++ & 1) ? ctx->aux[0] : ctx->stream);
      CKN(1);
    }
  }
  if (ctx->nmixed_z > 0) {
    ScatterArgsBase a = scatterArgs(ctx);
    a.Z = ctx->nmixed_z;
    a.zlist = ctx->mixed_z;
    launch_scattering<T>(as<T>(ctx->phi), as<T>(ctx->phi_out), as<T>(ctx->sigsT), a, acc,
                         two && (nl++ & 1) ? ctx->aux[0] : ctx->stream);
    CKN(1);
  }
  if (two) {
    CK(cudaEventRecord(ctx->join_ev[0], ctx->aux[0]));
    CK(cudaStreamWaitEvent(ctx->stream, ctx->join_ev[0], 0));
  }
  return KGB_OK;
}

// rowexp (tensor path): phi's exponents per (zone, moment) recorded by the
// LTimes that wrote phi, or null.
int doScattering(kgb_ctx *ctx, bool acc, const int *rowexp = nullptr) {
  FamScope fs(ctx, "scattering");
  if (ctx->tc_sc && ctx->use_tc_sc)
    return ctx->prec == KGB_FP64 ? scatterTensor<double>(ctx, acc, rowexp) : scatterTensor<float>(ctx, acc, rowexp);
  ScatterArgsBase a = scatterArgs(ctx);
  if (ctx->prec == KGB_FP64)
    launch_scattering<double>(as<double>(ctx->phi), as<double>(ctx->phi_out), as<double>(ctx->sigsT), a, acc, ctx->stream);
  else
    launch_scattering<float>(as<float>(ctx->phi), as<float>(ctx->phi_out), as<float>(ctx->sigsT), a, acc, ctx->stream);
  CKN(1);
  return KGB_OK;
}

int doSource(kgb_ctx *ctx, double q) {
  FamScope fs(ctx, "source");
  if (ctx->prec == KGB_FP64)
    launch_source<double>(as<double>(ctx->phi_out), ctx->nmix, ctx->mix_zone, ctx->mix_mat, ctx->mix_frac, ctx->G, ctx->M, q, ctx->stream);
  else
    launch_source<float>(as<float>(ctx->phi_out), ctx->nmix, ctx->mix_zone, ctx->mix_mat, ctx->mix_frac, ctx->G, ctx->M, q, ctx->stream);
  CKN((ctx->nmix * ctx->G > 0 ? 1 : 0));
  return KGB_OK;
}

// population into device slot `out` (no host synchronisation)
int doPopulation(kgb_ctx *ctx, double *out) {
  FamScope fs(ctx, "population");
  const int64_t rows = ctx->Z * ctx->G;
  if (ctx->prec == KGB_FP64)
    launch_population<double>(as<double>(ctx->psi), ctx->w_d, ctx->vol_d, rows, ctx->G, ctx->D, ctx->partials, ctx->npart, out, ctx->stream);
  else
    launch_population<float>(as<float>(ctx->psi), ctx->w_d, ctx->vol_d, rows, ctx->G, ctx->D, ctx->partials, ctx->npart, out, ctx->stream);
  CKN(2);
  return KGB_OK;
}

// Reports (and clears) a bounded device-side wait that gave up.
int checkDeviceError(kgb_ctx *ctx) {
  int h = 0;
  CK(cudaMemcpyAsync(&h, ctx->err_d, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if (h) {
    CK(cudaMemsetAsync(ctx->err_d, 0, sizeof(int), ctx->stream));
    return fail(ctx, KGB_ERR_TIMEOUT, "a tensor-core kernel's bounded wait gave up");
  }
  return KGB_OK;
}

// One source iteration.  part_slot: particle count of the new psi, fused into
// the sweep.  prev_slot: particle count of the psi the iteration starts from,
// taken from this iteration's own moments (one small pass over moment 0) --
// a solve counts every iterate that way and the last one after its loop.
int iterateDevice(kgb_ctx *ctx, double q, double *part_slot, double *prev_slot = nullptr) {
  int rc;
  // psi's row exponents, when the sweep that wrote psi recorded them
  const bool px = psiExpUsable(ctx);
  const int *rx = px && ctx->psi_exp_valid ? ctx->psi_exp : nullptr;
  ctx->psi_exp_valid = false;
  int *const pe = phiExpUsable(ctx) ? ctx->phi_exp : nullptr;  // phi's, for the scattering
  if ((rc = doLTimes(ctx, false, rx, pe))) return rc;  // phi = L psi        (kConst + LTimes)
  if (prev_slot) {
    FamScope fs(ctx, "population");
    const int64_t rows = ctx->Z * ctx->G;
    if (ctx->pop_scale != 0.0) {
      if (ctx->prec == KGB_FP64)
        launch_population_moments<double>(as<double>(ctx->phi), ctx->M, ctx->vol_d, rows, ctx->G, ctx->pop_scale,
                                          ctx->partials, ctx->npart, prev_slot, ctx->stream);
      else
        launch_population_moments<float>(as<float>(ctx->phi), ctx->M, ctx->vol_d, rows, ctx->G, ctx->pop_scale,
                                         ctx->partials, ctx->npart, prev_slot, ctx->stream);
      CKN(2);
    } else if ((rc = doPopulation(ctx, prev_slot))) {
      return rc;
    }
  }
  if ((rc = doScattering(ctx, false, pe))) return rc;  // phi_out = S phi    (kConst + scattering)
  if ((rc = doSource(ctx, q))) return rc;              // phi_out += Q
  // rhs = L+ phi_out (kConst + LPlusTimes), or formed cell by cell inside the sweep
  ctx->fuse_active = ctx->fuse_sweep && ctx->prec == KGB_MIXED && ctx->M <= kFuseMaxM;
  if (!ctx->fuse_active && (rc = doLPlusTimes(ctx, false))) return rc;
  if ((rc = sweepSolver(ctx, part_slot != nullptr, ctx->fuse_active, px ? ctx->psi_exp : nullptr)))
    return rc;  // psi = H^-1 rhs (+ population, + row exponents)
  ctx->psi_exp_valid = px;
  if (ctx->fuse_active) ctx->rhs_stale = true;
  if (part_slot) {
    FamScope fs(ctx, "population");
    launch_sum_partials(ctx->pop_slots, ctx->npop_slots, part_slot, ctx->stream);
    CKN(1);
  }
  return KGB_OK;
}

// ---------------------------------------------------------------------------
// Converged solves, the adjoint source iteration, response and gradients
// ---------------------------------------------------------------------------
MixArgs mixArgs(const kgb_ctx *ctx) {
  MixArgs a{};
  a.Z = ctx->Z;
  a.G = ctx->G;
  a.nx = ctx->nx;
  a.ny = ctx->ny;
  a.zmix_start = ctx->zmix_start;
  a.zmix_count = ctx->zmix_count;
  a.mix_mat = ctx->mix_mat;
  a.mix_frac = ctx->mix_frac;
  a.colsum = ctx->colsum_d;
  a.det = ctx->det_d;
  a.vol = ctx->vol_d;
  a.dx = ctx->dxyz_d[0];
  a.dy = ctx->dxyz_d[1];
  a.dz = ctx->dxyz_d[2];
  return a;
}

constexpr int kRespTerms = 13;  // per group: 4 terms for each of 3 materials, then the response

// Small buffers of the response path, allocated on first use; the detector
// starts as the whole domain.
int ensureResponseBuffers(kgb_ctx *ctx) {
  int rc;
  if (!ctx->phi_prev && (rc = dmalloc(ctx, &ctx->phi_prev, ctx->Z * ctx->G))) return rc;
  if (!ctx->norm_d && (rc = dmalloc(ctx, &ctx->norm_d, 2))) return rc;
  if (!ctx->colsum_d && (rc = dmalloc(ctx, &ctx->colsum_d, 3 * ctx->G))) return rc;
  if (!ctx->e0_d && (rc = dmalloc(ctx, &ctx->e0_d, 2 * ctx->D))) return rc;
  if (!ctx->det_d) {
    if ((rc = dmalloc(ctx, &ctx->det_d, ctx->Z))) return rc;
    launch_fill<double>(ctx->det_d, ctx->Z, 1.0, ctx->stream);
    CKN(1);
  }
  if (!ctx->resp_d) {
    const int64_t want = ((int64_t)ctx->nsm * 8 + ctx->G - 1) / ctx->G;
    ctx->resp_nb = (int)std::max<int64_t>(1, std::min<int64_t>(want, (ctx->Z + 3) / 4));
    if ((rc = dmalloc(ctx, &ctx->resp_part, (size_t)ctx->resp_nb * ctx->G * kRespTerms)) ||
        (rc = dmalloc(ctx, &ctx->resp_d, (size_t)ctx->G * kRespTerms)))
      return rc;
  }
  return KGB_OK;
}

// Tables of the adjoint operators, rebuilt when quadrature, L/L+ or sigs change:
// S^T (sigs uploaded untransposed, read by the scattering kernel as
// [mat][l][g'][g]) with its nonzero source ranges, the P0 out-scattering sums,
// moment-0 rows of L and L+, and tensor-core plans of L+^T and L^T.
template <typename T>
int prepareAdjointT(kgb_ctx *ctx) {
  int rc;
  if ((rc = ensureResponseBuffers(ctx))) return rc;
  if (!ctx->adj_stale) return KGB_OK;
  const int G = ctx->G, L1 = ctx->L + 1, D = ctx->D, M = ctx->M;
  std::vector<int> lo(G, G), hi(G, -1);
  std::vector<double> colsum((size_t)3 * G, 0.0);
  for (int m = 0; m < 3; ++m)
    for (int l = 0; l < L1; ++l)
      for (int gp = 0; gp < G; ++gp)
        for (int g = 0; g < G; ++g)
          if (ctx->sigs_h[(((size_t)m * L1 + l) * G + gp) * G + g] != 0.0) {
            lo[g] = std::min(lo[g], gp);
            hi[g] = std::max(hi[g], gp);
          }
  for (int m = 0; m < 3; ++m)
    for (int g = 0; g < G; ++g)
      for (int gp = 0; gp < G; ++gp) colsum[(size_t)m * G + g] += ctx->sigs_h[(((size_t)m * L1) * G + gp) * G + g];
  if (!ctx->sigsT_adj) {
    if ((rc = dalloc(ctx, &ctx->sigsT_adj, (size_t)3 * L1 * G * G * ctx->tsz)) ||
        (rc = dmalloc(ctx, &ctx->gp_lo_adj, G)) || (rc = dmalloc(ctx, &ctx->gp_hi_adj, G)))
      return rc;
  }
  if ((rc = uploadVec<T>(ctx, ctx->sigsT_adj, ctx->sigs_h))) return rc;
  std::vector<double> e0((size_t)2 * D);
  for (int d = 0; d < D; ++d) {
    e0[d] = ctx->ell_h[(size_t)d * M];
    e0[D + d] = ctx->ellp_h[(size_t)d * M];
  }
  CK(cudaMemcpyAsync(ctx->gp_lo_adj, lo.data(), G * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->gp_hi_adj, hi.data(), G * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->colsum_d, colsum.data(), colsum.size() * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->e0_d, e0.data(), e0.size() * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  // the response derivative w(d) vol det siga is L^T applied to a moment-0
  // source exactly when ell(0, d) = c0 w(d) for every direction
  const std::vector<double> &w = ctx->q[3];
  const double c0 = w[0] != 0.0 ? ctx->ell_h[0] / w[0] : 0.0;
  bool prop = c0 != 0.0;
  for (int d = 0; d < D && prop; ++d) prop = std::fabs(ctx->ell_h[(size_t)d * M] - c0 * w[d]) <= 1e-13 * std::fabs(c0 * w[d]);
  ctx->inv_c0 = prop ? 1.0 / c0 : 0.0;
  if ((rc = planTensorMomentsFrom<T>(ctx, ctx->ellp_h, ctx->ell_h, &ctx->tc_lt_adj, &ctx->tc_lt_img_adj,
                                     &ctx->tc_lt_exp_adj, &ctx->tc_lt_kpad_adj, &ctx->tc_lp_adj, &ctx->tc_lp_img_adj,
                                     &ctx->tc_lp_exp_adj, &ctx->tc_lp_nhalf_adj)))
    return rc;
  if ((rc = planTf32From(ctx, ctx->ellp_h, ctx->ell_h, &ctx->tf32_lt_img_adj, &ctx->tf32_lp_img_adj))) return rc;
  ctx->adj_stale = false;
  return KGB_OK;
}

int prepareAdjoint(kgb_ctx *ctx) {
  return ctx->prec == KGB_FP64 ? prepareAdjointT<double>(ctx) : prepareAdjointT<float>(ctx);
}

// Installs the adjoint operators for its lifetime: lam takes psi's place,
// L and L+ exchange (their [D][M] tables are each other's transposes), the
// scattering kernel reads S^T, and the sweep runs reversed.  Nothing may
// reallocate context buffers while it is installed.
struct AdjointView {
  kgb_ctx *c;
  explicit AdjointView(kgb_ctx *ctx) : c(ctx) { swap(); }
  ~AdjointView() { swap(); }
  AdjointView(const AdjointView &) = delete;
  AdjointView &operator=(const AdjointView &) = delete;
  void swap() {
    c->psi_exp_valid = false;  // the row exponents were psi's
    std::swap(c->psi, c->lam);
    std::swap(c->ell, c->ellp);
    std::swap(c->sigsT, c->sigsT_adj);
    std::swap(c->gp_lo, c->gp_lo_adj);
    std::swap(c->gp_hi, c->gp_hi_adj);
    std::swap(c->tc_lt, c->tc_lt_adj);
    std::swap(c->tc_lp, c->tc_lp_adj);
    std::swap(c->tc_lt_img, c->tc_lt_img_adj);
    std::swap(c->tc_lp_img, c->tc_lp_img_adj);
    std::swap(c->tc_lt_exp, c->tc_lt_exp_adj);
    std::swap(c->tc_lp_exp, c->tc_lp_exp_adj);
    std::swap(c->tc_lt_kpad, c->tc_lt_kpad_adj);
    std::swap(c->tc_lp_nhalf, c->tc_lp_nhalf_adj);
    std::swap(c->tf32_lt_img, c->tf32_lt_img_adj);
    std::swap(c->tf32_lp_img, c->tf32_lp_img_adj);
    std::swap(c->tc_sc_img, c->tc_sc_img_adj);
    std::swap(c->tc_sc_exp, c->tc_sc_exp_adj);
    c->flip ^= 1;
  }
};

int doAdjointSource(kgb_ctx *ctx) {
  FamScope fs(ctx, "source");
  const MixArgs a = mixArgs(ctx);
  if (ctx->prec == KGB_FP64)
    launch_adjoint_source<double>(as<double>(ctx->phi_out), ctx->M, as<double>(ctx->sigt), a, ctx->inv_c0, ctx->stream);
  else
    launch_adjoint_source<float>(as<float>(ctx->phi_out), ctx->M, as<float>(ctx->sigt), a, ctx->inv_c0, ctx->stream);
  CKN(1);
  return KGB_OK;
}

// Source iterations from a zero state until moment 0 of successive iterates
// changes by at most tol relative to its largest magnitude, or the change has
// not reached a new minimum for kStall iterations (the rounding floor, which
// the FP32 state of the mixed form meets near 1e-7; the change falls
// monotonically above it).  The change is measured
// on the moments each iteration computes first (phi = L psi of the previous
// iterate), so the test lags one sweep and the returned state is one
// iteration past the converged one.  With the adjoint operators installed it
// runs the adjoint iteration with the response source.
constexpr int kStall = 4;
int convergeLoop(kgb_ctx *ctx, bool adjoint, double q, double tol, int max_iter, int32_t *iters, double *change) {
  int rc;
  const int64_t rows = ctx->Z * ctx->G;
  CK(cudaMemsetAsync(ctx->psi, 0, rows * ctx->D * ctx->tsz, ctx->stream));
  CK(cudaMemsetAsync(ctx->phi_prev, 0, rows * sizeof(double), ctx->stream));
  // psi = 0 has row exponents 0; each sweep records the next ones
  ctx->psi_exp_valid = false;
  int *const rx = psiExpUsable(ctx) ? ctx->psi_exp : nullptr;
  if (rx) CK(cudaMemsetAsync(rx, 0, rows * sizeof(int), ctx->stream));
  int *const pe = phiExpUsable(ctx) ? ctx->phi_exp : nullptr;
  double ch = std::numeric_limits<double>::infinity(), best = ch;
  int it = 0, stall = 0;
  while (it < max_iter) {
    ++it;
    if ((rc = doLTimes(ctx, false, rx, pe))) return rc;
    CK(cudaMemsetAsync(ctx->norm_d, 0, 2 * sizeof(unsigned long long), ctx->stream));
    {
      FamScope fs(ctx, "convergence");
      if (ctx->prec == KGB_FP64)
        launch_change_norm<double>(as<double>(ctx->phi), ctx->M, ctx->phi_prev, rows, ctx->norm_d, ctx->stream);
      else
        launch_change_norm<float>(as<float>(ctx->phi), ctx->M, ctx->phi_prev, rows, ctx->norm_d, ctx->stream);
      CKN(1);
    }
    if ((rc = doScattering(ctx, false, pe))) return rc;
    if ((rc = adjoint ? doAdjointSource(ctx) : doSource(ctx, q))) return rc;
    if ((rc = doLPlusTimes(ctx, false))) return rc;
    if ((rc = sweepSolver(ctx, false, false, rx))) return rc;
    unsigned long long h[2] = {0ull, 0ull};
    CK(cudaMemcpyAsync(h, ctx->norm_d, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (it >= 2 && tol >= 0.0) {
      double dmax, amax;
      std::memcpy(&dmax, &h[0], sizeof(double));
      std::memcpy(&amax, &h[1], sizeof(double));
      if (!std::isfinite(dmax) || !std::isfinite(amax))
        return fail(ctx, KGB_ERR_STATE, "the source iteration produced a non-finite flux");
      ch = amax > 0.0 ? dmax / amax : (dmax > 0.0 ? std::numeric_limits<double>::infinity() : 0.0);
      if (ch <= tol) break;
      if (ch < best) {
        best = ch;
        stall = 0;
      } else if (++stall >= kStall) {
        break;
      }
    }
  }
  if (iters) *iters = it;
  if (change) *change = ch;
  return KGB_OK;
}

// Per-group response terms (kRespTerms per group) of state psi and, when lam
// is given, the adjoint terms against lam with moments from psi0.
int responseTermsOf(kgb_ctx *ctx, const void *psi, const void *psi0, const void *lam, std::vector<double> &out) {
  {
    FamScope fs(ctx, "response");
    const MixArgs a = mixArgs(ctx);
    const double *ell0 = ctx->e0_d, *ellp0 = ctx->e0_d + ctx->D;
    if (ctx->prec == KGB_FP64)
      launch_response<double>((const double *)psi, (const double *)psi0, (const double *)lam, ctx->D, ctx->w_d, ell0,
                              ellp0, as<double>(ctx->sigt), a, ctx->resp_part, ctx->resp_nb, ctx->resp_d, ctx->stream);
    else
      launch_response<float>((const float *)psi, (const float *)psi0, (const float *)lam, ctx->D, ctx->w_d, ell0,
                             ellp0, as<float>(ctx->sigt), a, ctx->resp_part, ctx->resp_nb, ctx->resp_d, ctx->stream);
    CKN(2);
  }
  out.assign((size_t)ctx->G * kRespTerms, 0.0);
  CK(cudaMemcpyAsync(out.data(), ctx->resp_d, out.size() * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return KGB_OK;
}

// One forward source iteration from state `in` (nullptr: zero) into `out`;
// the sweep writes only `out`, so both may be any psi-sized buffers.
int forwardStep(kgb_ctx *ctx, void *in, void *out, double q) {
  void *const keep = ctx->psi;
  int rc = KGB_OK;
  if (in) {
    ctx->psi = in;
    rc = doLTimes(ctx, false);
  } else if (cudaMemsetAsync(ctx->phi, 0, ctx->Z * ctx->G * ctx->M * ctx->tsz, ctx->stream) != cudaSuccess) {
    rc = fail(ctx, KGB_ERR_CUDA, "memset failed");
  }
  if (!rc) rc = doScattering(ctx, false);
  if (!rc) rc = doSource(ctx, q);
  if (!rc) rc = doLPlusTimes(ctx, false);
  ctx->psi = out;
  if (!rc) rc = sweepSolver(ctx, false);
  ctx->psi = keep;
  return rc;
}

// One step of the reverse pass through unrolled iterations (adjoint operators
// installed, psi = the reverse state): the first step sweeps the response
// source alone, later ones apply L^T S^T L+^T to the state and sweep.
int reverseStep(kgb_ctx *ctx, bool first) {
  int rc;
  if (first) {
    CK(cudaMemsetAsync(ctx->phi_out, 0, ctx->Z * ctx->G * ctx->M * ctx->tsz, ctx->stream));
    if ((rc = doAdjointSource(ctx))) return rc;
  } else {
    if ((rc = doLTimes(ctx, false))) return rc;
    if ((rc = doScattering(ctx, false))) return rc;
  }
  if ((rc = doLPlusTimes(ctx, false))) return rc;
  return sweepSolver(ctx, false);
}

// psi-sized device buffers held for one call
struct PsiBuffers {
  std::vector<void *> b;
  ~PsiBuffers() {
    for (void *p : b) cudaFree(p);
  }
};

}  // namespace

namespace {
// The particle count from the next iteration's moments saves the FP64 sweep
// its per-cell accumulation; FP32 moments would round the count, so the mixed
// form keeps the compensated sum fused into its (latency-bound) sweep.
bool lagPopulation(const kgb_ctx *ctx) { return ctx->prec == KGB_FP64 && ctx->pop_scale != 0.0; }

// After psi = 0: its row exponents are 0.
int resetPsiExp(kgb_ctx *ctx) {
  ctx->psi_exp_valid = false;
  if (!psiExpUsable(ctx)) return KGB_OK;
  CK(cudaMemsetAsync(ctx->psi_exp, 0, ctx->Z * ctx->G * sizeof(int), ctx->stream));
  ctx->psi_exp_valid = true;
  return KGB_OK;
}

// niter iterations from the current psi with their particle counts.
int solveIterations(kgb_ctx *ctx, int niter, double q) {
  int rc;
  if (!lagPopulation(ctx)) {
    for (int it = 0; it < niter; ++it)
      if ((rc = iterateDevice(ctx, q, ctx->parts_dev + it))) return rc;
    return KGB_OK;
  }
  // the count after iteration it-1 from iteration it's moments, the last one from psi
  for (int it = 0; it < niter; ++it)
    if ((rc = iterateDevice(ctx, q, nullptr, it > 0 ? ctx->parts_dev + it - 1 : nullptr))) return rc;
  return doPopulation(ctx, ctx->parts_dev + niter - 1);
}

// The whole solve (psi reset + niter iterations with their particle counts)
// captured once per (niter, q, stream) and replayed while the context's
// tables are unchanged.  A capture that fails leaves *out null: the caller
// runs the solve launch by launch.
int solveGraph(kgb_ctx *ctx, int niter, double q, const kgb_ctx::SolveGraph **out) {
  *out = nullptr;
  auto &v = ctx->solve_graphs;
  for (auto it = v.begin(); it != v.end();) {
    if (it->gen != ctx->gen) {
      cudaGraphExecDestroy(it->x);
      cudaGraphDestroy(it->g);
      it = v.erase(it);
    } else {
      ++it;
    }
  }
  for (auto &e : v)
    if (e.niter == niter && e.q == q && e.stream == ctx->stream) {
      *out = &e;
      return KGB_OK;
    }
  if (v.size() >= 4) {
    cudaGraphExecDestroy(v.front().x);
    cudaGraphDestroy(v.front().g);
    v.erase(v.begin());
  }
  if (cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    cudaGetLastError();
    return KGB_OK;
  }
  const int64_t l0 = ctx->launches;
  const std::string err0 = ctx->err;
  int rc = cudaMemsetAsync(ctx->psi, 0, ctx->Z * ctx->G * ctx->D * ctx->tsz, ctx->stream) == cudaSuccess
               ? KGB_OK : KGB_ERR_CUDA;
  if (!rc) rc = resetPsiExp(ctx);
  if (!rc) rc = solveIterations(ctx, niter, q);
  cudaGraph_t g = nullptr;
  const cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
  const int64_t captured = ctx->launches - l0;
  ctx->launches = l0;  // counted when replayed
  cudaGraphExec_t x = nullptr;
  if (rc || e != cudaSuccess || !g || cudaGraphInstantiate(&x, g, 0) != cudaSuccess) {
    cudaGetLastError();
    if (g) cudaGraphDestroy(g);
    ctx->err = err0;
    return KGB_OK;
  }
  v.push_back({niter, q, ctx->gen, ctx->stream, g, x, captured});
  *out = &v.back();
  return KGB_OK;
}
}  // namespace

namespace kgb {
int instance_view(kgb_ctx *ctx, InstanceView *v) {
  int rc = prepare(ctx);
  if (rc) return rc;
  ctx->psi_exp_valid = false;  // a batched solve writes psi through the view
  InstanceView x{};
  x.prec = ctx->prec;
  x.Z = ctx->Z;
  x.G = ctx->G; x.D = ctx->D; x.M = ctx->M; x.L = ctx->L; x.Gs = ctx->Gs; x.Ds = ctx->Ds;
  x.nx = ctx->nx; x.ny = ctx->ny; x.nz = ctx->nz;
  x.nsdom = ctx->dc.num();
  x.zonesets[0] = ctx->dc.Sx; x.zonesets[1] = ctx->dc.Sy; x.zonesets[2] = ctx->dc.Sz;
  x.psi = ctx->psi; x.rhs = ctx->rhs; x.phi = ctx->phi; x.phi_out = ctx->phi_out; x.sigt = ctx->sigt;
  for (int k = 0; k < 3; ++k) {
    x.plane[k] = ctx->plane[k];
    x.plane_chunk[k] = ctx->plane_chunk[k];
  }
  x.ell = ctx->ell; x.ellp = ctx->ellp; x.sigsT = ctx->sigsT; x.cx = ctx->cx; x.cy = ctx->cy; x.cz = ctx->cz;
  x.w = ctx->w_d; x.vol = ctx->vol_d; x.mix_frac = ctx->mix_frac;
  x.zmix_start = ctx->zmix_start; x.zmix_count = ctx->zmix_count; x.mix_mat = ctx->mix_mat;
  x.gp_lo = ctx->gp_lo; x.gp_hi = ctx->gp_hi;
  x.sdoms = ctx->sdoms_d;
  x.vol_uniform = ctx->vol_uniform;
  x.cls = ctx->use_recip ? ctx->cls_d : nullptr;
  x.inv = ctx->use_recip ? ctx->inv_d : nullptr;
  x.gen = ctx->gen;
  x.psi_exp = psiExpUsable(ctx) ? ctx->psi_exp : nullptr;
  x.psi_exp_w = psiExpWidth(ctx);
  *v = x;
  return KGB_OK;
}

int instance_op(kgb_ctx *ctx, InstanceOp op, double q, cudaStream_t s, const int *psi_exp) {
  cudaStream_t keep = ctx->stream;
  ctx->stream = s;
  // a batched iteration runs each problem's LTimes and then its scattering (same
  // stream), so LTimes can record phi's exponents for the scattering
  int *const pe = phiExpUsable(ctx) ? ctx->phi_exp : nullptr;
  int rc;
  switch (op) {
    case InstanceOp::LTimes: rc = doLTimes(ctx, false, psi_exp, pe); break;
    case InstanceOp::LPlusTimes: rc = doLPlusTimes(ctx, false); break;
    default:
      rc = doScattering(ctx, false, pe);
      if (!rc) rc = doSource(ctx, q);
      break;
  }
  ctx->stream = keep;
  return rc;
}
int instance_check(kgb_ctx *ctx) { return checkDeviceError(ctx); }
}  // namespace kgb

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

const char *kgb_version(void) { return "kripke_gb300 0.1 sm_103a"; }

int kgb_ctx_create(int device, kgb_ctx **out) {
  if (!out) return KGB_ERR_ARG;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) {
    cudaGetLastError();
    return KGB_ERR_CUDA;
  }
  if (cudaSetDevice(device) != cudaSuccess) return KGB_ERR_CUDA;
  kgb_ctx *c = new (std::nothrow) kgb_ctx();
  if (!c) return KGB_ERR_OOM;
  c->device = device;
  if (cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    return KGB_ERR_CUDA;
  }
  c->stream = c->own_stream;
  bool streams_ok = cudaEventCreateWithFlags(&c->fork_ev, cudaEventDisableTiming) == cudaSuccess;
  for (int i = 0; i < kgb_ctx::kMaxSweepStreams - 1 && streams_ok; ++i)
    streams_ok = cudaStreamCreateWithFlags(&c->aux[i], cudaStreamNonBlocking) == cudaSuccess &&
                 cudaEventCreateWithFlags(&c->join_ev[i], cudaEventDisableTiming) == cudaSuccess;
  if (!streams_ok) {
    cudaGetLastError();  // one stream only: sweeps stay on the context's stream
    c->sweep_streams = 1;
    c->max_streams = 1;
  }
  *out = c;
  return KGB_OK;
}

int kgb_ctx_destroy(kgb_ctx *ctx) {
  if (!ctx) return KGB_ERR_ARG;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  for (auto &kv : ctx->fams)
    for (auto &pr : kv.second.pending) {
      cudaEventDestroy(pr.first);
      cudaEventDestroy(pr.second);
    }
  freeAll(ctx);
  if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
  for (int i = 0; i < kgb_ctx::kMaxSweepStreams - 1; ++i) {
    if (ctx->aux[i]) cudaStreamDestroy(ctx->aux[i]);
    if (ctx->join_ev[i]) cudaEventDestroy(ctx->join_ev[i]);
  }
  if (ctx->fork_ev) cudaEventDestroy(ctx->fork_ev);
  delete ctx;
  return KGB_OK;
}

const char *kgb_last_error(const kgb_ctx *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int kgb_setup(kgb_ctx *ctx, const kgb_dims *d) {
  if (!ctx || !d) return KGB_ERR_ARG;
  CK(cudaSetDevice(ctx->device));
  if (d->layout < 0 || d->layout > 5) return fail(ctx, KGB_ERR_LAYOUT, "unknown layout");
  if (d->precision != KGB_FP64 && d->precision != KGB_MIXED) return fail(ctx, KGB_ERR_ARG, "unknown precision");
  if (d->nx < 1 || d->ny < 1 || d->nz < 1 || d->num_groups < 1 || d->num_directions < 8 || d->legendre_order < 0 ||
      d->legendre_order > 7)
    return fail(ctx, KGB_ERR_ARG, "bad problem size (zones >= 1, groups >= 1, directions >= 8, 0 <= legendre <= 7)");
  if (d->num_groupsets < 1 || d->num_groups % d->num_groupsets)
    return fail(ctx, KGB_ERR_ARG, "number of groups must be divisible by the number of group sets");
  if (d->num_dirsets < 1 || (d->num_dirsets % 8 && d->num_dirsets < 8) || d->num_directions % d->num_dirsets)
    return fail(ctx, KGB_ERR_ARG, "direction sets must be a multiple of 8 (or >= 8) and divide the directions");
  for (int k = 0; k < 3; ++k)
    if (d->num_zonesets[k] < 1) return fail(ctx, KGB_ERR_ARG, "zone sets must be >= 1");
  if (d->nx % d->num_zonesets[0] || d->ny % d->num_zonesets[1] || d->nz % d->num_zonesets[2])
    return fail(ctx, KGB_ERR_ARG, "zone sets must divide the zones");
  {
    // the SIMT moment kernels stage the whole [D][moment class] table in shared memory
    const int M = (d->legendre_order + 1) * (d->legendre_order + 1);
    const size_t need = (size_t)(d->precision == KGB_FP64 ? 8 : 4) * d->num_directions * moment_class(M);
    int optin = 0;
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device);
    if (optin > 0 && need > (size_t)optin)
      return fail(ctx, KGB_ERR_ARG,
                  "directions x moments too large: the moment tables (" + std::to_string(need) +
                      " bytes) exceed the " + std::to_string(optin) + " bytes of shared memory of a block");
  }
  cudaStreamSynchronize(ctx->stream);
  freeAll(ctx);
  ctx->dims = *d;
  ctx->prec = d->precision;
  ctx->tsz = ctx->prec == KGB_FP64 ? 8 : 4;
  // measured defaults: the digit-product tensor path wins for FP64 and for the
  // single-material zones' scattering in both forms (FP32 at 64^3: 4.6 against 6.5
  // ms); the mixed form's LTimes / LPlusTimes stay SIMT; kgb_autotune re-measures
  // every choice on the actual problem
  ctx->use_tc_lt = ctx->use_tc_lp = ctx->prec == KGB_FP64;
  ctx->use_tc_sc = true;
  // the tabulated reciprocal pays where the divide costs FP64 slots; in FP32 its
  // dependent table load costs more than the divide it saves
  ctx->allow_recip = ctx->prec == KGB_FP64;
  // default sweep tiles: the autotuner's choice on 32^3 and 64^3 problems (2x2x8 in
  // FP64, where the FP64 pipe wants the most chains in flight; 4x2x8 in FP32)
  if (!ctx->tiles_set) {
    ctx->tx = ctx->prec == KGB_FP64 ? 2 : 4;
    ctx->ty = 2;
    ctx->tz = 8;
  }
  ctx->dc.SP = d->num_groupsets;
  ctx->dc.SQ = d->num_dirsets;
  ctx->dc.Sx = d->num_zonesets[0];
  ctx->dc.Sy = d->num_zonesets[1];
  ctx->dc.Sz = d->num_zonesets[2];
  ctx->G = d->num_groups;
  ctx->D = d->num_directions;
  ctx->L = d->legendre_order;
  ctx->M = (ctx->L + 1) * (ctx->L + 1);
  ctx->Gs = ctx->G / ctx->dc.SP;
  ctx->Ds = ctx->D / ctx->dc.SQ;
  ctx->nx = d->nx; ctx->ny = d->ny; ctx->nz = d->nz;
  ctx->nxs = d->nx / ctx->dc.Sx; ctx->nys = d->ny / ctx->dc.Sy; ctx->nzs = d->nz / ctx->dc.Sz;
  ctx->Z = (int64_t)d->nx * d->ny * d->nz;
  ctx->Zs = (int64_t)ctx->nxs * ctx->nys * ctx->nzs;
  const int64_t nch = (int64_t)ctx->Gs * ctx->Ds;
  ctx->plane_chunk[0] = nch * ctx->nys * ctx->nzs;
  ctx->plane_chunk[1] = nch * ctx->nxs * ctx->nzs;
  ctx->plane_chunk[2] = nch * ctx->nxs * ctx->nys;
  const size_t T = ctx->tsz;
  int rc;
  // moments are allocated for whole 128-row tiles (the split-TF32 kernels copy whole tiles); the
  // padding is zeroed here and never read as part of a field
  const int64_t flux = ctx->Z * ctx->G * ctx->D, mom = tf32_padded_rows(ctx->Z * ctx->G) * ctx->M;
  if ((rc = dalloc(ctx, &ctx->psi, flux * T)) || (rc = dalloc(ctx, &ctx->rhs, flux * T)) ||
      (rc = dalloc(ctx, &ctx->phi, mom * T)) || (rc = dalloc(ctx, &ctx->phi_out, mom * T)) ||
      (rc = dalloc(ctx, &ctx->sigt, ctx->Z * ctx->G * T)))
    goto oom;
  for (int k = 0; k < 3; ++k)
    if ((rc = dalloc(ctx, &ctx->plane[k], ctx->plane_chunk[k] * ctx->dc.num() * T))) goto oom;
  if ((rc = dalloc(ctx, &ctx->ell, (size_t)ctx->D * ctx->M * T)) || (rc = dalloc(ctx, &ctx->ellp, (size_t)ctx->D * ctx->M * T)) ||
      (rc = dalloc(ctx, &ctx->sigsT, (size_t)3 * (ctx->L + 1) * ctx->G * ctx->G * T)) ||
      (rc = dalloc(ctx, &ctx->cx, (size_t)ctx->D * ctx->nx * T)) || (rc = dalloc(ctx, &ctx->cy, (size_t)ctx->D * ctx->ny * T)) ||
      (rc = dalloc(ctx, &ctx->cz, (size_t)ctx->D * ctx->nz * T)))
    goto oom;
  if ((rc = dmalloc(ctx, &ctx->w_d, ctx->D)) || (rc = dmalloc(ctx, &ctx->cos_d[0], ctx->D)) ||
      (rc = dmalloc(ctx, &ctx->cos_d[1], ctx->D)) || (rc = dmalloc(ctx, &ctx->cos_d[2], ctx->D)) ||
      (rc = dmalloc(ctx, &ctx->vol_d, ctx->Z)) || (rc = dmalloc(ctx, &ctx->dxyz_d[0], ctx->nx)) ||
      (rc = dmalloc(ctx, &ctx->dxyz_d[1], ctx->ny)) || (rc = dmalloc(ctx, &ctx->dxyz_d[2], ctx->nz)) ||
      (rc = dmalloc(ctx, &ctx->zmix_start, ctx->Z)) || (rc = dmalloc(ctx, &ctx->zmix_count, ctx->Z)) ||
      (rc = dmalloc(ctx, &ctx->gp_lo, ctx->G)) || (rc = dmalloc(ctx, &ctx->gp_hi, ctx->G)) ||
      (rc = dmalloc(ctx, &ctx->sdoms_d, ctx->dc.num())) || (rc = dmalloc(ctx, &ctx->ident_d, ctx->dc.num())) ||
      (rc = dmalloc(ctx, &ctx->levels_d, ctx->dc.num())))
    goto oom;
  {
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    ctx->nsm = nsm > 0 ? nsm : 152;
  }
  if ((rc = dalloc(ctx, (void **)&ctx->err_d, sizeof(int)))) goto oom;
  CK(cudaMemsetAsync(ctx->phi, 0, mom * T, ctx->stream));
  CK(cudaMemsetAsync(ctx->phi_out, 0, mom * T, ctx->stream));
  ctx->npart = 152 * 4;
  if ((rc = dmalloc(ctx, &ctx->partials, 2 * ctx->npart)) || (rc = dmalloc(ctx, &ctx->results, 16))) goto oom;
  {
    std::vector<int> ident(ctx->dc.num());
    for (int s = 0; s < ctx->dc.num(); ++s) ident[s] = s;
    CK(cudaMemcpyAsync(ctx->ident_d, ident.data(), ident.size() * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
  }
  for (auto &v : ctx->q) v.assign(ctx->D, 0.0);
  for (auto &v : ctx->qi) v.assign(ctx->D, 1);
  ctx->dxyz[0].assign(ctx->nx, 1.0);
  ctx->dxyz[1].assign(ctx->ny, 1.0);
  ctx->dxyz[2].assign(ctx->nz, 1.0);
  ctx->ell_h.assign((size_t)ctx->D * ctx->M, 0.0);
  ctx->ellp_h.assign((size_t)ctx->D * ctx->M, 0.0);
  ctx->sigs_h.assign((size_t)3 * (ctx->L + 1) * ctx->G * ctx->G, 0.0);
  ctx->vol_h.assign(ctx->Z, 0.0);
  for (int k = 0; k < 2; ++k) {
    ctx->zmap[k].assign(ctx->dc.chunks(S_R), std::vector<int>(ctx->Zs, 0));
    ctx->mimap[k].assign(ctx->dc.chunks(S_R), std::vector<int>());
  }
  ctx->mfrac.assign(ctx->dc.chunks(S_R), std::vector<double>());
  ctx->m2l.resize(ctx->M);
  for (int n = 0, nm = 0; n <= ctx->L; ++n)
    for (int m = -n; m <= n; ++m) ctx->m2l[nm++] = n;
  for (bool &h : ctx->have) h = false;
  ctx->have[fieldIndex(findField("moment_to_legendre"))] = true;
  ctx->dirty_quad = ctx->dirty_geom = ctx->dirty_ell = ctx->dirty_sigs = ctx->dirty_mix = ctx->dirty_vol = true;
  ctx->ready = true;
  if ((rc = buildTiles(ctx))) goto oom;
  CK(cudaStreamSynchronize(ctx->stream));
  return KGB_OK;
oom:
  {
    std::string msg = ctx->err;
    freeAll(ctx);
    ctx->err = msg;
  }
  return rc;
}

int kgb_num_subdomains(const kgb_ctx *ctx, int32_t *out) {
  if (!ctx || !out) return KGB_ERR_ARG;
  if (!ctx->ready) return KGB_ERR_STATE;
  *out = ctx->dc.num();
  return KGB_OK;
}

int kgb_field_bytes(kgb_ctx *ctx, const char *name, int64_t *nbytes) {
  if (!ctx || !nbytes) return KGB_ERR_ARG;
  if (!ctx->ready) return fail(ctx, KGB_ERR_STATE, "kgb_setup has not been called");
  const FieldInfo *f = findField(name);
  if (!f) return fail(ctx, KGB_ERR_ARG, std::string("unknown field '") + (name ? name : "(null)") + "'");
  *nbytes = fieldBytes(ctx, f);
  return KGB_OK;
}

int kgb_field_upload(kgb_ctx *ctx, const char *name, const void *host, int64_t nbytes) {
  if (!ctx) return KGB_ERR_ARG;
  if (!ctx->ready) return fail(ctx, KGB_ERR_STATE, "kgb_setup has not been called");
  const FieldInfo *f = findField(name);
  if (!f) return fail(ctx, KGB_ERR_ARG, std::string("unknown field '") + (name ? name : "(null)") + "'");
  if (!host && nbytes > 0) return fail(ctx, KGB_ERR_ARG, "null host pointer");
  ctx->have_lam = false;  // an adjoint state belongs to the inputs it was computed for
  ctx->psi_exp_valid = false;
  const int64_t want = fieldBytes(ctx, f);
  if (nbytes != want)
    return fail(ctx, KGB_ERR_ARG, std::string("field '") + name + "' expects " + std::to_string(want) + " bytes, got " + std::to_string(nbytes));
  if (!std::strcmp(f->name, "rhs")) ctx->rhs_stale = false;
  CK(cudaSetDevice(ctx->device));
  const int nch = numChunks(ctx, f);
  const int layout = ctx->dims.layout;
  if (deviceKind(f->kind)) {
    size_t maxc = 0;
    for (int ch = 0; ch < nch; ++ch) maxc = std::max<size_t>(maxc, chunkElems(chunkGeom(ctx, f, ch)) * 8);
    int rc = ensureStaging(ctx, maxc);
    if (rc) return rc;
    const char *src = (const char *)host;
    void *dev = deviceArray(ctx, f);
    for (int ch = 0; ch < nch; ++ch) {
      const int64_t ne = chunkElems(chunkGeom(ctx, f, ch));
      CK(cudaMemcpyAsync(ctx->staging, src, ne * 8, cudaMemcpyHostToDevice, ctx->stream));
      XposeDesc x = chunkXpose(ctx, f, ch);
      if (ctx->prec == KGB_FP64) launch_upload_xpose<double>(ctx->staging, as<double>(dev), x, ctx->stream);
      else launch_upload_xpose<float>(ctx->staging, as<float>(dev), x, ctx->stream);
      CKN(1);
      src += ne * 8;
    }
    CK(cudaStreamSynchronize(ctx->stream));
    ctx->have[fieldIndex(f)] = true;
    if (f->kind == K_SIGT) ctx->dirty_sigt = true;
    return KGB_OK;
  }
  // host-side inputs: convert the chunks into global host tables
  const double *hd = (const double *)host;
  const int32_t *hi = (const int32_t *)host;
  int64_t off = 0;
  for (int ch = 0; ch < nch; ++ch) {
    ChunkGeom g = chunkGeom(ctx, f, ch);
    int64_t st[4] = {1, 1, 1, 1};
    nestStrides(layout, g.nd, g.types, g.dims, st);
    int co[5];
    ctx->dc.chunkCoord(g.space, ch, co);
    const int dlo = co[1] * ctx->Ds;
    switch (f->kind) {
      case K_ELL:
        for (int m = 0; m < ctx->M; ++m)
          for (int d = 0; d < ctx->Ds; ++d) ctx->ell_h[(size_t)(dlo + d) * ctx->M + m] = hd[off + m * st[0] + d * st[1]];
        break;
      case K_ELLP:
        for (int d = 0; d < ctx->Ds; ++d)
          for (int m = 0; m < ctx->M; ++m) ctx->ellp_h[(size_t)(dlo + d) * ctx->M + m] = hd[off + d * st[0] + m * st[1]];
        break;
      case K_SIGS: {
        const int L1 = ctx->L + 1, G = ctx->G;
        for (int m = 0; m < 3; ++m)
          for (int l = 0; l < L1; ++l)
            for (int g2 = 0; g2 < G; ++g2)
              for (int gp = 0; gp < G; ++gp)
                ctx->sigs_h[(((size_t)m * L1 + l) * G + g2) * G + gp] = hd[off + m * st[0] + l * st[1] + g2 * st[2] + gp * st[3]];
        break;
      }
      case K_QD:
        for (int d = 0; d < ctx->Ds; ++d) ctx->q[f->which][dlo + d] = hd[off + d];
        break;
      case K_QI:
        for (int d = 0; d < ctx->Ds; ++d) {
          const int v = hi[off + d];
          if (v != 1 && v != -1) return fail(ctx, KGB_ERR_ARG, "direction flags must be +1 or -1");
          ctx->qi[f->which][dlo + d] = v;
        }
        break;
      case K_DXYZ: {
        const int n = (int)g.dims[0], o = co[2 + f->which] * n;
        for (int i = 0; i < n; ++i) {
          if (!(hd[off + i] > 0.0)) return fail(ctx, KGB_ERR_ARG, "zone widths must be positive");
          ctx->dxyz[f->which][o + i] = hd[off + i];
        }
        break;
      }
      case K_VOL: {
        const int io = co[2] * ctx->nxs, jo = co[3] * ctx->nys, ko = co[4] * ctx->nzs;
        for (int64_t zl = 0; zl < ctx->Zs; ++zl) {
          int64_t i = zl % ctx->nxs, j = (zl / ctx->nxs) % ctx->nys, k = zl / ((int64_t)ctx->nxs * ctx->nys);
          ctx->vol_h[((k + ko) * ctx->ny + (j + jo)) * ctx->nx + (i + io)] = hd[off + zl];
        }
        break;
      }
      case K_ZI: {
        const int r = ctx->dc.rIndex(co);
        ctx->zmap[f->which][r].assign(hi + off, hi + off + ctx->Zs);
        break;
      }
      case K_MI: {
        const int r = ctx->dc.rIndex(co);
        ctx->mimap[f->which][r].assign(hi + off, hi + off + g.dims[0]);
        break;
      }
      case K_MD: {
        const int r = ctx->dc.rIndex(co);
        ctx->mfrac[r].assign(hd + off, hd + off + g.dims[0]);
        break;
      }
      case K_M2L:
        for (int m = 0; m < ctx->M; ++m)
          if (hi[off + m] != ctx->m2l[m]) return fail(ctx, KGB_ERR_ARG, "moment_to_legendre must list n=0..L with 2n+1 moments each");
        break;
      default: break;
    }
    off += chunkElems(g);
  }
  switch (f->kind) {
    case K_ELL: case K_ELLP: ctx->dirty_ell = true; break;
    case K_SIGS: ctx->dirty_sigs = true; break;
    case K_QD: case K_QI: ctx->dirty_quad = true; ctx->dirty_geom = true; break;
    case K_DXYZ: ctx->dirty_geom = true; break;
    case K_VOL: ctx->dirty_vol = true; break;
    case K_ZI: case K_MI: case K_MD: ctx->dirty_mix = true; break;
    default: break;
  }
  if (f->kind == K_ZI && f->which == 1) {
    // counts changed: mixed-element fields must be uploaded again
    for (const char *n : {"mixelem_to_zone", "mixelem_to_material", "mixelem_to_fraction"}) ctx->have[fieldIndex(findField(n))] = false;
  }
  ctx->have[fieldIndex(f)] = true;
  return KGB_OK;
}

int kgb_field_download(kgb_ctx *ctx, const char *name, void *host, int64_t nbytes) {
  if (!ctx) return KGB_ERR_ARG;
  if (!ctx->ready) return fail(ctx, KGB_ERR_STATE, "kgb_setup has not been called");
  const FieldInfo *f = findField(name);
  if (!f) return fail(ctx, KGB_ERR_ARG, std::string("unknown field '") + (name ? name : "(null)") + "'");
  if (!host && nbytes > 0) return fail(ctx, KGB_ERR_ARG, "null host pointer");
  const int64_t want = fieldBytes(ctx, f);
  if (nbytes != want)
    return fail(ctx, KGB_ERR_ARG, std::string("field '") + name + "' holds " + std::to_string(want) + " bytes, got " + std::to_string(nbytes));
  CK(cudaSetDevice(ctx->device));
  if (!std::strcmp(f->name, "rhs")) {
    int rc = ensureRhs(ctx);
    if (rc) return rc;
  }
  const int nch = numChunks(ctx, f);
  if (deviceKind(f->kind)) {
    size_t maxc = 0;
    for (int ch = 0; ch < nch; ++ch) maxc = std::max<size_t>(maxc, chunkElems(chunkGeom(ctx, f, ch)) * 8);
    int rc = ensureStaging(ctx, maxc);
    if (rc) return rc;
    char *dst = (char *)host;
    const void *dev = deviceArray(ctx, f);
    for (int ch = 0; ch < nch; ++ch) {
      const int64_t ne = chunkElems(chunkGeom(ctx, f, ch));
      XposeDesc x = chunkXpose(ctx, f, ch);
      if (ctx->prec == KGB_FP64) launch_download_xpose<double>(as<const double>(const_cast<void *>(dev)), ctx->staging, x, ctx->stream);
      else launch_download_xpose<float>(as<const float>(const_cast<void *>(dev)), ctx->staging, x, ctx->stream);
      CKN(1);
      CK(cudaMemcpyAsync(dst, ctx->staging, ne * 8, cudaMemcpyDeviceToHost, ctx->stream));
      CK(cudaStreamSynchronize(ctx->stream));
      dst += ne * 8;
    }
    return KGB_OK;
  }
  // host-side inputs: rebuild Kripke's chunks from the global tables
  double *hd = (double *)host;
  int32_t *hi = (int32_t *)host;
  int64_t off = 0;
  for (int ch = 0; ch < nch; ++ch) {
    ChunkGeom g = chunkGeom(ctx, f, ch);
    int64_t st[4] = {1, 1, 1, 1};
    nestStrides(ctx->dims.layout, g.nd, g.types, g.dims, st);
    int co[5];
    ctx->dc.chunkCoord(g.space, ch, co);
    const int dlo = co[1] * ctx->Ds;
    switch (f->kind) {
      case K_ELL:
        for (int m = 0; m < ctx->M; ++m)
          for (int d = 0; d < ctx->Ds; ++d) hd[off + m * st[0] + d * st[1]] = ctx->ell_h[(size_t)(dlo + d) * ctx->M + m];
        break;
      case K_ELLP:
        for (int d = 0; d < ctx->Ds; ++d)
          for (int m = 0; m < ctx->M; ++m) hd[off + d * st[0] + m * st[1]] = ctx->ellp_h[(size_t)(dlo + d) * ctx->M + m];
        break;
      case K_SIGS: {
        const int L1 = ctx->L + 1, G = ctx->G;
        for (int m = 0; m < 3; ++m)
          for (int l = 0; l < L1; ++l)
            for (int g2 = 0; g2 < G; ++g2)
              for (int gp = 0; gp < G; ++gp)
                hd[off + m * st[0] + l * st[1] + g2 * st[2] + gp * st[3]] = ctx->sigs_h[(((size_t)m * L1 + l) * G + g2) * G + gp];
        break;
      }
      case K_QD:
        for (int d = 0; d < ctx->Ds; ++d) hd[off + d] = ctx->q[f->which][dlo + d];
        break;
      case K_QI:
        for (int d = 0; d < ctx->Ds; ++d) hi[off + d] = ctx->qi[f->which][dlo + d];
        break;
      case K_DXYZ: {
        const int n = (int)g.dims[0], o = co[2 + f->which] * n;
        for (int i = 0; i < n; ++i) hd[off + i] = ctx->dxyz[f->which][o + i];
        break;
      }
      case K_VOL: {
        const int io = co[2] * ctx->nxs, jo = co[3] * ctx->nys, ko = co[4] * ctx->nzs;
        for (int64_t zl = 0; zl < ctx->Zs; ++zl) {
          int64_t i = zl % ctx->nxs, j = (zl / ctx->nxs) % ctx->nys, k = zl / ((int64_t)ctx->nxs * ctx->nys);
          hd[off + zl] = ctx->vol_h[((k + ko) * ctx->ny + (j + jo)) * ctx->nx + (i + io)];
        }
        break;
      }
      case K_ZI: {
        const int r = ctx->dc.rIndex(co);
        std::copy(ctx->zmap[f->which][r].begin(), ctx->zmap[f->which][r].end(), hi + off);
        break;
      }
      case K_MI: {
        const int r = ctx->dc.rIndex(co);
        std::copy(ctx->mimap[f->which][r].begin(), ctx->mimap[f->which][r].end(), hi + off);
        break;
      }
      case K_MD: {
        const int r = ctx->dc.rIndex(co);
        std::copy(ctx->mfrac[r].begin(), ctx->mfrac[r].end(), hd + off);
        break;
      }
      case K_M2L:
        for (int m = 0; m < ctx->M; ++m) hi[off + m] = ctx->m2l[m];
        break;
      default: break;
    }
    off += chunkElems(g);
  }
  return KGB_OK;
}

int kgb_field_fill(kgb_ctx *ctx, const char *name, double value) {
  if (!ctx) return KGB_ERR_ARG;
  if (!ctx->ready) return fail(ctx, KGB_ERR_STATE, "kgb_setup has not been called");
  const FieldInfo *f = findField(name);
  if (!f) return fail(ctx, KGB_ERR_ARG, std::string("unknown field '") + (name ? name : "(null)") + "'");
  CK(cudaSetDevice(ctx->device));
  if (!std::strcmp(f->name, "rhs")) ctx->rhs_stale = false;
  return fillField(ctx, f, value);
}

int kgb_ltimes(kgb_ctx *ctx) {
  int rc = prepare(ctx);
  return rc ? rc : doLTimes(ctx, true);
}

int kgb_lplustimes(kgb_ctx *ctx) {
  int rc = prepare(ctx);
  if (!rc) rc = ensureRhs(ctx);
  return rc ? rc : doLPlusTimes(ctx, true);
}

int kgb_scattering(kgb_ctx *ctx) {
  int rc = prepare(ctx);
  return rc ? rc : doScattering(ctx, true);
}

int kgb_source(kgb_ctx *ctx, double q) {
  int rc = prepare(ctx);
  return rc ? rc : doSource(ctx, q);
}

int kgb_sweep_subdomain(kgb_ctx *ctx, int32_t sdom) {
  int rc = prepare(ctx);
  if (rc) return rc;
  if (sdom < 0 || sdom >= ctx->dc.num()) return fail(ctx, KGB_ERR_ARG, "subdomain id out of range");
  if ((rc = ensureRhs(ctx))) return rc;
  return sweepWaveAny(ctx, ctx->ident_d + sdom, 1);
}

int kgb_sweep_solver(kgb_ctx *ctx) {
  int rc = prepare(ctx);
  if (!rc) rc = ensureRhs(ctx);
  return rc ? rc : sweepSolver(ctx);
}

int kgb_population(kgb_ctx *ctx, double *out) {
  if (!out) return fail(ctx, KGB_ERR_ARG, "null output");
  int rc = prepare(ctx);
  if (rc) return rc;
  if ((rc = doPopulation(ctx, ctx->results))) return rc;
  CK(cudaMemcpyAsync(out, ctx->results, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return KGB_OK;
}

int kgb_balance(kgb_ctx *ctx, double out[5]) {
  if (!out) return fail(ctx, KGB_ERR_ARG, "null output");
  int rc = prepare(ctx);
  if (!rc) rc = ensureRhs(ctx);
  if (rc) return rc;
  const int64_t rows = ctx->Z * ctx->G;
  CK(cudaMemsetAsync(ctx->results, 0, 8 * sizeof(double), ctx->stream));
  if (ctx->prec == KGB_FP64)
    launch_balance_terms<double>(as<double>(ctx->psi), as<double>(ctx->rhs), as<double>(ctx->sigt), ctx->w_d, ctx->vol_d, rows, ctx->G, ctx->D, ctx->partials, ctx->npart, ctx->results, ctx->stream);
  else
    launch_balance_terms<float>(as<float>(ctx->psi), as<float>(ctx->rhs), as<float>(ctx->sigt), ctx->w_d, ctx->vol_d, rows, ctx->G, ctx->D, ctx->partials, ctx->npart, ctx->results, ctx->stream);
  CKN(3);
  // leakage through the planes of subdomains whose downwind face is the domain boundary
  const int S[3] = {ctx->dc.Sx, ctx->dc.Sy, ctx->dc.Sz};
  for (int s = 0; s < ctx->dc.num(); ++s) {
    const SdomDesc &d = ctx->sdoms_h[s];
    const int co[5] = {d.p, d.q, d.xs, d.ys, d.zs};
    const int dirv[3] = {d.id, d.jd, d.kd};
    for (int dim = 0; dim < 3; ++dim) {
      const int dn = co[2 + dim] + dirv[dim];
      if (dn >= 0 && dn < S[dim]) continue;
      // plane chunk [nb][na][Gs][Ds]; face area = wa(a) * wb(b) in global zone widths
      const double *wa, *wb;
      int na;
      if (dim == 0) { wa = ctx->dxyz_d[1] + d.jo; wb = ctx->dxyz_d[2] + d.ko; na = ctx->nys; }
      else if (dim == 1) { wa = ctx->dxyz_d[0] + d.io; wb = ctx->dxyz_d[2] + d.ko; na = ctx->nxs; }
      else { wa = ctx->dxyz_d[0] + d.io; wb = ctx->dxyz_d[1] + d.jo; na = ctx->nxs; }
      const int64_t ne = ctx->plane_chunk[dim];
      const int64_t off = (int64_t)s * ne;
      if (ctx->prec == KGB_FP64)
        launch_leakage<double>(as<double>(ctx->plane[dim]) + off, ne, ctx->Gs, ctx->Ds, d.dlo, na, ctx->w_d, ctx->cos_d[dim], wa, wb, ctx->partials, ctx->npart, ctx->results + 2, ctx->stream);
      else
        launch_leakage<float>(as<float>(ctx->plane[dim]) + off, ne, ctx->Gs, ctx->Ds, d.dlo, na, ctx->w_d, ctx->cos_d[dim], wa, wb, ctx->partials, ctx->npart, ctx->results + 2, ctx->stream);
      CKN(2);
    }
  }
  if ((rc = doPopulation(ctx, ctx->results + 3))) return rc;
  double h[4];
  CK(cudaMemcpyAsync(h, ctx->results, 4 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  out[0] = h[0];
  out[1] = h[1];
  out[2] = h[2];
  out[3] = h[3];
  out[4] = h[0] - h[1] - h[2];
  return KGB_OK;
}

int kgb_iterate(kgb_ctx *ctx, double q, double *part) {
  int rc = prepare(ctx);
  if (rc) return rc;
  // without part, a count is still formed on the device: of the state the iteration starts
  // from (FP64, from the moments; results[1]) or of the new state (mixed, fused; results[0])
  if ((rc = (part || !lagPopulation(ctx)) ? iterateDevice(ctx, q, ctx->results)
                                          : iterateDevice(ctx, q, nullptr, ctx->results + 1)))
    return rc;
  if (part) {
    CK(cudaMemcpyAsync(part, ctx->results, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return checkDeviceError(ctx);
  }
  return KGB_OK;
}

int kgb_solve(kgb_ctx *ctx, int32_t niter, double q, double *part) {
  int rc = prepare(ctx);
  if (rc) return rc;
  if (niter < 1) return fail(ctx, KGB_ERR_ARG, "niter must be >= 1");
  if (niter > ctx->parts_cap) {
    if (ctx->parts_dev) cudaFree(ctx->parts_dev);
    ctx->parts_dev = nullptr;
    ctx->parts_cap = 0;
    ++ctx->gen;
    if ((rc = dmalloc(ctx, &ctx->parts_dev, niter))) return rc;
    ctx->parts_cap = niter;
  }
  ctx->graph_active = false;
  if (ctx->use_graph && !ctx->timing) {
    const kgb_ctx::SolveGraph *sg = nullptr;
    if ((rc = solveGraph(ctx, niter, q, &sg))) return rc;
    if (sg) {
      CK(cudaGraphLaunch(sg->x, ctx->stream));
      ctx->launches += sg->launches;
      ctx->graph_active = true;
    }
  }
  if (!ctx->graph_active) {
    CK(cudaMemsetAsync(ctx->psi, 0, ctx->Z * ctx->G * ctx->D * ctx->tsz, ctx->stream));  // kConst(psi, 0)
    if ((rc = resetPsiExp(ctx)) || (rc = solveIterations(ctx, niter, q))) return rc;
  } else {
    ctx->psi_exp_valid = psiExpUsable(ctx);  // the replayed solve ended with a recording sweep
  }
  if (part) CK(cudaMemcpyAsync(part, ctx->parts_dev, niter * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return checkDeviceError(ctx);
}

int kgb_sync(kgb_ctx *ctx) {
  if (!ctx) return KGB_ERR_ARG;
  CK(cudaSetDevice(ctx->device));
  CK(cudaStreamSynchronize(ctx->stream));
  return ctx->err_d ? checkDeviceError(ctx) : KGB_OK;
}

int kgb_set_stream(kgb_ctx *ctx, void *s) {
  if (!ctx) return KGB_ERR_ARG;
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->stream = s ? (cudaStream_t)s : ctx->own_stream;
  return KGB_OK;
}

int kgb_set_option(kgb_ctx *ctx, const char *key, int64_t value) {
  if (!ctx || !key) return KGB_ERR_ARG;
  ++ctx->gen;
  if (!std::strcmp(key, "graph")) {
    ctx->use_graph = value != 0;
    return KGB_OK;
  }
  if (!std::strcmp(key, "sweep_tile_z")) {
    if (value < 1 || value > 1024) return fail(ctx, KGB_ERR_ARG, "sweep_tile_z must be in [1, 1024]");
    ctx->tz = (int)value;
    ctx->tiles_set = true;
    if (ctx->ready) return buildTiles(ctx);
    return KGB_OK;
  }
  if (!std::strcmp(key, "sweep_tile_xy")) {
    if (value != 44 && value != 42 && value != 22) return fail(ctx, KGB_ERR_ARG, "sweep_tile_xy must be 44, 42 or 22");
    ctx->tiles_set = true;
    ctx->tx = (int)(value / 10);
    ctx->ty = (int)(value % 10);
    if (ctx->ready) return buildTiles(ctx);
    return KGB_OK;
  }
  if (!std::strcmp(key, "moments_tensor")) {
    ctx->allow_tc = value != 0;
    ctx->use_tc_lt = ctx->use_tc_lp = value != 0;
    ctx->dirty_ell = true;
    return KGB_OK;
  }
  if (!std::strcmp(key, "moments_tf32")) {
    ctx->allow_tf32 = value != 0;
    ctx->use_tf32_lt = ctx->use_tf32_lp = value != 0;
    ctx->dirty_ell = true;
    ctx->adj_stale = true;
    ++ctx->gen;
    return KGB_OK;
  }
  if (!std::strcmp(key, "block_jacobi")) {
    if (value != 0 && value != 1) return fail(ctx, KGB_ERR_ARG, "block_jacobi must be 0 (sweep) or 1 (bj)");
    ctx->block_jacobi = value != 0;
    return KGB_OK;
  }
  if (!std::strcmp(key, "sweep_streams")) {
    if (value < 1 || value > kgb_ctx::kMaxSweepStreams) return fail(ctx, KGB_ERR_ARG, "sweep_streams must be 1 to 4");
    ctx->sweep_streams = (int)std::min<int64_t>(value, ctx->max_streams);
    return KGB_OK;
  }
  if (!std::strcmp(key, "fused_sweep")) {
    ctx->fuse_sweep = value != 0;
    return KGB_OK;
  }
  if (!std::strcmp(key, "sweep_l2_hints")) {
    ctx->sweep_l2_hints = value != 0;
    ++ctx->gen;  // captured solves bake the sweep arguments in
    return KGB_OK;
  }
  if (!std::strcmp(key, "row_exponents")) {
    ctx->allow_row_exp = value != 0;
    ctx->psi_exp_valid = false;
    return KGB_OK;
  }
  if (!std::strcmp(key, "scattering_tensor")) {
    ctx->allow_tc_sc = value != 0;
    ctx->use_tc_sc = value != 0;
    ctx->dirty_tcsc = true;
    return KGB_OK;
  }
  if (!std::strcmp(key, "sweep_reciprocals")) {
    ctx->allow_recip = value != 0;
    ctx->dirty_sigt = true;
    return KGB_OK;
  }
  return fail(ctx, KGB_ERR_ARG, std::string("unknown option '") + key + "'");
}

int kgb_autotune(kgb_ctx *ctx, double *best_ms, int32_t *tile_xy, int32_t *tile_z) {
  int rc = prepare(ctx);
  if (!rc) rc = ensureRhs(ctx);
  if (rc) return rc;
  const int xys[3] = {44, 42, 22};
  const int tzs[4] = {2, 4, 8, 16};
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  const bool timing = ctx->timing;
  ctx->timing = false;
  float best = 1e30f;
  int bxy = 44, btz = 4;
  // the sweep variant the solver runs: fused population partials unless the FP64
  // count comes from the next iteration's moments
  const bool pop = !lagPopulation(ctx);
  for (int xy : xys)
    for (int tz : tzs) {
      if (tz > 2 * ctx->nzs && tz != 2) continue;
      ctx->tx = xy / 10;
      ctx->ty = xy % 10;
      ctx->tz = tz;
      if ((rc = buildTiles(ctx))) break;
      if ((rc = sweepSolver(ctx, pop))) break;  // warm-up
      CK(cudaEventRecord(e0, ctx->stream));
      for (int r = 0; r < 2; ++r)
        if ((rc = sweepSolver(ctx, pop))) break;
      CK(cudaEventRecord(e1, ctx->stream));
      CK(cudaEventSynchronize(e1));
      float ms = 0.f;
      CK(cudaEventElapsedTime(&ms, e0, e1));
      ms *= 0.5f;
      if (ms < best) {
        best = ms;
        bxy = xy;
        btz = tz;
      }
    }
  ctx->timing = timing;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) return rc;
  ctx->tx = bxy / 10;
  ctx->ty = bxy % 10;
  ctx->tz = btz;
  if ((rc = buildTiles(ctx))) return rc;
  // moment transforms: tensor-core digit products or SIMT, whichever is faster here
  cudaEvent_t f0, f1;
  CK(cudaEventCreate(&f0));
  CK(cudaEventCreate(&f1));
  // mode 2: split-TF32 tensor cores (mixed form), 1: exact digit products, 0: SIMT
  auto setMode = [&](bool lt, int mode) {
    (lt ? ctx->use_tf32_lt : ctx->use_tf32_lp) = mode == 2;
    (lt ? ctx->use_tc_lt : ctx->use_tc_lp) = mode == 1;
  };
  auto timeIt = [&](bool lt, int mode, float &ms) -> int {
    setMode(lt, mode);
    int r = lt ? doLTimes(ctx, false) : doLPlusTimes(ctx, false);  // warm-up
    if (r) return r;
    CK(cudaEventRecord(f0, ctx->stream));
    for (int k = 0; k < 2 && !r; ++k) r = lt ? doLTimes(ctx, false) : doLPlusTimes(ctx, false);
    CK(cudaEventRecord(f1, ctx->stream));
    CK(cudaEventSynchronize(f1));
    CK(cudaEventElapsedTime(&ms, f0, f1));
    return r ? r : checkDeviceError(ctx);
  };
  for (int lt = 1; lt >= 0 && !rc; --lt) {
    const bool tf32 = ctx->prec == KGB_MIXED && ctx->allow_tf32 && (lt ? ctx->tf32_lt_img : ctx->tf32_lp_img);
    const bool tc = lt ? ctx->tc_lt : ctx->tc_lp;
    float best_t = 0.f;
    int best_mode = -1;
    for (int mode = 2; mode >= 0 && !rc; --mode) {
      if ((mode == 2 && !tf32) || (mode == 1 && !tc)) continue;
      float t = 0.f;
      if ((rc = timeIt(lt, mode, t))) break;
      if (best_mode < 0 || t < best_t) {
        best_t = t;
        best_mode = mode;
      }
    }
    if (!rc && best_mode >= 0) setMode(lt, best_mode);
  }
  // scattering: tensor-core digit products for single-material zones, or SIMT
  auto timeScat = [&](bool tc, float &ms) -> int {
    ctx->use_tc_sc = tc;
    int r = doScattering(ctx, false);
    if (r) return r;
    CK(cudaEventRecord(f0, ctx->stream));
    for (int k = 0; k < 2 && !r; ++k) r = doScattering(ctx, false);
    CK(cudaEventRecord(f1, ctx->stream));
    CK(cudaEventSynchronize(f1));
    CK(cudaEventElapsedTime(&ms, f0, f1));
    return r ? r : checkDeviceError(ctx);
  };
  if (!rc && ctx->tc_sc) {
    float t_tc = 0.f, t_simt = 0.f;
    if (!(rc = timeScat(true, t_tc)) && !(rc = timeScat(false, t_simt))) ctx->use_tc_sc = t_tc <= t_simt;
  }
  ++ctx->gen;  // kernel choices may have changed
  cudaEventDestroy(f0);
  cudaEventDestroy(f1);
  if (rc) return rc;
  if (best_ms) *best_ms = best;
  if (tile_xy) *tile_xy = bxy;
  if (tile_z) *tile_z = btz;
  return KGB_OK;
}

int kgb_get_option(kgb_ctx *ctx, const char *key, int64_t *value) {
  if (!ctx || !key || !value) return KGB_ERR_ARG;
  if (!std::strcmp(key, "sweep_tile_z")) *value = ctx->tz;
  else if (!std::strcmp(key, "sweep_tile_xy")) *value = ctx->tx * 10 + ctx->ty;
  else if (!std::strcmp(key, "sweep_reciprocals")) *value = ctx->allow_recip ? 1 : 0;
  else if (!std::strcmp(key, "sweep_reciprocals_active")) *value = ctx->use_recip ? 1 : 0;
  else if (!std::strcmp(key, "moments_tensor")) *value = ctx->allow_tc ? 1 : 0;
  else if (!std::strcmp(key, "moments_tensor_ltimes")) *value = (ctx->tc_lt && ctx->use_tc_lt) ? 1 : 0;
  else if (!std::strcmp(key, "moments_tensor_lplustimes")) *value = (ctx->tc_lp && ctx->use_tc_lp) ? 1 : 0;
  else if (!std::strcmp(key, "moments_tf32")) *value = ctx->allow_tf32 ? 1 : 0;
  else if (!std::strcmp(key, "moments_tf32_ltimes")) *value = tf32LtActive(ctx) ? 1 : 0;
  else if (!std::strcmp(key, "moments_tf32_lplustimes")) *value = tf32LpActive(ctx) ? 1 : 0;
  else if (!std::strcmp(key, "graph")) *value = ctx->use_graph ? 1 : 0;
  else if (!std::strcmp(key, "scattering_tensor")) *value = ctx->allow_tc_sc ? 1 : 0;
  else if (!std::strcmp(key, "scattering_tensor_active")) *value = (ctx->tc_sc && ctx->use_tc_sc) ? 1 : 0;
  else if (!std::strcmp(key, "graph_active")) *value = ctx->graph_active ? 1 : 0;
  else if (!std::strcmp(key, "block_jacobi")) *value = ctx->block_jacobi ? 1 : 0;
  else if (!std::strcmp(key, "fused_sweep")) *value = ctx->fuse_sweep ? 1 : 0;
  else if (!std::strcmp(key, "sweep_streams")) *value = ctx->sweep_streams;
  else if (!std::strcmp(key, "sweep_l2_hints")) *value = ctx->sweep_l2_hints ? 1 : 0;
  else if (!std::strcmp(key, "fused_sweep_active")) *value = ctx->fuse_active ? 1 : 0;
  else if (!std::strcmp(key, "row_exponents")) *value = ctx->allow_row_exp ? 1 : 0;
  else if (!std::strcmp(key, "phi_row_exponents_active")) *value = phiExpUsable(ctx) ? 1 : 0;
  else if (!std::strcmp(key, "psi_row_exponents_active")) *value = psiExpUsable(ctx) ? 1 : 0;
  else if (!std::strcmp(key, "psi_row_exponents_valid")) *value = ctx->psi_exp_valid ? 1 : 0;
  else return fail(ctx, KGB_ERR_ARG, std::string("unknown option '") + key + "'");
  return KGB_OK;
}

int kgb_set_timing(kgb_ctx *ctx, int on) {
  if (!ctx) return KGB_ERR_ARG;
  ctx->timing = on != 0;
  return KGB_OK;
}

int kgb_kernel_time(kgb_ctx *ctx, const char *family, double *ms, int64_t *launches) {
  if (!ctx || !family || !ms || !launches) return KGB_ERR_ARG;
  CK(cudaStreamSynchronize(ctx->stream));
  auto it = ctx->fams.find(family);
  if (it == ctx->fams.end()) {
    *ms = 0.0;
    *launches = 0;
    return KGB_OK;
  }
  TimerFam &f = it->second;
  for (auto &pr : f.pending) {
    float t = 0.f;
    cudaEventElapsedTime(&t, pr.first, pr.second);
    f.ms += t;
    cudaEventDestroy(pr.first);
    cudaEventDestroy(pr.second);
  }
  f.pending.clear();
  *ms = f.ms;
  *launches = f.launches;
  return KGB_OK;
}

int kgb_launch_count(kgb_ctx *ctx, int64_t *out) {
  if (!ctx || !out) return KGB_ERR_ARG;
  *out = ctx->launches;
  return KGB_OK;
}

// --- converged solves, the adjoint and gradients ---------------------------

int kgb_set_materials(kgb_ctx *ctx, const double *sigt, const double *sigs) {
  if (!ctx) return KGB_ERR_ARG;
  if (!ctx->ready) return fail(ctx, KGB_ERR_STATE, "kgb_setup has not been called");
  if (sigs) {
    ctx->sigs_h.assign(sigs, sigs + (size_t)3 * (ctx->L + 1) * ctx->G * ctx->G);
    ctx->have[fieldIndex(findField("data/sigs"))] = true;
    ctx->dirty_sigs = true;
  }
  if (sigt) ctx->have[fieldIndex(findField("sigt_zonal"))] = true;
  ctx->have_lam = false;
  int rc = prepare(ctx);  // mixture tables on the device
  if (rc || !sigt) return rc;
  if ((rc = ensureStaging(ctx, (size_t)3 * ctx->G * sizeof(double)))) return rc;
  CK(cudaMemcpyAsync(ctx->staging, sigt, (size_t)3 * ctx->G * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  const MixArgs a = mixArgs(ctx);
  if (ctx->prec == KGB_FP64)
    launch_material_sigt<double>(as<double>(ctx->sigt), ctx->staging, a, ctx->stream);
  else
    launch_material_sigt<float>(as<float>(ctx->sigt), ctx->staging, a, ctx->stream);
  CKN(1);
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->dirty_sigt = true;  // tabulated sweep reciprocals
  return prepare(ctx);
}

int kgb_set_response(kgb_ctx *ctx, const double *det, int64_t n) {
  if (!ctx) return KGB_ERR_ARG;
  if (!ctx->ready) return fail(ctx, KGB_ERR_STATE, "kgb_setup has not been called");
  if (det && n != ctx->Z) return fail(ctx, KGB_ERR_ARG, "detector weights need one value per zone");
  CK(cudaSetDevice(ctx->device));
  int rc = ensureResponseBuffers(ctx);
  if (rc) return rc;
  if (det) {
    CK(cudaMemcpyAsync(ctx->det_d, det, ctx->Z * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  } else {
    launch_fill<double>(ctx->det_d, ctx->Z, 1.0, ctx->stream);
    CKN(1);
  }
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->have_lam = false;
  return KGB_OK;
}

int kgb_solve_converged(kgb_ctx *ctx, double source_strength, double tol, int32_t max_iter, int32_t *iters,
                        double *change) {
  int rc = prepare(ctx);
  if (rc) return rc;
  if (max_iter < 1 || std::isnan(tol)) return fail(ctx, KGB_ERR_ARG, "need max_iter >= 1 and a tolerance");
  if ((rc = ensureResponseBuffers(ctx))) return rc;
  if ((rc = convergeLoop(ctx, false, source_strength, tol, max_iter, iters, change))) return rc;
  return checkDeviceError(ctx);
}

int kgb_adjoint_solve(kgb_ctx *ctx, double tol, int32_t max_iter, int32_t *iters, double *change) {
  int rc = prepare(ctx);
  if (rc) return rc;
  if (max_iter < 1 || std::isnan(tol)) return fail(ctx, KGB_ERR_ARG, "need max_iter >= 1 and a tolerance");
  if ((rc = prepareAdjoint(ctx))) return rc;
  if (ctx->inv_c0 == 0.0)
    return fail(ctx, KGB_ERR_ARG, "the adjoint source needs ell(0, d) proportional to the quadrature weight w(d)");
  if (!ctx->lam && (rc = dalloc(ctx, &ctx->lam, (size_t)ctx->Z * ctx->G * ctx->D * ctx->tsz))) return rc;
  ctx->have_lam = false;
  {
    AdjointView view(ctx);
    rc = convergeLoop(ctx, true, 0.0, tol, max_iter, iters, change);
  }
  if (rc) return rc;
  if ((rc = checkDeviceError(ctx))) return rc;
  ctx->have_lam = true;
  return KGB_OK;
}

int kgb_response(kgb_ctx *ctx, double *response) {
  if (!response) return fail(ctx, KGB_ERR_ARG, "null output");
  int rc = prepare(ctx);
  if (rc || (rc = prepareAdjoint(ctx))) return rc;
  std::vector<double> t;
  if ((rc = responseTermsOf(ctx, ctx->psi, nullptr, nullptr, t))) return rc;
  double r = 0.0;
  for (int g = 0; g < ctx->G; ++g) r += t[(size_t)g * kRespTerms + 12];
  *response = r;
  return KGB_OK;
}

int kgb_gradient(kgb_ctx *ctx, double *response, double *dsigt, double *dsigs, double *dq) {
  int rc = prepare(ctx);
  if (rc || (rc = prepareAdjoint(ctx))) return rc;
  if (!ctx->have_lam || !ctx->lam) return fail(ctx, KGB_ERR_STATE, "kgb_adjoint_solve has not run for these inputs");
  std::vector<double> t;
  if ((rc = responseTermsOf(ctx, ctx->psi, ctx->psi, ctx->lam, t))) return rc;
  const int G = ctx->G;
  double r = 0.0, q = 0.0;
  for (int g = 0; g < G; ++g) {
    const double *x = &t[(size_t)g * kRespTerms];
    r += x[12];
    q += x[3];  // material 0 carries the source
    for (int m = 0; m < 3; ++m) {
      if (dsigt) dsigt[m * G + g] = x[m * 4 + 0] - x[m * 4 + 1];
      if (dsigs) dsigs[m * G + g] = x[m * 4 + 2] - x[m * 4 + 0];
    }
  }
  if (response) *response = r;
  if (dq) *dq = q;
  return KGB_OK;
}

int kgb_gradient_unrolled(kgb_ctx *ctx, int32_t niter, double source_strength, int32_t stride, double *response,
                          double *dsigt, double *dsigs, double *dq) {
  int rc = prepare(ctx);
  if (rc || (rc = prepareAdjoint(ctx))) return rc;
  if (niter < 1) return fail(ctx, KGB_ERR_ARG, "need niter >= 1");
  if (ctx->inv_c0 == 0.0)
    return fail(ctx, KGB_ERR_ARG, "the adjoint source needs ell(0, d) proportional to the quadrature weight w(d)");
  if (!ctx->lam && (rc = dalloc(ctx, &ctx->lam, (size_t)ctx->Z * ctx->G * ctx->D * ctx->tsz))) return rc;
  ctx->have_lam = false;
  const int K = niter;
  const int c = stride > 0 ? std::min<int>(stride, K) : std::max(1, (int)std::ceil(std::sqrt((double)K)));
  const int ncp = (K - 1) / c;  // checkpoints psi_c, psi_2c, ... below psi_K
  const size_t pbytes = (size_t)ctx->Z * ctx->G * ctx->D * ctx->tsz;
  PsiBuffers cp, seg;
  for (int i = 0; i < ncp + c - 1; ++i) {
    void *p = nullptr;
    if (cudaMalloc(&p, pbytes) != cudaSuccess) {
      cudaGetLastError();
      return fail(ctx, KGB_ERR_OOM, "checkpoint buffers do not fit: raise the stride");
    }
    (i < ncp ? cp.b : seg.b).push_back(p);
  }
  // iterate j lives in: psi (j = K), a checkpoint (j a multiple of c) or a segment slot
  auto buf = [&](int j) -> void * {
    if (j == 0) return nullptr;
    if (j == K) return ctx->psi;
    return j % c == 0 ? cp.b[j / c - 1] : seg.b[j % c - 1];
  };
  for (int j = 1; j <= K; ++j)
    if ((rc = forwardStep(ctx, buf(j - 1), buf(j), source_strength))) return rc;
  const int G = ctx->G;
  std::vector<double> tot((size_t)G * kRespTerms, 0.0), t;
  bool first = true;
  for (int sgm = ncp; sgm >= 0; --sgm) {
    const int j0 = sgm * c, j1 = std::min(j0 + c, K);
    if (sgm < ncp)  // the last segment's iterates are still resident from the forward pass
      for (int j = j0 + 1; j < j1; ++j)
        if ((rc = forwardStep(ctx, buf(j - 1), buf(j), source_strength))) return rc;
    for (int k = j1 - 1; k >= j0; --k) {
      {
        AdjointView view(ctx);
        rc = reverseStep(ctx, first);
      }
      if (rc) return rc;
      if ((rc = responseTermsOf(ctx, buf(k + 1), buf(k), ctx->lam, t))) return rc;
      for (size_t i = 0; i < tot.size(); ++i) {
        const int term = (int)(i % kRespTerms);
        if (first || (term != 12 && term % 4 != 0)) tot[i] += t[i];  // E and R belong to psi_K alone
      }
      first = false;
    }
  }
  double r = 0.0, q = 0.0;
  for (int g = 0; g < G; ++g) {
    const double *x = &tot[(size_t)g * kRespTerms];
    r += x[12];
    q += x[3];
    for (int m = 0; m < 3; ++m) {
      if (dsigt) dsigt[m * G + g] = x[m * 4 + 0] - x[m * 4 + 1];
      if (dsigs) dsigs[m * G + g] = x[m * 4 + 2] - x[m * 4 + 0];
    }
  }
  if (response) *response = r;
  if (dq) *dq = q;
  return checkDeviceError(ctx);
}

int kgb_reset_timers(kgb_ctx *ctx) {
  if (!ctx) return KGB_ERR_ARG;
  CK(cudaStreamSynchronize(ctx->stream));
  for (auto &kv : ctx->fams)
    for (auto &pr : kv.second.pending) {
      cudaEventDestroy(pr.first);
      cudaEventDestroy(pr.second);
    }
  ctx->fams.clear();
  return KGB_OK;
}

}  // extern "C"
