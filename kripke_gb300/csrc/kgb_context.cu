// kgb_context.cu -- contexts and fields of the C ABI: create, set up, upload and
// download in Kripke's host layout (transposed on the device), and the derived
// device tables and kernel plans built lazily from the host inputs.
#include "kgb_ctx.h"

namespace kgb {
namespace api {


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
                  c->psi_exp, c->phi_exp, c->tf32_lt_img, c->tf32_lp_img, c->tf32_lt_img_adj, c->tf32_lp_img_adj,
                  c->lt_sym, c->lt_sym_adj};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  c->psi = c->rhs = c->phi = c->phi_out = c->sigt = nullptr;
  c->psi_exp = c->phi_exp = nullptr;
  c->psi_exp_valid = false;
  c->tf32_lt_img = c->tf32_lp_img = c->tf32_lt_img_adj = c->tf32_lp_img_adj = nullptr;
  c->lt_sym = c->lt_sym_adj = nullptr;
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
// Derived device tables (built lazily when inputs change)
// ---------------------------------------------------------------------------

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

template int planTensorMomentsFrom<double>(kgb_ctx *ctx, const std::vector<double> &lt_src, const std::vector<double> &lp_src,
                          bool *lt_ok, uint16_t **lt_img, int **lt_exp, int *lt_kpad, bool *lp_ok, uint16_t **lp_img,
                          int **lp_exp, int *lp_nhalf);
template int planTensorMomentsFrom<float>(kgb_ctx *ctx, const std::vector<double> &lt_src, const std::vector<double> &lp_src,
                          bool *lt_ok, uint16_t **lt_img, int **lt_exp, int *lt_kpad, bool *lp_ok, uint16_t **lp_img,
                          int **lp_exp, int *lp_nhalf);

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

int planLtSym(kgb_ctx *ctx, const std::vector<double> &lt_src, int **table) {
  if (*table) cudaFree(*table);
  *table = nullptr;
  std::vector<int> t;
  if (ctx->prec != KGB_MIXED || !ltimes_sym_table(lt_src.data(), ctx->D, ctx->M, t)) return KGB_OK;
  int rc;
  if ((rc = dmalloc(ctx, table, t.size()))) return rc;
  if (cudaMemcpyAsync(*table, t.data(), t.size() * sizeof(int), cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess ||
      cudaStreamSynchronize(ctx->stream) != cudaSuccess)
    return fail(ctx, KGB_ERR_CUDA, "octant-pair table upload failed");
  return KGB_OK;
}

bool ltSymActive(const kgb_ctx *ctx) {
  return ctx->prec == KGB_MIXED && ctx->allow_lt_stream && ctx->allow_lt_sym && ctx->lt_sym != nullptr &&
         ltimes_stream_applies(ctx->D, ctx->M);
}

bool tf32LtActive(const kgb_ctx *ctx) {
  return ctx->prec == KGB_MIXED && ctx->allow_tf32 && ctx->allow_tf32_lt && ctx->use_tf32_lt &&
         ctx->tf32_lt_img != nullptr;
}
bool tf32LpActive(const kgb_ctx *ctx) {
  return ctx->prec == KGB_MIXED && ctx->allow_tf32 && ctx->allow_tf32_lp && ctx->use_tf32_lp &&
         ctx->tf32_lp_img != nullptr;
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
  // the zone lists serve the tensor-core kernel and the mixed form's zone-blocked one
  const bool blk = ctx->prec == KGB_MIXED && ctx->allow_blk_sc && scatter_block_applies(G, ctx->L);
  if ((!ctx->allow_tc_sc && !blk) || G > 64) return KGB_OK;
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
  if (!ctx->allow_tc_sc) {
    CK(cudaStreamSynchronize(ctx->stream));  // the host list is freed on return
    return KGB_OK;
  }
  // digit images (N blocks of 32 columns): forward B[k][n] = S(n <- k), adjoint B[k][n] = S(k <- n);
  // they depend on the scattering tables only, so a new mix of zones keeps them
  const int kpad = (G + 31) / 32 * 32, nbk = (G + 31) / 32;
  if (!ctx->tcsc_img_stale && ctx->tc_sc_img && ctx->tc_sc_img_adj && ctx->tc_sc_kpad == kpad) {
    CK(cudaStreamSynchronize(ctx->stream));  // the host list is freed on return
    ctx->tc_sc = true;
    return KGB_OK;
  }
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
  ctx->tcsc_img_stale = false;
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
    if ((rc = planLtSym(ctx, ctx->ell_h, &ctx->lt_sym))) return rc;
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
    ctx->tcsc_img_stale = true;
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
  // population partials: one per (tile, subdomain, chain block); the streamed FP32
  // sweep's blocks may hold fewer chains (whole groups) than the per-step kernel's
  const int sbt = ctx->prec == KGB_FP64 ? 0 : stream_block_chains(ctx->Ds, ctx->Gs);
  const int64_t ncb = std::max<int64_t>((nchain + kSweepThreads - 1) / kSweepThreads, sbt > 0 ? nchain / sbt : 0);
  const int64_t nslots = (int64_t)tiles.size() * ctx->dc.num() * ncb;
  if (ctx->pop_slots) cudaFree(ctx->pop_slots);
  ctx->pop_slots = nullptr;
  if ((rc = dmalloc(ctx, &ctx->pop_slots, nslots))) return rc;
  ctx->npop_slots = nslots;
  CK(cudaMemcpyAsync(ctx->tiles_d, tiles.data(), tiles.size() * sizeof(int4), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return KGB_OK;
}


}  // namespace api
}  // namespace kgb

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


}  // extern "C"
