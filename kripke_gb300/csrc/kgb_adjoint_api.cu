// kgb_adjoint_api.cu -- converged solves, the adjoint source iteration, the
// region-integrated absorption response and its gradients (at the fixed point,
// and through unrolled iterations with checkpoints).
#include "kgb_ctx.h"

namespace kgb {
namespace api {

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
  if ((rc = planLtSym(ctx, ctx->ellp_h, &ctx->lt_sym_adj))) return rc;
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
    std::swap(c->lt_sym, c->lt_sym_adj);
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


}  // namespace api
}  // namespace kgb

extern "C" {

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


}  // extern "C"
