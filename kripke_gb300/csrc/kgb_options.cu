// kgb_options.cu -- options, the autotuner and the per-family timers of the C ABI.
#include "kgb_ctx.h"

namespace kgb {
namespace api {



}  // namespace api
}  // namespace kgb

extern "C" {

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
    ctx->use_tf32_lt = value != 0 && ctx->allow_tf32_lt;
    ctx->use_tf32_lp = value != 0 && ctx->allow_tf32_lp;
    ctx->dirty_ell = true;
    ctx->adj_stale = true;
    ++ctx->gen;
    return KGB_OK;
  }
  const bool tf32_lt = !std::strcmp(key, "moments_tf32_ltimes");
  if (tf32_lt || !std::strcmp(key, "moments_tf32_lplustimes")) {  // one transform, within "moments_tf32"
    (tf32_lt ? ctx->allow_tf32_lt : ctx->allow_tf32_lp) = value != 0;
    (tf32_lt ? ctx->use_tf32_lt : ctx->use_tf32_lp) = value != 0;
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
  if (!std::strcmp(key, "sweep_stream")) {
    ctx->allow_stream = value != 0;
    return KGB_OK;
  }
  if (!std::strcmp(key, "sweep_stream_stages")) {
    if (value < 1 || value > kStreamMaxStages) return fail(ctx, KGB_ERR_ARG, "sweep_stream_stages must be 1 to 4");
    ctx->stream_ns = (int)value;
    return KGB_OK;
  }
  if (!std::strcmp(key, "ltimes_stream")) {
    ctx->allow_lt_stream = value != 0;
    return KGB_OK;
  }
  if (!std::strcmp(key, "ltimes_symmetric")) {
    ctx->allow_lt_sym = value != 0;
    return KGB_OK;
  }
  if (!std::strcmp(key, "ltimes_stream_stages")) {
    if (value < 2 || value > 4) return fail(ctx, KGB_ERR_ARG, "ltimes_stream_stages must be 2 to 4");
    ctx->lt_stream_ns = (int)value;
    return KGB_OK;
  }
  if (!std::strcmp(key, "fused_sweep")) {
    ctx->fuse_sweep = value != 0;
    return KGB_OK;
  }
  if (!std::strcmp(key, "fused_ltimes")) {
    ctx->fuse_lt = value != 0;
    return KGB_OK;
  }
  if (!std::strcmp(key, "scattering_block")) {
    ctx->allow_blk_sc = ctx->use_blk_sc = value != 0;
    ctx->dirty_tcsc = true;  // the zone lists are (re)built with the scattering plan
    ctx->tcsc_img_stale = true;
    ++ctx->gen;
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
    ctx->tcsc_img_stale = true;
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
  const int tzs[5] = {2, 4, 8, 16, 32};
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  const bool timing = ctx->timing;
  ctx->timing = false;
  float best = 1e30f;
  int bxy = 44, btz = 4;
  // the streamed FP32 sweep against the per-step kernel, where both exist
  const bool allow_stream = ctx->allow_stream;
  bool bstream = allow_stream;
  // the sweep variant the solver runs: fused population partials unless the FP64
  // count comes from the next iteration's moments
  const bool pop = !lagPopulation(ctx);
  // one sweep shape: the mean of two timed sweeps after a warm-up one
  auto timeShape = [&](float &ms) -> int {
    int r = buildTiles(ctx);
    if (!r) r = sweepSolver(ctx, pop);  // warm-up
    if (r) return r;
    CK(cudaEventRecord(e0, ctx->stream));
    for (int k = 0; k < 2 && !r; ++k) r = sweepSolver(ctx, pop);
    if (r) return r;
    CK(cudaEventRecord(e1, ctx->stream));
    CK(cudaEventSynchronize(e1));
    CK(cudaEventElapsedTime(&ms, e0, e1));
    ms *= 0.5f;
    return KGB_OK;
  };
  for (int xy : xys)
    for (int streamed = 1; streamed >= 0 && !rc; --streamed)
      for (int tz : tzs) {
        if (tz > 2 * ctx->nzs && tz != 2) continue;
        ctx->tx = xy / 10;
        ctx->ty = xy % 10;
        ctx->allow_stream = true;
        const bool can_stream = allow_stream && streamUsable(ctx);
        if (streamed && !can_stream) continue;  // no streamed variant of this shape here
        if (tz == 32 && !streamed) continue;
        ctx->allow_stream = streamed != 0;
        ctx->tz = tz;
        float ms = 0.f;
        if ((rc = timeShape(ms))) break;
        if (ms < best) {
          best = ms;
          bxy = xy;
          btz = tz;
          bstream = streamed != 0;
        }
      }
  ctx->allow_stream = bstream;
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
    const bool tf32 = ctx->prec == KGB_MIXED && ctx->allow_tf32 && (lt ? ctx->allow_tf32_lt : ctx->allow_tf32_lp) &&
                      (lt ? ctx->tf32_lt_img : ctx->tf32_lp_img);
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
  // mode 2: zone-blocked FP32 (mixed form), 1: tensor-core digit products, 0: SIMT
  auto timeScat = [&](int mode, float &ms) -> int {
    ctx->use_blk_sc = mode == 2;
    ctx->use_tc_sc = mode == 1;
    int r = doScattering(ctx, false);
    if (r) return r;
    CK(cudaEventRecord(f0, ctx->stream));
    for (int k = 0; k < 2 && !r; ++k) r = doScattering(ctx, false);
    CK(cudaEventRecord(f1, ctx->stream));
    CK(cudaEventSynchronize(f1));
    CK(cudaEventElapsedTime(&ms, f0, f1));
    return r ? r : checkDeviceError(ctx);
  };
  {
    const bool blk = ctx->prec == KGB_MIXED && ctx->allow_blk_sc && ctx->pure_z != nullptr &&
                     scatter_block_applies(ctx->G, ctx->L);
    float best_t = 0.f;
    int best_mode = -1;
    for (int mode = 2; mode >= 0 && !rc; --mode) {
      if ((mode == 2 && !blk) || (mode == 1 && !ctx->tc_sc)) continue;
      float t = 0.f;
      if ((rc = timeScat(mode, t))) break;
      if (best_mode < 0 || t < best_t) {
        best_t = t;
        best_mode = mode;
      }
    }
    if (!rc && best_mode >= 0) {
      ctx->use_blk_sc = best_mode == 2;
      ctx->use_tc_sc = best_mode == 1;
    }
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
  else if (!std::strcmp(key, "scattering_tensor_active"))  // the zone-blocked kernel, when active, takes precedence
    *value = (ctx->tc_sc && ctx->use_tc_sc && !blockScatterActive(ctx)) ? 1 : 0;
  else if (!std::strcmp(key, "graph_active")) *value = ctx->graph_active ? 1 : 0;
  else if (!std::strcmp(key, "block_jacobi")) *value = ctx->block_jacobi ? 1 : 0;
  else if (!std::strcmp(key, "fused_sweep")) *value = ctx->fuse_sweep ? 1 : 0;
  else if (!std::strcmp(key, "sweep_stream")) *value = ctx->allow_stream ? 1 : 0;
  else if (!std::strcmp(key, "ltimes_stream")) *value = ctx->allow_lt_stream ? 1 : 0;
  else if (!std::strcmp(key, "ltimes_stream_stages")) *value = ctx->lt_stream_ns;
  else if (!std::strcmp(key, "ltimes_symmetric")) *value = ctx->allow_lt_sym ? 1 : 0;
  else if (!std::strcmp(key, "ltimes_symmetric_active")) *value = ltSymActive(ctx) ? 1 : 0;
  else if (!std::strcmp(key, "sweep_stream_stages")) *value = ctx->stream_ns;
  else if (!std::strcmp(key, "sweep_stream_active")) *value = streamUsable(ctx) ? 1 : 0;
  else if (!std::strcmp(key, "sweep_streams")) *value = ctx->sweep_streams;
  else if (!std::strcmp(key, "scattering_block")) *value = ctx->allow_blk_sc ? 1 : 0;
  else if (!std::strcmp(key, "scattering_block_active")) *value = blockScatterActive(ctx) ? 1 : 0;
  else if (!std::strcmp(key, "fused_sweep_active")) *value = ctx->fuse_active ? 1 : 0;
  else if (!std::strcmp(key, "fused_ltimes")) *value = ctx->fuse_lt ? 1 : 0;
  else if (!std::strcmp(key, "fused_ltimes_active")) *value = fusedLtUsable(ctx) ? 1 : 0;
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
