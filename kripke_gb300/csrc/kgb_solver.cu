// kgb_solver.cu -- kernel drivers and the source-iteration loop of the C ABI:
// LTimes, LPlusTimes, scattering, source, population and the sweep solver as
// SteadyStateSolver and SweepSolver call them, whole solves captured as CUDA
// graphs, and the views the batched driver takes of a context.
#include "kgb_ctx.h"

namespace kgb {
namespace api {

// ---------------------------------------------------------------------------
// Kernel drivers
// ---------------------------------------------------------------------------
// Runs of lanes of one group in the sweep's chain order (chains run over a
// direction set's directions fastest), for the sweep's row-exponent reduction:
// the largest power of two dividing the set size, at most 32 -- a group's chains
// start at multiples of the set size, so aligned runs of that length never mix
// two groups (24 directions: runs of 8, three atomics per group and cell); 0
// below runs of 4, where the atomics would cost the sweep more than the pass
// they save.
int psiExpWidth(const kgb_ctx *ctx) {
  const int ds = ctx->Ds;
  if (ds <= 0) return 0;
  const int w = std::min(ds & -ds, 32);
  return w >= 4 ? w : 0;
}

// The solver's sweep records psi's row exponents for the next tensor-core
// LTimes (FP64), which then skips its own pass over each row.  With more
// directions than one K chunk, every chunk scales by the whole row's exponent
// (as one launch over the whole row would; a pass would take each chunk's own).
bool psiExpUsable(const kgb_ctx *ctx) {
  return ctx->prec == KGB_FP64 && ctx->allow_row_exp && ctx->psi_exp && ctx->tc_lt && ctx->use_tc_lt &&
         psiExpWidth(ctx) > 0;
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
bool blockScatterActive(const kgb_ctx *ctx);

bool phiExpUsable(const kgb_ctx *ctx) {
  if (!ctx->allow_row_exp || !ctx->phi_exp || !ctx->tc_sc || !ctx->use_tc_sc || phiExpWidth(ctx) == 0) return false;
  if (blockScatterActive(ctx)) return false;
  const bool tensor = ctx->tc_lt && ctx->use_tc_lt;
  if (ctx->prec == KGB_FP64) return tensor && ctx->D <= ctx->tc_lt_kpad;
  return !tensor && !tf32LtActive(ctx) && ltimes_tiled_applies(ctx->D, ctx->M);
}

// rowexp: record psi's row exponents there (the caller zeroed it); null: psi
// changes without them, so the recorded ones no longer hold.
template <typename T>
int sweepWave(kgb_ctx *ctx, const int *wave_dev, int nwave, bool fused_pop, bool fused_rhs, int *rowexp,
              bool fused_lt) {
  SweepArgs<T> a{};
  if (fused_lt && fused_pop && !fused_rhs) {  // the epilogue's kernels carry the fused population
    a.phiacc = as<T>(ctx->phi);
    a.ell = as<T>(ctx->ell);
    a.M = ctx->M;
  }
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
  // the streamed FP32 kernel where it applies
  const bool stream = sizeof(T) == 4 && !fused_rhs && !fused_lt && streamUsable(ctx);
  if (stream) {
    a.stream_ns = ctx->stream_ns;
    a.err = ctx->err_d;
    a.nsdom = ctx->dc.num();  // the plane arrays' extent
  }
  {
    const int64_t nchain = (int64_t)ctx->Gs * ctx->Ds;
    const int64_t ncb = stream ? nchain / stream_block_chains(ctx->Ds, ctx->Gs) : (nchain + kSweepThreads - 1) / kSweepThreads;
    ctx->npop_used = (int64_t)ctx->tile_off.back() * ctx->dc.num() * ncb;
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
      if constexpr (sizeof(T) == 4) {
        if (stream) {
          if (!launch_sweep_step_stream(part[i], nt, pn[i], streamOf(i)))
            return fail(ctx, KGB_ERR_CUDA, "cuTensorMapEncodeTiled failed for the streamed sweep");
          CKN(1);
          continue;
        }
      }
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

int sweepWaveAny(kgb_ctx *ctx, const int *wave_dev, int nwave, bool fused_pop, bool fused_rhs,
                 int *rowexp, bool fused_lt) {
  return ctx->prec == KGB_FP64 ? sweepWave<double>(ctx, wave_dev, nwave, fused_pop, fused_rhs, rowexp, false)
                               : sweepWave<float>(ctx, wave_dev, nwave, fused_pop, fused_rhs, nullptr, fused_lt);
}

// The streamed FP32 sweep (sweep_stream.cu): allowed, the divide form, and a
// chain layout whose operand boxes it can copy.
bool streamUsable(const kgb_ctx *ctx) {
  return ctx->prec == KGB_MIXED && ctx->allow_stream && !ctx->use_recip &&
         sweep_stream_applies(ctx->D, ctx->G, ctx->Ds, ctx->Gs, ctx->tx, ctx->ty);
}

// The fused LTimes epilogue: the mixed forward sweep with its population fused, no
// LPlusTimes prologue, and a chain count that fills whole blocks.
bool fusedLtUsable(const kgb_ctx *ctx) {
  return ctx->fuse_lt && ctx->prec == KGB_MIXED && !ctx->flip && !(ctx->fuse_sweep && ctx->M <= kFuseMaxM) &&
         (ctx->Ds * ctx->Gs) % kSweepThreads == 0;
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
int sweepSolver(kgb_ctx *ctx, bool fused_pop, bool fused_rhs, int *rowexp, bool fused_lt) {
  for (int k = 0; k < 3; ++k) CK(cudaMemsetAsync(ctx->plane[k], 0, ctx->plane_chunk[k] * ctx->dc.num() * ctx->tsz, ctx->stream));
  if (fused_lt) CK(cudaMemsetAsync(ctx->phi, 0, ctx->Z * ctx->G * ctx->M * ctx->tsz, ctx->stream));  // kConst(phi, 0)
  if (rowexp) CK(cudaMemsetAsync(rowexp, 0, ctx->Z * ctx->G * sizeof(int), ctx->stream));
  // Block Jacobi (BlockJacobiComm.cpp:46-98 with SweepSolver.cpp:28-30): the
  // planes every subdomain receives are the ones saved right after the zeroing
  // above, so no subdomain waits on another and none hands its outgoing planes
  // on.  One launch sweeps all of them, each from zero inflow on every face.
  if (ctx->block_jacobi)
    return sweepWaveAny(ctx, ctx->levels_d, ctx->dc.num(), fused_pop, fused_rhs, rowexp, fused_lt);
  const int nlev = (int)ctx->level_off.size() - 1;
  const int S[3] = {ctx->dc.Sx, ctx->dc.Sy, ctx->dc.Sz};
  // the reversed (adjoint) orientation visits the zone-set levels last to first
  const int sgn = ctx->flip ? -1 : 1;
  for (int step = 0; step < nlev; ++step) {
    const int lv = ctx->flip ? nlev - 1 - step : step;
    const int b = ctx->level_off[lv], e = ctx->level_off[lv + 1];
    if (e == b) continue;
    int rc = sweepWaveAny(ctx, ctx->levels_d + b, e - b, fused_pop, fused_rhs, rowexp, fused_lt);
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
int doLTimes(kgb_ctx *ctx, bool acc, const int *rowexp, int *outexp) {
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
        const bool one = ctx->D <= kc && !acc;  // phi's record holds for a whole, fresh phi only
        if (outexp && !one) return fail(ctx, KGB_ERR_STATE, "phi exponent record needs one fresh LTimes launch");
        if (outexp) CK(cudaMemsetAsync(outexp, 0, ctx->Z * ctx->M * sizeof(int), ctx->stream));
        tcRows<double>(ctx, as<double>(ctx->psi) + k0, as<double>(ctx->phi), ctx->D, ctx->M, K, kc, ctx->M, 1, img,
                       ex, acc || c > 0, false, rowexp, outexp);
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
  if (ctx->prec == KGB_MIXED && !acc && ctx->allow_lt_stream && ltimes_stream_applies(ctx->D, ctx->M)) {
    // the TMA-fed SIMT kernel (bit for bit the register-tiled one), or its octant-pair form where
    // L allows it (half the multiply-adds; option ltimes_symmetric)
    if (launch_ltimes_stream(as<float>(ctx->psi), as<float>(ctx->phi), as<float>(ctx->ell), rows, ctx->D, ctx->M,
                             ctx->lt_stream_ns, ltSymActive(ctx) ? ctx->lt_sym : nullptr, ctx->err_d, ctx->nsm,
                             ctx->stream))
      return fail(ctx, KGB_ERR_CUDA, "streamed LTimes launch failed");
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
bool blockScatterActive(const kgb_ctx *ctx) {
  return ctx->prec == KGB_MIXED && ctx->allow_blk_sc && ctx->use_blk_sc && ctx->pure_z != nullptr &&
         scatter_block_applies(ctx->G, ctx->L);
}

int doScattering(kgb_ctx *ctx, bool acc, const int *rowexp) {
  FamScope fs(ctx, "scattering");
  if (blockScatterActive(ctx)) {  // mixed form: zone-blocked kernel, mixed zones SIMT
    launch_scatter_block(as<float>(ctx->phi), as<float>(ctx->phi_out), as<float>(ctx->sigsT), ctx->pure_z,
                         ctx->pure_off, ctx->G, ctx->L, ctx->gp_lo, ctx->gp_hi, acc, ctx->err_d, ctx->nsm, ctx->stream);
    CKN(1);
    if (ctx->nmixed_z > 0) {
      ScatterArgsBase a = scatterArgs(ctx);
      a.Z = ctx->nmixed_z;
      a.zlist = ctx->mixed_z;
      launch_scattering<float>(as<float>(ctx->phi), as<float>(ctx->phi_out), as<float>(ctx->sigsT), a, acc,
                               ctx->stream);
      CKN(1);
    }
    return KGB_OK;
  }
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
    return fail(ctx, KGB_ERR_TIMEOUT, "a device kernel's bounded wait gave up");
  }
  return KGB_OK;
}

// One source iteration.  part_slot: particle count of the new psi, fused into
// the sweep.  prev_slot: particle count of the psi the iteration starts from,
// taken from this iteration's own moments (one small pass over moment 0) --
// a solve counts every iterate that way and the last one after its loop.
int iterateDevice(kgb_ctx *ctx, double q, double *part_slot, double *prev_slot, bool lt_next) {
  int rc;
  // psi's row exponents, when the sweep that wrote psi recorded them
  const bool px = psiExpUsable(ctx);
  const int *rx = px && ctx->psi_exp_valid ? ctx->psi_exp : nullptr;
  ctx->psi_exp_valid = false;
  // phi = L psi already, added up by the previous iteration's sweep (same solve)
  const bool have_phi = ctx->phi_fused;
  ctx->phi_fused = false;
  int *const pe = !have_phi && phiExpUsable(ctx) ? ctx->phi_exp : nullptr;  // phi's, for the scattering
  if (!have_phi && (rc = doLTimes(ctx, false, rx, pe))) return rc;  // phi = L psi  (kConst + LTimes)
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
  // psi = H^-1 rhs (+ population, + row exponents, + the next iteration's phi)
  const bool lt = lt_next && part_slot != nullptr && !ctx->fuse_active;
  if ((rc = sweepSolver(ctx, part_slot != nullptr, ctx->fuse_active, px ? ctx->psi_exp : nullptr, lt))) return rc;
  ctx->psi_exp_valid = px;
  ctx->phi_fused = lt;
  if (ctx->fuse_active) ctx->rhs_stale = true;
  if (part_slot) {
    FamScope fs(ctx, "population");
    launch_sum_partials(ctx->pop_slots, ctx->npop_used, part_slot, ctx->stream);
    CKN(1);
  }
  return KGB_OK;
}


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
    // the last iteration's sweep adds no moments: phi ends as the reference leaves it, L of
    // the psi the last iteration started from
    const bool lt = fusedLtUsable(ctx);
    for (int it = 0; it < niter; ++it)
      if ((rc = iterateDevice(ctx, q, ctx->parts_dev + it, nullptr, lt && it + 1 < niter))) {
        ctx->phi_fused = false;
        return rc;
      }
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
  for (auto &e : v)
    if (e.gen == ctx->gen && e.niter == niter && e.q == q && e.stream == ctx->stream) {
      *out = &e;
      return KGB_OK;
    }
  // A solve of this shape captured before the tables changed: its executable graph is
  // updated in place from the new capture when the topology is the same (new buffers
  // or kernel arguments only), which costs far less than instantiating a new one.
  cudaGraphExec_t stale_x = nullptr;
  for (auto it = v.begin(); it != v.end();) {
    if (it->gen != ctx->gen) {
      if (!stale_x && it->niter == niter && it->q == q && it->stream == ctx->stream) {
        stale_x = it->x;
      } else {
        cudaGraphExecDestroy(it->x);
      }
      cudaGraphDestroy(it->g);
      it = v.erase(it);
    } else {
      ++it;
    }
  }
  if (v.size() >= 4) {
    cudaGraphExecDestroy(v.front().x);
    cudaGraphDestroy(v.front().g);
    v.erase(v.begin());
  }
  if (cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    cudaGetLastError();
    if (stale_x) cudaGraphExecDestroy(stale_x);
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
  if (!rc && e == cudaSuccess && g && stale_x) {
    cudaGraphExecUpdateResultInfo info;
    if (cudaGraphExecUpdate(stale_x, g, &info) == cudaSuccess) {
      x = stale_x;
    } else {
      cudaGetLastError();
      cudaGraphExecDestroy(stale_x);
    }
    stale_x = nullptr;
  }
  if (stale_x) cudaGraphExecDestroy(stale_x);
  if (rc || e != cudaSuccess || !g || (!x && cudaGraphInstantiate(&x, g, 0) != cudaSuccess)) {
    cudaGetLastError();
    if (x) cudaGraphExecDestroy(x);
    if (g) cudaGraphDestroy(g);
    ctx->err = err0;
    return KGB_OK;
  }
  v.push_back({niter, q, ctx->gen, ctx->stream, g, x, captured});
  *out = &v.back();
  return KGB_OK;
}

}  // namespace api
}  // namespace kgb

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

int instance_op(kgb_ctx *ctx, InstanceOp op, double q, cudaStream_t s, const int *psi_exp, double *pop) {
  cudaStream_t keep = ctx->stream;
  ctx->stream = s;
  // a batched iteration runs each problem's LTimes and then its scattering (same
  // stream), so LTimes can record phi's exponents for the scattering
  int *const pe = phiExpUsable(ctx) ? ctx->phi_exp : nullptr;
  int rc;
  switch (op) {
    case InstanceOp::LTimes: rc = doLTimes(ctx, false, psi_exp, pe); break;
    case InstanceOp::LPlusTimes: rc = doLPlusTimes(ctx, false); break;
    case InstanceOp::Sweep:
      rc = sweepSolver(ctx, true, false, const_cast<int *>(psi_exp), false);
      if (!rc && pop) {
        launch_sum_partials(ctx->pop_slots, ctx->npop_used, pop, s);
        if (cudaGetLastError() != cudaSuccess) rc = fail(ctx, KGB_ERR_CUDA, "population partial sum launch failed");
      }
      break;
    default:
      rc = doScattering(ctx, false, pe);
      if (!rc) rc = doSource(ctx, q);
      break;
  }
  ctx->stream = keep;
  return rc;
}
int instance_check(kgb_ctx *ctx) { return checkDeviceError(ctx); }
int instance_tiles(kgb_ctx *ctx, int tx, int ty, int tz) {
  if (ctx->tx == tx && ctx->ty == ty && ctx->tz == tz && ctx->tiles_d) return KGB_OK;
  ctx->tx = tx;
  ctx->ty = ty;
  ctx->tz = tz;
  ctx->tiles_set = true;
  return buildTiles(ctx);
}
int64_t instance_sweep_launches(const kgb_ctx *ctx) {
  const int np = std::max(1, std::min(ctx->sweep_streams, ctx->dc.num()));
  return (int64_t)ctx->nsteps * np + 1;  // the steps' parts and the population sum
}
}  // namespace kgb

extern "C" {

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


}  // extern "C"
