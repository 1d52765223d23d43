// batch.cu -- many independent Kripke problems advanced together on one GPU.
//
// Each problem is an ordinary context (its fields, generator and kernels are
// those of the single-problem path) with one zone set; the batch adds a
// driver that advances all of them with one launch per kernel family:
//   LTimes and LPlusTimes .... one launch per moment class, items = row ranges
//   scattering + source ...... one launch per Legendre order
//                              (these two in the mixed form; in FP64 each
//                              problem's own tensor-core kernels run instead,
//                              on parallel graph branches)
//   sweep .................... ONE persistent cooperative launch: every block
//                              takes (problem, subdomain, tile, chain block)
//                              items of the current global hyperplane step,
//                              a bounded grid barrier separates the steps
//   population ............... fused partials, one block per problem sums them
// and a whole solve (psi reset + niter iterations) is captured once into a
// CUDA graph and replayed.  Tile shapes (sweep tile footprint and depth, rows
// per moment work item) come from kgb_batch_autotune, which times the
// candidates on the batch itself.  Every problem's arithmetic is the
// single-problem path's, term for term, so a problem's psi and particle
// counts equal those of its own context run with the same sweep tile shape
// (and, when the batch uses its batched SIMT kernels, the context's SIMT ones).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <string>
#include <utility>
#include <vector>

#include "kgb_internal.h"

using namespace kgb;

struct kgb_batch {
  int device = 0;
  int prec = KGB_FP64;
  cudaStream_t stream = nullptr;
  std::string err;
  std::vector<kgb_ctx *> inst;

  // tuning (kgb_batch_set_option / kgb_batch_autotune)
  int tx = 2, ty = 2, tz = 8;
  int rows_per_item = 1024;
  // a grid-barrier wait of the persistent sweep gives up after this long (then KGB_ERR_TIMEOUT)
  int64_t barrier_wait_ns = 2000000000;
  bool use_graph = true;
  int own_mode = -1;  // 1: each problem's own LTimes/scattering/LPlusTimes kernels; 0: batched SIMT; -1: by precision
  // 1: each problem's own sweeps (per-step launches, the streamed FP32 sweep where it
  // applies) on parallel branches; 0: the persistent launch over all problems; -1: by precision
  int sweep_mode = -1;
  // the problems' psi row-exponent records (FP64, views[i].psi_exp) hold for their current psi:
  // set by a solve's reset and by every batched sweep, which records them; cleared by a new plan
  bool rec_ok = false;

  // streams the per-problem kernels fork onto (graph branches when captured); a phase
  // uses the first `branches` of them
  static constexpr int kForks = 8;
  int branches = 8;
  cudaStream_t aux[kForks] = {};
  cudaEvent_t fork_ev = nullptr, join_ev[kForks] = {};

  // plan
  bool planned = false;
  double q = 1.0;
  int nsm = 0, sweep_grid = 0, row_grid = 0, Dmax = 0, nsteps = 0;
  std::vector<InstanceView> views;
  std::vector<void *> owned;  // device allocations of the plan
  void *sweep_args = nullptr;
  int4 *sweep_items = nullptr;
  int *step_off = nullptr;
  BatchZero *zero = nullptr;
  int nzero = 0;
  unsigned int *bar = nullptr;
  int *err_d = nullptr;
  void *lt_desc = nullptr, *lp_desc = nullptr, *sc_desc = nullptr;
  BatchRows *rows_lt = nullptr, *rows_lp = nullptr, *rows_sc = nullptr;
  struct Class {
    int key;   // moment class (moments) or Legendre order (scattering)
    bool vec;  // 16-byte row loads (moments)
    int off, n;
  };
  std::vector<Class> lt_cls, lp_cls, sc_cls;
  const double **slot_ptrs = nullptr;
  int64_t *slot_n = nullptr;
  double *pop = nullptr;
  int pop_cap = 0;
  int64_t kernels_per_iter = 0;

  // captured solves, by iteration count
  std::map<int, std::pair<cudaGraph_t, cudaGraphExec_t>> graphs;
  bool graph_active = false;
  std::string graph_note;
  int64_t launches = 0;
};

namespace {

int fail(kgb_batch *b, int code, const std::string &msg) {
  if (b) b->err = msg;
  return code;
}

#define BCK(call)                                                                                   \
  do {                                                                                              \
    cudaError_t e_ = (call);                                                                        \
    if (e_ != cudaSuccess) return fail(b, KGB_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

void dropGraphs(kgb_batch *b) {
  for (auto &kv : b->graphs) {
    cudaGraphExecDestroy(kv.second.second);
    cudaGraphDestroy(kv.second.first);
  }
  b->graphs.clear();
  b->graph_active = false;
}

void freePlan(kgb_batch *b) {
  dropGraphs(b);
  for (void *p : b->owned) cudaFree(p);
  b->owned.clear();
  b->sweep_args = nullptr;
  b->sweep_items = nullptr;
  b->step_off = nullptr;
  b->zero = nullptr;
  b->bar = nullptr;
  b->err_d = nullptr;
  b->lt_desc = b->lp_desc = b->sc_desc = nullptr;
  b->rows_lt = b->rows_lp = b->rows_sc = nullptr;
  b->slot_ptrs = nullptr;
  b->slot_n = nullptr;
  b->pop = nullptr;
  b->pop_cap = 0;
  b->lt_cls.clear();
  b->lp_cls.clear();
  b->sc_cls.clear();
  b->planned = false;
}

template <typename P>
int devAlloc(kgb_batch *b, P **p, size_t n) {
  void *q = nullptr;
  if (cudaMalloc(&q, std::max<size_t>(n, 1) * sizeof(P)) != cudaSuccess) {
    cudaGetLastError();
    return fail(b, KGB_ERR_OOM, "batch plan allocation failed");
  }
  b->owned.push_back(q);
  *p = reinterpret_cast<P *>(q);
  return KGB_OK;
}

template <typename P>
int devUpload(kgb_batch *b, P **p, const std::vector<P> &v) {
  int rc = devAlloc(b, p, v.size());
  if (rc) return rc;
  if (!v.empty()) BCK(cudaMemcpyAsync(*p, v.data(), v.size() * sizeof(P), cudaMemcpyHostToDevice, b->stream));
  return KGB_OK;
}

bool sameViews(const InstanceView &a, const InstanceView &c) {
  return a.psi == c.psi && a.rhs == c.rhs && a.phi == c.phi && a.phi_out == c.phi_out && a.sigt == c.sigt &&
         a.plane[0] == c.plane[0] && a.plane[1] == c.plane[1] && a.plane[2] == c.plane[2] && a.ell == c.ell &&
         a.ellp == c.ellp && a.sigsT == c.sigsT && a.mix_frac == c.mix_frac && a.mix_mat == c.mix_mat &&
         a.zmix_start == c.zmix_start && a.gp_lo == c.gp_lo && a.sdoms == c.sdoms && a.cx == c.cx &&
         a.cls == c.cls && a.inv == c.inv && a.gen == c.gen;
}

// Row items of every problem, grouped by a class key (stable: problem order within a class).
template <typename KeyFn>
void groupRows(const std::vector<BatchRows> &rows, KeyFn key, std::vector<BatchRows> &out,
               std::vector<kgb_batch::Class> &cls) {
  std::map<std::pair<int, bool>, std::vector<BatchRows>> by;
  for (const BatchRows &r : rows) by[key(r.inst)].push_back(r);
  out.clear();
  cls.clear();
  for (auto &kv : by) {
    cls.push_back({kv.first.first, kv.first.second, (int)out.size(), (int)kv.second.size()});
    out.insert(out.end(), kv.second.begin(), kv.second.end());
  }
}

bool perProblem(const kgb_batch *b) { return b->own_mode < 0 ? b->prec == KGB_FP64 : b->own_mode == 1; }
bool ownSweeps(const kgb_batch *b) { return b->sweep_mode < 0 ? b->prec != KGB_FP64 : b->sweep_mode == 1; }

template <typename T>
int planT(kgb_batch *b) {
  freePlan(b);
  const int n = (int)b->inst.size();
  if (n == 0) return fail(b, KGB_ERR_STATE, "the batch has no problems");
  b->views.assign(n, InstanceView{});
  if (ownSweeps(b))  // the problems sweep with the batch's tiles (before their views: new tiles, new generation)
    for (int i = 0; i < n; ++i) {
      const int rc = instance_tiles(b->inst[i], b->tx, b->ty, b->tz);
      if (rc) return fail(b, rc, "problem " + std::to_string(i) + ": " + kgb_last_error(b->inst[i]));
    }
  for (int i = 0; i < n; ++i) {
    int rc = instance_view(b->inst[i], &b->views[i]);
    if (rc) return fail(b, rc, "problem " + std::to_string(i) + ": " + kgb_last_error(b->inst[i]));
  }
  std::vector<SweepArgs<T>> sa(n);
  std::vector<std::vector<int>> toff(n);
  std::vector<const double *> slot_ptrs(n);
  std::vector<int64_t> slot_n(n);
  int maxsteps = 0;
  b->Dmax = 0;
  int rc;
  for (int i = 0; i < n; ++i) {
    const InstanceView &v = b->views[i];
    b->Dmax = std::max(b->Dmax, v.D);
    // tiles in hyperplane order, as the single-problem sweep lists them
    const int ntx = (v.nx + b->tx - 1) / b->tx, nty = (v.ny + b->ty - 1) / b->ty, ntz = (v.nz + b->tz - 1) / b->tz;
    const int nst = ntx + nty + ntz - 2;
    std::vector<int4> tiles;
    toff[i].assign(1, 0);
    for (int s = 0; s < nst; ++s) {
      for (int c = 0; c < ntz; ++c)
        for (int y = 0; y < nty; ++y) {
          const int x = s - y - c;
          if (x >= 0 && x < ntx) tiles.push_back(make_int4(x, y, c, 0));
        }
      toff[i].push_back((int)tiles.size());
    }
    maxsteps = std::max(maxsteps, nst);
    int4 *tiles_d = nullptr;
    if ((rc = devUpload(b, &tiles_d, tiles))) return rc;
    const int ncb = (v.Gs * v.Ds + kSweepThreads - 1) / kSweepThreads;
    const int64_t nslots = (int64_t)tiles.size() * v.nsdom * ncb;
    double *slots = nullptr;
    if ((rc = devAlloc(b, &slots, nslots))) return rc;
    slot_ptrs[i] = slots;
    slot_n[i] = nslots;
    SweepArgs<T> a{};
    a.rhs = (const T *)v.rhs;
    a.psi = (T *)v.psi;
    a.sigt = (const T *)v.sigt;
    a.iplane = (T *)v.plane[0];
    a.jplane = (T *)v.plane[1];
    a.kplane = (T *)v.plane[2];
    a.cx = (const T *)v.cx;
    a.cy = (const T *)v.cy;
    a.cz = (const T *)v.cz;
    a.sdoms = v.sdoms;
    a.cls = v.cls;
    a.inv = (const T *)v.inv;
    a.tiles = tiles_d;
    a.nx = v.nx; a.ny = v.ny; a.nz = v.nz; a.G = v.G; a.D = v.D; a.Gs = v.Gs; a.Ds = v.Ds;
    a.nxs = v.nx; a.nys = v.ny; a.nzs = v.nz;
    a.tz = b->tz; a.tx = b->tx; a.ty = b->ty;
    a.pop = slots;
    a.nsdom = v.nsdom;
    a.w = v.w;
    a.vol = v.vol;
    a.vol_uniform = v.vol_uniform;
    if (sizeof(T) == 8 && v.psi_exp) {  // record psi's row exponents for the problem's next LTimes
      a.rowexp = v.psi_exp;
      a.rexp_w = v.psi_exp_w;
    }
    sa[i] = a;
  }
  // sweep work items by global step, then the plane zeroing ranges
  std::vector<int4> items;
  std::vector<int> soff;
  for (int s = 0; s < maxsteps; ++s) {
    soff.push_back((int)items.size());
    for (int i = 0; i < n; ++i) {
      if (s + 1 >= (int)toff[i].size()) continue;
      const InstanceView &v = b->views[i];
      const int ncb = (v.Gs * v.Ds + kSweepThreads - 1) / kSweepThreads;
      for (int t = toff[i][s]; t < toff[i][s + 1]; ++t)
        for (int sd = 0; sd < v.nsdom; ++sd)
          for (int cb = 0; cb < ncb; ++cb) items.push_back(make_int4(i, sd, t, cb));
    }
  }
  soff.push_back((int)items.size());
  if (items.size() > (size_t)0x7fffffff) return fail(b, KGB_ERR_ARG, "too many sweep work items");
  std::vector<BatchZero> zero;
  for (int i = 0; i < n; ++i)
    for (int k = 0; k < 3; ++k) {
      const int64_t total = b->views[i].plane_chunk[k] * b->views[i].nsdom;
      for (int64_t e = 0; e < total; e += (int64_t)1 << 16) zero.push_back({i, k, e, std::min(total, e + ((int64_t)1 << 16))});
    }
  for (int i = 0; i < n; ++i)
    if (sa[i].rowexp) {  // zeroed with the planes: the sweep takes atomic maxima
      const int64_t total = b->views[i].Z * b->views[i].G;
      for (int64_t e = 0; e < total; e += (int64_t)1 << 16) zero.push_back({i, 3, e, std::min(total, e + ((int64_t)1 << 16))});
    }
  b->rec_ok = false;
  b->nsteps = maxsteps;
  b->nzero = (int)zero.size();
  SweepArgs<T> *sa_d = nullptr;
  if ((rc = devUpload(b, &sa_d, sa)) || (rc = devUpload(b, &b->sweep_items, items)) ||
      (rc = devUpload(b, &b->step_off, soff)) || (rc = devUpload(b, &b->zero, zero)) ||
      (rc = devAlloc(b, &b->bar, 2)) || (rc = devAlloc(b, &b->err_d, 1)))
    return rc;
  b->sweep_args = sa_d;
  BCK(cudaMemsetAsync(b->err_d, 0, sizeof(int), b->stream));
  // row work items and their classes
  std::vector<BatchRows> rows;
  for (int i = 0; i < n; ++i) {
    const int64_t R = b->views[i].Z * b->views[i].G;
    for (int64_t r0 = 0; r0 < R; r0 += b->rows_per_item) rows.push_back({i, 0, r0, std::min(R, r0 + b->rows_per_item)});
  }
  std::vector<BatchRows> rl, rp, rs;
  const bool f32 = sizeof(T) == 4;
  groupRows(rows, [&](int i) { return std::make_pair(moment_class(b->views[i].M), (b->views[i].D * (int)sizeof(T)) % 16 == 0); },
            rl, b->lt_cls);
  groupRows(rows, [&](int i) { return std::make_pair(moment_class(b->views[i].M), f32 && (b->views[i].D * 4) % 16 == 0); },
            rp, b->lp_cls);
  groupRows(rows, [&](int i) { return std::make_pair(b->views[i].L, false); }, rs, b->sc_cls);
  std::vector<BatchMom<T>> lt(n), lp(n);
  std::vector<BatchScat<T>> sc(n);
  for (int i = 0; i < n; ++i) {
    const InstanceView &v = b->views[i];
    lt[i] = {(const T *)v.psi, (T *)v.phi, (const T *)v.ell, v.D, v.M};
    lp[i] = {(const T *)v.phi_out, (T *)v.rhs, (const T *)v.ellp, v.D, v.M};
    ScatterArgsBase a{};
    a.Z = v.Z; a.G = v.G; a.M = v.M; a.L = v.L;
    a.zmix_start = v.zmix_start; a.zmix_count = v.zmix_count; a.mix_mat = v.mix_mat; a.mix_frac = v.mix_frac;
    a.gp_lo = v.gp_lo; a.gp_hi = v.gp_hi;
    a.src_glo = 0; a.src_ghi = v.G; a.dst_glo = 0; a.dst_ghi = v.G;
    sc[i] = {(const T *)v.phi, (T *)v.phi_out, (const T *)v.sigsT, a, b->q};
  }
  BatchMom<T> *lt_d = nullptr, *lp_d = nullptr;
  BatchScat<T> *sc_d = nullptr;
  if ((rc = devUpload(b, &lt_d, lt)) || (rc = devUpload(b, &lp_d, lp)) || (rc = devUpload(b, &sc_d, sc)) ||
      (rc = devUpload(b, &b->rows_lt, rl)) || (rc = devUpload(b, &b->rows_lp, rp)) ||
      (rc = devUpload(b, &b->rows_sc, rs)) || (rc = devUpload(b, &b->slot_ptrs, slot_ptrs)) ||
      (rc = devUpload(b, &b->slot_n, slot_n)))
    return rc;
  b->lt_desc = lt_d;
  b->lp_desc = lp_d;
  b->sc_desc = sc_d;
  b->sweep_grid = batch_sweep_grid<T>(b->tx, b->ty, b->nsm);
  if (b->sweep_grid <= 0) return fail(b, KGB_ERR_CUDA, "the persistent sweep has no resident blocks");
  b->row_grid = b->nsm * 16;
  b->kernels_per_iter = perProblem(b) ? 3 * (int64_t)n : (int64_t)b->lt_cls.size() + b->lp_cls.size() + b->sc_cls.size();
  if (ownSweeps(b)) {
    for (int i = 0; i < n; ++i) b->kernels_per_iter += instance_sweep_launches(b->inst[i]);
  } else {
    b->kernels_per_iter += 2;  // the persistent sweep and the population sums
  }
  BCK(cudaStreamSynchronize(b->stream));
  b->planned = true;
  return KGB_OK;
}

int plan(kgb_batch *b) { return b->prec == KGB_FP64 ? planT<double>(b) : planT<float>(b); }

// Plans on first use and again when a problem's device arrays moved.
int ensurePlan(kgb_batch *b) {
  if (b->planned) {
    for (size_t i = 0; i < b->inst.size(); ++i) {
      InstanceView v{};
      int rc = instance_view(b->inst[i], &v);
      if (rc) return fail(b, rc, "problem " + std::to_string(i) + ": " + kgb_last_error(b->inst[i]));
      if (!sameViews(v, b->views[i])) {
        b->planned = false;
        break;
      }
    }
  }
  return b->planned ? KGB_OK : plan(b);
}

// Each problem's own kernels for one phase (the tensor-core digit products in
// FP64), spread over the batch's branches (streams forked from and joined back to the batch
// stream -- parallel branches of the captured graph.
// pop: the batch's population slots of this iteration (Sweep: each problem's count
// of the new psi goes to pop[i]; FP64 problems record psi's row exponents).
int forkPhase(kgb_batch *b, InstanceOp op, double *pop = nullptr) {
  BCK(cudaEventRecord(b->fork_ev, b->stream));
  const int nb = b->branches;
  for (int k = 0; k < nb; ++k) BCK(cudaStreamWaitEvent(b->aux[k], b->fork_ev, 0));
  for (size_t i = 0; i < b->inst.size(); ++i) {
    const bool sweep = op == InstanceOp::Sweep;
    const int *rx = (op == InstanceOp::LTimes && b->rec_ok) || sweep ? b->views[i].psi_exp : nullptr;
    const int rc = instance_op(b->inst[i], op, b->q, b->aux[i % nb], rx, sweep ? pop + i : nullptr);
    if (rc) return fail(b, rc, "problem " + std::to_string(i) + ": " + kgb_last_error(b->inst[i]));
  }
  for (int k = 0; k < nb; ++k) {
    BCK(cudaEventRecord(b->join_ev[k], b->aux[k]));
    BCK(cudaStreamWaitEvent(b->stream, b->join_ev[k], 0));
  }
  return KGB_OK;
}

// ev (optional, 6 events): recorded at the phase boundaries LTimes | scattering
// | LPlusTimes | sweep | population.
template <typename T>
int enqueueIteration(kgb_batch *b, double *pop_out, cudaEvent_t *ev = nullptr) {
  const auto *lt = (const BatchMom<T> *)b->lt_desc;
  const auto *lp = (const BatchMom<T> *)b->lp_desc;
  const auto *sc = (const BatchScat<T> *)b->sc_desc;
  const bool own = perProblem(b);
  int rc;
  if (ev) BCK(cudaEventRecord(ev[0], b->stream));
  if (own) {
    if ((rc = forkPhase(b, InstanceOp::LTimes))) return rc;
  } else {
    for (auto &c : b->lt_cls)
      launch_batch_moments<T>(lt, b->rows_lt + c.off, c.n, c.key, b->Dmax, false, c.vec,
                              std::min(c.n, b->row_grid), b->stream);
  }
  if (ev) BCK(cudaEventRecord(ev[1], b->stream));
  if (own) {
    if ((rc = forkPhase(b, InstanceOp::Scatter))) return rc;
  } else {
    for (auto &c : b->sc_cls)
      launch_batch_scattering<T>(sc, b->rows_sc + c.off, c.n, c.key, std::min(c.n, b->row_grid), b->stream);
  }
  if (ev) BCK(cudaEventRecord(ev[2], b->stream));
  if (own) {
    if ((rc = forkPhase(b, InstanceOp::LPlusTimes))) return rc;
  } else {
    for (auto &c : b->lp_cls)
      launch_batch_moments<T>(lp, b->rows_lp + c.off, c.n, c.key, b->Dmax, true, c.vec,
                              std::min(c.n, b->row_grid), b->stream);
  }
  BCK(cudaGetLastError());
  if (ev) BCK(cudaEventRecord(ev[3], b->stream));
  if (ownSweeps(b)) {
    // each problem's own sweep and population sum on parallel branches
    if ((rc = forkPhase(b, InstanceOp::Sweep, pop_out))) return rc;
    b->rec_ok = true;
    if (ev) BCK(cudaEventRecord(ev[4], b->stream));
  } else {
    BCK(cudaMemsetAsync(b->bar, 0, 2 * sizeof(unsigned int), b->stream));
    BatchSweepPlan p{b->sweep_items, b->step_off, b->nsteps, b->zero,
                     b->nzero,          b->bar,      b->err_d, (unsigned long long)b->barrier_wait_ns};
    BCK(launch_batch_sweep<T>((const SweepArgs<T> *)b->sweep_args, p, b->tx, b->ty, b->sweep_grid, b->stream));
    b->rec_ok = true;  // the sweep recorded psi's row exponents (FP64 problems with a record)
    if (ev) BCK(cudaEventRecord(ev[4], b->stream));
    launch_batch_pop_finish(b->slot_ptrs, b->slot_n, (int)b->inst.size(), pop_out, b->stream);
  }
  if (ev) BCK(cudaEventRecord(ev[5], b->stream));
  BCK(cudaGetLastError());
  return KGB_OK;
}

int enqueueSolve(kgb_batch *b, int niter) {
  for (auto &v : b->views) {
    BCK(cudaMemsetAsync(v.psi, 0, (size_t)v.Z * v.G * v.D * (b->prec == KGB_FP64 ? 8 : 4), b->stream));
    if (v.psi_exp) BCK(cudaMemsetAsync(v.psi_exp, 0, (size_t)v.Z * v.G * sizeof(int), b->stream));  // psi = 0
  }
  b->rec_ok = true;
  const int n = (int)b->inst.size();
  for (int it = 0; it < niter; ++it) {
    int rc = b->prec == KGB_FP64 ? enqueueIteration<double>(b, b->pop + (size_t)it * n)
                                 : enqueueIteration<float>(b, b->pop + (size_t)it * n);
    if (rc) return rc;
  }
  return KGB_OK;
}

int ensurePop(kgb_batch *b, int niter) {
  const int need = niter * (int)b->inst.size();
  if (need <= b->pop_cap) return KGB_OK;
  dropGraphs(b);  // captured solves write the old array
  double *p = nullptr;
  int rc = devAlloc(b, &p, need);
  if (rc) return rc;
  b->pop = p;
  b->pop_cap = need;
  return KGB_OK;
}

// Captures a whole solve of niter iterations; on any capture failure the
// solve runs launch by launch and the reason is kept (option "graph_active" 0).
int graphFor(kgb_batch *b, int niter, cudaGraphExec_t *exec) {
  *exec = nullptr;
  auto it = b->graphs.find(niter);
  if (it != b->graphs.end()) {
    *exec = it->second.second;
    return KGB_OK;
  }
  cudaGraph_t g = nullptr;
  if (cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    cudaGetLastError();
    b->graph_note = "stream capture could not start";
    return KGB_OK;
  }
  const int rc = enqueueSolve(b, niter);
  const cudaError_t e = cudaStreamEndCapture(b->stream, &g);
  if (rc || e != cudaSuccess || !g) {
    cudaGetLastError();
    if (g) cudaGraphDestroy(g);
    b->graph_note = std::string("capture failed: ") + (rc ? b->err : cudaGetErrorString(e));
    return KGB_OK;
  }
  cudaGraphExec_t x = nullptr;
  if (cudaGraphInstantiate(&x, g, 0) != cudaSuccess) {
    cudaGetLastError();
    cudaGraphDestroy(g);
    b->graph_note = "graph instantiation failed";
    return KGB_OK;
  }
  b->graphs[niter] = {g, x};
  *exec = x;
  return KGB_OK;
}

int checkBarrier(kgb_batch *b) {
  int h = 0;
  BCK(cudaMemcpyAsync(&h, b->err_d, sizeof(int), cudaMemcpyDeviceToHost, b->stream));
  BCK(cudaStreamSynchronize(b->stream));
  if (h) {
    BCK(cudaMemsetAsync(b->err_d, 0, sizeof(int), b->stream));
    return fail(b, KGB_ERR_TIMEOUT, "a grid barrier of the persistent sweep gave up waiting");
  }
  // the problems' own kernels report their bounded waits through their contexts
  if (perProblem(b) || ownSweeps(b))
    for (size_t i = 0; i < b->inst.size(); ++i)
      if (instance_check(b->inst[i]) != KGB_OK)
        return fail(b, KGB_ERR_TIMEOUT,
                    "problem " + std::to_string(i) + ": a kernel's bounded wait gave up");
  return KGB_OK;
}

int timeIteration(kgb_batch *b, float *ms) {
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  int rc = KGB_OK;
  for (int rep = 0; rep < 2 && !rc; ++rep) {
    cudaEventRecord(e0, b->stream);
    rc = b->prec == KGB_FP64 ? enqueueIteration<double>(b, b->pop) : enqueueIteration<float>(b, b->pop);
    cudaEventRecord(e1, b->stream);
  }
  if (!rc && cudaEventSynchronize(e1) == cudaSuccess) cudaEventElapsedTime(ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (!rc) rc = checkBarrier(b);
  return rc;
}

}  // namespace

extern "C" {

int kgb_batch_create(int device, int32_t precision, kgb_batch **out) {
  if (!out) return KGB_ERR_ARG;
  *out = nullptr;
  if (precision != KGB_FP64 && precision != KGB_MIXED) return KGB_ERR_ARG;
  if (cudaSetDevice(device) != cudaSuccess) {
    cudaGetLastError();
    return KGB_ERR_CUDA;
  }
  auto *b = new kgb_batch();
  b->device = device;
  b->prec = precision;
  if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    delete b;
    return KGB_ERR_CUDA;
  }
  bool ok = cudaEventCreateWithFlags(&b->fork_ev, cudaEventDisableTiming) == cudaSuccess;
  for (int k = 0; k < kgb_batch::kForks && ok; ++k)
    ok = cudaStreamCreateWithFlags(&b->aux[k], cudaStreamNonBlocking) == cudaSuccess &&
         cudaEventCreateWithFlags(&b->join_ev[k], cudaEventDisableTiming) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    kgb_batch_destroy(b);
    return KGB_ERR_CUDA;
  }
  int nsm = 0;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device);
  b->nsm = nsm > 0 ? nsm : 152;
  *out = b;
  return KGB_OK;
}

int kgb_batch_destroy(kgb_batch *b) {
  if (!b) return KGB_ERR_ARG;
  cudaSetDevice(b->device);
  cudaStreamSynchronize(b->stream);
  freePlan(b);
  for (kgb_ctx *c : b->inst) kgb_ctx_destroy(c);
  for (int k = 0; k < kgb_batch::kForks; ++k) {
    if (b->aux[k]) cudaStreamDestroy(b->aux[k]);
    if (b->join_ev[k]) cudaEventDestroy(b->join_ev[k]);
  }
  if (b->fork_ev) cudaEventDestroy(b->fork_ev);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return KGB_OK;
}

const char *kgb_batch_last_error(const kgb_batch *b) { return b ? b->err.c_str() : "null batch"; }

int kgb_batch_add(kgb_batch *b, const kgb_input *in, int32_t *index) {
  if (!b || !in) return KGB_ERR_ARG;
  if (in->num_zonesets[0] != 1 || in->num_zonesets[1] != 1 || in->num_zonesets[2] != 1)
    return fail(b, KGB_ERR_ARG, "batched problems use one zone set");
  if (in->legendre_order > 4) return fail(b, KGB_ERR_ARG, "batched problems need Legendre order <= 4");
  BCK(cudaSetDevice(b->device));
  kgb_ctx *c = nullptr;
  int rc = kgb_ctx_create(b->device, &c);
  if (rc) return fail(b, rc, "context creation failed");
  kgb_input x = *in;
  x.precision = b->prec;
  if ((rc = kgb_generate(c, &x))) {
    b->err = std::string("generation failed: ") + kgb_last_error(c);
    kgb_ctx_destroy(c);
    return rc;
  }
  b->inst.push_back(c);
  b->planned = false;
  dropGraphs(b);
  if (index) *index = (int32_t)b->inst.size() - 1;
  return KGB_OK;
}

int kgb_batch_size(const kgb_batch *b, int32_t *n) {
  if (!b || !n) return KGB_ERR_ARG;
  *n = (int32_t)b->inst.size();
  return KGB_OK;
}

int kgb_batch_context(kgb_batch *b, int32_t index, kgb_ctx **ctx) {
  if (!b || !ctx) return KGB_ERR_ARG;
  if (index < 0 || index >= (int32_t)b->inst.size()) return fail(b, KGB_ERR_ARG, "problem index out of range");
  *ctx = b->inst[index];
  return KGB_OK;
}

int kgb_batch_set_option(kgb_batch *b, const char *key, int64_t value) {
  if (!b || !key) return KGB_ERR_ARG;
  const std::string k(key);
  if (k == "sweep_tile_xy") {
    if (value != 44 && value != 42 && value != 22) return fail(b, KGB_ERR_ARG, "sweep_tile_xy must be 44, 42 or 22");
    b->tx = (int)(value / 10);
    b->ty = (int)(value % 10);
  } else if (k == "sweep_tile_z") {
    if (value < 1 || value > 64) return fail(b, KGB_ERR_ARG, "sweep_tile_z must be in [1, 64]");
    b->tz = (int)value;
  } else if (k == "rows_per_item") {
    if (value < 32 || value > (1 << 20)) return fail(b, KGB_ERR_ARG, "rows_per_item must be in [32, 2^20]");
    b->rows_per_item = (int)value;
  } else if (k == "barrier_wait_ns") {
    if (value < 0 || value > 60000000000ll) return fail(b, KGB_ERR_ARG, "barrier_wait_ns must be in [0, 6e10]");
    b->barrier_wait_ns = value;
  } else if (k == "graph") {
    b->use_graph = value != 0;
  } else if (k == "per_problem_kernels") {
    b->own_mode = value < 0 ? -1 : (value != 0 ? 1 : 0);
  } else if (k == "per_problem_sweeps") {
    b->sweep_mode = value < 0 ? -1 : (value != 0 ? 1 : 0);
  } else if (k == "branches") {
    if (value < 1 || value > kgb_batch::kForks) return fail(b, KGB_ERR_ARG, "branches must be in [1, 8]");
    b->branches = (int)value;
  } else {
    return fail(b, KGB_ERR_ARG, "unknown option '" + k + "'");
  }
  b->planned = false;
  dropGraphs(b);
  return KGB_OK;
}

int kgb_batch_get_option(kgb_batch *b, const char *key, int64_t *value) {
  if (!b || !key || !value) return KGB_ERR_ARG;
  const std::string k(key);
  if (k == "sweep_tile_xy") *value = b->tx * 10 + b->ty;
  else if (k == "sweep_tile_z") *value = b->tz;
  else if (k == "rows_per_item") *value = b->rows_per_item;
  else if (k == "barrier_wait_ns") *value = b->barrier_wait_ns;
  else if (k == "graph") *value = b->use_graph;
  else if (k == "per_problem_kernels") *value = perProblem(b);
  else if (k == "per_problem_sweeps") *value = ownSweeps(b);
  else if (k == "branches") *value = b->branches;
  else if (k == "graph_active") *value = b->graph_active;
  else if (k == "sweep_grid") *value = b->sweep_grid;
  else if (k == "sweep_steps") *value = b->nsteps;
  else if (k == "kernels_per_iteration") *value = b->kernels_per_iter;
  else return fail(b, KGB_ERR_ARG, "unknown option '" + k + "'");
  return KGB_OK;
}

int kgb_batch_solve(kgb_batch *b, int32_t niter, double source_strength, double *part) {
  if (!b) return KGB_ERR_ARG;
  if (niter < 1) return fail(b, KGB_ERR_ARG, "need niter >= 1");
  BCK(cudaSetDevice(b->device));
  if (source_strength != b->q) {
    b->q = source_strength;
    b->planned = false;  // the fused source is part of the scattering descriptors
  }
  int rc = ensurePlan(b);
  if (rc || (rc = ensurePop(b, niter))) return rc;
  cudaGraphExec_t exec = nullptr;
  b->graph_active = false;
  if (b->use_graph && (rc = graphFor(b, niter, &exec))) return rc;
  if (exec) {
    BCK(cudaGraphLaunch(exec, b->stream));
    b->graph_active = true;
  } else if ((rc = enqueueSolve(b, niter))) {
    return rc;
  }
  b->launches += b->kernels_per_iter * niter;
  if (part)
    BCK(cudaMemcpyAsync(part, b->pop, (size_t)niter * b->inst.size() * sizeof(double), cudaMemcpyDeviceToHost,
                        b->stream));
  return checkBarrier(b);
}

int kgb_batch_autotune(kgb_batch *b, double *best_ms) {
  if (!b) return KGB_ERR_ARG;
  BCK(cudaSetDevice(b->device));
  int rc = ensurePlan(b);
  if (rc || (rc = ensurePop(b, 1))) return rc;
  BCK(cudaStreamSynchronize(b->stream));
  // one iteration from psi = 0 gives every problem a realistic rhs
  if ((rc = enqueueSolve(b, 1)) || (rc = checkBarrier(b))) return rc;
  float best = 1e30f;
  int bx = b->tx, by = b->ty, bz = b->tz;
  const int xys[3][2] = {{2, 2}, {4, 2}, {4, 4}};
  const int zs[4] = {2, 4, 8, 16};
  // the persistent sweep or each problem's own sweeps, unless the caller fixed the choice
  const int fixed_sweep = b->sweep_mode;
  int bsweep = ownSweeps(b) ? 1 : 0;
  for (int sm = 0; sm < 2; ++sm) {
    if (fixed_sweep >= 0 && sm != fixed_sweep) continue;
    b->sweep_mode = sm;
    for (auto &xy : xys)
      for (int z : zs) {
        b->tx = xy[0];
        b->ty = xy[1];
        b->tz = z;
        if ((rc = plan(b)) || (rc = ensurePop(b, 1))) return rc;
        float ms = 0.f;
        if ((rc = timeIteration(b, &ms))) return rc;
        if (ms < best) {
          best = ms;
          bx = xy[0];
          by = xy[1];
          bz = z;
          bsweep = sm;
        }
      }
  }
  b->sweep_mode = fixed_sweep >= 0 ? fixed_sweep : bsweep;
  b->tx = bx;
  b->ty = by;
  b->tz = bz;
  int brows = b->rows_per_item;
  for (int rpi : {256, 1024, 4096}) {
    b->rows_per_item = rpi;
    if ((rc = plan(b)) || (rc = ensurePop(b, 1))) return rc;
    float ms = 0.f;
    if ((rc = timeIteration(b, &ms))) return rc;
    if (ms < best) {
      best = ms;
      brows = rpi;
    }
  }
  b->rows_per_item = brows;
  // batched SIMT transforms or each problem's own kernels (tensor-core scattering,
  // the problems' moment-path choices), unless the caller fixed the choice
  if (b->own_mode < 0) {
    int bmode = perProblem(b) ? 1 : 0;
    for (int mode : {0, 1}) {
      b->own_mode = mode;
      if ((rc = plan(b)) || (rc = ensurePop(b, 1))) return rc;
      float ms = 0.f;
      if ((rc = timeIteration(b, &ms))) return rc;
      if (ms < best) {
        best = ms;
        bmode = mode;
      }
    }
    b->own_mode = bmode;
  }
  if ((rc = plan(b))) return rc;
  if (best_ms) *best_ms = best;
  return KGB_OK;
}

int kgb_batch_profile(kgb_batch *b, double ms[5]) {
  if (!b || !ms) return KGB_ERR_ARG;
  BCK(cudaSetDevice(b->device));
  int rc = ensurePlan(b);
  if (rc || (rc = ensurePop(b, 1))) return rc;
  b->rec_ok = false;  // psi may have been written through a problem's own context since
  cudaEvent_t ev[6];
  for (auto &e : ev) BCK(cudaEventCreate(&e));
  for (int rep = 0; rep < 2 && !rc; ++rep)  // the second iteration is measured
    rc = b->prec == KGB_FP64 ? enqueueIteration<double>(b, b->pop, ev) : enqueueIteration<float>(b, b->pop, ev);
  if (!rc && cudaEventSynchronize(ev[5]) == cudaSuccess)
    for (int k = 0; k < 5; ++k) {
      float t = 0.f;
      cudaEventElapsedTime(&t, ev[k], ev[k + 1]);
      ms[k] = t;
    }
  for (auto &e : ev) cudaEventDestroy(e);
  if (!rc) rc = checkBarrier(b);
  return rc;
}

int kgb_batch_launch_count(kgb_batch *b, int64_t *out) {
  if (!b || !out) return KGB_ERR_ARG;
  *out = b->launches;
  return KGB_OK;
}

}  // extern "C"
