// kripke_oracle.cpp -- CPU oracle for Kripke's source-iteration hot path.
//
// TEST INFRASTRUCTURE ONLY: a plain C++17 restatement of the reference
// algorithm used as the parity checker and as the timed CPU baseline.  The
// product (kripke_gb300/) never links, loads or calls this file.
//
// Parity: the reference cannot be built here (its kernels are RAJA lambdas and
// RAJA/camp/BLT are absent), so this oracle is "parity unpinned" against the
// reference binaries.  tests/test_oracle.py pins it against analytic known
// answers instead.
//
// What each part restates (paths relative to the Kripke source tree):
//   nesting / strides ........ src/Kripke/VarTypes.h:67-101, Core/VarLayout.h:118-170
//   decomposition ............ Core/PartitionSpace.cpp:75-123,246-273, Generate/Decomp.cpp:23-56
//   energy sets .............. Generate/Energy.cpp:22-42
//   quadrature, L, L+ ........ Generate/Quadrature.cpp:46-183 (GaussLegendre, Pnm, Ynm),
//                              :192-310 (createQuadratureSet), :335-368 (moments),
//                              :424-455 (ell, ell_plus), :469-518 (upwind/downwind)
//   space, materials ......... Generate/Space.cpp:38-365
//   data (sigs) .............. Generate/Data.cpp:69-101
//   kernels .................. Kernel/LTimes.cpp:54-65, Kernel/LPlusTimes.cpp:49-60,
//                              Kernel/Scattering.cpp:59-100,137-145, Kernel/Source.cpp:57-76,
//                              Kernel/SweepSubdomain.cpp:26-111, Kernel/Population.cpp:40-64,88-100
//   loop orders .............. Arch/*.h Sequential DGZ (parity) and OpenMP DGZ (timing)
//   solver ................... SteadyStateSolver.cpp:24-115, SweepSolver.cpp:23-87,
//                              ParallelComm.cpp:61-185 (on-rank dependency queue + plane copy)
// Generator options that the reference lacks (100 cm cube geometry, seeded
// downscatter matrices, seeded per-group perturbation) are new and are
// specified in the comments where they are generated.
//
// Build: oracle/Makefile (-O2 -ffp-contract=off -fopenmp).

#include "kripke_oracle.h"

#include <algorithm>
#include <array>
#include <cfloat>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <random>
#include <string>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

thread_local std::string g_err;

// ---------------------------------------------------------------------------
// Index types and the six nestings (VarTypes.h:67-101)
// ---------------------------------------------------------------------------
enum IdxT { T_LONG, T_DIM, T_MAT, T_DIR, T_LEG, T_MOM, T_GGRP, T_GRP, T_ZONE, T_ZK, T_ZJ, T_ZI, T_MIX, T_NUM };

const IdxT kOrder[6][13] = {
  /* DGZ */ {T_LONG, T_DIM, T_MAT, T_DIR, T_LEG, T_MOM, T_GGRP, T_GRP, T_ZONE, T_ZK, T_ZJ, T_ZI, T_MIX},
  /* DZG */ {T_LONG, T_DIM, T_MAT, T_DIR, T_LEG, T_MOM, T_ZONE, T_ZK, T_ZJ, T_ZI, T_GGRP, T_GRP, T_MIX},
  /* GDZ */ {T_LONG, T_DIM, T_MAT, T_GGRP, T_GRP, T_DIR, T_LEG, T_MOM, T_ZONE, T_ZK, T_ZJ, T_ZI, T_MIX},
  /* GZD */ {T_LONG, T_DIM, T_MAT, T_GGRP, T_GRP, T_ZONE, T_ZK, T_ZJ, T_ZI, T_MIX, T_DIR, T_LEG, T_MOM},
  /* ZDG */ {T_LONG, T_DIM, T_MAT, T_ZONE, T_ZK, T_ZJ, T_ZI, T_MIX, T_DIR, T_LEG, T_MOM, T_GGRP, T_GRP},
  /* ZGD */ {T_LONG, T_DIM, T_MAT, T_ZONE, T_ZK, T_ZJ, T_ZI, T_MIX, T_GGRP, T_GRP, T_DIR, T_LEG, T_MOM},
};

int orderPos(int layout, IdxT t) {
  for (int i = 0; i < 13; ++i) if (kOrder[layout][i] == t) return i;
  return -1;
}

// Strides of a field chunk: its index types are sorted (stably, ties keep
// argument order) by their position in the nesting's order list; the first
// sorted index has the longest stride, the last is stride one.
void computeStrides(int layout, int n, const IdxT *types, const int64_t *dims, int64_t *strides) {
  std::array<std::pair<int, int>, 4> p;
  for (int i = 0; i < n; ++i) p[i] = {i, orderPos(layout, types[i])};
  std::stable_sort(p.begin(), p.begin() + n, [](auto a, auto b) { return a.second < b.second; });
  int64_t s = 1;
  for (int k = n - 1; k >= 0; --k) {
    strides[p[k].first] = s;
    s *= dims[p[k].first];
  }
}

// ---------------------------------------------------------------------------
// Partition spaces for a single rank (PartitionSpace.h:19-30)
// ---------------------------------------------------------------------------
enum Space { S_P, S_Q, S_RX, S_RY, S_RZ, S_R, S_PR, S_PQR, S_NULL };

struct Decomp {
  int SP = 1, SQ = 1, Sx = 1, Sy = 1, Sz = 1;
  int num() const { return SP * SQ * Sx * Sy * Sz; }
  std::array<int, 5> coord(int sdom) const {
    std::array<int, 5> c;
    c[4] = sdom % Sz; sdom /= Sz;
    c[3] = sdom % Sy; sdom /= Sy;
    c[2] = sdom % Sx; sdom /= Sx;
    c[1] = sdom % SQ; sdom /= SQ;
    c[0] = sdom;
    return c;
  }
  int sdomOf(const std::array<int, 5> &c) const {
    return (((c[0] * SQ + c[1]) * Sx + c[2]) * Sy + c[3]) * Sz + c[4];
  }
  int numChunks(Space s) const {
    switch (s) {
      case S_P: return SP; case S_Q: return SQ; case S_RX: return Sx; case S_RY: return Sy;
      case S_RZ: return Sz; case S_R: return Sx * Sy * Sz; case S_PR: return SP * Sx * Sy * Sz;
      case S_PQR: return num(); default: return 1;
    }
  }
  int chunkOf(Space s, int sdom) const {
    auto c = coord(sdom);
    switch (s) {
      case S_P: return c[0]; case S_Q: return c[1]; case S_RX: return c[2];
      case S_RY: return c[3]; case S_RZ: return c[4];
      case S_R: return (c[2] * Sy + c[3]) * Sz + c[4];
      case S_PR: return ((c[0] * Sx + c[2]) * Sy + c[3]) * Sz + c[4];
      case S_PQR: return sdom; default: return 0;
    }
  }
  // first subdomain that maps to a chunk (PartitionSpace::spaceToSubdomain)
  int sdomOfChunk(Space s, int chunk) const {
    std::array<int, 5> c{0, 0, 0, 0, 0};
    switch (s) {
      case S_P: c[0] = chunk; break; case S_Q: c[1] = chunk; break; case S_RX: c[2] = chunk; break;
      case S_RY: c[3] = chunk; break; case S_RZ: c[4] = chunk; break;
      case S_R: c[4] = chunk % Sz; chunk /= Sz; c[3] = chunk % Sy; c[2] = chunk / Sy; break;
      case S_PR: c[4] = chunk % Sz; chunk /= Sz; c[3] = chunk % Sy; chunk /= Sy; c[2] = chunk % Sx; c[0] = chunk / Sx; break;
      case S_PQR: return chunk; default: break;
    }
    return sdomOf(c);
  }
};

struct Field {
  Space space = S_NULL;
  int ndims = 1;
  IdxT types[4] = {T_LONG, T_LONG, T_LONG, T_LONG};
  bool is_int = false;
  std::vector<std::array<int64_t, 4>> dims, strides;
  std::vector<std::vector<double>> d;
  std::vector<std::vector<int32_t>> i;
  int64_t chunkSize(int c) const {
    int64_t s = 1;
    for (int k = 0; k < ndims; ++k) s *= dims[c][k];
    return s;
  }
};

struct QuadraturePoint {
  double xcos, ycos, zcos, w;
  int id, jd, kd, octant;
};

}  // namespace

struct orc_problem {
  orc_input in{};
  Decomp dc;
  int G = 0, Gs = 0, D = 0, Ds = 0, M = 0, L = 0;
  int nxs = 0, nys = 0, nzs = 0;  // zones per zone set
  std::vector<int> mix_per_r;     // mix elements per R chunk
  std::vector<int> legendre_of_moment;
  std::vector<std::array<int, 3>> upwind, downwind;  // per sdom, -1 = boundary
  std::map<std::string, Field> f;
  int threads = 0;
  bool block_jacobi = false;  // SteadyStateSolver's block_jacobi argument (--pmethod bj)
  double last_solve_s = 0.0;

  Field &fld(const char *n) { return f.at(n); }
  int sdomChunk(const char *n, int sdom) { return dc.chunkOf(f.at(n).space, sdom); }
  double *dptr(const char *n, int sdom) { Field &x = f.at(n); return x.d[dc.chunkOf(x.space, sdom)].data(); }
  int32_t *iptr(const char *n, int sdom) { Field &x = f.at(n); return x.i[dc.chunkOf(x.space, sdom)].data(); }
  const int64_t *strd(const char *n, int sdom) { Field &x = f.at(n); return x.strides[dc.chunkOf(x.space, sdom)].data(); }
  bool par() const { return threads > 0; }
};

namespace {

// Create a field over `space` whose chunk c has dimension sizes dimfn(c).
template <typename DimFn>
void addField(orc_problem &p, const char *name, Space space, bool is_int, std::initializer_list<IdxT> types, DimFn dimfn) {
  Field fl;
  fl.space = space;
  fl.is_int = is_int;
  fl.ndims = (int)types.size();
  int k = 0;
  for (IdxT t : types) fl.types[k++] = t;
  int nch = p.dc.numChunks(space);
  fl.dims.resize(nch);
  fl.strides.resize(nch);
  for (int c = 0; c < nch; ++c) {
    std::array<int64_t, 4> dm{1, 1, 1, 1};
    dimfn(c, dm);
    fl.dims[c] = dm;
    std::array<int64_t, 4> st{1, 1, 1, 1};
    computeStrides(p.in.layout, fl.ndims, fl.types, dm.data(), st.data());
    fl.strides[c] = st;
    if (is_int) fl.i.emplace_back(fl.chunkSize(c), 0);
    else fl.d.emplace_back(fl.chunkSize(c), 0.0);
  }
  p.f[name] = std::move(fl);
}

// ------------------------------ quadrature ---------------------------------
// Gauss-Legendre nodes/weights by Newton iteration on P_n (Quadrature.cpp:46-76).
void gaussLegendre(double x1, double x2, std::vector<double> &x, std::vector<double> &w, double eps) {
  int n = (int)x.size();
  int m = (n + 1) / 2;
  double xm = 0.5 * (x2 + x1), xl = 0.5 * (x2 - x1);
  for (int i = 1; i <= m; i++) {
    double z = cos(M_PI * (i - 0.25) / (n + 0.5)), z1, pp;
    do {
      double p1 = 1.0, p2 = 0.0, p3;
      for (int j = 1; j <= n; j++) {
        p3 = p2;
        p2 = p1;
        p1 = ((2.0 * j - 1.0) * z * p2 - (j - 1.0) * p3) / j;
      }
      pp = n * (z * p1 - p2) / (z * z - 1.0);
      z1 = z;
      z = z1 - p1 / pp;
    } while (fabs(z - z1) > eps);
    x[i - 1] = xm - xl * z;
    x[n - i] = xm + xl * z;
    w[i - 1] = 2.0 * xl / ((1.0 - z * z) * pp * pp);
    w[n - i] = w[i - 1];
  }
}

double factorial(int n) {
  double f = 1.0;
  for (int i = n; i > 0; --i) f *= (double)i;
  return f;
}

// Associated Legendre function P_n^m(x), m >= 0 (Quadrature.cpp:92-138).
double assocLegendre(int n, int m, double x) {
  double pmm = 1.0;
  if (m > 0) {
    double somx2 = sqrt((1.0 - x) * (1.0 + x)), fact = 1.0;
    for (int i = 1; i <= m; i++) {
      pmm *= -fact * somx2;
      fact += 2.0;
    }
  }
  if (n == m) return pmm;
  double pmmp1 = x * (2 * m + 1) * pmm;
  if (n == m + 1) return pmmp1;
  double pnn = 0;
  for (int nn = m + 2; nn <= n; nn++) {
    pnn = (x * (2 * nn - 1) * pmmp1 - (nn + m - 1) * pmm) / (nn - m);
    pmm = pmmp1;
    pmmp1 = pnn;
  }
  return pnn;
}

// Real spherical harmonic Y_n^m at direction (mu, eta, xi) (Quadrature.cpp:140-183).
double realYnm(int n, int m, double mu, double eta, double xi) {
  double tmp = fabs(eta / (mu + 1.e-20));
  double phi_tmp = atan(tmp), phi;
  if ((mu > 0) && (eta > 0)) phi = phi_tmp;
  else if ((mu < 0) && (eta > 0)) phi = M_PI - fabs(phi_tmp);
  else if ((mu < 0) && (eta < 0)) phi = M_PI + fabs(phi_tmp);
  else phi = 2.0 * M_PI - fabs(phi_tmp);
  double fac1 = factorial(n - std::abs(m));
  double fac2 = factorial(n + std::abs(m));
  double pnm = assocLegendre(n, std::abs(m), xi);
  tmp = ((double)m) * phi;
  double taum = (m >= 0) ? cos(tmp) : sin(-tmp);
  double dm0 = (m == 0) ? 1.0 : 0.0;
  tmp = ((2 * n + 1) * fac1) / (2.0 * (1.0 + dm0) * M_PI * fac2);
  return sqrt(tmp) * pnm * taum;
}

bool octantDescending(QuadraturePoint const &a, QuadraturePoint const &b) { return b.octant < a.octant; }

// Quadrature set (Quadrature.cpp:192-310): Gauss-Legendre product set sorted
// by octant (std::sort, descending), or the dummy "S2" with repeated points.
std::vector<QuadraturePoint> makeQuadrature(const orc_input &in) {
  std::vector<QuadraturePoint> dirs(in.num_directions);
  int np = in.quad_num_polar, na = in.quad_num_azimuthal;
  if (np > 0) {
    std::vector<double> pc(np), pw(np);
    gaussLegendre(-1.0, 1.0, pc, pw, DBL_EPSILON);
    std::vector<double> az(na), aw(na);
    double dangle = 2.0 * M_PI / ((double)na);
    for (int i = 0; i < na; i++) {
      az[i] = (i == 0) ? dangle / 2.0 : az[i - 1] + dangle;
      aw[i] = dangle;
    }
    int d = 0;
    for (int i = 0; i < np; i++) {
      for (int j = 0; j < na; j++) {
        double xc = sqrt(1.0 - pc[i] * pc[i]) * cos(az[j]);
        double yc = sqrt(1.0 - pc[i] * pc[i]) * sin(az[j]);
        double zc = pc[i];
        QuadraturePoint &q = dirs[d];
        q.id = (xc > 0.) ? 1 : -1;
        q.jd = (yc > 0.) ? 1 : -1;
        q.kd = (zc > 0.) ? 1 : -1;
        q.octant = (q.id == -1 ? 1 : 0) + (q.jd == -1 ? 2 : 0) + (q.kd == -1 ? 4 : 0);
        q.xcos = std::abs(xc);
        q.ycos = std::abs(yc);
        q.zcos = std::abs(zc);
        q.w = pw[i] * aw[j];
        ++d;
      }
    }
    std::sort(dirs.begin(), dirs.end(), octantDescending);
  } else {
    double mu = cos(M_PI / 4);
    double eta = sqrt(1 - mu * mu) * cos(M_PI / 4);
    double xi = sqrt(1 - mu * mu) * sin(M_PI / 4);
    int per = in.num_directions / 8, d = 0;
    for (int oct = 0; oct < 8; ++oct) {
      for (int sd = 0; sd < per; sd++, d++) {
        QuadraturePoint &q = dirs[d];
        q.id = (oct & 1) ? 1 : -1;
        q.jd = ((oct >> 1) & 1) ? 1 : -1;
        q.kd = ((oct >> 2) & 1) ? 1 : -1;
        q.octant = 0;  // value-initialised and never assigned by the reference
        q.w = 4.0 * M_PI / (double)in.num_directions;
        q.xcos = mu;
        q.ycos = eta;
        q.zcos = xi;
      }
    }
  }
  return dirs;
}

// ------------------------------ geometry -----------------------------------
// Kobayashi-3i material map (Space.cpp:142-177).
int materialKobayashi(double x, double y, double z) {
  x = std::abs(x); y = std::abs(y); z = std::abs(z);
  if (x <= 10.0 && y <= 10.0 && z <= 10.0) return 0;
  if (x <= 10.0 && y <= 60.0 && z <= 10.0) return 1;
  if (x <= 40.0 && y >= 50.0 && y <= 60.0 && z <= 10.0) return 1;
  if (x >= 30.0 && x <= 40.0 && y >= 50.0 && y <= 60.0 && z <= 40.0) return 1;
  if (x >= 30.0 && x <= 40.0 && y >= 50.0 && z >= 30.0 && z <= 40.0) return 1;
  return 2;
}

// 100 cm cube [0,100]^3: source block [0,10]^3, duct {x,z <= 10, y <= 60}
// (the first leg of the Kobayashi duct only), shield elsewhere.
int materialCube(double x, double y, double z) {
  if (x <= 10.0 && y <= 10.0 && z <= 10.0) return 0;
  if (x <= 10.0 && y <= 60.0 && z <= 10.0) return 1;
  return 2;
}

inline double unitDraw(std::mt19937_64 &rng) { return (double)(rng() >> 11) * 0x1.0p-53; }

bool generate(orc_problem &p) {
  const orc_input &in = p.in;
  // --- checks (InputVariables.cpp:52-109 plus divisibility asserts) ---
  if (in.layout < 0 || in.layout > 5) { g_err = "bad layout"; return false; }
  if (in.num_groups < 1 || in.num_groupsets < 1 || in.num_groups % in.num_groupsets) { g_err = "groups/groupsets"; return false; }
  if (in.num_directions < 8 || in.num_dirsets < 1 || (in.num_dirsets % 8 && in.num_dirsets < 8) || in.num_directions % in.num_dirsets) { g_err = "directions/dirsets"; return false; }
  if (in.legendre_order < 0) { g_err = "legendre order"; return false; }
  for (int k = 0; k < 3; ++k) if (in.num_zonesets_dim[k] < 1) { g_err = "zonesets"; return false; }
  if (in.nx % in.num_zonesets_dim[0] || in.ny % in.num_zonesets_dim[1] || in.nz % in.num_zonesets_dim[2]) { g_err = "zones/zonesets"; return false; }
  if (in.quad_num_polar > 0) {
    if (in.quad_num_polar % 4 || in.quad_num_azimuthal % 2 || in.quad_num_polar * in.quad_num_azimuthal != in.num_directions) {
      g_err = "quadrature sizes"; return false;
    }
  }
  p.dc.SP = in.num_groupsets; p.dc.SQ = in.num_dirsets;
  p.dc.Sx = in.num_zonesets_dim[0]; p.dc.Sy = in.num_zonesets_dim[1]; p.dc.Sz = in.num_zonesets_dim[2];
  p.G = in.num_groups; p.Gs = p.G / p.dc.SP;
  p.D = in.num_directions; p.Ds = p.D / p.dc.SQ;
  p.L = in.legendre_order; p.M = (p.L + 1) * (p.L + 1);
  p.nxs = in.nx / p.dc.Sx; p.nys = in.ny / p.dc.Sy; p.nzs = in.nz / p.dc.Sz;
  const int Gs = p.Gs, Ds = p.Ds, M = p.M, G = p.G;
  const int64_t Zs = (int64_t)p.nxs * p.nys * p.nzs;
  const int nxs = p.nxs, nys = p.nys, nzs = p.nzs;

  // --- per-(material, group) cross sections (new: seeded perturbation) ---
  std::mt19937_64 rng(in.seed);
  std::vector<double> sigt_mg(3 * G), sigs_mg(3 * G);
  for (int m = 0; m < 3; ++m)
    for (int g = 0; g < G; ++g) {
      double ft = 1.0, fs = 1.0;
      if (in.perturb) {
        ft = 1.0 + 0.2 * (2.0 * unitDraw(rng) - 1.0);
        fs = 1.0 + 0.2 * (2.0 * unitDraw(rng) - 1.0);
      }
      sigt_mg[m * G + g] = in.sigt[m] * ft;
      sigs_mg[m * G + g] = in.sigs[m] * fs;
    }

  // --- quadrature (Quadrature.cpp:315-455) ---
  p.legendre_of_moment.resize(M);
  {
    int nm = 0;
    for (int n = 0; n <= p.L; ++n)
      for (int m = -n; m <= n; ++m) p.legendre_of_moment[nm++] = n;
  }
  addField(p, "moment_to_legendre", S_NULL, true, {T_MOM}, [&](int, auto &dm) { dm[0] = M; });
  for (int nm = 0; nm < M; ++nm) p.fld("moment_to_legendre").i[0][nm] = p.legendre_of_moment[nm];

  auto pts = makeQuadrature(in);
  const char *dnames[] = {"quadrature/xcos", "quadrature/ycos", "quadrature/zcos", "quadrature/w"};
  for (auto n : dnames) addField(p, n, S_Q, false, {T_DIR}, [&](int, auto &dm) { dm[0] = Ds; });
  const char *inames[] = {"quadrature/id", "quadrature/jd", "quadrature/kd", "quadrature/octant"};
  for (auto n : inames) addField(p, n, S_Q, true, {T_DIR}, [&](int, auto &dm) { dm[0] = Ds; });
  for (int q = 0; q < p.dc.SQ; ++q)
    for (int d = 0; d < Ds; ++d) {
      auto &pt = pts[q * Ds + d];
      p.fld("quadrature/xcos").d[q][d] = pt.xcos;
      p.fld("quadrature/ycos").d[q][d] = pt.ycos;
      p.fld("quadrature/zcos").d[q][d] = pt.zcos;
      p.fld("quadrature/w").d[q][d] = pt.w;
      p.fld("quadrature/id").i[q][d] = pt.id;
      p.fld("quadrature/jd").i[q][d] = pt.jd;
      p.fld("quadrature/kd").i[q][d] = pt.kd;
      p.fld("quadrature/octant").i[q][d] = pt.octant;
    }
  addField(p, "ell", S_Q, false, {T_MOM, T_DIR}, [&](int, auto &dm) { dm[0] = M; dm[1] = Ds; });
  addField(p, "ell_plus", S_Q, false, {T_DIR, T_MOM}, [&](int, auto &dm) { dm[0] = Ds; dm[1] = M; });
  {
    const double SQRT4PI = std::sqrt(4 * M_PI);
    Field &fe = p.fld("ell"), &fp = p.fld("ell_plus");
    for (int q = 0; q < p.dc.SQ; ++q) {
      const int64_t *se = fe.strides[q].data(), *sp = fp.strides[q].data();
      int nm = 0;
      for (int n = 0; n <= p.L; n++)
        for (int m = -n; m <= n; m++, nm++)
          for (int d = 0; d < Ds; ++d) {
            auto &pt = pts[q * Ds + d];
            double xc = (pt.id) * (pt.xcos), yc = (pt.jd) * (pt.ycos), zc = (pt.kd) * (pt.zcos);
            double ynm = realYnm(n, m, xc, yc, zc);
            fe.d[q][nm * se[0] + d * se[1]] = pt.w * ynm / SQRT4PI;
            fp.d[q][d * sp[0] + nm * sp[1]] = ynm * SQRT4PI;
          }
    }
  }
  // upwind / downwind adjacency (Quadrature.cpp:469-518)
  p.upwind.resize(p.dc.num());
  p.downwind.resize(p.dc.num());
  const int S[3] = {p.dc.Sx, p.dc.Sy, p.dc.Sz};
  for (int s = 0; s < p.dc.num(); ++s) {
    auto c = p.dc.coord(s);
    int q = c[1];
    int sweep[3] = {pts[q * Ds].id, pts[q * Ds].jd, pts[q * Ds].kd};
    for (int dim = 0; dim < 3; ++dim) {
      auto up = c, dn = c;
      up[2 + dim] -= sweep[dim];
      dn[2 + dim] += sweep[dim];
      p.upwind[s][dim] = (up[2 + dim] < 0 || up[2 + dim] >= S[dim]) ? -1 : p.dc.sdomOf(up);
      p.downwind[s][dim] = (dn[2 + dim] < 0 || dn[2 + dim] >= S[dim]) ? -1 : p.dc.sdomOf(dn);
    }
  }

  // --- space (Space.cpp:38-365) ---
  double x_min, x_max, y_min, y_max, z_min, z_max;
  if (in.geometry == 1) {
    x_min = 0.0; x_max = 100.0; y_min = 0.0; y_max = 100.0; z_min = 0.0; z_max = 100.0;
  } else {
    x_min = -60.0; x_max = 60.0; y_min = -100.0; y_max = 100.0; z_min = -60.0; z_max = 60.0;
  }
  double dx = (x_max - x_min) / in.nx, dy = (y_max - y_min) / in.ny, dz = (z_max - z_min) / in.nz;
  addField(p, "dx", S_RX, false, {T_ZI}, [&](int, auto &dm) { dm[0] = nxs; });
  addField(p, "dy", S_RY, false, {T_ZJ}, [&](int, auto &dm) { dm[0] = nys; });
  addField(p, "dz", S_RZ, false, {T_ZK}, [&](int, auto &dm) { dm[0] = nzs; });
  for (auto &v : p.fld("dx").d) std::fill(v.begin(), v.end(), dx);
  for (auto &v : p.fld("dy").d) std::fill(v.begin(), v.end(), dy);
  for (auto &v : p.fld("dz").d) std::fill(v.begin(), v.end(), dz);
  double zone_volume = dx * dy * dz;
  addField(p, "volume", S_R, false, {T_ZONE}, [&](int, auto &dm) { dm[0] = Zs; });
  for (auto &v : p.fld("volume").d) std::fill(v.begin(), v.end(), zone_volume);

  int ns = in.num_material_subsamples;
  double sample_vol_frac = 1.0 / (double)(ns * ns * ns);
  int nr = p.dc.numChunks(S_R);
  std::vector<std::vector<std::array<double, 3>>> mix(nr);
  for (int r = 0; r < nr; ++r) {
    int sdom = p.dc.sdomOfChunk(S_R, r);
    auto c = p.dc.coord(sdom);
    double x0 = x_min + dx * (c[2] * nxs), y0 = y_min + dy * (c[3] * nys), z0 = z_min + dz * (c[4] * nzs);
    mix[r].assign(Zs, {0.0, 0.0, 0.0});
    for (int k = 0; k < nzs; k++)
      for (int j = 0; j < nys; j++)
        for (int i = 0; i < nxs; i++) {
          int64_t zone = ((int64_t)k * nys + j) * nxs + i;
          double xi = x0 + dx * i, yi = y0 + dy * j, zi = z0 + dz * k;
          for (int si = 0; si < ns; ++si)
            for (int sj = 0; sj < ns; ++sj)
              for (int sk = 0; sk < ns; ++sk) {
                double x = xi + dx * (si + 1) / (ns + 1);
                double y = yi + dy * (sj + 1) / (ns + 1);
                double z = zi + dz * (sk + 1) / (ns + 1);
                int mat = (in.geometry == 1) ? materialCube(x, y, z) : materialKobayashi(x, y, z);
                mix[r][zone][mat] += sample_vol_frac;
              }
        }
  }
  p.mix_per_r.assign(nr, 0);
  for (int r = 0; r < nr; ++r)
    for (auto &z : mix[r])
      for (int m = 0; m < 3; ++m) p.mix_per_r[r] += (z[m] > 0.0) ? 1 : 0;
  addField(p, "mixelem_to_zone", S_R, true, {T_MIX}, [&](int r, auto &dm) { dm[0] = p.mix_per_r[r]; });
  addField(p, "mixelem_to_material", S_R, true, {T_MIX}, [&](int r, auto &dm) { dm[0] = p.mix_per_r[r]; });
  addField(p, "mixelem_to_fraction", S_R, false, {T_MIX}, [&](int r, auto &dm) { dm[0] = p.mix_per_r[r]; });
  addField(p, "zone_to_num_mixelem", S_R, true, {T_ZONE}, [&](int, auto &dm) { dm[0] = Zs; });
  addField(p, "zone_to_mixelem", S_R, true, {T_ZONE}, [&](int, auto &dm) { dm[0] = Zs; });
  for (int r = 0; r < nr; ++r) {
    int me = 0;
    for (int64_t z = 0; z < Zs; ++z) {
      p.fld("zone_to_mixelem").i[r][z] = me;
      int cnt = 0;
      double zone_frac = 0.0;
      for (int m = 0; m < 3; ++m) {
        if (mix[r][z][m] > 0.0) {
          p.fld("mixelem_to_zone").i[r][me] = (int32_t)z;
          p.fld("mixelem_to_material").i[r][me] = m;
          p.fld("mixelem_to_fraction").d[r][me] = mix[r][z][m];
          zone_frac += mix[r][z][m];
          ++cnt;
          ++me;
        }
      }
      if (zone_frac != 1.0) { g_err = "zone fraction != 1"; return false; }
      p.fld("zone_to_num_mixelem").i[r][z] = cnt;
    }
  }
  // sigt_zonal(g,z) = sum over mix elements of fraction * sigma_t(material)  (Space.cpp:333-363)
  addField(p, "sigt_zonal", S_PR, false, {T_GRP, T_ZONE}, [&](int, auto &dm) { dm[0] = Gs; dm[1] = Zs; });
  {
    Field &fs = p.fld("sigt_zonal");
    for (int c = 0; c < p.dc.numChunks(S_PR); ++c) {
      int sdom = p.dc.sdomOfChunk(S_PR, c);
      int pg = p.dc.coord(sdom)[0];
      int r = p.dc.chunkOf(S_R, sdom);
      const int64_t *st = fs.strides[c].data();
      for (int g = 0; g < Gs; ++g)
        for (int me = 0; me < p.mix_per_r[r]; ++me) {
          int z = p.fld("mixelem_to_zone").i[r][me];
          int mat = p.fld("mixelem_to_material").i[r][me];
          fs.d[c][g * st[0] + z * st[1]] += p.fld("mixelem_to_fraction").d[r][me] * sigt_mg[mat * G + pg * Gs + g];
        }
    }
  }

  // --- data (Data.cpp:22-105) ---
  addField(p, "psi", S_PQR, false, {T_DIR, T_GRP, T_ZONE}, [&](int, auto &dm) { dm[0] = Ds; dm[1] = Gs; dm[2] = Zs; });
  addField(p, "rhs", S_PQR, false, {T_DIR, T_GRP, T_ZONE}, [&](int, auto &dm) { dm[0] = Ds; dm[1] = Gs; dm[2] = Zs; });
  addField(p, "phi", S_PR, false, {T_MOM, T_GRP, T_ZONE}, [&](int, auto &dm) { dm[0] = M; dm[1] = Gs; dm[2] = Zs; });
  addField(p, "phi_out", S_PR, false, {T_MOM, T_GRP, T_ZONE}, [&](int, auto &dm) { dm[0] = M; dm[1] = Gs; dm[2] = Zs; });
  addField(p, "i_plane", S_PQR, false, {T_DIR, T_GRP, T_ZJ, T_ZK}, [&](int, auto &dm) { dm[0] = Ds; dm[1] = Gs; dm[2] = nys; dm[3] = nzs; });
  addField(p, "j_plane", S_PQR, false, {T_DIR, T_GRP, T_ZI, T_ZK}, [&](int, auto &dm) { dm[0] = Ds; dm[1] = Gs; dm[2] = nxs; dm[3] = nzs; });
  addField(p, "k_plane", S_PQR, false, {T_DIR, T_GRP, T_ZI, T_ZJ}, [&](int, auto &dm) { dm[0] = Ds; dm[1] = Gs; dm[2] = nxs; dm[3] = nys; });
  addField(p, "data/sigs", S_NULL, false, {T_MAT, T_LEG, T_GGRP, T_GGRP}, [&](int, auto &dm) { dm[0] = 3; dm[1] = p.L + 1; dm[2] = G; dm[3] = G; });
  {
    Field &fs = p.fld("data/sigs");
    const int64_t *st = fs.strides[0].data();
    auto at = [&](int m, int l, int g, int gp) -> double & { return fs.d[0][m * st[0] + l * st[1] + g * st[2] + gp * st[3]]; };
    if (in.scatter == 1) {
      // New generator option: per material m and Legendre order l a seeded
      // lower-triangular matrix U[g][g'] (g >= g', uniform [0,1), drawn in
      // (m, l, g, g') order), columns scaled so that sum_g S0[g][g'] =
      // c_m * sigma_t(m, g') with the scattering ratio c_m = sigs[m] / sigt[m]
      // of the input (0.5 for the reference cross sections), order l damped
      // by 1/(2l+1).
      std::vector<double> U((size_t)G * G);
      for (int m = 0; m < 3; ++m)
        for (int l = 0; l <= p.L; ++l) {
          const double ratio = in.sigt[m] != 0.0 ? in.sigs[m] / in.sigt[m] : 0.0;
          std::fill(U.begin(), U.end(), 0.0);
          for (int g = 0; g < G; ++g)
            for (int gp = 0; gp <= g; ++gp) U[(size_t)g * G + gp] = unitDraw(rng);
          for (int gp = 0; gp < G; ++gp) {
            double col = 0.0;
            for (int g = gp; g < G; ++g) col += U[(size_t)g * G + gp];
            double scale = ratio * sigt_mg[m * G + gp] / col;
            for (int g = gp; g < G; ++g) at(m, l, g, gp) = (U[(size_t)g * G + gp] * scale) / (double)(2 * l + 1);
          }
        }
    } else {
      for (int m = 0; m < 3; ++m)
        for (int g = 0; g < G; ++g) at(m, 0, g, g) = sigs_mg[m * G + g];
    }
  }
  return true;
}

// ------------------------------ kernels ------------------------------------

void kLTimes(orc_problem &p) {
  for (int sdom = 0; sdom < p.dc.num(); ++sdom) {
    const double *psi = p.dptr("psi", sdom), *ell = p.dptr("ell", sdom);
    double *phi = p.dptr("phi", sdom);
    const int64_t *sp = p.strd("psi", sdom), *sf = p.strd("phi", sdom), *se = p.strd("ell", sdom);
    const int Ds = p.Ds, Gs = p.Gs, M = p.M;
    const int64_t Zs = (int64_t)p.nxs * p.nys * p.nzs;
#pragma omp parallel for collapse(2) schedule(static) if (p.par())
    for (int nm = 0; nm < M; ++nm)
      for (int g = 0; g < Gs; ++g)
        for (int d = 0; d < Ds; ++d) {
          double e = ell[nm * se[0] + d * se[1]];
          for (int64_t z = 0; z < Zs; ++z)
            phi[nm * sf[0] + g * sf[1] + z * sf[2]] += e * psi[d * sp[0] + g * sp[1] + z * sp[2]];
        }
  }
}

void kLPlusTimes(orc_problem &p) {
  for (int sdom = 0; sdom < p.dc.num(); ++sdom) {
    const double *phi_out = p.dptr("phi_out", sdom), *ellp = p.dptr("ell_plus", sdom);
    double *rhs = p.dptr("rhs", sdom);
    const int64_t *sr = p.strd("rhs", sdom), *sf = p.strd("phi_out", sdom), *se = p.strd("ell_plus", sdom);
    const int Ds = p.Ds, Gs = p.Gs, M = p.M;
    const int64_t Zs = (int64_t)p.nxs * p.nys * p.nzs;
#pragma omp parallel for collapse(2) schedule(static) if (p.par())
    for (int d = 0; d < Ds; ++d)
      for (int g = 0; g < Gs; ++g)
        for (int nm = 0; nm < M; ++nm) {
          double e = ellp[d * se[0] + nm * se[1]];
          for (int64_t z = 0; z < Zs; ++z)
            rhs[d * sr[0] + g * sr[1] + z * sr[2]] += e * phi_out[nm * sf[0] + g * sf[1] + z * sf[2]];
        }
  }
}

void kScattering(orc_problem &p) {
  Field &fphi = p.fld("phi");
  int nch = p.dc.numChunks(S_PR);
  const int G = p.G, Gs = p.Gs, M = p.M;
  const int64_t Zs = (int64_t)p.nxs * p.nys * p.nzs;
  const double *sigs = p.fld("data/sigs").d[0].data();
  const int64_t *ss = p.fld("data/sigs").strides[0].data();
  for (int csrc = 0; csrc < nch; ++csrc) {
    int ssrc = p.dc.sdomOfChunk(S_PR, csrc);
    for (int cdst = 0; cdst < nch; ++cdst) {
      int sdst = p.dc.sdomOfChunk(S_PR, cdst);
      int r = p.dc.chunkOf(S_R, ssrc);
      if (r != p.dc.chunkOf(S_R, sdst)) continue;
      int glo_src = p.dc.coord(ssrc)[0] * Gs, glo_dst = p.dc.coord(sdst)[0] * Gs;
      const double *phi = fphi.d[csrc].data();
      double *phi_out = p.fld("phi_out").d[cdst].data();
      const int64_t *sf = fphi.strides[csrc].data(), *so = p.fld("phi_out").strides[cdst].data();
      const int32_t *z2m = p.fld("zone_to_mixelem").i[r].data(), *z2n = p.fld("zone_to_num_mixelem").i[r].data();
      const int32_t *m2mat = p.fld("mixelem_to_material").i[r].data();
      const double *m2f = p.fld("mixelem_to_fraction").d[r].data();
      const int32_t *m2l = p.fld("moment_to_legendre").i[0].data();
      (void)G;
#pragma omp parallel for collapse(2) schedule(static) if (p.par())
      for (int nm = 0; nm < M; ++nm)
        for (int g = 0; g < Gs; ++g)
          for (int gp = 0; gp < Gs; ++gp)
            for (int64_t z = 0; z < Zs; ++z) {
              int n = m2l[nm];
              int mix_start = z2m[z], mix_stop = mix_start + z2n[z];
              double sigs_z = 0.0;
              for (int mix = mix_start; mix < mix_stop; ++mix) {
                int mat = m2mat[mix];
                sigs_z += sigs[mat * ss[0] + n * ss[1] + (g + glo_dst) * ss[2] + (gp + glo_src) * ss[3]] * m2f[mix];
              }
              phi_out[nm * so[0] + g * so[1] + z * so[2]] += sigs_z * phi[nm * sf[0] + gp * sf[1] + z * sf[2]];
            }
    }
  }
}

void kSource(orc_problem &p) {
  Field &fo = p.fld("phi_out");
  const double q = p.in.source_strength;
  for (int c = 0; c < p.dc.numChunks(S_PR); ++c) {
    int sdom = p.dc.sdomOfChunk(S_PR, c);
    int r = p.dc.chunkOf(S_R, sdom);
    double *phi_out = fo.d[c].data();
    const int64_t *so = fo.strides[c].data();
    const int32_t *m2z = p.fld("mixelem_to_zone").i[r].data(), *m2mat = p.fld("mixelem_to_material").i[r].data();
    const double *m2f = p.fld("mixelem_to_fraction").d[r].data();
    int nmix = p.mix_per_r[r];
#pragma omp parallel for collapse(2) schedule(static) if (p.par())
    for (int g = 0; g < p.Gs; ++g)
      for (int mix = 0; mix < nmix; ++mix)
        if (m2mat[mix] == 0) phi_out[0 * so[0] + g * so[1] + (int64_t)m2z[mix] * so[2]] += q * m2f[mix];
  }
}

void kSweep(orc_problem &p, int sdom) {
  const int Ds = p.Ds, Gs = p.Gs, ni = p.nxs, nj = p.nys, nk = p.nzs;
  const double *xcos = p.dptr("quadrature/xcos", sdom), *ycos = p.dptr("quadrature/ycos", sdom), *zcos = p.dptr("quadrature/zcos", sdom);
  const int32_t *idv = p.iptr("quadrature/id", sdom), *jdv = p.iptr("quadrature/jd", sdom), *kdv = p.iptr("quadrature/kd", sdom);
  const double *dx = p.dptr("dx", sdom), *dy = p.dptr("dy", sdom), *dz = p.dptr("dz", sdom);
  const double *sigt = p.dptr("sigt_zonal", sdom), *rhs = p.dptr("rhs", sdom);
  double *psi = p.dptr("psi", sdom);
  double *lf = p.dptr("i_plane", sdom), *fr = p.dptr("j_plane", sdom), *bo = p.dptr("k_plane", sdom);
  const int64_t *ss = p.strd("sigt_zonal", sdom), *sr = p.strd("rhs", sdom), *sp = p.strd("psi", sdom);
  const int64_t *si = p.strd("i_plane", sdom), *sj = p.strd("j_plane", sdom), *sk = p.strd("k_plane", sdom);
  // all directions of the subdomain share direction 0's traversal (SweepSubdomain.cpp:145-158)
  const int id = idv[0], jd = jdv[0], kd = kdv[0];
  const int i0 = id > 0 ? 0 : ni - 1, i1 = id > 0 ? ni : -1;
  const int j0 = jd > 0 ? 0 : nj - 1, j1 = jd > 0 ? nj : -1;
  const int k0 = kd > 0 ? 0 : nk - 1, k1 = kd > 0 ? nk : -1;
#pragma omp parallel for collapse(2) schedule(static) if (p.par())
  for (int d = 0; d < Ds; ++d)
    for (int g = 0; g < Gs; ++g)
      for (int k = k0; k != k1; k += kd)
        for (int j = j0; j != j1; j += jd)
          for (int i = i0; i != i1; i += id) {
            double xcos_dxi = 2.0 * xcos[d] / dx[i];
            double ycos_dyj = 2.0 * ycos[d] / dy[j];
            double zcos_dzk = 2.0 * zcos[d] / dz[k];
            int64_t z = ((int64_t)k * nj + j) * ni + i;
            double &plf = lf[d * si[0] + g * si[1] + j * si[2] + k * si[3]];
            double &pfr = fr[d * sj[0] + g * sj[1] + i * sj[2] + k * sj[3]];
            double &pbo = bo[d * sk[0] + g * sk[1] + i * sk[2] + j * sk[3]];
            double psi_dgz = (rhs[d * sr[0] + g * sr[1] + z * sr[2]] + plf * xcos_dxi + pfr * ycos_dyj + pbo * zcos_dzk) /
                             (xcos_dxi + ycos_dyj + zcos_dzk + sigt[g * ss[0] + z * ss[1]]);
            psi[d * sp[0] + g * sp[1] + z * sp[2]] = psi_dgz;
            plf = 2.0 * psi_dgz - plf;
            pfr = 2.0 * psi_dgz - pfr;
            pbo = 2.0 * psi_dgz - pbo;
          }
}

void zeroChunk(orc_problem &p, const char *name, int sdom) {
  Field &x = p.fld(name);
  auto &v = x.d[p.dc.chunkOf(x.space, sdom)];
  std::fill(v.begin(), v.end(), 0.0);
}

void kConstAll(orc_problem &p, const char *name, double value) {
  Field &x = p.fld(name);
  if (x.is_int) {
    for (auto &v : x.i) std::fill(v.begin(), v.end(), (int32_t)value);
  } else {
    for (auto &v : x.d) std::fill(v.begin(), v.end(), value);
  }
}

// SweepSolver.cpp:23-87 with the on-rank part of ParallelComm (dependency
// counts, ready list in queue order, plane copy to the downwind subdomain).
//
// With block_jacobi, BlockJacobiComm.cpp:23-98 instead: addSubdomain saves the
// planes into old_*_plane, and the first workRemaining() sends every queued
// subdomain's saved planes downwind (ParallelComm.cpp:146-162 copies them into
// the downwind subdomain's planes and drops its dependency count), after which
// every subdomain is ready and markComplete only dequeues.  The save follows
// kCopy's stated direction (old <- current); the reference's kCopy body
// (Kernel.h:60-72) assigns src = dst, which would instead fill the planes from
// the freshly allocated, unset old_*_plane storage.
void sweepSolver(orc_problem &p) {
  kConstAll(p, "i_plane", 0.0);
  kConstAll(p, "j_plane", 0.0);
  kConstAll(p, "k_plane", 0.0);
  std::vector<int> queue, depends;
  for (int s = 0; s < p.dc.num(); ++s) {
    int n = 0;
    for (int dim = 0; dim < 3; ++dim) if (p.upwind[s][dim] >= 0) ++n;
    queue.push_back(s);
    depends.push_back(n);
  }
  const char *planes[3] = {"i_plane", "j_plane", "k_plane"};
  if (p.block_jacobi) {
    std::vector<std::vector<double>> old[3];
    for (int dim = 0; dim < 3; ++dim) old[dim] = p.fld(planes[dim]).d;
    for (int s : std::vector<int>(queue)) {
      for (int dim = 0; dim < 3; ++dim) {
        int dn = p.downwind[s][dim];
        if (dn < 0) continue;
        for (size_t i = 0; i < queue.size(); ++i)
          if (queue[i] == dn) { depends[i]--; break; }
        Field &pl = p.fld(planes[dim]);
        pl.d[p.dc.chunkOf(pl.space, dn)] = old[dim][p.dc.chunkOf(pl.space, s)];
      }
    }
    while (!queue.empty()) {
      size_t idx = 0;
      while (idx < queue.size() && depends[idx] != 0) ++idx;
      if (idx == queue.size()) return;  // unreachable: every dependency was met by the sends
      int s = queue[idx];
      for (int dim = 0; dim < 3; ++dim)
        if (p.upwind[s][dim] == -1) zeroChunk(p, planes[dim], s);
      kSweep(p, s);
      queue.erase(queue.begin() + idx);
      depends.erase(depends.begin() + idx);
    }
    return;
  }
  while (!queue.empty()) {
    size_t idx = 0;
    while (idx < queue.size() && depends[idx] != 0) ++idx;
    if (idx == queue.size()) return;  // unreachable for a consistent DAG
    int s = queue[idx];
    for (int dim = 0; dim < 3; ++dim)
      if (p.upwind[s][dim] == -1) zeroChunk(p, planes[dim], s);
    kSweep(p, s);
    queue.erase(queue.begin() + idx);
    depends.erase(depends.begin() + idx);
    for (int dim = 0; dim < 3; ++dim) {
      int dn = p.downwind[s][dim];
      if (dn < 0) continue;
      for (size_t i = 0; i < queue.size(); ++i)
        if (queue[i] == dn) { depends[i]--; break; }
      Field &pl = p.fld(planes[dim]);
      pl.d[p.dc.chunkOf(pl.space, dn)] = pl.d[p.dc.chunkOf(pl.space, s)];
    }
  }
}

double kPopulation(orc_problem &p) {
  double part = 0.0;
  for (int sdom = 0; sdom < p.dc.num(); ++sdom) {
    const double *psi = p.dptr("psi", sdom), *w = p.dptr("quadrature/w", sdom), *vol = p.dptr("volume", sdom);
    const int64_t *sp = p.strd("psi", sdom);
    const int64_t Zs = (int64_t)p.nxs * p.nys * p.nzs;
    double red = 0.0;
#pragma omp parallel for collapse(2) schedule(static) reduction(+ : red) if (p.par())
    for (int d = 0; d < p.Ds; ++d)
      for (int g = 0; g < p.Gs; ++g)
        for (int64_t z = 0; z < Zs; ++z) red += w[d] * psi[d * sp[0] + g * sp[1] + z * sp[2]] * vol[z];
    part += red;
  }
  return part;
}

// Compensated sum (Neumaier): the balance adds up to 10^8 positive terms, where
// one running double would carry an error of order sqrt(n) ulps of the total.
struct CSum {
  double s = 0.0, c = 0.0;
  CSum &operator+=(double x) {
    const double t = s + x;
    c += std::fabs(s) >= std::fabs(x) ? (s - t) + x : (x - t) + s;
    s = t;
    return *this;
  }
  double value() const { return s + c; }
};

// Particle balance after a sweep (an extension of Kernel::population,
// Kernel/Population.cpp:51-63, to the emission, collision and leakage terms).
void kBalance(orc_problem &p, double out[5]) {
  CSum emis, coll, leak;
  const int64_t Zs = (int64_t)p.nxs * p.nys * p.nzs;
  for (int sdom = 0; sdom < p.dc.num(); ++sdom) {
    const double *psi = p.dptr("psi", sdom), *rhs = p.dptr("rhs", sdom), *w = p.dptr("quadrature/w", sdom);
    const double *vol = p.dptr("volume", sdom), *sigt = p.dptr("sigt_zonal", sdom);
    const int64_t *sp = p.strd("psi", sdom), *sr = p.strd("rhs", sdom), *ss = p.strd("sigt_zonal", sdom);
    for (int d = 0; d < p.Ds; ++d)
      for (int g = 0; g < p.Gs; ++g)
        for (int64_t z = 0; z < Zs; ++z) {
          emis += w[d] * rhs[d * sr[0] + g * sr[1] + z * sr[2]] * vol[z];
          coll += w[d] * sigt[g * ss[0] + z * ss[1]] * psi[d * sp[0] + g * sp[1] + z * sp[2]] * vol[z];
        }
    const double *cosv[3] = {p.dptr("quadrature/xcos", sdom), p.dptr("quadrature/ycos", sdom), p.dptr("quadrature/zcos", sdom)};
    const double *dxv = p.dptr("dx", sdom), *dyv = p.dptr("dy", sdom), *dzv = p.dptr("dz", sdom);
    const char *planes[3] = {"i_plane", "j_plane", "k_plane"};
    for (int dim = 0; dim < 3; ++dim) {
      if (p.downwind[sdom][dim] != -1) continue;
      const double *pl = p.dptr(planes[dim], sdom);
      const int64_t *st = p.strd(planes[dim], sdom);
      int na = dim == 0 ? p.nys : p.nxs, nb = dim == 2 ? p.nys : p.nzs;
      for (int d = 0; d < p.Ds; ++d)
        for (int g = 0; g < p.Gs; ++g)
          for (int b = 0; b < nb; ++b)
            for (int a = 0; a < na; ++a) {
              double area = dim == 0 ? dyv[a] * dzv[b] : (dim == 1 ? dxv[a] * dzv[b] : dxv[a] * dyv[b]);
              leak += w[d] * cosv[dim][d] * area * pl[d * st[0] + g * st[1] + a * st[2] + b * st[3]];
            }
    }
  }
  out[0] = emis.value();
  out[1] = coll.value();
  out[2] = leak.value();
  out[3] = kPopulation(p);
  out[4] = out[0] - out[1] - out[2];
}

}  // namespace

// ------------------------------ C interface --------------------------------
extern "C" {

void orc_default_input(orc_input *in) {
  std::memset(in, 0, sizeof(*in));
  in->nx = in->ny = in->nz = 16;
  in->num_directions = 96;
  in->num_groups = 32;
  in->legendre_order = 4;
  in->layout = 0;
  in->num_dirsets = 8;
  in->num_groupsets = 2;
  in->num_zonesets_dim[0] = in->num_zonesets_dim[1] = in->num_zonesets_dim[2] = 1;
  in->niter = 10;
  in->num_material_subsamples = 4;
  in->sigt[0] = 0.1; in->sigt[1] = 0.0001; in->sigt[2] = 0.1;
  in->sigs[0] = 0.05; in->sigs[1] = 0.00005; in->sigs[2] = 0.05;
  in->source_strength = 1.0;
  in->seed = 20261203ULL;
}

orc_problem *orc_create(const orc_input *in) {
  auto *p = new orc_problem();
  p->in = *in;
  try {
    if (!generate(*p)) { delete p; return nullptr; }
  } catch (const std::exception &e) {
    g_err = e.what();
    delete p;
    return nullptr;
  }
  return p;
}

void orc_destroy(orc_problem *p) { delete p; }
const char *orc_error(void) { return g_err.c_str(); }

void orc_set_block_jacobi(orc_problem *p, int on) { p->block_jacobi = on != 0; }

void orc_set_threads(orc_problem *p, int n) {
  p->threads = n;
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#endif
}

int32_t orc_num_sdoms(const orc_problem *p) { return p->dc.num(); }

int64_t orc_field_size(const orc_problem *p, const char *name) {
  auto it = p->f.find(name);
  if (it == p->f.end()) return -1;
  int64_t n = 0;
  for (size_t c = 0; c < it->second.dims.size(); ++c) n += it->second.chunkSize((int)c);
  return n;
}

int32_t orc_field_elem_bytes(const orc_problem *p, const char *name) {
  auto it = p->f.find(name);
  if (it == p->f.end()) return -1;
  return it->second.is_int ? 4 : 8;
}

int32_t orc_field_get(const orc_problem *p, const char *name, void *out) {
  auto it = p->f.find(name);
  if (it == p->f.end()) return -1;
  char *o = (char *)out;
  const Field &x = it->second;
  for (size_t c = 0; c < x.dims.size(); ++c) {
    size_t nb = x.chunkSize((int)c) * (x.is_int ? 4 : 8);
    std::memcpy(o, x.is_int ? (const void *)x.i[c].data() : (const void *)x.d[c].data(), nb);
    o += nb;
  }
  return 0;
}

int32_t orc_field_set(orc_problem *p, const char *name, const void *in) {
  auto it = p->f.find(name);
  if (it == p->f.end()) return -1;
  const char *s = (const char *)in;
  Field &x = it->second;
  for (size_t c = 0; c < x.dims.size(); ++c) {
    size_t nb = x.chunkSize((int)c) * (x.is_int ? 4 : 8);
    std::memcpy(x.is_int ? (void *)x.i[c].data() : (void *)x.d[c].data(), s, nb);
    s += nb;
  }
  return 0;
}

int32_t orc_sdom_info(const orc_problem *p, int32_t sdom, int32_t out[8]) {
  if (sdom < 0 || sdom >= p->dc.num()) return -1;
  auto c = p->dc.coord(sdom);
  out[0] = p->Ds; out[1] = p->Gs; out[2] = p->nxs; out[3] = p->nys; out[4] = p->nzs;
  out[5] = c[0] * p->Gs;  // group lower
  out[6] = c[1] * p->Ds;  // direction lower
  out[7] = p->M;
  return 0;
}

void orc_kconst(orc_problem *p, const char *name, double value) { kConstAll(*p, name, value); }
void orc_ltimes(orc_problem *p) { kLTimes(*p); }
void orc_lplustimes(orc_problem *p) { kLPlusTimes(*p); }
void orc_scattering(orc_problem *p) { kScattering(*p); }
void orc_source(orc_problem *p) { kSource(*p); }
void orc_sweep_subdomain(orc_problem *p, int32_t sdom) { kSweep(*p, sdom); }
void orc_sweep_solver(orc_problem *p) { sweepSolver(*p); }
double orc_population(orc_problem *p) { return kPopulation(*p); }
void orc_balance(orc_problem *p, double out[5]) { kBalance(*p, out); }

double orc_iterate(orc_problem *p) {
  kConstAll(*p, "phi", 0.0);
  kLTimes(*p);
  kConstAll(*p, "phi_out", 0.0);
  kScattering(*p);
  kSource(*p);
  kConstAll(*p, "rhs", 0.0);
  kLPlusTimes(*p);
  sweepSolver(*p);
  return kPopulation(*p);
}

int32_t orc_solve(orc_problem *p, int32_t niter, double *part) {
  auto t0 = std::chrono::steady_clock::now();
  kConstAll(*p, "psi", 0.0);
  for (int it = 0; it < niter; ++it) {
    double v = orc_iterate(p);
    if (part) part[it] = v;
  }
  p->last_solve_s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  return 0;
}

double orc_last_solve_seconds(const orc_problem *p) { return p->last_solve_s; }

}  // extern "C"
