// generate.cpp -- Kripke::generateProblem for kripke_gb300 (host C++).
//
// Produces the inputs of the source-iteration path the way the reference
// generator does (paths relative to the Kripke source tree) and hands them to
// the device through kgb_field_upload in Kripke's chunked host layout:
//   quadrature ........ Generate/Quadrature.cpp:46-76 (Gauss-Legendre by Newton),
//                       :192-310 (product set sorted by octant with std::sort,
//                       or the dummy S2 set), :140-183 (real Y_n^m), :424-455 (L, L+)
//   mesh/materials .... Generate/Space.cpp:105-330 (uniform mesh, 4^3 sub-sampled
//                       material fractions, mix elements), :333-363 (sigt_zonal)
//   scattering ........ Generate/Data.cpp:69-101 (diagonal P0 sigs)
// The reference's inputs must be reproduced bit for bit, so every formula keeps
// the reference's operation order.  Three generator options are new (the
// benchmark problems need them): the 100 cm cube geometry with only the first
// duct leg, seeded lower-triangular downscatter matrices (columns summing to
// the scattering ratio sigs/sigt times sigma_t), and a seeded +-20%
// per-(material, group) perturbation of sigma_t and sigma_s.  Random numbers:
// std::mt19937_64(seed), u = (x >> 11) * 2^-53, drawn first for the
// perturbation in (material, group, [t, s]) order, then for the downscatter
// matrices in (material, l, g, g' <= g) order.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "kgb.h"
#include "kgb_layout.h"

using namespace kgb;

namespace {

struct QPoint {
  double xcos, ycos, zcos, w;
  int id, jd, kd, octant;
};

// ---- angular set -----------------------------------------------------------
void gaussLegendreSet(int n, std::vector<double> &node, std::vector<double> &wt) {
  node.assign(n, 0.0);
  wt.assign(n, 0.0);
  const double xm = 0.5 * (1.0 + -1.0), xl = 0.5 * (1.0 - -1.0);
  for (int i = 1; i <= (n + 1) / 2; i++) {
    double z = cos(M_PI * (i - 0.25) / (n + 0.5));
    double z1, dp;
    do {
      double p0 = 1.0, pm1 = 0.0;  // P_j(z), P_{j-1}(z)
      for (int j = 1; j <= n; j++) {
        const double pm2 = pm1;
        pm1 = p0;
        p0 = ((2.0 * j - 1.0) * z * pm1 - (j - 1.0) * pm2) / j;
      }
      dp = n * (z * p0 - pm1) / (z * z - 1.0);
      z1 = z;
      z = z1 - p0 / dp;
    } while (fabs(z - z1) > DBL_EPSILON);
    node[i - 1] = xm - xl * z;
    node[n - i] = xm + xl * z;
    wt[i - 1] = 2.0 * xl / ((1.0 - z * z) * dp * dp);
    wt[n - i] = wt[i - 1];
  }
}

bool octantAfter(const QPoint &a, const QPoint &b) { return b.octant < a.octant; }

std::vector<QPoint> angularSet(const kgb_input &in) {
  std::vector<QPoint> pts(in.num_directions);
  if (in.quad_num_polar > 0) {
    std::vector<double> mu, wmu;
    gaussLegendreSet(in.quad_num_polar, mu, wmu);
    const int na = in.quad_num_azimuthal;
    const double dphi = 2.0 * M_PI / ((double)na);
    std::vector<double> phi(na);
    for (int j = 0; j < na; j++) phi[j] = (j == 0) ? dphi / 2.0 : phi[j - 1] + dphi;
    int d = 0;
    for (int i = 0; i < in.quad_num_polar; i++)
      for (int j = 0; j < na; j++, d++) {
        const double sx = sqrt(1.0 - mu[i] * mu[i]) * cos(phi[j]);
        const double sy = sqrt(1.0 - mu[i] * mu[i]) * sin(phi[j]);
        const double sz = mu[i];
        QPoint &q = pts[d];
        q.id = sx > 0. ? 1 : -1;
        q.jd = sy > 0. ? 1 : -1;
        q.kd = sz > 0. ? 1 : -1;
        q.octant = (q.id < 0 ? 1 : 0) | (q.jd < 0 ? 2 : 0) | (q.kd < 0 ? 4 : 0);
        q.xcos = std::abs(sx);
        q.ycos = std::abs(sy);
        q.zcos = std::abs(sz);
        q.w = wmu[i] * dphi;
      }
    std::sort(pts.begin(), pts.end(), octantAfter);  // same comparator and algorithm as the reference
  } else {
    const double mu = cos(M_PI / 4);
    const double eta = sqrt(1 - mu * mu) * cos(M_PI / 4);
    const double xi = sqrt(1 - mu * mu) * sin(M_PI / 4);
    const int per = in.num_directions / 8;
    for (int d = 0; d < in.num_directions; ++d) {
      const int oct = d / per;
      QPoint &q = pts[d];
      q.id = (oct & 1) ? 1 : -1;
      q.jd = (oct & 2) ? 1 : -1;
      q.kd = (oct & 4) ? 1 : -1;
      q.octant = 0;
      q.w = 4.0 * M_PI / (double)in.num_directions;
      q.xcos = mu;
      q.ycos = eta;
      q.zcos = xi;
    }
  }
  return pts;
}

double factorialD(int n) {
  double f = 1.0;
  for (int i = n; i > 0; --i) f *= (double)i;
  return f;
}

// P_n^m(x) for 0 <= m <= n by upward recurrence in n (with the Condon-Shortley phase)
double legendreP(int n, int m, double x) {
  double pmm = 1.0;
  if (m > 0) {
    const double s = sqrt((1.0 - x) * (1.0 + x));
    double f = 1.0;
    for (int i = 1; i <= m; i++) {
      pmm *= -f * s;
      f += 2.0;
    }
  }
  if (n == m) return pmm;
  double p1 = x * (2 * m + 1) * pmm;
  if (n == m + 1) return p1;
  double pn = 0;
  for (int k = m + 2; k <= n; k++) {
    pn = (x * (2 * k - 1) * p1 - (k + m - 1) * pmm) / (k - m);
    pmm = p1;
    p1 = pn;
  }
  return pn;
}

// real spherical harmonic at (mu, eta, xi); azimuth from atan(|eta/mu|) by quadrant
double sphHarm(int n, int m, double mu, double eta, double xi) {
  const double t = atan(fabs(eta / (mu + 1.e-20)));
  double az;
  if (mu > 0 && eta > 0) az = t;
  else if (mu < 0 && eta > 0) az = M_PI - fabs(t);
  else if (mu < 0 && eta < 0) az = M_PI + fabs(t);
  else az = 2.0 * M_PI - fabs(t);
  const int am = std::abs(m);
  const double f1 = factorialD(n - am), f2 = factorialD(n + am);
  const double p = legendreP(n, am, xi);
  const double ang = ((double)m) * az;
  const double tau = m >= 0 ? cos(ang) : sin(-ang);
  const double d0 = m == 0 ? 1.0 : 0.0;
  const double c = ((2 * n + 1) * f1) / (2.0 * (1.0 + d0) * M_PI * f2);
  return sqrt(c) * p * tau;
}

// ---- geometry ----------------------------------------------------------------
int materialAt(int geometry, double x, double y, double z) {
  if (geometry == 1) {
    if (x <= 10.0 && y <= 10.0 && z <= 10.0) return 0;
    if (x <= 10.0 && y <= 60.0 && z <= 10.0) return 1;
    return 2;
  }
  x = std::abs(x); y = std::abs(y); z = std::abs(z);
  if (x <= 10.0 && y <= 10.0 && z <= 10.0) return 0;
  if (x <= 10.0 && y <= 60.0 && z <= 10.0) return 1;
  if (x <= 40.0 && y >= 50.0 && y <= 60.0 && z <= 10.0) return 1;
  if (x >= 30.0 && x <= 40.0 && y >= 50.0 && y <= 60.0 && z <= 40.0) return 1;
  if (x >= 30.0 && x <= 40.0 && y >= 50.0 && z >= 30.0 && z <= 40.0) return 1;
  return 2;
}

double draw(std::mt19937_64 &r) { return (double)(r() >> 11) * 0x1.0p-53; }

// Per-material cross sections of the generator: sigma_t st[m][g], the
// isotropic in-group sigma_s ss[m][g], and the full scattering tables
// sg[m][l][g][g'] (destination g, source g').  All random draws of the
// generator happen here, in the documented order.
void materialTables(const kgb_input &in, std::vector<double> &st, std::vector<double> &ss, std::vector<double> &sg) {
  const int G = in.num_groups, L1 = in.legendre_order + 1;
  std::mt19937_64 rng(in.seed);
  st.assign((size_t)3 * G, 0.0);
  ss.assign((size_t)3 * G, 0.0);
  sg.assign((size_t)3 * L1 * G * G, 0.0);
  for (int m = 0; m < 3; ++m)
    for (int g = 0; g < G; ++g) {
      double ft = 1.0, fs = 1.0;
      if (in.perturb) {
        ft = 1.0 + 0.2 * (2.0 * draw(rng) - 1.0);
        fs = 1.0 + 0.2 * (2.0 * draw(rng) - 1.0);
      }
      st[m * G + g] = in.sigt[m] * ft;
      ss[m * G + g] = in.sigs[m] * fs;
    }
  auto at = [&](int m, int l, int g, int gp) -> double & { return sg[(((size_t)m * L1 + l) * G + g) * G + gp]; };
  if (in.scatter == 1) {
    std::vector<double> u((size_t)G * G);
    for (int m = 0; m < 3; ++m)
      for (int l = 0; l < L1; ++l) {
        // columns sum to c_m * sigma_t(m, g'), c_m = sigs[m] / sigt[m] (0.5 for the reference values)
        const double ratio = in.sigt[m] != 0.0 ? in.sigs[m] / in.sigt[m] : 0.0;
        std::fill(u.begin(), u.end(), 0.0);
        for (int g = 0; g < G; ++g)
          for (int gp = 0; gp <= g; ++gp) u[(size_t)g * G + gp] = draw(rng);
        for (int gp = 0; gp < G; ++gp) {
          double col = 0.0;
          for (int g = gp; g < G; ++g) col += u[(size_t)g * G + gp];
          const double scale = ratio * st[m * G + gp] / col;
          for (int g = gp; g < G; ++g) at(m, l, g, gp) = (u[(size_t)g * G + gp] * scale) / (double)(2 * l + 1);
        }
      }
  } else {
    for (int m = 0; m < 3; ++m)
      for (int g = 0; g < G; ++g) at(m, 0, g, g) = ss[m * G + g];
  }
}

struct Gen {
  kgb_ctx *ctx;
  const kgb_input &in;
  Decomp dc;
  int G, Gs, D, Ds, M, L, nxs, nys, nzs;
  int64_t Zs;

  Gen(kgb_ctx *c, const kgb_input &i) : ctx(c), in(i) {
    dc.SP = in.num_groupsets; dc.SQ = in.num_dirsets;
    dc.Sx = in.num_zonesets[0]; dc.Sy = in.num_zonesets[1]; dc.Sz = in.num_zonesets[2];
    G = in.num_groups; Gs = G / dc.SP;
    D = in.num_directions; Ds = D / dc.SQ;
    L = in.legendre_order; M = (L + 1) * (L + 1);
    nxs = in.nx / dc.Sx; nys = in.ny / dc.Sy; nzs = in.nz / dc.Sz;
    Zs = (int64_t)nxs * nys * nzs;
  }

  template <typename T>
  int put(const char *name, const std::vector<T> &v) {
    return kgb_field_upload(ctx, name, v.data(), (int64_t)(v.size() * sizeof(T)));
  }

  int run() {
    int rc;
    // per-(material, group) cross sections and scattering tables
    std::vector<double> st, ss, sgc;
    materialTables(in, st, ss, sgc);

    // --- angular data, one chunk per direction set ---
    std::vector<QPoint> pts = angularSet(in);
    {
      std::vector<double> xc(D), yc(D), zc(D), w(D);
      std::vector<int32_t> id(D), jd(D), kd(D);
      for (int d = 0; d < D; ++d) {  // Q chunks are contiguous direction ranges
        xc[d] = pts[d].xcos; yc[d] = pts[d].ycos; zc[d] = pts[d].zcos; w[d] = pts[d].w;
        id[d] = pts[d].id; jd[d] = pts[d].jd; kd[d] = pts[d].kd;
      }
      if ((rc = put("quadrature/xcos", xc)) || (rc = put("quadrature/ycos", yc)) || (rc = put("quadrature/zcos", zc)) ||
          (rc = put("quadrature/w", w)) || (rc = put("quadrature/id", id)) || (rc = put("quadrature/jd", jd)) ||
          (rc = put("quadrature/kd", kd)))
        return rc;
      std::vector<int32_t> m2l(M);
      for (int n = 0, nm = 0; n <= L; ++n)
        for (int m = -n; m <= n; ++m) m2l[nm++] = n;
      if ((rc = put("moment_to_legendre", m2l))) return rc;
      // L and L+ per direction set, in the host nesting
      const double SQRT4PI = std::sqrt(4 * M_PI);
      std::vector<double> ell((size_t)M * D), ellp((size_t)M * D);
      Idx te[2] = {I_MOM, I_DIR}, tp[2] = {I_DIR, I_MOM};
      int64_t de[2] = {M, Ds}, dp[2] = {Ds, M}, se[2], sp[2];
      nestStrides(in.layout, 2, te, de, se);
      nestStrides(in.layout, 2, tp, dp, sp);
      for (int q = 0; q < dc.SQ; ++q) {
        const size_t off = (size_t)q * M * Ds;
        int nm = 0;
        for (int n = 0; n <= L; n++)
          for (int m = -n; m <= n; m++, nm++)
            for (int d = 0; d < Ds; ++d) {
              const QPoint &pt = pts[q * Ds + d];
              const double y = sphHarm(n, m, (pt.id) * (pt.xcos), (pt.jd) * (pt.ycos), (pt.kd) * (pt.zcos));
              ell[off + nm * se[0] + d * se[1]] = pt.w * y / SQRT4PI;
              ellp[off + d * sp[0] + nm * sp[1]] = y * SQRT4PI;
            }
      }
      if ((rc = put("ell", ell)) || (rc = put("ell_plus", ellp))) return rc;
    }

    // --- mesh ---
    double x0g, x1g, y0g, y1g, z0g, z1g;
    if (in.geometry == 1) { x0g = 0.0; x1g = 100.0; y0g = 0.0; y1g = 100.0; z0g = 0.0; z1g = 100.0; }
    else { x0g = -60.0; x1g = 60.0; y0g = -100.0; y1g = 100.0; z0g = -60.0; z1g = 60.0; }
    const double dx = (x1g - x0g) / in.nx, dy = (y1g - y0g) / in.ny, dz = (z1g - z0g) / in.nz;
    if ((rc = put("dx", std::vector<double>(in.nx, dx))) || (rc = put("dy", std::vector<double>(in.ny, dy))) ||
        (rc = put("dz", std::vector<double>(in.nz, dz))))
      return rc;
    const double vol = dx * dy * dz;
    const int nr = dc.chunks(S_R);
    if ((rc = put("volume", std::vector<double>((size_t)nr * Zs, vol)))) return rc;

    // --- material fractions by sub-sampling, per zone set ---
    const int ns = in.num_material_subsamples;
    const double sfrac = 1.0 / (double)(ns * ns * ns);
    std::vector<int32_t> z2m((size_t)nr * Zs), z2n((size_t)nr * Zs), mz, mm;
    std::vector<double> mf;
    std::vector<int64_t> rmix_off(nr + 1, 0);
    for (int r = 0; r < nr; ++r) {
      int co[5];
      dc.chunkCoord(S_R, r, co);
      const double ox = x0g + dx * (co[2] * nxs), oy = y0g + dy * (co[3] * nys), oz = z0g + dz * (co[4] * nzs);
      int local = 0;
      for (int k = 0; k < nzs; k++)
        for (int j = 0; j < nys; j++)
          for (int i = 0; i < nxs; i++) {
            const int64_t z = ((int64_t)k * nys + j) * nxs + i;
            const double xi0 = ox + dx * i, yj0 = oy + dy * j, zk0 = oz + dz * k;
            double f[3] = {0.0, 0.0, 0.0};
            for (int a = 0; a < ns; ++a)
              for (int b = 0; b < ns; ++b)
                for (int c = 0; c < ns; ++c) {
                  const double x = xi0 + dx * (a + 1) / (ns + 1);
                  const double y = yj0 + dy * (b + 1) / (ns + 1);
                  const double zz = zk0 + dz * (c + 1) / (ns + 1);
                  f[materialAt(in.geometry, x, y, zz)] += sfrac;
                }
            z2m[(size_t)r * Zs + z] = local;
            int cnt = 0;
            for (int m = 0; m < 3; ++m)
              if (f[m] > 0.0) {
                mz.push_back((int32_t)z);
                mm.push_back(m);
                mf.push_back(f[m]);
                ++cnt;
                ++local;
              }
            z2n[(size_t)r * Zs + z] = cnt;
          }
      rmix_off[r + 1] = (int64_t)mf.size();
    }
    if ((rc = put("zone_to_num_mixelem", z2n)) || (rc = put("zone_to_mixelem", z2m)) ||
        (rc = put("mixelem_to_zone", mz)) || (rc = put("mixelem_to_material", mm)) ||
        (rc = put("mixelem_to_fraction", mf)))
      return rc;

    // --- sigt_zonal(g, z) = sum over the zone's mix elements of fraction * sigma_t ---
    {
      const int npr = dc.chunks(S_PR);
      std::vector<double> sz((size_t)npr * Gs * Zs, 0.0);
      Idx ts[2] = {I_GRP, I_ZONE};
      int64_t ds[2] = {Gs, Zs}, sst[2];
      nestStrides(in.layout, 2, ts, ds, sst);
      for (int c = 0; c < npr; ++c) {
        int co[5];
        dc.chunkCoord(S_PR, c, co);
        const int r = dc.rIndex(co);
        const size_t off = (size_t)c * Gs * Zs;
        for (int g = 0; g < Gs; ++g)
          for (int64_t e = rmix_off[r]; e < rmix_off[r + 1]; ++e)
            sz[off + g * sst[0] + (int64_t)mz[e] * sst[1]] += mf[e] * st[mm[e] * G + co[0] * Gs + g];
      }
      if ((rc = put("sigt_zonal", sz))) return rc;
    }

    // --- scattering matrices [mat][l][g][g'] in the host nesting ---
    {
      const int L1 = L + 1;
      std::vector<double> sg((size_t)3 * L1 * G * G, 0.0);
      Idx tg[4] = {I_MAT, I_LEG, I_GGRP, I_GGRP};
      int64_t dg[4] = {3, L1, G, G}, sgs[4];
      nestStrides(in.layout, 4, tg, dg, sgs);
      auto at = [&](int m, int l, int g, int gp) -> double & {
        return sg[m * sgs[0] + l * sgs[1] + g * sgs[2] + gp * sgs[3]];
      };
      for (int m = 0; m < 3; ++m)
        for (int l = 0; l < L1; ++l)
          for (int g = 0; g < G; ++g)
            for (int gp = 0; gp < G; ++gp) at(m, l, g, gp) = sgc[(((size_t)m * L1 + l) * G + g) * G + gp];
      if ((rc = put("data/sigs", sg))) return rc;
    }
    return KGB_OK;
  }
};

}  // namespace

extern "C" {

void kgb_default_input(kgb_input *in) {
  if (!in) return;
  std::memset(in, 0, sizeof(*in));
  in->nx = in->ny = in->nz = 16;
  in->num_directions = 96;
  in->num_groups = 32;
  in->legendre_order = 4;
  in->num_groupsets = 2;
  in->num_dirsets = 8;
  in->num_zonesets[0] = in->num_zonesets[1] = in->num_zonesets[2] = 1;
  in->layout = 0;
  in->precision = 0;
  in->num_material_subsamples = 4;
  in->seed = 20261203ULL;
  in->sigt[0] = 0.1; in->sigt[1] = 0.0001; in->sigt[2] = 0.1;
  in->sigs[0] = 0.05; in->sigs[1] = 0.00005; in->sigs[2] = 0.05;
}

int kgb_material_tables(const kgb_input *in, double *sigt, double *sigs) {
  if (!in || in->num_groups < 1 || in->legendre_order < 0 || in->scatter < 0 || in->scatter > 1) return KGB_ERR_ARG;
  std::vector<double> st, ss, sg;
  materialTables(*in, st, ss, sg);
  if (sigt) std::memcpy(sigt, st.data(), st.size() * sizeof(double));
  if (sigs) std::memcpy(sigs, sg.data(), sg.size() * sizeof(double));
  return KGB_OK;
}

int kgb_generate(kgb_ctx *ctx, const kgb_input *in) {
  if (!ctx || !in) return KGB_ERR_ARG;
  if (in->quad_num_polar > 0 &&
      (in->quad_num_polar % 4 || in->quad_num_azimuthal % 2 || in->quad_num_polar * in->quad_num_azimuthal != in->num_directions))
    return KGB_ERR_ARG;
  if (in->num_material_subsamples < 1 || in->geometry < 0 || in->geometry > 1 || in->scatter < 0 || in->scatter > 1)
    return KGB_ERR_ARG;
  kgb_dims d{};
  d.nx = in->nx; d.ny = in->ny; d.nz = in->nz;
  d.num_groups = in->num_groups;
  d.num_directions = in->num_directions;
  d.legendre_order = in->legendre_order;
  d.num_groupsets = in->num_groupsets;
  d.num_dirsets = in->num_dirsets;
  for (int k = 0; k < 3; ++k) d.num_zonesets[k] = in->num_zonesets[k];
  d.layout = in->layout;
  d.precision = in->precision;
  int rc = kgb_setup(ctx, &d);
  if (rc) return rc;
  Gen gen(ctx, *in);
  return gen.run();
}

}  // extern "C"
