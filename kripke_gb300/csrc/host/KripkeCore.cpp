// KripkeCore.cpp -- input variables, arch/layout names, the GB300 context
// variable, timers and problem generation for the kripke driver.
#include <nvtx3/nvToolsExt.h>
#include <strings.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstring>

#include "KripkeCore.h"

namespace Kripke {

std::string archToString(ArchV a) { return a == ArchV_GB300 ? "GB300" : "unknown"; }

ArchV stringToArch(const std::string &s) {
  // the reference's CUDA arch name selects the GPU path too
  if (!strcasecmp(s.c_str(), "GB300") || !strcasecmp(s.c_str(), "CUDA")) return ArchV_GB300;
  return ArchV_Unknown;
}

static const char *kLayoutNames[] = {"DGZ", "DZG", "GDZ", "GZD", "ZDG", "ZGD"};

std::string layoutToString(LayoutV l) { return (l >= 0 && l < LayoutV_num_values) ? kLayoutNames[l] : "unknown"; }

LayoutV stringToLayout(const std::string &s) {
  for (int l = 0; l < LayoutV_num_values; ++l)
    if (!strcasecmp(kLayoutNames[l], s.c_str())) return (LayoutV)l;
  return LayoutV_Unknown;
}

// Defaults of src/Kripke/InputVariables.cpp:17-47.
InputVariables::InputVariables()
    : nx(16), ny(16), nz(16), num_directions(96), num_groups(32), legendre_order(4), quad_num_polar(0),
      quad_num_azimuthal(0), al_v{ArchV_GB300, LayoutV_DGZ}, npx(1), npy(1), npz(1), num_dirsets(8),
      num_groupsets(2), niter(10), parallel_method(PMETHOD_SWEEP), num_material_subsamples(4), run_name("kripke"),
      geometry(0), scatter(0), perturb(0), seed(20261203ULL), precision(KGB_FP64), autotune(false), json(false) {
  num_zonesets_dim[0] = num_zonesets_dim[1] = num_zonesets_dim[2] = 1;
  sigt[0] = 0.1; sigt[1] = 0.0001; sigt[2] = 0.1;
  sigs[0] = 0.05; sigs[1] = 0.00005; sigs[2] = 0.05;
}

// Checks of src/Kripke/InputVariables.cpp:52-109, plus the single-rank limits.
bool InputVariables::checkValues() const {
  if (num_zonesets_dim[0] <= 0 || num_zonesets_dim[1] <= 0 || num_zonesets_dim[2] <= 0) {
    printf("Number of zone-sets in each dim need to be greater than or equal to 1\n");
    return true;
  }
  if (num_groups < 1) {
    printf("Number of groups (%d) needs to be at least 1\n", num_groups);
    return true;
  }
  if (num_groups % num_groupsets) {
    printf("Number of groups (%d) must be evenly divided by number of groupsets (%d)\n", num_groups, num_groupsets);
    return true;
  }
  if (num_directions < 8) {
    printf("Number of directions (%d) needs to be at least 8\n", num_directions);
    return true;
  }
  if (num_dirsets % 8 && num_dirsets < 8) {
    printf("Number of direction sets (%d) must be a multiple of 8\n", num_dirsets);
    return true;
  }
  if (num_directions % num_dirsets) {
    printf("Number of directions (%d) must be evenly divided by number of directionsets(%d)\n", num_directions,
           num_dirsets);
    return true;
  }
  if (legendre_order < 0) {
    printf("Legendre scattering order (%d) must be >= 0\n", legendre_order);
    return true;
  }
  if (niter < 1) {
    printf("You must run at least one iteration (%d)\n", niter);
    return true;
  }
  if (npx * npy * npz != 1) {
    printf("This build runs one rank on one GPU (--procs 1,1,1)\n");
    return true;
  }
  if (al_v.arch_v == ArchV_Unknown) {
    printf("Unknown architecture: this build runs the GB300 GPU path (--arch GB300)\n");
    return true;
  }
  if (al_v.layout_v == LayoutV_Unknown) {
    printf("Unknown data layout\n");
    return true;
  }
  return false;
}

namespace Core {

Gb300Context::Gb300Context(int device) {
  const int rc = kgb_ctx_create(device, &ctx);
  if (rc != KGB_OK) throw std::runtime_error("cannot create a GB300 context on device " + std::to_string(device));
}

Gb300Context::~Gb300Context() {
  if (ctx) kgb_ctx_destroy(ctx);
}

void Gb300Context::check(int rc, const char *what) const {
  if (rc != KGB_OK) throw std::runtime_error(std::string(what) + ": " + kgb_last_error(ctx));
}

}  // namespace Core

static double nowSeconds() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// Every KRIPKE_TIMER region is also an NVTX range of the same name (the
// reference opens a Caliper region there, src/Kripke/Timing.h:86-115).
void Timing::start(const std::string &name) {
  nvtxRangePushA(name.c_str());
  T &t = timers_[name];
  t.t0 = nowSeconds();
  t.running = true;
  ++t.count;
}

void Timing::stop(const std::string &name) {
  T &t = timers_[name];
  if (t.running) {
    t.elapsed += nowSeconds() - t.t0;
    t.running = false;
    nvtxRangePop();
  }
}

double Timing::getTotal(const std::string &name) const {
  auto it = timers_.find(name);
  return it == timers_.end() ? 0.0 : it->second.elapsed;
}

size_t Timing::getCount(const std::string &name) const {
  auto it = timers_.find(name);
  return it == timers_.end() ? 0 : it->second.count;
}

// Same table and machine-readable lines as src/Kripke/Timing.cpp:45-96.
void Timing::print() const {
  printf("\nTimers\n======\n\n");
  printf("  %-16s  %12s  %12s\n", "Timer", "Count", "Seconds");
  printf("  ----------------  ------------  ------------\n");
  for (auto &kv : timers_) printf("  %-16s  %12d  %12.5lf\n", kv.first.c_str(), (int)kv.second.count, kv.second.elapsed);
  printf("\nTIMER_NAMES:");
  bool first = true;
  for (auto &kv : timers_) {
    printf("%s%s", first ? "" : ",", kv.first.c_str());
    first = false;
  }
  printf("\nTIMER_DATA:");
  first = true;
  for (auto &kv : timers_) {
    printf("%s%lf", first ? "" : ",", kv.second.elapsed);
    first = false;
  }
  printf("\n");
}

// Field names the GB300 context holds (Kripke's DataStore names).
static const char *kDoubleFields[] = {"psi", "rhs", "phi", "phi_out", "i_plane", "j_plane", "k_plane", "ell",
                                      "ell_plus", "sigt_zonal", "data/sigs", "quadrature/xcos", "quadrature/ycos",
                                      "quadrature/zcos", "quadrature/w", "dx", "dy", "dz", "volume",
                                      "mixelem_to_fraction"};
static const char *kIntFields[] = {"quadrature/id", "quadrature/jd", "quadrature/kd", "zone_to_mixelem",
                                   "zone_to_num_mixelem", "mixelem_to_zone", "mixelem_to_material",
                                   "moment_to_legendre"};

void generateProblem(Core::DataStore &ds, const InputVariables &vars) {
  printf("\nGenerating Problem\n==================\n\n");
  ds.addVariable("timing", new Timing());
  KRIPKE_TIMER(ds, Generate);
  auto &al = ds.newVariable<ArchLayout>("al");
  al.al_v = vars.al_v;
  auto &g = ds.newVariable<Core::Gb300Context>("gb300", 0);

  kgb_input in;
  kgb_default_input(&in);
  in.nx = vars.nx; in.ny = vars.ny; in.nz = vars.nz;
  in.num_directions = vars.num_directions;
  in.num_groups = vars.num_groups;
  in.legendre_order = vars.legendre_order;
  in.quad_num_polar = vars.quad_num_polar;
  in.quad_num_azimuthal = vars.quad_num_azimuthal;
  in.num_groupsets = vars.num_groupsets;
  in.num_dirsets = vars.num_dirsets;
  for (int k = 0; k < 3; ++k) in.num_zonesets[k] = vars.num_zonesets_dim[k];
  in.layout = (int)vars.al_v.layout_v;
  in.precision = vars.precision;
  in.num_material_subsamples = vars.num_material_subsamples;
  in.geometry = vars.geometry;
  in.scatter = vars.scatter;
  in.perturb = vars.perturb;
  in.seed = vars.seed;
  for (int m = 0; m < 3; ++m) {
    in.sigt[m] = vars.sigt[m];
    in.sigs[m] = vars.sigs[m];
  }
  g.check(kgb_generate(g.ctx, &in), "kgb_generate");

  // sets of the decomposition (src/Kripke/Generate/*.cpp)
  const int G = vars.num_groups, D = vars.num_directions, M = (vars.legendre_order + 1) * (vars.legendre_order + 1);
  const int SP = vars.num_groupsets, SQ = vars.num_dirsets;
  const int SX = vars.num_zonesets_dim[0], SY = vars.num_zonesets_dim[1], SZ = vars.num_zonesets_dim[2];
  const int ns = SP * SQ * SX * SY * SZ;
  std::vector<size_t> gs(ns), gl(ns), dsz(ns), dl(ns), zs(ns, (size_t)(vars.nx / SX) * (vars.ny / SY) * (vars.nz / SZ));
  for (int s = 0; s < ns; ++s) {
    const int p = s / (SQ * SX * SY * SZ), q = (s / (SX * SY * SZ)) % SQ;
    gs[s] = G / SP; gl[s] = (size_t)p * (G / SP);
    dsz[s] = D / SQ; dl[s] = (size_t)q * (D / SQ);
  }
  ds.addVariable("Set/Group", new Core::Set(gs, gl, G));
  ds.addVariable("Set/Direction", new Core::Set(dsz, dl, D));
  ds.addVariable("Set/Zone", new Core::Set(zs, std::vector<size_t>(ns, 0), (size_t)vars.nx * vars.ny * vars.nz));
  ds.addVariable("Set/Moment", new Core::Set({(size_t)M}, {0}, M));
  for (const char *n : kDoubleFields) ds.addVariable(n, new Core::Field<double>(g, n));
  for (const char *n : kIntFields) ds.addVariable(n, new Core::Field<int32_t>(g, n));

  // field memory table (src/Kripke/Generate.cpp:58-93)
  std::vector<std::string> names(std::begin(kDoubleFields), std::end(kDoubleFields));
  std::sort(names.begin(), names.end());
  printf("  Memory breakdown of Field variables:\n");
  printf("  Field Variable            Num Elements    Megabytes\n");
  printf("  --------------            ------------    ---------\n");
  unsigned long total = 0;
  for (auto &n : names) {
    int64_t nb = 0;
    g.check(kgb_field_bytes(g.ctx, n.c_str(), &nb), "kgb_field_bytes");
    const unsigned long ne = (unsigned long)(nb / 8);
    total += ne;
    printf("  %-24s  %12lu %12.3lf\n", n.c_str(), ne, (double)ne * 8.0 / 1024.0 / 1024.0);
  }
  printf("  --------                  ------------    ---------\n");
  printf("  TOTAL                     %12lu %12.3lf\n", total, (double)total * 8.0 / 1024.0 / 1024.0);
  printf("\n  Generation Complete!\n");
}

}  // namespace Kripke
