// KripkeKernel.cpp -- Kripke::Kernel entry points and the solvers on the GB300 path.
//
// Each Kernel function keeps its reference signature (src/Kripke/Kernel.h:19-55)
// and timer name, looks up its operands by DataStore name, and forwards to the
// C ABI; the device owns the fields, so a call is one kernel launch sequence
// instead of a loop over subdomains.  Semantics follow the reference: LTimes,
// LPlusTimes and scattering accumulate, kConst zeroes, population returns the
// particle count.
#include <cstdio>

#include "KripkeCore.h"

namespace Kripke {

namespace {
Core::Gb300Context &gpu(Core::DataStore &ds) { return ds.getVariable<Core::Gb300Context>("gb300"); }

void deviceWrote(Core::DataStore &ds, const char *name) { ds.getVariable<Core::Field<double>>(name).markDeviceModified(); }
}  // namespace

namespace Kernel {

// src/Kripke/Kernel/LTimes.cpp:79-105
void LTimes(Core::DataStore &ds) {
  KRIPKE_TIMER(ds, LTimes);
  auto &g = gpu(ds);
  g.check(kgb_ltimes(g.ctx), "kgb_ltimes");
  g.check(kgb_sync(g.ctx), "kgb_sync");  // the timer measures the kernel, not its launch
  deviceWrote(ds, "phi");
}

// src/Kripke/Kernel/LPlusTimes.cpp:68-92
void LPlusTimes(Core::DataStore &ds) {
  KRIPKE_TIMER(ds, LPlusTimes);
  auto &g = gpu(ds);
  g.check(kgb_lplustimes(g.ctx), "kgb_lplustimes");
  g.check(kgb_sync(g.ctx), "kgb_sync");  // the timer measures the kernel, not its launch
  deviceWrote(ds, "rhs");
}

// src/Kripke/Kernel/Scattering.cpp:112-164
void scattering(Core::DataStore &ds) {
  KRIPKE_TIMER(ds, Scattering);
  auto &g = gpu(ds);
  g.check(kgb_scattering(g.ctx), "kgb_scattering");
  g.check(kgb_sync(g.ctx), "kgb_sync");  // the timer measures the kernel, not its launch
  deviceWrote(ds, "phi_out");
}

// src/Kripke/Kernel/Source.cpp:83-115 (strength 1.0, :98)
void source(Core::DataStore &ds) {
  KRIPKE_TIMER(ds, Source);
  auto &g = gpu(ds);
  g.check(kgb_source(g.ctx, 1.0), "kgb_source");
  g.check(kgb_sync(g.ctx), "kgb_sync");  // the timer measures the kernel, not its launch
  deviceWrote(ds, "phi_out");
}

// src/Kripke/Kernel/SweepSubdomain.cpp:115-124
void sweepSubdomain(Core::DataStore &ds, SdomId sdom_id) {
  KRIPKE_TIMER(ds, SweepSubdomain);
  auto &g = gpu(ds);
  g.check(kgb_sweep_subdomain(g.ctx, sdom_id), "kgb_sweep_subdomain");
  g.check(kgb_sync(g.ctx), "kgb_sync");  // the timer measures the kernel, not its launch
  for (const char *n : {"psi", "i_plane", "j_plane", "k_plane"}) deviceWrote(ds, n);
}

// src/Kripke/Kernel/Population.cpp:74-101
double population(Core::DataStore &ds) {
  KRIPKE_TIMER(ds, Population);
  auto &g = gpu(ds);
  double part = 0.0;
  g.check(kgb_population(g.ctx, &part), "kgb_population");
  return part;
}

// src/Kripke/Kernel.h:37-55
void kConst(Core::Field<double> &field, double value) {
  auto &g = field.context();
  g.check(kgb_field_fill(g.ctx, field.name().c_str(), value), "kgb_field_fill");
  field.markDeviceModified();
}

}  // namespace Kernel

// src/Kripke/SweepSolver.cpp:23-87: planes zeroed, vacuum boundaries cleared,
// subdomains swept in upwind order with the plane hand-off between zone sets,
// or, with block_jacobi (BlockJacobiComm.cpp), every subdomain from the zeroed
// planes with no hand-off.  The device schedules every subdomain of the list
// at once (all octants concurrently); a partial list is swept subdomain by
// subdomain.
void SweepSolver(Core::DataStore &ds, const std::vector<SdomId> &sdom_list, bool block_jacobi) {
  KRIPKE_TIMER(ds, SweepSolver);
  auto &g = gpu(ds);
  int64_t bj = 0;
  g.check(kgb_get_option(g.ctx, "block_jacobi", &bj), "kgb_get_option");
  if ((bj != 0) != block_jacobi) g.check(kgb_set_option(g.ctx, "block_jacobi", block_jacobi ? 1 : 0), "kgb_set_option");
  int32_t n = 0;
  g.check(kgb_num_subdomains(g.ctx, &n), "kgb_num_subdomains");
  if ((int)sdom_list.size() == n) {
    KRIPKE_TIMER(ds, SweepSubdomain);
    g.check(kgb_sweep_solver(g.ctx), "kgb_sweep_solver");
    g.check(kgb_sync(g.ctx), "kgb_sync");
  } else {
    for (const char *p : {"i_plane", "j_plane", "k_plane"}) Kernel::kConst(ds.getVariable<Core::Field<double>>(p), 0.0);
    for (SdomId s : sdom_list) Kernel::sweepSubdomain(ds, s);
  }
  for (const char *f : {"psi", "i_plane", "j_plane", "k_plane"}) deviceWrote(ds, f);
}

// src/Kripke/SteadyStateSolver.cpp:24-115
int SteadyStateSolver(Core::DataStore &ds, size_t max_iter, bool block_jacobi) {
  KRIPKE_TIMER(ds, Solve);
  printf("\nSteady State Solve\n==================\n\n");
  auto field = [&](const char *n) -> Core::Field<double> & { return ds.getVariable<Core::Field<double>>(n); };
  Kernel::kConst(field("psi"), 0.0);
  if (!ds.isVariableType<ParticleHistory>("particle_history")) ds.newVariable<ParticleHistory>("particle_history");
  auto &history = ds.getVariable<ParticleHistory>("particle_history");
  double part_last = 0.0;
  for (size_t iter = 0; iter < max_iter; ++iter) {
    Kernel::kConst(field("phi"), 0.0);
    Kernel::LTimes(ds);
    Kernel::kConst(field("phi_out"), 0.0);
    Kernel::scattering(ds);
    Kernel::source(ds);
    Kernel::kConst(field("rhs"), 0.0);
    Kernel::LPlusTimes(ds);
    {
      int32_t n = 0;
      auto &g = gpu(ds);
      g.check(kgb_num_subdomains(g.ctx, &n), "kgb_num_subdomains");
      std::vector<SdomId> list(n);
      for (int i = 0; i < n; ++i) list[i] = i;
      SweepSolver(ds, list, block_jacobi);
    }
    const double part = Kernel::population(ds);
    history.counts.push_back(part);
    printf("  iter %d: particle count=%e, change=%e\n", (int)iter, part, (part - part_last) / part);
    fflush(stdout);
    part_last = part;
  }
  printf("  Solver terminated\n");
  return 0;
}

}  // namespace Kripke
