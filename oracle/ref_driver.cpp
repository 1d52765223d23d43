/*
 * ref_driver.cpp -- a C interface over the REFERENCE's own code (Kripke's generator, Kernel::*
 * functions, SweepSolver and SteadyStateSolver, compiled from its sources against the stand-in
 * RAJA in oracle/refshim/), mirroring the oracle's orc_* interface so that tests can hold the
 * oracle to the reference on the same inputs.
 *
 * TEST INFRASTRUCTURE ONLY.  Built by oracle/ref_build.sh into oracle/_ref/ in a tree where the
 * reference sources are present; the product never loads it.
 *
 * Fields cross this interface exactly as the oracle moves them: the concatenation of a field's
 * chunks in chunk order (Core/DomainVar.cpp:15-39), each chunk in the problem's nesting.
 * Typed-index fields (zone_to_mixelem, mixelem_to_zone, mixelem_to_material,
 * moment_to_legendre) cross as int32, like the oracle's.
 */
#include <Kripke.h>
#include <Kripke/Core/DataStore.h>
#include <Kripke/Core/Field.h>
#include <Kripke/Generate.h>
#include <Kripke/InputVariables.h>
#include <Kripke/Kernel.h>
#include <Kripke/SteadyStateSolver.h>
#include <Kripke/SweepSolver.h>
#include <Kripke/VarTypes.h>

#include <fcntl.h>
#include <unistd.h>

#include <cstdint>
#include <cstring>
#include <exception>
#include <string>
#include <vector>

#include "kripke_oracle.h"

using namespace Kripke;
using namespace Kripke::Core;

namespace {

std::string g_error;

/* stdout of the reference (banner lines, per-iteration printout) goes to /dev/null while quiet */
struct Quiet {
  int saved = -1;
  explicit Quiet(bool on) {
    if (!on) return;
    fflush(stdout);
    saved = dup(1);
    int devnull = open("/dev/null", O_WRONLY);
    if (devnull >= 0) {
      dup2(devnull, 1);
      close(devnull);
    }
  }
  ~Quiet() {
    if (saved < 0) return;
    fflush(stdout);
    dup2(saved, 1);
    close(saved);
  }
};

}  // namespace

struct ref_problem {
  Kripke::Core::DataStore ds;
  bool quiet = true;
  bool block_jacobi = false;
};

namespace {

template <typename T>
FieldStorage<T> *storage(ref_problem *p, const char *name) {
  if (!p->ds.isVariableType<FieldStorage<T>>(name)) return nullptr;
  return &p->ds.getVariable<FieldStorage<T>>(name);
}

/* element kind: 0 double, 1 int, 2..5 typed index (8-byte value crossing as int32) */
int field_kind(ref_problem *p, const char *name) {
  if (storage<double>(p, name)) return 0;
  if (storage<int>(p, name)) return 1;
  if (storage<MixElem>(p, name)) return 2;
  if (storage<Material>(p, name)) return 3;
  if (storage<Zone>(p, name)) return 4;
  if (storage<Legendre>(p, name)) return 5;
  return -1;
}

template <typename T>
int64_t total_size(FieldStorage<T> *f) {
  int64_t n = 0;
  for (SdomId s : f->getWorkList()) n += (int64_t)f->size(s);
  return n;
}

template <typename T, typename Out, typename Conv>
void copy_out(FieldStorage<T> *f, Out *out, Conv conv) {
  for (SdomId s : f->getWorkList()) {
    T const *src = f->getData(s);
    size_t n = f->size(s);
    for (size_t i = 0; i < n; ++i) *out++ = conv(src[i]);
  }
}

template <typename T, typename In, typename Conv>
void copy_in(FieldStorage<T> *f, In const *in, Conv conv) {
  for (SdomId s : f->getWorkList()) {
    T *dst = f->getData(s);
    size_t n = f->size(s);
    for (size_t i = 0; i < n; ++i) dst[i] = conv(*in++);
  }
}

template <typename F>
int32_t guarded(F &&fn) {
  try {
    fn();
    return 0;
  } catch (std::exception const &e) {
    g_error = e.what();
    return -1;
  }
}

}  // namespace

extern "C" {

const char *ref_error(void) { return g_error.c_str(); }

/* Builds InputVariables (InputVariables.h:18-49) from the oracle's input record and runs
 * Kripke::generateProblem.  The record's extensions beyond the reference generator (the cube
 * geometry, seeded downscatter, perturbation, a source strength other than 1) are refused: the
 * caller writes such data into the fields instead. */
ref_problem *ref_create(const orc_input *in) {
  if (in->geometry != 0 || in->scatter != 0 || in->perturb != 0 || in->source_strength != 1.0) {
    g_error = "the reference generator has only the Kobayashi geometry, diagonal P0 sigs, no perturbation "
              "and unit source strength";
    return nullptr;
  }
  if (in->layout < 0 || in->layout > 5) {
    g_error = "layout must be 0..5";
    return nullptr;
  }
  InputVariables vars;
  vars.nx = in->nx;
  vars.ny = in->ny;
  vars.nz = in->nz;
  vars.num_directions = in->num_directions;
  vars.num_groups = in->num_groups;
  vars.legendre_order = in->legendre_order;
  vars.quad_num_polar = in->quad_num_polar;
  vars.quad_num_azimuthal = in->quad_num_azimuthal;
  vars.al_v = ArchLayoutV{ArchV_Sequential, (LayoutV)in->layout};
  vars.num_dirsets = in->num_dirsets;
  vars.num_groupsets = in->num_groupsets;
  for (int d = 0; d < 3; ++d) vars.num_zonesets_dim[d] = in->num_zonesets_dim[d];
  vars.niter = in->niter;
  vars.num_material_subsamples = in->num_material_subsamples;
  for (int m = 0; m < 3; ++m) {
    vars.sigt[m] = in->sigt[m];
    vars.sigs[m] = in->sigs[m];
  }
  ref_problem *p = new ref_problem();
  {
    Quiet q(true);
    if (vars.checkValues()) {
      g_error = "InputVariables::checkValues rejected the input";
      delete p;
      return nullptr;
    }
    Kripke::generateProblem(p->ds, vars);
  }
  return p;
}

void ref_destroy(ref_problem *p) { delete p; }

void ref_set_quiet(ref_problem *p, int on) { p->quiet = on != 0; }
void ref_set_block_jacobi(ref_problem *p, int on) { p->block_jacobi = on != 0; }

int64_t ref_field_size(ref_problem *p, const char *name) {
  switch (field_kind(p, name)) {
    case 0: return total_size(storage<double>(p, name));
    case 1: return total_size(storage<int>(p, name));
    case 2: return total_size(storage<MixElem>(p, name));
    case 3: return total_size(storage<Material>(p, name));
    case 4: return total_size(storage<Zone>(p, name));
    case 5: return total_size(storage<Legendre>(p, name));
    default: return -1;
  }
}

int32_t ref_field_elem_bytes(ref_problem *p, const char *name) {
  int k = field_kind(p, name);
  return k < 0 ? -1 : (k == 0 ? 8 : 4);
}

int32_t ref_field_get(ref_problem *p, const char *name, void *out) {
  auto d = [](double v) { return v; };
  auto i = [](int v) { return (int32_t)v; };
  auto t = [](auto v) { return (int32_t)*v; };
  switch (field_kind(p, name)) {
    case 0: copy_out(storage<double>(p, name), (double *)out, d); return 0;
    case 1: copy_out(storage<int>(p, name), (int32_t *)out, i); return 0;
    case 2: copy_out(storage<MixElem>(p, name), (int32_t *)out, t); return 0;
    case 3: copy_out(storage<Material>(p, name), (int32_t *)out, t); return 0;
    case 4: copy_out(storage<Zone>(p, name), (int32_t *)out, t); return 0;
    case 5: copy_out(storage<Legendre>(p, name), (int32_t *)out, t); return 0;
    default: g_error = std::string("unknown field ") + name; return -1;
  }
}

int32_t ref_field_set(ref_problem *p, const char *name, const void *in) {
  auto d = [](double v) { return v; };
  auto i = [](int32_t v) { return (int)v; };
  switch (field_kind(p, name)) {
    case 0: copy_in(storage<double>(p, name), (const double *)in, d); return 0;
    case 1: copy_in(storage<int>(p, name), (const int32_t *)in, i); return 0;
    case 2: copy_in(storage<MixElem>(p, name), (const int32_t *)in, [](int32_t v) { return MixElem(v); }); return 0;
    case 3: copy_in(storage<Material>(p, name), (const int32_t *)in, [](int32_t v) { return Material(v); }); return 0;
    case 4: copy_in(storage<Zone>(p, name), (const int32_t *)in, [](int32_t v) { return Zone(v); }); return 0;
    case 5: copy_in(storage<Legendre>(p, name), (const int32_t *)in, [](int32_t v) { return Legendre(v); }); return 0;
    default: g_error = std::string("unknown field ") + name; return -1;
  }
}

/* Kernel::kConst (Kernel.h:37-55) on a field of doubles */
int32_t ref_kconst(ref_problem *p, const char *name, double value) {
  FieldStorage<double> *f = storage<double>(p, name);
  if (!f) {
    g_error = std::string("not a field of doubles: ") + name;
    return -1;
  }
  Kripke::Kernel::kConst(*f, value);
  return 0;
}

int32_t ref_ltimes(ref_problem *p) { return guarded([&] { Kripke::Kernel::LTimes(p->ds); }); }
int32_t ref_lplustimes(ref_problem *p) { return guarded([&] { Kripke::Kernel::LPlusTimes(p->ds); }); }
int32_t ref_scattering(ref_problem *p) { return guarded([&] { Kripke::Kernel::scattering(p->ds); }); }
int32_t ref_source(ref_problem *p) { return guarded([&] { Kripke::Kernel::source(p->ds); }); }
int32_t ref_sweep_subdomain(ref_problem *p, int32_t sdom) {
  return guarded([&] { Kripke::Kernel::sweepSubdomain(p->ds, SdomId{sdom}); });
}

/* Kripke::SweepSolver over every subdomain, as SteadyStateSolver.cpp:82-92 calls it */
int32_t ref_sweep_solver(ref_problem *p) {
  return guarded([&] {
    PartitionSpace &pspace = p->ds.getVariable<PartitionSpace>("pspace");
    int n = (int)pspace.getNumSubdomains(SPACE_PQR);
    std::vector<SdomId> sdoms;
    for (SdomId i{0}; i < n; ++i) sdoms.push_back(i);
    Kripke::SweepSolver(p->ds, sdoms, p->block_jacobi);
  });
}

double ref_population(ref_problem *p) { return Kripke::Kernel::population(p->ds); }

int32_t ref_num_sdoms(ref_problem *p) {
  return (int32_t)p->ds.getVariable<PartitionSpace>("pspace").getNumSubdomains(SPACE_PQR);
}

/* Kripke::SteadyStateSolver (SteadyStateSolver.cpp:24-115) for niter iterations from psi = 0;
 * returns the population of the final iterate (the solver prints each one only with %e). */
int32_t ref_solve(ref_problem *p, int32_t niter, double *population) {
  return guarded([&] {
    {
      Quiet q(p->quiet);
      Kripke::SteadyStateSolver(p->ds, (size_t)niter, p->block_jacobi);
    }
    if (population) *population = Kripke::Kernel::population(p->ds);
  });
}

}  // extern "C"
