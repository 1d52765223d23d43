// kripke.cpp -- the command-line driver on the GB300 path.
//
// Same flags, defaults, printed sections and figures of merit as the
// reference driver (src/kripke.cpp:36-526); --arch selects GB300 (the
// reference's "CUDA" is accepted as a synonym).  Added flags select the
// benchmark generator options and the precision form:
//   --geometry kobayashi|cube   --scatter diag|down   --perturb   --seed N
//   --precision fp64|mixed      --autotune            --json
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <sstream>
#include <string>
#include <vector>

#include "KripkeCore.h"

using namespace Kripke;

namespace {

void usage() {
  InputVariables def;
  printf("Usage:  kripke [options...]\n\n");
  printf("Problem Size Options:\n---------------------\n");
  printf("  --groups <ngroups>     Number of energy groups\n                         Default:  --groups %d\n\n", def.num_groups);
  printf("  --legendre <lorder>    Scattering Legendre Expansion Order (0, 1, ...)\n                         Default:  --legendre %d\n\n", def.legendre_order);
  printf("  --quad [<ndirs>|<polar>:<azim>]\n                         Define the quadrature set to use\n"
         "                         Either a fake S2 with <ndirs> points,\n"
         "                         OR Gauss-Legendre with <polar> by <azim> points\n"
         "                         Default:  --quad %d\n\n", def.num_directions);
  printf("  --zones <x,y,z>        Number of zones in x,y,z\n                         Default:  --zones %d,%d,%d\n\n", def.nx, def.ny, def.nz);
  printf("\nPhysics Parameters:\n-------------------\n");
  printf("  --sigt <st0,st1,st2>   Total material cross-sections\n                         Default:   --sigt %lf,%lf,%lf\n\n", def.sigt[0], def.sigt[1], def.sigt[2]);
  printf("  --sigs <ss0,ss1,ss2>   Scattering material cross-sections\n                         Default:   --sigs %lf,%lf,%lf\n\n", def.sigs[0], def.sigs[1], def.sigs[2]);
  printf("  --geometry <g>         kobayashi (default) or cube (100 cm cube, first duct leg)\n");
  printf("  --scatter <s>          diag (default, P0 diagonal) or down (seeded lower-triangular)\n");
  printf("  --perturb              seeded +-20%% per (material, group) on sigma_t and sigma_s\n");
  printf("  --seed <n>             generator seed (default 20261203)\n\n");
  printf("\nOn-Node Options:\n----------------\n");
  printf("  --arch <ARCH>          Architecture selection\n                         Available: GB300 (CUDA is a synonym)\n                         Default:   --arch GB300\n\n");
  printf("  --layout <LAYOUT>      Data layout and loop nesting order\n                         Available: DGZ,DZG,GDZ,GZD,ZDG,ZGD\n                         Default:   --layout DGZ\n\n");
  printf("  --precision <p>        fp64 (default, the drop-in) or mixed\n");
  printf("  --autotune             pick sweep tiles and moment kernels by measurement before solving\n");
  printf("  --json                 also print one JSON line with the figures of merit\n\n");
  printf("\nParallel Decomposition Options:\n-------------------------------\n");
  printf("  --procs <npx,npy,npz>  Number of MPI ranks in each spatial dimension\n                         Default:  --procs 1,1,1 (this build: one rank)\n\n");
  printf("  --dset <ds>            Number of direction-sets\n                         Default:  --dset %d\n\n", def.num_dirsets);
  printf("  --gset <gs>            Number of energy group-sets\n                         Default:  --gset %d\n\n", def.num_groupsets);
  printf("  --zset <zx>,<zy>,<zz>  Number of zone-sets in x,y, and z\n                         Default:  --zset 1,1,1\n\n");
  printf("\nSolver Options:\n---------------\n");
  printf("  --niter <NITER>        Number of solver iterations to run\n                         Default:  --niter %d\n\n", def.niter);
  printf("  --pmethod <method>     Parallel solver method\n");
  printf("                         sweep: Full up-wind sweep (wavefront algorithm)\n");
  printf("                         bj: Block Jacobi\n");
  printf("                         Default: --pmethod sweep\n\n");
  exit(1);
}

std::vector<std::string> split(const std::string &s, char d) {
  std::vector<std::string> out;
  std::stringstream ss(s);
  std::string item;
  while (std::getline(ss, item, d)) out.push_back(item);
  return out;
}

}  // namespace

int main(int argc, char **argv) {
  printf("\n   _  __       _         _\n  | |/ /      (_)       | |\n  | ' /  _ __  _  _ __  | | __ ___\n"
         "  |  <  | '__|| || '_ \\ | |/ // _ \\ \n  | . \\ | |   | || |_) ||   <|  __/\n"
         "  |_|\\_\\|_|   |_|| .__/ |_|\\_\\\\___|\n                 | |\n                 |_|        %s\n\n",
         kgb_version());

  InputVariables vars;
  std::vector<std::string> args(argv + 1, argv + argc);
  size_t a = 0;
  auto pop = [&]() -> std::string {
    if (a >= args.size()) usage();
    return args[a++];
  };
  while (a < args.size()) {
    const std::string opt = pop();
    if (opt == "-h" || opt == "--help") usage();
    else if (opt == "--name") vars.run_name = pop();
    else if (opt == "--dset") vars.num_dirsets = std::atoi(pop().c_str());
    else if (opt == "--gset") vars.num_groupsets = std::atoi(pop().c_str());
    else if (opt == "--zset" || opt == "--zones" || opt == "--procs") {
      auto v = split(pop(), ',');
      if (v.size() != 3) usage();
      int *dst = opt == "--zset" ? vars.num_zonesets_dim : nullptr;
      const int x = std::atoi(v[0].c_str()), y = std::atoi(v[1].c_str()), z = std::atoi(v[2].c_str());
      if (dst) { dst[0] = x; dst[1] = y; dst[2] = z; }
      else if (opt == "--zones") { vars.nx = x; vars.ny = y; vars.nz = z; }
      else { vars.npx = x; vars.npy = y; vars.npz = z; }
    } else if (opt == "--pmethod") {
      const std::string m = pop();
      if (m == "sweep") vars.parallel_method = PMETHOD_SWEEP;
      else if (m == "bj") vars.parallel_method = PMETHOD_BJ;
      else usage();
    } else if (opt == "--groups") vars.num_groups = std::atoi(pop().c_str());
    else if (opt == "--quad") {
      auto p = split(pop(), ':');
      if (p.size() == 1) {
        vars.num_directions = std::atoi(p[0].c_str());
        vars.quad_num_polar = vars.quad_num_azimuthal = 0;
      } else if (p.size() == 2) {
        vars.quad_num_polar = std::atoi(p[0].c_str());
        vars.quad_num_azimuthal = std::atoi(p[1].c_str());
        vars.num_directions = vars.quad_num_polar * vars.quad_num_azimuthal;
      } else usage();
    } else if (opt == "--legendre") vars.legendre_order = std::atoi(pop().c_str());
    else if (opt == "--sigs" || opt == "--sigt") {
      auto v = split(pop(), ',');
      if (v.size() != 3) usage();
      double *dst = opt == "--sigs" ? vars.sigs : vars.sigt;
      for (int m = 0; m < 3; ++m) dst[m] = std::atof(v[m].c_str());
    } else if (opt == "--niter") vars.niter = std::atoi(pop().c_str());
    else if (opt == "--arch") vars.al_v.arch_v = stringToArch(pop());
    else if (opt == "--layout") vars.al_v.layout_v = stringToLayout(pop());
    else if (opt == "--geometry") {
      const std::string g = pop();
      if (g == "kobayashi") vars.geometry = 0;
      else if (g == "cube") vars.geometry = 1;
      else usage();
    } else if (opt == "--scatter") {
      const std::string g = pop();
      if (g == "diag") vars.scatter = 0;
      else if (g == "down") vars.scatter = 1;
      else usage();
    } else if (opt == "--perturb") vars.perturb = 1;
    else if (opt == "--seed") vars.seed = std::strtoull(pop().c_str(), nullptr, 10);
    else if (opt == "--precision") {
      const std::string p = pop();
      if (p == "fp64") vars.precision = KGB_FP64;
      else if (p == "mixed") vars.precision = KGB_MIXED;
      else usage();
    } else if (opt == "--autotune") vars.autotune = true;
    else if (opt == "--json") vars.json = true;
    else {
      printf("Unknwon options %s\n", opt.c_str());
      usage();
    }
  }
  if (vars.checkValues()) return 1;

  printf("\nInput Parameters\n================\n\n");
  printf("  Problem Size:\n");
  printf("    Zones:                 %d x %d x %d  (%d total)\n", vars.nx, vars.ny, vars.nz, vars.nx * vars.ny * vars.nz);
  printf("    Groups:                %d\n", vars.num_groups);
  printf("    Legendre Order:        %d\n", vars.legendre_order);
  printf("    Quadrature Set:        ");
  if (vars.quad_num_polar == 0) printf("Dummy S2 with %d points\n", vars.num_directions);
  else printf("Gauss-Legendre, %d polar, %d azimuthal (%d points)\n", vars.quad_num_polar, vars.quad_num_azimuthal, vars.num_directions);
  printf("\n  Physical Properties:\n");
  printf("    Total X-Sec:           sigt=[%lf, %lf, %lf]\n", vars.sigt[0], vars.sigt[1], vars.sigt[2]);
  printf("    Scattering X-Sec:      sigs=[%lf, %lf, %lf]\n", vars.sigs[0], vars.sigs[1], vars.sigs[2]);
  printf("    Geometry:              %s\n", vars.geometry ? "100 cm cube, first duct leg" : "Kobayashi 3i");
  printf("    Scattering matrix:     %s\n", vars.scatter ? "seeded lower-triangular downscatter" : "diagonal P0");
  printf("\n  Solver Options:\n    Number iterations:     %d\n", vars.niter);
  printf("\n  MPI Decomposition Options:\n    Total MPI tasks:       1\n    Spatial decomp:        1 x 1 x 1 MPI tasks\n    Block solve method:    %s\n",
         vars.parallel_method == PMETHOD_BJ ? "Block Jacobi" : "Sweep");
  printf("\n  Per-Task Options:\n");
  printf("    DirSets/Directions:    %d sets, %d directions/set\n", vars.num_dirsets, vars.num_directions / vars.num_dirsets);
  printf("    GroupSet/Groups:       %d sets, %d groups/set\n", vars.num_groupsets, vars.num_groups / vars.num_groupsets);
  printf("    Zone Sets:             %d x %d x %d\n", vars.num_zonesets_dim[0], vars.num_zonesets_dim[1], vars.num_zonesets_dim[2]);
  printf("    Architecture:          %s\n", archToString(vars.al_v.arch_v).c_str());
  printf("    Data Layout:           %s\n", layoutToString(vars.al_v.layout_v).c_str());
  printf("    Precision:             %s\n", vars.precision == KGB_FP64 ? "FP64" : "mixed (FP32 state, FP64 reductions)");

  try {
    Core::DataStore ds;
    generateProblem(ds, vars);
    if (vars.autotune) {
      auto &g = ds.getVariable<Core::Gb300Context>("gb300");
      double ms = 0;
      int32_t xy = 0, tz = 0;
      g.check(kgb_field_fill(g.ctx, "psi", 0.0), "kgb_field_fill");
      g.check(kgb_iterate(g.ctx, 1.0, nullptr), "kgb_iterate");
      g.check(kgb_autotune(g.ctx, &ms, &xy, &tz), "kgb_autotune");
      printf("\n  Autotuned sweep tiles: %dx%dx%d (%.3f ms per sweep)\n", xy / 10, xy % 10, tz, ms);
    }
    SteadyStateSolver(ds, vars.niter, vars.parallel_method == PMETHOD_BJ);
    auto &timing = ds.getVariable<Timing>("timing");
    timing.print();

    // figures of merit (src/kripke.cpp:491-516)
    const size_t num_unknowns = ds.getVariable<Core::Set>("Set/Group").globalSize() *
                                ds.getVariable<Core::Set>("Set/Direction").globalSize() *
                                ds.getVariable<Core::Set>("Set/Zone").globalSize();
    const size_t num_iter = timing.getCount("SweepSolver");
    const double solve_time = timing.getTotal("Solve");
    const double iter_time = solve_time / num_iter;
    const double grind_time = iter_time / num_unknowns;
    const double throughput = num_unknowns / iter_time;
    const double sweep_eff = 100.0 * timing.getTotal("SweepSubdomain") / timing.getTotal("SweepSolver");
    printf("\nFigures of Merit\n================\n\n");
    printf("  Throughput:         %e [unknowns/(second/iteration)]\n", throughput);
    printf("  Grind time :        %e [(seconds/iteration)/unknowns]\n", grind_time);
    printf("  Sweep efficiency :  %4.5lf [100.0 * SweepSubdomain time / SweepSolver time]\n", sweep_eff);
    printf("  Number of unknowns: %lu\n", (unsigned long)num_unknowns);
    if (vars.json) {
      printf("{\"throughput\": %.6e, \"grind_time\": %.6e, \"sweep_efficiency\": %.4f, \"unknowns\": %lu, \"iterations\": %lu, \"particle_counts\": [",
             throughput, grind_time, sweep_eff, (unsigned long)num_unknowns, (unsigned long)num_iter);
      const auto &counts = ds.getVariable<ParticleHistory>("particle_history").counts;
      for (size_t i = 0; i < counts.size(); ++i) printf("%s%.17g", i ? ", " : "", counts[i]);
      printf("]}\n");
    }
  } catch (const std::exception &e) {
    printf("ERROR: %s\n", e.what());
    return 1;
  }
  printf("\nEND\n");
  return 0;
}
