/*
 * Configuration header for building the reference's sources as a sequential, single-rank host
 * library (test infrastructure only: it pins the oracle).  The reference generates this file
 * with CMake; here no MPI, OpenMP, CUDA, HIP, CHAI or Caliper is enabled.
 */
#ifndef KRIPKE_CONFIG_H__
#define KRIPKE_CONFIG_H__

#define KRIPKE_VERSION "1.2.x (reference sources, sequential host build)"
#define KRIPKE_CXX_COMPILER "g++"
#define KRIPKE_CXX_FLAGS "-O2 -ffp-contract=off"
#define KRIPKE_LINK_FLAGS ""
#define KRIPKE_ARCH "Sequential"
#define KRIPKE_ARCHV_DEFAULT ArchV_Sequential
#define KRIPKE_LAYOUTV_DEFAULT LayoutV_DGZ

#endif
