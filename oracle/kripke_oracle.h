/*
 * kripke_oracle.h -- C interface of the CPU oracle for Kripke's source-iteration path.
 *
 * TEST INFRASTRUCTURE ONLY.  The oracle is a plain C++ restatement of the
 * reference algorithm (problem generation, the six kernels, the sweep
 * scheduler and the steady-state loop).  Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg may load it; the product path never does.
 *
 * Parity status: pinned to the reference itself.  oracle/ref_build.sh compiles
 * the reference's own sources (LLNL Kripke v1.2.x: generator, Kernel::*,
 * SweepSolver, SteadyStateSolver) against a project-written stand-in for the
 * RAJA loop names (oracle/refshim/), and this oracle equals that build bit for
 * bit -- every generated input, every kernel's output and the solved
 * psi/phi/phi_out/rhs -- on every configuration tests/test_ref_pin.py checks,
 * live and against the golden records in tests/golden/ (the particle count
 * differs by summation order only).  It is also pinned by analytic known
 * answers (closed-form diamond difference, pure absorber, quadrature
 * identities, exact material volumes) in tests/test_oracle.py.
 *
 * Data model: every field is stored exactly as the reference's
 * Core::Field stores it -- one chunk per subdomain of the field's partition
 * space, each chunk laid out in the selected nesting (DGZ..ZGD) with the
 * permutation rule of Core/VarLayout.h:118-170 -- and the get/set entry
 * points move the concatenation of all chunks in chunk order.
 */
#ifndef KRIPKE_ORACLE_H
#define KRIPKE_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Mirrors InputVariables (src/Kripke/InputVariables.h:18-49) plus the
 * generator options the benchmark configurations add. */
typedef struct orc_input {
  int32_t nx, ny, nz;
  int32_t num_directions;
  int32_t num_groups;
  int32_t legendre_order;
  int32_t quad_num_polar;       /* 0: dummy S2 (--quad N); >0: Gauss-Legendre */
  int32_t quad_num_azimuthal;
  int32_t layout;               /* 0..5 = DGZ, DZG, GDZ, GZD, ZDG, ZGD */
  int32_t num_dirsets;
  int32_t num_groupsets;
  int32_t num_zonesets_dim[3];
  int32_t niter;
  int32_t num_material_subsamples;
  int32_t geometry;             /* 0: Kobayashi 3i (reference), 1: 100 cm cube, first duct leg only */
  int32_t scatter;              /* 0: diagonal P0 sigs (reference), 1: seeded lower-triangular downscatter */
  int32_t perturb;              /* 1: seeded uniform +-20% per (material, group) on sigma_t and sigma_s */
  int32_t pad_;
  uint64_t seed;
  double sigt[3];
  double sigs[3];
  double source_strength;       /* reference: 1.0 (src/Kripke/Kernel/Source.cpp:98) */
} orc_input;

typedef struct orc_problem orc_problem;

void orc_default_input(orc_input *in);

/* Generate a problem (Kripke::generateProblem).  Returns NULL on bad input;
 * orc_error() then holds the message. */
orc_problem *orc_create(const orc_input *in);
void orc_destroy(orc_problem *p);
const char *orc_error(void);

/* 0 = sequential (reference Sequential policies, the parity oracle);
 * n > 0 = OpenMP with n threads (reference OpenMP policies, the timed CPU baseline). */
void orc_set_threads(orc_problem *p, int n);

/* 1: orc_sweep_solver (and every solve) runs the block Jacobi method
 * (--pmethod bj, SteadyStateSolver's block_jacobi argument); 0: the sweep. */
void orc_set_block_jacobi(orc_problem *p, int on);

int32_t orc_num_sdoms(const orc_problem *p);
/* Element count (all chunks) and element size in bytes of a named field; -1 if unknown. */
int64_t orc_field_size(const orc_problem *p, const char *name);
int32_t orc_field_elem_bytes(const orc_problem *p, const char *name);
int32_t orc_field_get(const orc_problem *p, const char *name, void *out);
int32_t orc_field_set(orc_problem *p, const char *name, const void *in);
/* Per-chunk sizes of the flux/moment sets, for the caller's bookkeeping. */
int32_t orc_sdom_info(const orc_problem *p, int32_t sdom, int32_t out[8]);

void orc_kconst(orc_problem *p, const char *name, double value);
void orc_ltimes(orc_problem *p);
void orc_lplustimes(orc_problem *p);
void orc_scattering(orc_problem *p);
void orc_source(orc_problem *p);
void orc_sweep_subdomain(orc_problem *p, int32_t sdom);
void orc_sweep_solver(orc_problem *p);
double orc_population(orc_problem *p);
/* emission = sum w*rhs*vol, collision = sum w*sigt*psi*vol, leakage = outflow
 * through the domain boundary, population; residual = emission-collision-leakage. */
void orc_balance(orc_problem *p, double out[5]);
/* Kripke::SteadyStateSolver: niter iterations; part[i] = particle count after iteration i. */
int32_t orc_solve(orc_problem *p, int32_t niter, double *part);
/* One source iteration on the current psi (no reset); returns the particle count. */
double orc_iterate(orc_problem *p);
/* Wall-clock seconds of the last orc_solve (the reference's "Solve" timer). */
double orc_last_solve_seconds(const orc_problem *p);

#ifdef __cplusplus
}
#endif
#endif
