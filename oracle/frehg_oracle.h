/*
 * frehg_oracle.h -- TEST INFRASTRUCTURE, NOT PRODUCT CODE.
 *
 * CPU restatement (C, FP64, OpenMP) of the zLi90/frehg groundwater path, used only as the
 * checker by tests/, __graft_entry__.smoke() and the cpu_baseline leg of bench.py.  The
 * product (frehg_gb300/) never links, loads or calls it.
 *
 * Parity pinning: the reference cannot be built here (it needs MPI, PETSc 3.25.1, Kokkos
 * 5.1.1, HDF5, yaml-cpp) and ships no golden vectors for this path (the legacy b2-gw output
 * files its tests read are absent).  The restatement is pinned by the known-answer and
 * invariant tests the reference holds for the path (tests/re/test_re_constitutive.cpp,
 * tests/re/test_re_3d.cpp, tests/re/test_re_b2_gw.cpp:109-153,
 * tests/linear/test_petsc_linear_solver.cpp, tests/linear/test_assembly_backend_independent.cpp),
 * re-run against it in tests/test_oracle_pins.py.  Element-wise parity with the reference
 * binary is therefore partial: invariants pinned, values unpinned.
 */
#ifndef FREHG_ORACLE_H
#define FREHG_ORACLE_H

#include "../include/frehg_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct or_re or_re;

/* ReSolver restatement (src/re/ReSolver.cpp).  Same call order as the reference. */
or_re* or_re_create(int nx, int ny, int nz, const frehg_re_params* p);
void or_re_destroy(or_re* st);
int or_re_set_params(or_re* st, const frehg_re_params* p);
int or_re_set_soil_map(or_re* st, const frehg_soil_params* classes, int nclass,
                       const int32_t* class_index, int is3d);
int or_re_set_cell_fields(or_re* st, const double* Ks, const double* alpha);
int or_re_attach_solver(or_re* st, const frehg_solver_config* cfg);
void or_re_initialize_geometry(or_re* st);
int or_re_set_initial_head(or_re* st, const double* h);
int or_re_set_initial_water_content(or_re* st, const double* wc);
void or_re_finalize_initial_state(or_re* st);
void or_re_initialize_uniform_column(or_re* st, double init_wc);
int or_re_set_top_flux_field(or_re* st, const double* q);
/* Returns FREHG_OK or FREHG_ERR_NOT_CONVERGED (KSP diverged: the reference throws). */
int or_re_advance_step(or_re* st);
double or_re_dt(const or_re* st);
double or_re_dt_used(const or_re* st);
double or_re_time(const or_re* st);
void or_re_set_dt(or_re* st, double dt);
void or_re_prime_adaptive_dt(or_re* st, double dt);
/* Copy a named halo field ((nx+2)(ny+2)(nz+2) doubles).  Returns FREHG_ERR_BAD_ARG on an
 * unknown name. */
int or_re_get_field(const or_re* st, const char* name, double* out_halo);
int or_re_last_ksp_its(const or_re* st);
/* the last assembled system: coef[7 n] (owned order, slots C W E S N Up Down) and b[n] */
void or_re_last_system(const or_re* st, double* coef, double* b);
int or_re_last_picard_its(const or_re* st);
double or_re_last_rnorm(const or_re* st);
long long or_re_total_ksp_its(const or_re* st);
double or_re_water_volume(const or_re* st);
int or_re_surface_exchange(or_re* st, double* eta, const double* bottom, double dt, double visc,
                           double min_depth, double* q_out, double* total);
void or_re_boundary_volumes(const or_re* st, double* top_in, double* bottom_in);
/* cumulative elastic (specific-storage) volume of the Picard step (not in reference) */
double or_re_elastic_volume(const or_re* st);

/* van Genuchten restatement (src/re/VanGenuchten.hpp:18-137). */
double or_vg_theta(const frehg_soil_params* s, double h);
double or_vg_head(const frehg_soil_params* s, double wc);
double or_vg_capacity(const frehg_soil_params* s, double h);
double or_vg_conductivity(const frehg_soil_params* s, double h, double Ks);
double or_vg_dKdwc(const frehg_soil_params* s, double wc, double Ks);

/* PETSc-semantics Krylov solve on a 7-point system given in owned order (k fastest, Decomp3D
 * on one rank).  coef holds 7 entries per row in the order centre, W, E, S, N, Up, Down
 * (DomainDecomposition.cpp:247-256); absent neighbours carry 0.  Returns the KSP converged
 * reason (>0 converged, <0 diverged) and the iteration count / final residual norm. */
int or_ksp_solve_stencil(int nx, int ny, int nz, const double* coef, const double* b, double* x,
                         const char* ksp_type, const char* pc_type, double rtol, double atol,
                         int max_it, int* its, double* rnorm);

int or_num_threads(void);

#ifdef __cplusplus
}
#endif

#endif /* FREHG_ORACLE_H */
