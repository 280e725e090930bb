/*
 * frehg_oracle.c -- TEST INFRASTRUCTURE, NOT PRODUCT CODE.
 *
 * CPU restatement of the zLi90/frehg groundwater path in C (FP64, OpenMP).  It is the checker
 * for the GPU path: only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg (and
 * its --impl reference arm) load it.  Every function cites the reference file:line it follows
 * (paths relative to the reference source tree).  The reference cannot be compiled here (MPI,
 * PETSc, Kokkos, HDF5, yaml-cpp are absent), so there is no oracle/_ref build; parity of this
 * restatement is pinned by the reference's own invariant / known-answer tests (see
 * tests/test_oracle_pins.py) -- element-wise values are unpinned.
 *
 * Storage mirrors the reference's halo-padded GwFields (src/re/GwFields.hpp:14-75) so that the
 * ghost-cell semantics (zero-initialised ghosts before the first boundary sweep, hn/wcn ghost
 * copies, ghost reads in the reallocation sweep) come out exactly as in the reference.  The
 * density/viscosity ratio fields r_rho* / r_visc* are identically 1 (baroclinic coupling is
 * rejected by the capability gate, Orchestrator.cpp:136-137) and are folded out: multiplying
 * by 1.0 is exact, so no value changes.
 *
 * Also holds the extensions that have no reference counterpart (marked "not in reference"):
 * the mixed-form modified Picard step, harmonic face means, unit-gradient free drainage,
 * a time-varying top flux, per-cell Ks / alpha fields and a closable mass budget.
 */
#include "frehg_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

/* PETSc KSPConvergedReason values used by the CG restatement. */
enum {
  KSP_CONVERGED_RTOL = 2,
  KSP_CONVERGED_ATOL = 3,
  KSP_DIVERGED_ITS = -3,
  KSP_DIVERGED_DTOL = -4,
  KSP_DIVERGED_INDEFINITE_PC = -8,
  KSP_DIVERGED_NANORINF = -9,
  KSP_DIVERGED_INDEFINITE_MAT = -10
};

int or_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* ============================ van Genuchten / Mualem ============================ */
/* src/re/VanGenuchten.hpp:18-137, same formula order (pow/exp/log from libm). */

static double vg_m(double n) { return 1.0 - 1.0 / n; }

/* VanGenuchten::wcm (VanGenuchten.hpp:22-29) */
static double vg_wcm(const frehg_soil_params* s) {
  const double mm = vg_m(s->n);
  if (s->use_mvg)
    return s->theta_r +
           (s->theta_s - s->theta_r) * pow(1.0 + pow(fabs(s->air_entry) * s->alpha, s->n), mm);
  return s->theta_s;
}

/* waterContentFromHead (VanGenuchten.hpp:31-47) */
double or_vg_theta(const frehg_soil_params* s, double h) {
  double wc;
  if (s->use_vg) {
    const double mm = vg_m(s->n);
    const double wcm_val = vg_wcm(s);
    const double se = pow(1.0 + pow(fabs(s->alpha * h), s->n), -mm);
    if (h > s->air_entry)
      wc = s->theta_s;
    else
      wc = s->theta_r + (wcm_val - s->theta_r) * se;
  } else {
    wc = s->theta_r + (s->theta_s - s->theta_r) * exp(0.1634 * h);
  }
  if (wc > s->theta_s) wc = s->theta_s;
  if (wc < s->theta_r) wc = s->theta_r;
  return wc;
}

/* headFromWaterContent (VanGenuchten.hpp:50-65) */
double or_vg_head(const frehg_soil_params* s, double wc) {
  const double eps = 1.0e-7;
  if (s->use_vg) {
    const double mm = vg_m(s->n);
    const double wcm_val = vg_wcm(s);
    double theta = wc;
    if (theta - s->theta_r < eps) theta = s->theta_r + eps;
    if (theta < s->theta_s)
      return -(1.0 / s->alpha) *
             pow(pow((wcm_val - s->theta_r) / (theta - s->theta_r), 1.0 / mm) - 1.0, 1.0 / s->n);
    return 0.0;
  }
  return log((wc - s->theta_r) / (s->theta_s - s->theta_r)) / 0.1634;
}

/* specificMoistureCapacity (VanGenuchten.hpp:68-81) */
double or_vg_capacity(const frehg_soil_params* s, double h) {
  const double mm = vg_m(s->n);
  const double wcm_val = vg_wcm(s);
  const double nume =
      s->alpha * s->n * mm * (wcm_val - s->theta_r) * pow(fabs(s->alpha * h), s->n - 1.0);
  const double deno = pow(1.0 + pow(fabs(s->alpha * h), s->n), mm + 1.0);
  double c = nume / deno;
  if (s->use_mvg) {
    if (h > s->air_entry) c = 0.0;
  } else if (h > 0.0) {
    c = 0.0;
  }
  return c;
}

/* conductivityFromHead (VanGenuchten.hpp:84-111) */
double or_vg_conductivity(const frehg_soil_params* s, double h, double Ks) {
  if (!s->use_vg) return Ks * exp(0.1634 * h);
  const double mm = vg_m(s->n);
  const double se = pow(1.0 + pow(fabs(s->alpha * h), s->n), -mm);
  const double wcm_val = vg_wcm(s);
  double Keff;
  if (s->use_mvg) {
    const double nume =
        1.0 - pow(1.0 - pow(se * (s->theta_s - s->theta_r) / (wcm_val - s->theta_r), 1.0 / mm), mm);
    const double deno =
        1.0 - pow(1.0 - pow((s->theta_s - s->theta_r) / (wcm_val - s->theta_r), 1.0 / mm), mm);
    Keff = (deno == 0.0) ? Ks : Ks * pow(se, 0.5) * pow(nume / deno, 2.0);
  } else {
    Keff = Ks * pow(se, 0.5) * pow(1.0 - pow(1.0 - pow(se, 1.0 / mm), mm), 2.0);
  }
  if (Keff > Ks) Keff = Ks;
  if (s->use_mvg) {
    if (h > s->air_entry) Keff = Ks;
  } else if (h > 0.0) {
    Keff = Ks;
  }
  return Keff;
}

/* dKdwc (VanGenuchten.hpp:114-136) */
double or_vg_dKdwc(const frehg_soil_params* s, double wc, double Ks) {
  double theta = wc;
  if (theta > 0.9999 * s->theta_s && theta < s->theta_s) theta = 0.9999 * s->theta_s;
  const double mm = vg_m(s->n);
  const double se = (theta - s->theta_r) / (s->theta_s - s->theta_r);
  if (s->use_mvg) {
    const double wcm_val = vg_wcm(s);
    const double c2 = (s->theta_s - s->theta_r) / (wcm_val - s->theta_r);
    const double c1 = 1.0 / pow(1.0 - pow(1.0 - pow(c2, 1.0 / mm), mm), 2.0);
    const double term0 = pow(1.0 - pow(c2 * se, 1.0 / mm), mm);
    const double term1 = 0.5 * c1 * Ks * pow(se, -0.5) * (1.0 - term0) * (1.0 - term0);
    const double term2 = 2.0 * c1 * Ks * c2 * pow(se, 0.5) * pow(c2 * se, 1.0 / mm - 1.0) *
                         (1.0 - term0) * pow(1.0 - pow(c2 * se, 1.0 / mm), mm - 1.0);
    return (term1 + term2) / (s->theta_s - s->theta_r);
  }
  const double term0 = pow(1.0 - pow(se, 1.0 / mm), mm);
  const double term1 = 0.5 * Ks * pow(se, -0.5) * (1.0 - term0) * (1.0 - term0);
  const double term2 = 2.0 * Ks * pow(se, (2.0 - mm) / (2.0 * mm)) * (1.0 - term0) *
                       pow(1.0 - pow(se, 1.0 / mm), mm - 1.0);
  return (term1 + term2) / (s->theta_s - s->theta_r);
}

/* ================================ solver state ================================== */

struct or_re {
  int nx, ny, nz;
  long nh; /* halo-array length (nx+2)(ny+2)(nz+2), Grid::nCell (Grid.hpp:174-176) */
  frehg_re_params p;
  frehg_solver_config cfg;
  int attached;
  /* SoilMap (src/soil/SoilMap.hpp:28-92) and the per-cell overrides (not in reference) */
  int nclass;
  frehg_soil_params* classes;
  int32_t* cls;
  int cls3d;
  double* fKs;
  double* falpha;
  /* GwFields (src/re/GwFields.hpp:52-59) minus the identically-one ratio fields */
  double *h, *hn, *wc, *wcn, *wch, *hwc, *ch;
  double *Kx, *Ky, *Kz, *qx, *qy, *qz;
  double *Gxp, *Gxm, *Gyp, *Gym, *Gzp, *Gzm, *Gct, *Grhs;
  double *room, *bot3d, *dz3d, *actv;
  double* qtop_field; /* ReSolver::qtop_field_ (ReSolver.hpp:154) */
  int has_qtop;
  double dtn, dt_used, time;
  /* owned-order 7-point system for the head solve (assembleAndSolve, ReSolver.cpp:560-636) */
  double *coef, *b_owned, *x_owned;
  int last_its, last_reason, last_picard;
  double last_rnorm;
  long long total_its;
  /* mass budget (not in reference) */
  double vol_top_in, vol_bot_in, vol_elastic;
};

/* Grid::getIndex (src/core/Grid.hpp:186-188) */
static inline long IX(const or_re* s, int i, int j, int k) {
  return (long)(i + 1) + (long)(j + 1) * (s->nx + 2) + (long)(k + 1) * (long)(s->nx + 2) * (s->ny + 2);
}
/* interior linear index i + j*nx + k*nx*ny */
static inline long IN(const or_re* s, int i, int j, int k) {
  return (long)i + (long)j * s->nx + (long)k * s->nx * s->ny;
}

/* ReSolver::soilAt (ReSolver.cpp:87-96): class of the clamped cell, plus the per-cell Ks /
 * alpha overrides (not in reference). */
static inline frehg_soil_params soil_at(const or_re* s, int i, int j, int k) {
  frehg_soil_params r = s->p.soil;
  if (s->cls || s->fKs || s->falpha) {
    const int ci = i < 0 ? 0 : (i >= s->nx ? s->nx - 1 : i);
    const int cj = j < 0 ? 0 : (j >= s->ny ? s->ny - 1 : j);
    const int ck = k < 0 ? 0 : (k >= s->nz ? s->nz - 1 : k);
    if (s->cls) {
      const long id = s->cls3d ? IN(s, ci, cj, ck) : (long)ci + (long)cj * s->nx;
      r = s->classes[s->cls[id]];
    }
    if (s->fKs) {
      const double K = s->fKs[IN(s, ci, cj, ck)];
      r.Ks_x = K;
      r.Ks_y = K;
      r.Ks_z = K;
    }
    if (s->falpha) r.alpha = s->falpha[IN(s, ci, cj, ck)];
  }
  /* Picard (not in reference): VG theta(h) without the air-entry switch, i.e. theta = theta_s
   * only for h > 0, so theta(h) is continuous like the VG K(h) and C(h) */
  if (s->p.scheme == 1 && !r.use_mvg) r.air_entry = 0.0;
  return r;
}

static double* zalloc(long n) {
  double* a = (double*)calloc((size_t)n, sizeof(double));
  return a;
}

or_re* or_re_create(int nx, int ny, int nz, const frehg_re_params* p) {
  if (nx < 1 || ny < 1 || nz < 1 || !p) return NULL;
  or_re* s = (or_re*)calloc(1, sizeof(or_re));
  s->nx = nx;
  s->ny = ny;
  s->nz = nz;
  s->nh = (long)(nx + 2) * (ny + 2) * (nz + 2);
  s->p = *p;
  frehg_solver_config_default(&s->cfg);
  double** arr[] = {&s->h,   &s->hn,  &s->wc,  &s->wcn, &s->wch, &s->hwc, &s->ch,   &s->Kx,
                    &s->Ky,  &s->Kz,  &s->qx,  &s->qy,  &s->qz,  &s->Gxp, &s->Gxm,  &s->Gyp,
                    &s->Gym, &s->Gzp, &s->Gzm, &s->Gct, &s->Grhs, &s->room, &s->bot3d,
                    &s->dz3d, &s->actv};
  for (size_t a = 0; a < sizeof(arr) / sizeof(arr[0]); ++a) *arr[a] = zalloc(s->nh);
  s->qtop_field = zalloc((long)(nx + 2) * (ny + 2));
  const long n = (long)nx * ny * nz;
  s->coef = zalloc(7 * n);
  s->b_owned = zalloc(n);
  s->x_owned = zalloc(n);
  return s;
}

void or_re_destroy(or_re* s) {
  if (!s) return;
  double* arr[] = {s->h,   s->hn,  s->wc,  s->wcn, s->wch, s->hwc, s->ch,   s->Kx,  s->Ky,
                   s->Kz,  s->qx,  s->qy,  s->qz,  s->Gxp, s->Gxm, s->Gyp,  s->Gym, s->Gzp,
                   s->Gzm, s->Gct, s->Grhs, s->room, s->bot3d, s->dz3d, s->actv, s->qtop_field,
                   s->coef, s->b_owned, s->x_owned, s->fKs, s->falpha};
  for (size_t a = 0; a < sizeof(arr) / sizeof(arr[0]); ++a) free(arr[a]);
  free(s->classes);
  free(s->cls);
  free(s);
}

int or_re_set_params(or_re* s, const frehg_re_params* p) {
  s->p = *p;
  return FREHG_OK;
}

int or_re_set_soil_map(or_re* s, const frehg_soil_params* classes, int nclass,
                       const int32_t* class_index, int is3d) {
  if (nclass < 1 || !classes || !class_index) return FREHG_ERR_BAD_ARG;
  const long n = is3d ? (long)s->nx * s->ny * s->nz : (long)s->nx * s->ny;
  for (long c = 0; c < n; ++c)
    if (class_index[c] < 0 || class_index[c] >= nclass) return FREHG_ERR_BAD_ARG;
  free(s->classes);
  free(s->cls);
  s->classes = (frehg_soil_params*)malloc(sizeof(frehg_soil_params) * (size_t)nclass);
  memcpy(s->classes, classes, sizeof(frehg_soil_params) * (size_t)nclass);
  s->cls = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
  memcpy(s->cls, class_index, sizeof(int32_t) * (size_t)n);
  s->nclass = nclass;
  s->cls3d = is3d ? 1 : 0;
  return FREHG_OK;
}

int or_re_set_cell_fields(or_re* s, const double* Ks, const double* alpha) {
  const long n = (long)s->nx * s->ny * s->nz;
  free(s->fKs);
  free(s->falpha);
  s->fKs = NULL;
  s->falpha = NULL;
  if (Ks) {
    s->fKs = (double*)malloc(sizeof(double) * (size_t)n);
    memcpy(s->fKs, Ks, sizeof(double) * (size_t)n);
  }
  if (alpha) {
    s->falpha = (double*)malloc(sizeof(double) * (size_t)n);
    memcpy(s->falpha, alpha, sizeof(double) * (size_t)n);
  }
  return FREHG_OK;
}

int or_re_attach_solver(or_re* s, const frehg_solver_config* cfg) {
  s->cfg = *cfg;
  s->attached = 1;
  return FREHG_OK;
}

/* buildColumnGeometry (ReSolver.cpp:104-131): every layer gets dz (dz_incre is ignored). */
void or_re_initialize_geometry(or_re* s) {
  const double dz0 = s->p.dz;
  for (int k = 0; k < s->nz; ++k)
    for (int j = 0; j < s->ny; ++j)
      for (int i = 0; i < s->nx; ++i) {
        const long c = IX(s, i, j, k);
        s->bot3d[c] = -dz0 * (double)(k + 1);
        s->dz3d[c] = dz0;
        s->actv[c] = 1.0;
      }
}

/* setInitialWaterContent (ReSolver.cpp:135-153) */
int or_re_set_initial_water_content(or_re* s, const double* wc) {
  for (int k = 0; k < s->nz; ++k)
    for (int j = 0; j < s->ny; ++j)
      for (int i = 0; i < s->nx; ++i) {
        const frehg_soil_params soil = soil_at(s, i, j, k);
        const long c = IX(s, i, j, k);
        const double w = wc[IN(s, i, j, k)];
        s->wc[c] = w;
        s->h[c] = or_vg_head(&soil, w);
        s->wcn[c] = w;
        s->hn[c] = s->h[c];
      }
  return FREHG_OK;
}

/* setInitialHead (ReSolver.cpp:155-173) */
int or_re_set_initial_head(or_re* s, const double* h) {
  for (int k = 0; k < s->nz; ++k)
    for (int j = 0; j < s->ny; ++j)
      for (int i = 0; i < s->nx; ++i) {
        const frehg_soil_params soil = soil_at(s, i, j, k);
        const long c = IX(s, i, j, k);
        const double hv = h[IN(s, i, j, k)];
        s->h[c] = hv;
        s->wc[c] = or_vg_theta(&soil, hv);
        s->wcn[c] = s->wc[c];
        s->hn[c] = hv;
      }
  return FREHG_OK;
}

static void update_diagnostics(or_re* s);

/* finalizeInitialState (ReSolver.cpp:175-178) */
void or_re_finalize_initial_state(or_re* s) {
  update_diagnostics(s);
  s->dtn = s->p.dt;
}

/* initializeUniformColumn (ReSolver.cpp:180-188) */
void or_re_initialize_uniform_column(or_re* s, double init_wc) {
  or_re_initialize_geometry(s);
  const long n = (long)s->nx * s->ny * s->nz;
  double* w = (double*)malloc(sizeof(double) * (size_t)n);
  for (long c = 0; c < n; ++c) w[c] = init_wc;
  or_re_set_initial_water_content(s, w);
  free(w);
  or_re_finalize_initial_state(s);
}

/* setTopFluxField (ReSolver.cpp:68-80) */
int or_re_set_top_flux_field(or_re* s, const double* q) {
  for (int j = 0; j < s->ny; ++j)
    for (int i = 0; i < s->nx; ++i)
      s->qtop_field[(i + 1) + (j + 1) * (s->nx + 2)] = q[i + j * s->nx];
  s->has_qtop = 1;
  return FREHG_OK;
}

/* =============================== PCA step pieces ================================ */

/* savePreviousStepFields (ReSolver.cpp:190-197): whole halo arrays, ghosts included. */
static void save_previous(or_re* s) {
  const long n = s->nh;
#pragma omp parallel for schedule(static)
  for (long c = 0; c < n; ++c) {
    s->hn[c] = s->h[c];
    s->wcn[c] = s->wc[c];
  }
}

/* updateDiagnostics (ReSolver.cpp:199-215) */
static void update_diagnostics(or_re* s) {
  const int nx = s->nx, ny = s->ny, nz = s->nz;
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const long c = IX(s, i, j, k);
        if (!(s->actv[c] > 0.5)) continue;
        const frehg_soil_params soil = soil_at(s, i, j, k);
        s->hwc[c] = or_vg_head(&soil, s->wc[c]);
        s->wch[c] = or_vg_theta(&soil, s->h[c]);
        s->ch[c] = or_vg_capacity(&soil, s->h[c]);
      }
}

/* computeKFace (ReSolver.cpp:217-380), one rank. */
static void compute_kface(or_re* s) {
  const int nx = s->nx, ny = s->ny, nz = s->nz;
  const int bc2 = s->p.bc_type[2];
  const int full3d = s->p.use_full3d;
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const long c = IX(s, i, j, k);
        if (!(s->actv[c] > 0.5)) continue;
        const frehg_soil_params soilC = soil_at(s, i, j, k);
        {
          const long ip = IX(s, i + 1, j, k);
          const frehg_soil_params soilXp = soil_at(s, i + 1, j, k);
          const double Kp = or_vg_conductivity(&soilXp, s->h[ip], soilXp.Ks_x);
          const double Km = or_vg_conductivity(&soilC, s->h[c], soilC.Ks_x);
          s->Kx[c] = 0.5 * (Kp + Km);
        }
        {
          const long jp = IX(s, i, j + 1, k);
          const frehg_soil_params soilYp = soil_at(s, i, j + 1, k);
          const double Kp = or_vg_conductivity(&soilYp, s->h[jp], soilYp.Ks_y);
          const double Km = or_vg_conductivity(&soilC, s->h[c], soilC.Ks_y);
          s->Ky[c] = 0.5 * (Kp + Km);
          if (j == ny - 1) { /* one rank owns the global y+ boundary */
            if (bc2 == 0)
              s->Ky[c] = 0.0;
            else if (bc2 == 1)
              s->Ky[c] = or_vg_conductivity(&soilC, s->h[c], soilC.Ks_y);
          }
        }
        {
          const long kp = IX(s, i, j, k + 1);
          const frehg_soil_params soilZp = soil_at(s, i, j, k + 1);
          const double Kp = or_vg_conductivity(&soilZp, s->h[kp], soilZp.Ks_z);
          const double Km = or_vg_conductivity(&soilC, s->h[c], soilC.Ks_z);
          if (k + 1 < nz && (k + 1) == 0)
            s->Kz[c] = Kp;
          else if (k + 1 >= nz)
            s->Kz[c] = Km;
          else if (!(s->actv[kp] > 0.5))
            s->Kz[c] = 0.0;
          else
            s->Kz[c] = 0.5 * (Kp + Km);
        }
      }

  if (!full3d) {
    /* vertical-only lateral boundary handling (ReSolver.cpp:287-310) */
    for (int k = 0; k < nz; ++k)
      for (int j = 0; j < ny; ++j) {
        const long im = IX(s, -1, j, k);
        const long c0 = IX(s, 0, j, k);
        const frehg_soil_params soil0 = soil_at(s, 0, j, k);
        const double Kp = or_vg_conductivity(&soil0, s->h[im], soil0.Ks_x);
        s->Kx[c0] = 0.5 * (Kp + Kp);
        if (s->p.bc_type[0] == 0) s->Kx[IX(s, -1, j, k)] = 0.0;
        if (s->p.bc_type[1] == 0) s->Kx[IX(s, nx, j, k)] = 0.0;
      }
    for (int k = 0; k < nz; ++k)
      for (int i = 0; i < nx; ++i) {
        const long jm = IX(s, i, -1, k);
        const frehg_soil_params soil0 = soil_at(s, i, 0, k);
        const double Kp = or_vg_conductivity(&soil0, s->h[jm], soil0.Ks_y);
        s->Ky[IX(s, i, 0, k)] = 0.5 * (Kp + Kp);
        if (s->p.bc_type[3] == 0) s->Ky[IX(s, i, -1, k)] = 0.0;
      }
  } else {
    /* 3D wall closure (ReSolver.cpp:311-337), one rank owns every wall */
    for (int k = 0; k < nz; ++k) {
      for (int j = 0; j < ny; ++j) {
        if (s->p.bc_type[0] == 0) s->Kx[IX(s, -1, j, k)] = 0.0;
        if (s->p.bc_type[1] == 0) s->Kx[IX(s, nx - 1, j, k)] = 0.0;
      }
      for (int i = 0; i < nx; ++i) {
        if (s->p.bc_type[3] == 0) s->Ky[IX(s, i, -1, k)] = 0.0;
        if (s->p.bc_type[2] == 0) s->Ky[IX(s, i, ny - 1, k)] = 0.0;
      }
    }
  }
  /* bottom k+ boundary (ReSolver.cpp:338-344) */
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i) {
      s->Kz[IX(s, i, j, nz)] = 0.0;
      if (s->p.bc_type[4] == 0) s->Kz[IX(s, i, j, nz - 1)] = 0.0;
    }
  /* top surface k- face (ReSolver.cpp:345-363) */
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i) {
      const long c = IX(s, i, j, 0);
      const long km = IX(s, i, j, -1);
      const frehg_soil_params soil = soil_at(s, i, j, 0);
      const double Kp = or_vg_conductivity(&soil, s->h[c], soil.Ks_z);
      if (s->p.sim_shallowwater) {
      } else if (s->p.bc_type[5] == 1) {
        s->Kz[km] = soil.Ks_z;
      } else if (s->p.bc_type[5] == 0) {
        s->Kz[km] = 0.0;
      } else {
        s->Kz[km] = Kp;
      }
    }
  /* vertical-only: lateral faces closed where unsaturated (ReSolver.cpp:365-379) */
  if (!full3d) {
    for (int k = 0; k < nz; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
          const long c = IX(s, i, j, k);
          if (s->wc[c] < soil_at(s, i, j, k).theta_s) {
            s->Kx[c] = 0.0;
            s->Kx[IX(s, i - 1, j, k)] = 0.0;
            s->Ky[c] = 0.0;
            s->Ky[IX(s, i, j - 1, k)] = 0.0;
          }
        }
  }
}

/* groundwaterMatCoeff (ReSolver.cpp:397-470) */
static void mat_coeff(or_re* s) {
  const int nx = s->nx, ny = s->ny, nz = s->nz;
  const double dx = s->p.dx, dy = s->p.dy, dtg = s->p.dt;
  const int bc2 = s->p.bc_type[2], bc3 = s->p.bc_type[3];
  const int bc4 = s->p.bc_type[4], bc5 = s->p.bc_type[5];
  const int sim_sw = s->p.sim_shallowwater;
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const long c = IX(s, i, j, k);
        if (!(s->actv[c] > 0.5)) {
          s->Gxp[c] = s->Gxm[c] = s->Gyp[c] = s->Gym[c] = s->Gzp[c] = s->Gzm[c] = 0.0;
          s->Gct[c] = 1.0;
          continue;
        }
        const frehg_soil_params soil = soil_at(s, i, j, k);
        const long im = IX(s, i - 1, j, k), jm = IX(s, i, j - 1, k), km = IX(s, i, j, k - 1);
        const double dzk = s->dz3d[IX(s, 0, 0, k)];
        const double Ax_k = dy * dzk;
        const double Ay_k = dx * dzk;
        const double V = dx * dy * dzk;
        s->Gxp[c] = -s->Kx[c] * dtg * Ax_k / dx;
        s->Gxm[c] = -s->Kx[im] * dtg * Ax_k / dx;
        s->Gyp[c] = -s->Ky[c] * dtg * Ay_k / dy;
        s->Gym[c] = -s->Ky[jm] * dtg * Ay_k / dy;
        if (j == ny - 1 && bc2 == 1) s->Gyp[c] = 2.0 * s->Gyp[c];
        if (j == 0 && bc3 == 1) s->Gym[c] = 2.0 * s->Gym[c];
        const double dz_down = (k + 1 < nz) ? s->dz3d[IX(s, 0, 0, k + 1)] : dzk;
        const double dzf_p = 0.5 * (dzk + dz_down);
        s->Gzp[c] = -s->Kz[c] * dtg / (dzk * dzf_p);
        s->Gzp[c] *= V;
        double dzf_m;
        if (k == 0)
          dzf_m = 0.5 * dzk;
        else
          dzf_m = 0.5 * (dzk + s->dz3d[IX(s, 0, 0, k - 1)]);
        s->Gzm[c] = -s->Kz[km] * dtg / (dzk * dzf_m);
        s->Gzm[c] *= V;
        s->Gct[c] = (s->ch[c] + soil.Ss * s->wcn[c] / soil.theta_s);
        s->Gct[c] *= V;
        s->Gct[c] -= (s->Gxp[c] + s->Gxm[c] + s->Gyp[c] + s->Gym[c]);
        if (!(k == nz - 1 && bc4 != 1)) s->Gct[c] -= s->Gzp[c];
        if (k == 0) {
          if (!sim_sw && bc5 == 1) s->Gct[c] -= s->Gzm[c];
        } else {
          s->Gct[c] -= s->Gzm[c];
        }
      }
}

/* groundwaterRhs (ReSolver.cpp:472-549), one rank. */
static void rhs(or_re* s) {
  const int nx = s->nx, ny = s->ny, nz = s->nz;
  const double dtg = s->p.dt;
  const int bc4 = s->p.bc_type[4], bc5 = s->p.bc_type[5];
  const int sim_sw = s->p.sim_shallowwater;
  const double htop = s->p.htop;
  const double qtop_uniform = s->p.qtop, qbot_uniform = s->p.qbot;
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const long c = IX(s, i, j, k);
        if (!(s->actv[c] > 0.5)) {
          s->Grhs[c] = s->hn[c];
          continue;
        }
        const frehg_soil_params soil = soil_at(s, i, j, k);
        const long im = IX(s, i - 1, j, k), jm = IX(s, i, j - 1, k), km = IX(s, i, j, k - 1);
        const long ip = IX(s, i + 1, j, k), jp = IX(s, i, j + 1, k), kp = IX(s, i, j, k + 1);
        const double dzk = s->dz3d[IX(s, 0, 0, k)];
        const double V = s->p.dx * s->p.dy * dzk;
        double g = (s->ch[c] + soil.Ss * s->wcn[c] / soil.theta_s) * s->hn[c] * V;
        g -= dtg * V * s->Kz[c] / dzk;
        g += dtg * V * s->Kz[km] / dzk;
        if (i == nx - 1) g -= s->Gxp[c] * s->hn[ip];
        if (i == 0) g -= s->Gxm[c] * s->hn[im];
        if (j == ny - 1) g -= s->Gyp[c] * s->hn[jp];
        if (j == 0) g -= s->Gym[c] * s->hn[jm];
        if (k == nz - 1) {
          if (bc4 == 1) g += s->Gzp[c] * s->hn[kp];
          if (bc4 == 2) g += dtg * V * (qbot_uniform + s->Kz[c]) / dzk;
        }
        if (k == 0 && !sim_sw && bc5 == 1) g -= s->Gzm[c] * htop;
        if (k == 0 && !sim_sw && bc5 == 2) {
          const double qcol =
              s->has_qtop ? s->qtop_field[(i + 1) + (j + 1) * (nx + 2)] : qtop_uniform;
          g += -dtg * V * (qcol + s->Kz[IX(s, i, j, -1)]) / dzk;
        }
        s->Grhs[c] = g;
      }
}

/* ============================ PETSc-semantics Krylov ============================= */
/* KSPSolve_CG with KSP_NORM_PRECONDITIONED and KSPConvergedDefault (PETSc 3.25.1), called
 * from PetscLinearSolver::solve (src/linear/backends/PetscLinearSolver.cpp:200-220): zero
 * initial guess, converged when ||B r|| <= max(rtol*||B b||, atol); divtol 1e4. */

#define OR_DOT_BLOCK 8192

/* Deterministic dot product: fixed blocks summed in order (any thread count). */
static double or_dot(const double* a, const double* b, long n) {
  const long nb = (n + OR_DOT_BLOCK - 1) / OR_DOT_BLOCK;
  double* part = (double*)malloc(sizeof(double) * (size_t)(nb > 0 ? nb : 1));
#pragma omp parallel for schedule(static)
  for (long q = 0; q < nb; ++q) {
    const long lo = q * OR_DOT_BLOCK;
    const long hi = lo + OR_DOT_BLOCK < n ? lo + OR_DOT_BLOCK : n;
    double acc = 0.0;
    for (long c = lo; c < hi; ++c) acc += a[c] * b[c];
    part[q] = acc;
  }
  double sum = 0.0;
  for (long q = 0; q < nb; ++q) sum += part[q];
  free(part);
  return sum;
}

typedef struct {
  int nx, ny, nz;
  long n;
  const double* coef; /* 7 per row: C, W, E, S, N, Up, Down */
} or_stencil;

/* row offsets of the 7 slots in owned order row = (j*nx + i)*nz + k */
static inline void stencil_offsets(const or_stencil* A, long off[7]) {
  off[0] = 0;
  off[1] = -(long)A->nz;                   /* W    (i-1) */
  off[2] = (long)A->nz;                    /* E    (i+1) */
  off[3] = -(long)A->nz * A->nx;           /* S    (j-1) */
  off[4] = (long)A->nz * A->nx;            /* N    (j+1) */
  off[5] = -1;                             /* Up   (k-1) */
  off[6] = 1;                              /* Down (k+1) */
}

/* MatMult on the AIJ row: sum over the stored columns in ascending column order
 * (S, W, Up, C, Down, E, N in owned numbering). */
static void or_matmult(const or_stencil* A, const double* x, double* y) {
  long off[7];
  stencil_offsets(A, off);
  static const int order[7] = {3, 1, 5, 0, 6, 2, 4};
  const long n = A->n;
#pragma omp parallel for schedule(static)
  for (long r = 0; r < n; ++r) {
    const double* a = A->coef + 7 * r;
    const int k = (int)(r % A->nz);
    const long col = r / A->nz;
    const int i = (int)(col % A->nx);
    const int j = (int)(col / A->nx);
    const int present[7] = {1, i > 0, i < A->nx - 1, j > 0, j < A->ny - 1, k > 0, k < A->nz - 1};
    double sum = 0.0;
    for (int q = 0; q < 7; ++q) {
      const int slot = order[q];
      if (present[slot]) sum += a[slot] * x[r + off[slot]];
    }
    y[r] = sum;
  }
}

typedef struct {
  int kind; /* 0 none, 1 jacobi, 2 sor (SSOR, omega 1) */
  double* invd;
  const or_stencil* A;
} or_pc;

/* PCJacobi: y = x * (1/diag), zero diagonal entries replaced by 1; PCSOR with
 * SOR_LOCAL_SYMMETRIC_SWEEP, omega = 1, zero initial guess: y = (D+U)^-1 D (D+L)^-1 x in
 * owned row order; PCNONE: y = x. */
static void or_pc_apply(const or_pc* pc, const double* x, double* y) {
  const or_stencil* A = pc->A;
  const long n = A->n;
  if (pc->kind == 0) {
    memcpy(y, x, sizeof(double) * (size_t)n);
    return;
  }
  if (pc->kind == 1) {
#pragma omp parallel for schedule(static)
    for (long r = 0; r < n; ++r) y[r] = x[r] * pc->invd[r];
    return;
  }
  long off[7];
  stencil_offsets(A, off);
  /* forward: lower neighbours are S, W, Up (smaller row numbers) */
  for (long r = 0; r < n; ++r) {
    const double* a = A->coef + 7 * r;
    const int k = (int)(r % A->nz);
    const long col = r / A->nz;
    const int i = (int)(col % A->nx);
    const int j = (int)(col / A->nx);
    double sum = x[r];
    if (j > 0) sum -= a[3] * y[r + off[3]];
    if (i > 0) sum -= a[1] * y[r + off[1]];
    if (k > 0) sum -= a[5] * y[r + off[5]];
    y[r] = sum * pc->invd[r];
  }
  for (long r = 0; r < n; ++r) y[r] = y[r] / pc->invd[r];
  for (long r = n - 1; r >= 0; --r) {
    const double* a = A->coef + 7 * r;
    const int k = (int)(r % A->nz);
    const long col = r / A->nz;
    const int i = (int)(col % A->nx);
    const int j = (int)(col / A->nx);
    double sum = y[r];
    if (k < A->nz - 1) sum -= a[6] * y[r + off[6]];
    if (i < A->nx - 1) sum -= a[2] * y[r + off[2]];
    if (j < A->ny - 1) sum -= a[4] * y[r + off[4]];
    y[r] = sum * pc->invd[r];
  }
}

/* KSPConvergedDefault */
static int or_converged(int it, double rnorm, double* rnorm0, double rtol, double atol,
                        double divtol, double* ttol) {
  if (it == 0) {
    *rnorm0 = rnorm;
    *ttol = rtol * rnorm > atol ? rtol * rnorm : atol;
  }
  if (isnan(rnorm) || isinf(rnorm)) return KSP_DIVERGED_NANORINF;
  if (rnorm <= *ttol) return rnorm < atol ? KSP_CONVERGED_ATOL : KSP_CONVERGED_RTOL;
  if (divtol > 0 && rnorm >= divtol * *rnorm0) return KSP_DIVERGED_DTOL;
  return 0;
}

static int or_ksp_cg(const or_stencil* A, const or_pc* pc, const double* b, double* x,
                     double rtol, double atol, int max_it, int* its_out, double* rnorm_out) {
  const long n = A->n;
  double* r = (double*)malloc(sizeof(double) * (size_t)n);
  double* z = (double*)malloc(sizeof(double) * (size_t)n);
  double* p = (double*)malloc(sizeof(double) * (size_t)n);
  double* w = (double*)malloc(sizeof(double) * (size_t)n);
  const double divtol = 1.0e4;
  double rnorm0 = 0.0, ttol = 0.0;
  int reason = 0, i = 0;
  double beta = 0.0, betaold = 0.0, dpi = 0.0, dpiold = 0.0, dp;
  memset(x, 0, sizeof(double) * (size_t)n); /* guess_zero: r = b */
  memcpy(r, b, sizeof(double) * (size_t)n);
  or_pc_apply(pc, r, z);
  dp = sqrt(or_dot(z, z, n));
  *its_out = 0;
  reason = or_converged(0, dp, &rnorm0, rtol, atol, divtol, &ttol);
  if (!reason) {
    beta = or_dot(z, r, n);
    do {
      *its_out = i + 1;
      if (beta == 0.0) {
        reason = KSP_CONVERGED_ATOL;
        break;
      }
      if (i == 0) {
        memcpy(p, z, sizeof(double) * (size_t)n);
      } else {
        const double bb = beta / betaold;
        if (bb < 0.0) {
          reason = KSP_DIVERGED_INDEFINITE_PC;
          break;
        }
#pragma omp parallel for schedule(static)
        for (long c = 0; c < n; ++c) p[c] = z[c] + bb * p[c];
      }
      dpiold = dpi;
      or_matmult(A, p, w);
      dpi = or_dot(p, w, n);
      if (dpi == 0.0 || (i > 0 && ((dpi > 0) != (dpiold > 0)))) {
        reason = KSP_DIVERGED_INDEFINITE_MAT;
        break;
      }
      const double a = beta / dpi;
#pragma omp parallel for schedule(static)
      for (long c = 0; c < n; ++c) {
        x[c] += a * p[c];
        r[c] -= a * w[c];
      }
      or_pc_apply(pc, r, z);
      dp = sqrt(or_dot(z, z, n));
      reason = or_converged(i + 1, dp, &rnorm0, rtol, atol, divtol, &ttol);
      if (reason) break;
      betaold = beta;
      beta = or_dot(z, r, n);
      ++i;
    } while (i < max_it);
    if (!reason && i >= max_it) reason = KSP_DIVERGED_ITS;
  }
  *rnorm_out = dp;
  free(r);
  free(z);
  free(p);
  free(w);
  return reason;
}

static int pc_kind_of(const char* pc_type) {
  if (!strcmp(pc_type, "none")) return 0;
  if (!strcmp(pc_type, "jacobi")) return 1;
  if (!strcmp(pc_type, "sor")) return 2;
  return -1;
}

int or_ksp_solve_stencil(int nx, int ny, int nz, const double* coef, const double* b, double* x,
                         const char* ksp_type, const char* pc_type, double rtol, double atol,
                         int max_it, int* its, double* rnorm) {
  if (strcmp(ksp_type, "cg") != 0) return FREHG_ERR_UNSUPPORTED * 1000;
  const int kind = pc_kind_of(pc_type);
  if (kind < 0) return FREHG_ERR_UNSUPPORTED * 1000;
  or_stencil A = {nx, ny, nz, (long)nx * ny * nz, coef};
  or_pc pc = {kind, NULL, &A};
  pc.invd = (double*)malloc(sizeof(double) * (size_t)A.n);
  for (long r = 0; r < A.n; ++r) {
    const double d = coef[7 * r];
    pc.invd[r] = 1.0 / (d == 0.0 ? 1.0 : d);
  }
  const int reason = or_ksp_cg(&A, &pc, b, x, rtol, atol, max_it, its, rnorm);
  free(pc.invd);
  return reason;
}

/* assembleAndSolve (ReSolver.cpp:560-636): one rank, owned row = (j*nx + i)*nz + k.  The
 * COO rows become the 7 fixed slots of or_stencil (columns are unique per row, so ADD_VALUES
 * onto zeroed entries stores each value once). */
static int assemble_and_solve(or_re* s) {
  const int nx = s->nx, ny = s->ny, nz = s->nz;
  const long n = (long)nx * ny * nz;
#pragma omp parallel for collapse(2) schedule(static)
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i)
      for (int k = 0; k < nz; ++k) {
        const long row = ((long)j * nx + i) * nz + k;
        const long lc = IX(s, i, j, k);
        double* a = s->coef + 7 * row;
        a[0] = s->Gct[lc];
        a[1] = i > 0 ? s->Gxm[lc] : 0.0;
        a[2] = i < nx - 1 ? s->Gxp[lc] : 0.0;
        a[3] = j > 0 ? s->Gym[lc] : 0.0;
        a[4] = j < ny - 1 ? s->Gyp[lc] : 0.0;
        a[5] = k > 0 ? s->Gzm[lc] : 0.0;
        a[6] = k < nz - 1 ? s->Gzp[lc] : 0.0;
        s->b_owned[row] = s->Grhs[lc];
      }
  int its = 0;
  double rnorm = 0.0;
  const int reason =
      or_ksp_solve_stencil(nx, ny, nz, s->coef, s->b_owned, s->x_owned, s->cfg.ksp_type,
                           s->cfg.pc_type, s->cfg.rtol, s->cfg.atol, s->cfg.max_it, &its, &rnorm);
  s->last_its = its;
  s->last_rnorm = rnorm;
  s->last_reason = reason;
  s->total_its += its;
  if (reason < 0) return FREHG_ERR_NOT_CONVERGED;
#pragma omp parallel for collapse(2) schedule(static)
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i)
      for (int k = 0; k < nz; ++k) s->h[IX(s, i, j, k)] = s->x_owned[((long)j * nx + i) * nz + k];
  (void)n;
  return FREHG_OK;
}

/* enforceHeadBc (ReSolver.cpp:638-669) */
static void enforce_head_bc(or_re* s) {
  const int nx = s->nx, ny = s->ny, nz = s->nz;
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j) {
      s->h[IX(s, -1, j, k)] = s->h[IX(s, 0, j, k)];
      s->h[IX(s, nx, j, k)] = s->h[IX(s, nx - 1, j, k)];
    }
  for (int k = 0; k < nz; ++k)
    for (int i = 0; i < nx; ++i) {
      s->h[IX(s, i, -1, k)] = s->h[IX(s, i, 0, k)];
      s->h[IX(s, i, ny, k)] = s->h[IX(s, i, ny - 1, k)];
    }
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i)
      s->h[IX(s, i, j, nz)] = s->p.bc_type[4] == 1 ? s->p.hbot : s->h[IX(s, i, j, nz - 1)];
  const int top_dir = !s->p.sim_shallowwater && s->p.bc_type[5] == 1;
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i) s->h[IX(s, i, j, -1)] = top_dir ? s->p.htop : s->h[IX(s, i, j, 0)];
}

/* darcyFluxZ (ReSolver.cpp:24-58) */
static double darcy_flux_z(const or_re* s, const frehg_soil_params* soilC,
                           const frehg_soil_params* soilZp, int i, int j, int k, int back) {
  const long c = IX(s, i, j, k);
  const double faceA = s->p.dx * s->p.dy;
  if (back && k == 0) {
    const long km = IX(s, i, j, -1);
    const double delta = 0.5 * s->dz3d[c];
    double kface = soilC->Ks_z;
    if (s->p.bc_type[5] == 0)
      kface = 0.0;
    else if (s->p.bc_type[5] == 2)
      kface = or_vg_conductivity(soilC, s->h[c], soilC->Ks_z);
    return faceA * kface * ((s->h[c] - s->h[km]) / delta - 1.0);
  }
  const long kp = IX(s, i, j, k + 1);
  double delta = 0.5 * (s->dz3d[c] + s->dz3d[kp]);
  if (k == s->nz - 1) {
    delta = 0.5 * s->dz3d[c];
    if (s->p.bc_type[4] == 0) return 0.0;
  }
  const double kc = or_vg_conductivity(soilC, s->h[c], soilC->Ks_z);
  const double ks = or_vg_conductivity(soilZp, s->h[kp], soilZp->Ks_z);
  const double kface = 0.5 * (kc + ks);
  return faceA * kface * ((s->h[kp] - s->h[c]) / delta - 1.0);
}

/* groundwaterFlux (ReSolver.cpp:671-743) */
static void groundwater_flux(or_re* s) {
  const int nx = s->nx, ny = s->ny, nz = s->nz;
  const double dx = s->p.dx, dy = s->p.dy;
  const int full3d = s->p.use_full3d;
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const long c = IX(s, i, j, k);
        if (!(s->actv[c] > 0.5)) continue;
        if (full3d) {
          const double dzk = s->dz3d[IX(s, 0, 0, k)];
          const long ip = IX(s, i + 1, j, k), jp = IX(s, i, j + 1, k);
          s->qx[c] = (dy * dzk) * s->Kx[c] * (s->h[ip] - s->h[c]) / dx;
          s->qy[c] = (dx * dzk) * s->Ky[c] * (s->h[jp] - s->h[c]) / dy;
        } else {
          s->qx[c] = 0.0;
          s->qy[c] = 0.0;
        }
        const frehg_soil_params sc = soil_at(s, i, j, k);
        const frehg_soil_params sz = soil_at(s, i, j, k + 1);
        s->qz[c] = darcy_flux_z(s, &sc, &sz, i, j, k, 0);
      }
  const double Az = dx * dy;
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i) {
      const long km = IX(s, i, j, -1);
      if (s->p.bc_type[5] == 2) {
        const double qcol = s->has_qtop ? s->qtop_field[(i + 1) + (j + 1) * (nx + 2)] : s->p.qtop;
        s->qz[km] = qcol * Az;
      } else {
        const frehg_soil_params st = soil_at(s, i, j, 0);
        s->qz[km] = darcy_flux_z(s, &st, &st, i, j, 0, 1);
      }
    }
  if (s->p.bc_type[4] == 2)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) s->qz[IX(s, i, j, nz - 1)] = s->p.qbot * Az;
}

/* checkRoom (ReSolver.cpp:745-760) */
static void check_room(or_re* s) {
  const int nx = s->nx, ny = s->ny, nz = s->nz;
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const long c = IX(s, i, j, k);
        if (!(s->actv[c] > 0.5))
          s->room[c] = 0.0;
        else
          s->room[c] = (soil_at(s, i, j, k).theta_s - s->wc[c]) * s->dz3d[IX(s, 0, 0, k)] *
                       s->p.dx * s->p.dy;
      }
}

/* updateWaterContent (ReSolver.cpp:762-786) */
static void update_water_content(or_re* s) {
  const int nx = s->nx, ny = s->ny, nz = s->nz;
  const double dtg = s->p.dt;
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const long c = IX(s, i, j, k);
        if (!(s->actv[c] > 0.5)) continue;
        const frehg_soil_params soil = soil_at(s, i, j, k);
        const double V = s->p.dx * s->p.dy * s->dz3d[IX(s, 0, 0, k)];
        const double coeff = V * (1.0 + 1.0 * soil.Ss * (s->h[c] - s->hn[c]) / soil.theta_s);
        const long imc = IX(s, i - 1, j, k), jmc = IX(s, i, j - 1, k), kmc = IX(s, i, j, k - 1);
        const double dqx = dtg * (s->qx[c] - s->qx[imc]);
        const double dqy = dtg * (s->qy[c] - s->qy[jmc]);
        const double dqz = dtg * (s->qz[c] - s->qz[kmc]);
        s->wc[c] = (s->wcn[c] * V + dqx + dqy + dqz) / coeff;
      }
}

/* reallocateWaterContent (ReSolver.cpp:788-837): serial k, j, i sweep, in place. */
static int adjacent_to_sat(const or_re* s, int i, int j, int k) {
  const long c = IX(s, i, j, k);
  if (s->wc[IX(s, i, j, k + 1)] >= soil_at(s, i, j, k + 1).theta_s) return 1;
  if (s->Kx[c] != 0.0 && s->wc[IX(s, i + 1, j, k)] >= soil_at(s, i + 1, j, k).theta_s) return 1;
  if (s->Kx[IX(s, i - 1, j, k)] != 0.0 && s->wc[IX(s, i - 1, j, k)] >= soil_at(s, i - 1, j, k).theta_s)
    return 1;
  if (s->Ky[c] != 0.0 && s->wc[IX(s, i, j + 1, k)] >= soil_at(s, i, j + 1, k).theta_s) return 1;
  if (s->Ky[IX(s, i, j - 1, k)] != 0.0 && s->wc[IX(s, i, j - 1, k)] >= soil_at(s, i, j - 1, k).theta_s)
    return 1;
  if (k == 0) {
    if (!s->p.sim_shallowwater && s->p.bc_type[5] == 1 && s->p.htop >= 0.0) return 1;
  } else if (s->wc[IX(s, i, j, k - 1)] >= soil_at(s, i, j, k - 1).theta_s) {
    return 1;
  }
  return 0;
}

static void reallocate(or_re* s) {
  for (int k = 0; k < s->nz; ++k)
    for (int j = 0; j < s->ny; ++j)
      for (int i = 0; i < s->nx; ++i) {
        const long c = IX(s, i, j, k);
        if (!(s->actv[c] > 0.5)) continue;
        const frehg_soil_params soil = soil_at(s, i, j, k);
        s->wch[c] = or_vg_theta(&soil, s->h[c]);
        s->hwc[c] = or_vg_head(&soil, s->wc[c]);
        if (s->wc[c] >= soil.theta_s) {
          s->wc[c] = soil.theta_s;
        } else if (!adjacent_to_sat(s, i, j, k)) {
          if (s->wc[c] < 0.9999 * soil.theta_s) s->h[c] = s->hwc[c];
        } else {
          s->wc[c] = s->wch[c];
        }
      }
}

/* clampWaterContent (ReSolver.cpp:839-853) */
static void clamp_wc(or_re* s) {
  const int nx = s->nx, ny = s->ny, nz = s->nz;
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const long c = IX(s, i, j, k);
        if (!(s->actv[c] > 0.5)) continue;
        const frehg_soil_params soil = soil_at(s, i, j, k);
        if (s->wc[c] > soil.theta_s)
          s->wc[c] = soil.theta_s;
        else if (s->wc[c] < soil.theta_r)
          s->wc[c] = soil.theta_r;
      }
}

/* enforceMoistureBc (ReSolver.cpp:855-878) */
static void enforce_moisture_bc(or_re* s) {
  const int nx = s->nx, ny = s->ny, nz = s->nz;
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j) {
      s->wc[IX(s, -1, j, k)] = s->wc[IX(s, 0, j, k)];
      s->wc[IX(s, nx, j, k)] = s->wc[IX(s, nx - 1, j, k)];
    }
  for (int k = 0; k < nz; ++k)
    for (int i = 0; i < nx; ++i) {
      s->wc[IX(s, i, -1, k)] = s->wc[IX(s, i, 0, k)];
      s->wc[IX(s, i, ny, k)] = s->wc[IX(s, i, ny - 1, k)];
    }
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i) {
      s->wc[IX(s, i, j, nz)] = s->wc[IX(s, i, j, nz - 1)];
      s->wc[IX(s, i, j, -1)] = s->wc[IX(s, i, j, 0)];
    }
}

/* adaptiveTimeStep (ReSolver.cpp:880-929), one rank. */
static void adaptive_time_step(or_re* s) {
  const double r_red = 0.75, r_inc = 1.25;
  double dq_max = 0.0, dt_Comin = 1.0e8;
  s->p.dt = s->dtn;
  for (int k = 0; k < s->nz; ++k)
    for (int j = 0; j < s->ny; ++j)
      for (int i = 0; i < s->nx; ++i) {
        const long c = IX(s, i, j, k);
        if (!(s->actv[c] > 0.5) || k == 0) continue;
        const frehg_soil_params soil = soil_at(s, i, j, k);
        const double dzk = s->dz3d[IX(s, 0, 0, k)];
        const double Ax = s->p.dy * dzk, Ay = s->p.dx * dzk, Az = s->p.dx * s->p.dy;
        const double qin = s->qx[c] / Ax + s->qy[c] / Ay + s->qz[c] / Az;
        const double qou = s->qx[IX(s, i - 1, j, k)] / Ax + s->qy[IX(s, i, j - 1, k)] / Ay +
                           s->qz[IX(s, i, j, k - 1)] / Az;
        const double dq = fabs(qin - qou) * s->p.dt / dzk;
        dq_max = dq_max > dq ? dq_max : dq; /* std::max(dq_max, dq) */
        if (s->wc[c] < soil.theta_s) {
          const double dk = or_vg_dKdwc(&soil, s->wc[c], soil.Ks_z);
          const double dt_Co = s->p.co_max * dzk / dk;
          dt_Comin = (dt_Co < dt_Comin) ? dt_Co : dt_Comin; /* std::min(dt_Comin, dt_Co) */
        }
      }
  if (dq_max > 0.02)
    s->p.dt *= r_red;
  else if (dq_max < 0.01)
    s->p.dt *= r_inc;
  if (s->p.dt > dt_Comin) s->p.dt = dt_Comin;
  if (s->p.dt > s->p.dt_max) s->p.dt = s->p.dt_max;
  if (s->p.dt < s->p.dt_min) s->p.dt = s->p.dt_min;
  s->dtn = s->p.dt;
}

/* boundary inflow volumes of the step (not in reference): top face inflow is -qz(top ghost
 * face) * dt, bottom face inflow is +qz(bottom cell) * dt. */
static void accumulate_boundary(or_re* s) {
  double top = 0.0, bot = 0.0;
  for (int j = 0; j < s->ny; ++j)
    for (int i = 0; i < s->nx; ++i) {
      top += -s->qz[IX(s, i, j, -1)] * s->p.dt;
      bot += s->qz[IX(s, i, j, s->nz - 1)] * s->p.dt;
    }
  s->vol_top_in += top;
  s->vol_bot_in += bot;
}

static int picard_step(or_re* s);

/* ReSolver::advanceStep (ReSolver.cpp:931-969) */
static int pca_step(or_re* s) {
  s->dt_used = s->p.dt;
  save_previous(s);
  update_diagnostics(s);
  compute_kface(s);
  mat_coeff(s);
  rhs(s);
  const int st = assemble_and_solve(s);
  if (st != FREHG_OK) return st;
  enforce_head_bc(s);
  compute_kface(s);
  groundwater_flux(s);
  if (s->p.use_corrector) {
    check_room(s);
    update_water_content(s);
  } else {
    for (int k = 0; k < s->nz; ++k)
      for (int j = 0; j < s->ny; ++j)
        for (int i = 0; i < s->nx; ++i) {
          const long c = IX(s, i, j, k);
          if (s->actv[c] > 0.5) {
            const frehg_soil_params soil = soil_at(s, i, j, k);
            s->wc[c] = or_vg_theta(&soil, s->h[c]);
          }
        }
  }
  accumulate_boundary(s);
  update_diagnostics(s);
  reallocate(s);
  clamp_wc(s);
  enforce_moisture_bc(s);
  s->time += s->dt_used;
  if (s->p.adaptive_dt) adaptive_time_step(s);
  return FREHG_OK;
}

int or_re_advance_step(or_re* s) {
  if (s->p.scheme == 1) return picard_step(s);
  return pca_step(s);
}

double or_re_dt(const or_re* s) { return s->p.dt; }
double or_re_dt_used(const or_re* s) { return s->dt_used; }
double or_re_time(const or_re* s) { return s->time; }
void or_re_set_dt(or_re* s, double dt) { s->p.dt = dt; }
void or_re_prime_adaptive_dt(or_re* s, double dt) {
  s->p.dt = dt;
  s->dtn = dt;
}
int or_re_last_ksp_its(const or_re* s) { return s->last_its; }
int or_re_last_picard_its(const or_re* s) { return s->last_picard; }
double or_re_last_rnorm(const or_re* s) { return s->last_rnorm; }
long long or_re_total_ksp_its(const or_re* s) { return s->total_its; }

double or_re_water_volume(const or_re* s) {
  double v = 0.0;
  for (int k = 0; k < s->nz; ++k)
    for (int j = 0; j < s->ny; ++j)
      for (int i = 0; i < s->nx; ++i)
        v += s->wc[IX(s, i, j, k)] * s->p.dx * s->p.dy * s->dz3d[IX(s, 0, 0, k)];
  return v;
}

void or_re_boundary_volumes(const or_re* s, double* top_in, double* bottom_in) {
  *top_in = s->vol_top_in;
  *bottom_in = s->vol_bot_in;
}

double or_re_elastic_volume(const or_re* s) { return s->vol_elastic; }

int or_re_get_field(const or_re* s, const char* name, double* out) {
  const struct {
    const char* n;
    const double* a;
  } tab[] = {{"h", s->h},       {"hn", s->hn},     {"wc", s->wc},     {"wcn", s->wcn},
             {"wch", s->wch},   {"hwc", s->hwc},   {"ch", s->ch},     {"Kx", s->Kx},
             {"Ky", s->Ky},     {"Kz", s->Kz},     {"qx", s->qx},     {"qy", s->qy},
             {"qz", s->qz},     {"Gxp", s->Gxp},   {"Gxm", s->Gxm},   {"Gyp", s->Gyp},
             {"Gym", s->Gym},   {"Gzp", s->Gzp},   {"Gzm", s->Gzm},   {"Gct", s->Gct},
             {"Grhs", s->Grhs}, {"room", s->room}, {"bot3d", s->bot3d}, {"dz3d", s->dz3d},
             {"actv", s->actv}};
  for (size_t q = 0; q < sizeof(tab) / sizeof(tab[0]); ++q)
    if (!strcmp(tab[q].n, name)) {
      memcpy(out, tab[q].a, sizeof(double) * (size_t)s->nh);
      return FREHG_OK;
    }
  return FREHG_ERR_BAD_ARG;
}

/* The last linear system the step assembled (7 coefficients per owned row, C W E S N Up Down,
 * and the right-hand side), for preconditioner studies in the tests. */
void or_re_last_system(const or_re* s, double* coef, double* b) {
  const long n = (long)s->nx * s->ny * s->nz;
  if (coef) memcpy(coef, s->coef, sizeof(double) * 7 * (size_t)n);
  if (b) memcpy(b, s->b_owned, sizeof(double) * (size_t)n);
}

/* ======================= modified Picard (not in reference) ====================== */
#include "frehg_oracle_picard.inc"

/* =========================== parameter defaults ================================== */
/* SoilParams.hpp:13-25 / ReSolver.hpp:24-46 / SolverConfig.hpp:14-20 defaults.  Defined here
 * too so the oracle library stands alone. */
void frehg_soil_params_default(frehg_soil_params* s) {
  s->alpha = 1.43;
  s->n = 1.56;
  s->theta_s = 0.33;
  s->theta_r = 0.0;
  s->Ks_x = 0.0;
  s->Ks_y = 0.0;
  s->Ks_z = 2.89e-6;
  s->Ss = 1.0e-5;
  s->use_vg = 1;
  s->use_mvg = 0;
  s->air_entry = -0.02;
}

void frehg_re_params_default(frehg_re_params* p) {
  memset(p, 0, sizeof(*p));
  frehg_soil_params_default(&p->soil);
  p->dx = 1.0;
  p->dy = 1.0;
  p->dz = 0.01;
  p->botz = -1.0;
  p->dt = 1.0e-4;
  p->dt_min = 1.0e-4;
  p->dt_max = 2.0;
  p->co_max = 2.0;
  p->adaptive_dt = 1;
  p->use_corrector = 1;
  p->bc_type[5] = 1;
  p->picard_max_it = 50;
  p->picard_tol = 1.0e-6;
}

void frehg_solver_config_default(frehg_solver_config* c) {
  memset(c, 0, sizeof(*c));
  strcpy(c->ksp_type, "cg");
  strcpy(c->pc_type, "jacobi");
  c->rtol = 1.0e-8;
  c->atol = 1.0e-50;
  c->max_it = 10000;
  c->precision = 0;
  c->ir_rtol = 1.0e-10;
  c->inner_rtol = 1.0e-4;
}

/* Coupling::exchange, groundwater and surface sides (src/coupling/Coupling.cpp:25-166), serial:
 * computeExchangeRates (:48-57), limitExchange (:82-97), applyExchangeToSurface (:113-117),
 * applyExchangeToGroundwater (:133-140), total = sum q dt (:159-161); a limited cell is set to
 * theta_s / theta_r exactly (the limit's intent; the reference reaches it up to rounding,
 * and a cell an ulp short of theta_s would then count as unsaturated).  Uniform soil
 * (re.params().soil), top-cell dz; eta / bottom / q per column (i + j*nx). */
int or_re_surface_exchange(or_re* s, double* eta, const double* bottom, double dt, double visc,
                           double min_depth, double* q_out, double* total) {
  const frehg_soil_params soil = s->p.soil;
  const double Az = s->p.dx * s->p.dy;
  const double dz = s->p.dz;
  const double V = Az * dz;
  const int nx = s->nx, ny = s->ny;
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i) {
      const long o = (long)i + (long)j * nx;
      const long ti = IX(s, i, j, 0);
      const double dept = fmax(eta[o] - bottom[o], 0.0);
      double q = Az * soil.Ks_z * visc * (s->h[ti] - dept) / (0.5 * dz);
      if (dept <= min_depth && q < 0.0) q = 0.0;
      q_out[o] = q;
    }
  /* bound[o]: +1 the cell was filled to its headroom, -1 drained to theta_r (set exactly;
   * wc - q dt / V reaches theta_s / theta_r only up to rounding) */
  signed char* bound = (signed char*)calloc((size_t)nx * ny, 1);
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i) {
      const long o = (long)i + (long)j * nx;
      double q = q_out[o];
      if (q == 0.0) continue;
      const long ti = IX(s, i, j, 0);
      const double wc_top = s->wc[ti];
      if (q < 0.0) {
        const double dept = fmax(eta[o] - bottom[o], 0.0);
        const double q_min_surf = -dept * Az / dt;
        const double q_min_gw = -(soil.theta_s - wc_top) * V / dt;
        if (q <= q_min_gw && q_min_gw >= q_min_surf) bound[o] = 1;
        q = fmax(q, fmax(q_min_surf, q_min_gw));
      } else {
        const double q_max_gw = (wc_top - soil.theta_r) * V / dt;
        if (q >= q_max_gw) bound[o] = -1;
        q = fmin(q, q_max_gw);
      }
      q_out[o] = q;
    }
  double sum = 0.0;
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i) {
      const long o = (long)i + (long)j * nx;
      const long ti = IX(s, i, j, 0);
      eta[o] += q_out[o] * dt / Az;
      double w = s->wc[ti] - q_out[o] * dt / V;
      w = fmin(fmax(w, soil.theta_r), soil.theta_s);
      if (bound[o]) w = bound[o] > 0 ? soil.theta_s : soil.theta_r;
      s->wc[ti] = w;
      s->h[ti] = or_vg_head(&soil, w);
    }
  for (long o = 0; o < (long)nx * ny; ++o) sum += q_out[o] * dt;
  *total = sum;
  free(bound);
  return FREHG_OK;
}

