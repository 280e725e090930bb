/*
 * frehg_gb300.h -- C ABI of the GB300 (sm_103a) groundwater hot path.
 *
 * Plain C: opaque handles, plain pointers and sizes, int status codes, no exceptions and no
 * library types across the boundary.  Every entry point names the reference interface it
 * replaces (paths relative to the zLi90/frehg source tree).
 *
 * Two handle families:
 *   frehg_re_*      -- the Richards-equation step (replaces class ReSolver,
 *                      src/re/ReSolver.hpp:48-156).  State lives in device memory; the step
 *                      runs entirely on the GPU.
 *   frehg_cg_*,     -- the linear-solver seam (replaces LinearSolver / SparseSystem,
 *   frehg_system_*     include/frehg2/linear/LinearSolver.hpp:18-33, SparseSystem.hpp:15-40)
 *                      for callers that assemble a 7-point system row by row.
 *
 * Layout conventions
 *   interior arrays : i fastest, then j, then k (k = 0 is the top layer); index i + j*nx + k*nx*ny.
 *                     This is the order ReSolver::setInitialHead takes (ReSolver.cpp:155-173).
 *   halo arrays     : (nx+2)*(ny+2)*(nz+2), index (i+1) + (j+1)(nx+2) + (k+1)(nx+2)(ny+2)
 *                     (Grid::getIndex, src/core/Grid.hpp:186-188).
 *   owned order     : the linear-solver row order of Decomp3D on one rank, k fastest:
 *                     row = (j*nx + i)*nz + k (src/linear/DomainDecomposition.cpp:235-245).
 *
 * Threading: one CUDA stream per handle; a handle is not thread-safe; handles are independent.
 */
#ifndef FREHG_GB300_H
#define FREHG_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------------------------------ */
/* Status codes.  The reference throws std::runtime_error (PetscLinearSolver.cpp:21-25,206-211); */
/* a C++ caller rethrows any non-zero code as that exception.                                  */
/* ------------------------------------------------------------------------------------------ */
enum {
  FREHG_OK = 0,
  FREHG_ERR_BAD_ARG = 1,        /* invalid argument (size, range, null pointer)              */
  FREHG_ERR_CUDA = 2,           /* a CUDA runtime call failed                                */
  FREHG_ERR_NOT_CONVERGED = 3,  /* Krylov solve diverged or hit max_it (KSP reason < 0)      */
  FREHG_ERR_NONFINITE = 4,      /* NaN/Inf met in a reduction                                */
  FREHG_ERR_STATE = 5,          /* call out of order (e.g. advance before initial state)     */
  FREHG_ERR_UNSUPPORTED = 6,    /* configuration the build does not realise                  */
  FREHG_ERR_NO_DEVICE = 7       /* no CUDA device / extension not loadable                   */
};

/* Text of the last error raised on the calling thread ("" when none). */
const char* frehg_last_error(void);

/* ------------------------------------------------------------------------------------------ */
/* Parameter blocks                                                                            */
/* ------------------------------------------------------------------------------------------ */

/* struct SoilParams (include/frehg2/re/SoilParams.hpp:13-25), same fields and defaults. */
typedef struct frehg_soil_params {
  double alpha;     /* VG alpha [1/m]                                 default 1.43    */
  double n;         /* VG n                                           default 1.56    */
  double theta_s;   /* saturated water content                        default 0.33    */
  double theta_r;   /* residual water content                         default 0.0     */
  double Ks_x;      /* saturated conductivity [m/s]                   default 0.0     */
  double Ks_y;      /*                                                default 0.0     */
  double Ks_z;      /*                                                default 2.89e-6 */
  double Ss;        /* specific storage [1/m]                         default 1e-5    */
  int32_t use_vg;   /* van Genuchten (1) or exponential (0)           default 1       */
  int32_t use_mvg;  /* modified VG with air entry                     default 0       */
  double air_entry; /* air-entry head [m]                             default -0.02   */
} frehg_soil_params;

/* struct ReParams (src/re/ReSolver.hpp:24-46) plus the extensions marked "not in reference". */
typedef struct frehg_re_params {
  frehg_soil_params soil; /* uniform soil / class 0                                          */
  double dx, dy, dz;      /* cell sizes [m]                 defaults 1, 1, 0.01              */
  double botz;            /* domain bottom elevation        default -1                       */
  double dt;              /* time step [s]                  default 1e-4                     */
  double dt_min, dt_max;  /* adaptive bounds                defaults 1e-4, 2                 */
  double co_max;          /* Courant limit                  default 2                        */
  int32_t adaptive_dt;    /* default 1 */
  int32_t use_corrector;  /* default 1 */
  int32_t use_full3d;     /* default 0 */
  int32_t follow_terrain; /* default 0 (1 is rejected: not realised by the reference step)    */
  int32_t sim_shallowwater; /* default 0 (coupled top face)                                   */
  int32_t baroclinic;     /* default 0 (1 is rejected, as Orchestrator.cpp:136-137 does)      */
  int32_t bc_type[6];     /* x-, x+, y-, y+, z+ (bottom), z- (top); 0 no-flux, 1 Dirichlet,
                             2 fixed flux; 3 unit-gradient free drainage (bottom, not in
                             reference).  default {0,0,0,0,0,1}                              */
  double htop, hbot;      /* Dirichlet heads [m]                                             */
  double qtop, qbot;      /* fixed fluxes [m/s]; qtop<0 = infiltration, qbot>0 = inflow      */
  /* ---- not in reference (spec extensions) ---- */
  int32_t scheme;         /* 0 = PCA predictor-corrector (ReSolver::advanceStep),
                             1 = mixed-form modified Picard (Celia et al. 1990)               */
  int32_t face_mean;      /* 0 = arithmetic 0.5(Kp+Km) (reference), 1 = harmonic              */
  int32_t picard_max_it;  /* default 50                                                      */
  double picard_tol;      /* |dh|_inf stopping test [m], default 1e-6                        */
  double rain_rate;       /* rain on the top face (bc_type[5] = 2) while t < rain_until [m/s,
                             < 0 downward; a top flux field, when set, replaces it per
                             column]; the face takes at most what a surface held at h = 0
                             admits (no ponding, the excess runs off); 0 disables             */
  double rain_until;      /* [s]                                                             */
  int32_t picard_dt_adapt;/* Picard-count driven dt (1) or fixed (0)                         */
  int32_t picard_fp64;    /* Picard constitutive relations, fluxes and final update
                             (van Genuchten classes) in native FP64 (1) or in float-float
                             arithmetic on the FP32 pipe, ~48 significant bits, several times
                             faster on GB300 (0); -1 (default): float-float with the mixed-
                             precision solve, FP64 with the FP64 solve                       */
  double picard_dh_max;   /* largest head change one Picard iteration applies per cell [m];
                             0 = unlimited (default)                                         */
} frehg_re_params;

/* struct SolverConfig (include/frehg2/linear/SolverConfig.hpp:14-20) plus precision keys. */
typedef struct frehg_solver_config {
  char ksp_type[16];      /* "cg" (default) or "fcg"                                         */
  char pc_type[16];       /* "jacobi" (default here); with precision 1 also "line" (vertical-
                             line tridiagonal), "unet" / "unet-line" (learned, RE handles)   */
  double rtol;            /* default 1e-8                                                    */
  double atol;            /* default 1e-50                                                   */
  int32_t max_it;         /* default 10000                                                   */
  int32_t precision;      /* 0 = fp64 throughout, 1 = fp32 Krylov under fp64 refinement      */
  double ir_rtol;         /* refinement stop: true relative residual, default 1e-10          */
  double inner_rtol;      /* fp32 inner solve relative tolerance, default 1e-4               */
} frehg_solver_config;

void frehg_soil_params_default(frehg_soil_params* s);
void frehg_re_params_default(frehg_re_params* p);
void frehg_solver_config_default(frehg_solver_config* c);

/* ------------------------------------------------------------------------------------------ */
/* Richards-equation step: replaces ReSolver (src/re/ReSolver.hpp:48-156).                      */
/* ------------------------------------------------------------------------------------------ */
typedef struct frehg_re frehg_re;

/* ReSolver(const Grid&, const MpiComm*) + setParams (ReSolver.hpp:50,53).  Allocates the device
 * state for an nx*ny*nz grid on the current CUDA device; at most 2^31 - 1 cells
 * (FREHG_ERR_ARG beyond). */
int frehg_re_create(int nx, int ny, int nz, const frehg_re_params* p, frehg_re** out);
int frehg_re_destroy(frehg_re* re);
/* ReSolver::setParams (ReSolver.hpp:53).  Grid sizes stay fixed. */
int frehg_re_set_params(frehg_re* re, const frehg_re_params* p);
int frehg_re_get_params(const frehg_re* re, frehg_re_params* p);

/* ReSolver::setSoilMap (ReSolver.hpp:59) with SoilMap::setClasses + setClassIndex/3D
 * (src/soil/SoilMap.hpp:33-43).  class_index has nx*ny (is3d = 0) or nx*ny*nz (is3d = 1)
 * entries in interior order; every id must lie in [0, nclass). */
int frehg_re_set_soil_map(frehg_re* re, const frehg_soil_params* classes, int nclass,
                          const int32_t* class_index, int is3d);
/* Not in reference: per-cell overrides of Ks (all three directions) and of alpha, as needed by
 * continuous random soil fields.  Either pointer may be NULL.  Interior order, nx*ny*nz each. */
int frehg_re_set_cell_fields(frehg_re* re, const double* Ks, const double* alpha);

/* ReSolver::attachSolver (ReSolver.hpp:67): the RE step uses cfg for its head solve. */
int frehg_re_attach_solver(frehg_re* re, const frehg_solver_config* cfg);

/* ReSolver::initializeGeometry / setInitialWaterContent / setInitialHead /
 * finalizeInitialState / initializeUniformColumn (ReSolver.hpp:73-79, ReSolver.cpp:104-188).
 * Host arrays, interior order.  finalize starts a run: on a handle that has stepped before,
 * the ghost values (zero until the first step writes them), the simulated time and the boundary
 * budgets restart as on a fresh handle, so a re-initialised handle steps like a new one. */
int frehg_re_initialize_geometry(frehg_re* re);
int frehg_re_set_initial_head(frehg_re* re, const double* h);
int frehg_re_set_initial_water_content(frehg_re* re, const double* wc);
int frehg_re_finalize_initial_state(frehg_re* re);
int frehg_re_initialize_uniform_column(frehg_re* re, double init_wc);

/* ReSolver::setTopFluxField (ReSolver.hpp:105): nx*ny values, index i + j*nx. */
int frehg_re_set_top_flux_field(frehg_re* re, const double* q);

/* ReSolver::advanceStep (ReSolver.cpp:931-969). */
int frehg_re_advance_step(frehg_re* re);
/* Convenience: nsteps calls of advanceStep on the handle's stream without host round trips
 * other than the Krylov convergence checks. */
int frehg_re_advance_steps(frehg_re* re, int nsteps);

/* ReSolver::dt / dtUsed / setDt / primeAdaptiveDt (ReSolver.hpp:87-98). */
int frehg_re_dt(const frehg_re* re, double* dt);
int frehg_re_dt_used(const frehg_re* re, double* dt);
int frehg_re_set_dt(frehg_re* re, double dt);
int frehg_re_prime_adaptive_dt(frehg_re* re, double dt);
/* Simulated time accumulated by advance_step [s] (not in reference; the driver keeps it). */
int frehg_re_time(const frehg_re* re, double* t);

/* ReSolver::fields() (ReSolver.hpp:84): copy one named GwFields array (src/re/GwFields.hpp:52-59)
 * to host memory in the halo layout ((nx+2)(ny+2)(nz+2) doubles).  Supported names:
 * h hn wc wcn wch hwc ch Kx Ky Kz qx qy qz room dz3d actv bot3d. */
int frehg_re_get_field(frehg_re* re, const char* name, double* out_halo);
/* Interior copy (nx*ny*nz, interior order) of h, wc, hn or wcn; device_out != 0 means out is a
 * device pointer (device-to-device copy). */
int frehg_re_get_interior(frehg_re* re, const char* name, double* out, int device_out);
/* The same copy to host memory without waiting (not in reference): it is ordered after the work
 * issued so far and runs on a copy stream of the handle, so that the copy of a step's result
 * overlaps the next step (which writes the other state buffer); calls that would overwrite the
 * copied buffer wait for it.  out must stay valid and unread until frehg_re_sync; page-locked
 * memory (cudaHostAlloc) makes the copy asynchronous.  Names: h, wc, hn, wcn. */
int frehg_re_get_interior_async(frehg_re* re, const char* name, double* out);

/* Perf counters (src/perf: cells_touched = cells*steps ReSolver.cpp:933, ksp_iterations :621). */
typedef struct frehg_re_counters {
  int64_t steps;
  int64_t cells_touched;
  int64_t ksp_iterations;
  int64_t picard_iterations;
  int64_t realloc_sweeps;
  int32_t last_ksp_iterations;
  int32_t last_picard_iterations;
  double last_residual_norm;
  int64_t kernel_launches;   /* kernels this handle launched (graph nodes included)      */
  int64_t ir_sweeps;         /* mixed precision: FP64 refinement sweeps (not in reference)  */
  int64_t fcg_fallbacks;     /* learned preconditioner dropped for Jacobi (not in reference) */
  double elastic_volume;     /* Picard: cumulative specific-storage volume [m^3]            */
  int64_t net_solves;        /* solves that applied the network (not in reference)          */
  int64_t net_skipped;       /* solves the time policy ran without it (not in reference)    */
  double net_ms;             /* host time of the solves that applied the network [ms]       */
  double plain_ms;           /* host time of the solves without the network [ms]            */
} frehg_re_counters;
int frehg_re_get_counters(const frehg_re* re, frehg_re_counters* c);

/* Total water volume sum(theta*V) in FP64 (Orchestrator.cpp:924-930 "water_vol_subs"), and the
 * cumulative top / bottom boundary inflow volumes (not in reference). */
int frehg_re_water_volume(frehg_re* re, double* vol);
int frehg_re_boundary_volumes(frehg_re* re, double* top_in, double* bottom_in);

/* Per-kernel timing (not in reference; benchmarking aid).  While profiling is on, every kernel
 * the handle launches is bracketed by CUDA events on the handle's stream (the Krylov loop then
 * runs without its CUDA graph), and duration, launch count and the algorithmic bytes of one
 * launch are accumulated per kernel name.  idle_launches counts the launches of the inner
 * Krylov iterations that found their solve already converged and returned at once (the inner
 * loop launches whole chunks of iterations); their bytes are not moved.  Turning profiling on
 * clears the table. */
typedef struct frehg_kernel_stat {
  char name[32];
  int64_t launches;
  double total_ms;
  double bytes_per_launch;
  int64_t idle_launches;
} frehg_kernel_stat;
int frehg_re_set_profiling(frehg_re* re, int on);
int frehg_re_kernel_stats(frehg_re* re, frehg_kernel_stat* out, int max, int* count);

/* Stream control: all work of the handle is issued on this stream (cudaStream_t passed as
 * void*; NULL = the handle's own stream).  frehg_re_sync waits for it. */
int frehg_re_set_stream(frehg_re* re, void* cuda_stream);
int frehg_re_sync(frehg_re* re);

/* ------------------------------------------------------------------------------------------ */
/* Linear-solver seam: replaces LinearSolver + SparseSystem + makeLinearSolver                  */
/* (include/frehg2/linear/LinearSolver.hpp:18-33, SparseSystem.hpp:15-40,                       */
/*  src/linear/backends/LinearSolverFactory.cpp:9-16).                                         */
/* ------------------------------------------------------------------------------------------ */
typedef struct frehg_cg frehg_cg;
typedef struct frehg_system frehg_system;

/* makeLinearSolver("gb300", cfg).  Unknown ksp/pc types give FREHG_ERR_UNSUPPORTED, as the
 * reference factory throws for an unknown backend (LinearSolverFactory.cpp:14-15). */
int frehg_cg_create(const frehg_solver_config* cfg, frehg_cg** out);
int frehg_cg_destroy(frehg_cg* cg);

/* LinearSolver::createSystem(const DecompBase&) + SparseSystem::preallocate for the 7-point
 * Decomp3D of one rank (nz = 1 gives the 5-point Decomp2D, row = j*nx + i). */
int frehg_system_create(frehg_cg* cg, int nx, int ny, int nz, frehg_system** out);
int frehg_system_destroy(frehg_system* sys);
int frehg_system_zero_entries(frehg_system* sys);     /* SparseSystem::zeroEntries   */
int frehg_system_begin_assembly(frehg_system* sys);   /* SparseSystem::beginAssembly */
int frehg_system_end_assembly(frehg_system* sys);     /* SparseSystem::endAssembly   */
/* SparseSystem::addRow: ADD_VALUES semantics; every column must be the row itself or one of its
 * 7-point neighbours, else FREHG_ERR_BAD_ARG. */
int frehg_system_add_row(frehg_system* sys, int global_row, int ncols, const int* cols,
                         const double* vals);
/* SparseSystem::addCOO: n triplets, duplicates summed (KokkosPetscBridgeDevice.cpp:55-61).
 * on_device != 0: the three arrays are device pointers. */
int frehg_system_add_coo(frehg_system* sys, const int* rows, const int* cols, const double* vals,
                         int64_t n, int on_device);
/* SparseSystem::setRhs / getSolution (owned order). */
int frehg_system_set_rhs(frehg_system* sys, const double* b, int on_device);
int frehg_system_get_solution(frehg_system* sys, double* x, int on_device);

/* LinearSolver::setup / solve (PetscLinearSolver.cpp:186-220): zero initial guess, stop when
 * the preconditioned residual norm <= max(rtol*||B b||, atol).  b and x are owned-order host
 * arrays (or device arrays when on_device != 0). */
int frehg_cg_setup(frehg_cg* cg, frehg_system* sys);
int frehg_cg_solve(frehg_cg* cg, frehg_system* sys, const double* b, double* x, int on_device);
int frehg_cg_iteration_count(const frehg_cg* cg, int* its);   /* getIterationCount */
int frehg_cg_residual_norm(const frehg_cg* cg, double* rnorm); /* getResidualNorm   */
int frehg_cg_converged_reason(const frehg_cg* cg, int* reason); /* KSPConvergedReason */
/* Not in reference: the FP64 Jacobi-PCG iteration (precision 0, pc_type "jacobi") as one
 * cooperative launch (direction, stencil product with p.w and update with the norms, separated
 * by grid barriers whose waits are bounded) or as three kernels.  on = 1: one launch wherever
 * the device has cooperative launches; 0: three kernels; -1 (default): one launch for systems
 * of at most 65,536 unknowns, where it is the faster form on GB300, three kernels above.  The
 * two forms sum the dot products over different block partitions, so their last bits (and, in
 * a borderline case, an iteration count) may differ. */
int frehg_cg_set_fused_iteration(frehg_cg* cg, int on);
/* Self-check of the one-launch iteration's grid barrier (not in reference): two cooperative
 * blocks meet at one barrier whose wait is bounded by `polls` polls; skip_block = 0 or 1 makes
 * that block return without arriving, so the other's wait runs out, sets the timeout flag and
 * the kernel ends normally (*timed_out = 1; the context stays usable); skip_block = -1: both
 * arrive (*timed_out = 0). */
int frehg_check_grid_barrier(int skip_block, long long polls, int* timed_out);

/* ------------------------------------------------------------------------------------------ */
/* Learned preconditioner (not in reference): 3-level 3D U-Net (16/32/64 channels, 3x3x3 conv,  */
/* BF16 weights and activations on the tensor cores, FP32 accumulation) with its own forward,   */
/* backward and Adam kernels.  Inputs are FP32 device arrays of nx*ny*nz cells (i fastest);     */
/* nx, ny, nz must be divisible by 4.                                                          */
/* ------------------------------------------------------------------------------------------ */
typedef struct frehg_unet frehg_unet;
int frehg_unet_create(uint64_t seed, frehg_unet** out);
int frehg_unet_destroy(frehg_unet* net);
int frehg_unet_num_params(const frehg_unet* net, int64_t* n);
/* FP32 master parameters to / from host memory (layout: per convolution W[27][cout][cin] then
 * b[cout], for c1a c1b c2a c2b c3a c3b d2a d2b d1a d1b; then the output w[16], b). */
int frehg_unet_get_params(frehg_unet* net, float* host);
int frehg_unet_set_params(frehg_unet* net, const float* host);
/* input channel scaling: ln K -> (ln K - mean) * scale; capacity -> C * cap_scale */
int frehg_unet_set_input_scaling(frehg_unet* net, float lnk_mean, float lnk_scale, float cap_scale);
/* y = rms(r) * NN(r / rms(r), ln K, C) */
int frehg_unet_forward(frehg_unet* net, int nx, int ny, int nz, const float* r, const float* lnk,
                       const float* cap, float* y, void* stream);
/* loss = mean((NN(r / rms r) - target / rms r)^2) and the parameter gradients (kept in the
 * network for frehg_unet_adam_step; copied to grad_host when it is not NULL). */
int frehg_unet_loss_grad(frehg_unet* net, int nx, int ny, int nz, const float* r,
                         const float* lnk, const float* cap, const float* target, double* loss,
                         float* grad_host, void* stream);
/* weight w multiplies the loss of frehg_unet_loss_grad and its gradients (default 1); training
 * sets w = 1 / mean((target / rms r)^2) per pair so that every pair's relative error counts
 * alike */
int frehg_unet_set_loss_weight(frehg_unet* net, float weight);
int frehg_unet_adam_step(frehg_unet* net, float lr, float beta1, float beta2, float eps,
                         void* stream);
/* floating-point operations of one forward application on an nx*ny*nz grid */
int frehg_unet_flops(int nx, int ny, int nz, double* flops);

/* Attach a network to an RE handle.  With pc_type "unet" ("unet-line") the head solves run
 * flexible CG inside the FP64 refinement loop (FP32 Krylov) with z = M r + NN(r, ln K, C),
 * M = I (the unit-diagonal Jacobi step) or the vertical-line solve.  The first solve after
 * attaching runs the network-free method (Jacobi- or line-PCG) and sets the fallback
 * threshold: a solve whose FCG iterations exceed twice that count continues without the
 * network.  net = NULL detaches. */
int frehg_re_attach_unet(frehg_re* re, frehg_unet* net);
/* Time policy of the learned preconditioner: every probe_every-th solve applies the network;
 * if that solve took longer than max_ratio times the last network-free solve, the solves up to
 * the next probe run without it, otherwise the network stays on.  A probe is skipped (the
 * network stays off) when one network application, timed once per attach, already takes longer
 * than max_ratio times the last network-free solve.  probe_every = 0 applies the network on
 * every solve (no time policy).  Defaults: 32, 1.0. */
int frehg_re_set_learned_policy(frehg_re* re, int probe_every, double max_ratio);
/* Picard assembly staged through the Tensor Memory Accelerator (not in reference): on = 1
 * stages the float-float assembly's inputs with cp.async.bulk.tensor into a shared-memory ring
 * (mixed-precision Picard handles with a per-cell Ks field and an even nx; other cases keep the
 * unstaged kernel).  Both kernels write the same bits; the unstaged one is the default because
 * the assembly is bound by float-float instruction issue, not by memory (the staged kernel moves
 * fewer DRAM bytes but runs about 5 % longer on GB300). */
int frehg_re_set_assembly_staging(frehg_re* re, int on);
/* Not in reference: frehg_cg_set_fused_iteration for the handle's FP64 Jacobi-PCG solves. */
int frehg_re_set_fused_iteration(frehg_re* re, int on);
/* Training pairs from the plain solver: assembles the next PCA step's system at the current
 * state (nothing advances), solves it with FP64 Jacobi-PCG, re-runs the iteration from zero and
 * at each iteration number iters[q] (increasing) stores the scaled residual r~ and a target
 * as FP32 into r_out + q*n, t_out + q*n; ln K (vertical) and C into lnk_out, cap_out.
 * target: 0 = the error x~* - x~, 1 = error - r~ (correction over the Jacobi step),
 * 2 = error - M^-1 r~ with M the vertical-line tridiagonal part of the scaled operator.
 * Device pointers, n = nx*ny*nz. */
int frehg_re_training_pairs(frehg_re* re, int npairs, const int* iters, int target,
                            float* r_out, float* t_out, float* lnk_out, float* cap_out);

/* Allocation-free CG solve.  No counterpart in the reference: it exists for callers that may
 * not allocate GPU memory themselves (a component under a host framework that owns the device
 * memory budget, or a time-critical loop that cannot take cudaMalloc's synchronisation).  The
 * caller passes device arrays only: the operator in owned order (diag; a_k, a_i, a_j = coupling
 * of each row with its k+1, i+1, j+1 neighbour, 0 where that neighbour is absent), b and x.
 * The solver's work space is one fixed device array inside the library, so:
 *   - at most 262,144 unknowns (nx*ny*nz); larger systems get FREHG_ERR_BAD_ARG;
 *   - every GPU that loads the library keeps that array (17,302,016 bytes, about 17.3 MB or
 *     16.5 MiB) until the process ends;
 *   - each call looks up the array's address on the current device; the first call on a
 *     device loads the library's device code there -- make it before any stream capture on
 *     the device;
 *   - all calls share the array: calls that overlap on the GPU race; serialise them;
 *   - no cudaMalloc, cudaFree or other allocating routine is called.
 * stream: cudaStream_t as void* (NULL = the legacy default stream).  Same stopping rule,
 * iteration count and residual norm as frehg_cg_solve in its three-kernel form
 * (frehg_cg_set_fused_iteration 0; Jacobi-PCG, PETSc semantics). */
int frehg_cg_solve_noalloc(int nx, int ny, int nz, const double* diag, const double* a_k,
                           const double* a_i, const double* a_j, const double* b, double* x,
                           const frehg_solver_config* cfg, void* stream, int* its,
                           double* rnorm);

/* Surface-water exchange through the top face, the groundwater side of Coupling::exchange
 * (src/coupling/Coupling.cpp:25-166) for a caller that owns the surface solver: per column
 * (index i + j*nx) the rate q = Az Ks_z visc (h_top - dept) / (dz/2) from the top cell's head
 * and the ponded depth dept = max(eta - bottom, 0) (no infiltration below min_depth), limited by
 * the ponded volume and the top cell's headroom (q < 0, infiltration) or drainable water
 * (q > 0, seepage); then eta += q dt / Az and the top cell's water content -= q dt / V (clamped
 * to [theta_r, theta_s], head from the water content).  Uses the handle's uniform soil
 * parameters, as the reference does.  eta is updated in place; q_out receives the limited
 * rates [m^3/s]; *total = sum q dt.  Host arrays, or device arrays with on_device != 0. */
int frehg_re_surface_exchange(frehg_re* re, double* eta, const double* bottom, double dt,
                              double visc, double min_depth, double* q_out, double* total,
                              int on_device);

/* Checkpoint and restart of the step state (the groundwater part of writeCheckpointNow /
 * loadCheckpointState, src/driver/Orchestrator.cpp:1461-1502, 688-747: the field state plus
 * primeAdaptiveDt).  h and wc are host arrays of nx*ny*nz values in interior order (the only
 * fields the next step reads; every other device array is recomputed by the step);
 * state[FREHG_CHECKPOINT_SCALARS] = {time, dt, dtn, dt_used, top inflow volume, bottom inflow
 * volume, elastic volume, ghosts written (1/0), the mixed-precision refinement's first residual
 * norms of the last first and later solves (the next solves' right-hand-side scales)}.  A
 * handle with the same parameters, soil, solver and top flux field restarted from a checkpoint
 * steps exactly like the run that wrote it (bit for bit).  Checkpoint between steps: between a
 * surface exchange and the next step the top layer's pre-exchange ghost copies are not part of
 * the state, and the checkpoint returns FREHG_ERR_STATE. */
#define FREHG_CHECKPOINT_SCALARS 10
int frehg_re_checkpoint(frehg_re* re, double* h, double* wc, double* state);
int frehg_re_restart(frehg_re* re, const double* h, const double* wc, const double* state);

/* Build information: returns the sm architecture the library was compiled for (e.g. 103). */
int frehg_build_arch(void);

/* Self-check of the library's elementary functions (not in reference): y[i] = f(x[i]) for
 * host arrays of n values, f = the library's FP64 exp, log, log1p, expm1 (fn 0-3) as used by
 * the constitutive kernels, the CUDA math library's (fn 4-7) for comparison, or the
 * float-float exp, log, log1p, expm1 (fn 8-11), the double -> float-float -> double round trip
 * (fn 12) and the float-float reciprocal (fn 13), each with the argument split from a double
 * and the result summed back into one. */
int frehg_fastmath_eval(int fn, const double* x, double* y, int64_t n);

/* Self-check of the constitutive evaluation (not in reference): K/Ks, theta and C at n heads
 * (host arrays) for one soil, by the FP64 forms (arith 0) or the float-float forms of the
 * Picard kernels (arith 1); continuous_theta 1 drops the air-entry switch of theta as the
 * Picard scheme does. */
int frehg_constit_eval(const frehg_soil_params* soil, int arith, int continuous_theta,
                       const double* h, int64_t n, double* kr, double* wc, double* cap);

/* Self-check of the network's tensor-core convolutions (not in reference): one 3x3x3
 * convolution of cin -> cout channels (a shape the network uses) on seeded random BF16 inputs,
 * by the tcgen05 kernel the network runs and by a warp-level mma.sync kernel; stores the largest
 * absolute difference of the two BF16 outputs and the largest output magnitude.  in_stride /
 * out_stride and in_off / out_off select channel slices of wider pixel records, as the
 * network's concatenations do. */
int frehg_unet_conv_check(int cin, int cout, int in_stride, int in_off, int out_stride,
                          int out_off, int nx, int ny, int nz, int relu, uint64_t seed,
                          double* max_diff, double* max_ref);

/* Self-check of the TMA-staged Picard assembly (not in reference): on the handle's current
 * state (a Picard handle in mixed precision, soil with a per-cell Ks field, even nx -- the case
 * the step stages through the Tensor Memory Accelerator), assembles the system once with the
 * staged kernel and once with the unstaged float-float kernel and stores the number of matrix
 * and right-hand-side entries whose bits differ in *mismatches (0: identical).  Returns
 * FREHG_ERR_UNSUPPORTED when the handle's case does not take the staged kernel. */
int frehg_re_check_staged_assembly(frehg_re* re, int64_t* mismatches);
/* Self-check of the staged assembly's bounded waits (not in reference): one launch whose
 * producer warp issues no copies, so every consumer's first wait on a stage runs out (after
 * about a second); the blocks finish without reading a stage, *err_word receives the kernel's
 * error word (2: a consumer's wait ran out) and the handle's word is cleared, so the handle
 * steps normally afterwards.  Same handles as frehg_re_check_staged_assembly. */
int frehg_re_check_staged_wait(frehg_re* re, int* err_word);

#ifdef __cplusplus
}
#endif

#endif /* FREHG_GB300_H */
