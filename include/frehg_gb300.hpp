// C++17 host interface over the C ABI of frehg_gb300.h: the reference's linear-solver seam
// (LinearSolver / SparseSystem / SolverConfig / makeLinearSolver, include/frehg2/linear/
// LinearSolver.hpp:18-33, SparseSystem.hpp:15-40, SolverConfig.hpp:14-20,
// src/linear/backends/LinearSolverFactory.cpp:9-16) and its groundwater solver (ReSolver,
// src/re/ReSolver.hpp:48-105), with the same method names and argument meanings.
//
// Arrays are std::vector<double> where the reference passes Kokkos views (RealArr1D) or
// std::vector; b and x of the seam are in the owned order of one rank, row = (j*nx + i)*nz + k
// (src/linear/DomainDecomposition.cpp:109-119).  Errors are thrown as std::runtime_error with
// the library's message, as the reference's backends throw (PetscLinearSolver.cpp:206-211);
// configurations the GPU path does not realise throw std::invalid_argument.
//
// Header only; link with -lfrehg_gb300.
#pragma once

#include <cstdio>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "frehg_gb300.h"

namespace frehg_gb300 {

using real = double;

inline void check(int rc, const char* what) {
  if (rc == FREHG_OK) return;
  const std::string msg = std::string(what) + ": " + frehg_last_error();
  if (rc == FREHG_ERR_UNSUPPORTED || rc == FREHG_ERR_BAD_ARG) throw std::invalid_argument(msg);
  throw std::runtime_error(msg);
}

// ---- configuration types -----------------------------------------------------------------

// struct SolverConfig (SolverConfig.hpp:14-20) plus the precision keys of this backend.
struct SolverConfig {
  std::string ksp_type = "cg";      // cg | fcg
  std::string pc_type = "jacobi";   // jacobi | sor (fp64) | line | unet | unet-line
  real rtol = 1e-8;
  real atol = 1e-50;
  int max_it = 10000;
  std::string precision = "fp64";   // fp64 | mixed (FP32 Krylov under FP64 refinement)
  real ir_rtol = 1e-10;             // refinement stop: true relative residual
  real inner_rtol = 1e-4;           // FP32 inner solve reduction

  frehg_solver_config raw() const {
    frehg_solver_config k;
    frehg_solver_config_default(&k);
    std::snprintf(k.ksp_type, sizeof k.ksp_type, "%s", ksp_type.c_str());
    std::snprintf(k.pc_type, sizeof k.pc_type, "%s", pc_type.c_str());
    k.rtol = rtol;
    k.atol = atol;
    k.max_it = max_it;
    if (precision != "fp64" && precision != "mixed")
      throw std::invalid_argument("SolverConfig: precision must be fp64 or mixed");
    k.precision = precision == "mixed" ? 1 : 0;
    k.ir_rtol = ir_rtol;
    k.inner_rtol = inner_rtol;
    return k;
  }
};

// struct SoilParams (include/frehg2/re/SoilParams.hpp:13-25) and struct ReParams
// (src/re/ReSolver.hpp:24-46): the C structs, initialised to the reference's defaults.
struct SoilParams : frehg_soil_params {
  SoilParams() { frehg_soil_params_default(this); }
};
struct ReParams : frehg_re_params {
  ReParams() { frehg_re_params_default(this); }
};

// Grid (src/core/Grid.hpp): interior sizes and spacings; getIndex is the halo-padded index
// of the reference, (i+1) + (j+1)(nx+2) + (k+1)(nx+2)(ny+2).
struct Grid {
  int nx = 1, ny = 1, nz = 1;
  real dx = 1.0, dy = 1.0, dz = 1.0;
  Grid() = default;
  Grid(int nx_, int ny_, int nz_, real dx_, real dy_, real dz_)
      : nx(nx_), ny(ny_), nz(nz_), dx(dx_), dy(dy_), dz(dz_) {}
  long nCell() const { return (long)(nx + 2) * (ny + 2) * (nz + 2); }
  long getIndex(int i, int j, int k) const {
    return (long)(i + 1) + (long)(j + 1) * (nx + 2) + (long)(k + 1) * (nx + 2) * (ny + 2);
  }
};

// Decomp3D of one rank (src/linear/DomainDecomposition.hpp:94-120, .cpp:109-185): the owned box
// of the one process whose global system the library solves.  Rows are numbered with k
// fastest, row = (j nx + i) nz + k; the STAR stencil's columns come in the reference's order
// (centre, W, E, S, N, Up, Down); packOwned / unpackOwned move between a halo-padded field
// ((nx+2)(ny+2)(nz+2), i fastest, Grid::getIndex) and the owned vector.
struct Decomp3D {
  int nx = 1, ny = 1, nz = 1;
  Decomp3D() = default;
  Decomp3D(int nx_, int ny_, int nz_) : nx(nx_), ny(ny_), nz(nz_) {}
  long nOwned() const { return (long)nx * ny * nz; }
  long globalRowCount() const { return nOwned(); }
  std::pair<long, long> ownershipRange() const { return {0L, nOwned()}; }
  long globalRow(int i, int j, int k) const { return ((long)j * nx + i) * nz + k; }
  // centre and in-domain W, E, S, N, Up (k-1, toward the surface), Down (k+1); up to 7
  void stencilColumns(int i, int j, int k, long* cols, int& ncols) const {
    ncols = 0;
    cols[ncols++] = globalRow(i, j, k);
    if (i - 1 >= 0) cols[ncols++] = globalRow(i - 1, j, k);
    if (i + 1 < nx) cols[ncols++] = globalRow(i + 1, j, k);
    if (j - 1 >= 0) cols[ncols++] = globalRow(i, j - 1, k);
    if (j + 1 < ny) cols[ncols++] = globalRow(i, j + 1, k);
    if (k - 1 >= 0) cols[ncols++] = globalRow(i, j, k - 1);
    if (k + 1 < nz) cols[ncols++] = globalRow(i, j, k + 1);
  }
  void ownedRowStencil(long local, long& global_row, long* cols, int& ncols) const {
    const int k = (int)(local % nz);
    const long horiz = local / nz;
    const int i = (int)(horiz % nx), j = (int)(horiz / nx);
    global_row = globalRow(i, j, k);
    stencilColumns(i, j, k, cols, ncols);
  }
  long localHaloFieldSize() const { return (long)(nx + 2) * (ny + 2) * (nz + 2); }
  long haloIndex(int i, int j, int k) const {
    return (long)(i + 1) + (long)(j + 1) * (nx + 2) + (long)(k + 1) * (nx + 2) * (ny + 2);
  }
  void packOwned(const std::vector<double>& field_halo, std::vector<double>& owned) const {
    owned.resize((size_t)nOwned());
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i)
        for (int k = 0; k < nz; ++k)
          owned[(size_t)globalRow(i, j, k)] = field_halo[(size_t)haloIndex(i, j, k)];
  }
  void unpackOwned(const std::vector<double>& owned, std::vector<double>& field_halo) const {
    field_halo.resize((size_t)localHaloFieldSize(), 0.0);
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i)
        for (int k = 0; k < nz; ++k)
          field_halo[(size_t)haloIndex(i, j, k)] = owned[(size_t)globalRow(i, j, k)];
  }
};

// ---- linear-solver seam ------------------------------------------------------------------

class SparseSystem {
 public:
  virtual ~SparseSystem() = default;
  virtual void preallocate(const Decomp3D& dd) = 0;
  virtual void beginAssembly() = 0;
  virtual void endAssembly() = 0;
  virtual void addRow(int global_row, int ncols, const int* global_cols, const real* vals) = 0;
  virtual void addCOO(const std::vector<int>& rows, const std::vector<int>& cols,
                      const std::vector<real>& vals) = 0;
  virtual void setRhs(const std::vector<real>& b_owned) = 0;
  virtual void getSolution(std::vector<real>& x_owned) = 0;
  virtual void zeroEntries() = 0;
};

class LinearSolver {
 public:
  virtual ~LinearSolver() = default;
  virtual std::unique_ptr<SparseSystem> createSystem(const Decomp3D& dd) = 0;
  virtual void setup(SparseSystem& A) = 0;
  virtual void solve(SparseSystem& A, const std::vector<real>& b, std::vector<real>& x) = 0;
  virtual int getIterationCount() const = 0;
  virtual real getResidualNorm() const = 0;
};

// The 7-point stencil system of the GPU backend: addRow decodes a row into diagonal and
// +x/+y/+z couplings and rejects columns that are not 7-point neighbours; endAssembly checks
// symmetry.
class StencilSystem : public SparseSystem {
 public:
  StencilSystem(frehg_cg* cg, const Decomp3D& dd) : n_(dd.nOwned()) {
    check(frehg_system_create(cg, dd.nx, dd.ny, dd.nz, &sys_), "StencilSystem");
  }
  ~StencilSystem() override { frehg_system_destroy(sys_); }
  StencilSystem(const StencilSystem&) = delete;
  StencilSystem& operator=(const StencilSystem&) = delete;
  void preallocate(const Decomp3D&) override {}  // the stencil pattern is fixed
  void beginAssembly() override { check(frehg_system_begin_assembly(sys_), "beginAssembly"); }
  void endAssembly() override { check(frehg_system_end_assembly(sys_), "endAssembly"); }
  void addRow(int row, int ncols, const int* cols, const real* vals) override {
    check(frehg_system_add_row(sys_, row, ncols, cols, vals), "addRow");
  }
  void addCOO(const std::vector<int>& r, const std::vector<int>& c,
              const std::vector<real>& v) override {
    if (r.size() != v.size() || c.size() != v.size())
      throw std::invalid_argument("addCOO: rows, cols and vals differ in length");
    check(frehg_system_add_coo(sys_, r.data(), c.data(), v.data(), (long)v.size(), 0),
          "addCOO");
  }
  void setRhs(const std::vector<real>& b) override {
    size_check(b.size(), "setRhs");
    check(frehg_system_set_rhs(sys_, b.data(), 0), "setRhs");
  }
  void getSolution(std::vector<real>& x) override {
    x.resize(n_);
    check(frehg_system_get_solution(sys_, x.data(), 0), "getSolution");
  }
  void zeroEntries() override { check(frehg_system_zero_entries(sys_), "zeroEntries"); }
  frehg_system* raw() { return sys_; }
  long size() const { return n_; }

 private:
  void size_check(size_t n, const char* what) const {
    if ((long)n != n_) throw std::invalid_argument(std::string(what) + ": wrong length");
  }
  frehg_system* sys_ = nullptr;
  long n_ = 0;
};

class GpuLinearSolver : public LinearSolver {
 public:
  explicit GpuLinearSolver(const SolverConfig& cfg) : cfg_(cfg) {
    const frehg_solver_config k = cfg.raw();
    check(frehg_cg_create(&k, &cg_), "makeLinearSolver");
  }
  ~GpuLinearSolver() override { frehg_cg_destroy(cg_); }
  GpuLinearSolver(const GpuLinearSolver&) = delete;
  GpuLinearSolver& operator=(const GpuLinearSolver&) = delete;
  std::unique_ptr<SparseSystem> createSystem(const Decomp3D& dd) override {
    return std::make_unique<StencilSystem>(cg_, dd);
  }
  void setup(SparseSystem& A) override { check(frehg_cg_setup(cg_, sys(A).raw()), "setup"); }
  void solve(SparseSystem& A, const std::vector<real>& b, std::vector<real>& x) override {
    StencilSystem& s = sys(A);
    if ((long)b.size() != s.size()) throw std::invalid_argument("solve: wrong length of b");
    x.resize(b.size());
    check(frehg_cg_solve(cg_, s.raw(), b.data(), x.data(), 0), "solve");
  }
  int getIterationCount() const override {
    int its = 0;
    check(frehg_cg_iteration_count(cg_, &its), "getIterationCount");
    return its;
  }
  real getResidualNorm() const override {
    double r = 0.0;
    check(frehg_cg_residual_norm(cg_, &r), "getResidualNorm");
    return r;
  }
  const SolverConfig& config() const { return cfg_; }
  // not in reference: the FP64 Jacobi-PCG iteration as one cooperative launch (1), three
  // kernels (0) or, by default, one launch up to 65,536 unknowns (-1)
  void setFusedIteration(int on) { check(frehg_cg_set_fused_iteration(cg_, on), "setFusedIteration"); }

 private:
  static StencilSystem& sys(SparseSystem& A) {
    auto* s = dynamic_cast<StencilSystem*>(&A);
    if (!s) throw std::invalid_argument("GpuLinearSolver: system was not created by it");
    return *s;
  }
  SolverConfig cfg_;
  frehg_cg* cg_ = nullptr;
};

// makeLinearSolver (LinearSolverFactory.cpp:9-16): "gb300" is the only backend built here; an
// unknown or not-built backend throws as the reference's factory does.
inline std::unique_ptr<LinearSolver> makeLinearSolver(const std::string& backend,
                                                      const SolverConfig& cfg) {
  if (backend == "gb300") return std::make_unique<GpuLinearSolver>(cfg);
  throw std::runtime_error("makeLinearSolver: unknown / not-built linear-solver backend '" +
                           backend + "' (only 'gb300' is built here)");
}

// ---- groundwater solver ------------------------------------------------------------------

// SoilMap (src/soil/SoilMap.hpp:28-92): class table plus per-column (2D) or per-cell (3D)
// class ids in interior order (li + lj*nx [+ k*nx*ny]).
struct SoilMap {
  std::vector<frehg_soil_params> classes;
  std::vector<int32_t> index;
  bool is3d = false;
  void setClasses(std::vector<frehg_soil_params> c) {
    if (c.empty()) throw std::invalid_argument("SoilMap::setClasses: empty class table");
    classes = std::move(c);
  }
  void setClassIndex(int nx, int ny, std::vector<int32_t> idx) {
    if ((long)idx.size() != (long)nx * ny)
      throw std::invalid_argument("SoilMap::setClassIndex: size mismatch");
    index = std::move(idx);
    is3d = false;
  }
  void setClassIndex3D(int nx, int ny, int nz, std::vector<int32_t> idx) {
    if ((long)idx.size() != (long)nx * ny * nz)
      throw std::invalid_argument("SoilMap::setClassIndex3D: size mismatch");
    index = std::move(idx);
    is3d = true;
  }
};

// Host copies of the GPU fields in the reference's halo layout (GwFields.hpp:14-75), taken on
// demand: h, wc, hn, wcn, qx, qy, qz, kr, wch.
class GwFields {
 public:
  explicit GwFields(frehg_re* re, const Grid& g) : re_(re), g_(g) {}
  std::vector<real> get(const std::string& name) const {
    std::vector<real> out((size_t)g_.nCell());
    check(frehg_re_get_field(re_, name.c_str(), out.data()), "fields");
    return out;
  }
  std::vector<real> h() const { return get("h"); }
  std::vector<real> wc() const { return get("wc"); }
  // Every array the GPU state materialises, paired with its GwFields name, for the reference's
  // checkpoint writer (GwFields::namedViews, GwFields.hpp:62-74; Orchestrator::
  // writeCheckpointNow stores each as "gw_<name>").  The matrix and density arrays (G*, r_*)
  // are rewritten by every step before they are read and are not materialised.
  std::vector<std::pair<std::string, std::vector<real>>> namedViews() const {
    static const char* const names[] = {"h",  "hn", "wc", "wcn", "wch",  "hwc",  "ch",  "Kx", "Ky",
                                        "Kz", "qx", "qy", "qz",  "room", "bot3d", "dz3d", "actv"};
    std::vector<std::pair<std::string, std::vector<real>>> v;
    for (const char* n : names) v.emplace_back(n, get(n));
    return v;
  }

 private:
  frehg_re* re_;
  Grid g_;
};

class ReSolver {
 public:
  explicit ReSolver(const Grid& grid) : grid_(grid) {
    ReParams p;
    p.dx = grid.dx;
    p.dy = grid.dy;
    p.dz = grid.dz;
    check(frehg_re_create(grid.nx, grid.ny, grid.nz, &p, &re_), "ReSolver");
    params_ = p;
  }
  ~ReSolver() { frehg_re_destroy(re_); }
  ReSolver(const ReSolver&) = delete;
  ReSolver& operator=(const ReSolver&) = delete;

  void setParams(const ReParams& p) {
    check(frehg_re_set_params(re_, &p), "setParams");
    params_ = p;
  }
  const ReParams& params() const { return params_; }
  void setSoilMap(const SoilMap* map) {
    if (!map) throw std::invalid_argument("setSoilMap: null map");
    check(frehg_re_set_soil_map(re_, map->classes.data(), (int)map->classes.size(),
                                map->index.data(), map->is3d ? 1 : 0),
          "setSoilMap");
  }
  // attachSolver(LinearSolver&, Decomp3D&) (ReSolver.hpp:66): the GPU step assembles and
  // solves on the device, so it takes the backend's configuration from the gb300 solver.
  void attachSolver(LinearSolver& solver, Decomp3D& dd) {
    auto* g = dynamic_cast<GpuLinearSolver*>(&solver);
    if (!g) throw std::invalid_argument("attachSolver: the GPU ReSolver needs the gb300 backend");
    if (dd.nx != grid_.nx || dd.ny != grid_.ny || dd.nz != grid_.nz)
      throw std::invalid_argument("attachSolver: decomposition does not match the grid");
    const frehg_solver_config k = g->config().raw();
    check(frehg_re_attach_solver(re_, &k), "attachSolver");
  }
  void initializeUniformColumn(real init_wc) {
    check(frehg_re_initialize_uniform_column(re_, init_wc), "initializeUniformColumn");
  }
  void initializeGeometry() { check(frehg_re_initialize_geometry(re_), "initializeGeometry"); }
  void setInitialWaterContent(const std::vector<double>& wc) {
    size_check(wc.size(), "setInitialWaterContent");
    check(frehg_re_set_initial_water_content(re_, wc.data()), "setInitialWaterContent");
  }
  void setInitialHead(const std::vector<double>& h) {
    size_check(h.size(), "setInitialHead");
    check(frehg_re_set_initial_head(re_, h.data()), "setInitialHead");
  }
  void finalizeInitialState() {
    check(frehg_re_finalize_initial_state(re_), "finalizeInitialState");
  }
  void advanceStep() {
    check(frehg_re_advance_step(re_), "advanceStep");
    double dt = 0.0;
    check(frehg_re_dt(re_, &dt), "dt");
    params_.dt = dt;
  }
  GwFields fields() const { return GwFields(re_, grid_); }
  const Grid& grid() const { return grid_; }
  real dt() const { return params_.dt; }
  real dtUsed() const {
    double d = 0.0;
    check(frehg_re_dt_used(re_, &d), "dtUsed");
    return d;
  }
  void setDt(real dt) {
    check(frehg_re_set_dt(re_, dt), "setDt");
    params_.dt = dt;
  }
  void primeAdaptiveDt(real dt) {
    check(frehg_re_prime_adaptive_dt(re_, dt), "primeAdaptiveDt");
    params_.dt = dt;
  }
  void setTopFluxField(const std::vector<real>& q) {
    if ((long)q.size() != (long)grid_.nx * grid_.ny)
      throw std::invalid_argument("setTopFluxField: one value per owned column required");
    check(frehg_re_set_top_flux_field(re_, q.data()), "setTopFluxField");
  }
  // interior field in interior order (i fastest, k slowest), not in the reference
  std::vector<real> interior(const std::string& name) const {
    std::vector<real> out((size_t)grid_.nx * grid_.ny * grid_.nz);
    check(frehg_re_get_interior(re_, name.c_str(), out.data(), 0), "interior");
    return out;
  }
  // start the copy of an interior field into out (size nx*ny*nz, page-locked for asynchrony);
  // complete after sync(); the copy overlaps the next step (not in the reference)
  void interiorAsync(const std::string& name, real* out) {
    check(frehg_re_get_interior_async(re_, name.c_str(), out), "interiorAsync");
  }
  void sync() { check(frehg_re_sync(re_), "sync"); }
  real waterVolume() const {
    double v = 0.0;
    check(frehg_re_water_volume(re_, &v), "waterVolume");
    return v;
  }
  // checkpoint / restart of the step state (writeCheckpointNow / loadCheckpointState)
  struct Checkpoint {
    std::vector<real> h, wc;
    double state[FREHG_CHECKPOINT_SCALARS];
  };
  Checkpoint checkpoint() const {
    Checkpoint cp;
    cp.h.resize((size_t)grid_.nx * grid_.ny * grid_.nz);
    cp.wc.resize(cp.h.size());
    check(frehg_re_checkpoint(re_, cp.h.data(), cp.wc.data(), cp.state), "checkpoint");
    return cp;
  }
  void restart(const Checkpoint& cp) {
    size_check(cp.h.size(), "restart");
    size_check(cp.wc.size(), "restart");
    check(frehg_re_restart(re_, cp.h.data(), cp.wc.data(), cp.state), "restart");
    params_.dt = cp.state[1];
  }
  // Restart from the reference's checkpoint record (the groundwater part of
  // Orchestrator::loadCheckpointState, Orchestrator.cpp:688-747): the gw_h and gw_wc arrays in
  // the halo layout (the arrays the next step reads; it recomputes the rest), then
  // primeAdaptiveDt(dt) and the record's time.  The head's ghost layer tells whether a step
  // has run (its enforceHeadBc wrote it; the first step after an initial state reads zeros).
  void restartFromFields(const std::vector<real>& h_halo, const std::vector<real>& wc_halo,
                         real dt, real time = 0.0) {
    if ((long)h_halo.size() != grid_.nCell() || (long)wc_halo.size() != grid_.nCell())
      throw std::runtime_error(
          "checkpoint load: field size mismatch (grid differs from checkpoint)");
    Checkpoint cp;
    const size_t n = (size_t)grid_.nx * grid_.ny * grid_.nz;
    cp.h.resize(n);
    cp.wc.resize(n);
    size_t q = 0;
    for (int k = 0; k < grid_.nz; ++k)
      for (int j = 0; j < grid_.ny; ++j)
        for (int i = 0; i < grid_.nx; ++i, ++q) {
          cp.h[q] = h_halo[(size_t)grid_.getIndex(i, j, k)];
          cp.wc[q] = wc_halo[(size_t)grid_.getIndex(i, j, k)];
        }
    bool ghosts = false;
    for (int k = -1; k <= grid_.nz && !ghosts; ++k)
      for (int j = -1; j <= grid_.ny && !ghosts; ++j)
        for (int i = -1; i <= grid_.nx; ++i) {
          const bool inner = i >= 0 && i < grid_.nx && j >= 0 && j < grid_.ny && k >= 0 &&
                             k < grid_.nz;
          if (!inner && h_halo[(size_t)grid_.getIndex(i, j, k)] != 0.0) {
            ghosts = true;
            break;
          }
        }
    for (double& v : cp.state) v = 0.0;
    cp.state[0] = time;
    cp.state[1] = cp.state[2] = cp.state[3] = dt;  // dt, dtn (primeAdaptiveDt), last dt
    cp.state[7] = ghosts ? 1.0 : 0.0;
    restart(cp);
  }
  // groundwater side of Coupling::exchange: eta (surface level per column, i + j*nx) is updated
  // in place, q (if given) receives the limited rates [m^3/s]; returns sum q dt
  real surfaceExchange(std::vector<real>& eta, const std::vector<real>& bottom, real dt,
                       real visc = 1.0, real minDepth = 0.0, std::vector<real>* q = nullptr) {
    const size_t ncol = (size_t)grid_.nx * grid_.ny;
    if (eta.size() != ncol || bottom.size() != ncol)
      throw std::invalid_argument("surfaceExchange: one value per owned column required");
    std::vector<real> rates(ncol);
    double total = 0.0;
    check(frehg_re_surface_exchange(re_, eta.data(), bottom.data(), dt, visc, minDepth,
                                    rates.data(), &total, 0),
          "surfaceExchange");
    if (q) *q = std::move(rates);
    return total;
  }
  frehg_re_counters counters() const {
    frehg_re_counters c;
    check(frehg_re_get_counters(re_, &c), "counters");
    return c;
  }
  frehg_re* raw() { return re_; }

 private:
  void size_check(size_t n, const char* what) const {
    if ((long)n != (long)grid_.nx * grid_.ny * grid_.nz)
      throw std::invalid_argument(std::string(what) + ": one value per interior cell required");
  }
  Grid grid_;
  ReParams params_;
  frehg_re* re_ = nullptr;
};

}  // namespace frehg_gb300
