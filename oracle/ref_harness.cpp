// TEST INFRASTRUCTURE, NOT PRODUCT CODE.
//
// Harness that drives the reference's OWN groundwater step -- src/re/ReSolver.cpp,
// src/re/VanGenuchten.hpp, src/linear/DomainDecomposition.cpp, src/core/Grid.cpp,
// src/core/MpiComm.cpp and src/soil/SoilMap.cpp, compiled unchanged from the reference tree by
// oracle/build_ref.py -- through a small C API, so that tests can check this repository's CPU
// restatement (oracle/frehg_oracle.c) against the reference itself and write golden vectors
// from it.  Only tests and the fixture generator load the result (oracle/_ref/).
//
// What is not the reference's code:
//   * Kokkos and MPI are replaced by the single-threaded, single-rank shims in oracle/ref_shim/.
//   * PETSc is absent, so the LinearSolver / SparseSystem pair below (the seam of
//     include/frehg2/linear/LinearSolver.hpp:18-33 and SparseSystem.hpp:15-40) stores the
//     rows ReSolver::assembleAndSolve adds (ReSolver.cpp:576-616, MatSetValues ADD_VALUES,
//     KokkosPetscBridge.cpp:16-33) and solves them with the oracle's restatement of PETSc's
//     KSPSolve_CG + KSPConvergedDefault with PCJacobi / PCSOR (or_ksp_solve_stencil).  The
//     Krylov arithmetic is therefore pinned by the reference's linear-solver tests, not by this
//     harness; everything around it (assembly, boundary folds, corrector, reallocation, clamp,
//     adaptive dt, initial state) is the reference's code.
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "core/Grid.hpp"
#include "core/MpiComm.hpp"
#include "frehg2/linear/LinearSolver.hpp"
#include "frehg2/linear/SolverConfig.hpp"
#include "frehg2/linear/SparseSystem.hpp"
#include "linear/DomainDecomposition.hpp"
#include "re/ReSolver.hpp"
#include "re/VanGenuchten.hpp"
#include "soil/SoilMap.hpp"

extern "C" {
#include "frehg_oracle.h"
}

namespace {

using frehg2::real;

// Owned-order 7-point rows of one rank (Decomp3D: row = (j*nx + i)*nz + k), held as the
// oracle's fixed slots centre, W, E, S, N, Up (k-1), Down (k+1).
class HarnessSystem : public frehg2::SparseSystem {
 public:
  HarnessSystem(int nx, int ny, int nz)
      : nx_(nx), ny_(ny), nz_(nz), coef_(7u * nx * ny * nz, 0.0), b_(nx * ny * nz, 0.0) {}

  void preallocate(const frehg2::DecompBase&) override {}
  void beginAssembly() override {}
  void endAssembly() override {}

  void addRow(int row, int ncols, const int* cols, const real* vals) override {
    int i, j, k;
    ijk(row, i, j, k);
    for (int c = 0; c < ncols; ++c) {
      int ci, cj, ck;
      ijk(cols[c], ci, cj, ck);
      int slot = -1;
      if (ci == i && cj == j && ck == k) slot = 0;
      else if (cj == j && ck == k && ci == i - 1) slot = 1;
      else if (cj == j && ck == k && ci == i + 1) slot = 2;
      else if (ci == i && ck == k && cj == j - 1) slot = 3;
      else if (ci == i && ck == k && cj == j + 1) slot = 4;
      else if (ci == i && cj == j && ck == k - 1) slot = 5;
      else if (ci == i && cj == j && ck == k + 1) slot = 6;
      if (slot < 0) throw std::runtime_error("harness: column outside the 7-point stencil");
      coef_[7u * row + slot] += vals[c];  // ADD_VALUES
    }
  }
  void addCOO(const frehg2::IntArr1D& rows, const frehg2::IntArr1D& cols,
              const frehg2::RealArr1D& vals) override {
    for (std::size_t e = 0; e < rows.size(); ++e) addRow(rows(e), 1, &cols(e), &vals(e));
  }
  void setRhs(const frehg2::RealArr1D& b) override {
    for (std::size_t r = 0; r < b_.size(); ++r) b_[r] = b(r);
  }
  void getSolution(frehg2::RealArr1D& x) override {
    for (std::size_t r = 0; r < x_.size(); ++r) x(r) = x_[r];
  }
  void zeroEntries() override { std::fill(coef_.begin(), coef_.end(), 0.0); }

  int nx_, ny_, nz_;
  std::vector<double> coef_, b_, x_;

 private:
  void ijk(int row, int& i, int& j, int& k) const {
    k = row % nz_;
    const int t = row / nz_;
    i = t % nx_;
    j = t / nx_;
  }
};

class HarnessSolver : public frehg2::LinearSolver {
 public:
  explicit HarnessSolver(frehg2::SolverConfig cfg) : cfg_(std::move(cfg)) {}
  std::unique_ptr<frehg2::SparseSystem> createSystem(const frehg2::DecompBase& dd) override {
    const auto& d3 = dynamic_cast<const frehg2::Decomp3D&>(dd);
    const auto sz = d3.globalSize();
    return std::make_unique<HarnessSystem>(std::get<0>(sz), std::get<1>(sz), std::get<2>(sz));
  }
  void setup(frehg2::SparseSystem&) override {}
  void solve(frehg2::SparseSystem& A, const frehg2::RealArr1D& b, frehg2::RealArr1D& x) override {
    auto& s = dynamic_cast<HarnessSystem&>(A);
    s.setRhs(b);
    s.x_.assign(s.b_.size(), 0.0);
    int its = 0;
    double rn = 0.0;
    const int reason = or_ksp_solve_stencil(s.nx_, s.ny_, s.nz_, s.coef_.data(), s.b_.data(),
                                            s.x_.data(), cfg_.ksp_type.c_str(),
                                            cfg_.pc_type.c_str(), cfg_.rtol, cfg_.atol,
                                            cfg_.max_it, &its, &rn);
    if (reason < 0)  // PetscLinearSolver.cpp:206-211
      throw std::runtime_error("harness solve: KSP diverged (reason " +
                               std::to_string(reason) + ")");
    its_ = its;
    rnorm_ = rn;
    total_its_ += its;
    s.getSolution(x);
  }
  int getIterationCount() const override { return its_; }
  real getResidualNorm() const override { return rnorm_; }

  frehg2::SolverConfig cfg_;
  int its_ = 0;
  double rnorm_ = 0.0;
  long long total_its_ = 0;
};

frehg2::SoilParams to_ref(const frehg_soil_params& s) {
  frehg2::SoilParams r;
  r.alpha = s.alpha;
  r.n = s.n;
  r.theta_s = s.theta_s;
  r.theta_r = s.theta_r;
  r.Ks_x = s.Ks_x;
  r.Ks_y = s.Ks_y;
  r.Ks_z = s.Ks_z;
  r.Ss = s.Ss;
  r.use_vg = s.use_vg != 0;
  r.use_mvg = s.use_mvg != 0;
  r.air_entry = s.air_entry;
  return r;
}

}  // namespace

struct ref_re {
  int nx, ny, nz;
  frehg2::MpiComm mc;
  frehg2::Grid grid;
  frehg2::Decomp3D dd;
  frehg2::ReSolver re;
  frehg2::SoilParams base;
  std::vector<frehg2::SoilParams> classes;
  std::vector<int> class_index;
  int class_3d = 0;
  std::vector<double> Ks, alpha;
  frehg2::SoilMap map;
  std::unique_ptr<HarnessSolver> solver;
  std::string err;

  ref_re(int nx_, int ny_, int nz_, const frehg_re_params& p)
      : nx(nx_), ny(ny_), nz(nz_), mc(nx_, ny_, 1, 1), grid(nx_, ny_, nz_, p.dx, p.dy, p.dz),
        dd(mc, nz_), re(grid, &mc) {}

  // The per-cell soil the oracle derives from a class map and per-cell Ks / alpha fields,
  // expressed as the reference's fully heterogeneous 3D SoilMap (src/soil/SoilMap.hpp:28-92):
  // one class per cell when per-cell fields are set.
  void rebuild_map() {
    const bool fields = !Ks.empty() || !alpha.empty();
    if (classes.empty() && !fields) {
      re.setSoilMap(nullptr);
      return;
    }
    if (!fields) {
      map.setClasses(classes);
      if (class_3d)
        map.setClassIndex3D(nx, ny, nz, class_index);
      else
        map.setClassIndex(nx, ny, class_index);
    } else {
      const std::size_t n = static_cast<std::size_t>(nx) * ny * nz;
      std::vector<frehg2::SoilParams> per(n);
      std::vector<int> idx(n);
      for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
          for (int i = 0; i < nx; ++i) {
            const std::size_t c = static_cast<std::size_t>(i) + static_cast<std::size_t>(nx) * (j + static_cast<std::size_t>(ny) * k);
            frehg2::SoilParams s = base;
            if (!classes.empty())
              s = classes[class_3d ? class_index[c] : class_index[i + static_cast<std::size_t>(nx) * j]];
            if (!Ks.empty()) s.Ks_x = s.Ks_y = s.Ks_z = Ks[c];
            if (!alpha.empty()) s.alpha = alpha[c];
            per[c] = s;
            idx[c] = static_cast<int>(c);
          }
      map.setClasses(per);
      map.setClassIndex3D(nx, ny, nz, idx);
    }
    re.setSoilMap(&map);
  }
};

namespace {
int fail(ref_re* s, const std::exception& e) {
  s->err = e.what();
  return FREHG_ERR_STATE;
}
}  // namespace

extern "C" {

const char* ref_re_last_error(const ref_re* s) { return s->err.c_str(); }

ref_re* ref_re_create(int nx, int ny, int nz, const frehg_re_params* p) {
  if (p->scheme != 0) return nullptr;  // the reference realises the PCA step only
  for (int b = 0; b < 6; ++b)
    if (p->bc_type[b] < 0 || p->bc_type[b] > 2) return nullptr;
  try {
    auto* s = new ref_re(nx, ny, nz, *p);
    frehg2::ReParams rp;
    rp.soil = to_ref(p->soil);
    rp.dx = p->dx;
    rp.dy = p->dy;
    rp.dz = p->dz;
    rp.botz = p->botz;
    rp.dt = p->dt;
    rp.dt_min = p->dt_min;
    rp.dt_max = p->dt_max;
    rp.co_max = p->co_max;
    rp.adaptive_dt = p->adaptive_dt != 0;
    rp.use_corrector = p->use_corrector != 0;
    rp.use_full3d = p->use_full3d != 0;
    rp.follow_terrain = p->follow_terrain != 0;
    rp.sim_shallowwater = p->sim_shallowwater != 0;
    rp.baroclinic = p->baroclinic != 0;
    for (int b = 0; b < 6; ++b) rp.bc_type[b] = p->bc_type[b];
    rp.htop = p->htop;
    rp.hbot = p->hbot;
    rp.qtop = p->qtop;
    rp.qbot = p->qbot;
    s->base = rp.soil;
    s->re.setParams(rp);
    return s;
  } catch (const std::exception&) {
    return nullptr;
  }
}

void ref_re_destroy(ref_re* s) { delete s; }

int ref_re_set_soil_map(ref_re* s, const frehg_soil_params* classes, int nclass,
                        const int32_t* index, int is3d) {
  try {
    s->classes.clear();
    for (int c = 0; c < nclass; ++c) s->classes.push_back(to_ref(classes[c]));
    const std::size_t n = is3d ? static_cast<std::size_t>(s->nx) * s->ny * s->nz
                               : static_cast<std::size_t>(s->nx) * s->ny;
    s->class_index.assign(index, index + n);
    s->class_3d = is3d;
    s->rebuild_map();
    return FREHG_OK;
  } catch (const std::exception& e) {
    return fail(s, e);
  }
}

int ref_re_set_cell_fields(ref_re* s, const double* Ks, const double* alpha) {
  try {
    const std::size_t n = static_cast<std::size_t>(s->nx) * s->ny * s->nz;
    s->Ks.clear();
    s->alpha.clear();
    if (Ks) s->Ks.assign(Ks, Ks + n);
    if (alpha) s->alpha.assign(alpha, alpha + n);
    s->rebuild_map();
    return FREHG_OK;
  } catch (const std::exception& e) {
    return fail(s, e);
  }
}

int ref_re_attach_solver(ref_re* s, const frehg_solver_config* c) {
  try {
    frehg2::SolverConfig cfg;
    cfg.ksp_type = c->ksp_type;
    cfg.pc_type = c->pc_type;
    cfg.rtol = c->rtol;
    cfg.atol = c->atol;
    cfg.max_it = c->max_it;
    s->solver = std::make_unique<HarnessSolver>(cfg);
    s->re.attachSolver(*s->solver, s->dd);
    return FREHG_OK;
  } catch (const std::exception& e) {
    return fail(s, e);
  }
}

void ref_re_initialize_geometry(ref_re* s) { s->re.initializeGeometry(); }

int ref_re_set_initial_head(ref_re* s, const double* h) {
  try {
    s->re.setInitialHead(std::vector<double>(h, h + static_cast<std::size_t>(s->nx) * s->ny * s->nz));
    return FREHG_OK;
  } catch (const std::exception& e) {
    return fail(s, e);
  }
}

int ref_re_set_initial_water_content(ref_re* s, const double* wc) {
  try {
    s->re.setInitialWaterContent(
        std::vector<double>(wc, wc + static_cast<std::size_t>(s->nx) * s->ny * s->nz));
    return FREHG_OK;
  } catch (const std::exception& e) {
    return fail(s, e);
  }
}

void ref_re_finalize_initial_state(ref_re* s) { s->re.finalizeInitialState(); }
void ref_re_initialize_uniform_column(ref_re* s, double wc0) { s->re.initializeUniformColumn(wc0); }

int ref_re_set_top_flux_field(ref_re* s, const double* q) {
  try {
    s->re.setTopFluxField(std::vector<double>(q, q + static_cast<std::size_t>(s->nx) * s->ny));
    return FREHG_OK;
  } catch (const std::exception& e) {
    return fail(s, e);
  }
}

int ref_re_advance_step(ref_re* s) {
  try {
    s->re.advanceStep();
    return FREHG_OK;
  } catch (const std::exception& e) {
    s->err = e.what();
    return FREHG_ERR_NOT_CONVERGED;
  }
}

double ref_re_dt(const ref_re* s) { return s->re.dt(); }
double ref_re_dt_used(const ref_re* s) { return s->re.dtUsed(); }
void ref_re_set_dt(ref_re* s, double dt) { s->re.setDt(dt); }
void ref_re_prime_adaptive_dt(ref_re* s, double dt) { s->re.primeAdaptiveDt(dt); }
int ref_re_last_ksp_its(const ref_re* s) { return s->solver ? s->solver->its_ : 0; }
long long ref_re_total_ksp_its(const ref_re* s) { return s->solver ? s->solver->total_its_ : 0; }

// Copy one of GwFields::namedViews (src/re/GwFields.hpp:62-74), halo layout.
int ref_re_get_field(ref_re* s, const char* name, double* out) {
  for (auto& nv : s->re.fields().namedViews()) {
    if (nv.first == name) {
      const auto& v = *nv.second;
      std::memcpy(out, v.data(), sizeof(double) * v.size());
      return FREHG_OK;
    }
  }
  return FREHG_ERR_BAD_ARG;
}

// VanGenuchten (src/re/VanGenuchten.hpp:18-137), the reference's own functions.
double ref_vg_theta(const frehg_soil_params* s, double h) {
  return frehg2::VanGenuchten::waterContentFromHead(to_ref(*s), h);
}
double ref_vg_head(const frehg_soil_params* s, double wc) {
  return frehg2::VanGenuchten::headFromWaterContent(to_ref(*s), wc);
}
double ref_vg_capacity(const frehg_soil_params* s, double h) {
  return frehg2::VanGenuchten::specificMoistureCapacity(to_ref(*s), h);
}
double ref_vg_conductivity(const frehg_soil_params* s, double h, double Ks) {
  return frehg2::VanGenuchten::conductivityFromHead(to_ref(*s), h, Ks);
}
double ref_vg_dKdwc(const frehg_soil_params* s, double wc, double Ks) {
  return frehg2::VanGenuchten::dKdwc(to_ref(*s), wc, Ks);
}

}  // extern "C"
