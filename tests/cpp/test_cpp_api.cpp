// C++ host interface end to end on the GPU (include/frehg_gb300.hpp): the linear-solver seam on
// a manufactured 3D Laplacian (the reference's PETSc boundary test, tests/linear/
// test_petsc_linear_solver.cpp:70-102, asks for L2 error < 1e-9), its error behaviour, and the
// ReSolver interface on the closed heterogeneous box of tests/re/test_re_3d.cpp:210-227 (water
// volume conserved to 1e-10 relative).  Prints one line per check; exit status 0 when all pass.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "frehg_gb300.hpp"

namespace g = frehg_gb300;

static int failures = 0;
#define EXPECT(cond, ...)                                  \
  do {                                                     \
    if (cond) {                                            \
      std::printf("ok   ");                                \
    } else {                                               \
      std::printf("FAIL ");                                \
      ++failures;                                          \
    }                                                      \
    std::printf(__VA_ARGS__);                              \
    std::printf("\n");                                     \
  } while (0)

// 7-point SPD operator: Laplacian with unit spacings on an nx x ny x nz box, zero Dirichlet
// values outside (diagonal 6 everywhere), rows in owned order row = (j*nx + i)*nz + k.
static void assemble_laplacian(g::SparseSystem& A, const g::Decomp3D& d) {
  A.beginAssembly();
  for (int j = 0; j < d.ny; ++j)
    for (int i = 0; i < d.nx; ++i)
      for (int k = 0; k < d.nz; ++k) {
        const int row = (int)d.globalRow(i, j, k);
        int cols[7];
        double vals[7];
        int n = 0;
        cols[n] = row;
        vals[n++] = 6.0;
        if (i > 0) { cols[n] = (int)d.globalRow(i - 1, j, k); vals[n++] = -1.0; }
        if (i + 1 < d.nx) { cols[n] = (int)d.globalRow(i + 1, j, k); vals[n++] = -1.0; }
        if (j > 0) { cols[n] = (int)d.globalRow(i, j - 1, k); vals[n++] = -1.0; }
        if (j + 1 < d.ny) { cols[n] = (int)d.globalRow(i, j + 1, k); vals[n++] = -1.0; }
        if (k > 0) { cols[n] = row - 1; vals[n++] = -1.0; }
        if (k + 1 < d.nz) { cols[n] = row + 1; vals[n++] = -1.0; }
        A.addRow(row, n, cols, vals);
      }
  A.endAssembly();
}

static std::vector<double> apply_laplacian(const std::vector<double>& x, const g::Decomp3D& d) {
  std::vector<double> y(x.size(), 0.0);
  for (int j = 0; j < d.ny; ++j)
    for (int i = 0; i < d.nx; ++i)
      for (int k = 0; k < d.nz; ++k) {
        const long r = d.globalRow(i, j, k);
        double v = 6.0 * x[r];
        if (i > 0) v -= x[d.globalRow(i - 1, j, k)];
        if (i + 1 < d.nx) v -= x[d.globalRow(i + 1, j, k)];
        if (j > 0) v -= x[d.globalRow(i, j - 1, k)];
        if (j + 1 < d.ny) v -= x[d.globalRow(i, j + 1, k)];
        if (k > 0) v -= x[r - 1];
        if (k + 1 < d.nz) v -= x[r + 1];
        y[r] = v;
      }
  return y;
}

static void seam(const char* precision, const char* pc = "jacobi") {
  g::Decomp3D d(12, 10, 8);
  g::SolverConfig cfg;
  cfg.rtol = 1e-12;
  cfg.precision = precision;
  cfg.pc_type = pc;
  cfg.ir_rtol = 1e-13;
  auto ls = g::makeLinearSolver("gb300", cfg);
  auto A = ls->createSystem(d);
  A->preallocate(d);
  assemble_laplacian(*A, d);
  std::vector<double> xe(d.nOwned());
  for (int j = 0; j < d.ny; ++j)
    for (int i = 0; i < d.nx; ++i)
      for (int k = 0; k < d.nz; ++k)
        xe[d.globalRow(i, j, k)] = std::sin(0.3 * i + 1.0) * std::cos(0.2 * j) * (1.0 + 0.1 * k);
  const std::vector<double> b = apply_laplacian(xe, d);
  std::vector<double> x;
  ls->setup(*A);
  ls->solve(*A, b, x);
  double e2 = 0.0, n2 = 0.0;
  for (size_t q = 0; q < xe.size(); ++q) {
    e2 += (x[q] - xe[q]) * (x[q] - xe[q]);
    n2 += xe[q] * xe[q];
  }
  const double rel = std::sqrt(e2 / n2);
  EXPECT(rel < 1e-9, "seam %s %s: manufactured Laplacian relative L2 error %.3e (%d iterations)",
         precision, pc, rel, ls->getIterationCount());
  // getSolution returns the last solve's x
  std::vector<double> x2;
  A->getSolution(x2);
  double d2 = 0.0;
  for (size_t q = 0; q < x.size(); ++q) d2 = std::fmax(d2, std::fabs(x2[q] - x[q]));
  EXPECT(d2 == 0.0, "seam %s %s: getSolution equals the solve's x", precision, pc);
  if (!std::strcmp(precision, "fp64") && !std::strcmp(pc, "jacobi")) {
    // the same solve as three kernels per iteration instead of one cooperative launch
    auto* gls = dynamic_cast<g::GpuLinearSolver*>(ls.get());
    EXPECT(gls != nullptr, "makeLinearSolver(\"gb300\") gives a GpuLinearSolver");
    if (!gls) return;
    const int its1 = ls->getIterationCount();
    std::vector<double> x3;
    gls->setFusedIteration(0);
    ls->solve(*A, b, x3);
    double dmax = 0.0;
    for (size_t q = 0; q < x.size(); ++q) dmax = std::max(dmax, std::fabs(x3[q] - x[q]));
    EXPECT(std::abs(ls->getIterationCount() - its1) <= 1 && dmax < 1e-10,
           "seam: one-launch and three-kernel iterations agree (%d / %d iterations, %.1e)", its1,
           ls->getIterationCount(), dmax);
    gls->setFusedIteration(-1);
  }
}

static void errors() {
  bool thrown = false;
  try {
    g::makeLinearSolver("petsc", g::SolverConfig());
  } catch (const std::runtime_error&) {
    thrown = true;
  }
  EXPECT(thrown, "makeLinearSolver rejects a backend that is not built");
  thrown = false;
  try {
    g::SolverConfig c;
    c.pc_type = "gamg";
    g::makeLinearSolver("gb300", c);
  } catch (const std::invalid_argument&) {
    thrown = true;
  }
  EXPECT(thrown, "pc_type gamg is rejected (std::invalid_argument)");
  thrown = false;
  try {
    auto ls = g::makeLinearSolver("gb300", g::SolverConfig());
    g::Decomp3D d(4, 4, 4);
    auto A = ls->createSystem(d);
    A->beginAssembly();
    const int cols[2] = {0, 9};  // (0,0,0) and a cell that is not a 7-point neighbour
    const double vals[2] = {6.0, -1.0};
    A->addRow(0, 2, cols, vals);
  } catch (const std::invalid_argument&) {
    thrown = true;
  }
  EXPECT(thrown, "addRow rejects a column outside the 7-point stencil");
}

static void closed_box() {
  const int nx = 4, ny = 4, nz = 8;
  g::Grid grid(nx, ny, nz, 2.0, 1.0, 0.05);
  g::ReSolver re(grid), re2(grid);
  g::ReParams p;
  p.dx = 2.0;
  p.dy = 1.0;
  p.dz = 0.05;
  p.botz = -0.05 * nz;
  p.dt = 5.0;
  p.adaptive_dt = 0;
  p.use_corrector = 1;
  p.use_full3d = 1;
  for (int q = 0; q < 6; ++q) p.bc_type[q] = 0;
  p.soil.alpha = 2.0;
  p.soil.n = 1.6;
  p.soil.theta_s = 0.45;
  p.soil.theta_r = 0.05;
  p.soil.Ks_x = p.soil.Ks_y = p.soil.Ks_z = 1.0e-5;
  p.soil.Ss = 0.0;
  g::SolverConfig cfg;
  cfg.rtol = 1e-13;
  auto ls = g::makeLinearSolver("gb300", cfg);
  auto ls2 = g::makeLinearSolver("gb300", cfg);
  g::Decomp3D dd(nx, ny, nz);
  std::vector<double> wc((size_t)nx * ny * nz);
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i)
        wc[i + nx * (j + ny * k)] = 0.20 + 0.03 * std::sin(0.9 * i) + 0.02 * std::cos(0.7 * j);
  for (g::ReSolver* r : {&re, &re2}) {
    r->setParams(p);
    r->attachSolver(r == &re ? *ls : *ls2, dd);
    r->initializeGeometry();
    r->setInitialWaterContent(wc);
    r->finalizeInitialState();
  }
  const double v0 = re.waterVolume();
  for (int s = 0; s < 39; ++s) re.advanceStep();
  // the last step's result copied while one more step runs: the copy holds the state before it
  std::vector<double> h_async((size_t)nx * ny * nz);
  const std::vector<double> h_before = re.interior("h");
  re.interiorAsync("h", h_async.data());
  re.advanceStep();
  re.sync();
  EXPECT(h_async == h_before, "interiorAsync: the copy holds the result of the step it follows");
  const double v1 = re.waterVolume();
  const double rel = std::fabs(v1 - v0) / v0;
  EXPECT(rel < 1e-10, "ReSolver closed box: water volume drift %.3e relative over 40 steps", rel);
  const std::vector<double> h = re.fields().h();
  EXPECT((long)h.size() == grid.nCell(), "fields().h() in the halo layout (%zu values)",
         h.size());
  EXPECT(std::isfinite(h[grid.getIndex(1, 2, 3)]) && re.dtUsed() == 5.0,
         "fields() readable, dtUsed %.1f", re.dtUsed());

  // the reference's checkpoint record (namedViews in the halo layout, dt) restarts a second
  // solver, which then steps exactly like the first
  const auto views = re.fields().namedViews();
  EXPECT(views.size() == 17 && views[0].first == "h" && views[2].first == "wc" &&
             (long)views[0].second.size() == grid.nCell() && views[0].second == h,
         "fields().namedViews(): %zu named halo arrays", views.size());
  re2.restartFromFields(views[0].second, views[2].second, re.dt());
  for (int s = 0; s < 2; ++s) {
    re.advanceStep();
    re2.advanceStep();
  }
  EXPECT(re.interior("h") == re2.interior("h") && re.interior("wc") == re2.interior("wc"),
         "restartFromFields: two more steps equal the continuous run's bit for bit");
  bool threw = false;
  try {
    re2.restartFromFields(std::vector<double>(3), views[2].second, re.dt());
  } catch (const std::runtime_error&) {
    threw = true;
  }
  EXPECT(threw, "restartFromFields refuses a record of another grid");
  const double v1b = re.waterVolume();

  // ponded water on half the columns infiltrates through the top face: the surface loses what
  // the soil gains
  std::vector<double> eta((size_t)nx * ny), bottom((size_t)nx * ny, 0.0), q;
  for (size_t c = 0; c < eta.size(); ++c) eta[c] = (c % 2) ? 0.004 : 0.0;
  double surf0 = 0.0, surf1 = 0.0;
  for (double e : eta) surf0 += e * 2.0 * 1.0;
  const double total = re.surfaceExchange(eta, bottom, 5.0, 1.0, 0.0, &q);
  for (double e : eta) surf1 += e * 2.0 * 1.0;
  const double v2 = re.waterVolume();
  EXPECT(total < 0.0 && q.size() == eta.size() && q[0] == 0.0 && q[1] < 0.0,
         "surfaceExchange: infiltration where ponded (total %.3e m^3)", total);
  const double bal = std::fabs((surf1 - surf0) + (v2 - v1b)) / std::fabs(total);
  EXPECT(bal < 1e-10 && std::fabs((surf0 - surf1) + total) < 1e-15,
         "surfaceExchange conserves water: imbalance %.3e of the exchanged volume", bal);
}

int main() {
  try {
    seam("fp64");
    seam("mixed");
    seam("fp64", "sor");
    errors();
    closed_box();
  } catch (const std::exception& e) {
    std::printf("FAIL unexpected exception: %s\n", e.what());
    return 2;
  }
  if (failures == 0) std::printf("ALL OK\n");
  return failures == 0 ? 0 : 1;
}
