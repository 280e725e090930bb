// Decomp3D of the C++ mirror on the CPU (no library, no GPU): the checks of the reference's
// tests/linear/test_decomp_3d.cpp:23-154 for one rank -- the global numbering is a bijection onto
// 0..n-1 with k fastest, the owned range covers it, the STAR stencil has 7 / 6 / 5 / 4 columns
// in the interior / on faces / edges / corners in the reference's order, z stays on the rank,
// ownedRowStencil agrees with stencilColumns, and pack / unpack round-trip a halo field.
#include <cstdio>
#include <vector>

#include "frehg_gb300.hpp"

static int failures = 0;
#define EXPECT(cond, ...)                 \
  do {                                    \
    if (!(cond)) {                        \
      ++failures;                         \
      std::printf("FAIL " __VA_ARGS__);   \
      std::printf("\n");                  \
    }                                     \
  } while (0)

int main() {
  namespace g = frehg_gb300;
  const int nx = 5, ny = 4, nz = 6;
  g::Decomp3D d(nx, ny, nz);
  const long n = d.globalRowCount();
  EXPECT(n == (long)nx * ny * nz, "row count %ld", n);
  EXPECT(d.ownershipRange().first == 0 && d.ownershipRange().second == n, "ownership range");
  std::vector<int> seen((size_t)n, 0);
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i)
      for (int k = 0; k < nz; ++k) {
        const long r = d.globalRow(i, j, k);
        EXPECT(r >= 0 && r < n, "row out of range");
        if (r >= 0 && r < n) seen[(size_t)r] += 1;
        if (k + 1 < nz) EXPECT(d.globalRow(i, j, k + 1) == r + 1, "k is the fastest index");
      }
  for (long r = 0; r < n; ++r)
    EXPECT(seen[(size_t)r] == 1, "row %ld numbered %d times", r, seen[(size_t)r]);
  long hist[8] = {0};
  for (long L = 0; L < n; ++L) {
    long row = -1, cols[7];
    int nc = 0;
    d.ownedRowStencil(L, row, cols, nc);
    EXPECT(row == L, "owned row %ld maps to %ld", L, row);
    const int k = (int)(L % nz), i = (int)((L / nz) % nx), j = (int)(L / ((long)nz * nx));
    long c2[7];
    int n2 = 0;
    d.stencilColumns(i, j, k, c2, n2);
    EXPECT(n2 == nc, "stencil sizes agree");
    for (int q = 0; q < nc && q < n2; ++q) EXPECT(cols[q] == c2[q], "stencil columns agree");
    EXPECT(cols[0] == row, "centre first");
    // the reference's order: W, E, S, N, Up, Down among those present
    long expect[7];
    int ne = 0;
    expect[ne++] = row;
    if (i > 0) expect[ne++] = d.globalRow(i - 1, j, k);
    if (i + 1 < nx) expect[ne++] = d.globalRow(i + 1, j, k);
    if (j > 0) expect[ne++] = d.globalRow(i, j - 1, k);
    if (j + 1 < ny) expect[ne++] = d.globalRow(i, j + 1, k);
    if (k > 0) expect[ne++] = row - 1;
    if (k + 1 < nz) expect[ne++] = row + 1;
    EXPECT(ne == nc, "column count");
    for (int q = 0; q < ne && q < nc; ++q) EXPECT(cols[q] == expect[q], "column order");
    if (nc >= 1 && nc <= 7) hist[nc] += 1;
  }
  // 7-point counts: interior 3x2x4 = 24 of 7, faces, edges, 8 corners of 4
  EXPECT(hist[7] == (long)(nx - 2) * (ny - 2) * (nz - 2), "interior rows %ld", hist[7]);
  EXPECT(hist[4] == 8, "corner rows %ld", hist[4]);
  EXPECT(hist[5] == 4L * ((nx - 2) + (ny - 2) + (nz - 2)), "edge rows %ld", hist[5]);
  EXPECT(hist[6] == 2L * ((nx - 2) * (ny - 2) + (nx - 2) * (nz - 2) + (ny - 2) * (nz - 2)),
         "face rows %ld", hist[6]);
  // pack / unpack between the halo layout and the owned vector
  std::vector<double> halo((size_t)d.localHaloFieldSize(), -1.0), owned, back;
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) halo[(size_t)d.haloIndex(i, j, k)] = 100.0 * k + 10.0 * j + i;
  d.packOwned(halo, owned);
  EXPECT((long)owned.size() == n, "owned size");
  EXPECT(owned[(size_t)d.globalRow(3, 2, 4)] == 423.0, "packed value");
  d.unpackOwned(owned, back);
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i)
        EXPECT(back[(size_t)d.haloIndex(i, j, k)] == halo[(size_t)d.haloIndex(i, j, k)],
               "round trip at %d %d %d", i, j, k);
  if (failures == 0) std::printf("ALL OK\n");
  return failures == 0 ? 0 : 1;
}
