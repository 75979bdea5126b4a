// CPU check of the single-instance SpMV's host plan builder (sell_plan.h):
// it plans seeded matrices -- a factor-model matrix (long rows cut into
// 32-entry pieces, a dense row split into thousands of pieces, rows of one
// entry, empty rows), a denser one, and a matrix of short rows (whole
// rows) -- checks every promise the kernels rely on, then runs the plan on
// the host the way the kernels do (one FMA chain per virtual row, split rows
// summed in piece order) and compares the product with a direct CSR
// product.
// Prints "OK" and exits 0, or prints the first failures and exits 1.
#include <cmath>
#include <cstdio>
#include <random>
#include <vector>

#include "sell_plan.h"

using namespace pdosgpu;

static int failures = 0;
#define CHECK(cond, ...)                   \
  do {                                     \
    if (!(cond)) {                         \
      if (failures < 20) {                 \
        std::printf("FAIL: " __VA_ARGS__); \
        std::printf("\n");                 \
      }                                    \
      ++failures;                          \
    }                                      \
  } while (0)

struct Csr {
  int32_t rows = 0, cols = 0;
  std::vector<int32_t> ptr{0}, col;
  std::vector<double> val;
  void add_row(std::vector<int32_t> c, std::mt19937 &g) {
    std::sort(c.begin(), c.end());
    c.erase(std::unique(c.begin(), c.end()), c.end());
    for (int32_t j : c) {
      col.push_back(j);
      val.push_back(std::uniform_real_distribution<double>(-1.0, 1.0)(g));
    }
    ptr.push_back((int32_t)col.size());
    ++rows;
  }
};

// factor rows: `k` rows with density `dens` over `n` columns, one dense
// budget row, `n` rows of one entry, a few empty rows
static Csr factor_matrix(int32_t n, int32_t k, double dens, uint32_t seed) {
  std::mt19937 g(seed);
  Csr A;
  A.cols = n + k + 1;
  std::vector<int32_t> all(n);
  for (int32_t j = 0; j < n; ++j) all[j] = j;
  A.add_row(all, g);  // budget row
  for (int32_t r = 0; r < k; ++r) {
    std::vector<int32_t> c;
    for (int32_t j = 0; j < n; ++j)
      if (std::uniform_real_distribution<double>(0.0, 1.0)(g) < dens) c.push_back(j);
    c.push_back(n + r);
    A.add_row(c, g);
  }
  A.add_row({}, g);
  for (int32_t j = 0; j < n; ++j) A.add_row({j}, g);
  A.add_row({}, g);
  A.add_row({n + k}, g);
  return A;
}

static Csr short_matrix(int32_t m, int32_t n, uint32_t seed) {
  std::mt19937 g(seed);
  Csr A;
  A.cols = n;
  for (int32_t r = 0; r < m; ++r) {
    const int len = (int)(g() % 40);
    std::vector<int32_t> c;
    for (int e = 0; e < len; ++e) c.push_back((int32_t)(g() % n));
    A.add_row(c, g);
  }
  return A;
}

static void check_plan(const char *name, const Csr &A) {
  SellHost h;
  h.build(A.ptr.data(), A.rows);
  const int64_t nnz = A.ptr[A.rows];
  CHECK(h.nvr % 32 == 0 && h.nslices == h.nvr / 32, "%s: slices", name);
  CHECK(h.slots == h.slice_off[h.nslices], "%s: slots", name);
  // every entry in exactly one slot, in its virtual row's lane
  std::vector<int> seen(nnz, 0);
  for (int32_t s = 0; s < h.nslices; ++s)
    for (int t = 0; t < 32; ++t) {
      const int32_t v = 32 * s + t;
      const int32_t w = (h.slice_off[s + 1] - h.slice_off[s]) / 32;
      CHECK(h.vr_len[v] <= w && h.vr_len[v] <= h.vrow, "%s: virtual row %d too long", name, v);
      for (int32_t e = 0; e < w; ++e) {
        const int32_t src = h.slot_src[(size_t)h.slice_off[s] + 32 * e + t];
        CHECK((src >= 0) == (e < h.vr_len[v]), "%s: slot of vrow %d step %d", name, v, e);
        if (src >= 0 && src < nnz) ++seen[src];
      }
    }
  for (int64_t i = 0; i < nnz; ++i) CHECK(seen[i] == 1, "%s: entry %lld placed %d times", name, (long long)i, seen[i]);
  // the virtual rows of a row cover its entries in order; split and heavy rows listed once
  std::vector<int> listed(A.rows, 0);
  for (int32_t r : h.split) ++listed[r];
  for (int32_t r : h.heavy) ++listed[r];
  for (size_t i = 0; i < h.heavy.size(); ++i)
    CHECK((h.vr_ptr[h.heavy[i] + 1] - h.vr_ptr[h.heavy[i]] > kGiantVrows) == ((int32_t)i < h.ngiant),
          "%s: giant rows first", name);
  for (int32_t r = 0; r < A.rows; ++r) {
    int32_t next = A.ptr[r];
    const int32_t nv = h.vr_ptr[r + 1] - h.vr_ptr[r];
    CHECK(nv >= 1, "%s: row %d without a virtual row", name, r);
    CHECK(listed[r] == (nv > 1 ? 1 : 0), "%s: row %d listed %d times as split or heavy", name, r, listed[r]);
    for (int32_t q = h.vr_ptr[r]; q < h.vr_ptr[r + 1]; ++q) {
      const int32_t p = h.vr_list[q], s = p / 32, t = p % 32;
      if (h.vr_len[p] > 0) CHECK(h.slot_src[(size_t)h.slice_off[s] + t] == next, "%s: row %d piece order", name, r);
      next += h.vr_len[p];
      CHECK(h.vr_row[p] == (nv == 1 ? r : -1), "%s: vr_row of row %d", name, r);
    }
    CHECK(next == A.ptr[r + 1], "%s: row %d pieces cover %d of %d entries", name, r, next - A.ptr[r],
          A.ptr[r + 1] - A.ptr[r]);
  }
  // run the plan on the host as the kernels do
  std::vector<double> x(A.cols), y(A.rows, 0.0), vsum(h.nvr, 0.0);
  std::mt19937 g(11);
  for (auto &v : x) v = std::uniform_real_distribution<double>(-1.0, 1.0)(g);
  for (int32_t s = 0; s < h.nslices; ++s)
    for (int t = 0; t < 32; ++t) {
      const int32_t v = 32 * s + t;
      double acc = 0.0;
      for (int32_t e = 0; e < h.vr_len[v]; ++e) {
        const int32_t src = h.slot_src[(size_t)h.slice_off[s] + 32 * e + t];
        acc = std::fma(A.val[src], x[A.col[src]], acc);
      }
      if (h.vr_row[v] >= 0)
        y[h.vr_row[v]] = acc;
      else
        vsum[v] = acc;
    }
  for (int32_t r = 0; r < A.rows; ++r) {
    if (h.vr_ptr[r + 1] - h.vr_ptr[r] > 1) {
      double sum = 0.0;
      for (int32_t q = h.vr_ptr[r]; q < h.vr_ptr[r + 1]; ++q) sum += vsum[h.vr_list[q]];
      y[r] = sum;
    }
    double d = 0.0, mag = 0.0;
    for (int32_t e = A.ptr[r]; e < A.ptr[r + 1]; ++e) {
      d += A.val[e] * x[A.col[e]];
      mag += std::fabs(A.val[e] * x[A.col[e]]);
    }
    CHECK(std::fabs(y[r] - d) <= 1e-12 * (1.0 + mag), "%s: row %d product %.17g, direct %.17g", name, r, y[r], d);
  }
  std::printf("%s: %d slices, %d virtual rows of at most %d, %zu split, %zu heavy (%d giant)\n", name,
              h.nslices, h.nvr, h.vrow, h.split.size(), h.heavy.size(), h.ngiant);
}

int main() {
  check_plan("factor rows", factor_matrix(70000, 200, 0.05, 3));
  check_plan("dense factor rows", factor_matrix(3000, 40, 0.5, 5));
  check_plan("short rows", short_matrix(5000, 3000, 9));
  if (failures) {
    std::printf("%d failures\n", failures);
    return 1;
  }
  std::printf("OK\n");
  return 0;
}
