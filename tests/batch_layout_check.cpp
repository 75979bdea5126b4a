// CPU check of the batch solver's host layout builder (batch_layout.h): it
// lays out the rows of seeded random block-diagonal matrices -- short rows,
// rows of a few dozen entries, rows longer than a piece (split rows), empty
// rows -- for many instances at once, sized and written in parallel as the
// solver does, and checks every structural promise the kernels rely on,
// including the lane-to-row map of instances that sort their rows.
// Prints "OK" and exits 0, or prints the first failures and exits 1.
#include <cmath>
#include <cstdio>
#include <random>
#include <vector>

#include "batch_layout.h"

using namespace pdosgpu::batch;

static int failures = 0;
#define CHECK(cond, ...)                 \
  do {                                   \
    if (!(cond)) {                       \
      if (failures < 20) {               \
        std::printf("FAIL: " __VA_ARGS__); \
        std::printf("\n");               \
      }                                  \
      ++failures;                        \
    }                                    \
  } while (0)

int main() {
  std::mt19937 g(7);
  const int count = 64;
  // stacked CSR: instance i owns rows [r0[i], r0[i+1]) and columns [c0[i], c0[i+1])
  std::vector<int32_t> ptr(1, 0), col;
  std::vector<int64_t> r0(1, 0), c0(1, 0);
  for (int i = 0; i < count; ++i) {
    const int m = 1 + (int)(g() % 700), n = 1 + (int)(g() % 3000);
    for (int r = 0; r < m; ++r) {
      const int kind = (int)(g() % 10);
      int len = kind < 4 ? (int)(g() % 4) : kind < 7 ? (int)(g() % 60) : kind < 9 ? (int)(g() % 400)
                                                                                : (int)(g() % 2600);
      len = std::min(len, n);
      std::vector<int32_t> cols(n);
      for (int j = 0; j < n; ++j) cols[j] = j;
      std::shuffle(cols.begin(), cols.end(), g);
      cols.resize(len);
      std::sort(cols.begin(), cols.end());
      for (int j : cols) col.push_back((int32_t)(c0.back() + j));
      ptr.push_back((int32_t)col.size());
    }
    r0.push_back(r0.back() + m);
    c0.push_back(c0.back() + n);
  }

  // the default layout parameters and other values the layout tuner tries
  const int params[][2] = {{kLongRow, kPiece}, {64, 256}, {256, 2048}, {32, 512}};
  long long total_elems = 0;
  for (const auto &lp : params) {
  HybBuild hb;
  hb.long_row = lp[0];
  hb.piece = lp[1];
  std::vector<Side> sides;
  build_layout<int32_t>(hb, count, [&](int64_t i, const int32_t *&p, const int32_t *&gi, int64_t &a, int64_t &b,
                                       int64_t &c) {
    p = ptr.data();
    gi = col.data();
    a = r0[i];
    b = r0[i + 1];
    c = c0[i];
  }, sides);

  std::vector<int> placed(col.size(), 0);
  for (size_t e = 0; e < hb.src.size(); ++e) {
    const int32_t p = hb.src[e];
    if (p < 0) continue;
    CHECK(p < (int32_t)col.size(), "element %zu points past the source", e);
    placed[p]++;
  }
  for (size_t k = 0; k < col.size(); ++k) CHECK(placed[k] == 1, "nonzero %zu placed %d times", k, placed[k]);

  int64_t nsplit_total = 0;
  for (int i = 0; i < count; ++i) {
    const Side &sd = sides[i];
    const int64_t m = r0[i + 1] - r0[i];
    CHECK(sd.rows == m, "instance %d: %d rows, expected %lld", i, sd.rows, (long long)m);
    std::vector<int> seen(m, 0);
    for (int s = 0; s < sd.nslices; ++s) {
      const int64_t k = sd.slice0 + s;
      const int w = hb.slice_w[k];
      const int64_t beg = hb.slice_beg[k];
      if (w < 0) {
        CHECK(-w % 4 == 0 && -w <= hb.long_row, "instance %d slice %d: width %d", i, s, w);
        CHECK(beg % 4 == 0, "instance %d slice %d: start %lld not 4-aligned", i, s, (long long)beg);
      } else {
        CHECK(w < 4, "instance %d slice %d: narrow width %d", i, s, w);
      }
      const int width = w < 0 ? -w : w;
      CHECK(beg + 32LL * width <= (int64_t)hb.idx.size(), "instance %d slice %d runs past the end", i, s);
      for (int lane = 0; lane < 32; ++lane) {
        const int64_t r = sd.sorted ? (int64_t)hb.slice_row[(size_t)k * 32 + lane] : 32LL * s + lane;
        if ((hb.slice_skip[k] >> lane) & 1u) {
          // a sorted instance packs its short rows: only its last slice has skipped lanes
          if (sd.sorted) CHECK(s == sd.nslices - 1, "instance %d: skipped lane inside sorted slice %d", i, s);
          continue;
        }
        CHECK(r < m, "instance %d slice %d: live lane past the last row", i, s);
        if (r >= m) continue;
        seen[r]++;
        const int64_t a = ptr[r0[i] + r], len = ptr[r0[i] + r + 1] - a;
        CHECK(len <= hb.long_row, "instance %d: long row %lld in a slice", i, (long long)r);
        for (int c = 0; c < width; ++c) {  // entry c of the lane's row
          const int64_t e = w < 0 ? beg + 128LL * (c / 4) + 4 * lane + c % 4 : beg + 32LL * c + lane;
          if (c < len) {
            CHECK(hb.src[e] == a + c, "instance %d row %lld entry %d misplaced", i, (long long)r, c);
            CHECK(hb.idx[e] == col[a + c] - c0[i], "instance %d row %lld entry %d: wrong index", i, (long long)r, c);
          } else {
            CHECK(hb.src[e] == -1, "instance %d row %lld: padding %d not marked", i, (long long)r, c);
          }
        }
      }
    }
    for (int k = 0; k < sd.npieces; ++k) {
      const int64_t pk = sd.piece0 + k;
      const int len = hb.piece_len[pk];
      CHECK(len % 4 == 0 && len > 0 && len <= hb.piece, "instance %d piece %d: length %d", i, k, len);
      CHECK(hb.piece_beg[pk] % 4 == 0, "instance %d piece %d: start not 4-aligned", i, k);
      const int32_t pr = hb.piece_row[pk];
      const int64_t r = pr >= 0 ? pr : ~pr;
      CHECK(r >= 0 && r < m, "instance %d piece %d: row %lld", i, k, (long long)r);
      if (r < 0 || r >= m) continue;
      const int64_t len_r = ptr[r0[i] + r + 1] - ptr[r0[i] + r];
      CHECK(len_r > hb.long_row, "instance %d: short row %lld in a piece", i, (long long)r);
      if (pr >= 0) seen[r]++;  // a whole row in one piece
    }
    for (int k = 0; k < sd.nsplit; ++k) {
      const int64_t sk = sd.split0 + k;
      const int64_t r = hb.split_row[sk];
      const int p0 = hb.split_p0[sk], np = hb.split_np[sk];
      CHECK(np > 1 && p0 >= 0 && p0 + np <= sd.npieces, "instance %d split %d: pieces [%d, %d)", i, k, p0, p0 + np);
      if (!(np > 1 && p0 >= 0 && p0 + np <= sd.npieces)) continue;
      for (int t = 0; t < np; ++t)
        CHECK(hb.piece_row[sd.piece0 + p0 + t] == ~(int32_t)r, "instance %d split %d: piece %d of another row", i, k, t);
      if (r >= 0 && r < m) seen[r]++;
    }
    nsplit_total += sd.nsplit;
    for (int64_t r = 0; r < m; ++r) CHECK(seen[r] == 1, "instance %d row %lld covered %d times", i, (long long)r, seen[r]);
  }
  CHECK(nsplit_total > 0, "no split rows were exercised");
  // run the layout as the kernels do -- slices (lane -> row, natural or
  // through slice_row), pieces (a warp's sum, whole rows to the epilogue,
  // split rows' partials summed in order) -- and compare with a direct CSR
  // product
  {
    std::vector<double> val(col.size()), x(c0.back());
    std::mt19937 gv(3);
    std::uniform_real_distribution<double> u(-1.0, 1.0);
    for (auto &v : val) v = u(gv);
    for (auto &v : x) v = u(gv);
    for (int i = 0; i < count; ++i) {
      const Side &sd = sides[i];
      const int64_t m = r0[i + 1] - r0[i];
      std::vector<double> y(m, std::nan("")), part(sd.npieces, 0.0);
      for (int s = 0; s < sd.nslices; ++s) {
        const int64_t k = sd.slice0 + s;
        const int w = hb.slice_w[k], width = w < 0 ? -w : w;
        for (int lane = 0; lane < 32; ++lane) {
          if ((hb.slice_skip[k] >> lane) & 1u) continue;
          double acc = 0.0;
          for (int c = 0; c < width; ++c) {
            const int64_t e = w < 0 ? hb.slice_beg[k] + 128LL * (c / 4) + 4 * lane + c % 4
                                    : hb.slice_beg[k] + 32LL * c + lane;
            if (hb.src[e] >= 0) acc = std::fma(val[hb.src[e]], x[c0[i] + hb.idx[e]], acc);
          }
          const int64_t r = sd.sorted ? (int64_t)hb.slice_row[(size_t)k * 32 + lane] : 32LL * s + lane;
          y[r] = acc;
        }
      }
      for (int q = 0; q < sd.npieces; ++q) {
        const int64_t pk = sd.piece0 + q;
        double acc = 0.0;
        for (int e = 0; e < hb.piece_len[pk]; ++e) {
          const int64_t at = hb.piece_beg[pk] + e;
          if (hb.src[at] >= 0) acc += val[hb.src[at]] * x[c0[i] + hb.idx[at]];
        }
        if (hb.piece_row[pk] >= 0)
          y[hb.piece_row[pk]] = acc;
        else
          part[q] = acc;
      }
      for (int q = 0; q < sd.nsplit; ++q) {
        const int64_t sk = sd.split0 + q;
        double acc = 0.0;
        for (int t = 0; t < hb.split_np[sk]; ++t) acc += part[hb.split_p0[sk] + t];
        y[hb.split_row[sk]] = acc;
      }
      for (int64_t r = 0; r < m; ++r) {
        double d = 0.0, mag = 0.0;
        for (int64_t e = ptr[r0[i] + r]; e < ptr[r0[i] + r + 1]; ++e) {
          d += val[e] * x[col[e]];
          mag += std::fabs(val[e] * x[col[e]]);
        }
        CHECK(std::fabs(y[r] - d) <= 1e-12 * (1.0 + mag), "instance %d row %lld: layout product %.17g, direct %.17g",
              i, (long long)r, y[r], d);
      }
    }
  }
  // sorted instances: inside each window of rows, slice lanes hold rows in
  // order of decreasing length
  int nsorted = 0;
  for (int i = 0; i < count; ++i) {
    const Side &sd = sides[i];
    if (!sd.sorted) continue;
    ++nsorted;
    int64_t prev_window = -1, prev_len = 0;
    for (int64_t q = 0; q < 32LL * sd.nslices; ++q) {
      const int64_t k = sd.slice0 + q / 32;
      if ((hb.slice_skip[k] >> (q % 32)) & 1u) continue;
      const int64_t r = hb.slice_row[(size_t)k * 32 + q % 32];
      const int64_t len = ptr[r0[i] + r + 1] - ptr[r0[i] + r], window = r / kSortWindow;
      CHECK(window >= prev_window, "instance %d: windows out of order", i);
      if (window == prev_window) CHECK(len <= prev_len, "instance %d: rows not sorted by length", i);
      prev_window = window;
      prev_len = len;
    }
  }
  CHECK(nsorted > 0, "no instance sorted its rows");
  // the same matrices in natural row order take more elements
  HybBuild nat;
  nat.long_row = lp[0];
  nat.piece = lp[1];
  nat.sort_rows = false;
  std::vector<Side> nsides;
  build_layout<int32_t>(nat, count, [&](int64_t i, const int32_t *&p, const int32_t *&gi, int64_t &a, int64_t &b,
                                        int64_t &c) {
    p = ptr.data();
    gi = col.data();
    a = r0[i];
    b = r0[i + 1];
    c = c0[i];
  }, nsides);
  CHECK(!nat.any_sorted && hb.any_sorted, "sorting switch");
  CHECK(hb.idx.size() < nat.idx.size(), "sorting did not shrink the layout");
  std::printf("long_row %d, piece %d: %d of %d instances sorted, %zu elements against %zu in natural order "
              "(%zu nonzeros)\n", lp[0], lp[1], nsorted, count, hb.idx.size(), nat.idx.size(), col.size());
  total_elems += (long long)hb.idx.size();
  }
  if (failures) {
    std::printf("%d failures\n", failures);
    return 1;
  }
  std::printf("OK %d instances, %zu nonzeros, %lld layout elements over %zu parameter sets\n", count, col.size(),
              total_elems, sizeof(params) / sizeof(params[0]));
  return 0;
}
