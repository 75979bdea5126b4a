// Host-side builder of the batch solver's hybrid matrix layout (no CUDA):
// for every instance and each side of it (rows of A, rows of A'), slices of
// 32 rows stored column-major and long rows cut into warp-wide pieces, with
// instance-local 16-bit gather indices.  Used by batch_engine.cuh and tested on the
// CPU.
#pragma once

#include <algorithm>
#include <atomic>
#include <cstdint>
#include <memory>
#include <thread>
#include <vector>

namespace pdosgpu {
namespace batch {

#ifndef PDOS_BATCH_PIECE
#define PDOS_BATCH_PIECE 1024
#endif
constexpr int kLongRow = 128;               // default: rows with more nonzeros go to warp-wide pieces
constexpr int kPiece = PDOS_BATCH_PIECE;    // default target nonzeros per piece

// One side (A: rows of A; At: rows of A', i.e. columns of A) of an instance
// in the hybrid layout: slices of 32 consecutive rows stored column-major
// (lane = row), and rows longer than kLongRow cut into pieces of at most
// kPiece nonzeros, one warp per piece.
struct Side {
  int64_t slice0, piece0, split0;
  int32_t nslices, npieces, nsplit, rows;
  int32_t sorted;  // 1: the slices hold the short rows sorted by length (slice_row maps lanes to rows)
};

// Rows sorted by length inside windows of this many rows when an
// instance's slices would otherwise pay more than kSortPadding of padding
// and the side holds at least kSortMinNnz nonzeros: a smaller instance is
// bound by latency, not by the bytes padding adds, and its epilogue would
// reach its rows out of order.
constexpr int kSortWindow = 1024;
constexpr double kSortPadding = 0.15;
constexpr int64_t kSortMinNnz = 32768;

// Work over instances on the host's cores (atomic counter, no exceptions).
template <class F>
void parallel_for(int64_t n, F &&f) {
  const unsigned hw = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
  const int nt = (int)std::max<int64_t>(1, std::min<int64_t>(n, hw));
  std::atomic<int64_t> next{0};
  auto body = [&]() {
    for (int64_t i = next.fetch_add(1); i < n; i = next.fetch_add(1)) f(i);
  };
  std::vector<std::thread> pool;
  for (int t = 1; t < nt; ++t) pool.emplace_back(body);
  body();
  for (auto &th : pool) th.join();
}

// A host array that is not zero-filled on allocation (its writers cover it).
template <typename T>
struct Raw {
  std::unique_ptr<T[]> p;
  size_t n = 0;
  void resize(size_t count) {
    p.reset(count ? new T[count] : nullptr);
    n = count;
  }
  T *data() { return p.get(); }
  const T *data() const { return p.get(); }
  size_t size() const { return n; }
  bool empty() const { return n == 0; }
  T &operator[](size_t i) { return p[i]; }
  const T &operator[](size_t i) const { return p[i]; }
  using value_type = T;
};

// Position in the layout arrays of one side.
struct Cursor {
  int64_t slice = 0, piece = 0, split = 0, elem = 0;
};

// The hybrid layout of one side for every instance.  walk<false> sizes an
// instance (advances a cursor), walk<true> writes it at a cursor; both make
// the same decisions, and every instance starts and ends on a multiple of
// 4 elements, so instances can be sized and written in parallel.
//
// Slices hold an instance's short rows (at most long_row nonzeros) 32 at a
// time, lane = row, padded to the slice's longest row.  In natural order a
// slice also keeps a lane for each long row and each row past the end
// (skipped).  When that order pays more than kSortPadding of padding, the
// instance is large enough (kSortMinNnz) and sorting saves a tenth of the
// elements, the short rows are instead sorted
// by length (longest first, stable) inside windows of kSortWindow rows and
// packed densely; slice_row then gives each lane's row.  Each row keeps its
// own entries in its own lane in their order, so its sum is the same chain
// of fused multiply-adds either way.
struct HybBuild {
  int long_row = kLongRow;  // rows with more nonzeros go to pieces (a multiple of 4, >= 4)
  int piece = kPiece;       // nonzeros per piece at most (a multiple of 4, >= 4)
  bool sort_rows = true;    // let an instance with much padding sort its rows
  std::vector<int64_t> slice_beg;
  std::vector<int32_t> slice_w;
  std::vector<uint32_t> slice_skip;
  std::vector<uint16_t> slice_row;  // [32 per slice] the row of each lane (sorted instances; else unused)
  bool any_sorted = false;          // some instance of this build sorted its rows
  std::vector<int32_t> piece_row, piece_len, split_row, split_p0, split_np;
  std::vector<int64_t> piece_beg;
  Raw<uint16_t> idx;  // per element: local gather index
  Raw<int32_t> src;   // per element: position of its value in the source array (-1: padding)

  void resize(const Cursor &t) {
    slice_beg.resize(t.slice);
    slice_w.resize(t.slice);
    slice_skip.resize(t.slice);
    slice_row.assign((size_t)t.slice * 32, 0);
    piece_row.resize(t.piece);
    piece_len.resize(t.piece);
    piece_beg.resize(t.piece);
    split_row.resize(t.split);
    split_p0.resize(t.split);
    split_np.resize(t.split);
    idx.resize(t.elem);
    src.resize(t.elem);
  }

  // Rows [r0, r1) of a row-wise matrix (ptr, gidx absolute); gather indices
  // are made local by subtracting c0.
  template <bool WRITE, typename Idx>
  Side walk(const int32_t *ptr, const Idx *gidx, int64_t r0, int64_t r1, int64_t c0, Cursor &c) {
    Side sd{};
    const int64_t R = r1 - r0;
    sd.rows = (int32_t)R;
    sd.slice0 = c.slice;
    sd.piece0 = c.piece;
    sd.split0 = c.split;
    auto put = [&](int32_t j, int32_t p) {
      if (WRITE) {
        idx[c.elem] = (uint16_t)j;
        src[c.elem] = p;
      }
      ++c.elem;
    };
    auto pad4 = [&]() {
      while (c.elem % 4) put(0, -1);  // zero entries up to 16-byte alignment
    };
    // rows of the slices' lanes: natural order (lane = row, -1 for a long row
    // or past the end) or, for an instance with much padding, its short rows
    // sorted by length inside windows
    auto len_of = [&](int64_t r) -> int64_t { return ptr[r0 + r + 1] - ptr[r0 + r]; };
    auto slice_elems = [&](const std::vector<int32_t> &lanes) {
      int64_t e = 0;
      for (size_t s0 = 0; s0 < lanes.size(); s0 += 32) {
        int64_t w = 0;
        for (size_t k = s0; k < std::min(lanes.size(), s0 + 32); ++k)
          if (lanes[k] >= 0) w = std::max(w, len_of(lanes[k]));
        e += 32 * (w >= 4 ? (w + 3) & ~3 : w);
      }
      return e;
    };
    std::vector<int32_t> lanes((size_t)((R + 31) / 32 * 32), -1);
    int64_t useful = 0;
    for (int64_t r = 0; r < R; ++r)
      if (len_of(r) <= long_row) {
        lanes[r] = (int32_t)r;
        useful += len_of(r);
      }
    if (sort_rows && R > 32 && ptr[r1] - ptr[r0] >= kSortMinNnz) {
      const int64_t natural = slice_elems(lanes);
      if (natural - useful > kSortPadding * natural) {
        std::vector<int32_t> sorted;
        for (int64_t w0 = 0; w0 < R; w0 += kSortWindow) {
          const size_t first = sorted.size();
          for (int64_t r = w0; r < std::min<int64_t>(R, w0 + kSortWindow); ++r)
            if (len_of(r) <= long_row) sorted.push_back((int32_t)r);
          std::stable_sort(sorted.begin() + first, sorted.end(),
                           [&](int32_t x, int32_t y) { return len_of(x) > len_of(y); });
        }
        sorted.resize((sorted.size() + 31) / 32 * 32, -1);
        if (10 * slice_elems(sorted) < 9 * natural) {
          lanes.swap(sorted);
          sd.sorted = 1;
        }
      }
    }
    for (size_t s0 = 0; s0 < lanes.size(); s0 += 32) {
      uint32_t skip = 0;
      int width = 0;
      for (int lane = 0; lane < 32; ++lane) {
        const int32_t r = lanes[s0 + lane];
        if (r < 0) {
          skip |= 1u << lane;
          continue;
        }
        width = std::max(width, (int)len_of(r));
      }
      const bool vec = width >= 4;
      if (vec) {
        width = (width + 3) & ~3;
        pad4();
      }
      if (WRITE) {
        slice_beg[c.slice] = c.elem;
        slice_w[c.slice] = vec ? -width : width;
        slice_skip[c.slice] = skip;
        for (int lane = 0; lane < 32; ++lane)
          slice_row[(size_t)c.slice * 32 + lane] = (uint16_t)(lanes[s0 + lane] >= 0 ? lanes[s0 + lane] : 0);
      }
      for (int cidx = 0; cidx < width; cidx += vec ? 4 : 1) {
        for (int lane = 0; lane < 32; ++lane) {
          for (int t = 0; t < (vec ? 4 : 1); ++t) {
            const int32_t r = lanes[s0 + lane];
            int32_t j = 0, p = -1;
            if (r >= 0) {
              const int64_t a = ptr[r0 + r], len = ptr[r0 + r + 1] - a;
              if (cidx + t < len) {
                p = (int32_t)(a + cidx + t);
                j = (int32_t)(gidx[a + cidx + t] - c0);
              }
            }
            put(j, p);
          }
        }
      }
      ++c.slice;
      ++sd.nslices;
    }
    for (int64_t r = 0; r < R; ++r) {
      const int64_t a = ptr[r0 + r], len = ptr[r0 + r + 1] - a;
      if (len <= long_row) continue;
      const int64_t np = (len + piece - 1) / piece;
      if (np > 1) {
        if (WRITE) {
          split_row[c.split] = (int32_t)r;
          split_p0[c.split] = (int32_t)(c.piece - sd.piece0);
          split_np[c.split] = (int32_t)np;
        }
        ++c.split;
        ++sd.nsplit;
      }
      for (int64_t k = 0; k < np; ++k) {  // nearly equal pieces
        const int64_t e0 = a + len * k / np, e1 = a + len * (k + 1) / np;
        pad4();
        const int64_t beg = c.elem;
        for (int64_t e = e0; e < e1; ++e) put((int32_t)(gidx[e] - c0), (int32_t)e);
        pad4();
        if (WRITE) {
          piece_row[c.piece] = np > 1 ? ~(int32_t)r : (int32_t)r;
          piece_beg[c.piece] = beg;
          piece_len[c.piece] = (int32_t)(c.elem - beg);
        }
        ++c.piece;
        ++sd.npieces;
      }
    }
    pad4();
    return sd;
  }
};

// Sizes every instance, turns the sizes into start cursors, then writes the
// instances in parallel; side(i) returns (ptr, gidx, r0, r1, c0) of one.
template <typename Idx, class SideOf>
void build_layout(HybBuild &hb, int64_t count, SideOf side, std::vector<Side> &out) {
  std::vector<Cursor> size(count);
  parallel_for(count, [&](int64_t i) {
    const int32_t *ptr;
    const Idx *gidx;
    int64_t r0, r1, c0;
    side(i, ptr, gidx, r0, r1, c0);
    Cursor c;
    hb.walk<false>(ptr, gidx, r0, r1, c0, c);
    size[i] = c;
  });
  std::vector<Cursor> start(count + 1);
  for (int64_t i = 0; i < count; ++i) {
    start[i + 1].slice = start[i].slice + size[i].slice;
    start[i + 1].piece = start[i].piece + size[i].piece;
    start[i + 1].split = start[i].split + size[i].split;
    start[i + 1].elem = start[i].elem + size[i].elem;
  }
  hb.resize(start[count]);
  out.assign(count, Side{});
  parallel_for(count, [&](int64_t i) {
    const int32_t *ptr;
    const Idx *gidx;
    int64_t r0, r1, c0;
    side(i, ptr, gidx, r0, r1, c0);
    Cursor c = start[i];
    out[i] = hb.walk<true>(ptr, gidx, r0, r1, c0, c);
  });
  hb.any_sorted = false;
  for (const Side &sd : out) hb.any_sorted |= sd.sorted != 0;
}

}  // namespace batch
}  // namespace pdosgpu
