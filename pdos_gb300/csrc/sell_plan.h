// Host-side construction of the sliced-ELL (SELL-32-sigma) plans of the
// single-instance SpMV: which source entry goes to which slot, the virtual
// rows of every row, and the split and heavy rows.  CUDA-free, so the plan
// can be checked on the CPU; the kernels that run a plan are in sell.cuh.
#pragma once

#include <algorithm>
#include <cstdint>
#include <numeric>
#include <vector>

namespace pdosgpu {

constexpr int kSigma = 4096;    // sorting window, in virtual rows
constexpr int kHeavyVrows = 64;    // rows with more pieces: combined by a warp
constexpr int kGiantVrows = 2048;  // rows with more pieces: combined by a CTA

// Host-side construction.  `ptr` is the row pointer array of a row-wise
// matrix; the plan maps every slice slot to a source position (or -1).
struct SellHost {
  int32_t rows = 0;
  int32_t nvr = 0;       // virtual rows (padded to a multiple of 32)
  int32_t nslices = 0;
  int64_t slots = 0;
  std::vector<int32_t> slice_off;  // [nslices+1]
  std::vector<int32_t> vr_len;     // [nvr]
  std::vector<int32_t> slot_src;   // [slots] source position or -1
  std::vector<int32_t> vr_ptr;     // [rows+1] virtual rows of each row ...
  std::vector<int32_t> vr_list;    // ... in chunk order (positions in slice order)
  std::vector<int32_t> heavy;      // rows with more than kHeavyVrows pieces,
                                   // those above kGiantVrows first
  int32_t ngiant = 0;
  std::vector<int32_t> vr_row;     // [nvr] row of a whole-row virtual row, else -1
  std::vector<int32_t> split;      // split rows with at most kHeavyVrows pieces
  int32_t vrow = 0;                // nonzeros per virtual row

  // Whole rows (up to 256) when at least half of the nonzeros sit in rows of
  // at most 256; otherwise pieces of 32.
  static int32_t choose_vrow(const int32_t *ptr, int32_t nrows) {
    int64_t nnz = ptr[nrows], short_nz = 0;
    int32_t longest_short = 1;
    for (int32_t r = 0; r < nrows; ++r) {
      const int32_t L = ptr[r + 1] - ptr[r];
      if (L <= 256) {
        short_nz += L;
        longest_short = std::max(longest_short, L);
      }
    }
    if (2 * short_nz < nnz) return 32;
    int32_t v = 32;
    while (v < longest_short) v *= 2;
    return v;
  }

  void build(const int32_t *ptr, int32_t nrows) {
    rows = nrows;
    vrow = choose_vrow(ptr, nrows);
    const int32_t kVrowMax = vrow;
    // virtual rows in natural order
    std::vector<int32_t> v_row, v_start, v_len;
    vr_ptr.assign(nrows + 1, 0);
    for (int32_t r = 0; r < nrows; ++r) {
      const int32_t L = ptr[r + 1] - ptr[r];
      const int32_t nch = L > 0 ? (L + kVrowMax - 1) / kVrowMax : 1;
      for (int32_t c = 0; c < nch; ++c) {
        v_row.push_back(r);
        v_start.push_back(ptr[r] + c * kVrowMax);
        v_len.push_back(std::min(kVrowMax, L - c * kVrowMax) > 0 ? std::min(kVrowMax, L - c * kVrowMax) : 0);
      }
      vr_ptr[r + 1] = vr_ptr[r] + nch;
      if (nch > kHeavyVrows)
        heavy.push_back(r);
      else if (nch > 1)
        split.push_back(r);
    }
    std::stable_partition(heavy.begin(), heavy.end(), [&](int32_t r) {
      return vr_ptr[r + 1] - vr_ptr[r] > kGiantVrows;
    });
    ngiant = 0;
    for (int32_t r : heavy)
      if (vr_ptr[r + 1] - vr_ptr[r] > kGiantVrows) ++ngiant;
    const int32_t nv = (int32_t)v_row.size();
    nvr = (nv + 31) / 32 * 32;
    // order: by length, longest first, stable, inside windows of kSigma
    std::vector<int32_t> order(nv);
    std::iota(order.begin(), order.end(), 0);
    for (int32_t w0 = 0; w0 < nv; w0 += kSigma) {
      const int32_t w1 = std::min(nv, w0 + kSigma);
      std::stable_sort(order.begin() + w0, order.begin() + w1,
                       [&](int32_t a, int32_t b) { return v_len[a] > v_len[b]; });
    }
    std::vector<int32_t> pos(nv);
    for (int32_t k = 0; k < nv; ++k) pos[order[k]] = k;
    vr_list.resize(nv);
    for (int32_t k = 0; k < nv; ++k) vr_list[k] = pos[k];  // natural virtual-row order -> position
    vr_len.assign(nvr, 0);
    vr_row.assign(nvr, -1);
    for (int32_t k = 0; k < nv; ++k) {
      vr_len[k] = v_len[order[k]];
      const int32_t r = v_row[order[k]];
      if (vr_ptr[r + 1] - vr_ptr[r] == 1) vr_row[k] = r;
    }
    nslices = nvr / 32;
    slice_off.assign(nslices + 1, 0);
    for (int32_t s = 0; s < nslices; ++s) {
      int32_t w = 0;
      for (int t = 0; t < 32; ++t) w = std::max(w, vr_len[32 * s + t]);
      slice_off[s + 1] = slice_off[s] + 32 * w;
    }
    slots = slice_off[nslices];
    slot_src.assign((size_t)slots, -1);
    for (int32_t s = 0; s < nslices; ++s)
      for (int t = 0; t < 32; ++t) {
        const int32_t k = 32 * s + t;
        if (k >= nv) continue;
        const int32_t src = v_start[order[k]];
        for (int32_t e = 0; e < vr_len[k]; ++e) slot_src[(size_t)slice_off[s] + 32 * e + t] = src + e;
      }
  }
};

}  // namespace pdosgpu
