// Family groups of a batch set-up wave (host only, CUDA-free; used by
// batch_engine.cuh and checked on the CPU): instances whose sizes, cone table and
// sparsity pattern (Ap, Ai) are identical and whose values differ at no more
// than a quarter of the nonzeros share one matrix layout.  At a varying
// entry the shared value array holds a quiet NaN whose low kBoxBits bits
// index the member's own value, so a group may vary at no more than
// 2^kBoxBits entries.
#pragma once

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <vector>

#include "batch_layout.h"
#include "pdos_gpu.h"

namespace pdosgpu {
namespace batch {

constexpr uint32_t kBoxBits = 22;
constexpr bool box_index_fits(int64_t t) { return t >= 0 && t < ((int64_t)1 << kBoxBits); }

// Members (wave indices, ascending) of one group; `vary` marks, per CSC
// position, where any member's value differs from the first member's.
struct FamilyGroup {
  std::vector<int64_t> members;
  std::vector<uint8_t> vary;
  int64_t nvary = 0;
};

// 64-bit mix of a problem's shape, cones and a sample of its pattern (a
// filter: equality is checked exactly afterwards).
inline uint64_t pattern_hash(const pdosgpu_problem &p) {
  uint64_t h = 0x9E3779B97F4A7C15ull;
  auto mix = [&](uint64_t v) {
    h ^= v + 0x9E3779B97F4A7C15ull + (h << 6) + (h >> 2);
    h *= 0xBF58476D1CE4E5B9ull;
  };
  mix((uint64_t)p.m);
  mix((uint64_t)p.n);
  mix((uint64_t)p.f);
  mix((uint64_t)p.l);
  mix((uint64_t)p.qsize);
  for (int64_t k = 0; k < p.qsize; ++k) mix((uint64_t)p.q[k]);
  constexpr int64_t kStride = 61;  // every 61st entry of Ap and Ai, and the last
  for (int64_t j = 0; j <= p.n; j += kStride) mix((uint64_t)p.Ap[j]);
  mix((uint64_t)p.Ap[p.n]);
  const int64_t nz = p.Ap[p.n];
  for (int64_t k = 0; k < nz; k += kStride) mix((uint64_t)p.Ai[k]);
  if (nz > 0) mix((uint64_t)p.Ai[nz - 1]);
  return h;
}

inline bool same_pattern(const pdosgpu_problem &a, const pdosgpu_problem &b) {
  if (a.m != b.m || a.n != b.n || a.f != b.f || a.l != b.l || a.qsize != b.qsize) return false;
  if (a.qsize > 0 && std::memcmp(a.q, b.q, sizeof(int64_t) * a.qsize) != 0) return false;
  if (std::memcmp(a.Ap, b.Ap, sizeof(int64_t) * (a.n + 1)) != 0) return false;
  const int64_t nz = a.Ap[a.n];
  return nz == 0 || std::memcmp(a.Ai, b.Ai, sizeof(int64_t) * nz) == 0;
}

// Family groups of at least two instances whose varying positions are at
// most a quarter of the nonzeros (and few enough for the NaN boxes).
// Instances with equal hashes are checked exactly against the first of
// them; those that differ are checked again among themselves (a few rounds
// at most: equal hashes of different patterns are rare).
inline std::vector<FamilyGroup> find_family_groups(const pdosgpu_problem *probs, int64_t cnt) {
  constexpr int kRounds = 8;
  std::vector<FamilyGroup> out;
  if (cnt < 2) return out;
  std::vector<uint64_t> key(cnt);
  parallel_for(cnt, [&](int64_t i) { key[i] = pattern_hash(probs[i]); });
  std::vector<int64_t> order(cnt);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return key[a] < key[b]; });
  std::vector<std::vector<int64_t>> cand;
  for (int64_t s0 = 0; s0 < cnt;) {
    int64_t s1 = s0 + 1;
    while (s1 < cnt && key[order[s1]] == key[order[s0]]) ++s1;
    if (s1 - s0 >= 2) {
      std::vector<int64_t> mem(order.begin() + s0, order.begin() + s1);
      std::sort(mem.begin(), mem.end());
      cand.push_back(std::move(mem));
    }
    s0 = s1;
  }
  for (auto &bucket : cand) {
    std::vector<int64_t> mem = std::move(bucket);
    for (int round = 0; round < kRounds && mem.size() >= 2; ++round) {
      const pdosgpu_problem &r = probs[mem[0]];
      std::vector<uint8_t> same(mem.size(), 1);
      parallel_for((int64_t)mem.size() - 1,
                   [&](int64_t k) { same[k + 1] = same_pattern(r, probs[mem[k + 1]]) ? 1 : 0; });
      FamilyGroup fg;
      std::vector<int64_t> rest;
      for (size_t k = 0; k < mem.size(); ++k) (same[k] ? fg.members : rest).push_back(mem[k]);
      mem = std::move(rest);
      if (fg.members.size() < 2) continue;
      const int64_t nz = r.Ap[r.n];
      fg.vary.assign(nz > 0 ? nz : 1, 0);
      const int64_t chunk = 4096, nchunks = (nz + chunk - 1) / chunk;
      parallel_for(nchunks, [&](int64_t c) {
        const int64_t k0 = c * chunk, k1 = std::min(nz, k0 + chunk);
        for (size_t k = 1; k < fg.members.size(); ++k) {
          const double *a = probs[fg.members[k]].Ax;
          for (int64_t e = k0; e < k1; ++e)
            if (a[e] != r.Ax[e]) fg.vary[e] = 1;
        }
      });
      for (int64_t e = 0; e < nz; ++e) fg.nvary += fg.vary[e];
      if (fg.nvary * 4 <= nz && box_index_fits(fg.nvary)) out.push_back(std::move(fg));
    }
  }
  return out;
}

}  // namespace batch
}  // namespace pdosgpu
