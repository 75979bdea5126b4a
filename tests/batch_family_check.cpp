// CPU check of the batch's family-group detection (batch_family.h): a wave
// mixing two families, a third instance set whose values vary too widely to
// share a layout, and unrelated instances, in interleaved order.  The second
// family's pattern differs from the first's only at entries the pattern hash
// does not sample, so both land in one hash bucket and must be told apart by
// the exact check.  Checks the members of every group, the varying positions
// (exactly the entries where some member differs from the first) and that
// nothing else is grouped.  Prints "OK" and exits 0, or the first failures
// and exits 1.
#include <cstdio>
#include <random>
#include <set>
#include <vector>

#include "batch_family.h"

using namespace pdosgpu::batch;

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

struct Inst {
  int64_t m = 0, n = 0;
  std::vector<int64_t> Ap, Ai, q;
  std::vector<double> Ax;
  pdosgpu_problem view() const {
    pdosgpu_problem p{};
    p.n = n;
    p.m = m;
    p.Ax = Ax.data();
    p.Ai = Ai.data();
    p.Ap = Ap.data();
    p.f = 1;
    p.l = m - 1 - (q.empty() ? 0 : q[0]);
    p.qsize = (int64_t)q.size();
    p.q = q.data();
    return p;
  }
};

// a random CSC pattern: m rows, n columns, `per` distinct sorted rows per column
static Inst random_pattern(int64_t m, int64_t n, int per, std::mt19937 &g) {
  Inst I;
  I.m = m;
  I.n = n;
  I.Ap.push_back(0);
  for (int64_t j = 0; j < n; ++j) {
    std::set<int64_t> rows;
    while ((int)rows.size() < per) rows.insert((int64_t)(g() % m));
    for (int64_t r : rows) I.Ai.push_back(r);
    I.Ap.push_back((int64_t)I.Ai.size());
  }
  I.q = {m / 4};
  std::uniform_real_distribution<double> u(-1.0, 1.0);
  for (size_t k = 0; k < I.Ai.size(); ++k) I.Ax.push_back(u(g));
  return I;
}

int main() {
  std::mt19937 g(5);
  std::uniform_real_distribution<double> u(-1.0, 1.0);
  const Inst A = random_pattern(300, 200, 6, g);
  const int64_t nz = (int64_t)A.Ai.size();
  // B: A's pattern with two entries moved to other rows, both at positions
  // the hash skips (not a multiple of 61, not the last)
  Inst B = A;
  for (int64_t k : {int64_t(1), int64_t(nz / 2 + 1)}) {
    if (k % 61 == 0) ++k;
    const int64_t col = std::upper_bound(B.Ap.begin(), B.Ap.end(), k) - B.Ap.begin() - 1;
    std::set<int64_t> used(B.Ai.begin() + B.Ap[col], B.Ai.begin() + B.Ap[col + 1]);
    int64_t r = 0;
    while (used.count(r)) ++r;
    B.Ai[k] = r;  // still a valid pattern for this check: only equality matters
  }
  CHECK(pattern_hash(A.view()) == pattern_hash(B.view()), "the two patterns should collide in the hash");
  // family members: the first member's values everywhere but a fixed set of
  // positions (about a fifth of them), where each member has its own values
  std::vector<uint8_t> vpos(nz, 0);
  for (int64_t k = 0; k < nz; k += 5) vpos[k] = 1;
  auto member = [&](const Inst &base) {
    Inst I = base;
    for (int64_t k = 0; k < nz; ++k)
      if (vpos[k]) I.Ax[k] = u(g);
    return I;
  };
  std::vector<Inst> wave;
  std::vector<int64_t> fam_a, fam_b, wide;
  auto add = [&](Inst I, std::vector<int64_t> *list) {
    if (list) list->push_back((int64_t)wave.size());
    wave.push_back(std::move(I));
  };
  for (int i = 0; i < 6; ++i) {
    add(member(A), &fam_a);
    if (i < 3) add(member(B), &fam_b);
    add(random_pattern(100 + i, 80, 4, g), nullptr);
  }
  // a set on a third pattern whose members differ at every entry
  const Inst C = random_pattern(250, 150, 5, g);
  for (int i = 0; i < 3; ++i) {
    Inst I = C;
    for (auto &v : I.Ax) v = u(g);
    add(std::move(I), &wide);
  }
  std::vector<pdosgpu_problem> probs;
  for (const Inst &I : wave) probs.push_back(I.view());
  const std::vector<FamilyGroup> groups = find_family_groups(probs.data(), (int64_t)probs.size());
  CHECK(groups.size() == 2, "expected 2 groups, found %zu", groups.size());
  for (const FamilyGroup &fg : groups) {
    const bool is_a = !fg.members.empty() && fg.members[0] == fam_a[0];
    const std::vector<int64_t> &want = is_a ? fam_a : fam_b;
    CHECK(fg.members == want, "group of %lld: wrong members", (long long)fg.members[0]);
    // varying positions: exactly where some member differs from the first
    int64_t nv = 0;
    for (int64_t k = 0; k < nz; ++k) {
      bool differs = false;
      for (int64_t i : fg.members) differs |= probs[i].Ax[k] != probs[fg.members[0]].Ax[k];
      CHECK((fg.vary[k] != 0) == differs, "group of %lld: vary[%lld]", (long long)fg.members[0], (long long)k);
      nv += differs;
    }
    CHECK(fg.nvary == nv && nv * 4 <= nz, "group of %lld: %lld varying of %lld", (long long)fg.members[0],
          (long long)fg.nvary, (long long)nz);
  }
  CHECK(box_index_fits(0) && box_index_fits((1 << kBoxBits) - 1) && !box_index_fits(1 << kBoxBits) &&
            !box_index_fits(-1),
        "box index range");
  if (failures) {
    std::printf("%d failures\n", failures);
    return 1;
  }
  std::printf("OK %zu groups in a wave of %zu instances\n", groups.size(), wave.size());
  return 0;
}
