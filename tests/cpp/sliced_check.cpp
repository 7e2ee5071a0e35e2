// Checks the sliced-ELL down table against the hop table it is built from:
// every state's entries (doubled bonds twice) appear exactly once in its
// lane (slots 4i..4i+3 of a lane form one 16-byte word), padding points at
// the zero elements past the row, and the slot order
// keeps the eight lanes of each quarter warp on distinct 16-byte bank groups
// (index mod 8).  Prints the shared-memory wavefronts of one warp's gathers
// per slot against the minimum of 4.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <set>
#include <vector>

#include "../../manybody_gb300/csrc/mb_internal.h"

namespace {

// Occupation masks with n of L bits in colex order (numeric order).
std::vector<uint32_t> sector(int L, int n) {
  std::vector<uint32_t> m;
  for (uint32_t s = 0; s < (1u << L); ++s)
    if (__builtin_popcount(s) == n) m.push_back(s);
  return m;
}

// Hop table of a bond list: entry = target << 8 | doubled << 1 | negative.
mb::HopTable hops(int L, int n, const std::vector<std::pair<int, int>>& bonds, bool double_some) {
  const auto m = sector(L, n);
  std::map<uint32_t, int32_t> rank;
  for (size_t i = 0; i < m.size(); ++i) rank[m[i]] = (int32_t)i;
  mb::HopTable t;
  t.off.push_back(0);
  for (uint32_t s : m) {
    for (size_t b = 0; b < bonds.size(); ++b) {
      for (int dir = 0; dir < 2; ++dir) {
        const int a = dir ? bonds[b].second : bonds[b].first;
        const int c = dir ? bonds[b].first : bonds[b].second;
        if (!((s >> a) & 1u) || ((s >> c) & 1u)) continue;
        const uint32_t tgt = (uint32_t)rank[s ^ (1u << a) ^ (1u << c)];
        const uint32_t neg = (uint32_t)(__builtin_popcount(s & ((1u << std::max(a, c)) - 1u) &
                                                           ~((1u << (std::min(a, c) + 1)) - 1u)) &
                                        1);
        const uint32_t dbl = (double_some && b % 5 == 0) ? 1u : 0u;
        t.ent.push_back(tgt << 8 | dbl << 1 | neg);
      }
    }
    t.off.push_back((int32_t)t.ent.size());
  }
  return t;
}

// entry of slot j, lane l in a group starting at base
uint32_t at(const mb::SlicedTable& s, int32_t base, int j, int l) {
  return s.ent[(size_t)base + 128 * (size_t)(j >> 2) + 4 * (size_t)l + (size_t)(j & 3)];
}

int check(const char* name, int L, int n, const std::vector<std::pair<int, int>>& bonds,
          bool double_some, double max_ratio) {
  const mb::HopTable t = hops(L, n, bonds, double_some);
  const int64_t D = (int64_t)t.off.size() - 1;
  const mb::SlicedTable s = mb::sliced_table(t, D);
  const int64_t ng = (D + 31) / 32;
  long long wave = 0, ideal = 0;
  for (int64_t g = 0; g < ng; ++g) {
    const int32_t base = s.grp[(size_t)(2 * g)], k = s.grp[(size_t)(2 * g + 1)];
    if (base % 4) {
      std::printf("%s: group %lld not 16-byte aligned\n", name, (long long)g);
      return 1;
    }
    for (int l = 0; l < 32; ++l) {
      const int64_t c = 32 * g + l;
      std::multiset<uint32_t> want, got;
      int nneg = 0;
      if (c < D) {
        for (int32_t j = t.off[(size_t)c]; j < t.off[(size_t)c + 1]; ++j) {
          const uint32_t e = t.ent[(size_t)j];
          const uint32_t w = (e >> 8) | ((e & 1u) << 31);
          const int mult = (e & 2u) ? 2 : 1;
          for (int r = 0; r < mult; ++r) want.insert(w);
          nneg += (int)(e & 1u) * mult;
        }
      }
      for (int j = 0; j < ((k + 3) & ~3); ++j) {
        const uint32_t w = at(s, base, j, l);
        const uint32_t idx = w & 0x7FFFFFFFu;
        if (idx >= (uint32_t)D) {
          if (w >> 31 || idx >= (uint32_t)(D + mb::kSlicedPads)) {
            std::printf("%s: bad padding %u at group %lld\n", name, w, (long long)g);
            return 1;
          }
        } else {
          got.insert(w);
        }
      }
      if (want != got || (c < D && s.nneg[(size_t)c] != nneg)) {
        std::printf("%s: state %lld entries differ\n", name, (long long)c);
        return 1;
      }
    }
    for (int j = 0; j < k; ++j) {
      for (int q = 0; q < 4; ++q) {
        std::map<uint32_t, std::set<uint32_t>> banks;
        for (int l = 8 * q; l < 8 * q + 8; ++l) {
          const uint32_t idx = at(s, base, j, l) & 0x7FFFFFFFu;
          banks[idx & 7u].insert(idx);
        }
        size_t worst = 0;
        for (auto& kv : banks) worst = std::max(worst, kv.second.size());
        wave += (long long)worst;
      }
      ideal += 4;
    }
  }
  const double ratio = ideal ? (double)wave / (double)ideal : 1.0;
  std::printf("%s: D=%lld wavefronts/minimum %.3f\n", name, (long long)D, ratio);
  return ratio <= max_ratio ? 0 : 1;
}

std::vector<std::pair<int, int>> square(int lx, int ly) {
  std::vector<std::pair<int, int>> b;
  for (int y = 0; y < ly; ++y)
    for (int x = 0; x < lx; ++x) {
      b.push_back({x + lx * y, (x + 1) % lx + lx * y});
      b.push_back({x + lx * y, x + lx * ((y + 1) % ly)});
    }
  return b;
}

std::vector<std::pair<int, int>> chain(int l) {
  std::vector<std::pair<int, int>> b;
  for (int i = 0; i < l; ++i) b.push_back({i, (i + 1) % l});
  return b;
}

}  // namespace

int main() {
  int bad = 0;
  bad += check("square 4x4 n=5", 16, 5, square(4, 4), false, 1.10);
  bad += check("square 4x4 n=6", 16, 6, square(4, 4), false, 1.10);
  bad += check("chain 16 n=8", 16, 8, chain(16), false, 1.10);
  bad += check("square 3x3 n=4 doubled", 9, 4, square(3, 3), true, 1.25);
  bad += check("chain 5 n=2", 5, 2, chain(5), false, 1.5);
  return bad ? 1 : 0;
}
