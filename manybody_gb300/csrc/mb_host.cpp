// Host side of the engine: sector bases, the Hubbard model's bond list, the
// per-spin hop tables, the tridiagonal eigensolver, and the basis / model
// entry points of the C ABI.
#include <algorithm>
#include <functional>
#include <cmath>
#include <cstring>
#include <map>
#include <string>
#include <type_traits>
#include <vector>

#include "mb_internal.h"

namespace mb {

static thread_local std::string g_last_error;

void set_last_error(const std::string& msg) { g_last_error = msg; }

const Binom& binom_table() {
  static const Binom table = [] {
    Binom b{};
    for (int n = 0; n < kMaxOrbitals + 2; ++n) {
      b.c[n][0] = 1;
      for (int k = 1; k <= n; ++k) b.c[n][k] = b.c[n - 1][k - 1] + (k <= n - 1 ? b.c[n - 1][k] : 0);
    }
    return b;
  }();
  return table;
}

// Masks with n of L bits set, in increasing numeric order (= colex order).
static SpinSector make_sector(int L, int n);

SpinSector make_spin_sector(int L, int n) { return make_sector(L, n); }

static SpinSector make_sector(int L, int n) {
  SpinSector s;
  s.L = L;
  s.n = n;
  s.D = binom_at(binom_table(), L, n);
  MB_REQUIRE(s.D <= kMaxSectorDim, MB_ERR_CAPACITY,
             "spin sector C(" + std::to_string(L) + "," + std::to_string(n) +
                 ") exceeds 2^23 states");
  s.masks.resize((size_t)s.D);
  if (n == 0) {
    s.masks[0] = 0;
    return s;
  }
  uint64_t m = (uint64_t(1) << n) - 1;
  for (int64_t r = 0; r < s.D; ++r) {
    s.masks[(size_t)r] = (uint32_t)m;
    // Gosper's hack: next integer with the same popcount.
    const uint64_t c = m & (~m + 1);
    const uint64_t rr = m + c;
    m = (((rr ^ m) >> 2) / c) | rr;
  }
  return s;
}

HopTable build_hop_table(const SpinSector& s, const mb_model_s& m) {
  HopTable t;
  const Binom& B = binom_table();
  t.off.resize((size_t)s.D + 1);
  t.off[0] = 0;
  std::vector<uint32_t> ent;
  ent.reserve((size_t)s.D * 8);
  for (int64_t r = 0; r < s.D; ++r) {
    const uint32_t mask = s.masks[(size_t)r];
    if (m.has_hop) {
      for (const auto& bd : m.bonds) {
        const uint32_t ba = (mask >> bd.a) & 1u, bb = (mask >> bd.b) & 1u;
        if (ba == bb) continue;
        const uint32_t target = mask ^ (1u << bd.a) ^ (1u << bd.b);
        const uint32_t between = ((1u << bd.b) - 1u) & ~((2u << bd.a) - 1u);
        const uint32_t sign = (uint32_t)__builtin_popcount(mask & between) & 1u;
        const int64_t tr = colex_rank(B, target);
        ent.push_back(((uint32_t)tr << 8) | sign | (bd.mult == 2 ? 2u : 0u));
      }
    }
    const int64_t deg = (int64_t)ent.size() - t.off[(size_t)r];
    t.max_degree = std::max<int>(t.max_degree, (int)deg);
    t.off[(size_t)r + 1] = (int32_t)ent.size();
    MB_REQUIRE(ent.size() < (size_t)INT32_MAX, MB_ERR_CAPACITY, "hop table too large");
  }
  t.ent = std::move(ent);
  bool any_self = false;
  for (int v : m.self_mult) any_self = any_self || v;
  if (any_self && m.has_hop) {
    t.has_self = true;
    t.self_energy.assign((size_t)s.D, 0.0);
    for (int64_t r = 0; r < s.D; ++r) {
      const uint32_t mask = s.masks[(size_t)r];
      double e = 0.0;
      for (int i = 0; i < m.L; ++i)
        if (m.self_mult[(size_t)i] && ((mask >> i) & 1u)) e += -2.0 * m.t * m.self_mult[(size_t)i];
      t.self_energy[(size_t)r] = e;
    }
  }
  return t;
}

std::vector<int32_t> rcm_order(const HopTable& t, int64_t D) {
  std::vector<int32_t> order;
  order.reserve((size_t)D);
  std::vector<char> seen((size_t)D, 0);
  auto deg = [&](int64_t r) { return t.off[(size_t)r + 1] - t.off[(size_t)r]; };
  std::vector<int32_t> nb;
  for (int64_t start = 0; (int64_t)order.size() < D; ++start) {
    if (seen[(size_t)start]) continue;
    // the first unvisited state roots a breadth-first sweep of its component
    size_t head = order.size();
    seen[(size_t)start] = 1;
    order.push_back((int32_t)start);
    while (head < order.size()) {
      const int32_t r = order[head++];
      nb.clear();
      for (int32_t j = t.off[(size_t)r]; j < t.off[(size_t)r + 1]; ++j) {
        const int32_t q = (int32_t)(t.ent[(size_t)j] >> 8);
        if (!seen[(size_t)q]) {
          seen[(size_t)q] = 1;
          nb.push_back(q);
        }
      }
      std::sort(nb.begin(), nb.end(), [&](int32_t a, int32_t b) {
        return deg(a) != deg(b) ? deg(a) < deg(b) : a < b;
      });
      order.insert(order.end(), nb.begin(), nb.end());
    }
  }
  std::reverse(order.begin(), order.end());
  return order;
}

SignedLists signed_lists(const HopTable& t, int64_t D) {
  SignedLists s;
  s.off.resize((size_t)D + 1);
  s.pos.resize((size_t)D);
  s.list.reserve(t.ent.size() + 1);
  s.off[0] = 0;
  for (int64_t r = 0; r < D; ++r) {
    const size_t start = s.list.size();
    for (int neg = 0; neg < 2; ++neg) {
      for (int32_t j = t.off[(size_t)r]; j < t.off[(size_t)r + 1]; ++j) {
        const uint32_t e = t.ent[(size_t)j];
        if ((int)(e & 1u) != neg) continue;
        s.list.push_back(e >> 8);
        if (e & 2u) s.list.push_back(e >> 8);
      }
      if (!neg) s.pos[(size_t)r] = (int32_t)(s.list.size() - start);
    }
    MB_REQUIRE(s.list.size() < (size_t)INT32_MAX, MB_ERR_CAPACITY, "hop table too large");
    s.off[(size_t)r + 1] = (int32_t)s.list.size();
    s.max_len = std::max(s.max_len, (int)(s.list.size() - start));
  }
  if (s.list.empty()) s.list.push_back(0u);
  return s;
}

namespace {

// Orders the entries of one quarter warp (8 lanes) over k slots: in each slot
// a maximum matching of lanes to bank groups (target mod 8), lanes that must
// take an entry now (as many left as slots) first, entries of the groups with
// the most entries left preferred (the greedy form of Koenig's edge
// colouring).  A lane left unmatched takes a padding zero element of a group
// no entry uses in that slot, or, if it must take an entry, its first one.
void order_quarter(std::vector<uint32_t> (&lst)[8], int k, uint32_t D, uint32_t* out) {
  constexpr uint32_t kIdx = 0x7FFFFFFFu;
  for (int j = 0; j < k; ++j) {
    const int left = k - j;
    int gdeg[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (auto& l : lst)
      for (uint32_t w : l) ++gdeg[(w & kIdx) & 7u];
    int order[8];
    for (int l = 0; l < 8; ++l) order[l] = l;
    std::stable_sort(order, order + 8, [&](int a, int b) {
      const bool fa = (int)lst[a].size() >= left, fb = (int)lst[b].size() >= left;
      if (fa != fb) return fa;
      return lst[a].size() > lst[b].size();
    });
    int match_g[8], pick[8];
    for (int i = 0; i < 8; ++i) match_g[i] = pick[i] = -1;
    // Kuhn's augmenting paths; candidates by descending group degree
    std::function<bool(int, unsigned&)> augment = [&](int l, unsigned& seen) -> bool {
      int cand[64];
      int nc = 0;
      for (int i = 0; i < (int)lst[l].size() && nc < 64; ++i) cand[nc++] = i;
      std::stable_sort(cand, cand + nc, [&](int a, int b) {
        return gdeg[(lst[l][(size_t)a] & kIdx) & 7u] > gdeg[(lst[l][(size_t)b] & kIdx) & 7u];
      });
      for (int ci = 0; ci < nc; ++ci) {
        const int g = (int)((lst[l][(size_t)cand[ci]] & kIdx) & 7u);
        if (seen & (1u << g)) continue;
        seen |= 1u << g;
        if (match_g[g] < 0 || augment(match_g[g], seen)) {
          match_g[g] = l;
          pick[l] = cand[ci];
          return true;
        }
      }
      return false;
    };
    for (int oi = 0; oi < 8; ++oi) {
      const int l = order[oi];
      if (lst[l].empty()) continue;
      unsigned seen = 0;
      augment(l, seen);
    }
    unsigned used = 0;
    uint32_t slot[8];
    bool taken[8] = {false, false, false, false, false, false, false, false};
    for (int l = 0; l < 8; ++l) {
      if (pick[l] < 0 && !lst[l].empty() && (int)lst[l].size() >= left) pick[l] = 0;
      if (pick[l] >= 0) {
        slot[l] = lst[l][(size_t)pick[l]];
        used |= 1u << ((slot[l] & kIdx) & 7u);
        taken[l] = true;
      }
    }
    // one padding element for every unmatched lane (same address: a broadcast)
    int pg = 0;
    while (pg < 8 && (used & (1u << pg))) ++pg;
    if (pg == 8) pg = 0;
    const uint32_t pad = D + ((uint32_t)pg + 8u - (D & 7u)) % 8u;
    for (int l = 0; l < 8; ++l) {
      if (taken[l]) {
        lst[l].erase(lst[l].begin() + pick[l]);
      } else {
        slot[l] = pad;
      }
      out[(size_t)32 * j + (size_t)l] = slot[l];
    }
  }
}

}  // namespace

SlicedTable sliced_table(const HopTable& t, int64_t D) {
  MB_REQUIRE(D + kSlicedPads < (int64_t(1) << 27), MB_ERR_CAPACITY,
             "sector too large for the sliced table");
  SlicedTable s;
  const int64_t ng = (D + 31) / 32;
  s.grp.resize((size_t)(2 * ng));
  s.nneg.assign((size_t)D, 0);
  std::vector<uint32_t> lst[4][8];
  std::vector<uint32_t> slots;
  for (int64_t g = 0; g < ng; ++g) {
    int k = 0;
    for (int l = 0; l < 32; ++l) {
      auto& col = lst[l >> 3][l & 7];
      col.clear();
      const int64_t c = 32 * g + l;
      if (c >= D) continue;
      for (int32_t j = t.off[(size_t)c]; j < t.off[(size_t)c + 1]; ++j) {
        const uint32_t e = t.ent[(size_t)j];
        const uint32_t w = (e >> 8) | ((e & 1u) << 31);
        col.push_back(w);
        if (e & 2u) col.push_back(w);
        s.nneg[(size_t)c] += (uint8_t)((e & 1u) * ((e & 2u) ? 2 : 1));
      }
      k = std::max(k, (int)col.size());
    }
    const size_t base = s.ent.size();
    const int k4 = (k + 3) & ~3;
    MB_REQUIRE(base + (size_t)32 * k4 < (size_t)INT32_MAX, MB_ERR_CAPACITY, "hop table too large");
    s.grp[(size_t)(2 * g)] = (int32_t)base;
    s.grp[(size_t)(2 * g + 1)] = k;
    slots.assign((size_t)32 * k, (uint32_t)D);
    for (int q = 0; q < 4; ++q) order_quarter(lst[q], k, (uint32_t)D, slots.data() + 8 * q);
    // slots 4i..4i+3 of a lane are one 16-byte word; the last word is padded
    s.ent.resize(base + (size_t)32 * k4, (uint32_t)D);
    for (int j = 0; j < k; ++j)
      for (int l = 0; l < 32; ++l)
        s.ent[base + 128 * (size_t)(j >> 2) + 4 * (size_t)l + (size_t)(j & 3)] =
            slots[(size_t)32 * j + (size_t)l];
  }
  if (s.ent.empty()) s.ent.push_back((uint32_t)D);
  return s;
}

SlicedTable16 sliced_table16(const SlicedTable& s, int64_t D) {
  MB_REQUIRE(D <= kSliced16MaxD, MB_ERR_CAPACITY, "sector too large for 16-bit table entries");
  SlicedTable16 h;
  const int64_t ng = (D + 31) / 32;
  h.grp.resize((size_t)(2 * ng));
  for (int64_t g = 0; g < ng; ++g) {
    const size_t base = (size_t)s.grp[(size_t)(2 * g)];
    const int k = s.grp[(size_t)(2 * g + 1)];
    const int k8 = (k + 7) & ~7;
    const size_t b16 = h.ent.size();
    h.grp[(size_t)(2 * g)] = (int32_t)b16;
    h.grp[(size_t)(2 * g + 1)] = k;
    // the slots past k in the last word are never read; they point at a zero
    h.ent.resize(b16 + (size_t)32 * k8, (uint16_t)D);
    for (int j = 0; j < k; ++j)
      for (int l = 0; l < 32; ++l) {
        const uint32_t w = s.ent[base + 128 * (size_t)(j >> 2) + 4 * (size_t)l + (size_t)(j & 3)];
        h.ent[b16 + 256 * (size_t)(j >> 3) + 8 * (size_t)l + (size_t)(j & 7)] =
            (uint16_t)((w & 0x7FFFu) | ((w >> 31) << 15));
      }
  }
  if (h.ent.empty()) h.ent.push_back((uint16_t)D);
  return h;
}

// Largest eigenvalue of the symmetric tridiagonal T_m (diagonal a, off-
// diagonal b) by bisection on the Sturm count (number of eigenvalues below x
// = number of negative pivots of the LDL^T factorisation of T - x).
double tridiag_max_eig(const double* a, const double* b, int m) {
  double lo = a[0], hi = a[0];
  for (int i = 0; i < m; ++i) {
    const double r = (i > 0 ? std::fabs(b[i - 1]) : 0.0) + (i + 1 < m ? std::fabs(b[i]) : 0.0);
    lo = std::min(lo, a[i] - r);
    hi = std::max(hi, a[i] + r);
  }
  const double tiny = 1e-300;
  for (int it = 0; it < 200; ++it) {
    const double mid = 0.5 * (lo + hi);
    if (!(mid > lo && mid < hi)) break;
    int below = 0;
    double q = 1.0;
    for (int i = 0; i < m; ++i) {
      q = a[i] - mid - (i > 0 ? b[i - 1] * b[i - 1] / q : 0.0);
      if (q == 0.0) q = -tiny;
      if (q < 0.0) ++below;
    }
    if (below == m) hi = mid;
    else lo = mid;
  }
  return hi;
}

int ritz_vector_steps(const std::vector<double>& a, const std::vector<double>& b, int m,
                      int every, double tol) {
  if (every <= 0) every = 10;
  double prev = 0.0;
  bool have = false;
  int loose = 0;  // first checkpoint within the FP32 rounding level
  for (int k = every; k < m; k += every) {
    const double th = tridiag_max_eig(a.data(), b.data(), k);
    const double moved = std::fabs(th - prev);
    if (have && moved <= tol * std::fabs(th)) return k;
    if (have && !loose && moved <= 1e-7 * std::fabs(th)) loose = k;
    prev = th;
    have = true;
  }
  return loose ? loose : m;
}

void fill_fused_tables(OpView& v, const HopTable& tu, const HopTable& td, int64_t Du, int64_t Dd,
                       const TableUpload& upload) {
  auto put = [&](const auto& vec) {
    using T = typename std::decay_t<decltype(vec)>::value_type;
    return (const T*)upload(vec.data(), sizeof(T) * vec.size());
  };
  const std::vector<int32_t> sched = rcm_order(tu, Du);
  v.row_sched = put(sched);
  const SignedLists ul = signed_lists(tu, Du);
  v.up_list = put(ul.list);
  v.up_loff = put(ul.off);
  v.up_lpos = put(ul.pos);
  v.max_up_list = ul.max_len;
  const SlicedTable sd = sliced_table(td, Dd);
  v.dn_sell = put(sd.ent);
  v.dn_sgrp = put(sd.grp);
  v.dn_nneg = put(sd.nneg);
  if (Dd <= kSliced16MaxD) {
    const SlicedTable16 h = sliced_table16(sd, Dd);
    v.dn_sell16 = put(h.ent);
    v.dn_sgrp16 = put(h.grp);
  }
  if (Du == Dd && tu.off == td.off && tu.ent == td.ent) {
    v.up_sell = v.dn_sell;
    v.up_sgrp = v.dn_sgrp;
    v.up_nneg = v.dn_nneg;
    v.up_sell16 = v.dn_sell16;
    v.up_sgrp16 = v.dn_sgrp16;
  } else {
    const SlicedTable su = sliced_table(tu, Du);
    v.up_sell = put(su.ent);
    v.up_sgrp = put(su.grp);
    v.up_nneg = put(su.nneg);
    if (Du <= kSliced16MaxD) {
      const SlicedTable16 h = sliced_table16(su, Du);
      v.up_sell16 = put(h.ent);
      v.up_sgrp16 = put(h.grp);
    }
  }
  v.row_split = 1;
  v.table_bits = 32;
  v.up_prefetch = 0;
  v.table_stage = 0;
  v.dn_max_words = 0;
  for (size_t g = 1; g < sd.grp.size(); g += 2) v.dn_max_words = std::max(v.dn_max_words, (sd.grp[g] + 3) / 4);
}

std::vector<double> u_fold_table(double u, bool has_u, int L) {
  std::vector<double> f((size_t)L + 1, 0.0);
  double acc = 0.0;
  for (int k = 1; k <= L; ++k) {
    acc = (k == 1) ? u : acc + u;
    f[(size_t)k] = has_u ? acc : 0.0;
  }
  return f;
}

// Symmetric tridiagonal eigenproblem by the implicit QL algorithm with
// Wilkinson shifts (Bowdler, Martin, Reinsch & Wilkinson, Numer. Math. 11,
// 1968; EISPACK tql2).  d: diagonal (n), e: off-diagonal (n-1).  On return d
// holds the eigenvalues ascending and z (if given, n*n column-major) the
// orthonormal eigenvectors.  Replaces arma::eig_sym on T_k
// (src/numerics/lanczos.h:258-270, evolve_state.h:33-47).
bool tridiag_eig(int n, std::vector<double>& d, const std::vector<double>& e_in,
                 std::vector<double>* z) {
  if (n <= 0) return true;
  std::vector<double> e((size_t)n, 0.0);
  for (int i = 0; i + 1 < n; ++i) e[(size_t)i] = e_in[(size_t)i];
  if (z) {
    z->assign((size_t)n * n, 0.0);
    for (int i = 0; i < n; ++i) (*z)[(size_t)i * n + i] = 1.0;
  }
  auto Z = [&](int row, int col) -> double& { return (*z)[(size_t)col * n + row]; };
  const double eps = 2.220446049250313e-16;
  for (int l = 0; l < n; ++l) {
    int iter = 0;
    while (true) {
      int m = l;
      for (; m < n - 1; ++m) {
        const double dd = std::fabs(d[(size_t)m]) + std::fabs(d[(size_t)m + 1]);
        if (std::fabs(e[(size_t)m]) <= eps * dd) break;
      }
      if (m == l) break;
      if (++iter > 64) return false;
      double g = (d[(size_t)l + 1] - d[(size_t)l]) / (2.0 * e[(size_t)l]);
      double r = std::hypot(g, 1.0);
      g = d[(size_t)m] - d[(size_t)l] + e[(size_t)l] / (g + std::copysign(r, g));
      double s = 1.0, c = 1.0, p = 0.0;
      bool deflated = false;
      for (int i = m - 1; i >= l; --i) {
        const double f = s * e[(size_t)i], b = c * e[(size_t)i];
        r = std::hypot(f, g);
        e[(size_t)i + 1] = r;
        if (r == 0.0) {
          d[(size_t)i + 1] -= p;
          e[(size_t)m] = 0.0;
          deflated = true;
          break;
        }
        s = f / r;
        c = g / r;
        g = d[(size_t)i + 1] - p;
        r = (d[(size_t)i] - g) * s + 2.0 * c * b;
        p = s * r;
        d[(size_t)i + 1] = g + p;
        g = c * r - b;
        if (z) {
          for (int k = 0; k < n; ++k) {
            const double zf = Z(k, i + 1);
            Z(k, i + 1) = s * Z(k, i) + c * zf;
            Z(k, i) = c * Z(k, i) - s * zf;
          }
        }
      }
      if (deflated) continue;
      d[(size_t)l] -= p;
      e[(size_t)l] = g;
      e[(size_t)m] = 0.0;
    }
  }
  // Selection sort, ascending, carrying vectors.
  for (int i = 0; i + 1 < n; ++i) {
    int k = i;
    for (int j = i + 1; j < n; ++j)
      if (d[(size_t)j] < d[(size_t)k]) k = j;
    if (k != i) {
      std::swap(d[(size_t)i], d[(size_t)k]);
      if (z)
        for (int r = 0; r < n; ++r) std::swap(Z(r, i), Z(r, k));
    }
  }
  return true;
}

}  // namespace mb

using namespace mb;

// Momentum (flat orbital index) of a set of occupied orbitals on a periodic
// lattice: the componentwise sum of the orbitals' coordinates modulo the
// sizes, first dimension fastest (src/utils/index.h:69-100).
namespace mb {

static int64_t mask_momentum(uint32_t mask, const std::vector<int64_t>& dims) {
  std::vector<int64_t> tot(dims.size(), 0);
  while (mask) {
    const int k = __builtin_ctz(mask);
    mask &= mask - 1;
    int64_t rest = k;
    for (size_t d = 0; d < dims.size(); ++d) {
      tot[d] = (tot[d] + rest % dims[d]) % dims[d];
      rest /= dims[d];
    }
  }
  int64_t flat = 0, stride = 1;
  for (size_t d = 0; d < dims.size(); ++d) {
    flat += tot[d] * stride;
    stride *= dims[d];
  }
  return flat;
}

// Flat index of k + sign * q on the lattice.
int64_t momentum_add(int64_t k, int64_t q, int sign, const std::vector<int64_t>& dims) {
  int64_t flat = 0, stride = 1;
  for (size_t d = 0; d < dims.size(); ++d) {
    const int64_t kd = k % dims[d], qd = q % dims[d];
    flat += ((kd + sign * qd + dims[d]) % dims[d]) * stride;
    k /= dims[d];
    q /= dims[d];
    stride *= dims[d];
  }
  return flat;
}

}  // namespace mb

extern "C" {

int mb_version(void) { return 10000; }

const char* mb_last_error(void) { return g_last_error.c_str(); }

int mb_basis_create_fixed_spin(int64_t orbitals, int64_t particles, int spin_projection,
                               mb_basis_t* out) {
  return guard([&] {
    MB_REQUIRE(out, MB_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    MB_REQUIRE(orbitals >= 1 && orbitals <= kMaxOrbitals, MB_ERR_CAPACITY,
               "orbitals must be in [1, 32]");
    MB_REQUIRE(particles >= 0 && particles <= 2 * orbitals, MB_ERR_INVALID_ARG,
               "particles must be in [0, 2*orbitals]");
    const int64_t sz = spin_projection;
    MB_REQUIRE(std::llabs(sz) <= particles, MB_ERR_INVALID_ARG, "|spin_projection| > particles");
    MB_REQUIRE((particles + sz) % 2 == 0, MB_ERR_INVALID_ARG,
               "particles + spin_projection must be even");
    const int64_t up = (particles + sz) / 2, down = particles - up;
    MB_REQUIRE(up <= orbitals && down <= orbitals, MB_ERR_INVALID_ARG,
               "more particles of one spin than orbitals");
    auto b = std::make_unique<mb_basis_s>();
    b->L = (int)orbitals;
    b->n_up = (int)up;
    b->n_down = (int)down;
    b->up = make_sector(b->L, b->n_up);
    b->down = make_sector(b->L, b->n_down);
    b->dim = b->up.D * b->down.D;
    MB_REQUIRE(b->dim < (int64_t)INT32_MAX, MB_ERR_CAPACITY, "sector dimension exceeds 2^31");
    *out = b.release();
  });
}

int mb_basis_create_fixed_number(int64_t orbitals, int64_t particles, mb_basis_t* out) {
  return guard([&] {
    MB_REQUIRE(out, MB_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    MB_REQUIRE(orbitals >= 1 && orbitals <= kMaxOrbitals, MB_ERR_CAPACITY,
               "orbitals must be in [1, 32]");
    MB_REQUIRE(particles >= 0 && particles <= 2 * orbitals, MB_ERR_INVALID_ARG,
               "particles must be in [0, 2*orbitals]");
    auto b = std::make_unique<mb_basis_s>();
    b->L = (int)orbitals;
    b->particles = (int)particles;
    b->n_up = -1;
    b->n_down = -1;
    const Binom& B = binom_table();
    b->sz_off.push_back(0);
    for (int64_t nu = std::max<int64_t>(0, particles - orbitals); nu <= std::min(particles, orbitals); ++nu) {
      const int64_t d = binom_at(B, (int)orbitals, (int)nu) * binom_at(B, (int)orbitals, (int)(particles - nu));
      MB_REQUIRE(binom_at(B, (int)orbitals, (int)nu) <= kMaxSectorDim &&
                     binom_at(B, (int)orbitals, (int)(particles - nu)) <= kMaxSectorDim,
                 MB_ERR_CAPACITY, "a spin sector exceeds 2^23 states");
      b->sz_nup.push_back((int)nu);
      b->sz_off.push_back(b->sz_off.back() + d);
    }
    b->dim = b->sz_off.back();
    MB_REQUIRE(b->dim < (int64_t)INT32_MAX, MB_ERR_CAPACITY, "basis dimension exceeds 2^31");
    *out = b.release();
  });
}

int mb_basis_create_momentum(const int64_t* dims, int ndim, int64_t particles,
                             int spin_projection, const int64_t* momentum, mb_basis_t* out) {
  return guard([&] {
    MB_REQUIRE(dims && momentum && out && ndim >= 1 && ndim <= 3, MB_ERR_INVALID_ARG,
               "NULL argument or ndim outside 1..3");
    *out = nullptr;
    int64_t L = 1;
    std::vector<int64_t> kd(dims, dims + ndim), kv(momentum, momentum + ndim);
    for (int d = 0; d < ndim; ++d) {
      MB_REQUIRE(dims[d] >= 1, MB_ERR_INVALID_ARG, "lattice sizes must be >= 1");
      MB_REQUIRE(momentum[d] >= 0 && momentum[d] < dims[d], MB_ERR_INVALID_ARG,
                 "momentum component outside [0, size)");
      L *= dims[d];
      MB_REQUIRE(L <= kMaxOrbitals, MB_ERR_CAPACITY, "more than 32 orbitals");
    }
    mb_basis_t full = nullptr;
    const int rc = mb_basis_create_fixed_spin(L, particles, spin_projection, &full);
    if (rc) throw Error(rc, mb_last_error());
    std::unique_ptr<mb_basis_s> b(full);
    b->kdims = kd;
    b->kvec = kv;
    int64_t K = 0, stride = 1;
    for (int d = 0; d < ndim; ++d) {
      K += kv[(size_t)d] * stride;
      stride *= kd[(size_t)d];
    }
    // down states grouped by momentum
    std::vector<std::vector<uint32_t>> dn_by_p((size_t)L);
    for (uint32_t m : b->down.masks) dn_by_p[(size_t)mask_momentum(m, kd)].push_back(m);
    const Binom& B = binom_table();
    std::vector<std::pair<int64_t, std::pair<uint32_t, uint32_t>>> states;
    for (uint32_t u : b->up.masks) {
      const int64_t pu = mask_momentum(u, kd);
      const auto& group = dn_by_p[(size_t)momentum_add(K, pu, -1, kd)];
      for (uint32_t d : group) states.push_back({reference_rank(B, u, d, b->L), {u, d}});
    }
    std::sort(states.begin(), states.end());
    b->dim = (int64_t)states.size();
    b->kup.resize(states.size());
    b->kdown.resize(states.size());
    b->kfull.resize(states.size());
    for (size_t i = 0; i < states.size(); ++i) {
      b->kfull[i] = states[i].first;
      b->kup[i] = states[i].second.first;
      b->kdown[i] = states[i].second.second;
    }
    *out = b.release();
  });
}

int mb_basis_destroy(mb_basis_t basis) {
  delete basis;
  return MB_OK;
}

int mb_basis_size(mb_basis_t basis, int64_t* dim) {
  return guard([&] {
    MB_REQUIRE(basis && dim, MB_ERR_INVALID_ARG, "NULL argument");
    *dim = basis->dim;
  });
}

int mb_basis_sector(mb_basis_t basis, int64_t* orbitals, int64_t* n_up, int64_t* n_down,
                    int64_t* dim_up, int64_t* dim_down) {
  return guard([&] {
    MB_REQUIRE(basis, MB_ERR_INVALID_ARG, "NULL basis");
    if (orbitals) *orbitals = basis->L;
    if (n_up) *n_up = basis->n_up;
    if (n_down) *n_down = basis->n_down;
    if (dim_up) *dim_up = basis->up.D;
    if (dim_down) *dim_down = basis->down.D;
  });
}

int mb_basis_export_reference_order(mb_basis_t basis, uint64_t* up_masks, uint64_t* down_masks) {
  return guard([&] {
    MB_REQUIRE(basis && up_masks && down_masks, MB_ERR_INVALID_ARG, "NULL argument");
    if (basis->momentum()) {
      for (int64_t i = 0; i < basis->dim; ++i) {
        up_masks[i] = basis->kup[(size_t)i];
        down_masks[i] = basis->kdown[(size_t)i];
      }
      return;
    }
    if (basis->all_sz()) {
      const Binom& B = binom_table();
      for (size_t blk = 0; blk < basis->sz_nup.size(); ++blk) {
        const SpinSector su = make_sector(basis->L, basis->sz_nup[blk]);
        const SpinSector sd = make_sector(basis->L, basis->particles - basis->sz_nup[blk]);
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < su.D * sd.D; ++i) {
          const uint32_t u = su.masks[(size_t)(i / sd.D)], d = sd.masks[(size_t)(i % sd.D)];
          const int64_t r = reference_rank_all(B, u, d, basis->L);
          up_masks[r] = u;
          down_masks[r] = d;
        }
      }
      return;
    }
    const Binom& B = binom_table();
    const int64_t Dd = basis->down.D;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < basis->dim; ++i) {
      const uint32_t u = basis->up.masks[(size_t)(i / Dd)], d = basis->down.masks[(size_t)(i % Dd)];
      const int64_t r = reference_rank(B, u, d, basis->L);
      up_masks[r] = u;
      down_masks[r] = d;
    }
  });
}

int mb_basis_index_of(mb_basis_t basis, uint64_t up_mask, uint64_t down_mask, int64_t* index) {
  return guard([&] {
    MB_REQUIRE(basis && index, MB_ERR_INVALID_ARG, "NULL argument");
    const uint64_t lim = basis->L >= 64 ? ~uint64_t(0) : ((uint64_t(1) << basis->L) - 1);
    if (basis->all_sz()) {
      MB_REQUIRE((up_mask & ~lim) == 0 && (down_mask & ~lim) == 0 &&
                     __builtin_popcountll(up_mask) + __builtin_popcountll(down_mask) == basis->particles,
                 MB_ERR_INVALID_ARG, "key is not in the basis");
      *index = reference_rank_all(binom_table(), (uint32_t)up_mask, (uint32_t)down_mask, basis->L);
      return;
    }
    MB_REQUIRE((up_mask & ~lim) == 0 && (down_mask & ~lim) == 0 &&
                   __builtin_popcountll(up_mask) == basis->n_up &&
                   __builtin_popcountll(down_mask) == basis->n_down,
               MB_ERR_INVALID_ARG, "key is not in the basis");
    *index = reference_rank(binom_table(), (uint32_t)up_mask, (uint32_t)down_mask, basis->L);
    if (basis->momentum()) {
      const auto it = std::lower_bound(basis->kfull.begin(), basis->kfull.end(), *index);
      MB_REQUIRE(it != basis->kfull.end() && *it == *index, MB_ERR_INVALID_ARG,
                 "key is not in the basis (other total momentum)");
      *index = it - basis->kfull.begin();
    }
  });
}

int mb_basis_permutation(mb_basis_t basis, int64_t* ref_of_tensor) {
  return guard([&] {
    MB_REQUIRE(basis && ref_of_tensor, MB_ERR_INVALID_ARG, "NULL argument");
    if (basis->momentum()) {  // operators on a momentum sector index it in reference order
      for (int64_t i = 0; i < basis->dim; ++i) ref_of_tensor[i] = i;
      return;
    }
    if (basis->all_sz()) {  // the sectors' tensor blocks, concatenated
      const Binom& B = binom_table();
      for (size_t blk = 0; blk < basis->sz_nup.size(); ++blk) {
        const SpinSector su = make_sector(basis->L, basis->sz_nup[blk]);
        const SpinSector sd = make_sector(basis->L, basis->particles - basis->sz_nup[blk]);
        const int64_t off = basis->sz_off[blk];
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < su.D * sd.D; ++i)
          ref_of_tensor[off + i] = reference_rank_all(B, su.masks[(size_t)(i / sd.D)],
                                                      sd.masks[(size_t)(i % sd.D)], basis->L);
      }
      return;
    }
    const Binom& B = binom_table();
    const int64_t Dd = basis->down.D;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < basis->dim; ++i)
      ref_of_tensor[i] = reference_rank(B, basis->up.masks[(size_t)(i / Dd)],
                                        basis->down.masks[(size_t)(i % Dd)], basis->L);
  });
}

int mb_hubbard_create(const int64_t* dims, int ndim, double t, double u, mb_model_t* out) {
  return guard([&] {
    MB_REQUIRE(out && dims, MB_ERR_INVALID_ARG, "NULL argument");
    *out = nullptr;
    MB_REQUIRE(ndim >= 1 && ndim <= 3, MB_ERR_INVALID_ARG, "ndim must be 1, 2 or 3");
    int64_t L = 1;
    for (int d = 0; d < ndim; ++d) {
      MB_REQUIRE(dims[d] >= 1, MB_ERR_INVALID_ARG, "lattice dimension of size zero");
      L *= dims[d];
      MB_REQUIRE(L <= kMaxOrbitals, MB_ERR_CAPACITY, "more than 32 sites");
    }
    MB_REQUIRE(std::isfinite(t) && std::isfinite(u), MB_ERR_INVALID_ARG, "t and U must be finite");
    auto m = std::make_unique<mb_model_s>();
    m->dims.assign(dims, dims + ndim);
    m->L = (int)L;
    m->t = t;
    m->u = u;
    m->has_hop = !(t * t < kTol * kTol);
    m->has_u = !(u * u < kTol * kTol);
    m->self_mult.assign((size_t)L, 0);
    const int64_t Lx = dims[0], Ly = ndim > 1 ? dims[1] : 1, Lz = ndim > 2 ? dims[2] : 1;
    std::map<std::pair<int, int>, int> pairs;  // ordered like the reference's site loops
    std::vector<std::pair<int, int>> order;
    for (int64_t x = 0; x < Lx; ++x)
      for (int64_t y = 0; y < Ly; ++y)
        for (int64_t z = 0; z < Lz; ++z) {
          const int site = (int)(x + Lx * (y + Ly * z));
          const int nb[3] = {(int)(((x + 1) % Lx) + Lx * (y + Ly * z)),
                             (int)(x + Lx * (((y + 1) % Ly) + Ly * z)),
                             (int)(x + Lx * (y + Ly * ((z + 1) % Lz)))};
          for (int d = 0; d < ndim; ++d) {
            if (nb[d] == site) {
              m->self_mult[(size_t)site] += 1;
              continue;
            }
            const auto key = std::make_pair(std::min(site, nb[d]), std::max(site, nb[d]));
            if (pairs[key]++ == 0) order.push_back(key);
          }
        }
    for (const auto& k : order) {
      const int mult = pairs[k];
      MB_REQUIRE(mult <= 2, MB_ERR_INVALID_ARG, "bond listed more than twice");
      m->bonds.push_back({k.first, k.second, mult});
    }
    int64_t terms = 0;
    if (m->has_hop) {
      terms += 4 * (int64_t)m->bonds.size();
      for (int v : m->self_mult) terms += v ? 2 : 0;
    }
    if (m->has_u) terms += L;
    m->n_terms = terms;
    *out = m.release();
  });
}

int mb_model_destroy(mb_model_t model) {
  delete model;
  return MB_OK;
}

int mb_hubbard_momentum_create(const int64_t* dims, int ndim, double t, double u,
                               mb_model_t* out) {
  return guard([&] {
    MB_REQUIRE(out && dims, MB_ERR_INVALID_ARG, "NULL argument");
    *out = nullptr;
    MB_REQUIRE(ndim >= 1 && ndim <= 3, MB_ERR_INVALID_ARG, "ndim must be 1, 2 or 3");
    int64_t L = 1;
    for (int d = 0; d < ndim; ++d) {
      MB_REQUIRE(dims[d] >= 1, MB_ERR_INVALID_ARG, "lattice dimension of size zero");
      L *= dims[d];
      MB_REQUIRE(L <= kMaxOrbitals, MB_ERR_CAPACITY, "more than 32 sites");
    }
    MB_REQUIRE(std::isfinite(t) && std::isfinite(u), MB_ERR_INVALID_ARG, "t and U must be finite");
    auto m = std::make_unique<mb_model_s>();
    m->dims.assign(dims, dims + ndim);
    m->L = (int)L;
    m->t = t;
    m->u = u;
    m->momentum = true;
    m->eps.assign((size_t)L, 0.0);
    int64_t kinetic = 0;
    for (int64_t k = 0; k < L; ++k) {
      // epsilon(k) = -2t sum_d cos(2 pi k_d / L_d), accumulated as the
      // reference does (hubbard_model_momentum.h:28-36)
      double e = 0.0;
      int64_t rest = k;
      for (int d = 0; d < ndim; ++d) {
        const double phase = 2.0 * 3.14159265358979323846 * (double)(rest % dims[d]) / (double)dims[d];
        e += -2.0 * t * std::cos(phase);
        rest /= dims[d];
      }
      if (e * e < kTol * kTol) e = 0.0;  // the expression drops |c| < 1000 eps
      m->eps[(size_t)k] = e;
      kinetic += e != 0.0 ? 2 : 0;
    }
    const double uon = u / (double)L;
    m->u_over_n = uon * uon < kTol * kTol ? 0.0 : uon;
    m->has_hop = kinetic > 0;
    m->has_u = m->u_over_n != 0.0;
    m->n_terms = kinetic + (m->has_u ? L * L * L : 0);
    *out = m.release();
  });
}

int mb_model_term_count(mb_model_t model, int64_t* n_terms) {
  return guard([&] {
    MB_REQUIRE(model && n_terms, MB_ERR_INVALID_ARG, "NULL argument");
    *n_terms = model->n_terms;
  });
}

int mb_kpm_jackson_kernel(int64_t n, double* g) {
  return guard([&] {
    MB_REQUIRE(g && n >= 0, MB_ERR_INVALID_ARG, "bad argument");
    const double pi = 3.14159265358979323846;
    const double denom = (double)(n + 1);
    const double cot_val = 1.0 / std::tan(pi / denom);
    for (int64_t k = 0; k <= n; ++k) {
      const double nd = (double)k;
      const double arg = pi * nd / denom;
      g[k] = ((denom - nd) * std::cos(arg) + std::sin(arg) * cot_val) / denom;
    }
  });
}

int mb_kpm_lorentz_kernel(int64_t n, double lambda, double* g) {
  return guard([&] {
    MB_REQUIRE(g && n >= 1, MB_ERR_INVALID_ARG, "bad argument");
    const double sl = std::sinh(lambda);
    for (int64_t k = 0; k <= n; ++k)
      g[k] = std::sinh(lambda * (1.0 - (double)k / (double)n)) / sl;
  });
}

}  // extern "C"
