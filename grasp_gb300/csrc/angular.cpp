// angular.cpp - T/V angular-coefficient lists of the Dirac-Coulomb
// Hamiltonian between jj-coupled CSFs (libgraspangular, host C++).
//
// Route: CSFs as determinant vectors, Slater-Condon rules between
// determinants, transformation of each radial integral's determinant
// coefficients to the CSF basis. See include/grasp_angular.h.
#include "../../include/grasp_angular.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

namespace {

thread_local std::string g_err;
int fail(int st, const std::string &m) {
  g_err = m;
  return st;
}

constexpr int KEYORB = 215;  // label packing key (rmcdhf90/setham.f90:244, 305-310)
constexpr int MAXSO = 256;   // spin-orbitals of one determinant

// ---------------------------------------------------------------------------
// Wigner 3j and Clebsch-Gordan coefficients (all angular momenta doubled)
// ---------------------------------------------------------------------------
struct Factorials {
  double f[171];
  Factorials() {
    f[0] = 1.0;
    for (int i = 1; i <= 170; ++i) f[i] = f[i - 1] * i;
  }
};
const Factorials &fact() {
  static Factorials F;
  return F;
}

// Racah's formula for (j1 j2 j3; m1 m2 m3), arguments doubled.
double threej(int j1, int j2, int j3, int m1, int m2, int m3) {
  if (m1 + m2 + m3 != 0) return 0.0;
  if (std::abs(m1) > j1 || std::abs(m2) > j2 || std::abs(m3) > j3) return 0.0;
  if (((j1 + m1) & 1) || ((j2 + m2) & 1) || ((j3 + m3) & 1)) return 0.0;
  if ((j1 + j2 + j3) & 1) return 0.0;
  if (j3 > j1 + j2 || j3 < std::abs(j1 - j2)) return 0.0;
  const double *f = fact().f;
  const int a = (j1 + j2 - j3) / 2, b = (j1 - j2 + j3) / 2, c = (-j1 + j2 + j3) / 2, d = (j1 + j2 + j3) / 2 + 1;
  const double delta = std::sqrt(f[a] * f[b] * f[c] / f[d]);
  const double pre = std::sqrt(f[(j1 + m1) / 2]) * std::sqrt(f[(j1 - m1) / 2]) * std::sqrt(f[(j2 + m2) / 2]) *
                     std::sqrt(f[(j2 - m2) / 2]) * std::sqrt(f[(j3 + m3) / 2]) * std::sqrt(f[(j3 - m3) / 2]);
  const int t1 = (j2 - j3 - m1) / 2, t2 = (j1 - j3 + m2) / 2;
  const int t3 = (j1 + j2 - j3) / 2, t4 = (j1 - m1) / 2, t5 = (j2 + m2) / 2;
  const int tmin = std::max(0, std::max(t1, t2)), tmax = std::min(t3, std::min(t4, t5));
  double sum = 0.0;
  for (int t = tmin; t <= tmax; ++t) {
    const double den = f[t] * f[t - t1] * f[t - t2] * f[t3 - t] * f[t4 - t] * f[t5 - t];
    sum += ((t & 1) ? -1.0 : 1.0) / den;
  }
  const int ph = (j1 - j2 - m3) / 2;
  return ((ph & 1) ? -1.0 : 1.0) * delta * pre * sum;
}

// <j1 m1 j2 m2 | J M>
double clebsch(int j1, int m1, int j2, int m2, int J, int M) {
  const double w = threej(j1, j2, J, m1, m2, -M);
  if (w == 0.0) return 0.0;
  const int ph = (j1 - j2 + M) / 2;
  return ((ph & 1) ? -1.0 : 1.0) * std::sqrt(J + 1.0) * w;
}

int lval(int kappa) { return kappa > 0 ? kappa : -kappa - 1; }
int twoj(int kappa) { return 2 * std::abs(kappa) - 1; }

// <kappa_a || C^k || kappa_b>
double redck(int ka, int k, int kb) {
  const int la = lval(ka), lb = lval(kb), ja = twoj(ka), jb = twoj(kb);
  if ((la + k + lb) & 1) return 0.0;
  const double w = threej(ja, 2 * k, jb, 1, 0, -1);
  const int ph = (ja + 1) / 2;
  return ((ph & 1) ? -1.0 : 1.0) * std::sqrt((ja + 1.0) * (jb + 1.0)) * w;
}

// ---------------------------------------------------------------------------
// Determinants: bit sets over the spin-orbitals, creation operators applied
// in increasing spin-orbital order (subshell by subshell, m ascending)
// ---------------------------------------------------------------------------
struct Det {
  uint64_t w[4] = {0, 0, 0, 0};
  bool operator==(const Det &o) const { return !std::memcmp(w, o.w, sizeof(w)); }
  bool operator<(const Det &o) const {
    for (int i = 3; i >= 0; --i)
      if (w[i] != o.w[i]) return w[i] < o.w[i];
    return false;
  }
  bool test(int p) const { return (w[p >> 6] >> (p & 63)) & 1; }
  void set(int p) { w[p >> 6] |= 1ull << (p & 63); }
  void clr(int p) { w[p >> 6] &= ~(1ull << (p & 63)); }
  // occupied spin-orbitals below p
  int below(int p) const {
    int n = 0;
    for (int i = 0; i < (p >> 6); ++i) n += __builtin_popcountll(w[i]);
    if (p & 63) n += __builtin_popcountll(w[p >> 6] & ((1ull << (p & 63)) - 1));
    return n;
  }
};
struct DetHash {
  size_t operator()(const Det &d) const {
    uint64_t h = 1469598103934665603ull;
    for (int i = 0; i < 4; ++i) h = (h ^ d.w[i]) * 1099511628211ull + (d.w[i] >> 29);
    return (size_t)h;
  }
};

int popdiff(const Det &a, const Det &b) {
  int n = 0;
  for (int i = 0; i < 4; ++i) n += __builtin_popcountll(a.w[i] ^ b.w[i]);
  return n;
}

// ---------------------------------------------------------------------------
// Small symmetric eigensolver (cyclic Jacobi) for the subshell-state spaces
// ---------------------------------------------------------------------------
void jacobi(int n, std::vector<double> &a, std::vector<double> &v, std::vector<double> &w) {
  v.assign((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) v[(size_t)i * n + i] = 1.0;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0;
    for (int p = 0; p < n; ++p)
      for (int q = p + 1; q < n; ++q) off += a[(size_t)p * n + q] * a[(size_t)p * n + q];
    if (off < 1e-30) break;
    for (int p = 0; p < n; ++p)
      for (int q = p + 1; q < n; ++q) {
        const double apq = a[(size_t)p * n + q];
        if (std::fabs(apq) < 1e-300) continue;
        const double app = a[(size_t)p * n + p], aqq = a[(size_t)q * n + q];
        const double theta = (aqq - app) / (2.0 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < n; ++k) {
          const double akp = a[(size_t)k * n + p], akq = a[(size_t)k * n + q];
          a[(size_t)k * n + p] = c * akp - s * akq;
          a[(size_t)k * n + q] = s * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) {
          const double apk = a[(size_t)p * n + k], aqk = a[(size_t)q * n + k];
          a[(size_t)p * n + k] = c * apk - s * aqk;
          a[(size_t)q * n + k] = s * apk + c * aqk;
        }
        for (int k = 0; k < n; ++k) {
          const double vkp = v[(size_t)k * n + p], vkq = v[(size_t)k * n + q];
          v[(size_t)k * n + p] = c * vkp - s * vkq;
          v[(size_t)k * n + q] = s * vkp + c * vkq;
        }
      }
  }
  w.resize(n);
  for (int i = 0; i < n; ++i) w[i] = a[(size_t)i * n + i];
}

// ---------------------------------------------------------------------------
// Subshell states |j^w nu J M> as vectors over the subshell's determinants
// (bit i = m = i - j). Highest weight from the null space of J+, seniority
// from the quasispin operator S+ S-, lower M by J-.
// ---------------------------------------------------------------------------
using SubVec = std::vector<std::pair<uint32_t, double>>;
struct SubState {
  int tJ = 0;
  std::vector<SubVec> byM;  // index (tM + tJ) / 2
};

int mask_tm(uint32_t mask, int tj) {
  int s = 0;
  for (int i = 0; i <= tj; ++i)
    if ((mask >> i) & 1) s += 2 * i - tj;
  return s;
}
int sign_below(uint32_t mask, int i) { return (__builtin_popcount(mask & ((1u << i) - 1)) & 1) ? -1 : 1; }

// P = S+ S- applied to one determinant (quasispin pair operators)
void apply_pairing(uint32_t mask, int tj, std::map<uint32_t, double> &out, double c) {
  // S- = sum_{m>0} (-1)^(j-m) a_{-m} a_{m}; S+ = sum_{m>0} (-1)^(j-m) a+_{m} a+_{-m}
  std::map<uint32_t, double> mid;
  for (int i = (tj + 1) / 2; i <= tj; ++i) {  // m = i - j > 0
    const int ineg = tj - i;                   // -m
    if (!((mask >> i) & 1) || !((mask >> ineg) & 1)) continue;
    const int ph = ((tj - (2 * i - tj)) / 2) & 1 ? -1 : 1;
    uint32_t m1 = mask;
    int s = sign_below(m1, i);
    m1 &= ~(1u << i);
    s *= sign_below(m1, ineg);
    m1 &= ~(1u << ineg);
    mid[m1] += c * ph * s;
  }
  for (auto &kv : mid) {
    for (int i = (tj + 1) / 2; i <= tj; ++i) {
      const int ineg = tj - i;
      if (((kv.first >> i) & 1) || ((kv.first >> ineg) & 1)) continue;
      const int ph = ((tj - (2 * i - tj)) / 2) & 1 ? -1 : 1;
      uint32_t m1 = kv.first;
      int s = sign_below(m1, ineg);
      m1 |= 1u << ineg;
      s *= sign_below(m1, i);
      m1 |= 1u << i;
      out[m1] += kv.second * ph * s;
    }
  }
}

// Highest-weight states (2M = 2J = tJ) of j^w: an orthonormal basis of the
// null space of J+ on the M = J determinants, split by seniority where J
// occurs more than once (eigenvectors of S+ S-, eigenvalue S(S+1) - Sz(Sz-1)
// with S = (2j+1-2nu)/4, Sz = (2w-2j-1)/4).
struct HighWeights {
  std::vector<uint32_t> s0;
  std::vector<std::vector<double>> vec;
  std::vector<int> nu;
};

double pairing_eig(int tj, int w, int nu) {
  const double S = (tj + 1 - 2.0 * nu) / 4.0, Sz = (2.0 * w - tj - 1) / 4.0;
  return S * (S + 1) - Sz * (Sz - 1);
}

int highest_weights(int tj, int w, int tJ, HighWeights &hw) {
  hw = HighWeights();
  std::vector<uint32_t> s1;
  for (uint32_t mask = 0; mask < (1u << (tj + 1)); ++mask) {
    if (__builtin_popcount(mask) != w) continue;
    const int tm = mask_tm(mask, tj);
    if (tm == tJ) hw.s0.push_back(mask);
    if (tm == tJ + 2) s1.push_back(mask);
  }
  const int n0 = (int)hw.s0.size(), n1 = (int)s1.size();
  if (n0 == 0) return 0;
  std::unordered_map<uint32_t, int> i1, i0;
  for (int i = 0; i < n1; ++i) i1[s1[i]] = i;
  for (int i = 0; i < n0; ++i) i0[hw.s0[i]] = i;
  std::vector<double> jp((size_t)n1 * n0, 0.0);
  for (int c = 0; c < n0; ++c) {
    const uint32_t mask = hw.s0[c];
    for (int i = 0; i < tj; ++i) {
      if (!((mask >> i) & 1) || ((mask >> (i + 1)) & 1)) continue;
      const uint32_t nm = (mask & ~(1u << i)) | (1u << (i + 1));
      jp[(size_t)i1[nm] * n0 + c] += std::sqrt((double)(tj - i) * (i + 1));
    }
  }
  std::vector<double> g((size_t)n0 * n0, 0.0);
  for (int a = 0; a < n0; ++a)
    for (int b = 0; b < n0; ++b) {
      double x = 0.0;
      for (int r = 0; r < n1; ++r) x += jp[(size_t)r * n0 + a] * jp[(size_t)r * n0 + b];
      g[(size_t)a * n0 + b] = x;
    }
  std::vector<double> v, ev;
  jacobi(n0, g, v, ev);
  std::vector<std::vector<double>> null;
  for (int i = 0; i < n0; ++i)
    if (std::fabs(ev[i]) < 1e-9) {
      std::vector<double> col(n0);
      for (int a = 0; a < n0; ++a) col[a] = v[(size_t)a * n0 + i];
      null.push_back(col);
    }
  const int nn = (int)null.size();
  if (nn == 0) return 0;
  // S+ S- on the M = J determinants, projected on the null space
  std::vector<double> pm((size_t)n0 * n0, 0.0);
  for (int c = 0; c < n0; ++c) {
    std::map<uint32_t, double> out;
    apply_pairing(hw.s0[c], tj, out, 1.0);
    for (auto &kv : out) pm[(size_t)i0[kv.first] * n0 + c] += kv.second;
  }
  std::vector<double> pn((size_t)nn * nn, 0.0);
  for (int a = 0; a < nn; ++a)
    for (int b = 0; b < nn; ++b) {
      double x = 0.0;
      for (int r = 0; r < n0; ++r)
        for (int c = 0; c < n0; ++c) x += null[a][r] * pm[(size_t)r * n0 + c] * null[b][c];
      pn[(size_t)a * nn + b] = x;
    }
  std::vector<double> vv, ew;
  jacobi(nn, pn, vv, ew);
  for (int i = 0; i < nn; ++i) {
    int nu = -1;
    for (int cand = w % 2; cand <= std::min(w, tj + 1 - w); cand += 2)
      if (std::fabs(ew[i] - pairing_eig(tj, w, cand)) < 1e-8) nu = cand;
    if (nu < 0) return fail(-1, "subshell state of unknown seniority");
    std::vector<double> x(n0, 0.0);
    for (int a = 0; a < nn; ++a)
      for (int r = 0; r < n0; ++r) x[r] += vv[(size_t)a * nn + i] * null[a][r];
    double nrm = 0.0;
    for (double y : x) nrm += y * y;
    nrm = std::sqrt(nrm);
    for (double &y : x) y /= nrm;
    hw.vec.push_back(x);
    hw.nu.push_back(nu);
  }
  return 0;
}

// Subshell states |j^w nu J M> with the phase of Clebsch-Gordan coupling:
// j^1 is a+_m; for w >= 2 the sign is the one that makes the state's
// overlap with sum CG(J_p M_p, j m | J M) |j^(w-1) nu_p J_p M_p> a+_m (the
// new electron's operator to the right) positive, for the first parent
// with a non-zero overlap, parents taken by lowest seniority, then lowest
// J_p; seniority-1 states of j^3 take a further (-1)^(j+1/2). For j^2 this
// is the antisymmetrised CG pair state; closed subshells follow the same
// rule (a closed s subshell is -a+_(1/2) a+_(-1/2) in ascending order).
// With these phases the CSFs are the reference's own: for a GRASP-written
// CSF list (1850 CSFs of Ge II with open j^1, j^2 and j^3 subshells, j up
// to 9/2) every mixing coefficient agrees with rmcdhf's in sign as well as
// magnitude. The rule is pinned that far: j^3 states only for j = 5/2 and
// 7/2, nothing beyond three electrons in one open subshell.
std::recursive_mutex g_sub_mu;
std::map<std::tuple<int, int, int, int>, SubState> g_sub_cache;

int cg_substate(int tj, int w, int nu, int tJ, const SubState *&out);

int build_substate(int tj, int w, int nu, int tJ, SubState &st) {
  st.tJ = tJ;
  st.byM.assign(tJ + 1, {});
  if (w == 0) {
    if (tJ != 0) return fail(-1, "empty subshell with J > 0");
    st.byM[0].push_back({0u, 1.0});
    return 0;
  }
  HighWeights hw;
  int rc = highest_weights(tj, w, tJ, hw);
  if (rc) return rc;
  if (hw.vec.empty()) return fail(-1, "subshell state with this J does not exist");
  int pick = -1;
  if (hw.vec.size() == 1) {
    pick = 0;
  } else {
    if (nu <= 0) return fail(-1, "subshell J with several seniorities needs the seniority");
    int count = 0;
    for (size_t i = 0; i < hw.nu.size(); ++i)
      if (hw.nu[i] == nu) {
        pick = (int)i;
        ++count;
      }
    if (count != 1) return fail(-1, "subshell state not fixed by J and seniority");
  }
  std::vector<double> x = hw.vec[pick];
  const int n0 = (int)hw.s0.size();
  double sg = 1.0;
  if (w == 1) {
    sg = x[0] < 0 ? -1.0 : 1.0;
  } else {
    std::vector<std::pair<int, int>> cands;  // (nu_p, tJp)
    for (int tJp = std::abs(tJ - tj); tJp <= tJ + tj; tJp += 2) {
      HighWeights ph;
      if (highest_weights(tj, w - 1, tJp, ph)) return -1;
      for (int v : ph.nu) cands.push_back({v, tJp});
    }
    // lowest parent seniority first, then lowest parent J
    std::sort(cands.begin(), cands.end());
    cands.erase(std::unique(cands.begin(), cands.end()), cands.end());
    std::unordered_map<uint32_t, int> i0;
    for (int i = 0; i < n0; ++i) i0[hw.s0[i]] = i;
    bool fixed = false;
    for (auto &c : cands) {
      const SubState *par = nullptr;
      if (cg_substate(tj, w - 1, c.first, c.second, par)) return -1;
      double ov = 0.0;
      for (int i = 0; i <= tj; ++i) {
        const int tm = 2 * i - tj, tMp = tJ - tm;
        if (std::abs(tMp) > c.second) continue;
        const double cg = clebsch(c.second, tMp, tj, tm, tJ, tJ);
        if (cg == 0.0) continue;
        for (auto &e : par->byM[(tMp + c.second) / 2]) {
          if ((e.first >> i) & 1) continue;
          const int above = __builtin_popcount(e.first >> (i + 1));
          const uint32_t nm = e.first | (1u << i);
          auto it = i0.find(nm);
          if (it == i0.end()) continue;
          ov += x[it->second] * cg * e.second * ((above & 1) ? -1.0 : 1.0);
        }
      }
      if (std::fabs(ov) > 1e-8) {
        sg = ov < 0 ? -1.0 : 1.0;
        // seniority-1 states of three electrons: (-1)^(j+1/2) against the
        // (j^2 0) parent
        if (w == 3 && hw.nu[pick] == 1 && (((tj + 1) / 2) & 1)) sg = -sg;
        fixed = true;
        break;
      }
    }
    if (!fixed) return fail(-1, "subshell state without a parent");
  }
  SubVec top;
  for (int i = 0; i < n0; ++i)
    if (std::fabs(x[i]) > 1e-14) top.push_back({hw.s0[i], sg * x[i]});
  st.byM[tJ] = top;
  // lowering: J- |J M> = sqrt((J+M)(J-M+1)) |J M-1>
  for (int tM = tJ; tM > -tJ; tM -= 2) {
    std::map<uint32_t, double> acc;
    for (auto &e : st.byM[(tM + tJ) / 2]) {
      for (int i = 1; i <= tj; ++i) {
        if (!((e.first >> i) & 1) || ((e.first >> (i - 1)) & 1)) continue;
        const uint32_t nm = (e.first & ~(1u << i)) | (1u << (i - 1));
        acc[nm] += e.second * std::sqrt((double)i * (tj - i + 1));
      }
    }
    const double norm = std::sqrt(((tJ + tM) / 2.0) * ((tJ - tM) / 2.0 + 1.0));
    SubVec lo;
    for (auto &kv : acc)
      if (std::fabs(kv.second) > 1e-15) lo.push_back({kv.first, kv.second / norm});
    st.byM[(tM - 2 + tJ) / 2] = lo;
  }
  return 0;
}

int cg_substate(int tj, int w, int nu, int tJ, const SubState *&out) {
  std::lock_guard<std::recursive_mutex> lk(g_sub_mu);
  auto key = std::make_tuple(tj, w, nu, tJ);
  auto it = g_sub_cache.find(key);
  if (it == g_sub_cache.end()) {
    SubState s;
    const int rc = build_substate(tj, w, nu, tJ, s);
    if (rc) return rc;
    it = g_sub_cache.emplace(key, std::move(s)).first;
  }
  out = &it->second;
  return 0;
}

// ---------------------------------------------------------------------------
// Block generation
// ---------------------------------------------------------------------------
struct Orb {
  int kappa, tj, l, off;
};

using Key = uint64_t;  // list (0 = T, 1 + k = V^k) << 32 | label
Key tkey(int a, int b) {  // 1-based orbitals, I(ab)
  if (a > b) std::swap(a, b);
  return (Key)(a * KEYORB + b);
}
Key vkey(int k, int a, int b, int c, int d) {  // R^k(ab;cd): rho_ac (electron 1), rho_bd (electron 2)
  if (a > c) std::swap(a, c);
  if (b > d) std::swap(b, d);
  if (a > b || (a == b && c > d)) {
    std::swap(a, b);
    std::swap(c, d);
  }
  const uint32_t lab = (uint32_t)(((a * KEYORB + c) * KEYORB + b) * KEYORB + d);
  return ((Key)(k + 1) << 32) | lab;
}

using Terms = std::vector<std::pair<Key, double>>;

struct Engine {
  std::vector<Orb> orbs;
  int nso = 0, kmax = 0;
  std::vector<int> so_orb, so_tm;  // orbital (0-based) and 2m of each spin-orbital
  std::vector<double> ck;          // <p|C^k_q|r>, q = m_p - m_r: [(p * nso + r) * (kmax + 1) + k]
  std::vector<char> core;          // orbital full in every CSF of the block

  double cmat(int p, int r, int k) const { return ck[((size_t)p * nso + r) * (kmax + 1) + k]; }

  // <pq|1/r12|rs> = sum_k A^k R^k(orb p orb q; orb r orb s): adds +-A^k to t
  void two_body(int p, int q, int r, int s, double f, Terms &t) const {
    if (so_tm[p] + so_tm[q] != so_tm[r] + so_tm[s]) return;
    const int qq = (so_tm[p] - so_tm[r]) / 2;
    const double ph = (qq & 1) ? -1.0 : 1.0;
    for (int k = 0; k <= kmax; ++k) {
      const double a = cmat(p, r, k);
      if (a == 0.0) continue;
      const double b = cmat(q, s, k);
      if (b == 0.0) continue;
      t.push_back({vkey(k, so_orb[p] + 1, so_orb[q] + 1, so_orb[r] + 1, so_orb[s] + 1), f * ph * a * b});
    }
  }
  // <pq||rs> = <pq|g|rs> - <pq|g|sr>
  void anti(int p, int q, int r, int s, double f, Terms &t) const {
    two_body(p, q, r, s, f, t);
    two_body(p, q, s, r, -f, t);
  }
};

struct BlockOut {
  int ncf = 0;
  int kmaxf = 0;
  std::vector<int64_t> iendc;
  std::vector<int32_t> irow;
  struct List {
    std::vector<int32_t> lab;
    std::vector<int64_t> start;
    std::vector<int32_t> iclmn, loc;
    std::vector<double> coeff;
  };
  std::vector<List> lists;  // T, V^0..V^kmaxf
};

struct Entry {
  int r, s;  // 0-based CSF indices, r >= s
  Key key;
  double c;
};

void add_terms(std::map<Key, double> &m, const Terms &t) {
  for (auto &e : t) m[e.first] += e.second;
}

}  // namespace

struct ga_block {
  BlockOut out;
};

extern "C" {

const char *ga_last_error(void) { return g_err.c_str(); }

int ga_block_generate(const ga_block_spec *spec, ga_block **outp) {
  if (!spec || !outp || spec->nw < 1 || spec->ncsf < 1 || !spec->nak || !spec->iq || !spec->jqs || !spec->xj ||
      spec->two_j < 0)
    return fail(-1, "ga_block_generate: bad arguments");
  *outp = nullptr;
  const int nw = spec->nw, ncsf = spec->ncsf;
  if (nw >= KEYORB) return fail(-1, "ga_block_generate: more subshells than the label key allows");
  const double cutoff = spec->cutoff < 0 ? 1e-12 : spec->cutoff;
  Engine E;
  E.orbs.resize(nw);
  for (int a = 0; a < nw; ++a) {
    const int kap = spec->nak[a];
    if (kap == 0 || std::abs(kap) > 7) return fail(-1, "ga_block_generate: kappa out of range");
    E.orbs[a] = {kap, twoj(kap), lval(kap), E.nso};
    E.nso += twoj(kap) + 1;
    E.kmax = std::max(E.kmax, twoj(kap));
  }
  if (E.nso > MAXSO) return fail(-1, "ga_block_generate: more than 256 spin-orbitals");
  for (int a = 0; a < nw; ++a)
    for (int i = 0; i <= E.orbs[a].tj; ++i) {
      E.so_orb.push_back(a);
      E.so_tm.push_back(2 * i - E.orbs[a].tj);
    }
  // <p|C^k_q|r> for all spin-orbital pairs
  E.ck.assign((size_t)E.nso * E.nso * (E.kmax + 1), 0.0);
  std::vector<double> red((size_t)nw * nw * (E.kmax + 1));
  for (int a = 0; a < nw; ++a)
    for (int c = 0; c < nw; ++c)
      for (int k = 0; k <= E.kmax; ++k) red[((size_t)a * nw + c) * (E.kmax + 1) + k] = redck(E.orbs[a].kappa, k, E.orbs[c].kappa);
  for (int p = 0; p < E.nso; ++p)
    for (int r = 0; r < E.nso; ++r) {
      const int a = E.so_orb[p], c = E.so_orb[r];
      const int ja = E.orbs[a].tj, jc = E.orbs[c].tj, ma = E.so_tm[p], mc = E.so_tm[r];
      for (int k = 0; k <= E.kmax; ++k) {
        const double rd = red[((size_t)a * nw + c) * (E.kmax + 1) + k];
        if (rd == 0.0) continue;
        const double w = threej(ja, 2 * k, jc, -ma, ma - mc, mc);
        if (w == 0.0) continue;
        const int ph = (ja - ma) / 2;
        E.ck[((size_t)p * E.nso + r) * (E.kmax + 1) + k] = ((ph & 1) ? -1.0 : 1.0) * w * rd;
      }
    }
  // subshells full in every CSF: the closed core of the block
  E.core.assign(nw, 1);
  for (int r = 0; r < ncsf; ++r)
    for (int a = 0; a < nw; ++a)
      if (spec->iq[(size_t)r * nw + a] != E.orbs[a].tj + 1) E.core[a] = 0;
  // ---- CSFs as determinant vectors (M = J) ----
  auto sub = [&](int tj, int w, int nu, int tJ, const SubState *&st) -> int { return cg_substate(tj, w, nu, tJ, st); };
  std::vector<std::vector<std::pair<Det, double>>> csfv(ncsf);
  for (int r = 0; r < ncsf; ++r) {
    const uint8_t *iq = spec->iq + (size_t)r * nw;
    Det base;
    std::vector<int> open;
    for (int a = 0; a < nw; ++a) {
      const int full = E.orbs[a].tj + 1;
      if (iq[a] > full) return fail(-1, "ga_block_generate: occupation above 2j+1");
      if (iq[a] == full)
        for (int i = 0; i < full; ++i) base.set(E.orbs[a].off + i);
      else if (iq[a] > 0)
        open.push_back(a);
    }
    // closed subshells carry the phase of their coupled state
    double closed_sign = 1.0;
    for (int a = 0; a < nw; ++a)
      if (iq[a] == E.orbs[a].tj + 1) {
        const SubState *st = nullptr;
        if (sub(E.orbs[a].tj, iq[a], 0, 0, st)) return fail(-1, "closed subshell state: " + g_err);
        closed_sign *= st->byM[0][0].second;
      }
    // coupled state of the open subshells so far, by 2M
    std::map<int, std::map<Det, double>> cur;
    cur[0][base] = closed_sign;
    int tX = 0;
    for (size_t oi = 0; oi < open.size(); ++oi) {
      const int a = open[oi];
      const int tj = E.orbs[a].tj, tJs = spec->jqs[(size_t)r * nw + a];
      const int nu = spec->nu ? spec->nu[(size_t)r * nw + a] : 0;
      const SubState *st = nullptr;
      int rc = sub(tj, iq[a], nu, tJs, st);
      if (rc) return fail(rc, "CSF " + std::to_string(r + 1) + ": " + g_err);
      const int tXn = oi == 0 ? tJs : spec->xj[(size_t)r * nw + a];
      if (tXn < std::abs(tX - tJs) || tXn > tX + tJs || ((tX + tJs + tXn) & 1))
        return fail(-1, "CSF " + std::to_string(r + 1) + ": coupling not allowed by the triangle rule");
      std::map<int, std::map<Det, double>> nxt;
      for (auto &cm : cur) {
        const int tM1 = cm.first;
        for (int tm2 = -tJs; tm2 <= tJs; tm2 += 2) {
          const int tM = tM1 + tm2;
          if (std::abs(tM) > tXn) continue;
          const double cg = clebsch(tX, tM1, tJs, tm2, tXn, tM);
          if (cg == 0.0) continue;
          const SubVec &sv = st->byM[(tm2 + tJs) / 2];
          auto &dst = nxt[tM];
          for (auto &d1 : cm.second)
            for (auto &s2 : sv) {
              Det d = d1.first;
              for (int i = 0; i <= tj; ++i)
                if ((s2.first >> i) & 1) d.set(E.orbs[a].off + i);
              dst[d] += cg * d1.second * s2.second;
            }
        }
      }
      cur.swap(nxt);
      tX = tXn;
    }
    if (tX != spec->two_j) return fail(-1, "CSF " + std::to_string(r + 1) + ": final J is not the block's J");
    auto it = cur.find(spec->two_j);
    if (it == cur.end()) return fail(-1, "CSF " + std::to_string(r + 1) + ": no M = J component");
    double nrm = 0.0;
    for (auto &kv : it->second)
      if (std::fabs(kv.second) > 1e-15) {
        csfv[r].push_back(kv);
        nrm += kv.second * kv.second;
      }
    if (std::fabs(nrm - 1.0) > 1e-9) return fail(-1, "CSF " + std::to_string(r + 1) + ": not normalised");
  }
  // ---- configurations (equal occupations) and their determinants ----
  std::map<std::vector<uint8_t>, int> confidx;
  std::vector<std::vector<int>> conf_csfs;
  std::vector<int> csf_conf(ncsf);
  for (int r = 0; r < ncsf; ++r) {
    std::vector<uint8_t> q(spec->iq + (size_t)r * nw, spec->iq + (size_t)(r + 1) * nw);
    auto it = confidx.find(q);
    if (it == confidx.end()) {
      it = confidx.emplace(q, (int)conf_csfs.size()).first;
      conf_csfs.push_back({});
    }
    conf_csfs[it->second].push_back(r);
    csf_conf[r] = it->second;
  }
  const int nconf = (int)conf_csfs.size();
  std::vector<std::vector<Det>> conf_dets(nconf);
  std::vector<std::vector<double>> conf_c(nconf);  // [ndet x ncsf_c]
  std::vector<std::vector<uint8_t>> conf_iq(nconf);
  for (auto &kv : confidx) conf_iq[kv.second] = kv.first;
  for (int c = 0; c < nconf; ++c) {
    std::map<Det, int> di;
    for (int r : conf_csfs[c])
      for (auto &e : csfv[r]) di.emplace(e.first, 0);
    int n = 0;
    for (auto &kv : di) {
      kv.second = n++;
      conf_dets[c].push_back(kv.first);
    }
    const int nc = (int)conf_csfs[c].size();
    conf_c[c].assign((size_t)n * nc, 0.0);
    for (int j = 0; j < nc; ++j)
      for (auto &e : csfv[conf_csfs[c][j]]) conf_c[c][(size_t)di[e.first] * nc + j] = e.second;
  }
  // ---- closed-core pieces ----
  // constant energy of the core, and for each active orbital a the core
  // potential sum_c [<pc|g|pc> - <pc|g|cp>] (the same for every m of a;
  // m = -j used), and for active a, b of equal kappa the one-body-like
  // core terms sum_c [<pc|g|rc> - <pc|g|cr>] with m_p = m_r
  std::vector<int> core_so;
  for (int p = 0; p < E.nso; ++p)
    if (E.core[E.so_orb[p]]) core_so.push_back(p);
  std::map<Key, double> core_const;
  for (int a = 0; a < nw; ++a)
    if (E.core[a]) core_const[tkey(a + 1, a + 1)] += E.orbs[a].tj + 1;
  {
    Terms t;
    for (size_t i = 0; i < core_so.size(); ++i)
      for (size_t j = i + 1; j < core_so.size(); ++j) E.anti(core_so[i], core_so[j], core_so[i], core_so[j], 1.0, t);
    add_terms(core_const, t);
  }
  std::vector<std::map<Key, double>> coreone((size_t)nw * nw);  // [a * nw + b], kappa_a = kappa_b, active
  for (int a = 0; a < nw; ++a) {
    if (E.core[a]) continue;
    for (int b = 0; b < nw; ++b) {
      if (E.core[b] || E.orbs[b].kappa != E.orbs[a].kappa) continue;
      Terms t;
      const int p = E.orbs[a].off, r = E.orbs[b].off;  // m = -j
      for (int c : core_so) E.anti(p, c, r, c, 1.0, t);
      add_terms(coreone[(size_t)a * nw + b], t);
      coreone[(size_t)a * nw + b][tkey(a + 1, b + 1)] += 1.0;  // I(ab)
    }
  }
  // ---- configuration pairs ----
  std::vector<std::pair<int, int>> pairs;
  for (int A = 0; A < nconf; ++A)
    for (int B = 0; B <= A; ++B) {
      int d = 0;
      for (int a = 0; a < nw; ++a) d += std::abs((int)conf_iq[A][a] - (int)conf_iq[B][a]);
      if (d <= 4) pairs.push_back({A, B});
    }
  std::atomic<size_t> next{0};
  std::mutex mu;
  std::vector<Entry> entries;
  std::string err;
  int nth = spec->nthreads > 0 ? spec->nthreads : (int)std::thread::hardware_concurrency();
  nth = std::max(1, std::min(nth, 64));
  auto worker = [&]() {
    std::vector<Entry> mine;
    for (;;) {
      const size_t pi = next.fetch_add(1);
      if (pi >= pairs.size()) break;
      const int A = pairs[pi].first, B = pairs[pi].second;
      const auto &dA = conf_dets[A], &dB = conf_dets[B];
      const int nA = (int)conf_csfs[A].size(), nB = (int)conf_csfs[B].size();
      const std::vector<double> &cA = conf_c[A], &cB = conf_c[B];
      std::unordered_map<Key, std::vector<double>> acc;
      Terms t;
      for (size_t I = 0; I < dA.size(); ++I)
        for (size_t J = 0; J < dB.size(); ++J) {
          const Det &dI = dA[I], &dJ = dB[J];
          const int nd = popdiff(dI, dJ);
          if (nd > 4) continue;
          t.clear();
          if (nd == 0) {
            // active pairs (core and one-body diagonal pieces are added per CSF)
            std::vector<int> occ;
            for (int p = 0; p < E.nso; ++p)
              if (dI.test(p) && !E.core[E.so_orb[p]]) occ.push_back(p);
            for (size_t i = 0; i < occ.size(); ++i)
              for (size_t j = i + 1; j < occ.size(); ++j) E.anti(occ[i], occ[j], occ[i], occ[j], 1.0, t);
          } else if (nd == 2) {
            int p = -1, r = -1;
            for (int x = 0; x < E.nso; ++x) {
              if (dI.test(x) && !dJ.test(x)) p = x;
              if (dJ.test(x) && !dI.test(x)) r = x;
            }
            Det w = dJ;
            int sg = w.below(r) & 1;
            w.clr(r);
            sg ^= w.below(p) & 1;
            const double f = sg ? -1.0 : 1.0;
            const int a = E.so_orb[p], b = E.so_orb[r];
            if (E.orbs[a].kappa == E.orbs[b].kappa && E.so_tm[p] == E.so_tm[r])
              for (auto &kv : coreone[(size_t)a * nw + b]) t.push_back({kv.first, f * kv.second});
            for (int x = 0; x < E.nso; ++x)
              if (w.test(x) && !E.core[E.so_orb[x]]) E.anti(p, x, r, x, f, t);
          } else {
            int pp[2], rr[2], np = 0, nr = 0;
            for (int x = 0; x < E.nso; ++x) {
              if (dI.test(x) && !dJ.test(x)) pp[np++] = x;
              if (dJ.test(x) && !dI.test(x)) rr[nr++] = x;
            }
            // <I| a+_p a+_q a_s a_r |J>, p < q, r < s
            const int p = pp[0], q = pp[1], r = rr[0], s = rr[1];
            Det w = dJ;
            int sg = w.below(r) & 1;
            w.clr(r);
            sg ^= w.below(s) & 1;
            w.clr(s);
            sg ^= w.below(q) & 1;
            w.set(q);
            sg ^= w.below(p) & 1;
            E.anti(p, q, r, s, sg ? -1.0 : 1.0, t);
          }
          if (t.empty()) continue;
          for (auto &e : t) {
            auto &v = acc[e.first];
            if (v.empty()) v.assign((size_t)nA * nB, 0.0);
            for (int i = 0; i < nA; ++i) {
              const double x = cA[I * nA + i];
              if (x == 0.0) continue;
              const double xe = x * e.second;
              for (int j = 0; j < nB; ++j) v[(size_t)i * nB + j] += xe * cB[J * nB + j];
            }
          }
        }
      if (A == B) {
        // one-body and core diagonal pieces: sum_a IQ(a) [I(aa) + core potential], core energy
        std::map<Key, double> dg = core_const;
        for (int a = 0; a < nw; ++a)
          if (!E.core[a] && conf_iq[A][a])
            for (auto &kv : coreone[(size_t)a * nw + a]) dg[kv.first] += conf_iq[A][a] * kv.second;
        if (spec->average_split) {
          // the pieces rmcdhf's SETHAM adds from IQ (setham.f90:75-209):
          // taken out here so that the lists hold the rest
          const std::vector<uint8_t> &q = conf_iq[A];
          auto clrx2 = [&](int a, int k, int b) {
            const double w = threej(E.orbs[a].tj, 2 * k, E.orbs[b].tj, 1, 0, -1);
            return w * w;
          };
          for (int a = 0; a < nw; ++a) {
            const int qa = q[a];
            if (!qa) continue;
            const bool fa = qa == E.orbs[a].tj + 1;
            dg[tkey(a + 1, a + 1)] -= qa;
            dg[vkey(0, a + 1, a + 1, a + 1, a + 1)] -= (double)(qa * (qa - 1) / 2);
            if (fa)
              for (int k = 2; k <= E.orbs[a].tj - 1; k += 2)
                dg[vkey(k, a + 1, a + 1, a + 1, a + 1)] -= -0.5 * clrx2(a, k, a) * qa * qa;
            for (int b = a + 1; b < nw; ++b) {
              const int qb = q[b];
              if (!qb) continue;
              dg[vkey(0, a + 1, b + 1, a + 1, b + 1)] -= (double)(qa * qb);
              if (!(fa || qb == E.orbs[b].tj + 1)) continue;
              const int kmin0 = std::abs(E.orbs[a].tj - E.orbs[b].tj) / 2;
              const int kmin = (E.orbs[a].kappa * E.orbs[b].kappa > 0) ? kmin0 : kmin0 + 1;
              const int kmax = (E.orbs[a].tj + E.orbs[b].tj) / 2;
              for (int k = kmin; k <= kmax; k += 2)
                dg[vkey(k, a + 1, b + 1, b + 1, a + 1)] -= -(double)(qa * qb) * clrx2(a, k, b);
            }
          }
        }
        for (auto &kv : dg) {
          auto &v = acc[kv.first];
          if (v.empty()) v.assign((size_t)nA * nB, 0.0);
          for (int i = 0; i < nA; ++i) v[(size_t)i * nB + i] += kv.second;
        }
      }
      for (auto &kv : acc)
        for (int i = 0; i < nA; ++i)
          for (int j = 0; j < nB; ++j) {
            const double c = kv.second[(size_t)i * nB + j];
            if (std::fabs(c) <= cutoff) continue;
            int r = conf_csfs[A][i], s = conf_csfs[B][j];
            if (r < s) {
              if (A == B) continue;  // the (s, r) copy is the stored one
              std::swap(r, s);
            }
            mine.push_back({r, s, kv.first, c});
          }
    }
    std::lock_guard<std::mutex> lk(mu);
    entries.insert(entries.end(), mine.begin(), mine.end());
  };
  {
    std::vector<std::thread> th;
    for (int i = 0; i < nth; ++i) th.emplace_back(worker);
    for (auto &x : th) x.join();
  }
  if (!err.empty()) return fail(-1, err);
  // ---- structure: each row's columns ascending, diagonal last ----
  std::vector<std::vector<int>> cols(ncsf);
  for (int r = 0; r < ncsf; ++r) cols[r].push_back(r);
  for (auto &e : entries)
    if (e.s != e.r) cols[e.r].push_back(e.s);
  ga_block *blk = new ga_block();
  BlockOut &o = blk->out;
  o.ncf = ncsf;
  o.iendc.assign(ncsf + 1, 0);
  for (int r = 0; r < ncsf; ++r) {
    auto &c = cols[r];
    std::sort(c.begin(), c.end());
    c.erase(std::unique(c.begin(), c.end()), c.end());
    o.iendc[r + 1] = o.iendc[r] + (int64_t)c.size();
  }
  o.irow.resize(o.iendc[ncsf]);
  for (int r = 0; r < ncsf; ++r)
    for (size_t i = 0; i < cols[r].size(); ++i) o.irow[o.iendc[r] + i] = cols[r][i] + 1;
  auto locof = [&](int r, int s) -> int32_t {
    auto &c = cols[r];
    const size_t i = std::lower_bound(c.begin(), c.end(), s) - c.begin();
    return (int32_t)(o.iendc[r] + (int64_t)i + 1);
  };
  // ---- lists grouped by label, contributions by position ----
  int kmaxf = 0;
  for (auto &e : entries)
    if ((e.key >> 32) > 0) kmaxf = std::max(kmaxf, (int)(e.key >> 32) - 1);
  o.kmaxf = kmaxf;
  o.lists.assign(kmaxf + 2, {});
  std::sort(entries.begin(), entries.end(), [&](const Entry &x, const Entry &y) {
    if (x.key != y.key) return x.key < y.key;
    if (x.r != y.r) return x.r < y.r;
    return x.s < y.s;
  });
  for (size_t i = 0; i < entries.size();) {
    const Key key = entries[i].key;
    BlockOut::List &L = o.lists[(int)(key >> 32)];
    L.lab.push_back((int32_t)(key & 0xffffffffu));
    L.start.push_back((int64_t)L.loc.size());
    for (; i < entries.size() && entries[i].key == key; ++i) {
      L.iclmn.push_back(entries[i].s + 1);
      L.loc.push_back(locof(entries[i].r, entries[i].s));
      L.coeff.push_back(entries[i].c);
    }
  }
  for (auto &L : o.lists) L.start.push_back((int64_t)L.loc.size());
  *outp = blk;
  return 0;
}

void ga_block_free(ga_block *b) { delete b; }

int ga_block_sizes(const ga_block *b, int *ncf, int64_t *nnz, int *kmaxf, int64_t *nlab, int64_t *ncontr) {
  if (!b) return fail(-1, "ga_block_sizes: no block");
  const BlockOut &o = b->out;
  if (ncf) *ncf = o.ncf;
  if (nnz) *nnz = o.iendc.back();
  if (kmaxf) *kmaxf = o.kmaxf;
  for (size_t i = 0; i < o.lists.size(); ++i) {
    if (nlab) nlab[i] = (int64_t)o.lists[i].lab.size();
    if (ncontr) ncontr[i] = (int64_t)o.lists[i].loc.size();
  }
  return 0;
}

int ga_block_structure(const ga_block *b, int64_t *iendc, int32_t *irow) {
  if (!b) return fail(-1, "ga_block_structure: no block");
  if (iendc) std::copy(b->out.iendc.begin(), b->out.iendc.end(), iendc);
  if (irow) std::copy(b->out.irow.begin(), b->out.irow.end(), irow);
  return 0;
}

int ga_block_list(const ga_block *b, int which, int32_t *lab, int64_t *start, int32_t *iclmn, int32_t *loc,
                  double *coeff) {
  if (!b || which < 0 || which >= (int)b->out.lists.size()) return fail(-1, "ga_block_list: bad list index");
  const auto &L = b->out.lists[which];
  if (lab) std::copy(L.lab.begin(), L.lab.end(), lab);
  if (start) std::copy(L.start.begin(), L.start.end(), start);
  if (iclmn) std::copy(L.iclmn.begin(), L.iclmn.end(), iclmn);
  if (loc) std::copy(L.loc.begin(), L.loc.end(), loc);
  if (coeff) std::copy(L.coeff.begin(), L.coeff.end(), coeff);
  return 0;
}

}  // extern "C"
