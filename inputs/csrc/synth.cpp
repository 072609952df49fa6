// synth.cpp - seeded input producers for the CI hot path (libgraspsynth).
// See inputs/grasp_synth.h for what is and is not physical here.
#include "../grasp_synth.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

namespace {

// CGAMMA for a real positive argument (lib9290/cgamma.f90): Stirling series
// with seven Bernoulli terms after shifting the argument to >= 10.
double cgamma_real(double argr) {
  static const double fnum[7] = {1.0, -1.0, 1.0, -1.0, 5.0, -691.0, 7.0};
  static const double fden[7] = {6.0, 30.0, 42.0, 30.0, 66.0, 2730.0, 6.0};
  const double pi = 4.0 * std::atan(1.0);
  const double hlntpi = 0.5 * std::log(pi + pi);
  double fn[7];
  for (int i = 0; i < 7; ++i) {
    const double twoi = 2.0 * (i + 1);
    fn[i] = fnum[i] / fden[i] / (twoi * (twoi - 1.0));
  }
  double argur = argr, ovlfac = 1.0;
  while (argur < 10.0) {
    ovlfac *= argur;
    argur += 1.0;
  }
  double clngr = (argur - 0.5) * std::log(argur) - argur + hlntpi;
  double fac = argur;
  const double obasq = 1.0 / (argur * argur);
  for (int i = 0; i < 7; ++i) {
    fac *= obasq;
    clngr += fn[i] * fac;
  }
  clngr -= std::log(ovlfac);
  return std::exp(clngr);
}

uint64_t splitmix(uint64_t x) {
  x += 0x9e3779b97f4a7c15ull;
  x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
  x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
  return x ^ (x >> 31);
}
double u01(uint64_t h) { return (double)(h >> 11) * (1.0 / 9007199254740992.0); }

bool tri(int la, int k, int lb) { return (k + la + lb) % 2 == 0 && std::abs(la - lb) <= k && k <= la + lb; }

}  // namespace

extern "C" int gs_dcbsrw(int n, int kappa, double z, double c, const double *r, int ntp, double accy, double *e,
                         double *pz, double *p, double *q, int *mtp) {
  // lib9290/dcbsrw.f90:103-232
  if (n <= 0 || kappa == 0 || kappa == n || std::abs(kappa) > n || z <= 0.0 || z > c || ntp < 2) return -1;
  const double alfa = 1.0 / c;
  const double fn = n, fkappa = kappa;
  const int k = std::abs(kappa);
  const double fk = k;
  const int nr = n - k;
  const double fnr = nr;
  const double zalfa = z * alfa;
  const double gamma = std::sqrt(fk * fk - zalfa * zalfa);
  const double twogp1 = gamma + gamma + 1.0;
  const double bign = std::sqrt(fn * fn - 2.0 * fnr * (fk - gamma));
  const double eps = 1.0 / std::sqrt(1.0 + std::pow(zalfa / (gamma + fnr), 2));
  *e = (1.0 - eps) * c * c;
  double nrfac = 1.0;
  for (int i = 1; i <= nr; ++i) nrfac *= i;
  const double rgamm1 = cgamma_real(twogp1 + fnr);
  const double rgamm2 = cgamma_real(twogp1);
  double fac = -std::sqrt(rgamm1) / (rgamm2 * std::sqrt(nrfac)) * std::sqrt(z / (2.0 * bign * bign * (bign - fkappa)));
  if (kappa > 0) fac = -fac;
  const double fg = fac * std::sqrt(1.0 + eps);
  const double ff = fac * std::sqrt(1.0 - eps);
  int iordr1, iordr2;
  if (nr == 0) {
    iordr1 = 0;
    iordr2 = 0;
  } else {
    iordr1 = nr - 1;
    iordr2 = nr;
  }
  std::vector<double> ta(n + 2, 0.0), tb(n + 2, 0.0);
  {
    double facl = 1.0, facn = 1.0, a = -fnr, an1 = a + 1.0, an2 = a, b = twogp1, bn = b;
    int kk = 0;
    for (;;) {
      ++kk;
      const double fden = 1.0 / (facn * bn);
      if (kk <= iordr1) ta[kk] = an1 * fden;
      if (kk <= iordr2) {
        tb[kk] = an2 * fden;
        a += 1.0;
        an1 *= (a + 1.0);
        an2 *= a;
        b += 1.0;
        bn *= b;
        facl += 1.0;
        facn *= facl;
        continue;
      }
      break;
    }
  }
  p[0] = 0.0;
  q[0] = 0.0;
  const double fac2 = (z + z) / bign;
  const double bignmk = bign - fkappa;
  for (int i = 1; i < ntp; ++i) {
    const double rho = fac2 * r[i];
    double rhon = rho, f1 = 1.0, f2 = 1.0;
    int kk = 0;
    for (;;) {
      ++kk;
      if (kk <= iordr1) f1 += ta[kk] * rhon;
      if (kk <= iordr2) {
        f2 += tb[kk] * rhon;
        rhon *= rho;
        continue;
      }
      break;
    }
    f1 = fnr * f1;
    f2 = bignmk * f2;
    const double ovlfac = std::exp(-0.5 * rho) * std::pow(rho, gamma);
    p[i] = fg * ovlfac * (f1 - f2);
    q[i] = ff * ovlfac * (f1 + f2);
  }
  const double cutoff = accy * 0.1;
  int m = ntp + 1;
  for (;;) {
    --m;
    if (m < 1) break;
    if (std::fabs(p[m - 1]) < cutoff || std::fabs(r[m - 1]) > 1.0e50) {
      p[m - 1] = 0.0;
      q[m - 1] = 0.0;
      continue;
    }
    break;
  }
  *mtp = m;
  *pz = fg * std::pow(fac2, gamma) * (fnr - bignmk);
  return 0;
}

extern "C" int gs_screenpar(int nw, const int *nak, int ncore, double *sigma) {
  int nel = 0;
  for (int i = 0; i < ncore && i < nw; ++i) {
    const int nkj = 2 * std::abs(nak[i]) - 1;
    sigma[i] = nel + (nkj + 1) / 2;
    nel += nkj + 1;
  }
  for (int i = ncore; i < nw; ++i) sigma[i] = nel;
  return 0;
}

// ---------------------------------------------------------------------------
// CSF space and synthetic lists
// ---------------------------------------------------------------------------
struct gs_block {
  int nw = 0, ncf = 0, kmaxf = 0;
  int64_t nnz = 0;
  std::vector<std::vector<uint8_t>> confs;
  std::vector<int> conf_of_csf, conf_first;
  std::vector<int64_t> iendc;
  std::vector<int32_t> irow;
  struct L {
    std::vector<int32_t> lab;
    std::vector<int64_t> start;
    std::vector<int32_t> iclmn, loc;
    std::vector<double> coeff;
  };
  std::vector<L> lists;  // 0 = T, 1 + k = V^k
};

namespace {

// number of ways to put q electrons in a j-subshell (2j = nkj) with total
// 2M = m2 (M-scheme distributions), indexed [m2 + offset]
struct MTable {
  // tab[nkj][q] -> vector over 2M from -maxM to maxM
  std::vector<std::vector<std::vector<int64_t>>> tab;
  int maxnkj = 0;
  explicit MTable(int maxnkj_) : maxnkj(maxnkj_) {
    tab.resize(maxnkj + 1);
    for (int nkj = 1; nkj <= maxnkj; nkj += 2) {
      const int ns = nkj + 1;
      tab[nkj].resize(ns + 1);
      const int off = ns * nkj;  // bound on |2M|
      for (int q = 0; q <= ns; ++q) tab[nkj][q].assign(2 * off + 1, 0);
      for (int mask = 0; mask < (1 << ns); ++mask) {
        const int q = __builtin_popcount(mask);
        int m2 = 0;
        for (int b = 0; b < ns; ++b)
          if (mask >> b & 1) m2 += -nkj + 2 * b;
        tab[nkj][q][m2 + off] += 1;
      }
    }
  }
  int64_t count(const std::vector<int> &nkj, const uint8_t *occ, int nw, int twoJ) const {
    // distribution of total 2M by convolution over subshells
    std::vector<int64_t> dist(1, 1);
    int lo = 0;  // 2M value of dist[0]
    for (int a = 0; a < nw; ++a) {
      const int q = occ[a];
      if (q == 0 || q == nkj[a] + 1) continue;
      const auto &t = tab[nkj[a]][q];
      const int off = (nkj[a] + 1) * nkj[a];
      std::vector<int64_t> nd(dist.size() + t.size() - 1, 0);
      for (size_t i = 0; i < dist.size(); ++i)
        if (dist[i])
          for (size_t j = 0; j < t.size(); ++j)
            if (t[j]) nd[i + j] += dist[i] * t[j];
      dist.swap(nd);
      lo += -off;
    }
    auto at = [&](int m2) -> int64_t {
      const int idx = m2 - lo;
      return (idx >= 0 && idx < (int)dist.size()) ? dist[idx] : 0;
    };
    return at(twoJ) - at(twoJ + 2);
  }
};

int rank_diff(const uint8_t *a, const uint8_t *b, int nw, int limit) {
  int d = 0;
  for (int i = 0; i < nw; ++i) {
    const int x = (int)a[i] - (int)b[i];
    if (x > 0) {
      d += x;
      if (d > limit) return d;
    }
  }
  return d;
}

}  // namespace

extern "C" int gs_block_generate(const gs_block_spec *sp, gs_block **out) {
  if (!sp || !out || sp->nw <= 0 || sp->nw >= 215 || sp->nref <= 0 || sp->max_rank < 0 || sp->max_rank > 2)
    return -1;
  const int nw = sp->nw;
  std::vector<int> nkj(nw), lval(nw), full(nw);
  int maxnkj = 1;
  for (int a = 0; a < nw; ++a) {
    const int kap = sp->nak[a];
    if (kap == 0) return -1;
    nkj[a] = 2 * std::abs(kap) - 1;
    lval[a] = kap > 0 ? kap : -kap - 1;
    full[a] = nkj[a] + 1;
    maxnkj = std::max(maxnkj, nkj[a]);
  }
  if (maxnkj > 19) return -1;
  const MTable mt(maxnkj);
  gs_block *B = new gs_block;
  B->nw = nw;
  // --- configurations: references, then their singles, then doubles
  std::unordered_map<std::string, int> seen;
  auto parity_of = [&](const uint8_t *o) {
    int p = 0;
    for (int a = 0; a < nw; ++a) p += o[a] * lval[a];
    return p & 1;
  };
  std::vector<std::vector<uint8_t>> all;
  auto add = [&](const std::vector<uint8_t> &c) {
    std::string key(c.begin(), c.end());
    if (seen.count(key)) return;
    seen.emplace(key, (int)all.size());
    all.push_back(c);
  };
  for (int r = 0; r < sp->nref; ++r) {
    std::vector<uint8_t> c(sp->refs + (size_t)r * nw, sp->refs + (size_t)(r + 1) * nw);
    add(c);
  }
  size_t lo = 0;
  for (int rank = 1; rank <= sp->max_rank; ++rank) {
    const size_t hi = all.size();
    for (size_t ci = lo; ci < hi; ++ci) {
      const std::vector<uint8_t> base = all[ci];
      for (int a = 0; a < nw; ++a) {
        if (sp->frozen[a] || base[a] == 0) continue;
        for (int b = 0; b < nw; ++b) {
          if (b == a || sp->frozen[b] || base[b] >= full[b]) continue;
          std::vector<uint8_t> c = base;
          c[a]--;
          c[b]++;
          add(c);
        }
      }
    }
    lo = 0;  // singles of everything generated so far (keeps order stable)
  }
  // keep parity and J-allowed configurations, in generation order
  int64_t ncf = 0;
  for (auto &c : all) {
    if (parity_of(c.data()) != sp->parity) continue;
    const int64_t n = mt.count(nkj, c.data(), nw, sp->two_j);
    if (n <= 0) continue;
    if (sp->max_ncf > 0 && ncf + n > sp->max_ncf) break;
    B->conf_first.push_back((int)ncf);
    B->confs.push_back(c);
    for (int64_t i = 0; i < n; ++i) B->conf_of_csf.push_back((int)B->confs.size() - 1);
    ncf += n;
  }
  const int nconf = (int)B->confs.size();
  B->conf_first.push_back((int)ncf);
  B->ncf = (int)ncf;
  if (ncf == 0) {
    delete B;
    return -2;
  }
  // --- neighbour configurations (rank <= 2), B < A, in increasing order
  std::vector<std::vector<int>> nb(nconf);
  {
    const int nt = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    std::vector<std::thread> th;
    for (int t = 0; t < nt; ++t)
      th.emplace_back([&, t] {
        for (int A = t; A < nconf; A += nt)
          for (int Bc = 0; Bc < A; ++Bc)
            if (rank_diff(B->confs[A].data(), B->confs[Bc].data(), nw, 2) <= 2) nb[A].push_back(Bc);
      });
    for (auto &x : th) x.join();
  }
  // natural density, thinning probability
  double pairs = 0;
  for (int A = 0; A < nconf; ++A) {
    const double na = B->conf_first[A + 1] - B->conf_first[A];
    pairs += na * (na + 1) / 2;
    for (int Bc : nb[A]) pairs += na * (B->conf_first[Bc + 1] - B->conf_first[Bc]);
  }
  const double natural = pairs / ((double)ncf * (ncf + 1) / 2);
  const double keep = (sp->density > 0 && natural > sp->density) ? sp->density / natural : 1.0;
  const uint64_t seed = sp->seed;
  auto keep_pair = [&](int r, int c) {
    if (r == c || keep >= 1.0) return true;
    return u01(splitmix(seed ^ ((uint64_t)r * 0x100000001b3ull + (uint64_t)c))) < keep;
  };
  // --- structure: lower triangle by rows, diagonal last
  B->iendc.assign(ncf + 1, 0);
  for (int r = 0; r < ncf; ++r) {
    const int A = B->conf_of_csf[r];
    for (int Bc : nb[A])
      for (int c = B->conf_first[Bc]; c < B->conf_first[Bc + 1]; ++c)
        if (keep_pair(r, c)) B->irow.push_back(c + 1);
    for (int c = B->conf_first[A]; c <= r; ++c)
      if (keep_pair(r, c)) B->irow.push_back(c + 1);
    B->iendc[r + 1] = (int64_t)B->irow.size();
  }
  B->nnz = (int64_t)B->irow.size();
  // --- lists
  const int kmaxf = sp->kmaxf;
  B->kmaxf = kmaxf;
  struct Tr {
    int32_t lab, loc, icl;
    double coeff;
  };
  std::vector<std::vector<Tr>> raw(kmaxf + 2);
  auto vlab = [&](int a, int b, int c, int d) -> int32_t {  // canonical R^k(ab;cd) label
    int ia = std::min(a, c), ic = std::max(a, c), ib = std::min(b, d), id = std::max(b, d);
    if (ia > ib || (ia == ib && ic > id)) {
      std::swap(ia, ib);
      std::swap(ic, id);
    }
    return (int32_t)((((int64_t)(ia + 1) * 215 + (ic + 1)) * 215 + (ib + 1)) * 215 + (id + 1));
  };
  const double scale = sp->coeff_scale > 0 ? sp->coeff_scale : 1.0;
  std::vector<int> dn, up, occ;
  for (int r = 0; r < ncf; ++r) {
    const int A = B->conf_of_csf[r];
    const uint8_t *qa = B->confs[A].data();
    for (int64_t pidx = B->iendc[r]; pidx < B->iendc[r + 1]; ++pidx) {
      const int c = B->irow[pidx] - 1;
      const int Bc = B->conf_of_csf[c];
      const uint8_t *qb = B->confs[Bc].data();
      const int32_t loc = (int32_t)(pidx + 1);
      uint64_t h = splitmix(seed * 31u + (uint64_t)loc);
      auto coef = [&](double s) {
        h = splitmix(h);
        return (2.0 * u01(h) - 1.0) * s * scale;
      };
      auto pick = [&](int n) {
        h = splitmix(h);
        return (int)(u01(h) * n);
      };
      dn.clear();
      up.clear();
      occ.clear();
      for (int a = 0; a < nw; ++a) {
        const int d = (int)qb[a] - (int)qa[a];  // column -> row excitation
        for (int t = 0; t < d; ++t) dn.push_back(a);
        for (int t = 0; t < -d; ++t) up.push_back(a);
        if (qa[a] && qb[a]) occ.push_back(a);
      }
      auto emit = [&](int k, int a, int b, int cc, int d, double v) {
        if (k < 0 || k > kmaxf) return;
        raw[1 + k].push_back({vlab(a, b, cc, d), loc, c + 1, v});
      };
      if (dn.empty()) {  // same configuration (includes the diagonal)
        std::vector<int> open;
        for (int a = 0; a < nw; ++a)
          if (qa[a] > 0 && qa[a] < full[a]) open.push_back(a);
        const int nlab = 1 + pick(4);
        for (int t = 0; t < nlab && !open.empty(); ++t) {
          const int a = open[pick((int)open.size())];
          const int b = occ.empty() ? a : occ[pick((int)occ.size())];
          if (a == b) {
            const int k = 2 * (1 + pick(std::max(1, nkj[a] / 2)));
            if (k <= nkj[a] - 1 && tri(lval[a], k, lval[a])) emit(k, a, a, a, a, coef(0.05));
          } else if (pick(2)) {
            const int k = 2 * (1 + pick(std::max(1, std::min(lval[a], lval[b]))));
            if (tri(lval[a], k, lval[a]) && tri(lval[b], k, lval[b])) emit(k, a, b, a, b, coef(0.05));
          } else {
            int k = std::abs(lval[a] - lval[b]) + 2 * pick(std::min(lval[a], lval[b]) + 1);
            if (tri(lval[a], k, lval[b])) emit(k, a, b, b, a, coef(0.05));
          }
        }
      } else if (dn.size() == 1) {  // single excitation a -> b
        const int a = dn[0], b = up[0];
        if (sp->nak[a] == sp->nak[b]) raw[0].push_back({(int32_t)(std::min(a, b) + 1) * 215 + (std::max(a, b) + 1), loc, c + 1, coef(0.5)});
        const int nsp = occ.empty() ? 0 : 1 + pick(std::min(3, (int)occ.size()));
        for (int t = 0; t < nsp; ++t) {
          const int s = occ[pick((int)occ.size())];
          for (int k = 0; k <= std::min(kmaxf, lval[a] + lval[b]); ++k) {
            if (tri(lval[a], k, lval[b]) && tri(lval[s], k, lval[s]) && pick(2)) emit(k, a, s, b, s, coef(0.3));
            if (tri(lval[a], k, lval[s]) && tri(lval[s], k, lval[b]) && pick(3) == 0) emit(k, a, s, s, b, coef(0.2));
          }
        }
      } else {  // double excitation a, a' -> b, b'
        const int a = dn[0], a2 = dn[1], b = up[0], b2 = up[1];
        for (int k = 0; k <= kmaxf; ++k) {
          if (tri(lval[a], k, lval[b]) && tri(lval[a2], k, lval[b2])) emit(k, a, a2, b, b2, coef(0.3));
          if (tri(lval[a], k, lval[b2]) && tri(lval[a2], k, lval[b]) && pick(2)) emit(k, a, a2, b2, b, coef(0.2));
        }
      }
    }
  }
  // group by label (counting sort, stable): the order SORTMEM leaves
  B->lists.resize(kmaxf + 2);
  for (int L = 0; L < kmaxf + 2; ++L) {
    auto &v = raw[L];
    std::vector<int32_t> labs;
    labs.reserve(v.size());
    for (auto &t : v) labs.push_back(t.lab);
    std::sort(labs.begin(), labs.end());
    labs.erase(std::unique(labs.begin(), labs.end()), labs.end());
    std::unordered_map<int32_t, int> id;
    id.reserve(labs.size() * 2);
    for (size_t i = 0; i < labs.size(); ++i) id.emplace(labs[i], (int)i);
    std::vector<int64_t> cnt(labs.size() + 1, 0);
    for (auto &t : v) cnt[id[t.lab] + 1]++;
    for (size_t i = 0; i < labs.size(); ++i) cnt[i + 1] += cnt[i];
    auto &o = B->lists[L];
    o.lab = labs;
    o.start = cnt;
    o.iclmn.assign(v.size(), 0);
    o.loc.assign(v.size(), 0);
    o.coeff.assign(v.size(), 0.0);
    std::vector<int64_t> cur(cnt.begin(), cnt.end() - 1);
    for (auto &t : v) {
      const int64_t p = cur[id[t.lab]]++;
      o.iclmn[p] = t.icl;
      o.loc[p] = t.loc;
      o.coeff[p] = t.coeff;
    }
    std::vector<Tr>().swap(v);
  }
  *out = B;
  return 0;
}

extern "C" void gs_block_free(gs_block *b) { delete b; }

extern "C" int gs_block_sizes(const gs_block *b, int *ncf, int64_t *nnz, int *nconf, int *kmaxf, int64_t *nlab,
                              int64_t *ncontr) {
  if (!b) return -1;
  if (ncf) *ncf = b->ncf;
  if (nnz) *nnz = b->nnz;
  if (nconf) *nconf = (int)b->confs.size();
  if (kmaxf) *kmaxf = b->kmaxf;
  for (size_t L = 0; L < b->lists.size(); ++L) {
    if (nlab) nlab[L] = (int64_t)b->lists[L].lab.size();
    if (ncontr) ncontr[L] = (int64_t)b->lists[L].loc.size();
  }
  return 0;
}

extern "C" int gs_block_structure(const gs_block *b, int64_t *iendc, int32_t *irow, uint8_t *iq) {
  if (!b) return -1;
  if (iendc) std::memcpy(iendc, b->iendc.data(), b->iendc.size() * sizeof(int64_t));
  if (irow) std::memcpy(irow, b->irow.data(), b->irow.size() * sizeof(int32_t));
  if (iq)
    for (int r = 0; r < b->ncf; ++r) std::memcpy(iq + (size_t)r * b->nw, b->confs[b->conf_of_csf[r]].data(), b->nw);
  return 0;
}

extern "C" int gs_block_list(const gs_block *b, int list, int32_t *lab, int64_t *start, int32_t *iclmn, int32_t *loc,
                             double *coeff) {
  if (!b || list < 0 || list >= (int)b->lists.size()) return -1;
  const auto &o = b->lists[list];
  if (lab) std::memcpy(lab, o.lab.data(), o.lab.size() * sizeof(int32_t));
  if (start) std::memcpy(start, o.start.data(), o.start.size() * sizeof(int64_t));
  if (iclmn) std::memcpy(iclmn, o.iclmn.data(), o.iclmn.size() * sizeof(int32_t));
  if (loc) std::memcpy(loc, o.loc.data(), o.loc.size() * sizeof(int32_t));
  if (coeff) std::memcpy(coeff, o.coeff.data(), o.coeff.size() * sizeof(double));
  return 0;
}

namespace {
inline uint64_t sh_mix(uint64_t x) {  // splitmix64 finaliser
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}
struct ShRng {
  uint64_t s;
  double u() {  // uniform in (0, 1)
    s = sh_mix(s);
    return ((double)(s >> 11) + 0.5) * (1.0 / 9007199254740992.0);
  }
  double normal() {  // Box-Muller, one value per call
    const double a = u(), b = u();
    return std::sqrt(-2.0 * std::log(a)) * std::cos(6.283185307179586 * b);
  }
};
// the columns of row r, ascending: Bernoulli(p) per column by geometric skips
template <class F> void sh_row(int r, double lq, uint64_t seed, F &&emit) {
  if (lq >= 0.0) return;  // p = 0
  ShRng g{sh_mix(seed ^ (0xD1B54A32D192ED03ull * (uint64_t)(r + 1)))};
  int64_t c = -1;
  for (;;) {
    c += 1 + (int64_t)std::floor(std::log(g.u()) / lq);
    if (c >= r) break;
    emit((int)c);
  }
}
}  // namespace

extern "C" int gs_synthetic_h(int ncf, double p, uint64_t seed, int64_t *iendc, int32_t *irow, double *emt) {
  if (ncf < 1 || !(p >= 0.0) || p >= 1.0 || !iendc || ((irow == nullptr) != (emt == nullptr))) return -1;
  const double lq = (p > 0.0) ? std::log1p(-p) : 0.0;
  const int nt = std::max(1, std::min(64, (int)std::thread::hardware_concurrency()));
  auto rows = [&](int t, bool fill) {
    const int r0 = (int)((int64_t)ncf * t / nt), r1 = (int)((int64_t)ncf * (t + 1) / nt);
    for (int r = r0; r < r1; ++r) {
      if (!fill) {
        int64_t k = 1;  // the diagonal
        sh_row(r, lq, seed, [&](int) { ++k; });
        iendc[r + 1] = k;
        continue;
      }
      int64_t q = iendc[r];
      ShRng g{sh_mix(~seed ^ (0x9E3779B97F4A7C15ull * (uint64_t)(r + 1)))};  // values
      sh_row(r, lq, seed, [&](int c) {
        irow[q] = c + 1;
        emt[q] = 2e-3 * g.normal();
        ++q;
      });
      irow[q] = r + 1;
      emt[q] = -1000.0 + 30.0 * std::sqrt((double)r / ncf) + 1e-3 * g.normal();
    }
  };
  auto run = [&](bool fill) {
    std::vector<std::thread> th;
    for (int t = 0; t < nt; ++t) th.emplace_back(rows, t, fill);
    for (auto &x : th) x.join();
  };
  if (!irow) {
    iendc[0] = 0;
    run(false);
    for (int r = 0; r < ncf; ++r) iendc[r + 1] += iendc[r];
    return 0;
  }
  run(true);
  return 0;
}
