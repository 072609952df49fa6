// hosteig.cpp - lowest eigenpairs of the small Rayleigh-Ritz matrix S
// (DVDSON's DSPEVX('V','I','U') call, libdvd90/dvdson.f90:724) on the host.
//
// S is at most LIM x LIM (LIM = 2 NVEC + 60 for rci): a few hundred
// kilo-flops of dependent FP64 work per Davidson iteration. A Grace core runs
// this several times faster than one GB300 SM (whose FP64 pipe is narrow),
// so the N-length work stays on the GPU and this k x k problem runs here,
// in FP64, once per iteration.
//
// Algorithm (the one DSPEVX uses): Householder reduction to tridiagonal form,
// eigenvalues by the implicit QL method with Wilkinson shifts, eigenvectors of
// the wanted eigenvalues by inverse iteration (re-orthogonalised within
// clusters), back-transformed by the stored reflectors. References:
// Golub & Van Loan, Matrix Computations (4th ed.), Alg. 8.3.1, 8.3.3, 8.2.2.
#include <algorithm>
#include <cmath>
#include <vector>

namespace gg {

namespace {

struct Tri {
  int n;
  std::vector<double> d, e, v, beta;  // e[i] = T(i+1, i); v: reflector k in column k
};

void tridiag(int n, std::vector<double> &A, Tri &T) {  // A: full, column-major, lower used
  T.n = n;
  T.d.assign(n, 0.0);
  T.e.assign(std::max(1, n - 1), 0.0);
  T.v.assign((size_t)n * n, 0.0);
  T.beta.assign(n, 0.0);
  std::vector<double> p(n), w(n);
  for (int k = 0; k + 2 < n; ++k) {
    const int m = n - k - 1, o = k + 1;
    double *x = &A[(size_t)k * n + o];
    double sig = 0.0;
    for (int i = 1; i < m; ++i) sig += x[i] * x[i];
    double *vk = &T.v[(size_t)k * n];
    vk[0] = 1.0;
    for (int i = 1; i < m; ++i) vk[i] = x[i];
    T.d[k] = A[(size_t)k * n + k];
    if (sig == 0.0) {
      T.e[k] = x[0];
      T.beta[k] = 0.0;
      continue;
    }
    const double mu = std::sqrt(x[0] * x[0] + sig);
    const double v0 = (x[0] <= 0.0) ? x[0] - mu : -sig / (x[0] + mu);
    const double beta = 2.0 * v0 * v0 / (sig + v0 * v0);
    for (int i = 1; i < m; ++i) vk[i] /= v0;
    T.e[k] = mu;
    T.beta[k] = beta;
    for (int i = 0; i < m; ++i) p[i] = 0.0;
    for (int j = 0; j < m; ++j) {
      const double *col = &A[(size_t)(o + j) * n + o];
      const double vj = vk[j];
      // four partial sums: independent chains instead of one dependent one
      double a0 = col[j] * vj, a1 = 0.0, a2 = 0.0, a3 = 0.0;
      int i = j + 1;
      for (; i + 3 < m; i += 4) {
        p[i] += col[i] * vj;
        p[i + 1] += col[i + 1] * vj;
        p[i + 2] += col[i + 2] * vj;
        p[i + 3] += col[i + 3] * vj;
        a0 += col[i] * vk[i];
        a1 += col[i + 1] * vk[i + 1];
        a2 += col[i + 2] * vk[i + 2];
        a3 += col[i + 3] * vk[i + 3];
      }
      for (; i < m; ++i) {
        p[i] += col[i] * vj;
        a0 += col[i] * vk[i];
      }
      p[j] += (a0 + a1) + (a2 + a3);
    }
    double pv = 0.0;
    for (int i = 0; i < m; ++i) {
      p[i] *= beta;
      pv += p[i] * vk[i];
    }
    const double half = 0.5 * beta * pv;
    for (int i = 0; i < m; ++i) w[i] = p[i] - half * vk[i];
    for (int j = 0; j < m; ++j) {
      double *col = &A[(size_t)(o + j) * n + o];
      const double vj = vk[j], wj = w[j];
      for (int i = j; i < m; ++i) col[i] -= vk[i] * wj + w[i] * vj;
    }
  }
  if (n >= 2) {
    T.d[n - 2] = A[(size_t)(n - 2) * n + (n - 2)];
    T.e[n - 2] = A[(size_t)(n - 2) * n + (n - 1)];
  }
  T.d[n - 1] = A[(size_t)(n - 1) * n + (n - 1)];
}

// eigenvalues of the tridiagonal (d, e) by implicit QL; returns false on no convergence
bool ql_values(int n, std::vector<double> d, std::vector<double> e, std::vector<double> &out) {
  e.resize(n, 0.0);
  // e[i] couples i and i+1; shift to the QL convention e[i] couples i-1, i
  std::vector<double> ee(n, 0.0);
  for (int i = 1; i < n; ++i) ee[i - 1] = e[i - 1];
  for (int l = 0; l < n; ++l) {
    int iter = 0, m;
    do {
      for (m = l; m < n - 1; ++m) {
        const double dd = std::fabs(d[m]) + std::fabs(d[m + 1]);
        if (std::fabs(ee[m]) <= 2.220446049250313e-16 * dd) break;
      }
      if (m != l) {
        if (iter++ == 60) return false;
        double g = (d[l + 1] - d[l]) / (2.0 * ee[l]);
        double r = std::sqrt(g * g + 1.0);  // |g| is bounded: e[l] is not negligible here
        g = d[m] - d[l] + ee[l] / (g + (g >= 0 ? std::fabs(r) : -std::fabs(r)));
        double s = 1.0, c = 1.0, p = 0.0;
        int i;
        for (i = m - 1; i >= l; --i) {
          double f = s * ee[i], b = c * ee[i];
          ee[i + 1] = (r = std::sqrt(f * f + g * g));
          if (r == 0.0) {
            d[i + 1] -= p;
            ee[m] = 0.0;
            break;
          }
          s = f / r;
          c = g / r;
          g = d[i + 1] - p;
          r = (d[i] - g) * s + 2.0 * c * b;
          d[i + 1] = g + (p = s * r);
          g = c * r - b;
        }
        if (r == 0.0 && i >= l) continue;
        d[l] -= p;
        ee[l] = g;
        ee[m] = 0.0;
      }
    } while (m != l);
  }
  out = d;
  std::sort(out.begin(), out.end());
  return true;
}

// Lowest m eigenvalues (ascending) of the tridiagonal (d, e) by Sturm-count
// bisection until each is isolated, then Newton's method on det(T - x I)
// kept inside the isolating bracket (Wilkinson, The Algebraic Eigenvalue
// Problem, ch. 5, sec. 37-38: the LDL^T pivots q_i of T - x I count the
// eigenvalues below x, and f'/f = sum q_i'/q_i with one division per step).
// blo/bhi, when given, are brackets known to hold eigenvalue j (the
// interlacing bounds from the previous, smaller projected matrix); they are
// padded by the rounding bound. The active searches are kept in contiguous
// arrays so that the recurrence vectorises across them. Returns false if a
// search does not finish.
bool tri_lowest(int n, const std::vector<double> &d, const std::vector<double> &e, int m, double *w,
                const double *blo = nullptr, const double *bhi = nullptr) {
  const double eps = 2.220446049250313e-16;
  std::vector<double> e2(n, 0.0);
  double gl = d[0], gu = d[0], tnorm = 0.0, emax2 = 0.0;
  for (int i = 0; i < n; ++i) {
    const double el = (i > 0) ? std::fabs(e[i - 1]) : 0.0, er = (i + 1 < n) ? std::fabs(e[i]) : 0.0;
    gl = std::min(gl, d[i] - el - er);
    gu = std::max(gu, d[i] + el + er);
    tnorm = std::max(tnorm, std::fabs(d[i]) + el + er);
    if (i + 1 < n) {
      e2[i] = e[i] * e[i];
      emax2 = std::max(emax2, e2[i]);
    }
  }
  const double pivmin = 2.2250738585072014e-308 * std::max(1.0, emax2) / eps;
  const double pad = 2.0 * eps * n * std::max(tnorm, 1e-300) + 2.0 * pivmin;
  gl -= pad;
  gu += pad;
  const double atol = 4.0 * eps * std::max(tnorm, 1e-300);
  std::vector<double> lo(m, gl), hi(m, gu), xj(m);
  std::vector<int> clo(m, 0), chi(m, n), newton(m, 0), iters(m, 0);
  if (blo && bhi)
    for (int j = 0; j < m; ++j) {
      // a hint is only a bound; an unusable one is ignored
      const double l = std::max(gl, blo[j] - 8.0 * pad), h = std::min(gu, bhi[j] + 8.0 * pad);
      if (l < h) {
        lo[j] = l;
        hi[j] = h;
        clo[j] = (l == gl) ? 0 : -1;  // counts at hinted ends are not known yet
        chi[j] = (h == gu) ? n : -1;
      }
    }
  // compacted state of the active searches
  std::vector<int> act(m);
  std::vector<double> x(m), inv(m), qp(m), S(m);
  std::vector<int> cnt(m);
  for (int j = 0; j < m; ++j) act[j] = j;
  int na = m;
  auto small = [&](int j) {
    return hi[j] - lo[j] <= atol + 2.0 * eps * std::max(std::fabs(lo[j]), std::fabs(hi[j]));
  };
  while (na > 0) {
    for (int a = 0; a < na; ++a) {
      const int j = act[a];
      x[a] = newton[j] ? xj[j] : 0.5 * (lo[j] + hi[j]);
      double q = d[0] - x[a];
      if (std::fabs(q) < pivmin) q = -pivmin;
      const double iv = 1.0 / q;
      cnt[a] = (q < 0.0);
      qp[a] = -1.0;
      S[a] = -iv;
      inv[a] = iv;
    }
    for (int i = 1; i < n; ++i) {
      const double di = d[i], ei2 = e2[i - 1];
      for (int a = 0; a < na; ++a) {
        const double ivp = inv[a];
        double q = (di - x[a]) - ei2 * ivp;
        q = (std::fabs(q) < pivmin) ? -pivmin : q;
        const double dq = -1.0 + ei2 * qp[a] * ivp * ivp;
        const double iv = 1.0 / q;
        cnt[a] += (q < 0.0);
        S[a] += dq * iv;
        qp[a] = dq;
        inv[a] = iv;
      }
    }
    int keep = 0;
    for (int a = 0; a < na; ++a) {
      const int j = act[a];
      if (++iters[j] > 300) return false;
      // keep lambda_j in [lo, hi): count(lo) <= j < count(hi)
      if (cnt[a] <= j) {
        lo[j] = x[a];
        clo[j] = cnt[a];
      } else {
        hi[j] = x[a];
        chi[j] = cnt[a];
      }
      bool done = small(j);
      if (!done && !newton[j] && clo[j] == j && chi[j] == j + 1) {
        newton[j] = 1;  // isolated: Newton from the middle of the bracket
        xj[j] = 0.5 * (lo[j] + hi[j]);
      } else if (!done && newton[j]) {
        const double step = (S[a] != 0.0) ? -1.0 / S[a] : 0.0;
        const double xn = x[a] + step;
        if (std::fabs(step) <= 2.0 * eps * std::fabs(x[a]) + pivmin) {
          done = true;
          xj[j] = (xn > lo[j] && xn < hi[j]) ? xn : x[a];
        } else {
          xj[j] = (xn > lo[j] && xn < hi[j]) ? xn : 0.5 * (lo[j] + hi[j]);
        }
      }
      if (done) {
        w[j] = newton[j] ? xj[j] : 0.5 * (lo[j] + hi[j]);
      } else {
        act[keep++] = j;
      }
    }
    na = keep;
  }
  for (int j = 1; j < m; ++j) w[j] = std::max(w[j], w[j - 1]);
  return true;
}

// Inverse iteration for one eigenvalue lam of T (Golub & Van Loan 8.2.2,
// with LAPACK DSTEIN's stopping rule): LU of T - lam I with partial pivoting,
// then solves from a fixed pseudo-random start, each followed by
// orthogonalisation against the earlier vectors of the same cluster (the
// n-long rows of orth, north of them) and normalisation. It stops two
// solves after the growth |y| of a solve first reached 1 / (10 n eps
// tnorm) (the normalised vector then has a residual at rounding level), and
// after four solves at most.
struct InvWork {
  std::vector<double> u0, u1, u2, l, r0;
  std::vector<char> piv;
  void size(int n) {
    if ((int)u0.size() >= n) return;
    u0.resize(n);
    u1.resize(n);
    u2.resize(n);
    l.resize(n);
    r0.resize(n);
    piv.resize(n);
  }
};

void inv_iter(const Tri &T, double lam, double *x, const double *orth, int north, unsigned seed, double tnorm,
              InvWork &W) {
  const int n = T.n;
  if (n == 1) {
    x[0] = 1.0;
    return;
  }
  const double eps = 2.220446049250313e-16;
  const double tiny = eps * std::max(tnorm, 1e-300);
  W.size(n);
  double *u0 = W.u0.data(), *u1 = W.u1.data(), *u2 = W.u2.data(), *l = W.l.data(), *r0 = W.r0.data();
  char *piv = W.piv.data();
  double a0 = T.d[0] - lam, a1 = T.e[0];
  for (int i = 0; i < n; ++i) {
    double sub = 0, b0 = 0, b1 = 0;
    if (i + 1 < n) {
      sub = T.e[i];
      b0 = T.d[i + 1] - lam;
      b1 = (i + 2 < n) ? T.e[i + 1] : 0.0;
    }
    if (i + 1 < n && std::fabs(sub) > std::fabs(a0)) {
      piv[i] = 1;
      const double m = a0 / sub;
      l[i] = m;
      u0[i] = sub;
      u1[i] = b0;
      u2[i] = b1;
      const double n0 = a1 - m * b0, n1 = -m * b1;
      a0 = n0;
      a1 = n1;
    } else {
      piv[i] = 0;
      if (a0 == 0.0) a0 = tiny;
      const double m = (i + 1 < n) ? sub / a0 : 0.0;
      l[i] = m;
      u0[i] = a0;
      u1[i] = a1;
      u2[i] = 0.0;
      a0 = b0 - m * a1;
      a1 = b1;
    }
  }
  for (int i = 0; i < n; ++i) {
    double d = u0[i];
    if (std::fabs(d) < tiny) d = d < 0 ? -tiny : tiny;
    r0[i] = 1.0 / d;
  }
  unsigned s = 2463534242u ^ (seed * 2654435761u);
  for (int i = 0; i < n; ++i) {
    s ^= s << 13;
    s ^= s >> 17;
    s ^= s << 5;
    x[i] = (double)(s & 0xffff) / 65536.0 - 0.5 + 1e-3;
  }
  {  // start with unit norm, so that the growth of the first solve is |y|
    double nrm = 0.0;
    for (int i = 0; i < n; ++i) nrm += x[i] * x[i];
    const double inv = 1.0 / std::sqrt(nrm);
    for (int i = 0; i < n; ++i) x[i] *= inv;
  }
  const double grown = 1.0 / (10.0 * n * eps * std::max(tnorm, 1e-300));
  int extra = -1;
  for (int it = 0; it < 4; ++it) {
    for (int i = 0; i + 1 < n; ++i) {
      if (piv[i]) std::swap(x[i], x[i + 1]);
      x[i + 1] -= l[i] * x[i];
    }
    for (int i = n - 1; i >= 0; --i) {
      double v = x[i];
      if (i + 1 < n) v -= u1[i] * x[i + 1];
      if (i + 2 < n) v -= u2[i] * x[i + 2];
      x[i] = v * r0[i];
    }
    double nrm = 0.0;
    for (int i = 0; i < n; ++i) nrm += x[i] * x[i];
    const double growth = std::sqrt(nrm);
    for (int q = 0; q < north; ++q) {
      const double *oq = orth + (size_t)q * n;
      double dot = 0.0;
      for (int i = 0; i < n; ++i) dot += oq[i] * x[i];
      for (int i = 0; i < n; ++i) x[i] -= dot * oq[i];
    }
    nrm = 0.0;
    for (int i = 0; i < n; ++i) nrm += x[i] * x[i];
    nrm = std::sqrt(nrm);
    if (nrm == 0.0) nrm = 1.0;
    const double inv = 1.0 / nrm;
    for (int i = 0; i < n; ++i) x[i] *= inv;
    if (extra < 0 && growth >= grown) extra = 1;  // one more solve after the first large growth
    else if (extra > 0 && --extra == 0) break;
  }
}

}  // namespace

// Lowest m eigenvalues of the symmetric n x n matrix given in packed upper
// storage (AP(i + j(j-1)/2) = A(i,j), i <= j), w[m] ascending, and the
// eigenvectors of the lowest mvec of them, z[n x mvec]. blo/bhi (may be
// null): bounds known to hold eigenvalue j, used when 2m <= n.
int sym_eig_lowest(int n, const double *ap, int m, int mvec, double *w, double *z, const double *blo,
                   const double *bhi) {
  if (n <= 0 || m <= 0 || m > n || mvec < 0 || mvec > m) return -1;
  std::vector<double> A((size_t)n * n);
  for (int j = 0; j < n; ++j)
    for (int i = 0; i <= j; ++i) {
      const double v = ap[i + (size_t)j * (j + 1) / 2];
      A[(size_t)j * n + i] = v;
      A[(size_t)i * n + j] = v;
    }
  Tri T;
  tridiag(n, A, T);
  std::vector<double> ev;
  if (2 * m <= n) {
    // the lowest few: isolate and refine each (the DSTEBZ route of DSPEVX)
    ev.assign(m, 0.0);
    if (!tri_lowest(n, T.d, T.e, m, ev.data(), blo, bhi)) return -2;
  } else if (!ql_values(n, T.d, T.e, ev)) {
    return -2;
  }
  double tnorm = 0.0;
  for (int i = 0; i < n; ++i)
    tnorm = std::max(tnorm, std::fabs(T.d[i]) + (i > 0 ? std::fabs(T.e[i - 1]) : 0.0) +
                                (i + 1 < n ? std::fabs(T.e[i]) : 0.0));
  const double ortol = 1e-3 * tnorm, eps = 2.220446049250313e-16;
  // vectors of the current cluster, n-long rows
  std::vector<double> cluster((size_t)n * std::max(mvec, 1));
  int ncl = 0;
  InvWork work;
  std::vector<double> x(n);
  // eigenvectors of T, row-major [n][mvec] so that the back-transformation
  // below runs all vectors together
  std::vector<double> Y((size_t)n * std::max(mvec, 1));
  double prev = 0.0;
  for (int j = 0; j < m; ++j) w[j] = ev[j];
  for (int j = 0; j < mvec; ++j) {
    double lam = ev[j];
    if (j > 0 && lam - prev > ortol) ncl = 0;
    if (j > 0 && lam - prev < 10.0 * eps * std::fabs(lam)) lam = prev + 10.0 * eps * std::fabs(lam);
    inv_iter(T, lam, x.data(), cluster.data(), ncl, (unsigned)j + 1u, tnorm, work);
    std::copy(x.begin(), x.end(), cluster.begin() + (size_t)ncl * n);
    ++ncl;
    prev = lam;
    for (int i = 0; i < n; ++i) Y[(size_t)i * mvec + j] = x[i];
  }
  // z = H_0 H_1 ... H_{n-3} y: reflectors applied last to first, to every
  // vector at once (dots over rows, vectorised across the vectors)
  std::vector<double> dots(std::max(mvec, 1));
  for (int k = n - 3; k >= 0 && mvec > 0; --k) {
    const double beta = T.beta[k];
    if (beta == 0.0) continue;
    const double *vk = &T.v[(size_t)k * n];
    const int mm = n - k - 1;
    double *Yk = &Y[(size_t)(k + 1) * mvec];
    for (int j = 0; j < mvec; ++j) dots[j] = 0.0;
    for (int i = 0; i < mm; ++i) {
      const double vi = vk[i];
      const double *yi = Yk + (size_t)i * mvec;
      for (int j = 0; j < mvec; ++j) dots[j] += vi * yi[j];
    }
    for (int j = 0; j < mvec; ++j) dots[j] *= beta;
    for (int i = 0; i < mm; ++i) {
      const double vi = vk[i];
      double *yi = Yk + (size_t)i * mvec;
      for (int j = 0; j < mvec; ++j) yi[j] -= dots[j] * vi;
    }
  }
  for (int j = 0; j < mvec; ++j)
    for (int i = 0; i < n; ++i) z[(size_t)j * n + i] = Y[(size_t)i * mvec + j];
  return 0;
}

}  // namespace gg
