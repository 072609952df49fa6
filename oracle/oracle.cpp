// oracle.cpp - CPU FP64 restatement of GRASP's CI hot path (test infrastructure).
//
// This file is the checker for the CUDA path; it is never linked into the
// product library. Each function restates one reference subroutine in the
// reference's loop order and FP64 arithmetic; the citation above each
// function names the reference file and lines it follows (paths relative to
// the GRASP source tree). Internally arrays are 1-based, like the Fortran.
#include "oracle.h"

#include <algorithm>
#include <array>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <vector>

namespace {

constexpr int KLIMIT = 20;  // yzk.f90:54
constexpr int KEYORB = 215; // parameter_def_M.f90:22

// Integer power by repeated squaring: the algorithm of libgcc's __powidf2,
// which gfortran uses for REAL**INTEGER with a run-time exponent
// (yzk.f90:76, RTTK(2:N,K) = R(2:N)**K).
double powi(double x, int m) {
  unsigned n = m < 0 ? -(unsigned)m : (unsigned)m;
  double y = (n % 2) ? x : 1.0;
  while (n >>= 1) {
    x = x * x;
    if (n % 2) y = y * x;
  }
  return m < 0 ? 1.0 / y : y;
}

template <class F> void parallel_for(int64_t n, int nthreads, F f) {
  if (nthreads <= 1 || n < 2) {
    for (int64_t i = 0; i < n; ++i) f(i, 0);
    return;
  }
  std::atomic<int64_t> next{0};
  std::vector<std::thread> th;
  const int64_t chunk = 64;
  for (int t = 0; t < nthreads; ++t)
    th.emplace_back([&, t] {
      for (;;) {
        int64_t b = next.fetch_add(chunk);
        if (b >= n) break;
        int64_t e = std::min(n, b + chunk);
        for (int64_t i = b; i < e; ++i) f(i, t);
      }
    });
  for (auto &x : th) x.join();
}

} // namespace

struct or_ctx {
  int n = 0;
  double rnt = 0, h = 0, c = 0, accy = 0;
  std::vector<double> R, RP, RPOR, ZZ; // 1-based, NNN1 = n + 10 (+1 slot)
  double C1 = 0, C2 = 0, C3 = 0, C4 = 0;
  double CNC5C[6][5] = {};  // CNC5C(2:5, 2:4)
  double A13[14][14] = {};  // LIC13_C A(13,13)
  // YZK's SAVEd power tables (yzk.f90:70-95), one row per k = 1..KLIMIT
  std::vector<double> RTTK, RTTKM, RTTK1, RTTKM1, RM;
  int nw = 0, ld = 0;
  std::vector<int> NAK, MF, NKL, NKJ; // 1-based
  std::vector<double> PF, QF;         // [ld x nw] column-major
  double pf(int i, int j) const { return PF[(size_t)(j - 1) * ld + (i - 1)]; }
  double qf(int i, int j) const { return QF[(size_t)(j - 1) * ld + (i - 1)]; }
  size_t nn1() const { return (size_t)n + 16; }
  double rttk(int k, int i) const { return RTTK[(size_t)k * nn1() + i]; }
  double rttkm(int k, int i) const { return RTTKM[(size_t)k * nn1() + i]; }
  double rttk1(int k, int i) const { return RTTK1[(size_t)k * nn1() + i]; }
  double rttkm1(int k, int i) const { return RTTKM1[(size_t)k * nn1() + i]; }
};

namespace {

// ---------------------------------------------------------------------------
// QUAD: lib9290/quad.f90:52-103
// ---------------------------------------------------------------------------
double quad(const or_ctx *g, int mtp, double *TA /* 1-based */) {
  const int mtpm1 = mtp - 1;
  for (int i = 2; i <= mtpm1; ++i) {
    const double tai = TA[i];
    if (std::fabs(tai) <= 0.0) continue;
    const int ip1 = i + 1;
    const double taip1 = TA[ip1];
    const double quott = taip1 / tai;
    if (quott <= 0.0) continue;
    const double frip1 = taip1 / g->RP[ip1];
    double fri = tai / g->RP[i];
    const double ratio = frip1 / fri;
    const double rip1 = g->R[ip1], ri = g->R[i];
    const double sigma = std::log(ratio) / std::log(rip1 / ri);
    fri = ri * fri;
    double result = fri / (sigma + 1.0);
    TA[mtp + 1] = TA[mtp + 2] = TA[mtp + 3] = 0.0;
    result = result + g->C1 * tai;
    double s = 0.0;
    for (int j = ip1; j <= mtp; j += 4)
      s = s + (g->C2 * (TA[j] + TA[j + 2]) + g->C3 * TA[j + 1] + g->C4 * TA[j + 3]);
    result = result + s;
    if ((mtp - i) % 4 == 0) result = result - g->C1 * TA[mtp];
    return result;
  }
  return 0.0;
}

// ---------------------------------------------------------------------------
// YZK: lib9290/yzk.f90:58-224.  ZK -> TA, YK -> TB (1-based, >= n + 5 slots).
// Returns MTP = min(MF(I), MF(J)).
// ---------------------------------------------------------------------------
int yzk(const or_ctx *g, int K, int I, int J, double *ZK, double *YK) {
  const int N = g->n;
  const int MTP = std::min(g->MF[I], g->MF[J]);
  const int MTPP1 = MTP + 1, MTPP3 = MTP + 3, MTPP4 = MTP + 4;
  std::vector<double> RHOP(g->nn1(), 0.0), TEMP(g->nn1(), 0.0), WK(g->nn1(), 0.0);
  for (int ii = 2; ii <= MTP; ++ii)
    RHOP[ii] = g->RP[ii] * (g->pf(ii, I) * g->pf(ii, J) + g->qf(ii, I) * g->qf(ii, J));
  TEMP[1] = 0.0;
  if (K == 0)
    for (int ii = 2; ii <= MTP; ++ii) TEMP[ii] = RHOP[ii];
  else
    for (int ii = 2; ii <= MTP; ++ii) TEMP[ii] = g->rttk(K, ii) * RHOP[ii];
  for (int ii = MTPP1; ii <= MTPP4; ++ii) TEMP[ii] = 0.0;
  ZK[1] = 0.0;
  for (int ii = 2; ii <= 4; ++ii) {
    double sum = 0.0;
    for (int kk = 2; kk <= 5; ++kk) sum = sum + g->CNC5C[kk][ii] * TEMP[kk];
    ZK[ii] = sum;
  }
  for (int ii = 5; ii <= MTPP3; ++ii) {
    const double rtmp = g->C1 * (TEMP[ii - 4] + TEMP[ii]) + g->C2 * (TEMP[ii - 3] + TEMP[ii - 1]) +
                        g->C3 * TEMP[ii - 2];
    ZK[ii] = ZK[ii - 4] + rtmp;
  }
  double zklim;
  if (K == 0) {
    zklim = (I == J) ? 1.0 : 0.0;
    for (int kk = MTPP3; kk >= MTP; --kk) {
      const double dif = ZK[kk] - zklim;
      if (std::fabs(dif) <= g->accy) continue;
      // ZK(KK : KK-((-2-KK)/(-4)-1)*4 : -4) = ... - DIF   (yzk.f90:162-163)
      const int end = kk - ((kk + 2) / 4 - 1) * 4;
      for (int idx = kk; idx >= end; idx -= 4) ZK[idx] = ZK[idx] - dif;
    }
  } else {
    zklim = ZK[MTPP3];
  }
  if (K == 0) {
    for (int ii = MTPP4; ii <= N; ++ii) ZK[ii] = zklim;
  } else {
    for (int ii = 2; ii <= MTPP3; ++ii) ZK[ii] = ZK[ii] * g->rttkm(K, ii);
    for (int ii = MTPP4; ii <= N; ++ii) ZK[ii] = zklim * g->rttkm(K, ii);
  }
  const int NP4 = N + 4;
  for (int ii = NP4; ii >= MTPP1; --ii) WK[ii] = 0.0;
  TEMP[1] = 0.0;
  if (K == 0)
    for (int ii = 2; ii <= MTP; ++ii) TEMP[ii] = RHOP[ii] * g->RM[ii];
  else
    for (int ii = 2; ii <= MTP; ++ii) TEMP[ii] = RHOP[ii] * g->rttkm1(K, ii);
  for (int ii = MTP; ii >= 2; --ii)
    WK[ii] = WK[ii + 4] + g->C1 * (TEMP[ii] + TEMP[ii + 4]) + g->C2 * (TEMP[ii + 1] + TEMP[ii + 3]) +
             g->C3 * TEMP[ii + 2];
  WK[1] = 0.0;
  if (K == 0)
    for (int ii = 2; ii <= MTP; ++ii) WK[ii] = WK[ii] * g->R[ii];
  else
    for (int ii = 2; ii <= MTP; ++ii) WK[ii] = WK[ii] * g->rttk1(K, ii);
  YK[1] = 0.0;
  for (int ii = 2; ii <= N; ++ii) YK[ii] = ZK[ii] + WK[ii];
  return MTP;
}

// SLATER: lib9290/slater.f90:52-67
double slater(const or_ctx *g, int IA, int IB, int IC, int ID, int K, double *TA, double *TB) {
  int mtp = yzk(g, K, IB, ID, TA, TB);
  if (K == 0 && IB == ID)
    mtp = std::min(g->MF[IA], g->MF[IC]);
  else
    mtp = std::min(std::min(mtp, g->MF[IA]), g->MF[IC]);
  TA[1] = 0.0;
  for (int i = 2; i <= mtp; ++i)
    TA[i] = (g->pf(i, IA) * g->pf(i, IC) + g->qf(i, IA) * g->qf(i, IC)) * g->RPOR[i] * TB[i];
  return quad(g, mtp, TA);
}

// DPBDT: lib9290/dpbdt.f90:39-99.  d/di of PF(:,J), QF(:,J) into TA, TB.
void dpbdt(const or_ctx *g, int J, double *TA, double *TB) {
  const int N = g->n;
  const double A1 = g->A13[7][1], A2 = g->A13[7][2], A3 = g->A13[7][3], A4 = g->A13[7][4],
               A5 = g->A13[7][5], A6 = g->A13[7][6];
  for (int i = 1; i <= 6; ++i) {
    double hp = 0.0, hq = 0.0;
    for (int k = 1; k <= 13; ++k) hp = hp + g->A13[i][k] * g->pf(k, J);
    for (int k = 1; k <= 13; ++k) hq = hq + g->A13[i][k] * g->qf(k, J);
    TA[i] = hp;
    TB[i] = hq;
  }
  for (int i = 7; i <= N - 6; ++i) {
    TA[i] = A1 * (g->pf(i - 6, J) - g->pf(i + 6, J)) + A2 * (g->pf(i - 5, J) - g->pf(i + 5, J)) +
            A3 * (g->pf(i - 4, J) - g->pf(i + 4, J)) + A4 * (g->pf(i - 3, J) - g->pf(i + 3, J)) +
            A5 * (g->pf(i - 2, J) - g->pf(i + 2, J)) + A6 * (g->pf(i - 1, J) - g->pf(i + 1, J));
    TB[i] = A1 * (g->qf(i - 6, J) - g->qf(i + 6, J)) + A2 * (g->qf(i - 5, J) - g->qf(i + 5, J)) +
            A3 * (g->qf(i - 4, J) - g->qf(i + 4, J)) + A4 * (g->qf(i - 3, J) - g->qf(i + 3, J)) +
            A5 * (g->qf(i - 2, J) - g->qf(i + 2, J)) + A6 * (g->qf(i - 1, J) - g->qf(i + 1, J));
  }
  for (int i = N - 5; i <= N; ++i) {
    const int irow = i - N + 13;
    double hp = 0.0, hq = 0.0;
    for (int k = 1; k <= 13; ++k) hp = hp + g->A13[irow][k] * g->pf(N - 13 + k, J);
    for (int k = 1; k <= 13; ++k) hq = hq + g->A13[irow][k] * g->qf(N - 13 + k, J);
    TA[i] = hp;
    TB[i] = hq;
  }
}

// RINTI: lib9290/rinti.f90:53-100
double rinti(const or_ctx *g, int J, int K, int MODE, double *TA, double *TB, int *err) {
  if (g->NAK[J] != g->NAK[K]) {
    if (err) *err = 1;
    return 0.0;
  }
  const int mtp = std::max(g->MF[J], g->MF[K]);
  const double C = g->c;
  dpbdt(g, K, TA, TB);
  TA[1] = 0.0;
  for (int i = 2; i <= mtp; ++i) TA[i] = g->qf(i, J) * TA[i] - g->pf(i, J) * TB[i];
  double piece1 = quad(g, mtp, TA);
  piece1 = C * piece1 / g->h;
  TA[1] = 0.0;
  for (int i = 2; i <= mtp; ++i) TA[i] = g->RP[i] * g->qf(i, J) * g->qf(i, K);
  double piece2 = quad(g, mtp, TA);
  piece2 = -2.0 * C * C * piece2;
  TA[1] = 0.0;
  for (int i = 2; i <= mtp; ++i)
    TA[i] = g->RPOR[i] * (g->pf(i, J) * g->qf(i, K) + g->qf(i, J) * g->pf(i, K));
  double piece3 = quad(g, mtp, TA);
  piece3 = piece3 * C * (double)g->NAK[K];
  double piece4 = 0.0;
  if (MODE == 0) {
    TA[1] = 0.0;
    for (int i = 2; i <= mtp; ++i)
      TA[i] = g->RPOR[i] * g->ZZ[i] * (g->pf(i, J) * g->pf(i, K) + g->qf(i, J) * g->qf(i, K));
    piece4 = quad(g, mtp, TA);
    piece4 = -piece4;
  }
  if (err) *err = 0;
  return piece1 + piece2 + piece3 + piece4;
}

// GAM(I) = log((I-1)!) from FACTT (lib9290/factt.f90)
struct Gam {
  double g[512];
  Gam() {
    g[1] = 1.0;
    g[2] = 1.0;
    double x = 2.0;
    for (int i = 3; i <= 30; ++i) {
      g[i] = g[i - 1] * x;
      x = x + 1.0;
    }
    for (int i = 1; i <= 30; ++i) g[i] = std::log(g[i]);
    x = 30.0;
    for (int i = 31; i < 512; ++i) {
      g[i] = g[i - 1] + std::log(x);
      x = x + 1.0;
    }
  }
};
const Gam &gam() {
  static Gam G;
  return G;
}

// CLRX: lib9290/clrx.f90
double clrx(int kappaa, int k, int kappab) {
  const double *GAM = gam().g;
  const int ka = std::abs(kappaa), kb = std::abs(kappab);
  if (std::abs(ka - kb) <= k && ka + kb - 1 >= k) {
    double exptrm = -std::log((double)(ka * kb));
    const int kapkb = ka + kb, kabkp = kapkb + k, kamkb = ka - kb, kbmka = kb - ka;
    exptrm = 0.5 * (exptrm + GAM[kapkb - k] + GAM[kamkb + k + 1] + GAM[kbmka + k + 1] - GAM[kabkp + 1]);
    double r;
    if (kabkp % 2 == 0) {
      r = ((3 * kabkp / 2) % 2 == 0) ? 1.0 : -1.0;
      exptrm = exptrm + GAM[(kabkp + 2) / 2] - GAM[(kapkb - k) / 2] - GAM[(kamkb + k + 2) / 2] -
               GAM[(kbmka + k + 2) / 2];
    } else {
      r = (((3 * kabkp - 1) / 2) % 2 == 0) ? 1.0 : -1.0;
      exptrm = exptrm + GAM[(kabkp + 1) / 2] - GAM[(kapkb - k + 1) / 2] - GAM[(kamkb + k + 1) / 2] -
               GAM[(kbmka + k + 1) / 2];
    }
    return r * std::exp(exptrm);
  }
  return 0.0;
}

// FCO: rmcdhf90/fco.f90 ; GCO: rmcdhf90/gco.f90
double fco(const or_ctx *g, int K, const uint8_t *iqr /* IQ(:,IR), 0-based by orbital */, int IA, int IB) {
  if (IA == IB) {
    const int iqa = iqr[IA - 1];
    if (K == 0) return (double)((iqa * (iqa - 1)) / 2);
    const int iqf = g->NKJ[IA] + 1;
    if (iqa == iqf) {
      const double fac = clrx(g->NAK[IA], K, g->NAK[IA]) * (double)iqa;
      return -0.5 * fac * fac;
    }
    return 0.0;
  }
  if (K == 0) return (double)(iqr[IA - 1] * iqr[IB - 1]);
  return 0.0;
}
double gco(const or_ctx *g, int K, const uint8_t *iqr, int IA, int IB) {
  const int iqa = iqr[IA - 1], iqb = iqr[IB - 1];
  if (iqa == g->NKJ[IA] + 1 || iqb == g->NKJ[IB] + 1) {
    const double fac = clrx(g->NAK[IA], K, g->NAK[IB]);
    return -(double)(iqa * iqb) * fac * fac;
  }
  return 0.0;
}

// ---------------------------------------------------------------------------
// Dense symmetric eigen-solver for selected lowest eigenpairs: restatement of
// the algorithm of LAPACK DSPEVX('V','I',...) = DSPTRD (Householder
// tridiagonalisation) + DSTEBZ (bisection with Sturm counts) + DSTEIN
// (inverse iteration with re-orthogonalisation inside clusters) + DOPMTR
// (back transformation).  Written from the published algorithms (Golub & Van
// Loan, Matrix Computations, 4th ed., Alg. 8.3.1, 8.4.1 and sec. 8.2.2).
// ---------------------------------------------------------------------------
struct Tridiag {
  int n;
  std::vector<double> d, e;     // d[0..n-1], e[0..n-2] (T(i+1,i))
  std::vector<double> v;        // Householder vectors, column k stored in [k*n ...]
  std::vector<double> beta;     // reflector scalars
};

// A is full symmetric n x n, column-major; lower triangle is used and destroyed.
void householder_tridiag(int n, std::vector<double> &A, Tridiag &T) {
  T.n = n;
  T.d.assign(n, 0.0);
  T.e.assign(n > 1 ? n - 1 : 1, 0.0);
  T.v.assign((size_t)n * n, 0.0);
  T.beta.assign(n, 0.0);
  auto a = [&](int i, int j) -> double & { return A[(size_t)j * n + i]; };
  std::vector<double> p(n), w(n);
  for (int k = 0; k + 2 < n; ++k) {
    const int m = n - k - 1; // length of x = A(k+1:n-1, k)
    double *x = &a(k + 1, k);
    double sigma = 0.0;
    for (int i = 1; i < m; ++i) sigma += x[i] * x[i];
    double *vk = &T.v[(size_t)k * n];
    vk[0] = 1.0;
    for (int i = 1; i < m; ++i) vk[i] = x[i];
    double beta = 0.0, alpha = x[0];
    if (sigma == 0.0) {
      beta = 0.0;
      T.e[k] = alpha;
    } else {
      const double mu = std::sqrt(x[0] * x[0] + sigma);
      const double v0 = (x[0] <= 0.0) ? x[0] - mu : -sigma / (x[0] + mu);
      beta = 2.0 * v0 * v0 / (sigma + v0 * v0);
      for (int i = 1; i < m; ++i) vk[i] /= v0;
      T.e[k] = mu; // H x = mu e1
    }
    T.beta[k] = beta;
    T.d[k] = a(k, k);
    if (beta == 0.0) continue;
    // p = beta * A22 v  (A22 symmetric, lower triangle stored)
    const int o = k + 1;
    for (int i = 0; i < m; ++i) p[i] = 0.0;
    for (int j = 0; j < m; ++j) {
      const double vj = vk[j];
      const double *col = &a(o, o + j);
      p[j] += col[j] * vj;
      double acc = 0.0;
      for (int i = j + 1; i < m; ++i) {
        p[i] += col[i] * vj;
        acc += col[i] * vk[i];
      }
      p[j] += acc;
    }
    for (int i = 0; i < m; ++i) p[i] *= beta;
    double pv = 0.0;
    for (int i = 0; i < m; ++i) pv += p[i] * vk[i];
    const double half = 0.5 * beta * pv;
    for (int i = 0; i < m; ++i) w[i] = p[i] - half * vk[i];
    for (int j = 0; j < m; ++j) {
      double *col = &a(o, o + j);
      const double vj = vk[j], wj = w[j];
      for (int i = j; i < m; ++i) col[i] -= vk[i] * wj + w[i] * vj;
    }
  }
  if (n >= 2) {
    T.d[n - 2] = a(n - 2, n - 2);
    T.e[n - 2] = a(n - 1, n - 2);
  }
  T.d[n - 1] = a(n - 1, n - 1);
}

// number of eigenvalues of T strictly less than x (Sturm count, LDL^T pivots)
int sturm_count(const Tridiag &T, double x, double pivmin) {
  int cnt = 0;
  double q = T.d[0] - x;
  if (std::fabs(q) < pivmin) q = -pivmin;
  if (q < 0) ++cnt;
  for (int i = 1; i < T.n; ++i) {
    q = (T.d[i] - x) - T.e[i - 1] * T.e[i - 1] / q;
    if (std::fabs(q) < pivmin) q = -pivmin;
    if (q < 0) ++cnt;
  }
  return cnt;
}

// eigenvalues il..iu (1-based, ascending) by bisection
void bisect(const Tridiag &T, int il, int iu, double *w) {
  const int n = T.n;
  double lo = T.d[0], hi = T.d[0], tnorm = 0.0, emax2 = 0.0;
  for (int i = 0; i < n; ++i) {
    double r = 0.0;
    if (i > 0) r += std::fabs(T.e[i - 1]);
    if (i + 1 < n) r += std::fabs(T.e[i]);
    lo = std::min(lo, T.d[i] - r);
    hi = std::max(hi, T.d[i] + r);
    tnorm = std::max(tnorm, std::fabs(T.d[i]) + r);
    if (i + 1 < n) emax2 = std::max(emax2, T.e[i] * T.e[i]);
  }
  const double eps = 2.220446049250313e-16;
  const double safmin = 2.2250738585072014e-308;
  const double pivmin = std::max(safmin * std::max(1.0, emax2), safmin);
  lo -= 2.0 * eps * tnorm + 2.0 * pivmin;
  hi += 2.0 * eps * tnorm + 2.0 * pivmin;
  for (int j = il; j <= iu; ++j) {
    double a = lo, b = hi;
    for (int it = 0; it < 200; ++it) {
      const double mid = 0.5 * (a + b);
      if (b - a <= 2.0 * eps * std::max(std::fabs(a), std::fabs(b)) + 2.0 * pivmin) break;
      if (mid <= a || mid >= b) break;
      if (sturm_count(T, mid, pivmin) >= j)
        b = mid;
      else
        a = mid;
    }
    w[j - il] = 0.5 * (a + b);
  }
}

// inverse iteration for eigenvector of T at eigenvalue lam; x[n] out (unit norm)
void inverse_iteration(const Tridiag &T, double lam, double *x, const std::vector<std::vector<double>> &orth,
                       unsigned seed) {
  const int n = T.n;
  if (n == 1) {
    x[0] = 1.0;
    return;
  }
  double tnorm = 0.0;
  for (int i = 0; i < n; ++i)
    tnorm = std::max(tnorm, std::fabs(T.d[i]) + (i > 0 ? std::fabs(T.e[i - 1]) : 0.0) +
                                (i + 1 < n ? std::fabs(T.e[i]) : 0.0));
  const double eps = 2.220446049250313e-16;
  const double tiny = eps * std::max(tnorm, 1e-300);
  // LU with partial pivoting of (T - lam I): rows i have up to 3 upper entries
  std::vector<double> u0(n), u1(n), u2(n), l(n);
  std::vector<int> piv(n);
  {
    double a0 = T.d[0] - lam, a1 = T.e[0];
    for (int i = 0; i < n; ++i) {
      double b0 = 0, b1 = 0, sub = 0;
      if (i + 1 < n) {
        sub = T.e[i];
        b0 = T.d[i + 1] - lam;
        b1 = (i + 2 < n) ? T.e[i + 1] : 0.0;
      }
      // current row: [a0 a1 0] at columns i, i+1, i+2 ; next row: [sub b0 b1]
      if (i + 1 < n && std::fabs(sub) > std::fabs(a0)) {
        piv[i] = 1;
        const double m = a0 / sub;
        l[i] = m;
        u0[i] = sub;
        u1[i] = b0;
        u2[i] = b1;
        const double na0 = a1 - m * b0, na1 = -m * b1;
        a0 = na0;
        a1 = na1;
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
    if (u0[n - 1] == 0.0) u0[n - 1] = tiny;
  }
  // start vector: deterministic pseudo-random
  unsigned s = 12345u + seed * 7919u;
  for (int i = 0; i < n; ++i) {
    s = s * 1664525u + 1013904223u;
    x[i] = ((s >> 8) & 0xffff) / 65536.0 - 0.5 + 1e-3;
  }
  for (int it = 0; it < 5; ++it) {
    // forward: apply L^{-1} with row interchanges
    for (int i = 0; i + 1 < n; ++i) {
      if (piv[i]) std::swap(x[i], x[i + 1]);
      x[i + 1] -= l[i] * x[i];
    }
    // back substitution
    for (int i = n - 1; i >= 0; --i) {
      double v = x[i];
      if (i + 1 < n) v -= u1[i] * x[i + 1];
      if (i + 2 < n) v -= u2[i] * x[i + 2];
      double d = u0[i];
      if (std::fabs(d) < tiny) d = (d < 0 ? -tiny : tiny);
      x[i] = v / d;
    }
    // re-orthogonalise against cluster members
    for (const auto &q : orth) {
      double dot = 0.0;
      for (int i = 0; i < n; ++i) dot += q[i] * x[i];
      for (int i = 0; i < n; ++i) x[i] -= dot * q[i];
    }
    double nrm = 0.0;
    for (int i = 0; i < n; ++i) nrm += x[i] * x[i];
    nrm = std::sqrt(nrm);
    if (nrm == 0.0) nrm = 1.0;
    for (int i = 0; i < n; ++i) x[i] /= nrm;
  }
}

// back transformation z = Q x, Q = H_0 H_1 ... H_{n-3}
void back_transform(const Tridiag &T, double *z) {
  const int n = T.n;
  for (int k = n - 3; k >= 0; --k) {
    const double beta = T.beta[k];
    if (beta == 0.0) continue;
    const double *vk = &T.v[(size_t)k * n];
    const int m = n - k - 1;
    double *zz = z + k + 1;
    double dot = 0.0;
    for (int i = 0; i < m; ++i) dot += vk[i] * zz[i];
    dot *= beta;
    for (int i = 0; i < m; ++i) zz[i] -= dot * vk[i];
  }
}

int dspevx_lowest(int n, const double *ap, int il, int iu, double *w, double *z) {
  if (n <= 0 || il < 1 || iu > n || il > iu) return -1;
  std::vector<double> A((size_t)n * n, 0.0);
  for (int j = 1; j <= n; ++j)
    for (int i = 1; i <= j; ++i) {
      const double v = ap[(i - 1) + (size_t)j * (j - 1) / 2];
      A[(size_t)(j - 1) * n + (i - 1)] = v;
      A[(size_t)(i - 1) * n + (j - 1)] = v;
    }
  Tridiag T;
  householder_tridiag(n, A, T);
  const int m = iu - il + 1;
  bisect(T, il, iu, w);
  double tnorm = 0.0;
  for (int i = 0; i < n; ++i)
    tnorm = std::max(tnorm, std::fabs(T.d[i]) + (i > 0 ? std::fabs(T.e[i - 1]) : 0.0) +
                                (i + 1 < n ? std::fabs(T.e[i]) : 0.0));
  const double ortol = 1e-3 * tnorm;
  const double eps = 2.220446049250313e-16;
  std::vector<std::vector<double>> cluster;
  std::vector<double> x(n);
  double prev = 0.0;
  for (int j = 0; j < m; ++j) {
    double lam = w[j];
    if (j > 0 && lam - prev > ortol) cluster.clear();
    // separate numerically equal eigenvalues (as DSTEIN does)
    if (j > 0 && lam - prev < 10.0 * eps * std::fabs(lam)) lam = prev + 10.0 * eps * std::fabs(lam);
    inverse_iteration(T, lam, x.data(), cluster, (unsigned)j);
    cluster.emplace_back(x.begin(), x.end());
    prev = lam;
    double *zj = z + (size_t)j * n;
    for (int i = 0; i < n; ++i) zj[i] = x[i];
    back_transform(T, zj);
  }
  return 0;
}

// ---------------------------------------------------------------------------
// Reference-BLAS-order vector kernels used by DVDSON
// ---------------------------------------------------------------------------
double ddot(int64_t n, const double *x, const double *y) {
  double s = 0.0;
  for (int64_t i = 0; i < n; ++i) s += x[i] * y[i];
  return s;
}
// y = A x, A [n x k] column-major (DGEMV 'N', alpha 1, beta 0)
void dgemv_n(int64_t n, int k, const double *A, const double *x, double *y) {
  for (int64_t i = 0; i < n; ++i) y[i] = 0.0;
  for (int j = 0; j < k; ++j) {
    const double t = x[j];
    const double *a = A + (size_t)j * n;
    for (int64_t i = 0; i < n; ++i) y[i] += t * a[i];
  }
}
// y = A^T x, A [n x k] (DGEMV 'T')
void dgemv_t(int64_t n, int k, const double *A, int64_t lda, const double *x, double *y) {
  for (int j = 0; j < k; ++j) y[j] = ddot(n, A + (size_t)j * lda, x);
}

// SPICMV2 (lib9290/spicmv2.f90:42-57) + DMERGE (dmerge.f90:36-40)
void spicmv2(int n, int m, const int64_t *iendc, const int32_t *irow, const double *emt, const double *b,
             double *c, int nthreads) {
  if (nthreads <= 1) {
    for (int64_t i = 0; i < (int64_t)n * m; ++i) c[i] = 0.0;
    int64_t ibeg = 1;
    for (int icol = 1; icol <= n; ++icol) {
      const int64_t iend = iendc[icol];
      const int64_t nelc = iend - ibeg + 1;
      for (int iv = 0; iv < m; ++iv) {
        const double *B = b + (size_t)iv * n;
        double *C = c + (size_t)iv * n;
        const double diag = C[icol - 1] + emt[iend - 1] * B[icol - 1];
        double dsum = 0.0;
        const double dconst = B[icol - 1];
        for (int64_t i = 0; i < nelc - 1; ++i) {
          const int32_t r = irow[ibeg - 1 + i];
          dsum = dsum + emt[ibeg - 1 + i] * B[r - 1];
          C[r - 1] = C[r - 1] + dconst * emt[ibeg - 1 + i];
        }
        C[icol - 1] = diag + dsum;
      }
      ibeg = iend + 1;
    }
    return;
  }
  // Row-block decomposition with private accumulators reduced at the end:
  // the decomposition of rci_mpi's SPODMV/SPICMVmpi (rows per rank, then an
  // all-reduce of C).
  std::vector<std::vector<double>> part(nthreads, std::vector<double>((size_t)n * m, 0.0));
  std::vector<std::thread> th;
  for (int t = 0; t < nthreads; ++t)
    th.emplace_back([&, t] {
      double *cc = part[t].data();
      for (int icol = 1 + t; icol <= n; icol += nthreads) {
        const int64_t ibeg = iendc[icol - 1] + 1, iend = iendc[icol];
        for (int iv = 0; iv < m; ++iv) {
          const double *B = b + (size_t)iv * n;
          double *C = cc + (size_t)iv * n;
          double dsum = 0.0;
          const double dconst = B[icol - 1];
          for (int64_t i = ibeg; i < iend; ++i) {
            const int32_t r = irow[i - 1];
            dsum += emt[i - 1] * B[r - 1];
            C[r - 1] += dconst * emt[i - 1];
          }
          C[icol - 1] += emt[iend - 1] * B[icol - 1] + dsum;
        }
      }
    });
  for (auto &x : th) x.join();
  parallel_for((int64_t)n * m, nthreads, [&](int64_t i, int) {
    double s = 0.0;
    for (int t = 0; t < nthreads; ++t) s += part[t][i];
    c[i] = s;
  });
}

// MGS_NRM (libdvd90/dvdson.f90:1417-1508); b is 1-based-by-offset: vectors
// [0, kp) old, [kp, kp + nnew) new, each of length n.
void mgs_nrm(int64_t n, int kp, int nnew, double *scra, double *b) {
  for (int pass = 0; pass < 2; ++pass) {
    const size_t newstart = (size_t)kp * n;
    size_t kcur = 0;
    for (int k = 0; k < kp; ++k) {
      size_t jcur = newstart;
      dgemv_t(n, nnew, b + jcur, n, b + kcur, scra);
      for (int j = 0; j < nnew; ++j) {
        for (int64_t mm = 0; mm < n; ++mm) b[jcur + mm] = b[jcur + mm] - scra[j] * b[kcur + mm];
        jcur += n;
      }
      kcur += n;
    }
    for (int k = 1; k <= nnew; ++k) {
      size_t jcur = kcur + n;
      double dnm = ddot(n, b + kcur, b + kcur);
      dnm = std::sqrt(dnm);
      const double s = 1.0 / dnm;
      for (int64_t mm = 0; mm < n; ++mm) b[kcur + mm] *= s;
      dgemv_t(n, nnew - k, b + jcur, n, b + kcur, scra);
      for (int j = k + 1; j <= nnew; ++j) {
        for (int64_t mm = 0; mm < n; ++mm) b[jcur + mm] = b[jcur + mm] - scra[j - k - 1] * b[kcur + mm];
        jcur += n;
      }
      kcur += n;
    }
  }
}

// ADDS (dvdson.f90:484-514): new columns of S = B^T A B, packed upper
void adds(int64_t n, int kpass, int nncv, const double *basis, const double *ab, double *S) {
  size_t idstart = (size_t)kpass * n;
  int64_t isstart = (int64_t)kpass * (kpass + 1) / 2;
  for (int iv = 1; iv <= nncv; ++iv) {
    size_t ibstart = 0;
    for (int ibv = 1; ibv <= kpass + iv; ++ibv) {
      S[isstart + ibv - 1] = ddot(n, basis + ibstart, ab + idstart);
      ibstart += n;
    }
    isstart += kpass + iv;
    idstart += n;
  }
}

// MULTBC (dvdson.f90:953-1000): B(:,1:m) = B(:,1:k) C(k x m), row by row
void multbc(int64_t n, int k, int m, const double *C, double *temp, double *B) {
  for (int64_t irow = 0; irow < n; ++irow) {
    for (int j = 0; j < m; ++j) {
      double s = 0.0;
      for (int i = 0; i < k; ++i) s += C[(size_t)j * k + i] * B[irow + (size_t)i * n];
      temp[j] = s;
    }
    for (int j = 0; j < m; ++j) B[irow + (size_t)j * n] = temp[j];
  }
}

} // namespace

// ===========================================================================
// extern "C" API
// ===========================================================================
extern "C" {

or_ctx *or_create(int n, double rnt, double h, double c, const double *zz) {
  if (n < 20) return nullptr;
  or_ctx *g = new or_ctx;
  g->n = n;
  g->rnt = rnt;
  g->h = h;
  g->c = c;
  const size_t nn1 = g->nn1();
  g->R.assign(nn1, 0.0);
  g->RP.assign(nn1, 0.0);
  g->RPOR.assign(nn1, 0.0);
  g->ZZ.assign(nn1, 0.0);
  // RADGRD, HP == 0 branch (radgrd.f90:38-60)
  const int np10 = n + 10;
  g->R[1] = 0.0;
  g->RPOR[1] = 0.0;
  g->RP[1] = rnt;
  const double eph = std::exp(h);
  double ett = 1.0;
  for (int i = 2; i <= np10; ++i) {
    ett = eph * ett;
    const double ettm1 = ett - 1.0;
    g->R[i] = rnt * ettm1;
    g->RP[i] = rnt * ett;
    g->RPOR[i] = ett / ettm1;
  }
  if (zz)
    for (int i = 1; i <= n; ++i) g->ZZ[i] = zz[i - 1];
  // SETQIC (setqic.f90): A13 = B13 / 479001600 ; CNC5C ; C1..C4
  static const double B13[13][13] = {
      {-1486442880.0, 5748019200.0, -15807052800.0, 35126784000.0, -59276448000.0, 75873853440.0,
       -73766246400.0, 54195609600.0, -29638224000.0, 11708928000.0, -3161410560.0, 522547200.0, -39916800.0},
      {-39916800.0, -967524480.0, 2634508800.0, -4390848000.0, 6586272000.0, -7903526400.0, 7376624640.0,
       -5269017600.0, 2822688000.0, -1097712000.0, 292723200.0, -47900160.0, 3628800.0},
      {3628800.0, -87091200.0, -684478080.0, 1596672000.0, -1796256000.0, 1916006400.0, -1676505600.0,
       1149603840.0, -598752000.0, 228096000.0, -59875200.0, 9676800.0, -725760.0},
      {-725760.0, 13063680.0, -143700480.0, -476910720.0, 1077753600.0, -862202880.0, 670602240.0,
       -431101440.0, 215550720.0, -79833600.0, 20528640.0, -3265920.0, 241920.0},
      {241920.0, -3870720.0, 31933440.0, -212889600.0, -303937920.0, 766402560.0, -447068160.0, 255467520.0,
       -119750400.0, 42577920.0, -10644480.0, 1658880.0, -120960.0},
      {-120960.0, 1814400.0, -13305600.0, 66528000.0, -299376000.0, -148262400.0, 558835200.0, -239500800.0,
       99792000.0, -33264000.0, 7983360.0, -1209600.0, 86400.0},
      {86400.0, -1244160.0, 8553600.0, -38016000.0, 128304000.0, -410572800.0, 0.0, 410572800.0,
       -128304000.0, 38016000.0, -8553600.0, 1244160.0, -86400.0},
      {-86400.0, 1209600.0, -7983360.0, 33264000.0, -99792000.0, 239500800.0, -558835200.0, 148262400.0,
       299376000.0, -66528000.0, 13305600.0, -1814400.0, 120960.0},
      {120960.0, -1658880.0, 10644480.0, -42577920.0, 119750400.0, -255467520.0, 447068160.0, -766402560.0,
       303937920.0, 212889600.0, -31933440.0, 3870720.0, -241920.0},
      {-241920.0, 3265920.0, -20528640.0, 79833600.0, -215550720.0, 431101440.0, -670602240.0, 862202880.0,
       -1077753600.0, 476910720.0, 143700480.0, -13063680.0, 725760.0},
      {725760.0, -9676800.0, 59875200.0, -228096000.0, 598752000.0, -1149603840.0, 1676505600.0,
       -1916006400.0, 1796256000.0, -1596672000.0, 684478080.0, 87091200.0, -3628800.0},
      {-3628800.0, 47900160.0, -292723200.0, 1097712000.0, -2822688000.0, 5269017600.0, -7376624640.0,
       7903526400.0, -6586272000.0, 4390848000.0, -2634508800.0, 967524480.0, 39916800.0},
      {39916800.0, -522547200.0, 3161410560.0, -11708928000.0, 29638224000.0, -54195609600.0, 73766246400.0,
       -75873853440.0, 59276448000.0, -35126784000.0, 15807052800.0, -5748019200.0, 1486442880.0}};
  const double factor13 = 1.0 / 479001600.0;
  for (int j = 1; j <= 13; ++j)
    for (int i = 1; i <= 13; ++i) g->A13[i][j] = B13[i - 1][j - 1] * factor13;
  static const double C5NUM[6][6] = {// [i 1..5][j 2..5]
                                     {0, 0, 0, 0, 0, 0},
                                     {0, 0, 251.0, 232.0, 243.0, 224.0},
                                     {0, 0, 646.0, 992.0, 918.0, 1024.0},
                                     {0, 0, -264.0, 192.0, 648.0, 384.0},
                                     {0, 0, 106.0, 32.0, 378.0, 1024.0},
                                     {0, 0, -19.0, -8.0, -27.0, 224.0}};
  const double factor = h / 720.0;
  for (int j = 2; j <= 4; ++j)
    for (int i = 2; i <= 5; ++i) g->CNC5C[i][j] = factor * C5NUM[i][j];
  g->C1 = factor * C5NUM[1][5];
  g->C2 = factor * C5NUM[2][5];
  g->C3 = factor * C5NUM[3][5];
  g->C4 = g->C1 + g->C1;
  // ACCY = H**6 (getcid.f90:262); gfortran evaluates a constant integer
  // power by the multiplication chain x^6 = (x^2 * x)^2.
  {
    const double h2 = h * h, h3 = h2 * h;
    g->accy = h3 * h3;
  }
  // YZK power tables for k = 1..KLIMIT (yzk.f90:70-95)
  g->RTTK.assign(nn1 * (KLIMIT + 1), 0.0);
  g->RTTKM.assign(nn1 * (KLIMIT + 1), 0.0);
  g->RTTK1.assign(nn1 * (KLIMIT + 1), 0.0);
  g->RTTKM1.assign(nn1 * (KLIMIT + 1), 0.0);
  g->RM.assign(nn1, 0.0);
  for (int i = 2; i <= n; ++i) g->RM[i] = 1.0 / g->R[i];
  for (int k = 1; k <= KLIMIT; ++k)
    for (int i = 2; i <= n; ++i) {
      const double t = powi(g->R[i], k);
      g->RTTK[k * nn1 + i] = t;
      g->RTTKM[k * nn1 + i] = 1.0 / t;
      g->RTTK1[k * nn1 + i] = t * g->R[i];
      g->RTTKM1[k * nn1 + i] = 1.0 / (t * g->R[i]);
    }
  return g;
}

void or_destroy(or_ctx *g) { delete g; }

void or_get_grid(const or_ctx *g, double *r, double *rp, double *rpor) {
  for (int i = 1; i <= g->n + 10; ++i) {
    r[i - 1] = g->R[i];
    rp[i - 1] = g->RP[i];
    rpor[i - 1] = g->RPOR[i];
  }
}

void or_get_qic(const or_ctx *g, double *c1234, double *cnc5c) {
  c1234[0] = g->C1;
  c1234[1] = g->C2;
  c1234[2] = g->C3;
  c1234[3] = g->C4;
  for (int j = 2; j <= 4; ++j)
    for (int i = 2; i <= 5; ++i) cnc5c[(j - 2) * 4 + (i - 2)] = g->CNC5C[i][j];
}

int or_set_orbitals(or_ctx *g, int nw, int ld, const int *nak, const int *mf, const double *pf,
                    const double *qf) {
  if (nw <= 0 || ld < g->n) return -1;
  g->nw = nw;
  g->ld = ld;
  g->NAK.assign(nw + 1, 0);
  g->MF.assign(nw + 1, 0);
  g->NKL.assign(nw + 1, 0);
  g->NKJ.assign(nw + 1, 0);
  for (int j = 1; j <= nw; ++j) {
    g->NAK[j] = nak[j - 1];
    g->MF[j] = mf[j - 1];
    if (g->MF[j] + 3 > g->n + 10 || g->MF[j] < 2) return -2;
    const int kap = nak[j - 1];
    g->NKL[j] = kap > 0 ? kap : -kap - 1;
    g->NKJ[j] = 2 * std::abs(kap) - 1;
  }
  g->PF.assign(pf, pf + (size_t)ld * nw);
  g->QF.assign(qf, qf + (size_t)ld * nw);
  return 0;
}

double or_quad(const or_ctx *g, int mtp, double *ta) { return quad(g, mtp, ta - 1); }

int or_yzk(or_ctx *g, int k, int i, int j, double *yk_out) {
  std::vector<double> TA(g->nn1(), 0.0), TB(g->nn1(), 0.0);
  const int mtp = yzk(g, k, i, j, TA.data(), TB.data());
  for (int ii = 1; ii <= g->n; ++ii) yk_out[ii - 1] = TB[ii];
  return mtp;
}

double or_slater(or_ctx *g, int ia, int ib, int ic, int id, int k) {
  std::vector<double> TA(g->nn1(), 0.0), TB(g->nn1(), 0.0);
  return slater(g, ia, ib, ic, id, k, TA.data(), TB.data());
}

// YPOT (rmcdhf90/ypot.f90:35-49): YP(:N) = ZZ(:N), then for each index of
// the list YP(:N) = YP(:N) - COEFF*TB(:N) with TB from YZK(K, IOY1, IOY2);
// NYA = (IOY2*KEY + IOY1)*KEY + K, KEY = 215. yp[0..N-1] = YP(1..N).
int or_ypot(or_ctx *g, int ncof, const int32_t *nya, const double *ya, double *yp) {
  const int N = g->n, KEY = 215;
  std::vector<double> YP(g->nn1(), 0.0), TA(g->nn1(), 0.0), TB(g->nn1(), 0.0);
  for (int i = 1; i <= N; ++i) YP[i] = g->ZZ[i];
  for (int idx = 0; idx < ncof; ++idx) {
    int label = nya[idx];
    const int K = label % KEY;
    label /= KEY;
    const int IOY1 = label % KEY, IOY2 = label / KEY;
    if (IOY1 < 1 || IOY1 > g->nw || IOY2 < 1 || IOY2 > g->nw || K > KLIMIT) return -1;
    const double COEFF = ya[idx];
    yzk(g, K, IOY1, IOY2, TA.data(), TB.data());
    for (int i = 1; i <= N; ++i) YP[i] = YP[i] - COEFF * TB[i];
  }
  for (int i = 1; i <= N; ++i) yp[i - 1] = YP[i];
  return 0;
}

// XPOT (rmcdhf90/xpot.f90:31-54): XP = XQ = 0; for each index, TB from
// YZK(K, IOY1, IOY2), COEFF = XA/C, CTB = COEFF*TB(I), XP(I) += CTB*QF(I,IORB),
// XQ(I) -= CTB*PF(I,IORB); NXA = ((IORB*KEY + IOY2)*KEY + IOY1)*KEY + K.
int or_xpot(or_ctx *g, int ncof, const int32_t *nxa, const double *xa, double *xp, double *xq) {
  const int N = g->n, KEY = 215;
  std::vector<double> XP(g->nn1(), 0.0), XQ(g->nn1(), 0.0), TA(g->nn1(), 0.0), TB(g->nn1(), 0.0);
  for (int idx = 0; idx < ncof; ++idx) {
    int label = nxa[idx];
    const int K = label % KEY;
    label /= KEY;
    const int IOY1 = label % KEY;
    label /= KEY;
    const int IOY2 = label % KEY, IORB = label / KEY;
    if (IOY1 < 1 || IOY1 > g->nw || IOY2 < 1 || IOY2 > g->nw || IORB < 1 || IORB > g->nw || K > KLIMIT) return -1;
    yzk(g, K, IOY1, IOY2, TA.data(), TB.data());
    const double COEFF = xa[idx] / g->c;
    for (int i = 1; i <= N; ++i) {
      const double CTB = COEFF * TB[i];
      XP[i] = XP[i] + CTB * g->qf(i, IORB);
      XQ[i] = XQ[i] - CTB * g->pf(i, IORB);
    }
  }
  for (int i = 1; i <= N; ++i) {
    xp[i - 1] = XP[i];
    xq[i - 1] = XQ[i];
  }
  return 0;
}

// LAGCON (rmcdhf90/lagcon.f90:32-56, NPROCS = 1): XP, XQ 1-based.
static void lagcon(const or_ctx *g, int J, double ucfj, int nec, const int32_t *iecc, const double *ecv, double accy,
                   double *XP, double *XQ) {
  const int KEY = 215;
  if (nec == 0) return;
  const double EPS = accy * 0.01;
  const double WB = 1.0 / (ucfj * g->c) / 1.0;
  for (int k = 0; k < nec; ++k) {
    const int L1 = iecc[k] / KEY, L2 = iecc[k] - KEY * L1;
    int M;
    if (J == L1)
      M = L2;
    else if (J == L2)
      M = L1;
    else
      continue;
    const double WA = ecv[k] * WB;
    if (std::fabs(WA) < EPS) continue;
    for (int i = 1; i <= g->MF[M]; ++i) {
      const double WARI = WA * g->R[i];
      XP[i] = XP[i] + WARI * g->qf(i, M);
      XQ[i] = XQ[i] - WARI * g->pf(i, M);
    }
  }
}

// DACON (rmcdhf90/dacon.f90:25-46): XP, XQ 1-based.
static void dacon(const or_ctx *g, int nd, const int32_t *nda, const double *da, double *XP, double *XQ) {
  const double TWOC = g->c + g->c;
  std::vector<double> TA(g->nn1(), 0.0), TB(g->nn1(), 0.0);
  for (int k = 0; k < nd; ++k) {
    const int IORB = nda[k];
    dpbdt(g, IORB, TA.data(), TB.data());
    const int MFI = g->MF[IORB];
    const double COEFF = da[k], FK = (double)g->NAK[IORB];
    for (int i = 2; i <= MFI; ++i) {
      const double RPORII = 1.0 / (g->h * g->RPOR[i]);
      const double PFI = g->pf(i, IORB), QFI = g->qf(i, IORB);
      const double ZBCI = g->ZZ[i] / g->c;
      XP[i] = XP[i] + COEFF * (TA[i] * RPORII + FK * PFI - (TWOC * g->R[i] + ZBCI) * QFI);
      XQ[i] = XQ[i] + COEFF * (TB[i] * RPORII - FK * QFI + ZBCI * PFI);
    }
  }
}

// one orbital's lists as SETCOF leaves them in scf_C
struct or_cof {
  int ny;
  const int32_t *nya;
  const double *ya;
  int nx;
  const int32_t *nxa;
  const double *xa;
  int nd;
  const int32_t *nda;
  const double *da;
};

// YPOT, XPOT, [LAGCON], DACON for orbital J: YP, XP, XQ 1-based (nn1 each)
static int potentials(or_ctx *g, const or_cof *c, bool lag, int J, double ucfj, int nec, const int32_t *iecc,
                      const double *ecv, double accy, std::vector<double> &YP, std::vector<double> &XP,
                      std::vector<double> &XQ) {
  const int N = g->n;
  std::vector<double> yp(N), xp(N), xq(N);
  if (or_ypot(g, c->ny, c->nya, c->ya, yp.data()) || or_xpot(g, c->nx, c->nxa, c->xa, xp.data(), xq.data()))
    return -1;
  YP.assign(g->nn1(), 0.0);
  XP.assign(g->nn1(), 0.0);
  XQ.assign(g->nn1(), 0.0);
  for (int i = 1; i <= N; ++i) {
    YP[i] = yp[i - 1];
    XP[i] = xp[i - 1];
    XQ[i] = xq[i - 1];
  }
  if (lag) lagcon(g, J, ucfj, nec, iecc, ecv, accy, XP.data(), XQ.data());
  dacon(g, c->nd, c->nda, c->da, XP.data(), XQ.data());
  return 0;
}

// COFPOT (rmcdhf90/cofpot.f90:29-33) after SETCOF: YPOT, XPOT, LAGCON, DACON.
int or_cofpot(or_ctx *g, int j, double ucfj, const or_cof *cof, int nec, const int32_t *iecc, const double *ecv,
              double accy, double *yp, double *xp, double *xq) {
  std::vector<double> YP, XP, XQ;
  if (potentials(g, cof, true, j, ucfj, nec, iecc, ecv, accy, YP, XP, XQ)) return -1;
  for (int i = 1; i <= g->n; ++i) {
    yp[i - 1] = YP[i];
    xp[i - 1] = XP[i];
    xq[i - 1] = XQ[i];
  }
  return 0;
}

// SETLAG (rmcdhf90/setlag.f90:140-223): ECV of each pair, in pair order, the
// potentials of J and M recomputed when they change (JLAST, MLAST).
int or_setlag(or_ctx *g, int nec, const int32_t *iecc, const double *ucf, const int *lfix, const or_cof *cof,
              double *ecv) {
  const int KEY = 215;
  const double P001 = 1.0e-01;
  const double C = g->c;
  std::vector<double> YPJ, XPJ, XQJ, YPM, XPM, XQM;
  std::vector<double> TA(g->nn1(), 0.0), T1(g->nn1(), 0.0), T2(g->nn1(), 0.0);
  int JLAST = 0, MLAST = 0;
  for (int li = 0; li < nec; ++li) {
    const int M = iecc[li] / KEY, J = iecc[li] - KEY * M;
    if (J != JLAST) {
      if (potentials(g, &cof[J - 1], false, J, 0.0, 0, nullptr, nullptr, 0.0, YPJ, XPJ, XQJ)) return -1;
      JLAST = J;
    }
    if (M != MLAST) {
      if (potentials(g, &cof[M - 1], false, M, 0.0, 0, nullptr, nullptr, 0.0, YPM, XPM, XQM)) return -1;
      MLAST = M;
    }
    const double UCFJ = ucf[J - 1], UCFM = ucf[M - 1];
    const int MTP = std::max(g->MF[J], g->MF[M]);
    int err = 0;
    auto pm = [&](int i) { return g->pf(i, M); };
    auto qm = [&](int i) { return g->qf(i, M); };
    auto pj = [&](int i) { return g->pf(i, J); };
    auto qj = [&](int i) { return g->qf(i, J); };
    std::fill(TA.begin(), TA.end(), 0.0);
    if (lfix[M - 1]) {
      for (int i = 2; i <= MTP; ++i)
        TA[i] = g->RPOR[i] * ((pm(i) * XQJ[i] - qm(i) * XPJ[i]) * C + (pm(i) * pj(i) + qm(i) * qj(i)) * YPJ[i]);
      const double RESULT = quad(g, MTP, TA.data());
      const double RIJM = rinti(g, M, J, 1, T1.data(), T2.data(), &err);
      ecv[li] = (RESULT - RIJM) * UCFJ;
    } else if (lfix[J - 1]) {
      for (int i = 2; i <= MTP; ++i)
        TA[i] = g->RPOR[i] * ((pj(i) * XQM[i] - qj(i) * XPM[i]) * C + (pj(i) * pm(i) + qj(i) * qm(i)) * YPM[i]);
      const double RESULT = quad(g, MTP, TA.data());
      const double RIJM = rinti(g, J, M, 1, T1.data(), T2.data(), &err);
      ecv[li] = (RESULT - RIJM) * UCFM;
    } else {
      const double QDIF = std::fabs((UCFJ - UCFM) / std::max(UCFJ, UCFM));
      if (QDIF > P001) {
        const double OBQDIF = 1.0 / UCFJ - 1.0 / UCFM;
        for (int i = 2; i <= MTP; ++i)
          TA[i] = g->RPOR[i] * ((pm(i) * XQJ[i] - qm(i) * XPJ[i] - pj(i) * XQM[i] + qj(i) * XPM[i]) * C +
                                (YPJ[i] - YPM[i]) * (pm(i) * pj(i) + qm(i) * qj(i)));
        const double RESULT = quad(g, MTP, TA.data());
        ecv[li] = RESULT / OBQDIF;
      } else {
        const double OBQSUM = 1.0 / UCFJ + 1.0 / UCFM;
        for (int i = 2; i <= MTP; ++i)
          TA[i] = g->RPOR[i] * ((pm(i) * XQJ[i] - qm(i) * XPJ[i] + pj(i) * XQM[i] - qj(i) * XPM[i]) * C +
                                (YPJ[i] + YPM[i]) * (pm(i) * pj(i) + qm(i) * qj(i)));
        const double RESULT = quad(g, MTP, TA.data());
        const double RIJM = rinti(g, M, J, 1, T1.data(), T2.data(), &err);
        ecv[li] = (RESULT - 2.0 * RIJM) / OBQSUM;
      }
    }
    if (err) return -2;
  }
  return 0;
}

// ---------------------------------------------------------------------------
// Breit integrals: BESSEL, ZKF, RKINT, SKINT, BRRA, BRINTF, TRIANGBREIT1/2,
// GENINTBREIT1/2 (rci90). BRINTF is restated as a function of its arguments:
// the reference keeps the Bessel functions of the last pairs in four slots
// (bess_C KEEP) and skips BESSEL calls whose slot already holds the
// function; here each needed slot is evaluated. The results agree wherever
// the reference's slot holds the function it reads (slot 1: pair (IA,IB),
// slot 2: pair (IC,ID)); where it skips a call for two equal orbitals
// (zero frequency, brintf.f90:47-48) it reads the slot's earlier content.
// ---------------------------------------------------------------------------
struct or_bess {
  std::vector<double> J, N;  // 1-based
  double w = 0.0;
};

// BESSEL (rci90/bessel.f90:85-205): (j_nn(wr) series and asymptotic forms)
static void bessel(const or_ctx *g, double wfact, const double *E, double accy, int ia, int ib, int nn, or_bess &b) {
  const int N = g->n;
  b.J.assign(g->nn1(), 0.0);
  b.N.assign(g->nn1(), 0.0);
  const double EPSI = std::sqrt(0.1 * accy);
  const double W = wfact * std::fabs(E[ia - 1] - E[ib - 1]) / g->c;
  b.w = W;
  if (W < EPSI * EPSI) return;
  int JCHAN = N + 1;
  for (int j = 2; j <= N; ++j) {
    const double WA = -0.5 * ((g->R[j] * W) * (g->R[j] * W));
    double X1 = 1.0, X2 = 1.0, S1 = 0.0, S2 = 0.0;
    bool done = false;
    for (int i = 1; i <= 4; ++i) {
      X1 = X1 * WA / (double)(i * (2 * (nn + i) + 1));
      X2 = X2 * WA / (double)(i * (2 * (i - nn) - 1));
      S1 = S1 + X1;
      S2 = S2 + X2;
      if (std::fabs(X1) >= std::fabs(S1) * EPSI || std::fabs(X2) >= std::fabs(S2) * EPSI) continue;
      b.J[j] = S1;
      b.N[j] = S2;
      done = true;
      break;
    }
    if (!done) {
      JCHAN = j;
      break;
    }
  }
  if (JCHAN > N) return;
  double DFNM, DFN;
  if (nn == 0) {
    DFNM = 1.0;
    DFN = 1.0;
  } else {
    DFNM = 1.0;
    for (int i = 3; i <= 2 * nn - 1; i += 2) DFNM = DFNM * (double)i;
    DFN = DFNM * (double)(2 * nn + 1);
  }
  DFNM = 1.0 / DFNM;
  const int IREM = nn % 4;  // MOD: the sign of nn
  double SSN, SCN;
  int ISWAP;
  switch (IREM) {
    case 1: SSN = -1.0; SCN = 1.0; ISWAP = 1; break;
    case 2: SSN = -1.0; SCN = -1.0; ISWAP = 0; break;
    case 3: SSN = 1.0; SCN = -1.0; ISWAP = 1; break;
    default: SSN = 1.0; SCN = 1.0; ISWAP = 0; break;
  }
  for (int j = JCHAN; j <= N; ++j) {
    const double WA = W * g->R[j];
    double SN, CN;
    if (ISWAP == 0) {
      SN = SSN * std::sin(WA);
      CN = SCN * std::cos(WA);
    } else {
      SN = SSN * std::cos(WA);
      CN = SCN * std::sin(WA);
    }
    const double OBWA = 1.0 / WA;
    double B = OBWA;
    double S1 = B * SN, S2 = B * CN;
    for (int i = 1; i <= nn; ++i) {
      const double SKEEP = SN;
      SN = CN;
      CN = -SKEEP;
      B = B * OBWA * (double)((nn + i) * (nn - i + 1)) / (double)(2 * i);
      S1 = S1 + B * SN;
      S2 = S2 + B * CN;
    }
    S1 = S1 * DFN / powi(WA, nn) - 1.0;
    S2 = S2 * powi(WA, nn + 1) * DFNM - 1.0;
    b.J[j] = S1;
    b.N[j] = S2;
  }
}

// ZKF (rci90/zkf.f90:32-75): ZK from TA(2:MTP), 1-based; R**K for K < 0 is
// 1/R**|K| (the reference fills its power array only for K > 0).
static void zkf(const or_ctx *g, int K, int MTP, const double *TA, double *ZK) {
  const int N = g->n;
  std::vector<double> RTTK(g->nn1(), 0.0), RHOP(g->nn1(), 0.0), TEMP(g->nn1(), 0.0);
  if (K != 0)
    for (int i = 2; i <= N; ++i) RTTK[i] = powi(g->R[i], K);
  const int MTPP1 = MTP + 1, MTPP3 = MTP + 3, MTPP4 = MTP + 4;
  for (int i = 2; i <= MTP; ++i) RHOP[i] = g->RP[i] * TA[i];
  TEMP[1] = 0.0;
  for (int i = 2; i <= MTP; ++i) TEMP[i] = (K == 0) ? RHOP[i] : RTTK[i] * RHOP[i];
  for (int i = MTPP1; i <= MTPP4; ++i) TEMP[i] = 0.0;
  ZK[1] = 0.0;
  for (int ii = 2; ii <= 4; ++ii) {
    double SUM = 0.0;
    for (int kk = 2; kk <= 5; ++kk) SUM = SUM + g->CNC5C[kk][ii] * TEMP[kk];
    ZK[ii] = SUM;
  }
  for (int ii = 5; ii <= MTPP3; ++ii)
    ZK[ii] = ZK[ii - 4] + g->C1 * (TEMP[ii - 4] + TEMP[ii]) + g->C2 * (TEMP[ii - 3] + TEMP[ii - 1]) +
             g->C3 * TEMP[ii - 2];
  const double ZKLIM = ZK[MTPP3];
  if (K == 0) {
    for (int i = MTPP4; i <= N; ++i) ZK[i] = ZKLIM;
  } else {
    for (int i = 2; i <= MTPP3; ++i) ZK[i] = ZK[i] / RTTK[i];
    for (int i = MTPP4; i <= N; ++i) ZK[i] = ZKLIM / RTTK[i];
  }
}

// RKINT (rci90/rkint.f90:40-60): bj, bn = slot IW's BESSJ(1,IW), BESSN(1,IW)
// (null for IW = 0)
static double rkint(const or_ctx *g, const double *RAC, int IA, int IC, const double *RBD, int IB, int ID, int K,
                    const double *bj, const double *bn) {
  const int MXRBD = std::min(g->MF[IB], g->MF[ID]), MXRAC = std::min(g->MF[IA], g->MF[IC]);
  std::vector<double> TA(g->nn1(), 0.0), TB(g->nn1(), 0.0);
  for (int i = 1; i <= MXRAC; ++i) TA[i] = bj ? RAC[i] * (1.0 + bj[i]) : RAC[i];
  int MTP = MXRAC;
  zkf(g, K, MTP, TA.data(), TB.data());
  MTP = std::min(MTP, MXRBD);
  TA[1] = 0.0;
  for (int i = 2; i <= MTP; ++i) TA[i] = bn ? RBD[i] * (1.0 + bn[i]) * TB[i] * g->RPOR[i] : RBD[i] * TB[i] * g->RPOR[i];
  return quad(g, MTP, TA.data());
}

// SKINT (rci90/skint.f90:43-85): slot IW's BESSJ(1..2,IW), BESSN(1..2,IW)
// and WIJ(IW)
static double skint(const or_ctx *g, const double *RAC, int IA, int IC, const double *RBD, int IB, int ID, int K,
                    const or_bess &b1, const or_bess &b2) {
  const double EPSI = 1.0e-10;
  const double W = b1.w;
  const double WK = (double)(K + K + 1);
  const int MXRAC = std::min(g->MF[IA], g->MF[IC]), MXRBD = std::min(g->MF[IB], g->MF[ID]);
  std::vector<double> TA(g->nn1(), 0.0), TB(g->nn1(), 0.0), TKEEP(g->nn1(), 0.0);
  for (int i = 1; i <= MXRAC; ++i) TA[i] = RAC[i];
  int MTP = MXRAC;
  zkf(g, K - 1, MTP, TA.data(), TB.data());
  double SK;
  if (std::fabs(W) < EPSI) {
    for (int i = 1; i <= MTP; ++i) TKEEP[i] = TB[i];
    zkf(g, K + 1, MTP, TA.data(), TB.data());
    MTP = std::min(MTP, MXRBD);
    TA[1] = 0.0;
    for (int i = 2; i <= MTP; ++i) TA[i] = RBD[i] * g->RPOR[i] * (TB[i] - TKEEP[i]);
    const double VALU = quad(g, MTP, TA.data());
    SK = WK * VALU * 0.5;
  } else {
    for (int i = 1; i <= MTP; ++i) TKEEP[i] = TB[i];
    for (int i = 1; i <= MTP; ++i) TA[i] = -TA[i] * b1.J[i];
    zkf(g, K - 1, MTP, TA.data(), TB.data());
    MTP = std::min(MTP, MXRBD);
    TA[1] = 0.0;
    for (int i = 2; i <= MTP; ++i)
      TA[i] = ((1.0 + b2.N[i]) * TB[i] - TKEEP[i] * b2.N[i]) * RBD[i] / powi(g->R[i], 2) * g->RPOR[i];
    double VALU = quad(g, MTP, TA.data());
    SK = powi(WK / W, 2) * VALU;
    for (int i = 1; i <= MXRBD; ++i) TA[i] = RBD[i] * (1.0 + b2.J[i]);
    MTP = MXRBD;
    zkf(g, K + 1, MTP, TA.data(), TB.data());
    MTP = std::min(MTP, MXRAC);
    TA[1] = 0.0;
    for (int i = 2; i <= MTP; ++i) TA[i] = RAC[i] * (1.0 + b1.N[i]) * TB[i] * g->R[i] * g->RP[i];
    VALU = quad(g, MTP, TA.data());
    SK = SK - VALU * W * W / (double)((2 * K + 3) * (2 * K - 1));
  }
  return SK;
}

// BRRA (rci90/brra.f90:36-118) with BRINTF's argument order (IA, IB, IC, ID)
// = BRRA's (IA, IC, IB, ID); s[iw][ik]: the Bessel slots
static double brra(const or_ctx *g, int ITYPE, int IA, int IC, int IB, int ID, int K, or_bess s[3][3]) {
  const double HALF = 0.5, TWO = 2.0;
  const int MXRAC = std::min(g->MF[IA], g->MF[IC]), MXRBD = std::min(g->MF[IB], g->MF[ID]);
  std::vector<double> RAC(g->nn1(), 0.0), RBD(g->nn1(), 0.0);
  for (int i = 1; i <= MXRAC; ++i) RAC[i] = g->pf(i, IA) * g->qf(i, IC);
  for (int i = 1; i <= MXRBD; ++i) RBD[i] = g->pf(i, IB) * g->qf(i, ID);
  auto R = [&](bool rac, int iw) {
    const double *bj = iw ? s[iw][1].J.data() : nullptr, *bn = iw ? s[iw][1].N.data() : nullptr;
    return rac ? rkint(g, RAC.data(), IA, IC, RBD.data(), IB, ID, K, bj, bn)
               : rkint(g, RBD.data(), IB, ID, RAC.data(), IA, IC, K, bj, bn);
  };
  auto S = [&](int iw) { return skint(g, RAC.data(), IA, IC, RBD.data(), IB, ID, K, s[iw][1], s[iw][2]); };
  switch (ITYPE) {
    case 1:
      if (IA == IB && IC == ID) return TWO * R(true, 1);
      if (IA == ID && IC == IB) return R(true, 1) + R(false, 1);
      return (R(true, 1) + R(true, 2) + R(false, 1) + R(false, 2)) * HALF;
    case 2:
      if ((IA == IB && IC == ID) || (IA == ID && IC == IB)) return S(1);
      return (S(1) + S(2)) * HALF;
    case 3:
      if (IA == IC) {
        for (int i = 1; i <= MXRBD; ++i) RBD[i] = RBD[i] + g->pf(i, ID) * g->qf(i, IB);
        return (R(true, 0) + R(false, 0) + R(true, 2) + R(false, 2)) * HALF;
      }
      for (int i = 1; i <= MXRAC; ++i) RAC[i] = RAC[i] + g->pf(i, IC) * g->qf(i, IA);
      return (R(true, 1) + R(false, 1) + R(true, 0) + R(false, 0)) * HALF;
    case 4:
      return R(true, 0) + R(false, 0);
    case 5:
      if (IA == ID && IC == IB) return R(true, 1) + R(false, 1);
      return TWO * R(true, 1);
    default:
      return S(1);
  }
}

// BRINTF (rci90/brintf.f90:34-69): slot 1 = pair (IA, IB), slot 2 = pair
// (IC, ID); order K (types 1, 3, 5) or K - 1 and K + 1 (types 2, 6)
double brintf(const or_ctx *g, int ITYPE, int IA, int IB, int IC, int ID, int K, double wfact, const double *E,
              double accy) {
  or_bess s[3][3];
  if (ITYPE == 1 || ITYPE == 3 || ITYPE == 5) {
    bessel(g, wfact, E, accy, IA, IB, K, s[1][1]);
    if (ITYPE != 5) bessel(g, wfact, E, accy, IC, ID, K, s[2][1]);
  } else if (ITYPE == 2 || ITYPE == 6) {
    bessel(g, wfact, E, accy, IA, IB, K - 1, s[1][1]);
    bessel(g, wfact, E, accy, IA, IB, K + 1, s[1][2]);
    if (ITYPE == 2) {
      bessel(g, wfact, E, accy, IC, ID, K - 1, s[2][1]);
      bessel(g, wfact, E, accy, IC, ID, K + 1, s[2][2]);
    }
  }
  return brra(g, ITYPE, IA, IB, IC, ID, K, s);
}

// TRIANGBREIT1 (rci90/triangbreit1.f90:27-46), TRIANGBREIT2 (triangbreit2.f90:27-42)
static bool triangbreit(const or_ctx *g, int type, int IA, int IB, int IC, int ID, int K) {
  const int LA = g->NKL[IA], LB = g->NKL[IB], LC = g->NKL[IC], LD = g->NKL[ID];
  const int JA = g->NKJ[IA], JB = g->NKJ[IB], JC = g->NKJ[IC], JD = g->NKJ[ID];
  auto side = [&](int par, int l, int x, int la, int lb, int ja, int jb) {
    return ((l + x + la + lb) % 2 == par) && std::abs(ja - jb) <= 2 * x && std::abs(ja + jb) >= 2 * x;
  };
  if (type == 1) {
    for (int L = K - 1; L <= K + 1; ++L)
      if (side(1, K - L, L, LA, LB, JA, JB) && side(1, K - L, L, LC, LD, JC, JD)) return true;
    return false;
  }
  return side(0, 0, K, LA, LB, JA, JB) && side(0, 0, K, LC, LD, JC, JD);
}

double or_brintf(or_ctx *g, int type, int ia, int ib, int ic, int id, int k, double wfact, const double *E,
                 double accy) {
  return brintf(g, type, ia, ib, ic, id, k, wfact, E, accy);
}

// GENINTBREIT1 / GENINTBREIT2 (rci90/genintbreit1.f90:50-100,
// genintbreit2.f90:50-100): NB, INDTP ((IA*KEY+IB)*KEY+IC)*KEY+ID with KEY =
// NW + 1, VALTP = BRINTF(type, ...), KSTARTBREIT(0:J2MAX+1). With ind null
// only NB and kstart are returned. nthreads host threads share the values.
int64_t or_genintbreit(or_ctx *g, int type, double wfact, const double *E, double accy, int32_t *ind, double *val,
                       int32_t *kstart, int *j2max_out, int nthreads) {
  const int NW = g->nw, KEY = NW + 1;
  int J2MAX = g->NKJ[1];
  for (int i = 2; i <= NW; ++i) J2MAX = std::max(J2MAX, g->NKJ[i]);
  if (j2max_out) *j2max_out = J2MAX;
  std::vector<std::array<int, 5>> items;
  int64_t NB = 0;
  if (kstart) kstart[0] = 1;
  for (int K = 0; K <= J2MAX; ++K) {
    for (int IA = 1; IA <= NW; ++IA)
      for (int IB = 1; IB <= NW; ++IB)
        for (int IC = 1; IC <= NW; ++IC)
          for (int ID = 1; ID <= NW; ++ID)
            if (triangbreit(g, type, IA, IB, IC, ID, K)) {
              ++NB;
              if (ind) items.push_back({K, IA, IB, IC, ID});
            }
    if (kstart) kstart[K + 1] = (int32_t)(NB + 1);
  }
  if (ind) {
    parallel_for((int64_t)items.size(), nthreads, [&](int64_t i, int) {
      const auto &t = items[i];
      ind[i] = ((t[1] * KEY + t[2]) * KEY + t[3]) * KEY + t[4];
      val[i] = brintf(g, type, t[1], t[2], t[3], t[4], t[0], wfact, E, accy);
    });
  }
  return NB;
}

double or_rinti(or_ctx *g, int j, int k, int mode, int *err) {
  std::vector<double> TA(g->nn1(), 0.0), TB(g->nn1(), 0.0);
  return rinti(g, j, k, mode, TA.data(), TB.data(), err);
}

int or_triangrk(int la, int k, int lb) {
  if ((k + la + lb) % 2 != 0) return 0;
  if (std::abs(la - lb) > k) return 0;
  if (la + lb < k) return 0;
  return 1;
}

int64_t or_genintrk(or_ctx *g, int kmax, int32_t *indteirk, double *valteirk, int32_t *kstart, int *j2max_out,
                    int nthreads) {
  const int NW = g->nw;
  const int KEY = NW + 1;
  int j2max = g->NKJ[1];
  for (int i = 2; i <= NW; ++i) j2max = std::max(j2max, g->NKJ[i]);
  if (j2max_out) *j2max_out = j2max;
  const int kloop = kmax < 0 ? j2max : kmax;
  if (kloop > KLIMIT) return -1;
  struct Q {
    int a, b, c, d, k;
  };
  std::vector<Q> qs;
  int64_t N = 0;
  if (kstart) kstart[0] = 1;
  for (int K = 0; K <= kloop; ++K) {
    for (int IA = 1; IA <= NW; ++IA)
      for (int IB = IA; IB <= NW; ++IB)
        for (int IC = IA; IC <= NW; ++IC)
          if (or_triangrk(g->NKL[IA], K, g->NKL[IC]))
            for (int ID = IB; ID <= NW; ++ID)
              if (or_triangrk(g->NKL[IB], K, g->NKL[ID])) {
                ++N;
                if (indteirk) {
                  indteirk[N - 1] = ((IA * KEY + IB) * KEY + IC) * KEY + ID;
                  qs.push_back({IA, IB, IC, ID, K});
                }
              }
    if (kstart) kstart[K + 1] = (int32_t)(N + 1);
  }
  if (valteirk) {
    std::vector<std::vector<double>> ta(std::max(1, nthreads), std::vector<double>(g->nn1(), 0.0));
    std::vector<std::vector<double>> tb(std::max(1, nthreads), std::vector<double>(g->nn1(), 0.0));
    parallel_for((int64_t)qs.size(), nthreads, [&](int64_t i, int t) {
      const Q &q = qs[i];
      valteirk[i] = slater(g, q.a, q.b, q.c, q.d, q.k, ta[t].data(), tb[t].data());
    });
  }
  return N;
}

int or_rkintc(int nw, const int32_t *indteirk, const double *valteirk, const int32_t *kstart, int ia, int ib,
              int ic, int id, int k, double *tegral) {
  const int KEY = nw + 1;
  int IA = ia, IB = ib, IC = ic, ID = id;
  if (IA > IC) std::swap(IA, IC);
  if (IB > ID) std::swap(IB, ID);
  if (IA > IB) {
    std::swap(IA, IB);
    std::swap(IC, ID);
  }
  const int32_t index = ((IA * KEY + IB) * KEY + IC) * KEY + ID;
  int64_t jl = kstart[k], ju = kstart[k + 1] - 1;
  if (ju < jl || index < indteirk[jl - 1] || index > indteirk[ju - 1]) return -1;
  while (ju - jl > 1) {
    const int64_t jm = (ju + jl) / 2;
    if (indteirk[jm - 1] > index)
      ju = jm;
    else
      jl = jm;
  }
  int64_t loc;
  if (index == indteirk[ju - 1])
    loc = ju;
  else if (index == indteirk[jl - 1])
    loc = jl;
  else
    return -1;
  *tegral = valteirk[loc - 1];
  return 0;
}

double or_clrx(int kappaa, int k, int kappab) { return clrx(kappaa, k, kappab); }

int or_setham(or_ctx *g, int ncf, int64_t nelmnt, const int64_t *iendc, const uint8_t *iq, const or_list *tlist,
              int kmaxf, const or_list *vlists, double *emt) {
  const int NW = g->nw;
  std::vector<double> TA(g->nn1(), 0.0), TB(g->nn1(), 0.0);
  auto IQ = [&](int ir) { return iq + (size_t)(ir - 1) * NW; };
  auto E = [&](int64_t loc) -> double & { return emt[loc - 1]; };
  // I(a,a) pieces (setham.f90:83-100)
  for (int ia = 1; ia <= NW; ++ia) {
    bool set = false;
    double diaa = 0.0;
    for (int ir = 1; ir <= ncf; ++ir) {
      const int itmp = IQ(ir)[ia - 1];
      if (itmp <= 0) continue;
      if (!set) {
        diaa = rinti(g, ia, ia, 0, TA.data(), TB.data(), nullptr);
        set = true;
      }
      E(iendc[ir]) = E(iendc[ir]) + (double)itmp * diaa;
    }
  }
  // F0(a,a) (setham.f90:107-122)
  for (int ia = 1; ia <= NW; ++ia) {
    bool set = false;
    double f0aa = 0.0;
    for (int ir = 1; ir <= ncf; ++ir) {
      const double coef = fco(g, 0, IQ(ir), ia, ia);
      if (coef == 0.0) continue;
      if (!set) {
        f0aa = slater(g, ia, ia, ia, ia, 0, TA.data(), TB.data());
        set = true;
      }
      E(iendc[ir]) = E(iendc[ir]) + coef * f0aa;
    }
  }
  // Fk(a,a) (setham.f90:129-152)
  {
    int km = 0, K = 0;
    do {
      K = K + 2;
      for (int ia = 1; ia <= NW; ++ia) {
        const int k0 = g->NKJ[ia] - 1;
        km = std::max(k0, km);
        if (K > k0) continue;
        bool set = false;
        double fkaa = 0.0;
        for (int ir = 1; ir <= ncf; ++ir) {
          const double coef = fco(g, K, IQ(ir), ia, ia);
          if (coef == 0.0) continue;
          if (!set) {
            fkaa = slater(g, ia, ia, ia, ia, K, TA.data(), TB.data());
            set = true;
          }
          E(iendc[ir]) = E(iendc[ir]) + coef * fkaa;
        }
      }
    } while (K < km);
  }
  // F0(a,b) (setham.f90:159-176)
  for (int ia = 1; ia <= NW - 1; ++ia)
    for (int ib = ia + 1; ib <= NW; ++ib) {
      bool set = false;
      double f0ab = 0.0;
      for (int ir = 1; ir <= ncf; ++ir) {
        const double coef = fco(g, 0, IQ(ir), ia, ib);
        if (coef == 0.0) continue;
        if (!set) {
          f0ab = slater(g, ia, ib, ia, ib, 0, TA.data(), TB.data());
          set = true;
        }
        E(iendc[ir]) = E(iendc[ir]) + coef * f0ab;
      }
    }
  // Gk(a,b) (setham.f90:183-219)
  {
    int km = 0, K = -1;
    do {
      K = K + 1;
      for (int ia = 1; ia <= NW - 1; ++ia) {
        const int nkjia = g->NKJ[ia];
        for (int ib = ia + 1; ib <= NW; ++ib) {
          const int nkjib = g->NKJ[ib];
          int kmin;
          if (g->NAK[ia] * g->NAK[ib] > 0)
            kmin = std::abs((nkjia - nkjib) / 2);
          else
            kmin = std::abs((nkjia - nkjib) / 2) + 1;
          if ((K - kmin) % 2 != 0) continue;
          const int kmaxab = (nkjia + nkjib) / 2;
          km = std::max(kmaxab, km);
          if (K < kmin || K > kmaxab) continue;
          bool set = false;
          double gkab = 0.0;
          for (int ir = 1; ir <= ncf; ++ir) {
            const double coef = gco(g, K, IQ(ir), ia, ib);
            if (coef == 0.0) continue;
            if (!set) {
              gkab = slater(g, ia, ib, ib, ia, K, TA.data(), TB.data());
              set = true;
            }
            E(iendc[ir]) = E(iendc[ir]) + coef * gkab;
          }
        }
      }
    } while (K < km);
  }
  // T list (setham.f90:238-275)
  for (int64_t l = 0; l < tlist->nlab; ++l) {
    const int32_t lab = tlist->lab[l];
    const int ia = lab % KEYORB, ib = lab / KEYORB;
    const double tegral = rinti(g, ia, ib, 0, TA.data(), TB.data(), nullptr);
    for (int64_t i = tlist->start[l]; i < tlist->start[l + 1]; ++i) {
      const int32_t loc = tlist->loc[i];
      if ((int64_t)loc > nelmnt || loc < 1) return -1;
      E(loc) = E(loc) + tegral * tlist->coeff[i];
    }
  }
  // V^k lists (setham.f90:281-342)
  for (int K = 0; K <= kmaxf; ++K) {
    const or_list *vl = &vlists[K];
    for (int64_t l = 0; l < vl->nlab; ++l) {
      int32_t lab = vl->lab[l];
      const int id = lab % KEYORB;
      lab = lab / KEYORB;
      const int ib = lab % KEYORB;
      lab = lab / KEYORB;
      const int ic = lab % KEYORB;
      const int ia = lab / KEYORB;
      const double tegral = slater(g, ia, ib, ic, id, K, TA.data(), TB.data());
      for (int64_t i = vl->start[l]; i < vl->start[l + 1]; ++i) {
        const int32_t loc = vl->loc[i];
        if ((int64_t)loc > nelmnt || loc < 1) return -1;
        E(loc) = E(loc) + tegral * vl->coeff[i];
      }
    }
  }
  return 0;
}

// DSUBRS (rmcdhf90/dsubrs.f90:20-33), block-local CSF indices
static double dsubrs(int eol, int I, int J, const or_block &B) {
  if (eol) {
    double d = 0.0;
    for (int k = 1; k <= B.nev; ++k)
      d = d + B.evec[(size_t)(k - 1) * B.ncf + (I - 1)] * B.evec[(size_t)(k - 1) * B.ncf + (J - 1)] * B.wt[k - 1];
    return d;
  }
  return I == J ? B.wt[I - 1] : 0.0;
}

// SETCOF (rmcdhf90/setcof.f90:48-524): the reference's loops, lists in the
// order it builds them, a repeated label of a later block merged into the
// first entry with that label
int or_setcof(or_ctx *g, int nblocks, const or_block *blocks, int eol, int J, double UCFJ, int cap, int *ny,
              int32_t *nya, double *ya, int *nx, int32_t *nxa, double *xa, int *nd, int32_t *nda, double *da) {
  const int KEY = 215, NW = g->nw;
  std::vector<int32_t> NYA, NXA, NDA;
  std::vector<double> YA, XA, DA;
  auto merge = [](std::vector<int32_t> &lab, std::vector<double> &val, int32_t l, double v, bool search) {
    if (search)
      for (size_t i = 0; i < lab.size(); ++i)
        if (lab[i] == l) {
          val[i] = val[i] + v;
          return;
        }
    lab.push_back(l);
    val.push_back(v);
  };
  const int NAKJ = g->NAK[J], NKJJ = g->NKJ[J];
  // :73-105
  int64_t ILABEL = 0;
  int64_t NWTERM = (int64_t)KEY * (KEY + 1);
  for (int IB = 1; IB <= NW; ++IB) {
    ILABEL = ILABEL + NWTERM;
    const int KMAX = (IB == J) ? NKJJ - 1 : 0;
    for (int K = 0; K <= KMAX; K += 2) {
      double SUMR = 0.0;
      for (int nb = 0; nb < nblocks; ++nb) {
        const or_block &B = blocks[nb];
        for (int IR = 1; IR <= B.ncf; ++IR)
          SUMR = SUMR + dsubrs(eol, IR, IR, B) * fco(g, K, B.iq + (size_t)(IR - 1) * NW, J, IB);
      }
      const double YKAB = (IB == J) ? 2.0 * SUMR / UCFJ : SUMR / UCFJ;
      NYA.push_back((int32_t)(K + ILABEL));
      YA.push_back(YKAB);
    }
  }
  // :107-147
  ILABEL = (int64_t)KEY * J;
  NWTERM = (int64_t)KEY * KEY * (KEY + 1);
  for (int IB = 1; IB <= NW; ++IB) {
    ILABEL = ILABEL + NWTERM;
    if (IB == J) continue;
    const int NKJIB = g->NKJ[IB];
    const int KMIN = (NAKJ * g->NAK[IB] > 0) ? std::abs((NKJJ - NKJIB) / 2) : std::abs((NKJJ - NKJIB) / 2) + 1;
    const int KMAX = (NKJJ + NKJIB) / 2;
    for (int K = KMIN; K <= KMAX; K += 2) {
      double SUMR = 0.0;
      for (int nb = 0; nb < nblocks; ++nb) {
        const or_block &B = blocks[nb];
        for (int IR = 1; IR <= B.ncf; ++IR)
          SUMR = SUMR + dsubrs(eol, IR, IR, B) * gco(g, K, B.iq + (size_t)(IR - 1) * NW, J, IB);
      }
      NXA.push_back((int32_t)(K + ILABEL));
      XA.push_back(SUMR / UCFJ);
    }
  }
  // the column (ICLMN) owning each position of a block
  auto owners = [](const or_block &B) {
    std::vector<int32_t> own((size_t)B.iendc[B.ncf]);
    for (int c = 1; c <= B.ncf; ++c)
      for (int64_t p = B.iendc[c - 1]; p < B.iendc[c]; ++p) own[p] = c;
    return own;
  };
  auto label_sum = [&](const or_block &B, const std::vector<int32_t> &own, const or_list &L, int64_t l) {
    double SUM = 0.0;
    for (int64_t i = L.start[l]; i < L.start[l + 1]; ++i) {
      const int IR = B.irow[L.loc[i] - 1], IC = own[L.loc[i] - 1];
      double CONTR = dsubrs(eol, IR, IC, B) * L.coeff[i];
      if (IR != IC) CONTR = CONTR + CONTR;
      SUM = SUM + CONTR;
    }
    return 0.5 * SUM / UCFJ;
  };
  // :188-285, the T list of each block
  for (int nb = 0; nb < nblocks; ++nb) {
    const or_block &B = blocks[nb];
    const std::vector<int32_t> own = owners(B);
    for (int64_t l = 0; l < B.tlist.nlab; ++l) {
      const int LAB = B.tlist.lab[l];
      const int IA = LAB % KEY, IB = LAB / KEY;
      if (IA != J && IB != J) continue;
      const double SUM = label_sum(B, own, B.tlist, l);
      merge(NDA, DA, IA == J ? IB : IA, SUM, nb > 0);
    }
  }
  // :287-515, the V^k lists, k by k, block by block
  int KMAXF = -1;
  for (int nb = 0; nb < nblocks; ++nb) KMAXF = std::max(KMAXF, blocks[nb].kmaxf);
  for (int K = 0; K <= KMAXF; ++K)
    for (int nb = 0; nb < nblocks; ++nb) {
      const or_block &B = blocks[nb];
      if (K > B.kmaxf) continue;
      const std::vector<int32_t> own = owners(B);
      const or_list &L = B.vlists[K];
      for (int64_t l = 0; l < L.nlab; ++l) {
        int LAB = L.lab[l];
        int INDEXS[5];
        INDEXS[4] = LAB % KEY;
        LAB = LAB / KEY;
        INDEXS[2] = LAB % KEY;
        LAB = LAB / KEY;
        INDEXS[3] = LAB % KEY;
        INDEXS[1] = LAB / KEY;
        int IRANK = 0;
        for (int t = 1; t <= 4; ++t) IRANK += (INDEXS[t] == J);
        if (IRANK == 0) continue;
        const double SUM = label_sum(B, own, L, l);
        auto wrap = [](int il) { return il > 4 ? il - 4 : il; };
        if (IRANK == 1) {
          int ITHIS = -911;
          for (int IIND = 1; IIND <= 4; ++IIND) {
            if (INDEXS[IIND] != J) continue;
            const int IORB = INDEXS[wrap(IIND + 2)], IYO1 = INDEXS[wrap(IIND + 1)], IYO2 = INDEXS[wrap(IIND + 3)];
            ITHIS = ((IORB * KEY + IYO2) * KEY + IYO1) * KEY + K;
            break;
          }
          merge(NXA, XA, ITHIS, SUM, nb > 0);
        } else if (IRANK == 2) {
          int IFOUND = 0, LOC1 = 0, LOC2 = 0;
          for (int IIND = 1; IIND <= 4; ++IIND) {
            if (INDEXS[IIND] != J) continue;
            if (IFOUND == 0) {
              LOC1 = IIND;
              IFOUND = IFOUND + 1;
            } else if (IFOUND == 1) {
              LOC2 = IIND;
              break;
            }
          }
          if (LOC2 - LOC1 == 2) {
            const int IYO2 = INDEXS[wrap(LOC1 + 3)], IYO1 = INDEXS[wrap(LOC1 + 1)];
            merge(NYA, YA, (IYO2 * KEY + IYO1) * KEY + K, SUM + SUM, nb > 0);
          } else {
            const int IORB = INDEXS[wrap(LOC1 + 2)], IYO1 = INDEXS[wrap(LOC1 + 1)], IYO2 = INDEXS[wrap(LOC1 + 3)];
            merge(NXA, XA, ((IORB * KEY + IYO2) * KEY + IYO1) * KEY + K, SUM + SUM, nb > 0);
          }
        } else if (IRANK == 3) {
          int ITHIS = -911, ITHIS2 = -911;
          for (int IIND = 1; IIND <= 4; ++IIND) {
            if (INDEXS[IIND] == J) continue;
            const int INDIND = INDEXS[IIND];
            ITHIS = (INDIND * KEY + J) * KEY + K;
            ITHIS2 = ((INDIND * KEY + J) * KEY + J) * KEY + K;
          }
          merge(NYA, YA, ITHIS, SUM + SUM, nb > 0);
          merge(NXA, XA, ITHIS2, SUM, nb > 0);
        } else {
          merge(NYA, YA, (J * KEY + J) * KEY + K, 4.0 * SUM, nb > 0);
        }
      }
    }
  *ny = (int)NYA.size();
  *nx = (int)NXA.size();
  *nd = (int)NDA.size();
  if (*ny > cap || *nx > cap || *nd > cap) return -2;
  std::copy(NYA.begin(), NYA.end(), nya);
  std::copy(YA.begin(), YA.end(), ya);
  std::copy(NXA.begin(), NXA.end(), nxa);
  std::copy(XA.begin(), XA.end(), xa);
  std::copy(NDA.begin(), NDA.end(), nda);
  std::copy(DA.begin(), DA.end(), da);
  return 0;
}

double or_shift_eav(int ncf, const int64_t *iendc, double *emt) {
  double eav = 0.0;
  for (int ir = 1; ir <= ncf; ++ir) eav = eav + emt[iendc[ir] - 1];
  eav = eav / ncf;
  for (int i = 1; i <= ncf; ++i) emt[iendc[i] - 1] = emt[iendc[i] - 1] - eav;
  return eav;
}

void or_spicmv2(int n, int m, const int64_t *iendc, const int32_t *irow, const double *emt, const double *b,
                double *c) {
  spicmv2(n, m, iendc, irow, emt, b, c, 1);
}

// SPODMV (rci90/spodmv.f90:65-80): the rows as rci.res holds them (NELC
// entries, the diagonal EMT(NELC) last and unshifted), DIAG = C(ICOL,IV) +
// (EMT(NELC) - EAV) B(ICOL,IV), then DMERGE (dmerge.f90:35-40) over the
// other NELC - 1 entries, C(ICOL,IV) = DIAG + DL.
void or_spodmv(int n, int m, const int64_t *iendc, const int32_t *irow, const double *emt, double eav,
               const double *b, double *c) {
  for (int64_t i = 0; i < (int64_t)n * m; ++i) c[i] = 0.0;
  for (int icol = 1; icol <= n; ++icol) {
    const int64_t p0 = iendc[icol - 1], nelc = iendc[icol] - p0;
    const double *e = emt + p0;
    const int32_t *ir = irow + p0;
    for (int iv = 0; iv < m; ++iv) {
      const double *B = b + (size_t)iv * n;
      double *C = c + (size_t)iv * n;
      const double diag = C[icol - 1] + (e[nelc - 1] - eav) * B[icol - 1];
      const double dconst = B[icol - 1];
      double dsum = 0.0;
      for (int64_t i = 0; i < nelc - 1; ++i) {
        dsum = dsum + e[i] * B[ir[i] - 1];
        C[ir[i] - 1] = C[ir[i] - 1] + dconst * e[i];
      }
      C[icol - 1] = diag + dsum;
    }
  }
}

// DNICMV (rci90/dnicmv.f90:52-64) with DMERGE_DNICMV (:100-104): the lower
// triangle packed by rows, row ICOL = EMT(IBEG..IEND), IEND = IEND + ICOL;
// DIAG = C(ICOL,IV) + EMT(IEND) B(ICOL,IV), DL = DOT_PRODUCT(EMT(IBEG..IEND-1),
// B(1..ICOL-1)), C(1..ICOL-1) += B(ICOL) EMT(IBEG..IEND-1), C(ICOL) = DIAG + DL.
void or_dnicmv(int n, int m, const double *emt, const double *b, double *c) {
  for (int64_t i = 0; i < (int64_t)n * m; ++i) c[i] = 0.0;
  int64_t ibeg = 0;
  for (int icol = 1; icol <= n; ++icol) {
    const double *e = emt + ibeg;
    for (int iv = 0; iv < m; ++iv) {
      const double *B = b + (size_t)iv * n;
      double *C = c + (size_t)iv * n;
      const double diag = C[icol - 1] + e[icol - 1] * B[icol - 1];
      double dsum = 0.0;
      for (int i = 0; i < icol - 1; ++i) dsum = dsum + e[i] * B[i];
      const double dconst = B[icol - 1];
      for (int i = 0; i < icol - 1; ++i) C[i] = C[i] + dconst * e[i];
      C[icol - 1] = diag + dsum;
    }
    ibeg += icol;
  }
}

int or_dspevx(int n, const double *ap, int il, int iu, double *w, double *z) {
  return dspevx_lowest(n, ap, il, iu, w, z);
}

int or_iniest2(int nmax, int ncf, int niv, double *basis, const double *emt, const int64_t *iendc,
               const int32_t *irow) {
  const int ns = std::min(nmax, ncf);
  std::vector<double> ap((size_t)ns * (ns + 1) / 2, 0.0);
  int64_t joffspar = 0;
  for (int j = 1; j <= ns; ++j) {
    const int64_t joffnorm = (int64_t)j * (j - 1) / 2;
    for (int64_t ir = joffspar + 1; ir <= iendc[j]; ++ir) ap[irow[ir - 1] + joffnorm - 1] = emt[ir - 1];
    joffspar = iendc[j];
  }
  std::vector<double> eig(niv), vec((size_t)ns * niv);
  const int info = dspevx_lowest(ns, ap.data(), 1, niv, eig.data(), vec.data());
  for (int64_t i = 0; i < (int64_t)ncf * niv; ++i) basis[i] = 0.0;
  for (int j = 0; j < niv; ++j)
    for (int i = 0; i < ns; ++i) basis[(size_t)ncf * j + i] = vec[(size_t)ns * j + i];
  for (int j = 0; j < niv; ++j) basis[(size_t)niv * ncf + j] = eig[j];
  return info;
}

int or_gdvd(int n, const int64_t *iendc, const int32_t *irow, const double *emt, double *diag,
            const or_dvd_params *p, double *work, int64_t lwork, int *nloops_out, int *nmv_out, int *ierr_out,
            int nthreads) {
  const int LIM = p->lim, ILOW = p->ilow, IHIGH = p->ihigh, MBLOCK = p->mblock, MAXITER = p->maxiter;
  int NIV = p->niv;
  const double CRITE = p->crite, CRITC = p->critc, CRITR = p->critr;
  int IERR = 0, NMV = 0, NLOOPS = 0;
  // GDVD: NIV == 0 is an error (gdvd.f90:60-64)
  if (NIV == 0) {
    *ierr_out = -1000;
    return -1;
  }
  // DVDSON argument checks (dvdson.f90:297-384), ISELEC range given by ILOW..IHIGH
  if (LIM > n) IERR += 1;
  if (LIM <= 0) IERR += 2;
  if (ILOW <= 0 || ILOW > n) IERR += 4;
  if (IHIGH > n) IERR += 8;
  const int NEIG = IHIGH - ILOW + 1;
  if (NEIG <= 0) IERR += 16;
  if (NEIG > LIM) IERR += 32;
  if (IERR) {
    *ierr_out = IERR;
    return -1;
  }
  const int NUME = IHIGH;
  if (ILOW + IHIGH - 1 > n) { // HIEND: highest eigenpairs are not used by MANEIG
    *ierr_out = -2;
    return -1;
  }
  if (NEIG > NUME) IERR += 64;
  if (NUME > LIM || (NUME == LIM && NUME != n)) IERR += 128;
  if (MBLOCK < 1 || MBLOCK > NEIG) IERR += 256;
  if (lwork < (int64_t)LIM * (2 * (int64_t)n + LIM + (NUME + 10)) + NUME) IERR += 512;
  if (NIV > LIM) IERR += 4096;
  if (IERR) {
    *ierr_out = IERR;
    return -1;
  }
  std::vector<int> ISELEC(NEIG);
  for (int i = 0; i < NEIG; ++i) ISELEC[i] = ILOW + i;
  // workspace map (dvdson.f90:405-420), NOC = 0, 0-based offsets
  double *BASIS = work;
  double *EIGVAL = BASIS + (size_t)n * LIM;
  double *AB = EIGVAL + LIM;
  double *S = AB + (size_t)n * LIM;
  double *TEMPS = S + (size_t)LIM * (LIM + 1) / 2;
  double *SVEC = TEMPS + (size_t)LIM * (LIM + 1) / 2;
  double *SCRA1 = SVEC + (size_t)LIM * LIM;
  double *OLDVAL = SCRA1 + 8 * LIM;
  std::vector<int> INCV(LIM + 1), ICV(NUME + 2), IND(std::max(NEIG, LIM) + 1);
  std::vector<double> ROWLAST(std::max(NEIG, LIM) + 1);
  std::vector<double> basis_copy;
  auto OP = [&](int m, const double *b, double *c) {
    spicmv2(n, m, iendc, irow, emt, b, c, nthreads);
    NMV += m;
  };
  // INITDVD (dvdson.f90:848-948) with NUME + 1
  {
    const int NUME1 = NUME + 1;
    if (NIV == 0) {
      for (int64_t i = 0; i < n; ++i) BASIS[i] = 1.0 / std::sqrt((double)n);
      NIV = 1;
    }
    int IST = 1, IEND = NIV, NEW = NIV;
    for (;;) {
      OP(NEW, BASIS + (size_t)(IST - 1) * n, AB + (size_t)(IST - 1) * n);
      if (IEND < NUME1) {
        NEW = std::min(NUME1 - IEND, IEND - IST + 1);
        std::memcpy(BASIS + (size_t)IEND * n, AB + (size_t)(IST - 1) * n, sizeof(double) * (size_t)n * NEW);
        mgs_nrm(n, IEND, NEW, SCRA1, BASIS);
        IST = IEND + 1;
        IEND = IEND + NEW;
        continue;
      }
      break;
    }
    NIV = IEND;
    adds(n, 0, NIV, BASIS, AB, S);
  }
  NLOOPS = 1;
  // DVDRVR (dvdson.f90:559-842)
  for (int i = 1; i <= NUME; ++i) {
    EIGVAL[i - 1] = 1.0e30;
    ICV[i] = 0;
  }
  int KPASS = NIV, NNCV = KPASS;
  int REST = std::max(LIM / 2, 2 * NUME);
  REST = std::min(REST, LIM - 3);
  bool DONE = false;
  for (;;) {
    const int IFIND = std::min(KPASS, REST);
    for (int i = 0; i < IFIND; ++i) OLDVAL[i] = EIGVAL[i];
    std::memcpy(TEMPS, S, sizeof(double) * (size_t)KPASS * (KPASS + 1) / 2);
    const int info = dspevx_lowest(KPASS, TEMPS, 1, IFIND, EIGVAL, SVEC);
    if (info != 0) {
      IERR = -std::abs(info);
      *ierr_out = IERR;
      return -1;
    }
    // TSTSEL (dvdson.f90:1260-1413)
    {
      int NNCE = 0;
      for (int i = 0; i < NEIG; ++i) {
        const int ival = ISELEC[i];
        if (std::fabs(OLDVAL[ival - 1] - EIGVAL[ival - 1]) < CRITE) continue;
        ++NNCE;
      }
      if (NNCE == 0) {
        DONE = true;
      } else {
        int ICNT = 0;
        for (int i = 0; i < NEIG; ++i) {
          const int64_t icur = (int64_t)KPASS * ISELEC[i]; // 1-based SVEC index
          double tmax = std::fabs(SVEC[icur - 1]);
          for (int l = 1; l <= NNCV - 1; ++l) tmax = std::max(tmax, std::fabs(SVEC[icur - l - 1]));
          if (tmax < CRITC) {
            ICV[ISELEC[i]] = 1;
          } else {
            ICV[ISELEC[i]] = 0;
            ++ICNT;
            IND[ICNT] = ISELEC[i];
            ROWLAST[ICNT] = tmax;
          }
        }
        NNCV = ICNT;
        DONE = (NNCV == 0);
        for (int i = 1; i <= NNCV; ++i) {
          int indx = 1;
          double best = std::fabs(ROWLAST[i]);
          for (int q = 2; q <= NNCV - i + 1; ++q)
            if (std::fabs(ROWLAST[i + q - 1]) > best) {
              best = std::fabs(ROWLAST[i + q - 1]);
              indx = q;
            }
          INCV[i] = IND[indx + i - 1];
          std::swap(ROWLAST[indx + i - 1], ROWLAST[i]);
          std::swap(IND[indx + i - 1], IND[i]);
        }
      }
    }
    if (DONE || KPASS >= n) break;
    if (KPASS == LIM) {
      // OVFLOW (dvdson.f90:1179-1256)
      multbc(n, KPASS, REST, SVEC, SCRA1, BASIS);
      multbc(n, KPASS, REST, SVEC, SCRA1, AB);
      for (int64_t i = 0; i < (int64_t)REST * (REST + 1) / 2; ++i) S[i] = 0.0;
      for (int64_t i = 0; i < (int64_t)REST * REST; ++i) SVEC[i] = 0.0;
      int64_t ind = 0, icur = 0;
      for (int i = 1; i <= REST; ++i) {
        S[ind + i - 1] = EIGVAL[i - 1];
        SVEC[icur + i - 1] = 1.0;
        icur += REST;
        ind += i;
      }
      KPASS = REST;
    }
    // NEWVEC (dvdson.f90:1002-1172)
    {
      double *EPSIL = SCRA1 + LIM;
      size_t icur = (size_t)KPASS * n;
      int nadded = 0, icvc = 0;
      const int limadd = std::min(LIM, MBLOCK + KPASS);
      DONE = false;
      for (int i = 1; i <= NNCV; ++i) {
        const int indx = INCV[i];
        dgemv_n(n, KPASS, BASIS, SVEC + (size_t)(indx - 1) * KPASS, BASIS + icur);
        dgemv_n(n, KPASS, AB, SVEC + (size_t)(indx - 1) * KPASS, AB + icur);
        const double ev = EIGVAL[indx - 1];
        for (int64_t q = 0; q < n; ++q) AB[icur + q] += (-ev) * BASIS[icur + q];
        const double sqres = ddot(n, AB + icur, AB + icur);
        SCRA1[indx - 1] = std::sqrt(sqres);
        if (SCRA1[indx - 1] < CRITR) {
          ++icvc;
          ICV[indx] = 1;
          if (icvc < NNCV) continue;
          DONE = true;
          break;
        }
        double gap;
        if (indx == 1) {
          gap = std::fabs(EIGVAL[1] - EIGVAL[0]);
        } else {
          const double gaplow = std::fabs(EIGVAL[indx - 1] - EIGVAL[indx - 2]);
          const double gapup = std::fabs(EIGVAL[indx] - EIGVAL[indx - 1]);
          gap = std::min(gaplow, gapup);
        }
        double dl = std::fabs(OLDVAL[indx - 1] - EIGVAL[indx - 1]);
        // p->robust: on the first pass OLDVAL still holds DVDRVR's 1e30
        // sentinel (dvdson.f90:703), which makes RHSEPS ~ 1e13 and the first
        // correction vector useless; the robust variant uses DL = 0 there.
        if (p->robust && OLDVAL[indx - 1] >= 1.0e29) dl = 0.0;
        const double res = SCRA1[indx - 1];
        const double rhseps = (gap > res) ? std::sqrt(dl * res) : std::min(dl, std::sqrt(dl));
        EPSIL[indx - 1] = 0.0;
        for (int64_t q = 0; q < n; ++q) AB[icur + q] += (-rhseps) * BASIS[icur + q];
        ++nadded;
        INCV[nadded] = indx;
        if (nadded + KPASS == limadd) break;
        icur += n;
      }
      if (DONE) break;
      NNCV = nadded;
    }
    // GDVD preconditioner, IRC = 1 (gdvd.f90:93-134): w = r / (DIAG - lambda)
    {
      size_t icurv = 0;
      for (int i = 1; i <= NNCV; ++i) {
        const int indx = INCV[i];
        const double value = EIGVAL[indx - 1];
        const double *r = AB + (size_t)KPASS * n + icurv;
        double *w = BASIS + (size_t)KPASS * n + icurv;
        for (int64_t j = 0; j < n; ++j) diag[j] = diag[j] - value;
        for (int64_t j = 0; j < n; ++j) {
          if (std::fabs(diag[j]) > 1.0e-06)
            w[j] = r[j] / diag[j];
          else
            w[j] = r[j] * 1.0e06;
        }
        for (int64_t j = 0; j < n; ++j) diag[j] = diag[j] + value;
        icurv += n;
      }
    }
    mgs_nrm(n, KPASS, NNCV, SCRA1 + LIM, BASIS);
    OP(NNCV, BASIS + (size_t)KPASS * n, AB + (size_t)KPASS * n);
    adds(n, KPASS, NNCV, BASIS, AB, S);
    KPASS += NNCV;
    ++NLOOPS;
    if (NLOOPS <= MAXITER) continue;
    IERR += 2048;
    --NLOOPS;
    KPASS -= NNCV;
    break;
  }
  // label 30 (dvdson.f90:821-836)
  for (int i = 0; i < NUME; ++i) OLDVAL[i] = std::fabs(OLDVAL[i] - EIGVAL[i]);
  multbc(n, KPASS, NUME, SVEC, SCRA1, BASIS);
  multbc(n, KPASS, NUME, SVEC, SCRA1, AB);
  for (int i = 0; i < NUME; ++i) {
    double *t = AB + (size_t)NUME * n;
    for (int64_t q = 0; q < n; ++q) t[q] = AB[(size_t)i * n + q] + (-EIGVAL[i]) * BASIS[(size_t)i * n + q];
    SCRA1[i] = std::sqrt(ddot(n, t, t));
  }
  // DVDSON epilogue (dvdson.f90:466-474): eigenvalues after the eigenvectors
  std::vector<double> ev(EIGVAL, EIGVAL + NUME), od(OLDVAL, OLDVAL + NUME), rn(SCRA1, SCRA1 + NUME);
  for (int i = 0; i < NUME; ++i) {
    BASIS[(size_t)n * NUME + i] = ev[i];
    BASIS[(size_t)(n + 1) * NUME + i] = od[i];
    BASIS[(size_t)(n + 2) * NUME + i] = rn[i];
  }
  *nloops_out = NLOOPS;
  *nmv_out = NMV;
  *ierr_out = IERR;
  return IERR == 0 ? 0 : 1;
}

int or_maneig(int flavour, int ncf, int nvec, const int64_t *iendc, const int32_t *irow, const double *emt,
              double *eval, double *evec, int *nloops, int *nmv, int *ierr, int nthreads, int robust,
              int maxiter_override, double *seconds) {
  using clk = std::chrono::steady_clock;
  const auto t_start = clk::now();
  if (seconds) seconds[0] = seconds[1] = 0.0;
  *nloops = 0;
  *nmv = 0;
  *ierr = 0;
  if (ncf == 1) {
    eval[0] = 0.0;
    evec[0] = 1.0;
    return 0;
  }
  const int IOLPCK = 2000, N1000 = 4000;
  bool dense = (flavour == 0) ? (ncf <= IOLPCK) : false;
  if (dense) {
    // rci90/maneig.f90:157-241: packed upper from the lower-triangle rows
    std::vector<double> ap((size_t)ncf * (ncf + 1) / 2, 0.0);
    for (int i = 1; i <= ncf; ++i) {
      const int64_t iofset = (int64_t)i * (i - 1) / 2;
      for (int64_t ir = iendc[i - 1] + 1; ir <= iendc[i]; ++ir) ap[iofset + irow[ir - 1] - 1] = emt[ir - 1];
    }
    const int rc = dspevx_lowest(ncf, ap.data(), 1, nvec, eval, evec);
    if (rc) return rc;
  } else {
    int lim, maxitr, niv;
    if (flavour == 0) {
      lim = std::min(ncf, 2 * nvec + 60);
      maxitr = std::max(nvec * 200, ncf / 10);
      niv = nvec;
    } else {
      lim = std::min(ncf, 2 * nvec + 40);
      niv = std::min(nvec, ncf);
      maxitr = std::min(nvec * 200, ncf);
    }
    const int64_t lwork = 2 * (int64_t)ncf * lim + (int64_t)lim * lim * 2 + 11 * (int64_t)lim + nvec;
    std::vector<double> work(lwork, 0.0), diag(ncf);
    for (int ic = 1; ic <= ncf; ++ic) diag[ic - 1] = emt[iendc[ic] - 1];
    const int nmax = (flavour == 0) ? 2000 : N1000;
    or_iniest2(nmax, ncf, niv, work.data(), emt, iendc, irow);
    const auto t_ini = clk::now();
    if (seconds) seconds[0] = std::chrono::duration<double>(t_ini - t_start).count();
    if (maxiter_override > 0) maxitr = maxiter_override;
    if (flavour == 0 || ncf > N1000) {
      or_dvd_params p;
      p.lim = lim;
      p.ilow = 1;
      p.ihigh = niv;
      p.niv = niv;
      p.mblock = 1;
      p.maxiter = maxitr;
      p.crite = 1.0e-17;
      p.critc = 1.0e-9;
      p.critr = 1.0e-9;
      p.ortho = std::max(1e-9, p.critr);
      p.robust = robust;
      int rc = or_gdvd(ncf, iendc, irow, emt, diag.data(), &p, work.data(), lwork, nloops, nmv, ierr, nthreads);
      if (rc < 0) return rc;
    }
    if (seconds) seconds[1] = std::chrono::duration<double>(clk::now() - t_ini).count();
    const int64_t nend = (int64_t)ncf * niv;
    for (int j = 0; j < nvec; ++j) {
      eval[j] = work[nend + j];
      std::memcpy(evec + (size_t)ncf * j, work.data() + (size_t)ncf * j, sizeof(double) * ncf);
    }
  }
  // sign fix: dominant component positive (rci90/maneig.f90:532-555)
  for (int j = 0; j < nvec; ++j) {
    double *v = evec + (size_t)ncf * j;
    double amax = 0.0;
    int ia = 0;
    for (int i = 0; i < ncf; ++i) {
      const double wa = std::fabs(v[i]);
      if (wa <= amax) continue;
      amax = wa;
      ia = i;
    }
    if (v[ia] >= 0.0) continue;
    for (int i = 0; i < ncf; ++i) v[i] = -v[i];
  }
  return 0;
}

} // extern "C"
