// breit.cu - the transverse-photon (Breit) radial integrals of rci on the GPU:
// GENINTBREIT1/2's tables (rci90/genintbreit1.f90, genintbreit2.f90) and
// BRINTF (rci90/brintf.f90) for any list of integrals (what BRINT3-6 compute
// on demand).
//
// BRINTF(type, a, b, c, d, k) combines up to four RKINT (rkint.f90) or two
// SKINT (skint.f90) terms; each term is one QUAD (quad.f90) of a product
// with one or two ZKF functions (zkf.f90: Z_k of a radial product, the
// stride-4 Newton-Cotes chain), the frequency-dependent terms weighted by
// spherical Bessel factors (bessel.f90). On the device:
//
//  0. k_plan_table / k_plan_items: the integrals and their terms. A table
//     row (k, a, b) holds the (c, d) whose TRIANGBREIT pair masks share a
//     bit, in the reference's order; one pass counts each row's integrals
//     and terms, the host scans the counts, a second pass writes them.
//  1. k_bessel: every Bessel function the integrals need, (pair, order) with
//     W = WFACT |E(a) - E(b)| / C, one block each: the series where it
//     converges in four terms, the asymptotic form from the first point where
//     it does not (JCHAN), as bessel.f90:104-201.
//  2. k_breit_jobs: one thread per QUAD term. The thread runs the ZKF chain
//     (or two) point by point and feeds each TA(i) straight into a streaming
//     QUAD (head search, power-law head term, stride-4 group sums, end
//     correction), so no ZK or TA array is stored: a term costs one pass
//     over its points. The arithmetic is the reference's, operation by
//     operation (compiled without FMA contraction), so the values are the
//     oracle's to the rounding of log, sin and cos.
//  3. k_breit_combine: each integral from its terms, BRRA's and SKINT's
//     combinations (brra.f90:36-118, skint.f90:70-83).
//
// BRINTF is evaluated as a function of its arguments: the reference keeps
// the last Bessel functions in four slots (bess_C KEEP) and skips a BESSEL
// call whose slot already holds the function; slot 1 holds pair (a, b),
// slot 2 pair (c, d). Where the reference skips the call for two equal
// orbitals (zero frequency, brintf.f90:47-48) its slot keeps earlier
// content; here that slot is the zero-frequency function (zero).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <vector>

#include "gg_internal.cuh"

namespace gg {
namespace {

constexpr int KLIM = 20;  // the power tables' rows (YZK's KLIMIT)

__device__ __forceinline__ double pfv(const double *P, int ld, int i, int j) {
  return P[(size_t)(j - 1) * ld + (i - 1)];
}

// libgcc's __powidf2 algorithm (gfortran's REAL**INTEGER)
__device__ __forceinline__ double powi_d(double x, int m) {
  unsigned n = m < 0 ? -(unsigned)m : (unsigned)m;
  double y = (n % 2) ? x : 1.0;
  while (n >>= 1) {
    x = x * x;
    if (n % 2) y = y * x;
  }
  return m < 0 ? 1.0 / y : y;
}

struct BessDesc {
  double w;  // W (> EPSI^2)
  int nn;    // order
};

// BESSEL (rci90/bessel.f90:96-201) for one (pair, order): BJ, BN at points
// 1..N ([f][np]). Series at each point while every earlier point converged
// in four terms; from the first that does not (JCHAN), the asymptotic form.
__global__ void __launch_bounds__(128) k_bessel(const BessDesc *__restrict__ bd, const double *__restrict__ R, int n,
                                                int np, double epsi, double *__restrict__ BJ,
                                                double *__restrict__ BN) {
  __shared__ int jchan_s;
  const BessDesc d = bd[blockIdx.x];
  double *J = BJ + (size_t)blockIdx.x * np, *N = BN + (size_t)blockIdx.x * np;
  const int nn = d.nn;
  const double W = d.w;
  if (threadIdx.x == 0) jchan_s = n + 1;
  __syncthreads();
  for (int j = 2 + threadIdx.x; j <= n; j += blockDim.x) {
    const double WA = -0.5 * ((R[j] * W) * (R[j] * W));
    double X1 = 1.0, X2 = 1.0, S1 = 0.0, S2 = 0.0;
    bool done = false;
    for (int i = 1; i <= 4; ++i) {
      X1 = X1 * WA / (double)(i * (2 * (nn + i) + 1));
      X2 = X2 * WA / (double)(i * (2 * (i - nn) - 1));
      S1 = S1 + X1;
      S2 = S2 + X2;
      if (fabs(X1) >= fabs(S1) * epsi || fabs(X2) >= fabs(S2) * epsi) continue;
      done = true;
      break;
    }
    J[j] = S1;
    N[j] = S2;
    if (!done) atomicMin(&jchan_s, j);
  }
  if (threadIdx.x == 0) {
    J[1] = 0.0;
    N[1] = 0.0;
  }
  __syncthreads();
  const int jchan = jchan_s;
  if (jchan > n) return;
  double DFNM = 1.0, DFN = 1.0;
  if (nn != 0) {
    for (int i = 3; i <= 2 * nn - 1; i += 2) DFNM = DFNM * (double)i;
    DFN = DFNM * (double)(2 * nn + 1);
  }
  DFNM = 1.0 / DFNM;
  const int irem = nn % 4;
  const double SSN = (irem == 1 || irem == 2) ? -1.0 : 1.0;
  const double SCN = (irem == 2 || irem == 3) ? -1.0 : 1.0;
  const bool swap = (irem == 1 || irem == 3);
  for (int j = jchan + threadIdx.x; j <= n; j += blockDim.x) {
    const double WA = W * R[j];
    double SN, CN;
    if (!swap) {
      SN = SSN * sin(WA);
      CN = SCN * cos(WA);
    } else {
      SN = SSN * cos(WA);
      CN = SCN * sin(WA);
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
    J[j] = S1 * DFN / powi_d(WA, nn) - 1.0;
    N[j] = S2 * powi_d(WA, nn + 1) * DFNM - 1.0;
  }
}

// One QUAD term. form 0: RKINT (one chain of order k from src (1 + BJ);
// TA = part (1 + BN) ZK RPOR); 1: SKINT at zero frequency (chains k - 1 and
// k + 1 of src; TA = part RPOR (ZK+ - ZK-)); 2: SKINT's first term (chains
// k - 1 of src and of (-src) BJ; TA = ((1 + BN) ZK2 - ZK1 BN) part / R^2
// RPOR); 3: SKINT's second term (chain k + 1 of src (1 + BJ); TA = part
// (1 + BN) ZK R RP). src and part are P_x Q_y (+ P_y Q_x with the aug flag);
// a Bessel index of -1 is the zero function.
struct BrJob {
  unsigned char form, sx, sy, px, py, flags;  // flags: 1 src aug, 2 part aug
  signed char k, pad;
  int bj, bn;
};

struct ChainState {
  double z0, z1, z2, z3;      // ZK(II-4 .. II-1)
  double t0, t1, t2, t3;      // TEMP(II-4 .. II-1)
};

// streaming QUAD (lib9290/quad.f90:52-103) over TA(2..mtp) fed in order
struct QuadStream {
  int mtp, head, cnt;
  double prev, result, s, g0, g1, g2, last;
  __device__ void init(int m) {
    mtp = m;
    head = 0;
    cnt = 0;
    prev = 0.0;
    result = 0.0;
    s = 0.0;
    last = 0.0;
  }
  __device__ __forceinline__ void group(double g3, const QuadConst &q) {
    s = s + (q.C2 * (g0 + g2) + q.C3 * g1 + q.C4 * g3);
  }
  __device__ __forceinline__ void push(int i, double ta, const double *R, const double *RP, const QuadConst &q) {
    last = ta;
    if (head) {
      switch (cnt) {
        case 0: g0 = ta; break;
        case 1: g1 = ta; break;
        case 2: g2 = ta; break;
        default: group(ta, q); break;
      }
      cnt = (cnt + 1) & 3;
      return;
    }
    // head search at i - 1 (2 <= i - 1 <= mtp - 1)
    const int h = i - 1;
    if (h >= 2 && fabs(prev) > 0.0) {
      const double tai = prev, taip1 = ta;
      const double quott = taip1 / tai;
      if (quott > 0.0) {
        const double frip1 = taip1 / RP[h + 1];
        double fri = tai / RP[h];
        const double ratio = frip1 / fri;
        const double sigma = log(ratio) / log(R[h + 1] / R[h]);
        fri = R[h] * fri;
        result = fri / (sigma + 1.0);
        result = result + q.C1 * tai;
        head = h;
        g0 = ta;  // the first group starts at h + 1
        cnt = 1;
        return;
      }
    }
    prev = ta;
  }
  __device__ __forceinline__ double finish(const QuadConst &q) {
    if (!head) return 0.0;
    if (cnt == 1) {
      g1 = 0.0;
      g2 = 0.0;
      group(0.0, q);
    } else if (cnt == 2) {
      g2 = 0.0;
      group(0.0, q);
    } else if (cnt == 3) {
      group(0.0, q);
    }
    double r = result + s;
    if ((mtp - head) % 4 == 0) r = r - q.C1 * last;
    return r;
  }
};

__device__ __forceinline__ double prod(const double *PF, const double *QF, int ld, int i, int x, int y, bool aug) {
  double v = pfv(PF, ld, i, x) * pfv(QF, ld, i, y);
  if (aug) v = v + pfv(PF, ld, i, y) * pfv(QF, ld, i, x);
  return v;
}

__global__ void __launch_bounds__(128) k_breit_jobs(const BrJob *__restrict__ jobs, int64_t njobs,
                                                    const double *__restrict__ PF, const double *__restrict__ QF,
                                                    int ld, const int *__restrict__ MF, const double *__restrict__ R,
                                                    const double *__restrict__ RP, const double *__restrict__ RPOR,
                                                    const double *__restrict__ Pow, int np, QuadConst q,
                                                    const double *__restrict__ BJt, const double *__restrict__ BNt,
                                                    double *__restrict__ out) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= njobs) return;
  const BrJob jb = jobs[t];
  const int form = jb.form, K = jb.k;
  const bool saug = jb.flags & 1, paug = jb.flags & 2;
  const int mtpz = min(MF[jb.sx], MF[jb.sy]);
  const int mtpq = min(mtpz, min(MF[jb.px], MF[jb.py]));
  const double *BJ = jb.bj >= 0 ? BJt + (size_t)jb.bj * np : nullptr;
  const double *BN = jb.bn >= 0 ? BNt + (size_t)jb.bn * np : nullptr;
  // chain orders: form 0: k; 1: k - 1 (a) and k + 1 (b); 2: k - 1, k - 1; 3: k + 1
  const int ka = (form == 0) ? K : (form == 3 ? K + 1 : K - 1);
  const int kb = (form == 1) ? K + 1 : K - 1;
  const bool two = (form == 1 || form == 2);
  // RTTK rows: k > 0 the R**k row, k = -1 the 1/R row (R**-1), k = 0 unused
  const double *rta = ka > 0 ? Pow + (size_t)ka * np : (ka < 0 ? Pow : nullptr);
  const double *rtb = kb > 0 ? Pow + (size_t)kb * np : (kb < 0 ? Pow : nullptr);
  // TEMP(i) of chain a and b, 0 beyond MTPZ (zkf.f90:48-57)
  auto temps = [&](int i, double &ta_, double &tb_) {
    if (i > mtpz) {
      ta_ = 0.0;
      tb_ = 0.0;
      return;
    }
    const double src = prod(PF, QF, ld, i, jb.sx, jb.sy, saug);
    const double bj = BJ ? BJ[i] : 0.0;
    double inA, inB = 0.0;
    if (form == 0 || form == 3) {
      inA = src * (1.0 + bj);
    } else if (form == 1) {
      inA = src;
      inB = src;
    } else {
      inA = src;
      inB = -src * bj;
    }
    const double rhoA = RP[i] * inA;
    ta_ = (ka == 0) ? rhoA : rta[i] * rhoA;
    if (two) {
      const double rhoB = RP[i] * inB;
      tb_ = (kb == 0) ? rhoB : rtb[i] * rhoB;
    } else {
      tb_ = 0.0;
    }
  };
  // ZK(2..4) from TEMP(2..5) (zkf.f90:58-64)
  double T[4][2];
  for (int i = 0; i < 4; ++i) temps(i + 2, T[i][0], T[i][1]);
  ChainState A, B;
  A.z0 = 0.0;
  B.z0 = 0.0;
  double za[3], zb[3];
  for (int ii = 2; ii <= 4; ++ii) {
    double sa = 0.0, sb = 0.0;
    for (int kk = 2; kk <= 5; ++kk) {
      sa = sa + q.CNC5C[kk - 2][ii - 2] * T[kk - 2][0];
      sb = sb + q.CNC5C[kk - 2][ii - 2] * T[kk - 2][1];
    }
    za[ii - 2] = sa;
    zb[ii - 2] = sb;
  }
  A.z1 = za[0]; A.z2 = za[1]; A.z3 = za[2];
  B.z1 = zb[0]; B.z2 = zb[1]; B.z3 = zb[2];
  A.t0 = 0.0; A.t1 = T[0][0]; A.t2 = T[1][0]; A.t3 = T[2][0];
  B.t0 = 0.0; B.t1 = T[0][1]; B.t2 = T[1][1]; B.t3 = T[2][1];
  double nextA = T[3][0], nextB = T[3][1];  // TEMP(5)
  QuadStream Q;
  Q.init(mtpq);
  for (int i = 2; i <= mtpq; ++i) {
    double zA, zB;
    if (i <= 4) {
      zA = za[i - 2];
      zB = zb[i - 2];
    } else {
      // ZK(II) = ZK(II-4) + C1 (TEMP(II-4) + TEMP(II)) + C2 (TEMP(II-3) +
      // TEMP(II-1)) + C3 TEMP(II-2) (zkf.f90:65-68)
      double tA, tB;
      if (i == 5) {
        tA = nextA;
        tB = nextB;
      } else {
        temps(i, tA, tB);
      }
      zA = A.z0 + q.C1 * (A.t0 + tA) + q.C2 * (A.t1 + A.t3) + q.C3 * A.t2;
      A.z0 = A.z1; A.z1 = A.z2; A.z2 = A.z3; A.z3 = zA;
      A.t0 = A.t1; A.t1 = A.t2; A.t2 = A.t3; A.t3 = tA;
      if (two) {
        zB = B.z0 + q.C1 * (B.t0 + tB) + q.C2 * (B.t1 + B.t3) + q.C3 * B.t2;
        B.z0 = B.z1; B.z1 = B.z2; B.z2 = B.z3; B.z3 = zB;
        B.t0 = B.t1; B.t1 = B.t2; B.t2 = B.t3; B.t3 = tB;
      } else {
        zB = 0.0;
      }
    }
    // ZK(i) / RTTK(i) for k != 0 (zkf.f90:70-74)
    const double ZA = (ka == 0) ? zA : zA / rta[i];
    const double ZB = two ? ((kb == 0) ? zB : zB / rtb[i]) : 0.0;
    const double part = prod(PF, QF, ld, i, jb.px, jb.py, paug);
    const double bn = BN ? BN[i] : 0.0;
    double ta;
    if (form == 0)
      ta = part * (1.0 + bn) * ZA * RPOR[i];
    else if (form == 1)
      ta = part * RPOR[i] * (ZB - ZA);
    else if (form == 2)
      ta = ((1.0 + bn) * ZB - ZA * bn) * part / powi_d(R[i], 2) * RPOR[i];
    else
      ta = part * (1.0 + bn) * ZA * R[i] * RP[i];
    Q.push(i, ta, R, RP, q);
  }
  out[t] = Q.finish(q);
}

// One integral: its first term, the combination (code) and SKINT's data.
// code: 0 2 q0; 1 q0 + q1; 2 (((q0 + q1) + q2) + q3) / 2; 3 S(1);
// 4 (S(1) + S(2)) / 2. S(w) = (WK / W)^2 qa - qb W W / ((2K+3)(2K-1)) at a
// frequency, WK qa / 2 at zero frequency (|W| < 1e-10).
struct BrInt {
  int q0;
  short code, k;
  double w1, w2;
};

__device__ __forceinline__ double skint_comb(const double *v, int &at, double W, int K) {
  const double WK = (double)(K + K + 1);
  if (fabs(W) < 1.0e-10) return WK * v[at++] * 0.5;
  double sk = powi_d(WK / W, 2) * v[at++];
  sk = sk - v[at++] * W * W / (double)((2 * K + 3) * (2 * K - 1));
  return sk;
}

__global__ void k_breit_combine(const BrInt *__restrict__ ints, int64_t n, const double *__restrict__ v,
                                double *__restrict__ out) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= n) return;
  const BrInt b = ints[t];
  int at = b.q0;
  double r;
  switch (b.code) {
    case 0: r = 2.0 * v[at]; break;
    case 1: r = v[at] + v[at + 1]; break;
    case 2: r = (v[at] + v[at + 1] + v[at + 2] + v[at + 3]) * 0.5; break;
    case 3: r = skint_comb(v, at, b.w1, b.k); break;
    default: {
      const double s1 = skint_comb(v, at, b.w1, b.k);
      const double s2 = skint_comb(v, at, b.w2, b.k);
      r = (s1 + s2) * 0.5;
    }
  }
  out[t] = r;
}

// ---------------------------------------------------------------------------
// the terms of each integral (brintf.f90:34-69, brra.f90:36-118), planned on
// the device: one thread per integral (or per (k, a, b) row of a table)
// counts its terms, the counts are scanned, the same thread writes them.
// ---------------------------------------------------------------------------
struct PlanTabs {
  const double *W;   // [a][b]: W = WFACT |E(a) - E(b)| / C
  const int *bid;    // [order + 1][min(a,b)][max(a,b)]: Bessel function, -1 zero
  int nw;
};

__device__ __forceinline__ int bes_id(const PlanTabs &T, int x, int y, int nn) {
  const int lo = min(x, y), hi = max(x, y);
  return T.bid[((size_t)(nn + 1) * T.nw + (lo - 1)) * T.nw + (hi - 1)];
}

// BRINTF(type, a, b, c, d, k): RAC = P_a Q_b, RBD = P_c Q_d; Bessel slot 1
// pair (a, b), slot 2 pair (c, d). Returns the number of terms; with bi and
// jb set, writes the integral's record (first term q0) and its terms.
__device__ int plan_one(int type, int a, int b, int c, int d, int K, const PlanTabs &T, int q0, BrInt *bi,
                        BrJob *jb) {
  auto w = [&](int x, int y) { return T.W[(size_t)(x - 1) * T.nw + (y - 1)]; };
  int n = 0;
  auto job = [&](int form, int sx, int sy, bool saug, int px, int py, bool paug, int bj, int bn) {
    if (jb) {
      BrJob j;
      j.form = (unsigned char)form;
      j.sx = (unsigned char)sx;
      j.sy = (unsigned char)sy;
      j.px = (unsigned char)px;
      j.py = (unsigned char)py;
      j.flags = (unsigned char)((saug ? 1 : 0) | (paug ? 2 : 0));
      j.k = (signed char)K;
      j.pad = 0;
      j.bj = bj;
      j.bn = bn;
      jb[n] = j;
    }
    ++n;
  };
  auto R = [&](bool rac, int iw, bool augac, bool augbd) {
    const int f = iw == 0 ? -1 : (iw == 1 ? bes_id(T, a, b, K) : bes_id(T, c, d, K));
    if (rac)
      job(0, a, b, augac, c, d, augbd, f, f);
    else
      job(0, c, d, augbd, a, b, augac, f, f);
  };
  auto S = [&](int iw) {
    const int x = iw == 1 ? a : c, y = iw == 1 ? b : d;
    if (fabs(w(x, y)) < 1.0e-10) {
      job(1, a, b, false, c, d, false, -1, -1);
    } else {
      const int f1 = bes_id(T, x, y, K - 1), f2 = bes_id(T, x, y, K + 1);
      job(2, a, b, false, c, d, false, f1, f2);
      job(3, c, d, false, a, b, false, f2, f1);
    }
  };
  int code;
  switch (type) {
    case 1:
      if (a == c && b == d) {
        code = 0;
        R(true, 1, false, false);
      } else if (a == d && b == c) {
        code = 1;
        R(true, 1, false, false);
        R(false, 1, false, false);
      } else {
        code = 2;
        R(true, 1, false, false);
        R(true, 2, false, false);
        R(false, 1, false, false);
        R(false, 2, false, false);
      }
      break;
    case 2:
      if ((a == c && b == d) || (a == d && b == c)) {
        code = 3;
        S(1);
      } else {
        code = 4;
        S(1);
        S(2);
      }
      break;
    case 3:
      code = 2;
      if (a == b) {
        R(true, 0, false, true);
        R(false, 0, false, true);
        R(true, 2, false, true);
        R(false, 2, false, true);
      } else {
        R(true, 1, true, false);
        R(false, 1, true, false);
        R(true, 0, true, false);
        R(false, 0, true, false);
      }
      break;
    case 4:
      code = 1;
      R(true, 0, false, false);
      R(false, 0, false, false);
      break;
    case 5:
      if (a == d && b == c) {
        code = 1;
        R(true, 1, false, false);
        R(false, 1, false, false);
      } else {
        code = 0;
        R(true, 1, false, false);
      }
      break;
    default:
      code = 3;
      S(1);
      break;
  }
  if (bi) {
    BrInt r;
    r.q0 = q0;
    r.code = (short)code;
    r.k = (short)K;
    r.w1 = w(a, b);
    r.w2 = w(c, d);
    *bi = r;
  }
  return n;
}

// a table row: the (c, d) that TRIANGBREIT admits with (k, a, b) (pair
// masks share a bit), in the reference's order; pass 0 counts integrals and
// terms, pass 1 writes them from the scanned offsets
__global__ void k_plan_table(int type, int nw, int kmax, const unsigned char *__restrict__ mask, PlanTabs T,
                             int pass, int *__restrict__ cnt_i, int *__restrict__ cnt_j,
                             const int64_t *__restrict__ off_i, const int64_t *__restrict__ off_j,
                             int32_t *__restrict__ ind, BrInt *__restrict__ ints, BrJob *__restrict__ jobs) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (kmax + 1) * nw * nw) return;
  const int K = t / (nw * nw), a = (t / nw) % nw + 1, b = t % nw + 1;
  const int KEY = nw + 1;
  const unsigned char *mk = mask + (size_t)K * (nw + 1) * (nw + 1);
  const unsigned char mab = mk[a * (nw + 1) + b];
  int ni = 0, nj = 0;
  if (mab) {
    int64_t pi = pass ? off_i[t] : 0, pj = pass ? off_j[t] : 0;
    for (int c = 1; c <= nw; ++c)
      for (int d = 1; d <= nw; ++d)
        if (mab & mk[c * (nw + 1) + d]) {
          if (pass) {
            ind[pi] = ((a * KEY + b) * KEY + c) * KEY + d;
            const int q = plan_one(type, a, b, c, d, K, T, (int)pj, ints + pi, jobs + pj);
            ++pi;
            pj += q;
          } else {
            ++ni;
            nj += plan_one(type, a, b, c, d, K, T, 0, nullptr, nullptr);
          }
        }
  }
  if (!pass) {
    cnt_i[t] = ni;
    cnt_j[t] = nj;
  }
}

// a list of integrals (items[6 t ..] = type, a, b, c, d, k)
__global__ void k_plan_items(const int32_t *__restrict__ items, int n, PlanTabs T, int pass, int *__restrict__ cnt_j,
                             const int64_t *__restrict__ off_j, BrInt *__restrict__ ints, BrJob *__restrict__ jobs) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int32_t *it = items + 6 * (size_t)t;
  if (pass)
    plan_one(it[0], it[1], it[2], it[3], it[4], it[5], T, (int)off_j[t], ints + t, jobs + off_j[t]);
  else
    cnt_j[t] = plan_one(it[0], it[1], it[2], it[3], it[4], it[5], T, 0, nullptr, nullptr);
}

template <class T> int upload_vec(DBuf<T> &b, const std::vector<T> &h, cudaStream_t s) {
  GG_TRY(b.alloc(std::max<size_t>(1, h.size())));
  if (!h.empty()) GG_CUDA(cudaMemcpyAsync(b.p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, s));
  return GG_OK;
}

// the host side of a plan: the frequencies, the Bessel functions the
// integrals read (pair, order) with their ids, on the device
struct Plan {
  gg_ctx *ctx = nullptr;
  int nw = 0;
  double wfact = 0, epsi = 0;
  std::vector<double> e, W;
  std::vector<int> bid;  // [order + 1][lo][hi]
  std::vector<BessDesc> bess;
  DBuf<double> dW;
  DBuf<int> dbid;
  int norders() const { return KLIM + 3; }
  int &slot(int x, int y, int nn) {
    const int lo = std::min(x, y), hi = std::max(x, y);
    return bid[((size_t)(nn + 1) * nw + (lo - 1)) * nw + (hi - 1)];
  }
  void need(int x, int y, int nn) {
    int &s = slot(x, y, nn);
    if (s != -2) return;
    const double w = W[(size_t)(x - 1) * nw + (y - 1)];
    if (w < epsi * epsi) {
      s = -1;
    } else {
      s = (int)bess.size();
      bess.push_back(BessDesc{w, nn});
    }
  }
  int upload(cudaStream_t s) {
    for (int &v : bid)
      if (v == -2) v = -1;
    GG_TRY(upload_vec(dW, W, s));
    GG_TRY(upload_vec(dbid, bid, s));
    return GG_OK;
  }
  PlanTabs tabs() const { return PlanTabs{dW.p, dbid.p, nw}; }
};

int make_plan(gg_ctx *ctx, double wfact, const double *e, double accy, Plan &P) {
  GG_TRY(ensure_orbitals(ctx));
  const Orbitals &o = ctx->orb;
  if (!e) return fail(GG_ERR_ARG, "Breit integrals: orbital energies required");
  if (o.nw > 214) return fail(GG_ERR_ARG, "Breit integrals: more than 214 orbitals");
  P.ctx = ctx;
  P.nw = o.nw;
  P.wfact = wfact;
  P.epsi = std::sqrt(0.1 * (accy > 0 ? accy : std::pow(ctx->grid.h, 6)));
  P.e.assign(e, e + o.nw);
  P.W.assign((size_t)o.nw * o.nw, 0.0);
  for (int x = 1; x <= o.nw; ++x)
    for (int y = 1; y <= o.nw; ++y)
      P.W[(size_t)(x - 1) * o.nw + (y - 1)] = wfact * std::fabs(e[x - 1] - e[y - 1]) / ctx->grid.c;
  P.bid.assign((size_t)P.norders() * o.nw * o.nw, -2);
  return GG_OK;
}

// the Bessel functions, the terms and the combinations; values into out
// (host, ni integrals); *kernel_ms: device time of these kernels
int run_terms(gg_ctx *ctx, const Plan &P, const BrJob *djobs, int64_t nj, const BrInt *dints, int64_t ni,
              double *out, double *kernel_ms = nullptr) {
  const Grid &g = ctx->grid;
  const Orbitals &o = ctx->orb;
  cudaStream_t s = ctx->stream;
  const int nb = (int)P.bess.size();
  DBuf<BessDesc> dbd;
  DBuf<double> dBJ, dBN, dv, dout;
  GG_TRY(upload_vec(dbd, P.bess, s));
  GG_TRY(dBJ.alloc((size_t)std::max(1, nb) * g.np));
  GG_TRY(dBN.alloc((size_t)std::max(1, nb) * g.np));
  GG_TRY(dv.alloc(std::max<int64_t>(1, nj)));
  GG_TRY(dout.alloc(std::max<int64_t>(1, ni)));
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (kernel_ms) {
    GG_CUDA(cudaEventCreate(&e0));
    GG_CUDA(cudaEventCreate(&e1));
    GG_CUDA(cudaEventRecord(e0, s));
  }
  if (nb > 0) {
    k_bessel<<<nb, 128, 0, s>>>(dbd.p, g.dR.p, g.n, g.np, P.epsi, dBJ.p, dBN.p);
    ::gg::note_launch();
  }
  if (nj > 0) {
    k_breit_jobs<<<(unsigned)((nj + 127) / 128), 128, 0, s>>>(djobs, nj, o.dPF.p, o.dQF.p, o.ld, o.dMF.p, g.dR.p,
                                                               g.dRP.p, g.dRPOR.p, g.dPow.p, g.np, g.q, dBJ.p,
                                                               dBN.p, dv.p);
    ::gg::note_launch();
  }
  if (ni > 0) {
    k_breit_combine<<<(unsigned)((ni + 255) / 256), 256, 0, s>>>(dints, ni, dv.p, dout.p);
    ::gg::note_launch();
  }
  GG_CUDA(cudaGetLastError());
  if (kernel_ms) GG_CUDA(cudaEventRecord(e1, s));
  if (ni > 0) GG_CUDA(cudaMemcpyAsync(out, dout.p, ni * sizeof(double), cudaMemcpyDeviceToHost, s));
  GG_CUDA(cudaStreamSynchronize(s));
  if (kernel_ms) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    *kernel_ms = ms;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
  }
  return GG_OK;
}

// exclusive scan of counts into int64 offsets; returns the total
int64_t scan(const std::vector<int> &cnt, std::vector<int64_t> &off) {
  off.resize(cnt.size());
  int64_t t = 0;
  for (size_t i = 0; i < cnt.size(); ++i) {
    off[i] = t;
    t += cnt[i];
  }
  return t;
}

}  // namespace
}  // namespace gg

using namespace gg;

extern "C" {

int gg_genintbreit(gg_ctx *ctx, int type, double wfact, const double *e, double accy, int64_t *nb_out,
                   int *j2max_out) {
  if (!ctx || (type != 1 && type != 2)) return fail(GG_ERR_ARG, "gg_genintbreit: type 1 or 2");
  GG_CUDA(cudaSetDevice(ctx->device));
  Plan P;
  GG_TRY(make_plan(ctx, wfact, e, accy, P));
  GG_TRY(timer_start(ctx));
  const auto th0 = std::chrono::steady_clock::now();
  const Orbitals &o = ctx->orb;
  const int nw = o.nw;
  int j2max = o.nkj[1];
  for (int i = 2; i <= nw; ++i) j2max = std::max(j2max, o.nkj[i]);
  if (j2max + 1 > KLIM) return fail(GG_ERR_ARG, "gg_genintbreit: 2j above 19");
  BreitTable &T = ctx->breit[type - 1];
  T.valid = false;
  T.j2max = j2max;
  cudaStream_t s = ctx->stream;
  // TRIANGBREIT1 (rci90/triangbreit1.f90:27-46) and TRIANGBREIT2
  // (triangbreit2.f90:27-42) factor into one condition per pair: type 1
  // admits (a, b, c, d) when some L in K-1..K+1 admits both pairs, type 2
  // when both pairs are admitted at L = K. mask[k][pair] holds those bits
  // (per L); the Bessel functions the admitted integrals read are those of
  // the pairs with a mask bit, at order k (type 1) or k -+ 1 (type 2).
  const size_t msz = (size_t)(nw + 1) * (nw + 1);
  std::vector<unsigned char> mask((size_t)(j2max + 1) * msz, 0);
  for (int K = 0; K <= j2max; ++K)
    for (int a = 1; a <= nw; ++a)
      for (int b = 1; b <= nw; ++b) {
        unsigned char m = 0;
        const int la = o.nkl[a], lb = o.nkl[b], ja = o.nkj[a], jb = o.nkj[b];
        if (type == 1) {
          for (int t = 0; t < 3; ++t) {
            const int L = K - 1 + t;
            if ((K + la + lb) % 2 == 1 && std::abs(ja - jb) <= 2 * L && std::abs(ja + jb) >= 2 * L) m |= 1 << t;
          }
          if (m) P.need(a, b, K);
        } else if ((K + la + lb) % 2 == 0 && std::abs(ja - jb) <= 2 * K && std::abs(ja + jb) >= 2 * K) {
          m = 1;
          P.need(a, b, K - 1);
          P.need(a, b, K + 1);
        }
        mask[(size_t)K * msz + (size_t)a * (nw + 1) + b] = m;
      }
  GG_TRY(P.upload(s));
  DBuf<unsigned char> dmask;
  GG_TRY(upload_vec(dmask, mask, s));
  const int rows = (j2max + 1) * nw * nw;
  DBuf<int> dci, dcj;
  GG_TRY(dci.alloc(rows));
  GG_TRY(dcj.alloc(rows));
  k_plan_table<<<(rows + 127) / 128, 128, 0, s>>>(type, nw, j2max, dmask.p, P.tabs(), 0, dci.p, dcj.p, nullptr,
                                                  nullptr, nullptr, nullptr, nullptr);
  ::gg::note_launch();
  GG_CUDA(cudaGetLastError());
  std::vector<int> ci(rows), cj(rows);
  GG_CUDA(cudaMemcpyAsync(ci.data(), dci.p, rows * sizeof(int), cudaMemcpyDeviceToHost, s));
  GG_CUDA(cudaMemcpyAsync(cj.data(), dcj.p, rows * sizeof(int), cudaMemcpyDeviceToHost, s));
  GG_CUDA(cudaStreamSynchronize(s));
  std::vector<int64_t> oi, oj;
  const int64_t ni = scan(ci, oi), nj = scan(cj, oj);
  if (ni > INT32_MAX || nj > INT32_MAX) return fail(GG_ERR_RANGE, "gg_genintbreit: table too large");
  T.kstart.assign(j2max + 2, 1);
  for (int K = 0; K <= j2max; ++K) T.kstart[K + 1] = (int32_t)((K + 1 <= j2max ? oi[(size_t)(K + 1) * nw * nw] : ni) + 1);
  DBuf<int64_t> doi, doj;
  DBuf<int32_t> dind;
  DBuf<BrInt> dints;
  DBuf<BrJob> djobs;
  GG_TRY(upload_vec(doi, oi, s));
  GG_TRY(upload_vec(doj, oj, s));
  GG_TRY(dind.alloc(std::max<int64_t>(1, ni)));
  GG_TRY(dints.alloc(std::max<int64_t>(1, ni)));
  GG_TRY(djobs.alloc(std::max<int64_t>(1, nj)));
  k_plan_table<<<(rows + 127) / 128, 128, 0, s>>>(type, nw, j2max, dmask.p, P.tabs(), 1, nullptr, nullptr, doi.p,
                                                  doj.p, dind.p, dints.p, djobs.p);
  ::gg::note_launch();
  GG_CUDA(cudaGetLastError());
  T.n = ni;
  T.hInd.resize(ni);
  if (ni > 0) GG_CUDA(cudaMemcpyAsync(T.hInd.data(), dind.p, ni * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  ctx->stats[32] = 1e3 * std::chrono::duration<double>(std::chrono::steady_clock::now() - th0).count();
  T.hVal.assign(std::max<int64_t>(1, ni), 0.0);
  GG_TRY(run_terms(ctx, P, djobs.p, nj, dints.p, ni, T.hVal.data(), &ctx->stats[33]));
  T.hVal.resize(ni);
  T.valid = true;
  double ms = 0;
  GG_TRY(timer_stop(ctx, &ms));
  ctx->stats[31] = ms;
  if (nb_out) *nb_out = T.n;
  if (j2max_out) *j2max_out = j2max;
  return GG_OK;
}

int gg_get_breit_table(gg_ctx *ctx, int type, int32_t *indtp, double *valtp, int32_t *kstart) {
  if (!ctx || (type != 1 && type != 2)) return fail(GG_ERR_ARG, "gg_get_breit_table: type 1 or 2");
  const BreitTable &T = ctx->breit[type - 1];
  if (!T.valid) return fail(GG_ERR_STATE, "gg_get_breit_table: no table of this type (call gg_genintbreit)");
  if (indtp) std::copy(T.hInd.begin(), T.hInd.end(), indtp);
  if (valtp) std::copy(T.hVal.begin(), T.hVal.end(), valtp);
  if (kstart) std::copy(T.kstart.begin(), T.kstart.end(), kstart);
  return GG_OK;
}

// BRINT1 / BRINT2 (rci90/brint1.f90:30-66): binary search in the k range
int gg_brint(gg_ctx *ctx, int type, int ia, int ib, int ic, int id, int k, double *tegral) {
  if (!ctx || (type != 1 && type != 2) || !tegral) return fail(GG_ERR_ARG, "gg_brint: bad arguments");
  const BreitTable &T = ctx->breit[type - 1];
  if (!T.valid) return fail(GG_ERR_STATE, "gg_brint: no table of this type (call gg_genintbreit)");
  const int nw = ctx->orb.nw, KEY = nw + 1;
  if (k < 0 || k > T.j2max || ia < 1 || ib < 1 || ic < 1 || id < 1 || ia > nw || ib > nw || ic > nw || id > nw)
    return fail(GG_ERR_NOTFOUND, "gg_brint: integral not in the table");
  const int32_t index = ((ia * KEY + ib) * KEY + ic) * KEY + id;
  const int32_t *b = T.hInd.data() + (T.kstart[k] - 1), *e = T.hInd.data() + (T.kstart[k + 1] - 1);
  const int32_t *p = std::lower_bound(b, e, index);
  if (p == e || *p != index) return fail(GG_ERR_NOTFOUND, "gg_brint: integral not in the table");
  *tegral = T.hVal[p - T.hInd.data()];
  return GG_OK;
}

int gg_brintf(gg_ctx *ctx, int n, const int32_t *items, double wfact, const double *e, double accy, double *out) {
  if (!ctx || n < 0 || (n > 0 && (!items || !out))) return fail(GG_ERR_ARG, "gg_brintf: bad arguments");
  if (n == 0) return GG_OK;
  GG_CUDA(cudaSetDevice(ctx->device));
  Plan P;
  GG_TRY(make_plan(ctx, wfact, e, accy, P));
  const int nw = ctx->orb.nw;
  // the Bessel functions the integrals read (brintf.f90:34-69)
  for (int t = 0; t < n; ++t) {
    const int32_t *it = items + 6 * (size_t)t;
    if (it[0] < 1 || it[0] > 6) return fail(GG_ERR_ARG, "gg_brintf: type outside 1..6");
    for (int j = 1; j <= 4; ++j)
      if (it[j] < 1 || it[j] > nw) return fail(GG_ERR_ARG, "gg_brintf: orbital outside the orbital set");
    const int K = it[5];
    if (K < 0 || K + 1 > KLIM) return fail(GG_ERR_ARG, "gg_brintf: k outside 0..19");
    switch (it[0]) {
      case 1: case 3: P.need(it[1], it[2], K); P.need(it[3], it[4], K); break;
      case 5: P.need(it[1], it[2], K); break;
      case 2: P.need(it[3], it[4], K - 1); P.need(it[3], it[4], K + 1);  // fall through
      case 6: P.need(it[1], it[2], K - 1); P.need(it[1], it[2], K + 1); break;
      default: break;
    }
  }
  cudaStream_t s = ctx->stream;
  GG_TRY(P.upload(s));
  DBuf<int32_t> ditems;
  DBuf<int> dcj;
  GG_TRY(ditems.alloc((size_t)6 * n));
  GG_CUDA(cudaMemcpyAsync(ditems.p, items, (size_t)6 * n * sizeof(int32_t), cudaMemcpyHostToDevice, s));
  GG_TRY(dcj.alloc(n));
  k_plan_items<<<(n + 127) / 128, 128, 0, s>>>(ditems.p, n, P.tabs(), 0, dcj.p, nullptr, nullptr, nullptr);
  ::gg::note_launch();
  GG_CUDA(cudaGetLastError());
  std::vector<int> cj(n);
  GG_CUDA(cudaMemcpyAsync(cj.data(), dcj.p, n * sizeof(int), cudaMemcpyDeviceToHost, s));
  GG_CUDA(cudaStreamSynchronize(s));
  std::vector<int64_t> oj;
  const int64_t nj = scan(cj, oj);
  DBuf<int64_t> doj;
  DBuf<BrInt> dints;
  DBuf<BrJob> djobs;
  GG_TRY(upload_vec(doj, oj, s));
  GG_TRY(dints.alloc(n));
  GG_TRY(djobs.alloc(std::max<int64_t>(1, nj)));
  k_plan_items<<<(n + 127) / 128, 128, 0, s>>>(ditems.p, n, P.tabs(), 1, nullptr, doj.p, dints.p, djobs.p);
  ::gg::note_launch();
  GG_CUDA(cudaGetLastError());
  return run_terms(ctx, P, djobs.p, nj, dints.p, n, out);
}

}  // extern "C"
