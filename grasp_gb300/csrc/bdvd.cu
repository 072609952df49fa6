// bdvd.cu - MANEIG for many CI blocks at once: a batched Davidson whose whole
// iteration runs on the GPU for every block together.
//
// The reference solves the J/parity blocks of a run one after another
// (rci90/matrix.f90:177-187 calls MANEIG per block): dense DSPEVX when
// NCF <= 2000 (rci90/maneig.f90:157-241), DVDSON otherwise. A run over many
// ions and J values has hundreds of blocks of a few hundred to a few thousand
// CSFs; one block alone fills a few SMs for a few microseconds per kernel,
// so here all blocks advance in lockstep through one sequence of kernels:
//
//   eig      one CTA per block: the k x k projected matrix S (k <= LIM) is
//            reduced to tridiagonal form by Householder reflections in shared
//            memory; its lowest eigenvalues by Sturm bisection and Newton
//            steps; eigenvectors by inverse iteration (re-orthogonalised
//            inside clusters), back-transformed by the reflectors
//   ritz     Ritz vectors X = V y, residuals R = W y - theta X, |R| per tile
//   conv     per block: residual test (|r_j| <= CRITR), the targets that get a
//            new vector, restart decision (basis full: collapse to REST Ritz
//            vectors, as OVFLOW does, libdvd90/dvdson.f90:716-717)
//   restart  V <- V Y(:, 1:REST), W <- W Y(:, 1:REST), S <- diag(theta)
//   precond  t_j = r_j / (DIAG - theta_j), or r_j 1e6 where |DIAG - theta_j|
//            <= 1e-6 (GDVD's preconditioner, libdvd90/gdvd.f90:114-129)
//   CGS2     two passes of classical Gram-Schmidt of the new vectors against
//            the basis, then two rounds of Cholesky QR among them; a vector
//            whose norm falls below 1e-8 of its norm before is dropped
//   spmm     W_new = H V_new for all blocks, one warp per row, up to four
//            vectors per pass over the row; FP64 or hi+lo FP32 split values
//   S        the new columns of S = V^T W
//
// Every reduction has a fixed order (per-tile partials added in tile order),
// so results do not change from run to run. The iteration is captured once as
// a CUDA graph and replayed; converged blocks drop out inside the kernels.
//
// Differences from the reference, on purpose: small blocks (NCF <= LIM) are
// solved exactly by this same code with the full unit basis instead of DSPEVX;
// larger ones start from the unit vectors of the lowest diagonal elements
// (the Rayleigh-Ritz solution of that principal submatrix) instead of
// INIEST2, add up to NVEC vectors per iteration (MBLOCK = NVEC) and stop on
// the residual norm alone.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <numeric>
#include <string>
#include <tuple>
#include <vector>

#include "gg_internal.cuh"

namespace gg {
namespace {

constexpr int TR = 128;     // rows per tile
// batched matvec variants for the autotuner: rows per CTA x threads per CTA
constexpr int SPMM_TR[3] = {64, 128, 256};
constexpr int SPMM_T[2] = {128, 256};
constexpr int SPMM_NVAR = 6;
constexpr int BT = 256;     // threads of the tile kernels
constexpr int RT = 128;     // threads of the row-per-thread tile kernels (= TR)
constexpr int EIG_T = 256;  // threads of the projected eigensolver
constexpr int MAXL = 128;   // largest LIM
constexpr int MAXR = 16;    // most roots per block
constexpr int AC = 32;      // A columns staged per pass of the dot kernel
constexpr int RG = 16;      // rows per group in the restart kernel

struct BDesc {
  int n, r, lim, rest, m0, maxiter;
  int row0, tile0, ntile, pofs;
  long long voff, xoff;  // V/W (n x lim) and X/R (n x r) offsets
  long long soff;        // S and Y (lim x lim) offset
  long long coff;        // C offset (max(lim, MAXR) x MAXR)
  const int64_t *ptr;
  const int32_t *col;
  const unsigned short *col16;  // 16-bit copy of col (NCF <= 65536), or null
  const double *val;
  const float *hi, *lo;
  const double *diag;
};

struct BState {
  int m;        // basis size
  int active;   // 1 while some target is unconverged
  int ncur;     // new vectors at columns [m, m + ncur)
  int nprev;    // new vectors before the last Cholesky QR round
  int restart;  // collapse the basis this iteration
  int iters, nmv, ierr;
  int nv;       // eigenvectors of S computed this iteration
  int mprev;    // size of the leading block of S whose eigenvalues are in theta
  int neold;    // how many of them are valid
  int newt[MAXR];
  double theta[MAXL];
  double rn[MAXR];
  double nrm0[MAXR];
};

struct BTile {
  int b, r0, nr;
};

// 32 bytes of one row's x values: four FP64 values or four hi + lo pairs
struct __align__(32) X32 {
  double a, b, c, d;
};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// ---------------------------------------------------------------------------
// Projected eigenproblem, one CTA per block.
// ---------------------------------------------------------------------------
struct EigShape {
  int lmax, nvmax;
  __host__ __device__ int lda() const { return lmax | 1; }
  __host__ __device__ size_t bytes() const {
    // A, seven vectors, Z, scalars, FP32 copies of d and e^2
    return sizeof(double) * ((size_t)lmax * lda() + 7 * (size_t)lmax + (size_t)lmax * nvmax + 8) +
           sizeof(float) * 2 * (size_t)lmax;
  }
};

// LU of the tridiagonal T - lam I with partial pivoting, and inverse
// iteration from a fixed pseudo-random start (Golub & Van Loan, 4th ed.,
// sec. 8.2.2); x is re-orthogonalised against ncl earlier vectors of the same
// cluster (columns cl[] of Z) at every step. The pivots are inverted once, so
// the solves multiply instead of divide (GB300 issues FP64 slowly; a division
// is a sequence of FP64 instructions).
__device__ void inv_iter_dev(int n, const double *d, const double *e, double lam, double tnorm, double *x,
                             const double *Z, int ldz, const int *cl, int ncl, unsigned seed) {
  if (n == 1) {
    x[0] = 1.0;
    return;
  }
  double l[MAXL], ru0[MAXL], u1[MAXL], u2[MAXL];
  unsigned char piv[MAXL];
  const double tiny = 2.220446049250313e-16 * fmax(tnorm, 1e-300);
  double a0 = d[0] - lam, a1 = e[0];
  for (int i = 0; i < n; ++i) {
    double sub = 0, b0 = 0, b1 = 0;
    if (i + 1 < n) {
      sub = e[i];
      b0 = d[i + 1] - lam;
      b1 = (i + 2 < n) ? e[i + 1] : 0.0;
    }
    double u0;
    if (i + 1 < n && fabs(sub) > fabs(a0)) {
      piv[i] = 1;
      const double m = a0 / sub;
      l[i] = m;
      u0 = sub;
      u1[i] = b0;
      u2[i] = b1;
      const double n0 = a1 - m * b0, n1 = -m * b1;
      a0 = n0;
      a1 = n1;
    } else {
      piv[i] = 0;
      if (a0 == 0.0) a0 = tiny;
      u0 = a0;
      const double m = (i + 1 < n) ? sub / a0 : 0.0;
      l[i] = m;
      u1[i] = a1;
      u2[i] = 0.0;
      a0 = b0 - m * a1;
      a1 = b1;
    }
    if (fabs(u0) < tiny) u0 = u0 < 0 ? -tiny : tiny;
    ru0[i] = 1.0 / u0;
  }
  unsigned s = 2463534242u ^ (seed * 2654435761u);
  for (int i = 0; i < n; ++i) {
    s ^= s << 13;
    s ^= s >> 17;
    s ^= s << 5;
    x[i] = (double)(s & 0xffff) / 65536.0 - 0.5 + 1e-3;
  }
  for (int it = 0; it < 2; ++it) {
    for (int i = 0; i + 1 < n; ++i) {
      if (piv[i]) {
        const double t = x[i];
        x[i] = x[i + 1];
        x[i + 1] = t;
      }
      x[i + 1] -= l[i] * x[i];
    }
    for (int i = n - 1; i >= 0; --i) {
      double v = x[i];
      if (i + 1 < n) v -= u1[i] * x[i + 1];
      if (i + 2 < n) v -= u2[i] * x[i + 2];
      x[i] = v * ru0[i];
    }
    for (int c = 0; c < ncl; ++c) {
      const double *q = Z + (size_t)cl[c] * ldz;
      double dot = 0.0;
      for (int i = 0; i < n; ++i) dot += q[i] * x[i];
      for (int i = 0; i < n; ++i) x[i] -= dot * q[i];
    }
    double nrm = 0.0;
    for (int i = 0; i < n; ++i) nrm += x[i] * x[i];
    nrm = sqrt(nrm);
    if (nrm == 0.0) nrm = 1.0;
    const double inv = 1.0 / nrm;
    for (int i = 0; i < n; ++i) x[i] *= inv;
  }
}

// Sturm count of T - xI (number of eigenvalues below x) and, for Newton's
// method, f'/f of det(T - xI) (Wilkinson, The Algebraic Eigenvalue Problem,
// ch. 5, sec. 37-38: the LDL^T pivots q_i count the eigenvalues below x and
// f'/f = sum q_i'/q_i).
__device__ __forceinline__ int sturm64(int m, const double *dd, const double *e2, double x, double pivmin,
                                       double *fpf) {
  double q = dd[0] - x;
  if (fabs(q) < pivmin) q = -pivmin;
  double inv = 1.0 / q, Sd = -inv, qp = -1.0;
  int cnt = (q < 0.0);
  for (int i = 1; i < m; ++i) {
    const double ei2 = e2[i - 1];
    double qi = fma(-ei2, inv, dd[i] - x);
    qi = (fabs(qi) < pivmin) ? -pivmin : qi;
    const double dq = fma(ei2 * qp, inv * inv, -1.0);
    const double iv = 1.0 / qi;
    cnt += (qi < 0.0);
    Sd = fma(dq, iv, Sd);
    qp = dq;
    inv = iv;
  }
  *fpf = Sd;
  return cnt;
}

__device__ __forceinline__ int sturm32(int m, const float *d, const float *e2, float x, float pivmin) {
  float q = d[0] - x;
  if (fabsf(q) < pivmin) q = -pivmin;
  int cnt = (q < 0.f);
  for (int i = 1; i < m; ++i) {
    q = (d[i] - x) - __fdividef(e2[i - 1], q);
    if (fabsf(q) < pivmin) q = -pivmin;
    cnt += (q < 0.f);
  }
  return cnt;
}

__global__ void __launch_bounds__(EIG_T) k_b_eig(const BDesc *__restrict__ desc, BState *__restrict__ st,
                                                 const double *__restrict__ Spool, double *__restrict__ Ypool,
                                                 EigShape sh) {
  extern __shared__ double smem[];
  const int b = blockIdx.x;
  BState &S = st[b];
  if (!S.active) return;
  const BDesc D = desc[b];
  const int m = S.m, r = D.r, L = D.lim;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int lda = sh.lda();
  double *A = smem;                          // [m][lda], column-major, lower triangle used
  double *dd = A + (size_t)sh.lmax * lda;    // d
  double *ee = dd + sh.lmax;                 // e (subdiagonal)
  double *bt = ee + sh.lmax;                 // beta of each reflector
  double *vv = bt + sh.lmax;                 // current reflector
  double *pp = vv + sh.lmax;                 // p, then w
  double *ev = pp + sh.lmax;                 // eigenvalues
  double *e2 = ev + sh.lmax;                 // e^2
  double *Z = e2 + sh.lmax;                  // eigenvectors [nv][m]
  double *scal = Z + (size_t)sh.lmax * sh.nvmax;  // scalars
  float *d32 = reinterpret_cast<float *>(scal + 8);  // FP32 copies of d and e^2
  float *e232 = d32 + sh.lmax;
  // the eigenvectors needed: r, or REST when the basis may be collapsed
  const bool may_restart = (m + r > L) && (m > D.rest);
  const int nv = min(m, may_restart ? max(D.rest, r) : r);
  const int ne = min(m, max(nv, r + 1));
  const double *Sb = Spool + D.soff;
  for (int idx = tid; idx < m * m; idx += EIG_T) {
    const int i = idx % m, j = idx / m;
    if (i >= j) A[(size_t)j * lda + i] = Sb[(size_t)j * L + i];
  }
  __syncthreads();
  // Householder tridiagonalisation (Golub & Van Loan, Alg. 8.3.1). GB300
  // spends the same FP64 issue slots on a warp instruction whatever its
  // active lanes, so the steps are laid out to keep lanes busy: one thread
  // per row for p = A22 v, and the rank-2 update over the packed lower
  // triangle only.
  for (int k = 0; k + 2 < m; ++k) {
    const int o = k + 1, mm = m - k - 1;
    double *xk = A + (size_t)k * lda + o;
    if (warp == 0) {
      double sig = 0.0;
      for (int i = 1 + lane; i < mm; i += 32) sig = fma(xk[i], xk[i], sig);
      sig = warp_sum(sig);
      if (lane == 0) {
        const double x0 = xk[0];
        dd[k] = A[(size_t)k * lda + k];
        if (sig == 0.0) {
          ee[k] = x0;
          bt[k] = 0.0;
          scal[0] = 1.0;
        } else {
          const double mu = sqrt(x0 * x0 + sig);
          const double v0 = (x0 <= 0.0) ? x0 - mu : -sig / (x0 + mu);
          ee[k] = mu;
          bt[k] = 2.0 * v0 * v0 / (sig + v0 * v0);
          scal[0] = 1.0 / v0;
        }
      }
    }
    __syncthreads();
    const double beta = bt[k];
    if (beta == 0.0) continue;
    const double rv0 = scal[0];
    for (int i = tid; i < mm; i += EIG_T) {
      const double v = (i == 0) ? 1.0 : xk[i] * rv0;
      vv[i] = v;
      if (i > 0) xk[i] = v;  // kept for the back-transformation
    }
    __syncthreads();
    // p = beta A22 v, one thread per row
    for (int i = tid; i < mm; i += EIG_T) {
      const double *row = A + (size_t)o * lda + (o + i);  // A(o+i, o+j), j <= i, at row[j * lda]
      const double *col = A + (size_t)(o + i) * lda + o;  // A(o+j, o+i), j >= i, at col[j]
      double s0 = 0.0, s1 = 0.0;
      int j = 0;
      for (; j + 1 < i; j += 2) {
        s0 = fma(row[(size_t)j * lda], vv[j], s0);
        s1 = fma(row[(size_t)(j + 1) * lda], vv[j + 1], s1);
      }
      for (; j < i; ++j) s0 = fma(row[(size_t)j * lda], vv[j], s0);
      for (j = i; j + 1 < mm; j += 2) {
        s0 = fma(col[j], vv[j], s0);
        s1 = fma(col[j + 1], vv[j + 1], s1);
      }
      for (; j < mm; ++j) s0 = fma(col[j], vv[j], s0);
      pp[i] = beta * (s0 + s1);
    }
    __syncthreads();
    if (warp == 0) {
      double pv = 0.0;
      for (int i = lane; i < mm; i += 32) pv = fma(pp[i], vv[i], pv);
      pv = warp_sum(pv);
      if (lane == 0) scal[1] = 0.5 * beta * pv;
    }
    __syncthreads();
    {
      const double half = scal[1];
      for (int i = tid; i < mm; i += EIG_T) pp[i] = fma(-half, vv[i], pp[i]);
    }
    __syncthreads();
    // A22 -= v w^T + w v^T on the lower triangle, packed index t -> (i >= j)
    const int ntri = mm * (mm + 1) / 2;
    for (int t = tid; t < ntri; t += EIG_T) {
      int i = (int)((sqrtf(8.0f * (float)t + 1.0f) - 1.0f) * 0.5f);
      while (i * (i + 1) / 2 > t) --i;
      while ((i + 1) * (i + 2) / 2 <= t) ++i;
      const int j = t - i * (i + 1) / 2;
      double &a = A[(size_t)(o + j) * lda + (o + i)];
      a = fma(-vv[i], pp[j], fma(-pp[i], vv[j], a));
    }
    __syncthreads();
  }
  if (tid == 0) {
    if (m >= 2) {
      dd[m - 2] = A[(size_t)(m - 2) * lda + (m - 2)];
      ee[m - 2] = A[(size_t)(m - 2) * lda + (m - 1)];
    }
    dd[m - 1] = A[(size_t)(m - 1) * lda + (m - 1)];
  }
  __syncthreads();
  if (warp == 0) {  // norms and Gershgorin bounds; FP32 copies for the coarse search
    double tn = 0.0, em = 0.0, glo = 1e308, ghi = -1e308;
    for (int i = lane; i < m; i += 32) {
      const double el = (i > 0) ? fabs(ee[i - 1]) : 0.0, er = (i + 1 < m) ? fabs(ee[i]) : 0.0;
      glo = fmin(glo, dd[i] - el - er);
      ghi = fmax(ghi, dd[i] + el + er);
      tn = fmax(tn, fabs(dd[i]) + el + er);
      if (i + 1 < m) {
        e2[i] = ee[i] * ee[i];
        em = fmax(em, e2[i]);
        e232[i] = (float)e2[i];
      }
      d32[i] = (float)dd[i];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      tn = fmax(tn, __shfl_xor_sync(0xffffffffu, tn, o));
      em = fmax(em, __shfl_xor_sync(0xffffffffu, em, o));
      glo = fmin(glo, __shfl_xor_sync(0xffffffffu, glo, o));
      ghi = fmax(ghi, __shfl_xor_sync(0xffffffffu, ghi, o));
    }
    if (lane == 0) {
      scal[2] = tn;
      scal[3] = em;
      scal[4] = glo;
      scal[5] = ghi;
    }
  }
  __syncthreads();
  // lowest ne eigenvalues, one lane per target (warps take 32 targets each).
  // 1. FP32 bisection on Sturm counts of the FP32 copy of T, inside the
  //    bracket from Cauchy interlacing: the leading mprev x mprev block of S
  //    is the matrix of the previous pass (or, after a restart, diag(theta)),
  //    whose eigenvalues are in theta, so with k = m - mprev new columns
  //    theta_old[j - k] <= lambda_j <= theta_old[j].
  // 2. FP64: the bracket lambda32 +- delta (delta covers the FP32 copy's
  //    perturbation) is checked by two FP64 counts, then bisection until
  //    isolated and safeguarded Newton steps on det(T - xI).
  {
    const double eps = 2.220446049250313e-16;
    const double tnorm = scal[2];
    const double pivmin = 2.2250738585072014e-308 * fmax(1.0, scal[3]) / eps;
    const double pad = 2.0 * eps * m * fmax(tnorm, 1e-300) + 2.0 * pivmin;
    const double atol = 4.0 * eps * fmax(tnorm, 1e-300);
    const double gl = scal[4] - pad, gu = scal[5] + pad;
    const int kadd = (S.mprev > 0 && m >= S.mprev) ? m - S.mprev : m;
    const int neold = (S.mprev > 0 && m >= S.mprev) ? S.neold : 0;
    const float eps32 = 5.9604645e-08f;
    const float piv32 = 1e-30f * fmaxf(1.0f, (float)scal[3]);
    for (int j = tid; j < ne; j += EIG_T) {
      // 1. coarse FP32 search
      double blo = gl, bhi = gu;
      {
        const double bl = (j - kadd >= 0 && j - kadd < neold) ? S.theta[j - kadd] - 8.0 * pad : gl;
        const double bh = (j < neold) ? S.theta[j] + 8.0 * pad : gu;
        if (fmax(gl, bl) < fmin(gu, bh)) {
          blo = fmax(gl, bl);
          bhi = fmin(gu, bh);
        }
      }
      const float tol32 = 8.0f * eps32 * fmaxf((float)tnorm, 1e-30f);
      float lo = (float)blo, hi = (float)bhi;
      if (sturm32(m, d32, e232, lo, piv32) > j) lo = (float)gl;  // hint did not hold
      if (sturm32(m, d32, e232, hi, piv32) <= j) hi = (float)gu;
      for (int it = 0; it < 80 && hi - lo > tol32; ++it) {
        const float x = 0.5f * (lo + hi);
        if (sturm32(m, d32, e232, x, piv32) <= j) lo = x;
        else hi = x;
      }
      // 2. FP64 refinement in lambda32 +- delta: verify both ends (a failed
      // end is replaced by the Gershgorin bound), then bisect until lambda_j
      // is isolated and take safeguarded Newton steps
      const double l32 = 0.5 * ((double)lo + (double)hi);
      const double delta = 64.0 * (double)eps32 * m * fmax(tnorm, 1e-300);
      double dlo = fmax(gl, l32 - delta), dhi = fmin(gu, l32 + delta), fpf;
      int clo = 0, chi = m;
      if (dlo > gl) {
        const int c = sturm64(m, dd, e2, dlo, pivmin, &fpf);
        if (c <= j) {
          clo = c;
        } else {  // lambda_j < dlo
          dhi = dlo;
          chi = c;
          dlo = gl;
        }
      }
      if (dhi < gu && chi == m) {
        const int c = sturm64(m, dd, e2, dhi, pivmin, &fpf);
        if (c > j) {
          chi = c;
        } else {  // lambda_j >= dhi
          dlo = dhi;
          clo = c;
          dhi = gu;
        }
      }
      bool newton = clo == j && chi == j + 1;  // already isolated: Newton from the FP32 estimate
      double xj = (l32 > dlo && l32 < dhi) ? l32 : 0.5 * (dlo + dhi), w = 0.5 * (dlo + dhi);
      for (int it = 0; it < 200; ++it) {
        const double x = newton ? xj : 0.5 * (dlo + dhi);
        const int cnt = sturm64(m, dd, e2, x, pivmin, &fpf);
        if (cnt <= j) {
          dlo = x;
          clo = cnt;
        } else {
          dhi = x;
          chi = cnt;
        }
        bool done = dhi - dlo <= atol + 2.0 * eps * fmax(fabs(dlo), fabs(dhi));
        if (!done && !newton && clo == j && chi == j + 1) {
          newton = true;  // isolated: Newton from the FP32 estimate
          xj = (l32 > dlo && l32 < dhi) ? l32 : 0.5 * (dlo + dhi);
        } else if (!done && newton) {
          const double step = (fpf != 0.0) ? -1.0 / fpf : 0.0;
          const double xn = x + step;
          if (fabs(step) <= 2.0 * eps * fabs(x) + pivmin) {
            done = true;
            xj = (xn > dlo && xn < dhi) ? xn : x;
          } else {
            xj = (xn > dlo && xn < dhi) ? xn : 0.5 * (dlo + dhi);
          }
        }
        w = newton ? xj : 0.5 * (dlo + dhi);
        if (done) break;
      }
      ev[j] = w;
    }
  }
  __syncthreads();
  if (tid == 0)
    for (int j = 1; j < ne; ++j) ev[j] = fmax(ev[j], ev[j - 1]);
  __syncthreads();
  // eigenvectors of T: clusters (consecutive eigenvalues closer than
  // 1e-3 |T|) are done by one thread in order, each vector orthogonalised
  // against the earlier ones of its cluster
  {
    const double eps = 2.220446049250313e-16;
    const double tnorm = scal[2], ortol = 1e-3 * tnorm;
    for (int j = tid; j < nv; j += EIG_T) {
      if (j > 0 && ev[j] - ev[j - 1] <= ortol) continue;  // not the first of its cluster
      int cl[MAXL];
      int ncl = 0;
      double prev = 0.0;
      for (int jj = j; jj < nv; ++jj) {
        if (jj > j && ev[jj] - ev[jj - 1] > ortol) break;
        double lam = ev[jj];
        if (jj > j && lam - prev < 10.0 * eps * fabs(lam)) lam = prev + 10.0 * eps * fabs(lam);
        inv_iter_dev(m, dd, ee, lam, tnorm, Z + (size_t)jj * m, Z, m, cl, ncl, (unsigned)jj + 1u);
        cl[ncl++] = jj;
        prev = lam;
      }
    }
  }
  __syncthreads();
  // back-transformation y = H_0 H_1 ... H_{m-3} z: per reflector, one warp
  // per vector for the dot products, then all threads for the update
  for (int k = m - 3; k >= 0; --k) {
    const double beta = bt[k];
    if (beta == 0.0) continue;
    const int o = k + 1, mm = m - k - 1;
    const double *vk = A + (size_t)k * lda + o;  // vk[0] is implicitly 1
    for (int c = warp; c < nv; c += EIG_T / 32) {
      const double *zc = Z + (size_t)c * m + o;
      double s0 = 0.0;
      for (int i = lane; i < mm; i += 32) s0 = fma((i == 0) ? 1.0 : vk[i], zc[i], s0);
      s0 = warp_sum(s0);
      if (lane == 0) pp[c] = beta * s0;
    }
    __syncthreads();
    for (int idx = tid; idx < mm * nv; idx += EIG_T) {
      const int i = idx % mm, c = idx / mm;
      Z[(size_t)c * m + o + i] -= pp[c] * ((i == 0) ? 1.0 : vk[i]);
    }
    __syncthreads();
  }
  double *Yb = Ypool + D.soff;
  for (int idx = tid; idx < m * nv; idx += EIG_T) {
    const int i = idx % m, c = idx / m;
    Yb[(size_t)c * L + i] = Z[(size_t)c * m + i];
  }
  for (int j = tid; j < ne; j += EIG_T) S.theta[j] = ev[j];
  if (tid == 0) {
    S.nv = nv;
    S.mprev = m;
    S.neold = ne;
  }
}

// ---------------------------------------------------------------------------
// Tall-skinny kernels over row tiles of all blocks.
// ---------------------------------------------------------------------------

// One thread per row: x_j = V(i, 0:m) y_j, u_j = W(i, 0:m) y_j, the residual
// u_j - theta_j x_j, and the tile's |R_j|^2 partials in a fixed order. NR is
// r rounded up to an instantiated size; GB300 issues FP64 slowly, so no FMA
// is spent on unused columns.
template <int NR>
__device__ __forceinline__ void ritz_rows(const BDesc &D, const BTile &T, const BState &S, bool row,
                                          const double *__restrict__ V, const double *__restrict__ W,
                                          const double *Ys, double *__restrict__ X, double *__restrict__ R,
                                          double *red, double *__restrict__ part, int r) {
  const int m = S.m, n = D.n, i = T.r0 + threadIdx.x;
  double x[NR], u[NR];
#pragma unroll
  for (int j = 0; j < NR; ++j) x[j] = u[j] = 0.0;
  if (row) {
    const double *Vi = V + D.voff + i, *Wi = W + D.voff + i;
#pragma unroll 4
    for (int k = 0; k < m; ++k) {
      const double v = Vi[(size_t)k * n], w = Wi[(size_t)k * n];
#pragma unroll
      for (int j = 0; j < NR; ++j)
        if (j < r) {
          x[j] = fma(v, Ys[k * r + j], x[j]);
          u[j] = fma(w, Ys[k * r + j], u[j]);
        }
    }
  }
#pragma unroll
  for (int j = 0; j < NR; ++j) {
    if (j >= r) break;
    double res = 0.0;
    if (row) {
      res = fma(-S.theta[j], x[j], u[j]);
      X[D.xoff + (size_t)j * n + i] = x[j];
      R[D.xoff + (size_t)j * n + i] = res;
    }
    red[threadIdx.x] = res * res;
    __syncthreads();
    for (int h = RT / 2; h > 0; h >>= 1) {
      if (threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
      __syncthreads();
    }
    if (threadIdx.x == 0) part[j] = red[0];
    __syncthreads();
  }
}

// Ritz vectors and residuals of the r targets, |R_j|^2 partials per tile
__global__ void __launch_bounds__(RT) k_b_ritz(const BTile *__restrict__ tiles, const BDesc *__restrict__ desc,
                                               const BState *__restrict__ st, const double *__restrict__ V,
                                               const double *__restrict__ W, const double *__restrict__ Ypool,
                                               double *__restrict__ X, double *__restrict__ R,
                                               double *__restrict__ part, int ps) {
  const BTile T = tiles[blockIdx.x];
  const BState &S = st[T.b];
  if (!S.active) return;
  const BDesc D = desc[T.b];
  const int m = S.m, r = D.r, L = D.lim;
  __shared__ double Ys[MAXL * MAXR];
  __shared__ double red[RT];
  const double *Yb = Ypool + D.soff;
  for (int idx = threadIdx.x; idx < m * r; idx += RT) {
    const int k = idx / r, j = idx % r;
    Ys[idx] = Yb[(size_t)j * L + k];  // Ys[k * r + j]
  }
  __syncthreads();
  const bool row = threadIdx.x < T.nr;
  switch (r) {
    case 1: ritz_rows<1>(D, T, S, row, V, W, Ys, X, R, red, part + (size_t)blockIdx.x * ps, r); break;
    case 2: ritz_rows<2>(D, T, S, row, V, W, Ys, X, R, red, part + (size_t)blockIdx.x * ps, r); break;
    case 3: ritz_rows<3>(D, T, S, row, V, W, Ys, X, R, red, part + (size_t)blockIdx.x * ps, r); break;
    case 4: ritz_rows<4>(D, T, S, row, V, W, Ys, X, R, red, part + (size_t)blockIdx.x * ps, r); break;
    case 5:
    case 6: ritz_rows<6>(D, T, S, row, V, W, Ys, X, R, red, part + (size_t)blockIdx.x * ps, r); break;
    case 7:
    case 8: ritz_rows<8>(D, T, S, row, V, W, Ys, X, R, red, part + (size_t)blockIdx.x * ps, r); break;
    default: ritz_rows<MAXR>(D, T, S, row, V, W, Ys, X, R, red, part + (size_t)blockIdx.x * ps, r); break;
  }
}

// per block: residual norms, convergence, the targets that get new vectors,
// and the restart decision. A block whose basis spans its whole space
// (m = n) is converged: its Ritz pairs are exact up to rounding.
__global__ void k_b_conv(const BDesc *__restrict__ desc, BState *__restrict__ st, const double *__restrict__ part,
                         int ps, int nb, double critr, int *__restrict__ nactive) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nb) return;
  BState &S = st[b];
  if (!S.active) return;
  const BDesc D = desc[b];
  int nun = 0;
  for (int j = 0; j < D.r; ++j) {
    double s = 0.0;
    for (int t = 0; t < D.ntile; ++t) s += part[(size_t)(D.tile0 + t) * ps + j];
    S.rn[j] = sqrt(s);
    if (!(S.rn[j] <= critr) && S.m < D.n) S.newt[nun++] = j;
  }
  S.iters += 1;
  S.restart = 0;
  S.ncur = 0;
  if (nun == 0) {
    S.active = 0;
    return;
  }
  if (S.iters >= D.maxiter) {
    S.ierr |= 2048;  // DVDSON's "maximum number of iterations" bit
    S.active = 0;
    return;
  }
  int m = S.m;
  if (m + nun > D.lim && m > D.rest && S.nv >= D.rest) {
    S.restart = 1;
    m = D.rest;
  }
  nun = min(nun, D.lim - m);
  if (nun <= 0) {
    S.ierr |= 2048;
    S.active = 0;
    return;
  }
  S.ncur = nun;
  atomicAdd(nactive, 1);
}

// basis collapse: V(:, 1:REST) = V(:, 1:m) Y(:, 1:REST), the same for W;
// rows are staged RG at a time so that the update is in place
__global__ void __launch_bounds__(BT) k_b_restart(const BTile *__restrict__ tiles, const BDesc *__restrict__ desc,
                                                  const BState *__restrict__ st, double *__restrict__ V,
                                                  double *__restrict__ W, const double *__restrict__ Ypool) {
  extern __shared__ double sm[];
  const BTile T = tiles[blockIdx.x];
  const BState &S = st[T.b];
  if (!S.active || !S.restart) return;
  const BDesc D = desc[T.b];
  const int m = S.m, rest = D.rest, n = D.n, L = D.lim;
  double *Ys = sm;                   // [k][rest]
  double *Rs = sm + (size_t)m * rest;  // [g][m]
  const double *Yb = Ypool + D.soff;
  for (int idx = threadIdx.x; idx < m * rest; idx += BT) {
    const int k = idx / rest, c = idx % rest;
    Ys[idx] = Yb[(size_t)c * L + k];
  }
  __syncthreads();
  for (int pass = 0; pass < 2; ++pass) {
    double *base = (pass ? W : V) + D.voff;
    for (int g0 = 0; g0 < T.nr; g0 += RG) {
      const int ng = min(RG, T.nr - g0);
      for (int idx = threadIdx.x; idx < ng * m; idx += BT) {
        const int g = idx % ng, k = idx / ng;
        Rs[g * m + k] = base[(size_t)k * n + T.r0 + g0 + g];
      }
      __syncthreads();
      for (int idx = threadIdx.x; idx < ng * rest; idx += BT) {
        const int g = idx % ng, c = idx / ng;
        double s0 = 0.0, s1 = 0.0;
        int k = 0;
        for (; k + 1 < m; k += 2) {
          s0 = fma(Rs[g * m + k], Ys[k * rest + c], s0);
          s1 = fma(Rs[g * m + k + 1], Ys[(k + 1) * rest + c], s1);
        }
        if (k < m) s0 = fma(Rs[g * m + k], Ys[k * rest + c], s0);
        base[(size_t)c * n + T.r0 + g0 + g] = s0 + s1;
      }
      __syncthreads();
    }
  }
}

// after the collapse: S = diag(theta_1..REST), m = REST
__global__ void k_b_restart_fin(const BDesc *__restrict__ desc, BState *__restrict__ st, double *__restrict__ Spool) {
  const int b = blockIdx.x;
  BState &S = st[b];
  if (!S.active || !S.restart) return;
  const BDesc D = desc[b];
  const int rest = D.rest, L = D.lim;
  double *Sb = Spool + D.soff;
  for (int idx = threadIdx.x; idx < rest * rest; idx += blockDim.x) {
    const int i = idx % rest, j = idx / rest;
    Sb[(size_t)j * L + i] = (i == j) ? S.theta[i] : 0.0;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    S.m = rest;
    S.restart = 0;
    S.mprev = rest;  // S's leading block is now diag(theta_1..REST)
    S.neold = rest;
  }
}

// new vectors from the residuals of the unconverged targets
__global__ void __launch_bounds__(RT) k_b_precond(const BTile *__restrict__ tiles, const BDesc *__restrict__ desc,
                                                  const BState *__restrict__ st, double *__restrict__ V,
                                                  const double *__restrict__ R) {
  const BTile T = tiles[blockIdx.x];
  const BState &S = st[T.b];
  if (!S.active || threadIdx.x >= T.nr) return;
  const BDesc D = desc[T.b];
  const int i = T.r0 + threadIdx.x, n = D.n, m = S.m;
  const double di = D.diag[i];
  for (int q = 0; q < S.ncur; ++q) {
    const int j = S.newt[q];
    const double rr = R[D.xoff + (size_t)j * n + i];
    const double d = di - S.theta[j];
    V[D.voff + (size_t)(m + q) * n + i] = (fabs(d) > 1.0e-06) ? rr / d : rr * 1.0e06;
  }
}

// dot products of column sets, one partial per tile:
//   MODE 0  V(:, 0:m)^T V(:, m:m+c), plus the squared norms of the new columns
//   MODE 1  V(:, m:m+c)^T V(:, m:m+c)
//   MODE 2  V(:, 0:m+c)^T W(:, m:m+c)
// part[tile][a * c + q]; the new columns are staged in shared memory, the
// others AC at a time; one thread per (a, q) sums the tile's rows in order.
template <int MODE>
__global__ void __launch_bounds__(BT) k_b_dots(const BTile *__restrict__ tiles, const BDesc *__restrict__ desc,
                                               const BState *__restrict__ st, const double *__restrict__ V,
                                               const double *__restrict__ W, double *__restrict__ part, int ps) {
  extern __shared__ double sm[];
  const BTile T = tiles[blockIdx.x];
  const BState &S = st[T.b];
  if (!S.active) return;
  const int nb = S.ncur;
  if (nb <= 0) return;
  const BDesc D = desc[T.b];
  const int m = S.m, n = D.n, nr = T.nr;
  const int na = (MODE == 0) ? m : (MODE == 1 ? nb : m + nb);
  const int a0 = (MODE == 1) ? m : 0;
  double *Bs = sm;                  // [i][MAXR]
  double *As = sm + TR * MAXR;      // [i][AC + 1]
  const double *Bbase = ((MODE == 2) ? W : V) + D.voff + (size_t)m * n + T.r0;
  const double *Abase = V + D.voff + (size_t)a0 * n + T.r0;
  double *out = part + (size_t)blockIdx.x * ps;
  for (int idx = threadIdx.x; idx < nr * nb; idx += BT) {
    const int i = idx % nr, q = idx / nr;
    Bs[i * MAXR + q] = Bbase[(size_t)q * n + i];
  }
  __syncthreads();
  for (int ac = 0; ac < na; ac += AC) {
    const int nac = min(AC, na - ac);
    for (int idx = threadIdx.x; idx < nr * nac; idx += BT) {
      const int i = idx % nr, a = idx / nr;
      As[i * (AC + 1) + a] = Abase[(size_t)(ac + a) * n + i];
    }
    __syncthreads();
    for (int pr = threadIdx.x; pr < nac * nb; pr += BT) {
      const int a = pr % nac, q = pr / nac;
      double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
      int i = 0;
      for (; i + 3 < nr; i += 4) {
        s0 = fma(As[i * (AC + 1) + a], Bs[i * MAXR + q], s0);
        s1 = fma(As[(i + 1) * (AC + 1) + a], Bs[(i + 1) * MAXR + q], s1);
        s2 = fma(As[(i + 2) * (AC + 1) + a], Bs[(i + 2) * MAXR + q], s2);
        s3 = fma(As[(i + 3) * (AC + 1) + a], Bs[(i + 3) * MAXR + q], s3);
      }
      for (; i < nr; ++i) s0 = fma(As[i * (AC + 1) + a], Bs[i * MAXR + q], s0);
      out[(ac + a) * nb + q] = (s0 + s1) + (s2 + s3);
    }
    __syncthreads();
  }
  if (MODE == 0)
    for (int q = threadIdx.x; q < nb; q += BT) {
      double s0 = 0.0, s1 = 0.0;
      int i = 0;
      for (; i + 1 < nr; i += 2) {
        s0 = fma(Bs[i * MAXR + q], Bs[i * MAXR + q], s0);
        s1 = fma(Bs[(i + 1) * MAXR + q], Bs[(i + 1) * MAXR + q], s1);
      }
      if (i < nr) s0 = fma(Bs[i * MAXR + q], Bs[i * MAXR + q], s0);
      out[na * nb + q] = s0 + s1;
    }
}

// per block: the tile partials added in tile order, then
//   MODE 0  C = the Gram-Schmidt coefficients (first pass: norms kept in nrm0)
//   MODE 1  Cholesky of the new columns' Gram matrix, dropping columns whose
//           pivot is below (1e-8 x reference norm)^2; C = the nprev x ncur
//           matrix that maps the old new columns to the kept orthonormal ones
//   MODE 2  the new columns of S (mirrored), m += ncur
template <int MODE>
__global__ void __launch_bounds__(256) k_b_colsum(const BDesc *__restrict__ desc, BState *__restrict__ st,
                                                  const double *__restrict__ part, int ps, double *__restrict__ Spool,
                                                  double *__restrict__ Cpool, int first) {
  __shared__ double buf[(MAXL + 1) * MAXR];
  const int b = blockIdx.x;
  BState &S = st[b];
  if (!S.active) return;
  const int nb = S.ncur;
  if (nb <= 0) return;
  const BDesc D = desc[b];
  const int m = S.m, L = D.lim;
  const int na = (MODE == 0) ? m + 1 : (MODE == 1 ? nb : m + nb);
  for (int pr = threadIdx.x; pr < na * nb; pr += blockDim.x) {
    double s = 0.0;
    for (int t = 0; t < D.ntile; ++t) s += part[(size_t)(D.tile0 + t) * ps + pr];
    buf[pr] = s;
  }
  __syncthreads();
  double *C = Cpool + D.coff;
  if (MODE == 0) {
    for (int pr = threadIdx.x; pr < m * nb; pr += blockDim.x) C[pr] = buf[pr];
    if (first)
      for (int q = threadIdx.x; q < nb; q += blockDim.x) S.nrm0[q] = sqrt(buf[m * nb + q]);
  } else if (MODE == 1) {
    if (threadIdx.x == 0) {
      double Rm[MAXR][MAXR];
      int keep[MAXR];
      int nk = 0;
      for (int q = 0; q < nb; ++q) {
        double rq[MAXR];
        double dq = buf[q * nb + q];
        for (int c = 0; c < nk; ++c) {
          const int p = keep[c];
          double v = buf[p * nb + q];
          for (int c2 = 0; c2 < c; ++c2) v -= Rm[c2][c] * rq[c2];
          rq[c] = v / Rm[c][c];
          dq -= rq[c] * rq[c];
        }
        const double ref = first ? S.nrm0[q] : 1.0;
        const double thr = 1e-16 * ref * ref;
        if (dq > thr && dq > 1e-280) {
          for (int c = 0; c < nk; ++c) Rm[c][nk] = rq[c];
          Rm[nk][nk] = sqrt(dq);
          keep[nk++] = q;
        }
      }
      // C[q][c]: column c of the kept orthonormal set in terms of the inputs
      for (int q = 0; q < nb; ++q)
        for (int c = 0; c < MAXR; ++c) C[q * MAXR + c] = 0.0;
      for (int c = 0; c < nk; ++c) {
        double inv[MAXR];  // column c of R^{-1}
        for (int i = 0; i < nk; ++i) inv[i] = 0.0;
        inv[c] = 1.0 / Rm[c][c];
        for (int i = c - 1; i >= 0; --i) {
          double s = 0.0;
          for (int l = i + 1; l <= c; ++l) s += Rm[i][l] * inv[l];
          inv[i] = -s / Rm[i][i];
        }
        for (int i = 0; i <= c; ++i) C[keep[i] * MAXR + c] = inv[i];
      }
      S.nprev = nb;
      S.ncur = nk;
      if (nk == 0) {
        S.ierr |= 2048;
        S.active = 0;
      }
    }
  } else {
    double *Sb = Spool + D.soff;
    for (int pr = threadIdx.x; pr < na * nb; pr += blockDim.x) {
      const int a = pr / nb, q = pr % nb;
      if (a >= m && a > m + q) continue;  // the new-new block: upper half only, mirrored
      const double v = buf[pr];
      Sb[(size_t)(m + q) * L + a] = v;
      Sb[(size_t)a * L + (m + q)] = v;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      S.m = m + nb;
      S.nmv += nb;
      S.ncur = 0;
    }
  }
}

// one row of V(:, m+q) -= V(:, 0:m) C(:, q), q < nb <= NB
template <int NB>
__device__ __forceinline__ void sub_row(double *Vi, int m, int n, const double *Cs, int nb) {
  double acc[NB];
#pragma unroll
  for (int q = 0; q < NB; ++q) acc[q] = 0.0;
#pragma unroll 4
  for (int a = 0; a < m; ++a) {
    const double v = Vi[(size_t)a * n];
#pragma unroll
    for (int q = 0; q < NB; ++q)
      if (q < nb) acc[q] = fma(v, Cs[a * nb + q], acc[q]);
  }
#pragma unroll
  for (int q = 0; q < NB; ++q)
    if (q < nb) Vi[(size_t)(m + q) * n] -= acc[q];
}

// new columns minus their projections: V(:, m+q) -= V(:, 0:m) C(:, q)
__global__ void __launch_bounds__(RT) k_b_sub(const BTile *__restrict__ tiles, const BDesc *__restrict__ desc,
                                              const BState *__restrict__ st, double *__restrict__ V,
                                              const double *__restrict__ Cpool) {
  __shared__ double Cs[MAXL * MAXR];
  const BTile T = tiles[blockIdx.x];
  const BState &S = st[T.b];
  if (!S.active) return;
  const int nb = S.ncur;
  if (nb <= 0) return;
  const BDesc D = desc[T.b];
  const int m = S.m, n = D.n;
  const double *C = Cpool + D.coff;
  for (int idx = threadIdx.x; idx < m * nb; idx += RT) Cs[idx] = C[idx];
  __syncthreads();
  if (threadIdx.x >= T.nr) return;
  double *Vi = V + D.voff + T.r0 + threadIdx.x;
  switch (nb) {
    case 1: sub_row<1>(Vi, m, n, Cs, nb); break;
    case 2: sub_row<2>(Vi, m, n, Cs, nb); break;
    case 3: sub_row<3>(Vi, m, n, Cs, nb); break;
    case 4: sub_row<4>(Vi, m, n, Cs, nb); break;
    case 5:
    case 6: sub_row<6>(Vi, m, n, Cs, nb); break;
    case 7:
    case 8: sub_row<8>(Vi, m, n, Cs, nb); break;
    default: sub_row<MAXR>(Vi, m, n, Cs, nb); break;
  }
}

// kept orthonormal new columns: V(:, m+c) = sum_q V_old(:, m+q) C[q][c]
__global__ void __launch_bounds__(RT) k_b_apply(const BTile *__restrict__ tiles, const BDesc *__restrict__ desc,
                                                const BState *__restrict__ st, double *__restrict__ V,
                                                const double *__restrict__ Cpool) {
  __shared__ double Cs[MAXR * MAXR];
  const BTile T = tiles[blockIdx.x];
  const BState &S = st[T.b];
  if (!S.active) return;
  const int np = S.nprev, nc = S.ncur;
  if (np <= 0) return;
  const BDesc D = desc[T.b];
  const int m = S.m, n = D.n;
  const double *C = Cpool + D.coff;
  for (int idx = threadIdx.x; idx < MAXR * MAXR; idx += RT) Cs[idx] = (idx < np * MAXR) ? C[idx] : 0.0;
  __syncthreads();
  if (threadIdx.x >= T.nr) return;
  double *Vi = V + D.voff + T.r0 + threadIdx.x;
  double x[MAXR];
#pragma unroll
  for (int q = 0; q < MAXR; ++q) x[q] = (q < np) ? Vi[(size_t)(m + q) * n] : 0.0;
#pragma unroll
  for (int c = 0; c < MAXR; ++c) {
    if (c >= nc) break;
    double s = 0.0;
#pragma unroll
    for (int q = 0; q < MAXR; ++q)
      if (q < np) s = fma(x[q], Cs[q * MAXR + c], s);
    Vi[(size_t)(m + c) * n] = s;
  }
}

// row-major copies of the new columns for the matvec gathers: FP64, or the
// hi + lo FP32 split
template <bool SPLIT>
__global__ void __launch_bounds__(RT) k_b_gatherx(const BTile *__restrict__ tiles, const BDesc *__restrict__ desc,
                                                  const BState *__restrict__ st, const double *__restrict__ V,
                                                  double *__restrict__ XD, float2 *__restrict__ XS) {
  const BTile T = tiles[blockIdx.x];
  const BState &S = st[T.b];
  if (!S.active || threadIdx.x >= T.nr) return;
  const int nc = S.ncur;
  if (nc <= 0) return;
  const BDesc D = desc[T.b];
  const int i = T.r0 + threadIdx.x, n = D.n, m = S.m;
  const size_t g = (size_t)(D.row0 + i) * MAXR;
  for (int q = 0; q < nc; ++q) {
    const double v = V[D.voff + (size_t)(m + q) * n + i];
    if (SPLIT) {
      const float h = __double2float_rn(v);
      XS[g + q] = make_float2(h, __double2float_rn(v - (double)h));
    } else {
      XD[g + q] = v;
    }
  }
}

// double-float helpers (Dekker / Knuth error-free transformations). This file
// is compiled with FMA contraction on (its FP64 loops want it), so every step
// of the error-free sums uses the _rn intrinsics, which are never contracted.
struct dfl {
  float h, l;
};
__device__ __forceinline__ dfl two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}
__device__ __forceinline__ dfl df_add(dfl a, dfl b) {
  dfl s = two_sum(a.h, b.h);
  const float t = __fadd_rn(__fadd_rn(s.l, a.l), b.l);
  const float h = __fadd_rn(s.h, t);
  return {h, __fsub_rn(t, __fsub_rn(h, s.h))};
}

// One row of W(:, m+q0 : m+q0+NQ) = H V(...): a warp over the row's entries,
// x gathered from shared memory (staged) or from the row-major copy. After
// the cross-lane sums every lane holds every column's total, and lane q
// finishes column q, so the FP64 epilogue is one warp instruction for all
// columns (GB300 charges FP64 issue per warp instruction).
template <int NQ>
__device__ __forceinline__ void spmm_row_split(const BDesc &D, int i, int64_t p0, int64_t p1, int m, int q0, int lane,
                                               bool staged, const X32 *__restrict__ smx,
                                               const char *__restrict__ gx, size_t gstride,
                                               const double *__restrict__ V, double *__restrict__ W) {
  const int n = D.n;
  float sh[NQ], sl[NQ];
#pragma unroll
  for (int q = 0; q < NQ; ++q) sh[q] = sl[q] = 0.f;
  auto add = [&](float ah, float al, int c) {
    const float2 *xr = staged ? reinterpret_cast<const float2 *>(smx + c)
                              : reinterpret_cast<const float2 *>(gx + c * gstride);
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      // Dot2 (Ogita, Rump & Oishi, SIAM J. Sci. Comput. 26 (2005) 1955): the
      // running sum takes each product's high part through an error-free
      // TwoSum; rounding errors and the products' low parts gather in sl
      const float2 x = xr[q];
      const float ph = __fmul_rn(ah, x.x);
      const float t = fmaf(ah, x.y, fmaf(al, x.x, fmaf(ah, x.x, -ph)));
      const float s = __fadd_rn(sh[q], ph);
      const float bb = __fsub_rn(s, sh[q]);
      const float err = __fadd_rn(__fsub_rn(sh[q], __fsub_rn(s, bb)), __fsub_rn(ph, bb));
      sh[q] = s;
      sl[q] = __fadd_rn(sl[q], __fadd_rn(err, t));
    }
  };
#pragma unroll 4
  for (int64_t p = p0 + lane; p < p1; p += 32)
    add(__ldg(D.hi + p), __ldg(D.lo + p), D.col16 ? (int)__ldg(D.col16 + p) : __ldg(D.col + p));
  float h = 0.f, l = 0.f;
#pragma unroll
  for (int q = 0; q < NQ; ++q) {
    dfl acc = two_sum(sh[q], sl[q]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      dfl other;
      other.h = __shfl_xor_sync(0xffffffffu, acc.h, o);
      other.l = __shfl_xor_sync(0xffffffffu, acc.l, o);
      acc = df_add(acc, other);
    }
    if (lane == q) {
      h = acc.h;
      l = acc.l;
    }
  }
  if (lane < NQ) {
    const size_t o = D.voff + (size_t)(m + q0 + lane) * n + i;
    W[o] = ((double)h + (double)l) + D.diag[i] * V[o];
  }
}

// FP64 form: one DFMA per entry and column; each column's sum is reduced
// across the warp and lane q writes column q.
template <int NQ>
__device__ __forceinline__ void spmm_row_fp64(const BDesc &D, int i, int64_t p0, int64_t p1, int m, int q0, int lane,
                                              bool staged, const X32 *__restrict__ smx,
                                              const char *__restrict__ gx, size_t gstride,
                                              double *__restrict__ W) {
  const int n = D.n;
  double acc[NQ];
#pragma unroll
  for (int q = 0; q < NQ; ++q) acc[q] = 0.0;
#pragma unroll 4
  for (int64_t p = p0 + lane; p < p1; p += 32) {
    const double v = __ldg(D.val + p);
    const int c = D.col16 ? (int)__ldg(D.col16 + p) : __ldg(D.col + p);
    const double *xr = staged ? reinterpret_cast<const double *>(smx + c)
                              : reinterpret_cast<const double *>(gx + c * gstride);
#pragma unroll
    for (int q = 0; q < NQ; ++q) acc[q] = fma(v, xr[q], acc[q]);
  }
  double t = 0.0;
#pragma unroll
  for (int q = 0; q < NQ; ++q) {
    const double sq = warp_sum(acc[q]);
    if (lane == q) t = sq;
  }
  if (lane < NQ) W[D.voff + (size_t)(m + q0 + lane) * n + i] = t;
}

// W(:, m:m+c) = H V(:, m:m+c) for every block. One CTA per row tile, one
// warp per row, up to four columns per pass over the row. The block's x
// values of those columns (FP64, or hi + lo FP32 pairs: 32 bytes per row) are
// staged in shared memory when the block has at most sx_rows rows, so the
// column gathers hit shared memory; larger blocks gather from the L2-resident
// row-major copy. FP64: one DFMA per entry and column. SPLIT: off-diagonal
// values as hi + lo FP32, double-float sums, the diagonal term in FP64.
template <bool SPLIT>
__global__ void __launch_bounds__(256) k_b_spmm(const BTile *__restrict__ tiles, const BDesc *__restrict__ desc,
                                                const BState *__restrict__ st, const double *__restrict__ V,
                                                double *__restrict__ W, const double *__restrict__ XD,
                                                const float2 *__restrict__ XS, int sx_rows) {
  extern __shared__ X32 smx[];
  const BTile T = tiles[blockIdx.x];
  const BState &S = st[T.b];
  if (!S.active) return;
  const int nc = S.ncur;
  if (nc <= 0) return;
  const BDesc D = desc[T.b];
  const int n = D.n, m = S.m, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const bool staged = n <= sx_rows;
  for (int q0 = 0; q0 < nc; q0 += 4) {
    const char *gx = SPLIT ? reinterpret_cast<const char *>(XS + (size_t)D.row0 * MAXR + q0)
                           : reinterpret_cast<const char *>(XD + (size_t)D.row0 * MAXR + q0);
    const size_t gstride = SPLIT ? MAXR * sizeof(float2) : MAXR * sizeof(double);
    if (staged) {
      __syncthreads();
      for (int r = threadIdx.x; r < n; r += blockDim.x) smx[r] = *reinterpret_cast<const X32 *>(gx + r * gstride);
      __syncthreads();
    }
    const int nq = min(4, nc - q0);
    const int step = blockDim.x / 32;
    int64_t p0 = 0, p1 = 0;
    if (warp < T.nr) {
      p0 = D.ptr[T.r0 + warp];
      p1 = D.ptr[T.r0 + warp + 1];
    }
    for (int rr = warp; rr < T.nr; rr += step) {
      const int i = T.r0 + rr;
      // the next row's bounds are fetched before this row's work
      int64_t n0 = 0, n1 = 0;
      if (rr + step < T.nr) {
        n0 = D.ptr[i + step];
        n1 = D.ptr[i + step + 1];
      }
      if (SPLIT) {
        switch (nq) {
          case 1: spmm_row_split<1>(D, i, p0, p1, m, q0, lane, staged, smx, gx, gstride, V, W); break;
          case 2: spmm_row_split<2>(D, i, p0, p1, m, q0, lane, staged, smx, gx, gstride, V, W); break;
          case 3: spmm_row_split<3>(D, i, p0, p1, m, q0, lane, staged, smx, gx, gstride, V, W); break;
          default: spmm_row_split<4>(D, i, p0, p1, m, q0, lane, staged, smx, gx, gstride, V, W); break;
        }
      } else {
        switch (nq) {
          case 1: spmm_row_fp64<1>(D, i, p0, p1, m, q0, lane, staged, smx, gx, gstride, W); break;
          case 2: spmm_row_fp64<2>(D, i, p0, p1, m, q0, lane, staged, smx, gx, gstride, W); break;
          case 3: spmm_row_fp64<3>(D, i, p0, p1, m, q0, lane, staged, smx, gx, gstride, W); break;
          default: spmm_row_fp64<4>(D, i, p0, p1, m, q0, lane, staged, smx, gx, gstride, W); break;
        }
      }
      p0 = n0;
      p1 = n1;
    }
  }
}

// unit start vectors e_p for the m0 listed rows of each block
__global__ void __launch_bounds__(RT) k_b_init(const BTile *__restrict__ tiles, const BDesc *__restrict__ desc,
                                               const int *__restrict__ pidx, double *__restrict__ V) {
  const BTile T = tiles[blockIdx.x];
  if (threadIdx.x >= T.nr) return;
  const BDesc D = desc[T.b];
  const int i = T.r0 + threadIdx.x;
  for (int k = 0; k < D.m0; ++k) V[D.voff + (size_t)k * D.n + i] = (pidx[D.pofs + k] == i) ? 1.0 : 0.0;
}

// start-up chunks: the next up to MAXR of the m0 start vectors become "new"
__global__ void k_b_setnew(const BDesc *__restrict__ desc, BState *__restrict__ st, int nb) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nb) return;
  BState &S = st[b];
  S.ncur = min(MAXR, desc[b].m0 - S.m);
}

}  // namespace

// ---------------------------------------------------------------------------
// Host driver
// ---------------------------------------------------------------------------
namespace {

// the batched matvec's tuned variant per batch shape, for this process
struct BatchTuneKey {
  int dev, nb, ntot;
  long long nnz;
  int prec;
  bool operator<(const BatchTuneKey &o) const {
    return std::tie(dev, nb, ntot, nnz, prec) < std::tie(o.dev, o.nb, o.ntot, o.nnz, o.prec);
  }
};
struct BatchTuneEntry {
  int variant = 3;
  double ms[SPMM_NVAR] = {};
};
std::mutex g_btune_mu;
std::map<BatchTuneKey, BatchTuneEntry> g_btune;

struct BatchRun {
  gg_ctx *ctx;
  int nb = 0, ntiles = 0, ntot = 0;
  int precision = GG_FP64;
  double critr = 1e-9;
  std::vector<BDesc> hd;
  std::vector<BTile> ht;
  EigShape eig{};
  size_t restart_smem = 0, dots_smem = 0;
  int sx_rows = 0;  // blocks up to this many rows stage x in shared memory
  int ps = 0;
  DBuf<BDesc> dDesc;
  DBuf<BState> dSt;
  DBuf<BTile> dTiles;
  // the batched matvec's own tiles, per autotuner variant: SPMM_TR[v / 2]
  // rows per CTA, SPMM_T[v % 2] threads; and each group's tile range in them
  std::vector<BTile> hsp_tiles[3];
  DBuf<BTile> dSpTiles[3];
  int sp_t0[3][3] = {}, sp_nt[3][3] = {};  // [tile size][all, group 0, group 1]
  int sp_var = 3;                          // 128 rows, 256 threads
  DBuf<int> dPidx, dNact;
  DBuf<double> V, W, X, R, Sp, Yp, Cp, part, XD;
  DBuf<float2> XS;
  int *hNact = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  int graph_kernels = 0;
  ~BatchRun() {
    if (gexec) cudaGraphExecDestroy(gexec);
    if (graph) cudaGraphDestroy(graph);
    if (hNact) cudaFreeHost(hNact);
    if (evFork) cudaEventDestroy(evFork);
    if (evJoin) cudaEventDestroy(evJoin);
    if (s2) cudaStreamDestroy(s2);
  }

  // a contiguous range of blocks and their tiles
  struct Group {
    int b0 = 0, nb = 0, t0 = 0, nt = 0;
  };
  Group all, grp[2];
  cudaStream_t s2 = nullptr;
  cudaEvent_t evFork = nullptr, evJoin = nullptr;

  // the kernels that add the new columns [m, m + ncur) to the basis: matvec
  // and S update
  int gidx(const Group &g) const { return &g == &all ? 0 : (&g == &grp[0] ? 1 : 2); }
  // W = H V for the new columns of the group's blocks with matvec variant v
  void launch_spmm(cudaStream_t s, const Group &g, int v) {
    const int ts = v / 2, gi = gidx(g), nt = sp_nt[ts][gi];
    if (nt == 0) return;
    const BTile *tl = dSpTiles[ts].p + sp_t0[ts][gi];
    const int thr = SPMM_T[v % 2];
    const size_t sx = (size_t)sx_rows * sizeof(X32);
    if (precision == GG_SPLIT)
      k_b_spmm<true><<<nt, thr, sx, s>>>(tl, dDesc.p, dSt.p, V.p, W.p, XD.p, XS.p, sx_rows);
    else
      k_b_spmm<false><<<nt, thr, sx, s>>>(tl, dDesc.p, dSt.p, V.p, W.p, XD.p, XS.p, sx_rows);
  }
  int enqueue_expand(cudaStream_t s, const Group &g, int *count, const cudaEvent_t *tune_ev = nullptr,
                     double *tune_ms = nullptr) {
    if (g.nb == 0) return GG_OK;
    const BTile *tl = dTiles.p + g.t0;
    const BDesc *de = dDesc.p + g.b0;
    BState *sb = dSt.p + g.b0;
    double *pt = part.p + (size_t)g.t0 * ps;
    if (precision == GG_SPLIT)
      k_b_gatherx<true><<<g.nt, RT, 0, s>>>(tl, dDesc.p, dSt.p, V.p, XD.p, XS.p);
    else
      k_b_gatherx<false><<<g.nt, RT, 0, s>>>(tl, dDesc.p, dSt.p, V.p, XD.p, XS.p);
    if (tune_ev) {
      // the autotuner: every variant computes the same W (each row is one
      // warp's whatever the tiles, and W is overwritten), so all run here,
      // each between events
      for (int v = 0; v < SPMM_NVAR; ++v) {
        GG_CUDA(cudaEventRecord(tune_ev[2 * v], s));
        launch_spmm(s, g, v);
        GG_CUDA(cudaEventRecord(tune_ev[2 * v + 1], s));
      }
      GG_CUDA(cudaEventSynchronize(tune_ev[2 * SPMM_NVAR - 1]));
      double best = 1e300;
      for (int v = 0; v < SPMM_NVAR; ++v) {
        float ms = 0.f;
        GG_CUDA(cudaEventElapsedTime(&ms, tune_ev[2 * v], tune_ev[2 * v + 1]));
        tune_ms[v] = ms;
        if (ms < best) {
          best = ms;
          sp_var = v;
        }
      }
      *count += SPMM_NVAR - 1;
    } else {
      launch_spmm(s, g, sp_var);
    }
    k_b_dots<2><<<g.nt, BT, dots_smem, s>>>(tl, dDesc.p, dSt.p, V.p, W.p, pt, ps);
    k_b_colsum<2><<<g.nb, 256, 0, s>>>(de, sb, part.p, ps, Sp.p, Cp.p, 0);
    *count += 4;
    GG_CUDA(cudaGetLastError());
    return GG_OK;
  }

  // projected eigenproblem, Ritz pairs and residuals, convergence, restart,
  // new vectors and their orthonormalisation
  int enqueue_main(cudaStream_t s, const Group &g, int *count) {
    if (g.nb == 0) return GG_OK;
    const BTile *tl = dTiles.p + g.t0;
    const BDesc *de = dDesc.p + g.b0;
    BState *sb = dSt.p + g.b0;
    double *pt = part.p + (size_t)g.t0 * ps;
    k_b_eig<<<g.nb, EIG_T, eig.bytes(), s>>>(de, sb, Sp.p, Yp.p, eig);
    k_b_ritz<<<g.nt, RT, 0, s>>>(tl, dDesc.p, dSt.p, V.p, W.p, Yp.p, X.p, R.p, pt, ps);
    k_b_conv<<<(g.nb + 127) / 128, 128, 0, s>>>(de, sb, part.p, ps, g.nb, critr, dNact.p);
    k_b_restart<<<g.nt, BT, restart_smem, s>>>(tl, dDesc.p, dSt.p, V.p, W.p, Yp.p);
    k_b_restart_fin<<<g.nb, 256, 0, s>>>(de, sb, Sp.p);
    k_b_precond<<<g.nt, RT, 0, s>>>(tl, dDesc.p, dSt.p, V.p, R.p);
    *count += 6;
    for (int pass = 0; pass < 2; ++pass) {
      k_b_dots<0><<<g.nt, BT, dots_smem, s>>>(tl, dDesc.p, dSt.p, V.p, W.p, pt, ps);
      k_b_colsum<0><<<g.nb, 256, 0, s>>>(de, sb, part.p, ps, Sp.p, Cp.p, pass == 0);
      k_b_sub<<<g.nt, RT, 0, s>>>(tl, dDesc.p, dSt.p, V.p, Cp.p);
      *count += 3;
    }
    for (int pass = 0; pass < 2; ++pass) {
      k_b_dots<1><<<g.nt, BT, dots_smem, s>>>(tl, dDesc.p, dSt.p, V.p, W.p, pt, ps);
      k_b_colsum<1><<<g.nb, 256, 0, s>>>(de, sb, part.p, ps, Sp.p, Cp.p, pass == 0);
      k_b_apply<<<g.nt, RT, 0, s>>>(tl, dDesc.p, dSt.p, V.p, Cp.p);
      *count += 3;
    }
    GG_CUDA(cudaGetLastError());
    return GG_OK;
  }

  // one Davidson iteration for every active block. The blocks are split in
  // two groups whose iterations are staggered: group 0 runs the main part
  // then the expansion, group 1 the expansion then the main part, on two
  // streams, so one group's projected eigenproblems (FP64 pipe) run beside
  // the other group's matvec (FP32 pipe and memory). Per block the sequence
  // of steps is the same as without groups.
  int enqueue_iteration(cudaStream_t s, bool fork, int *count) {
    GG_CUDA(cudaMemsetAsync(dNact.p, 0, sizeof(int), s));
    cudaStream_t sb = s;
    if (fork && grp[1].nb > 0) {
      GG_CUDA(cudaEventRecord(evFork, s));
      GG_CUDA(cudaStreamWaitEvent(s2, evFork, 0));
      sb = s2;
    }
    GG_TRY(enqueue_main(s, grp[0], count));
    GG_TRY(enqueue_expand(s, grp[0], count));
    GG_TRY(enqueue_expand(sb, grp[1], count));
    GG_TRY(enqueue_main(sb, grp[1], count));
    if (sb != s) {
      GG_CUDA(cudaEventRecord(evJoin, sb));
      GG_CUDA(cudaStreamWaitEvent(s, evJoin, 0));
    }
    GG_CUDA(cudaMemcpyAsync(hNact, dNact.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    GG_CUDA(cudaGetLastError());
    return GG_OK;
  }
};

}  // namespace
}  // namespace gg

using namespace gg;

extern "C" int gg_maneig_batched(gg_ctx *ctx, int nblocks, gg_hmat *const *hs, const int *nvec,
                                 const gg_dvd_params *p, double *eval, double *evec, int *nloops, int *nmv,
                                 int *ierr) {
  if (!ctx || nblocks < 1 || !hs || !nvec || !eval) return fail(GG_ERR_ARG, "gg_maneig_batched: bad arguments");
  GG_CUDA(cudaSetDevice(ctx->device));
  const int precision = p ? p->precision : GG_FP64;
  if (precision != GG_FP64 && precision != GG_SPLIT) return fail(GG_ERR_ARG, "gg_maneig_batched: bad precision");
  BatchRun B;
  B.ctx = ctx;
  B.nb = nblocks;
  B.precision = precision;
  B.critr = (p && p->critr > 0) ? p->critr : 1.0e-9;
  for (int b = 0; b < nblocks; ++b) {
    gg_hmat *h = hs[b];
    if (!h || nvec[b] < 1 || nvec[b] > MAXR || nvec[b] > h->ncf)
      return fail(GG_ERR_ARG, "gg_maneig_batched: bad block or NVEC (1 <= NVEC <= min(NCF, 16))");
    if (!h->emt_valid) return fail(GG_ERR_STATE, "gg_maneig_batched: EMT not assembled");
    if (h->host_prec >= 0) return fail(GG_ERR_ARG, "gg_maneig_batched: host-resident blocks are solved by gg_maneig");
    if (h->ctx->device != ctx->device) return fail(GG_ERR_ARG, "gg_maneig_batched: blocks on another device");
    if (h->ncf >= (1 << 30)) return fail(GG_ERR_ARG, "gg_maneig_batched: block too large");
  }
  GG_TRY(timer_start(ctx));
  // every block's symmetric matrix (built on its own context's stream) is
  // final before the solve starts
  for (int b = 0; b < nblocks; ++b) GG_TRY(refresh_sym_values(hs[b]));
  for (int b = 0; b < nblocks; ++b)
    if (hs[b]->ctx != ctx) GG_CUDA(cudaStreamSynchronize(hs[b]->ctx->stream));
  // layout
  int row0 = 0;
  long long voff = 0, xoff = 0, soff = 0, coff = 0;
  int pofs = 0, lmax = 1, rmax = 1, nvmax = 1, maxit = 1;
  std::vector<int> hpidx;
  std::vector<std::vector<double>> diag(nblocks);
  for (int b = 0; b < nblocks; ++b) {
    diag[b].resize(hs[b]->ncf);
    GG_CUDA(cudaMemcpyAsync(diag[b].data(), hs[b]->dDiag.p, hs[b]->ncf * sizeof(double), cudaMemcpyDeviceToHost,
                            ctx->stream));
  }
  GG_CUDA(cudaStreamSynchronize(ctx->stream));
  for (int b = 0; b < nblocks; ++b) {
    gg_hmat *h = hs[b];
    BDesc d{};
    d.n = h->ncf;
    d.r = nvec[b];
    int L = std::min(d.n, 2 * d.r + 60);  // rci90/maneig.f90:389-403
    if (p && p->lim > 0) L = std::min(d.n, p->lim);
    L = std::min(L, MAXL);
    if (L < std::min(d.n, 2 * d.r)) return fail(GG_ERR_ARG, "gg_maneig_batched: LIM too small");
    d.lim = L;
    d.rest = std::max(d.r, std::min(std::max(L / 2, 2 * d.r), L - 3));  // OVFLOW, dvdson.f90:716-717
    d.rest = std::min(d.rest, std::min(L, 64));
    d.m0 = (d.n <= L) ? d.n : std::min(L - d.r, std::max(2 * d.r, std::min(24, L / 2)));
    d.maxiter = (p && p->maxiter > 0) ? p->maxiter : std::max(200 * d.r, d.n / 10);
    d.row0 = row0;
    d.tile0 = (int)B.ht.size();
    d.ntile = (d.n + TR - 1) / TR;
    for (int t = 0; t < d.ntile; ++t) B.ht.push_back(BTile{b, t * TR, std::min(TR, d.n - t * TR)});
    d.pofs = pofs;
    d.voff = voff;
    d.xoff = xoff;
    d.soff = soff;
    d.coff = coff;
    d.ptr = h->dSymPtr.p;
    d.col = h->dSymCol.p;
    d.col16 = h->sym_col16 ? h->dSymCol16.p : nullptr;
    d.val = h->dSymVal.p;
    d.hi = h->dSymHi.p;
    d.lo = h->dSymLo.p;
    d.diag = h->dDiag.p;
    // start vectors: the m0 lowest diagonal elements (ties by index)
    std::vector<int> order(d.n);
    std::iota(order.begin(), order.end(), 0);
    const std::vector<double> &dg = diag[b];
    std::partial_sort(order.begin(), order.begin() + d.m0, order.end(),
                      [&](int x, int y) { return dg[x] < dg[y] || (dg[x] == dg[y] && x < y); });
    hpidx.insert(hpidx.end(), order.begin(), order.begin() + d.m0);
    pofs += d.m0;
    row0 += d.n;
    voff += (long long)d.n * L;
    xoff += (long long)d.n * d.r;
    soff += (long long)L * L;
    coff += (long long)std::max(L, MAXR) * MAXR;
    lmax = std::max(lmax, L);
    rmax = std::max(rmax, d.r);
    nvmax = std::max(nvmax, std::min(L, std::max(d.rest, d.r)));
    maxit = std::max(maxit, d.maxiter);
    B.hd.push_back(d);
  }
  B.ntot = row0;
  B.ntiles = (int)B.ht.size();
  // two groups of contiguous blocks with about half the rows each
  B.all = BatchRun::Group{0, nblocks, 0, B.ntiles};
  {
    int split = nblocks;
    if (nblocks >= 2) {
      long long acc = 0;
      split = 1;
      for (int b = 0; b < nblocks - 1; ++b) {
        acc += B.hd[b].n;
        split = b + 1;
        if (2 * acc >= row0) break;
      }
    }
    B.grp[0] = BatchRun::Group{0, split, 0, split < nblocks ? B.hd[split].tile0 : B.ntiles};
    B.grp[1] = BatchRun::Group{split, nblocks - split, B.grp[0].nt, B.ntiles - B.grp[0].nt};
    // the batched matvec's tiles for each tile size of the autotuner
    for (int ts = 0; ts < 3; ++ts) {
      std::vector<BTile> &v = B.hsp_tiles[ts];
      v.clear();
      int first_of_split = 0;
      for (int b = 0; b < nblocks; ++b) {
        if (b == split) first_of_split = (int)v.size();
        const int n = B.hd[b].n, tr = SPMM_TR[ts];
        for (int r0 = 0; r0 < n; r0 += tr) v.push_back(BTile{b, r0, std::min(tr, n - r0)});
      }
      if (split >= nblocks) first_of_split = (int)v.size();
      const int tot = (int)v.size();
      B.sp_t0[ts][0] = 0;
      B.sp_nt[ts][0] = tot;
      B.sp_t0[ts][1] = 0;
      B.sp_nt[ts][1] = first_of_split;
      B.sp_t0[ts][2] = first_of_split;
      B.sp_nt[ts][2] = tot - first_of_split;
    }
  }
  B.eig = EigShape{lmax, nvmax};
  B.ps = (lmax + 1) * MAXR;
  B.restart_smem = sizeof(double) * ((size_t)lmax * 64 + (size_t)RG * lmax);
  B.dots_smem = sizeof(double) * ((size_t)TR * MAXR + (size_t)TR * (AC + 1));
  {
    int nmax = 0;
    for (auto &d : B.hd) nmax = std::max(nmax, d.n);
    B.sx_rows = std::min(nmax, 6144);  // 6144 rows x 32 bytes = 192 KB
  }
  GG_CUDA(cudaFuncSetAttribute(k_b_spmm<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)(B.sx_rows * sizeof(X32))));
  GG_CUDA(cudaFuncSetAttribute(k_b_spmm<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)(B.sx_rows * sizeof(X32))));
  GG_CUDA(cudaFuncSetAttribute(k_b_eig, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)B.eig.bytes()));
  GG_CUDA(cudaFuncSetAttribute(k_b_restart, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)B.restart_smem));
  GG_CUDA(cudaFuncSetAttribute(k_b_dots<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)B.dots_smem));
  GG_CUDA(cudaFuncSetAttribute(k_b_dots<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)B.dots_smem));
  GG_CUDA(cudaFuncSetAttribute(k_b_dots<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)B.dots_smem));
  std::vector<BState> hst(nblocks);
  for (auto &s : hst) {
    std::memset(&s, 0, sizeof(BState));
    s.active = 1;
  }
  cudaStream_t s = ctx->stream;
  GG_TRY(B.dDesc.alloc(nblocks));
  GG_TRY(B.dSt.alloc(nblocks));
  GG_TRY(B.dTiles.alloc(B.ntiles));
  GG_TRY(B.dPidx.alloc(std::max(pofs, 1)));
  GG_TRY(B.dNact.alloc(1));
  GG_TRY(B.V.alloc(voff));
  GG_TRY(B.W.alloc(voff));
  GG_TRY(B.X.alloc(xoff));
  GG_TRY(B.R.alloc(xoff));
  GG_TRY(B.Sp.alloc(soff));
  GG_TRY(B.Yp.alloc(soff));
  GG_TRY(B.Cp.alloc(coff));
  GG_TRY(B.part.alloc((size_t)B.ntiles * B.ps));
  if (precision == GG_SPLIT)
    GG_TRY(B.XS.alloc((size_t)B.ntot * MAXR));
  else
    GG_TRY(B.XD.alloc((size_t)B.ntot * MAXR));
  if (cudaMallocHost(&B.hNact, sizeof(int)) != cudaSuccess) return fail(GG_ERR_NOMEM, "cudaMallocHost");
  note_alloc();
  GG_CUDA(cudaMemcpyAsync(B.dDesc.p, B.hd.data(), nblocks * sizeof(BDesc), cudaMemcpyHostToDevice, s));
  GG_CUDA(cudaMemcpyAsync(B.dSt.p, hst.data(), nblocks * sizeof(BState), cudaMemcpyHostToDevice, s));
  GG_CUDA(cudaMemcpyAsync(B.dTiles.p, B.ht.data(), B.ntiles * sizeof(BTile), cudaMemcpyHostToDevice, s));
  GG_CUDA(cudaMemcpyAsync(B.dPidx.p, hpidx.data(), pofs * sizeof(int), cudaMemcpyHostToDevice, s));
  for (int ts = 0; ts < 3; ++ts) {
    const size_t tot = B.hsp_tiles[ts].size();
    GG_TRY(B.dSpTiles[ts].alloc(std::max<size_t>(tot, 1)));
    GG_CUDA(cudaMemcpyAsync(B.dSpTiles[ts].p, B.hsp_tiles[ts].data(), tot * sizeof(BTile), cudaMemcpyHostToDevice,
                            s));
  }
  GG_CUDA(cudaMemsetAsync(B.Sp.p, 0, soff * sizeof(double), s));
  GG_CUDA(cudaMemsetAsync(B.part.p, 0, (size_t)B.ntiles * B.ps * sizeof(double), s));
  // start: V = unit vectors, W = H V and S = V^T W, MAXR columns at a time
  int launches = 0;
  k_b_init<<<B.ntiles, RT, 0, s>>>(B.dTiles.p, B.dDesc.p, B.dPidx.p, B.V.p);
  ++launches;
  int m0max = 0;
  for (auto &d : B.hd) m0max = std::max(m0max, d.m0);
  // the batched matvec variant: tuned on this batch shape's first start-up
  // expansion, then kept for the shape in this process
  long long nnz_all = 0;
  for (int b = 0; b < nblocks; ++b) nnz_all += hs[b]->sym_nnz;
  const BatchTuneKey tkey{ctx->device, nblocks, B.ntot, nnz_all, precision};
  bool tune = false;
  double tms[SPMM_NVAR] = {};
  {
    std::lock_guard<std::mutex> lk(g_btune_mu);
    auto it = g_btune.find(tkey);
    if (it != g_btune.end()) {
      B.sp_var = it->second.variant;
      std::copy(it->second.ms, it->second.ms + SPMM_NVAR, tms);
    } else {
      tune = true;
    }
  }
  std::vector<cudaEvent_t> tev;
  if (tune) {
    tev.resize(2 * SPMM_NVAR);
    for (auto &e : tev) GG_CUDA(cudaEventCreate(&e));
  }
  for (int c0 = 0; c0 < m0max; c0 += MAXR) {
    k_b_setnew<<<(nblocks + 127) / 128, 128, 0, s>>>(B.dDesc.p, B.dSt.p, nblocks);
    ++launches;
    const bool t = tune && c0 == 0;
    const int rc = B.enqueue_expand(s, B.all, &launches, t ? tev.data() : nullptr, t ? tms : nullptr);
    if (t) {
      for (auto &e : tev) cudaEventDestroy(e);
      tev.clear();
    }
    GG_TRY(rc);
    if (t) {
      std::lock_guard<std::mutex> lk(g_btune_mu);
      BatchTuneEntry &en = g_btune[tkey];
      en.variant = B.sp_var;
      std::copy(tms, tms + SPMM_NVAR, en.ms);
    }
  }
  ctx->btune_var = B.sp_var;
  std::copy(tms, tms + SPMM_NVAR, ctx->btune_ms);
  GG_CUDA(cudaGetLastError());
  // the iteration, captured once and replayed until no block is active
  int per_iter = 0;
  {
    GG_CUDA(cudaStreamCreateWithFlags(&B.s2, cudaStreamNonBlocking));
    GG_CUDA(cudaEventCreateWithFlags(&B.evFork, cudaEventDisableTiming));
    GG_CUDA(cudaEventCreateWithFlags(&B.evJoin, cudaEventDisableTiming));
    GG_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    const int rc = B.enqueue_iteration(s, true, &per_iter);
    cudaGraph_t g = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(s, &g);
    if (rc != GG_OK) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    if (ce != cudaSuccess) return fail(GG_ERR_CUDA, std::string("batched Davidson capture: ") + cudaGetErrorString(ce));
    B.graph = g;
    GG_CUDA(cudaGraphInstantiate(&B.gexec, B.graph, 0));
  }
  int iters = 0;
  for (;;) {
    GG_CUDA(cudaGraphLaunch(B.gexec, s));
    launches += per_iter;
    ++iters;
    GG_CUDA(cudaStreamSynchronize(s));
    if (*B.hNact == 0) break;
    if (iters > maxit + 2) break;  // every block stops at its own MAXITER before this
  }
  note_launches(launches);
  // results: eigenvalues from the states, vectors from X (already in the
  // concatenated EVEC layout), then the reference's sign convention
  GG_CUDA(cudaMemcpyAsync(hst.data(), B.dSt.p, nblocks * sizeof(BState), cudaMemcpyDeviceToHost, s));
  if (evec) GG_CUDA(cudaMemcpyAsync(evec, B.X.p, xoff * sizeof(double), cudaMemcpyDeviceToHost, s));
  GG_CUDA(cudaStreamSynchronize(s));
  double ms = 0;
  GG_TRY(timer_stop(ctx, &ms));
  int any_err = 0;
  size_t eo = 0;
  for (int b = 0; b < nblocks; ++b) {
    const BDesc &d = B.hd[b];
    for (int j = 0; j < d.r; ++j) eval[eo + j] = hst[b].theta[j];
    eo += d.r;
    if (nloops) nloops[b] = hst[b].iters;
    if (nmv) nmv[b] = hst[b].nmv;
    if (ierr) ierr[b] = hst[b].ierr;
    any_err |= hst[b].ierr;
    if (evec)
      for (int j = 0; j < d.r; ++j) {  // dominant component positive (rci90/maneig.f90:532-555)
        double *v = evec + d.xoff + (size_t)j * d.n;
        double amax = 0.0;
        int ia = 0;
        for (int i = 0; i < d.n; ++i) {
          const double wa = std::fabs(v[i]);
          if (wa <= amax) continue;
          amax = wa;
          ia = i;
        }
        if (v[ia] < 0.0)
          for (int i = 0; i < d.n; ++i) v[i] = -v[i];
      }
  }
  ctx->stats[3] = ms;
  ctx->stats[21] = iters;
  ctx->stats[22] = per_iter;
  if (any_err & 2048) return fail(GG_ERR_CONVERGE, "batched DVDSON: a block reached MAXITER (IERR 2048)");
  return GG_OK;
}
