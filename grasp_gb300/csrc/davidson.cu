// davidson.cu - MANEIG / GDVD / DVDSON on the GPU.
//
// Follows libdvd90/dvdson.f90 (Stathopoulos & Fischer's block Davidson-Liu)
// step by step: INITDVD (Krylov completion to NUME+1 vectors), the DSPEVX of
// the projected matrix S, TSTSEL, OVFLOW restarts, NEWVEC with the robust
// shift, GDVD's diagonal preconditioner (gdvd.f90:93-134, including its
// DIAG - lambda + lambda update), Gram-Schmidt, OP = H x, ADDS.
//
// Placement. Everything of length N (the basis BASIS and AB = H BASIS,
// Ritz vectors, residuals, preconditioning, Gram-Schmidt, new columns of
// S, the matvec) runs on the GPU in FP64 (the matvec optionally in the hi+lo
// split). The k x k projected eigenproblem (k <= LIM) and the scalar control
// flow run on the host, as in the reference. Two small device-to-host
// copies per iteration (a residual norm and one column of S) synchronise
// the two.
//
// Differences from the reference, all at rounding level:
//  - Gram-Schmidt is two-pass classical (CGS2), the reference's mgs_nrm is
//    two-pass modified; both leave the new vector orthonormal to working
//    precision.
//  - Dot products are blocked reductions, not sequential sums.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "gg_internal.cuh"

namespace gg {
namespace {

constexpr int TPB = 256;
constexpr int RB = 1024;  // rows per block in the partial-dot kernels
constexpr int CG = 8;     // columns per block in the partial-dot kernels

// partial dots part[rb * k + j] = sum_{i in row block rb} B[i, j] w[i], j < k
__global__ void k_dots_part(const double *__restrict__ B, int64_t ld, int k, const double *__restrict__ w, int n,
                            double *__restrict__ part) {
  __shared__ double s[CG][TPB];
  const int rb = blockIdx.x, j0 = blockIdx.y * CG;
  double acc[CG];
#pragma unroll
  for (int c = 0; c < CG; ++c) acc[c] = 0.0;
  const int i0 = rb * RB, i1 = min(n, i0 + RB);
  for (int i = i0 + threadIdx.x; i < i1; i += TPB) {
    const double wi = w[i];
#pragma unroll
    for (int c = 0; c < CG; ++c)
      if (j0 + c < k) acc[c] = fma(B[(size_t)(j0 + c) * ld + i], wi, acc[c]);
  }
#pragma unroll
  for (int c = 0; c < CG; ++c) s[c][threadIdx.x] = acc[c];
  __syncthreads();
  for (int st = TPB / 2; st > 0; st >>= 1) {
    if ((int)threadIdx.x < st)
#pragma unroll
      for (int c = 0; c < CG; ++c) s[c][threadIdx.x] += s[c][threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x < CG && j0 + (int)threadIdx.x < k) part[(size_t)rb * k + j0 + threadIdx.x] = s[threadIdx.x][0];
}

// out[j] = sum over row blocks of part (fixed order)
__global__ void k_dots_reduce(const double *__restrict__ part, int nrb, int k, double *__restrict__ out) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= k) return;
  double s = 0.0;
  for (int r = 0; r < nrb; ++r) s += part[(size_t)r * k + j];
  out[j] = s;
}

// w -= B[:, 0:k] coef  (coef on the device)
__global__ void k_sub_gemv(double *__restrict__ w, const double *__restrict__ B, int64_t ld, int k,
                           const double *__restrict__ coef, int n) {
  __shared__ double c[1024];
  for (int j = threadIdx.x; j < k; j += blockDim.x) c[j] = coef[j];
  __syncthreads();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double acc = 0.0;
  for (int j = 0; j < k; ++j) acc = fma(B[(size_t)j * ld + i], c[j], acc);
  w[i] -= acc;
}

// partial sums of squares
__global__ void k_sq_part(const double *__restrict__ w, int n, double *__restrict__ part) {
  __shared__ double s[TPB];
  double acc = 0.0;
  for (int i = blockIdx.x * TPB + threadIdx.x; i < n; i += gridDim.x * TPB) acc = fma(w[i], w[i], acc);
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int st = TPB / 2; st > 0; st >>= 1) {
    if ((int)threadIdx.x < st) s[threadIdx.x] += s[threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = s[0];
}

// w *= 1/sqrt(sum(part)); every block reduces the partials in the same order
__global__ void k_normalize(double *__restrict__ w, int n, const double *__restrict__ part, int np) {
  __shared__ double sc;
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < np; ++i) s += part[i];
    const double dnm = sqrt(s);
    sc = 1.0 / dnm;
  }
  __syncthreads();
  const double f = sc;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) w[i] *= f;
}

// Ritz vector and residual (NEWVEC, dvdson.f90:1100-1111):
//   b = BASIS s ; a = AB s ; r = a - lambda b ; part = partial sums of r^2
__global__ void k_ritz(const double *__restrict__ B, const double *__restrict__ AB, int64_t ld, int k,
                       const double *__restrict__ s, double lam, double *__restrict__ bout, double *__restrict__ rout,
                       int n, double *__restrict__ part) {
  __shared__ double sv[1024];
  __shared__ double red[TPB];
  for (int j = threadIdx.x; j < k; j += blockDim.x) sv[j] = s[j];
  __syncthreads();
  const int i = blockIdx.x * TPB + threadIdx.x;
  double r2 = 0.0;
  if (i < n) {
    double b = 0.0, a = 0.0;
    for (int j = 0; j < k; ++j) {
      b = fma(B[(size_t)j * ld + i], sv[j], b);
      a = fma(AB[(size_t)j * ld + i], sv[j], a);
    }
    const double r = a + (-lam) * b;
    bout[i] = b;
    rout[i] = r;
    r2 = r * r;
  }
  red[threadIdx.x] = r2;
  __syncthreads();
  for (int st = TPB / 2; st > 0; st >>= 1) {
    if ((int)threadIdx.x < st) red[threadIdx.x] += red[threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// robust shift + GDVD diagonal preconditioner (gdvd.f90:114-129):
//   r <- r - rhseps b ; DIAG <- DIAG - lambda ; w = r/DIAG (|DIAG| > 1e-6)
//   or r*1e6 ; DIAG <- DIAG + lambda ; BASIS column <- w
__global__ void k_precond(double *__restrict__ r, const double *__restrict__ b, double rhseps, double lam,
                          double *__restrict__ diag, double *__restrict__ w, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double rr = r[i] + (-rhseps) * b[i];
  r[i] = rr;
  const double d = diag[i] - lam;
  w[i] = (fabs(d) > 1.0e-06) ? rr / d : rr * 1.0e06;
  diag[i] = d + lam;
}

// out[:, j] = sum_{i<k} B[:, i] C[i + j k], j < m   (MULTBC)
__global__ void k_multbc(const double *__restrict__ B, int64_t ld, int k, const double *__restrict__ C, int m,
                         double *__restrict__ out, int n) {
  extern __shared__ double cs[];
  for (int t = threadIdx.x; t < k * m; t += blockDim.x) cs[t] = C[t];
  __syncthreads();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int j = 0; j < m; ++j) {
    double acc = 0.0;
    for (int q = 0; q < k; ++q) acc = fma(B[(size_t)q * ld + i], cs[(size_t)j * k + q], acc);
    out[(size_t)j * ld + i] = acc;
  }
}

// t = AB_j - lambda_j B_j, partial sums of t^2 for the final residual norms
__global__ void k_final_res_part(const double *__restrict__ B, const double *__restrict__ AB, int64_t ld, int j,
                                 double lam, int n, double *__restrict__ part) {
  __shared__ double s[TPB];
  double acc = 0.0;
  for (int i = blockIdx.x * TPB + threadIdx.x; i < n; i += gridDim.x * TPB) {
    const double t = AB[(size_t)j * ld + i] + (-lam) * B[(size_t)j * ld + i];
    acc = fma(t, t, acc);
  }
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int st = TPB / 2; st > 0; st >>= 1) {
    if ((int)threadIdx.x < st) s[threadIdx.x] += s[threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = s[0];
}

struct Dvd {
  gg_ctx *ctx;
  gg_hmat *h;
  int precision;
  int n, lim;
  int64_t ld;
  cudaStream_t s;
  DBuf<double> B, AB, T, diag, part, small, dots;
  int nrb;
  int nmv = 0;
  double mv_ms = 0;
  int mv_count = 0;
  double t_eig = 0, t_wait = 0;  // host seconds: projected eigenproblem, device-to-host waits
  std::vector<cudaEvent_t> evs;   // matvec start/stop pairs, read once at the end
  size_t ev_used = 0;
  cudaEvent_t e0 = nullptr, e1 = nullptr;

  int init(gg_ctx *c, gg_hmat *hm, int prec, int nn, int lm) {
    ctx = c;
    h = hm;
    precision = prec;
    n = nn;
    lim = lm;
    s = c->stream;
    ld = ((int64_t)n + 31) / 32 * 32;
    nrb = (n + RB - 1) / RB;
    GG_TRY(B.alloc((size_t)ld * lim));
    GG_TRY(AB.alloc((size_t)ld * lim));
    GG_TRY(T.alloc((size_t)ld * lim));
    GG_TRY(diag.alloc(n));
    GG_TRY(part.alloc((size_t)std::max(nrb * lim, (n + TPB - 1) / TPB + 1024)));
    GG_TRY(small.alloc(4096));
    GG_TRY(dots.alloc(lim + 8));
    GG_CUDA(cudaMemsetAsync(B.p, 0, (size_t)ld * lim * 8, s));
    GG_CUDA(cudaMemsetAsync(AB.p, 0, (size_t)ld * lim * 8, s));
    GG_CUDA(cudaEventCreate(&e0));
    GG_CUDA(cudaEventCreate(&e1));
    return GG_OK;
  }
  ~Dvd() {
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    for (cudaEvent_t e : evs) cudaEventDestroy(e);
  }
  double *col(DBuf<double> &X, int j) { return X.p + (size_t)j * ld; }

  // OP (gdvd.f90:137-142): AB[:, j0:j0+m) = H BASIS[:, j0:j0+m); each launch
  // is bracketed by events that are read after the solve (no extra sync)
  int op(int j0, int m) {
    for (int v = 0; v < m; ++v) {
      if (ev_used + 2 > evs.size()) {
        for (int q = 0; q < 64; ++q) {
          cudaEvent_t e;
          GG_CUDA(cudaEventCreate(&e));
          evs.push_back(e);
        }
      }
      GG_CUDA(cudaEventRecord(evs[ev_used], s));
      GG_TRY(spmv(h, precision, col(B, j0 + v), col(AB, j0 + v), 1, s));
      GG_CUDA(cudaEventRecord(evs[ev_used + 1], s));
      ev_used += 2;
      ++mv_count;
    }
    nmv += m;
    return GG_OK;
  }
  int collect_matvec_time() {
    GG_CUDA(cudaStreamSynchronize(s));
    for (size_t q = 0; q + 1 < ev_used; q += 2) {
      float ms = 0.f;
      GG_CUDA(cudaEventElapsedTime(&ms, evs[q], evs[q + 1]));
      mv_ms += ms;
    }
    ev_used = 0;
    return GG_OK;
  }
  // out[0:k] = BASIS[:, 0:k]^T w  (device)
  int dots_dev(const DBuf<double> &X, int k, const double *w, double *out) {
    if (k <= 0) return GG_OK;
    dim3 g(nrb, (k + CG - 1) / CG);
    k_dots_part<<<g, TPB, 0, s>>>(X.p, ld, k, w, n, part.p); ::gg::note_launch();
    k_dots_reduce<<<(k + 127) / 128, 128, 0, s>>>(part.p, nrb, k, out); ::gg::note_launch();
    GG_CUDA(cudaGetLastError());
    return GG_OK;
  }
  // two-pass classical Gram-Schmidt of column j against columns 0..j-1,
  // normalised after each pass (mgs_nrm, dvdson.f90:1417-1508)
  int orthonormalize(int j) {
    double *w = col(B, j);
    const int nb = std::min((n + TPB - 1) / TPB, 1024);
    for (int pass = 0; pass < 2; ++pass) {
      if (j > 0) {
        GG_TRY(dots_dev(B, j, w, dots.p));
        k_sub_gemv<<<(n + TPB - 1) / TPB, TPB, 0, s>>>(w, B.p, ld, j, dots.p, n); ::gg::note_launch();
      }
      k_sq_part<<<nb, TPB, 0, s>>>(w, n, part.p); ::gg::note_launch();
      k_normalize<<<nb, TPB, 0, s>>>(w, n, part.p, nb); ::gg::note_launch();
      GG_CUDA(cudaGetLastError());
    }
    return GG_OK;
  }
  // S(1:kp+1, kp+1) for new column kp (0-based) of AB, into host Sp (packed upper)
  int adds(int kp, std::vector<double> &S) {
    GG_TRY(dots_dev(B, kp + 1, col(AB, kp), dots.p));
    std::vector<double> hcol(kp + 1);
    GG_CUDA(cudaMemcpyAsync(hcol.data(), dots.p, (kp + 1) * sizeof(double), cudaMemcpyDeviceToHost, s));
    const auto t0 = std::chrono::steady_clock::now();
    GG_CUDA(cudaStreamSynchronize(s));
    t_wait += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    const size_t off = (size_t)kp * (kp + 1) / 2;
    for (int i = 0; i <= kp; ++i) S[off + i] = hcol[i];
    return GG_OK;
  }
  // X[:, 0:m) = X[:, 0:k) C (k x m)
  int multbc(DBuf<double> &X, int k, int m, const double *hC) {
    if ((size_t)k * m > small.n) GG_TRY(small.alloc((size_t)k * m));
    GG_CUDA(cudaMemcpyAsync(small.p, hC, (size_t)k * m * sizeof(double), cudaMemcpyHostToDevice, s));
    const size_t sm = (size_t)k * m * sizeof(double);
    if (sm > 48 * 1024) GG_CUDA(cudaFuncSetAttribute(k_multbc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    k_multbc<<<(n + TPB - 1) / TPB, TPB, sm, s>>>(X.p, ld, k, small.p, m, T.p, n); ::gg::note_launch();
    GG_CUDA(cudaGetLastError());
    GG_CUDA(cudaMemcpy2DAsync(X.p, ld * 8, T.p, ld * 8, (size_t)n * 8, m, cudaMemcpyDeviceToDevice, s));
    return GG_OK;
  }
  double host_sum_sqrt(int np) {
    std::vector<double> hp(np);
    cudaMemcpyAsync(hp.data(), part.p, np * sizeof(double), cudaMemcpyDeviceToHost, s);
    const auto t0 = std::chrono::steady_clock::now();
    cudaStreamSynchronize(s);
    t_wait += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    double a = 0.0;
    for (int i = 0; i < np; ++i) a += hp[i];
    return std::sqrt(a);
  }
};

struct DvdParams {
  int lim, nume, niv, mblock, maxiter;
  double crite, critc, critr;
  int robust;  // 1: first-pass shift uses DL = 0 instead of |1e30 - lambda|
};

// DVDSON for ILOW = 1, IHIGH = NUME; BASIS columns 0..niv-1 hold the initial
// estimates on entry. On exit BASIS[:, 0:nume) are the eigenvectors and
// eigval[0:nume] the eigenvalues.
int dvdson(Dvd &D, const DvdParams &P, std::vector<double> &eigval_out, std::vector<double> &resid_out, int *nloops_out,
           int *ierr_out) {
  const int n = D.n, LIM = P.lim, NUME = P.nume, MBLOCK = P.mblock, MAXITER = P.maxiter;
  int NIV = P.niv;
  int IERR = 0;
  if (LIM > n) IERR += 1;
  if (LIM <= 0) IERR += 2;
  if (NUME > LIM || (NUME == LIM && NUME != n)) IERR += 128;
  if (MBLOCK < 1 || MBLOCK > NUME) IERR += 256;
  if (NIV > LIM) IERR += 4096;
  if (IERR) {
    *ierr_out = IERR;
    return fail(GG_ERR_ARG, "DVDSON: inconsistent LIM / NUME / MBLOCK / NIV (IERR " + std::to_string(IERR) + ")");
  }
  // OLDVAL receives IFIND = min(KPASS, REST) values each pass (dvdson.f90:722),
  // more than its declared NUME + 1 (the reference's copy runs into the slack
  // at the end of WORK): size it LIM.
  std::vector<double> S((size_t)LIM * (LIM + 1) / 2, 0.0), SVEC((size_t)LIM * LIM, 0.0), EIGVAL(LIM + 2, 0.0),
      OLDVAL(LIM + 2, 0.0), SCRA1(8 * LIM, 0.0);
  std::vector<int> INCV(LIM + 2, 0), ICV(NUME + 2, 0), IND(LIM + 2, 0);
  std::vector<double> ROWLAST(LIM + 2, 0.0);
  // INITDVD (dvdson.f90:848-948) with NUME + 1
  {
    const int NUME1 = NUME + 1;
    int IST = 1, IEND = NIV, NEW = NIV;
    for (;;) {
      GG_TRY(D.op(IST - 1, NEW));
      if (IEND < NUME1) {
        NEW = std::min(NUME1 - IEND, IEND - IST + 1);
        GG_CUDA(cudaMemcpy2DAsync(D.col(D.B, IEND), D.ld * 8, D.col(D.AB, IST - 1), D.ld * 8, (size_t)n * 8, NEW,
                                  cudaMemcpyDeviceToDevice, D.s));
        for (int v = 0; v < NEW; ++v) GG_TRY(D.orthonormalize(IEND + v));
        IST = IEND + 1;
        IEND = IEND + NEW;
        continue;
      }
      break;
    }
    NIV = IEND;
    for (int j = 0; j < NIV; ++j) GG_TRY(D.adds(j, S));
  }
  int NLOOPS = 1;
  for (int i = 0; i < NUME; ++i) {
    EIGVAL[i] = 1.0e30;
    ICV[i + 1] = 0;
  }
  int KPASS = NIV, NNCV = KPASS;
  int REST = std::max(LIM / 2, 2 * NUME);
  REST = std::min(REST, LIM - 3);
  bool DONE = false;
  std::vector<double> tmpS, w, z;
  for (;;) {
    const int IFIND = std::min(KPASS, REST);
    for (int i = 0; i < IFIND; ++i) OLDVAL[i] = EIGVAL[i];
    w.assign(IFIND, 0.0);
    // DSPEVX returns IFIND eigenpairs; only the first NUME eigenvectors are
    // read afterwards (TSTSEL, NEWVEC, MULTBC), all IFIND = REST when the
    // basis is full and OVFLOW collapses onto them.
    const int nvecs = (KPASS == LIM) ? IFIND : std::min(IFIND, NUME);
    const auto te0 = std::chrono::steady_clock::now();
    if (sym_eig_lowest(KPASS, S.data(), IFIND, nvecs, w.data(), SVEC.data()) != 0) {
      *ierr_out = -1;
      return fail(GG_ERR_CONVERGE, "DVDSON: projected eigenproblem failed");
    }
    D.t_eig += std::chrono::duration<double>(std::chrono::steady_clock::now() - te0).count();
    for (int i = 0; i < IFIND; ++i) EIGVAL[i] = w[i];
    // TSTSEL (dvdson.f90:1260-1413)
    {
      int NNCE = 0;
      for (int i = 1; i <= NUME; ++i)
        if (!(std::fabs(OLDVAL[i - 1] - EIGVAL[i - 1]) < P.crite)) ++NNCE;
      if (NNCE == 0) {
        DONE = true;
      } else {
        int ICNT = 0;
        for (int i = 1; i <= NUME; ++i) {
          const int64_t icur = (int64_t)KPASS * i;
          double tmax = std::fabs(SVEC[icur - 1]);
          for (int l = 1; l <= NNCV - 1; ++l) tmax = std::max(tmax, std::fabs(SVEC[icur - l - 1]));
          if (tmax < P.critc) {
            ICV[i] = 1;
          } else {
            ICV[i] = 0;
            ++ICNT;
            IND[ICNT] = i;
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
    if (KPASS == LIM) {  // OVFLOW (dvdson.f90:1179-1256)
      GG_TRY(D.multbc(D.B, KPASS, REST, SVEC.data()));
      GG_TRY(D.multbc(D.AB, KPASS, REST, SVEC.data()));
      std::fill(S.begin(), S.end(), 0.0);
      std::fill(SVEC.begin(), SVEC.begin() + (size_t)REST * REST, 0.0);
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
    int nadded = 0, icvc = 0;
    double lam_added = 0.0, rhseps_added = 0.0;
    {
      const int limadd = std::min(LIM, MBLOCK + KPASS);
      DONE = false;
      for (int i = 1; i <= NNCV; ++i) {
        const int indx = INCV[i];
        GG_CUDA(cudaMemcpyAsync(D.small.p, SVEC.data() + (size_t)(indx - 1) * KPASS, KPASS * sizeof(double),
                                cudaMemcpyHostToDevice, D.s));
        const int nb = (n + TPB - 1) / TPB;
        // ICUR = column KPASS + NADDED (a converged target is overwritten)
        k_ritz<<<nb, TPB, 0, D.s>>>(D.B.p, D.AB.p, D.ld, KPASS, D.small.p, EIGVAL[indx - 1],
                                    D.col(D.B, KPASS + nadded), D.col(D.AB, KPASS + nadded), n, D.part.p); ::gg::note_launch();
        GG_CUDA(cudaGetLastError());
        const double res = D.host_sum_sqrt(nb);
        SCRA1[indx - 1] = res;
        if (res < P.critr) {
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
        // On the first pass OLDVAL still holds DVDRVR's 1e30 sentinel
        // (dvdson.f90:703): the reference then shifts by RHSEPS ~ 1e13 and its
        // first correction vector carries no new direction, after which the
        // coefficient test (CRITC) can end the iteration early. robust = 1
        // uses DL = 0 on that pass instead.
        if (P.robust && OLDVAL[indx - 1] >= 1.0e29) dl = 0.0;
        const double rhseps = (gap > res) ? std::sqrt(dl * res) : std::min(dl, std::sqrt(dl));
        ++nadded;
        INCV[nadded] = indx;
        lam_added = EIGVAL[indx - 1];
        rhseps_added = rhseps;
        // shift + preconditioner for this column now (MBLOCK columns at most)
        k_precond<<<(n + TPB - 1) / TPB, TPB, 0, D.s>>>(D.col(D.AB, KPASS + nadded - 1), D.col(D.B, KPASS + nadded - 1),
                                                        rhseps_added, lam_added, D.diag.p, D.col(D.B, KPASS + nadded - 1),
                                                        n); ::gg::note_launch();
        GG_CUDA(cudaGetLastError());
        if (nadded + KPASS == limadd) break;
      }
      if (DONE) break;
      NNCV = nadded;
    }
    // Gram-Schmidt of the new vectors, OP, ADDS
    for (int v = 0; v < NNCV; ++v) GG_TRY(D.orthonormalize(KPASS + v));
    GG_TRY(D.op(KPASS, NNCV));
    for (int v = 0; v < NNCV; ++v) GG_TRY(D.adds(KPASS + v, S));
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
  GG_TRY(D.multbc(D.B, KPASS, NUME, SVEC.data()));
  GG_TRY(D.multbc(D.AB, KPASS, NUME, SVEC.data()));
  resid_out.assign(NUME, 0.0);
  for (int i = 0; i < NUME; ++i) {
    const int nb = std::min((n + TPB - 1) / TPB, 1024);
    k_final_res_part<<<nb, TPB, 0, D.s>>>(D.B.p, D.AB.p, D.ld, i, EIGVAL[i], n, D.part.p); ::gg::note_launch();
    GG_CUDA(cudaGetLastError());
    resid_out[i] = D.host_sum_sqrt(nb);
  }
  eigval_out.assign(EIGVAL.begin(), EIGVAL.begin() + NUME);
  *nloops_out = NLOOPS;
  *ierr_out = IERR;
  return D.collect_matvec_time();
}

// Leading ns x ns block of a matrix as its own hmat (INIEST2's sub-matrix).
int leading_block(gg_hmat *h, int ns, gg_hmat **out) {
  gg_ctx *ctx = h->ctx;
  const int64_t nnz = h->hIendc[ns];
  gg_hmat *b = new gg_hmat;
  b->ctx = ctx;
  b->ncf = ns;
  b->nnz = nnz;
  b->hIendc.assign(h->hIendc.begin(), h->hIendc.begin() + ns + 1);
  int st = b->dIendc.alloc(ns + 1);
  if (!st) st = b->dIrow.alloc(nnz);
  if (!st) st = b->dEmt.alloc(nnz);
  if (!st) st = b->dDiag.alloc(ns);
  if (st) {
    delete b;
    return st;
  }
  cudaStream_t s = ctx->stream;
  cudaMemcpyAsync(b->dIendc.p, h->dIendc.p, (ns + 1) * sizeof(int64_t), cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(b->dIrow.p, h->dIrow.p, nnz * sizeof(int32_t), cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(b->dEmt.p, h->dEmt.p, nnz * sizeof(double), cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(b->dDiag.p, h->dDiag.p, ns * sizeof(double), cudaMemcpyDeviceToDevice, s);
  if (cudaGetLastError() != cudaSuccess) {
    delete b;
    return fail(GG_ERR_CUDA, "leading_block: copy failed");
  }
  b->emt_valid = true;
  *out = b;
  return GG_OK;
}

// Unit vectors on the niv lowest diagonal entries as starting basis.
int unit_start(Dvd &D, gg_hmat *h, int niv) {
  std::vector<double> d(h->ncf);
  GG_CUDA(cudaMemcpyAsync(d.data(), h->dDiag.p, h->ncf * sizeof(double), cudaMemcpyDeviceToHost, D.s));
  GG_CUDA(cudaStreamSynchronize(D.s));
  std::vector<int> idx(h->ncf);
  for (int i = 0; i < h->ncf; ++i) idx[i] = i;
  std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return d[a] < d[b]; });
  const double one = 1.0;
  for (int j = 0; j < niv; ++j)
    GG_CUDA(cudaMemcpyAsync(D.col(D.B, j) + idx[j], &one, sizeof(double), cudaMemcpyHostToDevice, D.s));
  GG_CUDA(cudaStreamSynchronize(D.s));
  return GG_OK;
}

}  // namespace
}  // namespace gg

using namespace gg;

extern "C" int gg_maneig(gg_ctx *ctx, gg_hmat *h, int nvec, const gg_dvd_params *p, double *eval, double *evec,
                         int *nloops, int *nmv, int *ierr) {
  if (!ctx || !h || h->ctx != ctx || nvec < 1 || nvec > h->ncf || !eval)
    return fail(GG_ERR_ARG, "gg_maneig: bad arguments");
  if (!h->emt_valid) return fail(GG_ERR_STATE, "gg_maneig: EMT not assembled");
  GG_CUDA(cudaSetDevice(ctx->device));
  const int flavour = p ? p->flavour : 0;
  const int precision = p ? p->precision : GG_FP64;
  const int ncf = h->ncf;
  int dummy_nl = 0, dummy_nmv = 0, dummy_ierr = 0;
  if (!nloops) nloops = &dummy_nl;
  if (!nmv) nmv = &dummy_nmv;
  if (!ierr) ierr = &dummy_ierr;
  *nloops = 0;
  *nmv = 0;
  *ierr = 0;
  GG_TRY(timer_start(ctx));
  ctx->stats[4] = 0;
  ctx->stats[5] = 0;
  ctx->stats[6] = spmv_bytes(h, precision, 1);
  if (ncf == 1) {  // trivial case (maneig.f90:122-137)
    eval[0] = 0.0;
    if (evec) evec[0] = 1.0;
    double ms = 0;
    GG_TRY(timer_stop(ctx, &ms));
    ctx->stats[3] = ms;
    return GG_OK;
  }
  DvdParams P;
  P.nume = nvec;
  P.niv = nvec;
  P.mblock = 1;
  P.crite = (p && p->crite > 0) ? p->crite : 1.0e-17;
  P.critc = (p && p->critc > 0) ? p->critc : 1.0e-9;
  P.critr = (p && p->critr > 0) ? p->critr : 1.0e-9;
  P.robust = (p && p->robust) ? 1 : 0;
  int nmax;
  if (flavour == 0) {  // rci90/maneig.f90:389-403
    P.lim = std::min(ncf, 2 * nvec + 60);
    P.maxiter = std::max(nvec * 200, ncf / 10);
    nmax = 2000;
  } else {  // rmcdhf90/maneig.f90:104-171
    P.lim = std::min(ncf, 2 * nvec + 40);
    P.maxiter = std::min(nvec * 200, ncf);
    nmax = 4000;
  }
  if (p && p->lim > 0) P.lim = std::min(ncf, p->lim);
  if (p && p->maxiter > 0) P.maxiter = p->maxiter;
  if (P.lim < nvec + 1 && P.lim != ncf) return fail(GG_ERR_ARG, "gg_maneig: LIM too small");
  if (P.lim > 1024) return fail(GG_ERR_ARG, "gg_maneig: LIM above 1024 is not supported");
  GG_TRY(refresh_sym_values(h));
  std::vector<double> ev, res;
  double mv_ms = 0;
  int mv_count = 0, nmv_total = 0, nl_total = 0;
  // Stage 1 (INIEST2, lib9290/iniest2.f90:49-95): lowest eigenvectors of the
  // leading ns x ns block, here by the same Davidson solver from unit vectors.
  const int ns = std::min(nmax, ncf);
  gg_hmat *blk = h;
  if (ns < ncf) GG_TRY(leading_block(h, ns, &blk));
  struct Guard {
    gg_hmat *b, *h;
    ~Guard() {
      if (b != h) gg_hmat_destroy(b);
    }
  } guard{blk, h};
  Dvd D1;
  {
    GG_TRY(refresh_sym_values(blk));
    DvdParams P1 = P;
    // stands in for INIEST2's dense DSPEVX: converge on the residual (no
    // coefficient test) from a sane first shift
    P1.robust = 1;
    P1.critc = 0.0;
    // block Davidson: up to NUME correction vectors per pass, so far fewer
    // projected eigenproblems than one vector per pass
    P1.mblock = nvec;
    P1.lim = std::min(ns, P.lim);
    if (ns < ncf && P1.lim < P.nume + 1) P1.lim = ns;
    GG_TRY(D1.init(ctx, blk, precision, ns, P1.lim));
    GG_CUDA(cudaMemcpyAsync(D1.diag.p, blk->dDiag.p, ns * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
    GG_TRY(unit_start(D1, blk, nvec));
    int nl = 0, ie = 0;
    GG_TRY(dvdson(D1, P1, ev, res, &nl, &ie));
    mv_ms += D1.mv_ms;
    mv_count += D1.mv_count;
    nmv_total += D1.nmv;
    nl_total += nl;
    *ierr = ie;
    ctx->stats[8] = nl;      // stage-1 (leading block) loops
    ctx->stats[9] = 0;       // stage-2 loops
    ctx->stats[10] = D1.mv_ms;
  }
  Dvd *Dout = &D1;
  Dvd D2;
  if (ns < ncf) {
    // Stage 2: GDVD on the whole block from the zero-padded estimates
    GG_TRY(D2.init(ctx, h, precision, ncf, P.lim));
    GG_CUDA(cudaMemcpyAsync(D2.diag.p, h->dDiag.p, ncf * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
    GG_CUDA(cudaMemcpy2DAsync(D2.B.p, D2.ld * 8, D1.B.p, D1.ld * 8, (size_t)ns * 8, nvec, cudaMemcpyDeviceToDevice,
                              ctx->stream));
    int nl = 0, ie = 0;
    GG_TRY(dvdson(D2, P, ev, res, &nl, &ie));
    mv_ms += D2.mv_ms;
    mv_count += D2.mv_count;
    nmv_total += D2.nmv;
    nl_total += nl;
    *ierr = ie;
    Dout = &D2;
    ctx->stats[9] = nl;
    ctx->stats[11] = D2.mv_ms;
    ctx->stats[12] = D2.mv_count;
  }
  for (int j = 0; j < nvec; ++j) eval[j] = ev[j];
  std::vector<double> hv;
  if (evec) {
    GG_CUDA(cudaMemcpy2DAsync(evec, (size_t)ncf * 8, Dout->B.p, Dout->ld * 8, (size_t)ncf * 8, nvec,
                              cudaMemcpyDeviceToHost, ctx->stream));
    GG_CUDA(cudaStreamSynchronize(ctx->stream));
    // dominant component positive (rci90/maneig.f90:532-555)
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
      if (v[ia] < 0.0)
        for (int i = 0; i < ncf; ++i) v[i] = -v[i];
    }
  }
  double ms = 0;
  GG_TRY(timer_stop(ctx, &ms));
  ctx->stats[3] = ms;
  ctx->stats[4] = mv_ms;
  ctx->stats[5] = mv_count;
  ctx->stats[13] = 1e3 * (D1.t_eig + D2.t_eig);    // host projected eigenproblem ms
  ctx->stats[14] = 1e3 * (D1.t_wait + D2.t_wait);  // host waits on device results ms
  *nloops = nl_total;
  *nmv = nmv_total;
  if (*ierr & 2048) return fail(GG_ERR_CONVERGE, "DVDSON: maximum number of iterations reached (IERR 2048)");
  return GG_OK;
}
