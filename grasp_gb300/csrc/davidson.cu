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
// The N-length kernels are tall-skinny FP64 products (N ~ 1e4..1e6 rows,
// k <= LIM columns). GB300 issues FP64 at a small fraction of its FP32 rate,
// so they are laid out for FP64 issue: transposed products give each thread
// 16 independent FMA chains (16 columns) and reduce through warp shuffles;
// row products tile 32 rows x 8 column chunks per block so that all SMs hold
// enough independent chains. All reductions run in a fixed order: results are
// reproducible run to run.
//
// Differences from the reference, all at rounding level:
//  - Gram-Schmidt is two-pass classical (CGS2), the reference's mgs_nrm is
//    two-pass modified; both leave the new vector orthonormal to working
//    precision.
//  - Dot products are blocked reductions, not sequential sums.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <type_traits>
#include <vector>

#include "gg_internal.cuh"

namespace gg {
namespace {

constexpr int TPB = 256;
constexpr int RT = 128;        // threads (= rows) per block of the block-pass Ritz kernel
constexpr int RR = 64;         // rows per block of the row kernels (k_ritz, k_csub)
constexpr int RCH = 4;         // column chunks per row: threads per row of the row kernels
constexpr int RTH = RR * RCH;  // threads per block of the row kernels
constexpr int CD_T = 256;      // threads of the column-dot kernel (8 warps)
constexpr int CD_G = 4;        // columns per warp group of the column-dot kernel
constexpr int CD_MAXR = 1024;  // rows per block of the column-dot kernel, at most
constexpr int CS_T = 256;      // threads of the column-sum kernel
constexpr int SV_MAX = 1024;   // LIM bound: shared copies of s and of the coefficients
constexpr int RC = 32;         // rows per block of MULTBC (one per lane)
constexpr int NCH = 8;         // warps of MULTBC

// device scalars of one pass (slots of Dvd::scal)
constexpr int SC_RN2 = 0;   // |r|^2 of the last Ritz residual
constexpr int SC_RHS = 1;   // RHSEPS of the robust shift
constexpr int SC_CONV = 2;  // 1.0 when |r| < CRITR
constexpr int SC_F1 = 3;    // 1/|w| after Gram-Schmidt pass 1
constexpr int SC_F2 = 4;    // 1/|w| after pass 2
constexpr int SC_N = 16;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// double-float helpers (Dekker / Knuth error-free transformations; this file
// is compiled without FMA contraction so that they stay exact)
struct df {
  float h, l;
};
__device__ __forceinline__ df two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  const float e = (a - (s - bb)) + (b - bb);
  return {s, e};
}
__device__ __forceinline__ df df_add(df a, df b) {
  df s = two_sum(a.h, b.h);
  const float t = s.l + a.l + b.l;
  const float h = s.h + t;
  return {h, t - (h - s.h)};
}

// Sum of one value per thread over a block of NT threads, in a fixed order;
// the result is valid in thread 0.
template <int NT> __device__ __forceinline__ double block_sum(double v, double *red) {
  v = warp_sum(v);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
#pragma unroll
    for (int q = 0; q < NT / 32; ++q) t += red[q];
  return t;
}

// ---------------------------------------------------------------------------
// The parameters of one Davidson pass. Graph replays read them from device
// memory (written by the graph's first node from pinned host memory); the
// launch-by-launch path passes them by value. The kernels are the same.
// ---------------------------------------------------------------------------
struct IterParams {
  int c;         // column written by this pass
  int k;         // basis columns the Ritz vector is built from
  double lam;    // EIGVAL(INDX)
  double gap;    // NEWVEC's GAP for INDX
  double dl;     // NEWVEC's DL for INDX
  double critr;  // CRITR
};
struct PSrc {
  const IterParams *dp;
  IterParams hv;
  __device__ __forceinline__ IterParams get() const { return dp ? *dp : hv; }
};

// Last block of a grid to arrive (after its own partial was written):
// true in every thread of that block.
__device__ __forceinline__ bool arrive_last(unsigned *counter, bool *flag) {
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) *flag = (atomicAdd(counter, 1u) == gridDim.x - 1);
  __syncthreads();
  return *flag;
}


// Row products of the row kernels: thread (row rl, chunk ch) of a block of
// RR rows x RCH chunks sums X[i, j] v[j] over its chunk of columns with four
// independent chains (loads of several columns in flight); the chunk sums
// are combined in chunk order through shared memory by the caller.
__device__ __forceinline__ double chunk_dot(const double *__restrict__ px, int64_t ld, const double *v, int jb,
                                            int je) {
  double t0 = 0.0, t1 = 0.0, t2 = 0.0, t3 = 0.0;
  int j = jb;
#pragma unroll 2
  for (; j + 3 < je; j += 4) {
    const size_t o = (size_t)j * ld;
    const double x0 = px[o], x1 = px[o + ld], x2 = px[o + 2 * ld], x3 = px[o + 3 * ld];
    t0 = fma(x0, v[j], t0);
    t1 = fma(x1, v[j + 1], t1);
    t2 = fma(x2, v[j + 2], t2);
    t3 = fma(x3, v[j + 3], t3);
  }
  for (; j < je; ++j) t0 = fma(px[(size_t)j * ld], v[j], t0);
  return (t0 + t1) + (t2 + t3);
}

// Ritz vector and residual (NEWVEC, dvdson.f90:1100-1111):
//   b = BASIS s ; a = AB s ; r = a - lambda b -> BASIS(:, c), AB(:, c).
// The last block adds the per-block |r|^2 in order and derives NEWVEC's
// robust shift (dvdson.f90:1139-1160) and the convergence flag.
__global__ void __launch_bounds__(RTH) k_ritz(double *B, double *AB, int64_t ld, PSrc ps,
                                              const double *__restrict__ s, int n, double *__restrict__ part,
                                              unsigned *__restrict__ counter, double *__restrict__ scal) {
  const IterParams P = ps.get();
  const int k = P.k, c = P.c;
  __shared__ double sv[SV_MAX];
  __shared__ double pb[RCH][RR], pa[RCH][RR];
  __shared__ double red[RTH / 32];
  __shared__ bool last;
  for (int j = threadIdx.x; j < k; j += RTH) sv[j] = s[j];
  __syncthreads();
  const int rl = threadIdx.x % RR, ch = threadIdx.x / RR;
  const int i = blockIdx.x * RR + rl;
  const int per = (k + RCH - 1) / RCH, jb = min(k, ch * per), je = min(k, jb + per);
  double bs = 0.0, as = 0.0;
  if (i < n) {
    bs = chunk_dot(B + i, ld, sv, jb, je);
    as = chunk_dot(AB + i, ld, sv, jb, je);
  }
  pb[ch][rl] = bs;
  pa[ch][rl] = as;
  __syncthreads();
  double r = 0.0;
  if (ch == 0 && i < n) {
    double bb = pb[0][rl], aa = pa[0][rl];
#pragma unroll
    for (int q = 1; q < RCH; ++q) {
      bb += pb[q][rl];
      aa += pa[q][rl];
    }
    r = fma(-P.lam, bb, aa);
    B[(size_t)c * ld + i] = bb;
    AB[(size_t)c * ld + i] = r;
  }
  const double t = block_sum<RTH>(r * r, red);
  if (threadIdx.x == 0) part[blockIdx.x] = t;
  if (!arrive_last(counter, &last)) return;
  double u = 0.0;
  for (int q = threadIdx.x; q < (int)gridDim.x; q += RTH) u += __ldcg(part + q);
  __syncthreads();
  u = block_sum<RTH>(u, red);
  if (threadIdx.x == 0) {
    const double res = sqrt(u);
    scal[SC_RN2] = u;
    scal[SC_RHS] = (P.gap > res) ? sqrt(P.dl * res) : fmin(P.dl, sqrt(P.dl));
    scal[SC_CONV] = (res < P.critr) ? 1.0 : 0.0;
    *counter = 0u;
  }
}

// robust shift + GDVD diagonal preconditioner (gdvd.f90:114-129) of column c:
//   r <- r - rhseps b ; DIAG <- DIAG - lambda ; w = r/DIAG (|DIAG| > 1e-6)
//   or r*1e6 ; DIAG <- DIAG + lambda ; BASIS column <- w
__device__ __forceinline__ double precond_row(double *bc, double *rc, double *diag, int i, double rhseps, double lam) {
  const double rr = fma(-rhseps, bc[i], rc[i]);
  rc[i] = rr;
  const double d = diag[i] - lam;
  const double w = (fabs(d) > 1.0e-06) ? rr / d : rr * 1.0e06;
  bc[i] = w;
  diag[i] = d + lam;
  return w;
}

__global__ void k_precond(double *B, double *AB, int64_t ld, PSrc ps, const double *__restrict__ scal,
                          double *__restrict__ diag, int n) {
  const IterParams P = ps.get();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  precond_row(B + (size_t)P.c * ld, AB + (size_t)P.c * ld, diag, i, scal[SC_RHS], P.lam);
}

// out[j] = f sum_i X[i, j] w[i] for j < k = c + kofs, w = column c of W
// (c from the pass parameters; f = scal[fslot], or 1 when fslot < 0).
// PRE = true first applies the shift and preconditioner to column c (W is
// then BASIS; AB and DIAG are updated too). Skipped entirely when skip
// points to a non-zero flag.
//
// Layout: block b owns rows [b R, b R + R); it stages w for them in shared
// memory, then warp g takes column groups g, g + 8, ... of 4 columns: lanes
// stride the rows (coalesced 256-byte loads, 4 independent FMA chains) and
// a transpose butterfly reduces the 4 sums over the 32 lanes with 6 adds per
// lane. The last block adds the per-block partials in block order.
template <bool PRE>
__global__ void __launch_bounds__(CD_T) k_cdots(const double *X, int64_t ld, PSrc ps, int kofs, double *W, double *AB,
                                                double *diag, const double *scal, const double *skip, int n,
                                                int rows, int pitch, double *__restrict__ part) {
  if (skip && *skip != 0.0) return;
  const IterParams P = ps.get();
  const int c = P.c, k = c + kofs;
  __shared__ double ws[CD_MAXR];
  const int r0 = blockIdx.x * rows;
  const int nr = min(rows, n - r0);
  double *wc = W + (size_t)c * ld;
  if (PRE) {
    const double rhseps = scal[SC_RHS];
    double *rc = AB + (size_t)c * ld;
    for (int t = threadIdx.x; t < nr; t += CD_T) ws[t] = precond_row(wc, rc, diag, r0 + t, rhseps, P.lam);
  } else {
    for (int t = threadIdx.x; t < nr; t += CD_T) ws[t] = wc[r0 + t];
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int ngrp = (k + CD_G - 1) / CD_G;
  const bool hi16 = (lane & 16) != 0, hi8 = (lane & 8) != 0;
  for (int g = wid; g < ngrp; g += CD_T / 32) {
    const int j0 = g * CD_G;
    double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
    const double *x0 = X + (size_t)j0 * ld + r0;
    if (j0 + CD_G <= k) {
      for (int t = lane; t < nr; t += 32) {
        const double wv = ws[t];
        a0 = fma(x0[t], wv, a0);
        a1 = fma(x0[t + ld], wv, a1);
        a2 = fma(x0[t + 2 * ld], wv, a2);
        a3 = fma(x0[t + 3 * ld], wv, a3);
      }
    } else {
      const int m = k - j0;
      for (int t = lane; t < nr; t += 32) {
        const double wv = ws[t];
        a0 = fma(x0[t], wv, a0);
        if (m > 1) a1 = fma(x0[t + ld], wv, a1);
        if (m > 2) a2 = fma(x0[t + 2 * ld], wv, a2);
      }
    }
    // lanes with bit 4 clear keep columns 0, 1; set: 2, 3
    const double s0 = hi16 ? a0 : a2, s1 = hi16 ? a1 : a3;
    const double k0 = (hi16 ? a2 : a0) + __shfl_xor_sync(0xffffffffu, s0, 16);
    const double k1 = (hi16 ? a3 : a1) + __shfl_xor_sync(0xffffffffu, s1, 16);
    // bit 3 clear keeps the first of the pair
    double v = (hi8 ? k1 : k0) + __shfl_xor_sync(0xffffffffu, hi8 ? k0 : k1, 8);
    v += __shfl_xor_sync(0xffffffffu, v, 4);
    v += __shfl_xor_sync(0xffffffffu, v, 2);
    v += __shfl_xor_sync(0xffffffffu, v, 1);
    const int q = (lane >> 3) & 3;  // column of v
    if ((lane & 7) == 0 && j0 + q < k) part[(size_t)(j0 + q) * pitch + blockIdx.x] = v;
  }
}

// out[j] = f sum_b part[j pitch + b] over the nb block partials of k_cdots,
// j < k = c + kofs; one block per column, partials added in a fixed order
// (f = scal[fslot], or 1 when fslot < 0). packed: out is a packed upper
// matrix and the sums go to its column c.
__global__ void __launch_bounds__(CS_T) k_colsum(const double *__restrict__ part, int pitch, int nb, PSrc ps, int kofs,
                                                 const double *skip, const double *__restrict__ scal, int fslot,
                                                 double *__restrict__ out, int packed) {
  if (skip && *skip != 0.0) return;
  const IterParams P = ps.get();
  const int j = blockIdx.x;
  if (j >= P.c + kofs) return;
  if (packed) out += (size_t)P.c * (P.c + 1) / 2;  // column c of a packed upper matrix
  __shared__ double red[CS_T / 32];
  const double *pj = part + (size_t)j * pitch;
  double u = 0.0;
  for (int b = threadIdx.x; b < nb; b += CS_T) u += pj[b];
  u = block_sum<CS_T>(u, red);
  if (threadIdx.x == 0) out[j] = (fslot >= 0) ? scal[fslot] * u : u;
}

// Gram-Schmidt update of column c:
//   w <- f w - sum_{j<c} X[:, j] coef[j]   (f = scal[fin], or 1 when fin < 0)
// and scal[fout] = 1/|w| (the last block adds the block partials in order).
__global__ void __launch_bounds__(RTH) k_csub(double *X, int64_t ld, PSrc ps, const double *__restrict__ coef,
                                              const double *skip, int fin, int fout, int n,
                                              double *__restrict__ part, unsigned *__restrict__ counter,
                                              double *scal) {
  if (skip && *skip != 0.0) return;
  const IterParams P = ps.get();
  const int k = P.c;
  __shared__ double cs[SV_MAX];
  __shared__ double pt[RCH][RR];
  __shared__ double red[RTH / 32];
  __shared__ bool last;
  for (int j = threadIdx.x; j < k; j += RTH) cs[j] = coef[j];
  __syncthreads();
  const int rl = threadIdx.x % RR, ch = threadIdx.x / RR;
  const int i = blockIdx.x * RR + rl;
  const int per = (k + RCH - 1) / RCH, jb = min(k, ch * per), je = min(k, jb + per);
  pt[ch][rl] = (i < n) ? chunk_dot(X + i, ld, cs, jb, je) : 0.0;
  __syncthreads();
  double wn = 0.0;
  if (ch == 0 && i < n) {
    double t = pt[0][rl];
#pragma unroll
    for (int q = 1; q < RCH; ++q) t += pt[q][rl];
    double *w = X + (size_t)k * ld + i;
    const double w0 = (fin >= 0) ? scal[fin] * (*w) : *w;
    wn = w0 - t;
    *w = wn;
  }
  const double sq = block_sum<RTH>(wn * wn, red);
  if (threadIdx.x == 0) part[blockIdx.x] = sq;
  if (!arrive_last(counter, &last)) return;
  double u = 0.0;
  for (int q = threadIdx.x; q < (int)gridDim.x; q += RTH) u += __ldcg(part + q);
  __syncthreads();
  u = block_sum<RTH>(u, red);
  if (threadIdx.x == 0) {
    scal[fout] = 1.0 / sqrt(u);
    *counter = 0u;
  }
}

// ---------------------------------------------------------------------------
// Block passes (MBLOCK > 1): the Ritz vectors and residuals of all targets
// in one sweep over BASIS and AB, then the shifts and preconditioners of the
// targets NEWVEC keeps, in NEWVEC's order.
// ---------------------------------------------------------------------------
constexpr int MT_MAX = 16;     // targets per sweep
constexpr int MT_SMEM = 4096;  // doubles of Ritz coefficients held in shared memory

// For targets t < nt: b_t = BASIS s_t -> T(:, 2t), r_t = AB s_t - lambda_t b_t
// -> T(:, 2t + 1), rn2[t] = |r_t|^2 (block partials added in order by the
// last block). s_t = S + t k.
// Targets [g NT, g NT + NT) for g = blockIdx.y (nt in all); the last block
// of the whole grid adds the partials of every target in block order.
template <int NT>
__global__ void __launch_bounds__(RT) k_ritz_multi(const double *__restrict__ B, const double *__restrict__ AB,
                                                   int64_t ld, int k, int nt, const double *__restrict__ S,
                                                   const double *__restrict__ lam, double *__restrict__ T, int n,
                                                   double *__restrict__ part, unsigned *__restrict__ counter,
                                                   double *__restrict__ rn2) {
  pdl_wait();
  __shared__ double sv[MT_SMEM];
  __shared__ double red[RT / 32];
  __shared__ bool last;
  const int t0 = blockIdx.y * NT;
  for (int q = threadIdx.x; q < NT * k; q += RT) sv[q] = S[(size_t)t0 * k + q];
  __syncthreads();
  const int i = blockIdx.x * RT + threadIdx.x;
  double bacc[NT], aacc[NT];
#pragma unroll
  for (int t = 0; t < NT; ++t) bacc[t] = aacc[t] = 0.0;
  if (i < n) {
    for (int j = 0; j < k; ++j) {
      const double bj = B[(size_t)j * ld + i], aj = AB[(size_t)j * ld + i];
#pragma unroll
      for (int t = 0; t < NT; ++t) {
        bacc[t] = fma(bj, sv[t * k + j], bacc[t]);
        aacc[t] = fma(aj, sv[t * k + j], aacc[t]);
      }
    }
  }
#pragma unroll
  for (int t = 0; t < NT; ++t) {
    double r = 0.0;
    if (i < n) {
      r = fma(-lam[t0 + t], bacc[t], aacc[t]);
      T[(size_t)(2 * (t0 + t)) * ld + i] = bacc[t];
      T[(size_t)(2 * (t0 + t) + 1) * ld + i] = r;
    }
    const double sq = block_sum<RT>(r * r, red);
    if (threadIdx.x == 0) part[(size_t)(t0 + t) * gridDim.x + blockIdx.x] = sq;
    __syncthreads();
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = (atomicAdd(counter, 1u) == gridDim.x * gridDim.y - 1);
  __syncthreads();
  if (!last) return;
  for (int t = 0; t < nt; ++t) {
    double u = 0.0;
    for (int q = threadIdx.x; q < (int)gridDim.x; q += RT) u += __ldcg(part + (size_t)t * gridDim.x + q);
    u = block_sum<RT>(u, red);
    if (threadIdx.x == 0) rn2[t] = u;
    __syncthreads();
  }
  if (threadIdx.x == 0) *counter = 0u;
}

struct PrecList {
  int m;
  int col[MT_MAX];      // BASIS column of the new vector
  int t[MT_MAX];        // its target (columns 2t, 2t+1 of T)
  double lam[MT_MAX];   // EIGVAL(INDX)
  double rhs[MT_MAX];   // RHSEPS
};

// shifts and GDVD preconditioners (gdvd.f90:114-129) of the kept targets in
// NEWVEC's order, DIAG updated after each as in the reference
__global__ void k_precond_multi(double *__restrict__ B, const double *__restrict__ T, int64_t ld, PrecList L,
                                double *__restrict__ diag, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double dg = diag[i];
  for (int q = 0; q < L.m; ++q) {
    const double b = T[(size_t)(2 * L.t[q]) * ld + i], r = T[(size_t)(2 * L.t[q] + 1) * ld + i];
    const double rr = fma(-L.rhs[q], b, r);
    const double d = dg - L.lam[q];
    B[(size_t)L.col[q] * ld + i] = (fabs(d) > 1.0e-06) ? rr / d : rr * 1.0e06;
    dg = d + L.lam[q];
  }
  diag[i] = dg;
}

// NEWVEC's choices for a block pass (dvdson.f90:1002-1172) on the device, so
// that the Ritz sweep, the preconditioners and the block pass follow each
// other without a host round trip. Inputs per candidate target t (in
// TSTSEL's order): its eigenvalue, GAP and DL (from EIGVAL and OLDVAL on the
// host); rn2[t] = |r_t|^2 from the Ritz sweep. Same decisions in the same
// order as the reference: a target with |r| < CRITR converges (DONE when all
// have), the others are kept with RHSEPS = sqrt(DL |r|) when GAP > |r| and
// min(DL, sqrt(DL)) otherwise, up to LIMADD - KPASS of them.
struct NvIn {
  int nt, kpass, limadd;
  double critr;
  double lam[MT_MAX], gap[MT_MAX], dl[MT_MAX];
};
struct NvOut {
  int nadded, done;
  double res[MT_MAX];
};
// hi + lo FP32 pair of an FP64 value (its nearest float and the rest)
__device__ __forceinline__ float2 split2(double v) {
  const float h = __double2float_rn(v);
  return make_float2(h, __double2float_rn(v - (double)h));
}

// a / b to about 2^-46 relative: an FP32 reciprocal of b refined by one
// Newton step on the quotient (three FP64 operations instead of the FP64
// division's longer sequence; |b| > 1e-6 here, far inside FP32's range
// after the cast for the matrices' diagonal scales)
__device__ __forceinline__ double quot(double a, double b) {
  const double y = (double)__frcp_rn(__double2float_rn(b));
  const double q0 = a * y;
  return fma(fma(-b, q0, a), y, q0);
}

// NEWVEC's choices and the preconditioners of the kept targets in one
// kernel: every CTA makes the choices (the square roots in parallel, lane t;
// the choices by thread 0 in TSTSEL's order), block 0 also writes them for
// the host; then each thread preconditions its row for the kept targets in
// NEWVEC's order (GDVD, gdvd.f90:114-129, DIAG updated after each as in the
// reference) and zeroes columns kpass + L.m .. kpass + mg - 1 of the pass
// (the block pass then drops them)
__global__ void k_newvec_precond(const NvIn *__restrict__ in, const double *__restrict__ rn2,
                                 NvOut *__restrict__ out, double *__restrict__ B, const double *__restrict__ T,
                                 int64_t ld, double *__restrict__ diag, int n, int mg, int kpass,
                                 float2 *__restrict__ wx) {
  pdl_wait();
  __shared__ double sres[MT_MAX], srhs[MT_MAX];
  __shared__ PrecList L;
  const int nt = in->nt, t = threadIdx.x;
  if (t < nt) {
    const double res = sqrt(rn2[t]), gap = in->gap[t], dl = in->dl[t];
    sres[t] = res;
    if (blockIdx.x == 0) out->res[t] = res;
    srhs[t] = (gap > res) ? sqrt(dl * res) : fmin(dl, sqrt(dl));
  }
  __syncthreads();
  if (t == 0) {
    PrecList l;
    l.m = 0;
    int icvc = 0, nadded = 0, done = 0;
    for (int i = 0; i < nt; ++i) {
      const double res = sres[i];
      if (res < in->critr) {
        ++icvc;
        if (icvc < nt) continue;
        done = 1;
        break;
      }
      ++nadded;
      l.col[l.m] = in->kpass + nadded - 1;
      l.t[l.m] = i;
      l.lam[l.m] = in->lam[i];
      l.rhs[l.m] = srhs[i];
      ++l.m;
      if (nadded + in->kpass == in->limadd) break;
    }
    L = l;
    if (blockIdx.x == 0) {
      out->nadded = nadded;
      out->done = done;
    }
  }
  __syncthreads();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int m = L.m;
  double dg = diag[i];
  for (int q = 0; q < m; ++q) {
    const int tq = L.t[q];
    const double b = T[(size_t)(2 * tq) * ld + i], r = T[(size_t)(2 * tq + 1) * ld + i];
    const double rr = fma(-L.rhs[q], b, r);
    const double lam = L.lam[q];
    const double d = dg - lam;
    const double v = (fabs(d) > 1.0e-06) ? quot(rr, d) : rr * 1.0e06;
    B[(size_t)L.col[q] * ld + i] = v;
    if (wx) wx[(size_t)(L.col[q] - kpass) * ld + i] = split2(v);
    dg = d + lam;
  }
  diag[i] = dg;
  for (int q = m; q < mg; ++q) {
    B[(size_t)(kpass + q) * ld + i] = 0.0;
    if (wx) wx[(size_t)q * ld + i] = make_float2(0.f, 0.f);
  }
}

// column c <- scal[fslot] * column c; with xs, also its hi+lo split for the matvec
__global__ void k_cscale(double *X, int64_t ld, PSrc ps, const double *skip, const double *__restrict__ scal,
                         int fslot, int n, float2 *__restrict__ xs) {
  if (skip && *skip != 0.0) return;
  const IterParams P = ps.get();
  const double f = scal[fslot];
  double *w = X + (size_t)P.c * ld;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double v = f * w[i];
    w[i] = v;
    if (xs) {
      const float hv = __double2float_rn(v);
      xs[i] = make_float2(hv, __double2float_rn(v - (double)hv));
    }
  }
}

// out[:, j] = sum_{q<k} X[:, q] C[q + j k], j < m   (MULTBC)
// Block = 32 rows x 8 warps; warp w computes output columns w, w+8, ... with
// up to 8 accumulators each pass; C is read through the read-only cache.
__global__ void __launch_bounds__(TPB) k_multbc(const double *__restrict__ X, int64_t ld, int k,
                                                const double *__restrict__ C, int m, double *__restrict__ out, int n) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int i = blockIdx.x * RC + lane;
  if (i >= n) return;
  for (int jb = wid; jb < m; jb += NCH * 8) {
    double acc[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) acc[u] = 0.0;
    for (int q = 0; q < k; ++q) {
      const double x = X[(size_t)q * ld + i];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int j = jb + u * NCH;
        if (j < m) acc[u] = fma(x, __ldg(C + (size_t)j * k + q), acc[u]);
      }
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int j = jb + u * NCH;
      if (j < m) out[(size_t)j * ld + i] = acc[u];
    }
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

// ---------------------------------------------------------------------------
// Block Gram-Schmidt for the block pass (MBLOCK > 1). The m new columns
// kpass .. kpass+m-1 (kpass = pv[0].c on the device) are orthogonalised
// against the basis by two passes of block classical Gram-Schmidt, then among
// themselves by two rounds of Cholesky QR. A column whose Cholesky pivot is
// not above 1e-14 of its own squared norm (or is zero) is dropped and the
// kept columns are compacted: the pass adds nk <= m columns (bst[0]). The
// span is the one of DVDSON's MGS_NRM (dvdson.f90:1417-1508), which
// normalises such a column instead. Then OP per kept column and the new
// columns of S (packed upper) from one block of dot products. The dot
// products are per-CTA partials over row ranges, added in CTA order.
//   MODE 0  X = B(:, 0:kpass),      W = B(:, kpass:kpass+m)
//   MODE 1  X = W = B(:, kpass:kpass+c), c = bst[0]
//   MODE 2  X = B(:, 0:kpass+c),    W = AB(:, kpass:kpass+c)
// ---------------------------------------------------------------------------
constexpr int BD_R = 64, BD_T = 256, BD_AC = 32, BD_RED = 1024;
constexpr int BD_PAIRS = (BD_AC * MT_MAX + BD_T - 1) / BD_T;

template <int MODE>
__global__ void __launch_bounds__(BD_T) k_bd_dots(const double *__restrict__ B, const double *__restrict__ AB,
                                                  int64_t ld, const IterParams *__restrict__ pv, int m,
                                                  const int *__restrict__ bst, int n, int cpc,
                                                  double *__restrict__ part, int ps) {
  pdl_wait();
  __shared__ double Bs[BD_R * MT_MAX];       // [i][q]
  __shared__ double As[BD_R * (BD_AC + 1)];  // [i][a]
  const int kpass = pv[0].c;
  const int nb = (MODE == 0) ? m : bst[0];
  if (nb <= 0) return;
  const int na = (MODE == 0) ? kpass : (MODE == 1 ? nb : kpass + nb);
  const int a0 = (MODE == 1) ? kpass : 0;
  const double *Wb = ((MODE == 2) ? AB : B) + (size_t)kpass * ld;
  const double *Xb = B + (size_t)a0 * ld;
  double *out = part + (size_t)blockIdx.x * ps;
  const int rbeg = blockIdx.x * cpc * BD_R, rend = min(n, rbeg + cpc * BD_R);
  for (int ac = blockIdx.y * BD_AC; ac < na; ac += gridDim.y * BD_AC) {
    const int nac = min(BD_AC, na - ac), np = nac * nb;
    double acc[BD_PAIRS];
#pragma unroll
    for (int k = 0; k < BD_PAIRS; ++k) acc[k] = 0.0;
    for (int r0 = rbeg; r0 < rend; r0 += BD_R) {
      const int nr = min(BD_R, rend - r0);
      for (int idx = threadIdx.x; idx < nr * nb; idx += BD_T) {
        const int i = idx % nr, q = idx / nr;
        Bs[i * MT_MAX + q] = Wb[(size_t)q * ld + r0 + i];
      }
      for (int idx = threadIdx.x; idx < nr * nac; idx += BD_T) {
        const int i = idx % nr, a = idx / nr;
        As[i * (BD_AC + 1) + a] = Xb[(size_t)(ac + a) * ld + r0 + i];
      }
      __syncthreads();
#pragma unroll
      for (int k = 0; k < BD_PAIRS; ++k) {
        const int pr = threadIdx.x + k * BD_T;
        if (pr < np) {
          const int a = pr % nac, q = pr / nac;
          double s0 = 0.0, s1 = 0.0;
          int i = 0;
          for (; i + 1 < nr; i += 2) {
            s0 = fma(As[i * (BD_AC + 1) + a], Bs[i * MT_MAX + q], s0);
            s1 = fma(As[(i + 1) * (BD_AC + 1) + a], Bs[(i + 1) * MT_MAX + q], s1);
          }
          if (i < nr) s0 = fma(As[i * (BD_AC + 1) + a], Bs[i * MT_MAX + q], s0);
          acc[k] += s0 + s1;
        }
      }
      __syncthreads();
    }
#pragma unroll
    for (int k = 0; k < BD_PAIRS; ++k) {
      const int pr = threadIdx.x + k * BD_T;
      if (pr < np) out[(ac + pr % nac) * nb + pr / nac] = acc[k];
    }
  }
}

// sum over the CTA partials of k_bd_dots for outputs o0 .. o0+32: lane = output,
// warps take CTAs w, w + nw, ...; the warp sums are then added in warp order
__device__ __forceinline__ double bd_reduce(const double *__restrict__ part, int ps, int ntiles, int o, bool ok,
                                           double *red) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  double u = 0.0;
  if (ok)
#pragma unroll 8
    for (int t = w; t < ntiles; t += nw) u += part[(size_t)t * ps + o];
  red[w * 32 + lane] = u;
  __syncthreads();
  double sum = 0.0;
  if (w == 0)
    for (int v = 0; v < nw; ++v) sum += red[v * 32 + lane];
  return sum;
}

// the same over double-float partials (the split kernels' CTA sums), added
// in double-float on the FP32 pipes: GB300 issues FP64 adds at about 1/70
// of its FP32 rate, and these reductions run on few SMs
__device__ __forceinline__ double bd_reduce(const float2 *__restrict__ part, int ps, int ntiles, int o, bool ok,
                                           float2 *red) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  df u{0.f, 0.f};
  if (ok)
#pragma unroll 8
    for (int t = w; t < ntiles; t += nw) {
      const float2 p = part[(size_t)t * ps + o];
      u = df_add(u, df{p.x, p.y});
    }
  red[w * 32 + lane] = make_float2(u.h, u.l);
  __syncthreads();
  df sum{0.f, 0.f};
  if (w == 0)
    for (int v = 0; v < nw; ++v) {
      const float2 p = red[v * 32 + lane];
      sum = df_add(sum, df{p.x, p.y});
    }
  return (double)sum.h + (double)sum.l;
}

// MODE 0: Gram-Schmidt coefficients C = X^T W (kpass x m, row a at a m);
// MODE 2: the new columns of S into dS (packed upper, S(i, j) at
// j (j+1)/2 + i - kpass (kpass+1)/2: the columns from kpass on).
// 32 outputs per CTA. P: the partials' type (double, or float2 double-float
// sums of the split kernels). set_bst: block 0 also starts the pass's
// column counts (bst = {m, m}), read first by the Gram dots after it.
template <int MODE, typename P>
__global__ void __launch_bounds__(BD_T) k_bd_reduce(const IterParams *__restrict__ pv, int m,
                                                    int *__restrict__ bst, const P *__restrict__ part,
                                                    int ps, int ntiles, double *__restrict__ C,
                                                    double *__restrict__ dS, int set_bst, int cgs) {
  pdl_wait();
  __shared__ P red[BD_T];
  // cgs (MODE 0, split form): 0 = first pass (its partials also hold the
  // new columns' squared norms, at na nb + q), 1 = second pass (skipped
  // when bst[2] says the first one was enough); -1 neither
  if (MODE == 0 && cgs == 1 && bst[2]) return;
  const int kpass = pv[0].c;
  if (MODE == 0 && set_bst && blockIdx.x == 0 && threadIdx.x == 0) {
    bst[0] = m;
    bst[1] = m;
  }
  const int nb = (MODE == 0) ? m : bst[0];
  const int na = (MODE == 0) ? kpass : kpass + nb;
  const int nout = na * nb + ((MODE == 0 && cgs == 0) ? nb : 0);
  const int o = blockIdx.x * 32 + (threadIdx.x & 31);
  if (nb <= 0 || (int)blockIdx.x * 32 >= nout) return;
  const bool ok = o < nout;
  const double sum = bd_reduce(part, ps, ntiles, o, ok, red);
  if (threadIdx.x >= 32 || !ok) return;
  if (MODE == 0) {
    C[o] = sum;
  } else {
    const int a = o / nb, j = kpass + o % nb;
    if (a <= j) dS[(size_t)j * (j + 1) / 2 + a - (size_t)kpass * (kpass + 1) / 2] = sum;
  }
}

// Cholesky QR step: G = W^T W (reduced from the partials), G = R^T R with
// drops; C[q MT_MAX + c] = the map from current column q to kept column c
// (R^-1 on the kept rows), bst[1] = columns before, bst[0] = kept. The last
// round also writes the matvec skip flags of the m columns. Right-looking
// Cholesky on the Schur complement in shared memory by one warp (one column
// per step), then one lane per column of R^-1. When G is
// within 1e-8 of the identity (the second round, after a first one), R^-1 =
// I - F to first order (F the upper triangle of G - I, diagonal halved):
// its error is O(|G - I|^2) and it needs no serial chain of square roots and
// divisions, which are slow in FP64.
template <typename P>
__global__ void __launch_bounds__(BD_RED) k_bd_chol(int m, int *__restrict__ bst, const P *__restrict__ part,
                                                    int ps, int ntiles, double *__restrict__ C,
                                                    double *__restrict__ skipf, int last) {
  pdl_wait();
  __shared__ P red[BD_RED];
  __shared__ double G[MT_MAX * MT_MAX];   // Schur complement [q][q']
  __shared__ double R[MT_MAX * MT_MAX];   // row c of R over the current columns
  __shared__ double Ri[MT_MAX * MT_MAX];  // R^-1 of the kept columns [i][c]
  __shared__ double g0[MT_MAX], invd[MT_MAX];
  __shared__ int keep[MT_MAX], pos[MT_MAX];
  const int nb = bst[0];
  const int tid = threadIdx.x;
  // 8 groups of 32 outputs, 4 warps per group
  const int grp = tid >> 7, sub = (tid >> 5) & 3, lane = tid & 31;
  const int o = grp * 32 + lane;
  const bool ok = nb > 0 && o < nb * nb;
  if constexpr (std::is_same<P, double>::value) {
    double u = 0.0;
    if (ok)
#pragma unroll 8
      for (int t = sub; t < ntiles; t += 4) u += part[(size_t)t * ps + o];
    red[tid] = u;
    __syncthreads();
    if (sub == 0 && ok) G[o] = ((red[tid] + red[tid + 32]) + red[tid + 64]) + red[tid + 96];
  } else {
    // double-float sums (FP32 pipes)
    df u{0.f, 0.f};
    if (ok)
#pragma unroll 8
      for (int t = sub; t < ntiles; t += 4) {
        const float2 p = part[(size_t)t * ps + o];
        u = df_add(u, df{p.x, p.y});
      }
    red[tid] = make_float2(u.h, u.l);
    __syncthreads();
    if (sub == 0 && ok) {
      df g{0.f, 0.f};
#pragma unroll
      for (int v = 0; v < 4; ++v) g = df_add(g, df{red[tid + 32 * v].x, red[tid + 32 * v].y});
      G[o] = (double)g.h + (double)g.l;
    }
  }
  __syncthreads();
  const bool near = __syncthreads_and(tid >= nb * nb || fabs(G[tid] - ((tid / nb == tid % nb) ? 1.0 : 0.0)) <= 1e-8);
  if (near) {
    if (tid < MT_MAX * MT_MAX) {
      const int q = tid / MT_MAX, c = tid % MT_MAX;
      double v = 0.0;
      if (q < nb && c < nb) v = (q == c) ? 1.0 - 0.5 * (G[q * nb + q] - 1.0) : (q < c ? -G[q * nb + c] : 0.0);
      C[tid] = v;
    }
    if (tid == 0) bst[1] = nb;  // bst[0] stays nb
    if (last && tid < m) skipf[tid] = (tid < nb) ? 0.0 : 1.0;
    return;
  }
  // The factorisation by warp 0 alone: its steps then need warp syncs only.
  // GB300 issues an FP64 warp instruction in about as many cycles as FP32
  // issues 70, so the serial chain is kept short: G16 holds G with a fixed
  // row pitch of 16 (no division by nb), only the lower triangle of the
  // Schur complement is updated, its entries listed with their column
  // descending so that step q updates a prefix of the list (ceil(T_q / 32)
  // instructions, T_q = (nb - q - 1)(nb - q) / 2), and 1/sqrt(pivot) is an
  // FP32 estimate refined by two Newton steps.
  if (tid >= 32) return;
  double *G16 = Ri;  // R^-1 is formed after the factorisation; until then its storage holds G
  __shared__ unsigned char pa[MT_MAX * (MT_MAX + 1) / 2], pb[MT_MAX * (MT_MAX + 1) / 2];
  for (int e = lane; e < MT_MAX * MT_MAX; e += 32) {
    const int r = e >> 4, c = e & 15;
    G16[e] = (r < nb && c < nb) ? G[r * nb + c] : 0.0;
  }
  if (lane == 0) {
    int e = 0;
    for (int c = nb - 1; c >= 0; --c)
      for (int r = c; r < nb; ++r) {
        pa[e] = (unsigned char)r;
        pb[e] = (unsigned char)c;
        ++e;
      }
  }
  if (lane < nb) pos[lane] = -1;
  __syncwarp();
  if (lane < nb) g0[lane] = G16[lane * 17];
  __syncwarp();
  int nk = 0;  // uniform
  for (int q = 0; q < nb; ++q) {
    const double dq = G16[q * 17];
    if (dq > 1e-14 * g0[q] && dq > 1e-300) {
      double inv;
      if (dq > 1e-36 && dq < 1e36) {
        double y = (double)rsqrtf((float)dq);
        y = y * fma(-0.5 * dq * y, y, 1.5);
        inv = y * fma(-0.5 * dq * y, y, 1.5);
      } else {
        inv = rsqrt(dq);
      }
      const double rd = dq * inv;
      if (lane < nb) R[nk * MT_MAX + lane] = (lane < q) ? 0.0 : (lane == q ? rd : G16[lane * 16 + q] * inv);
      __syncwarp();
      const int tq = (nb - q - 1) * (nb - q) / 2;
      for (int e = lane; e < tq; e += 32) {
        const int r = pa[e], c = pb[e];
        G16[r * 16 + c] -= R[nk * MT_MAX + r] * R[nk * MT_MAX + c];
      }
      if (lane == 0) {
        keep[nk] = q;
        pos[q] = nk;
        invd[nk] = inv;
      }
      ++nk;
    }
    __syncwarp();
  }
  __syncwarp();
  // column c of R_kk^-1, R_kk(i, j) = R[i][keep[j]]
  if (lane < nk) {
    const int c = lane;
    Ri[c * MT_MAX + c] = invd[c];
    for (int i = c - 1; i >= 0; --i) {
      double sum = 0.0;
      for (int l = i + 1; l <= c; ++l) sum += R[i * MT_MAX + keep[l]] * Ri[l * MT_MAX + c];
      Ri[i * MT_MAX + c] = -sum * invd[i];
    }
  }
  __syncwarp();
  for (int e = lane; e < MT_MAX * MT_MAX; e += 32) {
    const int q = e / MT_MAX, c = e % MT_MAX;
    const int i = (q < nb) ? pos[q] : -1;
    C[e] = (i >= 0 && c < nk && i <= c) ? Ri[i * MT_MAX + c] : 0.0;
  }
  if (lane == 0) {
    bst[1] = nb;
    bst[0] = nk;
  }
  if (last && lane < m) skipf[lane] = (lane < nk) ? 0.0 : 1.0;
}


// new columns minus their projections: B(:, kpass+q) -= B(:, 0:kpass) C(:, q)
constexpr int BD_CCH = 64;  // rows of C staged per step
// (columns q0 = blockIdx.y M .. q0 + M of the m; C row a at a m)
template <int M>
__global__ void __launch_bounds__(RT) k_bd_sub(double *__restrict__ B, int64_t ld, const IterParams *__restrict__ pv,
                                               const double *__restrict__ C, int m, int n) {
  pdl_wait();
  __shared__ double Cs[BD_CCH * M];
  const int ka = pv[0].c, q0 = blockIdx.y * M;
  const int i = blockIdx.x * RT + threadIdx.x;
  double acc[M];
#pragma unroll
  for (int q = 0; q < M; ++q) acc[q] = 0.0;
  for (int a0 = 0; a0 < ka; a0 += BD_CCH) {
    const int na = min(BD_CCH, ka - a0);
    __syncthreads();
    for (int idx = threadIdx.x; idx < na * M; idx += RT) Cs[idx] = C[(size_t)(a0 + idx / M) * m + q0 + idx % M];
    __syncthreads();
    if (i < n) {
#pragma unroll 4
      for (int a = 0; a < na; ++a) {
        const double v = B[(size_t)(a0 + a) * ld + i];
#pragma unroll
        for (int q = 0; q < M; ++q) acc[q] = fma(v, Cs[a * M + q], acc[q]);
      }
    }
  }
  if (i >= n) return;
#pragma unroll
  for (int q = 0; q < M; ++q) B[(size_t)(ka + q0 + q) * ld + i] -= acc[q];
}

// kept orthonormal columns: B(:, kpass+c) = sum_q B_old(:, kpass+q) C[q][c],
// c < bst[0], q < bst[1]; the last round also writes each kept column's hi + lo
// FP32 copy for the block matvec (xs: interleaved by row, mp = spmm_pitch(m)
// per row, zeros beyond the kept columns) and into the split copy of the basis (xstore,
// column kpass + c)
template <int NP>
__device__ __forceinline__ void bd_apply_rows(double *__restrict__ B, int64_t ld, int kpass, int nc,
                                              const double *Cs, int i, float2 *xs, int mp, float2 *xstore) {
  double x[NP];
#pragma unroll
  for (int q = 0; q < NP; ++q) x[q] = B[(size_t)(kpass + q) * ld + i];
  for (int c = 0; c < nc; ++c) {
    double sum = 0.0;
#pragma unroll
    for (int q = 0; q < NP; ++q) sum = fma(x[q], Cs[q * MT_MAX + c], sum);
    B[(size_t)(kpass + c) * ld + i] = sum;
    if (xs) {
      const float h = __double2float_rn(sum);
      const float2 v = make_float2(h, __double2float_rn(sum - (double)h));
      xs[(size_t)i * mp + c] = v;
      xstore[(size_t)(kpass + c) * ld + i] = v;
    }
  }
  if (xs)
    for (int c = nc; c < mp; ++c) xs[(size_t)i * mp + c] = make_float2(0.f, 0.f);
}

__global__ void __launch_bounds__(RT) k_bd_apply(double *__restrict__ B, int64_t ld, const IterParams *__restrict__ pv,
                                                 const int *__restrict__ bst, const double *__restrict__ C, int n,
                                                 float2 *__restrict__ xs, int mp, float2 *__restrict__ xstore) {
  pdl_wait();
  __shared__ double Cs[MT_MAX * MT_MAX];
  const int kpass = pv[0].c, np = bst[1], nc = bst[0];
  for (int idx = threadIdx.x; idx < MT_MAX * MT_MAX; idx += RT) Cs[idx] = C[idx];
  __syncthreads();
  const int i = blockIdx.x * RT + threadIdx.x;
  if (i >= n || np <= 0) return;
  switch (np) {
#define BD_CASE(K) \
  case K: bd_apply_rows<K>(B, ld, kpass, nc, Cs, i, xs, mp, xstore); break;
    BD_CASE(1) BD_CASE(2) BD_CASE(3) BD_CASE(4) BD_CASE(5) BD_CASE(6) BD_CASE(7) BD_CASE(8)
    BD_CASE(9) BD_CASE(10) BD_CASE(11) BD_CASE(12) BD_CASE(13) BD_CASE(14) BD_CASE(15) BD_CASE(16)
#undef BD_CASE
    default: break;
  }
}

// ---------------------------------------------------------------------------
// Split-precision block pass (SPLIT): the dot products and linear
// combinations of the block pass on hi + lo FP32 copies of the basis
// (x = hi + lo to 2^-48 relative), each product and sum in Dot2 form (Ogita,
// Rump & Oishi, SIAM J. Sci. Comput. 26 (2005) 1955): the running sum takes
// each product's high part through an error-free TwoSum, the rounding errors
// and the low parts gather in a second float. On GB300 an FP64 FMA costs 64
// times the issue of an FP32 one; the eleven FP32 operations of a Dot2 step
// make these kernels about five times faster than their FP64 forms at about
// 2^-48 relative accuracy, the accuracy of the split matvec. The FP64
// columns stay the master copies; Bx and ABx hold the split copies of the
// basis columns and of their products with H.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void dot2_step(float &sh, float &sl, float ah, float al, float xh, float xl) {
  const float ph = __fmul_rn(ah, xh);
  const float t = fmaf(ah, xl, fmaf(al, xh, fmaf(ah, xh, -ph)));
  const float sn = __fadd_rn(sh, ph);
  const float bb = __fsub_rn(sn, sh);
  const float err = __fadd_rn(__fsub_rn(sh, __fsub_rn(sn, bb)), __fsub_rn(ph, bb));
  sh = sn;
  sl = __fadd_rn(sl, __fadd_rn(err, t));
}

// k_bd_apply in split form: each row's np column values are split into hi +
// lo floats and combined with the split C by Dot2 sums (FP32 pipes); the
// FP64 result is the sum's hi + lo, whose split is the same pair, so the
// matvec copy (xs) and the basis store (xstore) hold exactly the FP64 value
template <int NP>
__device__ __forceinline__ void bdx_apply_rows(double *__restrict__ B, int64_t ld, int kpass, int nc,
                                               const float2 *Cs, int i, float2 *xs, int mp, float2 *xstore,
                                               float2 *wx) {
  float2 x[NP];
#pragma unroll
  for (int q = 0; q < NP; ++q) x[q] = wx[(size_t)q * ld + i];
  for (int c = 0; c < nc; ++c) {
    float h = 0.f, l = 0.f;
#pragma unroll
    for (int q = 0; q < NP; ++q) {
      const float2 cq = Cs[q * MT_MAX + c];
      dot2_step(h, l, cq.x, cq.y, x[q].x, x[q].y);
    }
    const df v = two_sum(h, l);
    B[(size_t)(kpass + c) * ld + i] = (double)v.h + (double)v.l;
    wx[(size_t)c * ld + i] = make_float2(v.h, v.l);
    if (xs) {
      const float2 v2 = make_float2(v.h, v.l);
      xs[(size_t)i * mp + c] = v2;
      xstore[(size_t)(kpass + c) * ld + i] = v2;
    }
  }
  if (xs)
    for (int c = nc; c < mp; ++c) xs[(size_t)i * mp + c] = make_float2(0.f, 0.f);
}

__global__ void __launch_bounds__(RT) k_bdx_apply(double *__restrict__ B, int64_t ld, const IterParams *__restrict__ pv,
                                                  const int *__restrict__ bst, const double *__restrict__ C, int n,
                                                  float2 *__restrict__ xs, int mp, float2 *__restrict__ xstore,
                                                  float2 *__restrict__ wx) {
  pdl_wait();
  __shared__ float2 Cs[MT_MAX * MT_MAX];
  const int kpass = pv[0].c, np = bst[1], nc = bst[0];
  for (int idx = threadIdx.x; idx < MT_MAX * MT_MAX; idx += RT) Cs[idx] = split2(C[idx]);
  __syncthreads();
  const int i = blockIdx.x * RT + threadIdx.x;
  if (i >= n || np <= 0) return;
  switch (np) {
#define BD_CASE(K) \
  case K: bdx_apply_rows<K>(B, ld, kpass, nc, Cs, i, xs, mp, xstore, wx); break;
    BD_CASE(1) BD_CASE(2) BD_CASE(3) BD_CASE(4) BD_CASE(5) BD_CASE(6) BD_CASE(7) BD_CASE(8)
    BD_CASE(9) BD_CASE(10) BD_CASE(11) BD_CASE(12) BD_CASE(13) BD_CASE(14) BD_CASE(15) BD_CASE(16)
#undef BD_CASE
    default: break;
  }
}

constexpr int SP = 4;  // lanes per row of the small-block forms
template <int L>
__device__ __forceinline__ df df_lanes(float sh, float sl) {
  df acc = two_sum(sh, sl);
#pragma unroll
  for (int o = 1; o < L; o <<= 1) {
    df other;
    other.h = __shfl_xor_sync(0xffffffffu, acc.h, o);
    other.l = __shfl_xor_sync(0xffffffffu, acc.l, o);
    acc = df_add(acc, other);
  }
  return acc;
}

// hi + lo copies of columns c0 .. c0+nc of X
__global__ void k_split_cols(const double *__restrict__ X, int64_t ld, int c0, int nc, int n, float2 *__restrict__ Xx) {
  pdl_wait();
  const int64_t tot = (int64_t)nc * n;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < tot; e += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(e / n), i = (int)(e % n);
    const size_t o = (size_t)(c0 + c) * ld + i;
    Xx[o] = split2(X[o]);
  }
}

// k_bd_dots in split form (same MODEs, same partial layout); X from the
// split store (MODE 0, 2) or the FP64 new columns (MODE 1), W split while it
// is staged; MODE 2 also writes the split copies of the new AB columns.
template <int MODE>
__global__ void __launch_bounds__(BD_T) k_bdx_dots(const double *__restrict__ B, const double *__restrict__ AB,
                                                   const float2 *__restrict__ Bx, float2 *__restrict__ ABx,
                                                   int64_t ld, const IterParams *__restrict__ pv, int m,
                                                   const int *__restrict__ bst, int n, int cpc,
                                                   float2 *__restrict__ part, int ps, int cgs,
                                                   const float2 *__restrict__ wx) {
  pdl_wait();
  __shared__ float2 Bs[BD_R * MT_MAX];       // [i][q]
  __shared__ float2 As[BD_R * (BD_AC + 1)];  // [i][a]
  // the second Gram-Schmidt pass, when the first one kept enough of every
  // column (bst[2], set by the first pass's update)
  if (MODE == 0 && cgs == 1 && bst[2]) return;
  const int kpass = pv[0].c;
  const int nb = (MODE == 0) ? m : bst[0];
  if (nb <= 0) return;
  const int na = (MODE == 0) ? kpass : (MODE == 1 ? nb : kpass + nb);
  const double *Wb = ((MODE == 2) ? AB : B) + (size_t)kpass * ld;
  float2 *out = part + (size_t)blockIdx.x * ps;
  const int rbeg = blockIdx.x * cpc * BD_R, rend = min(n, rbeg + cpc * BD_R);
  if (MODE == 0 && cgs == 0 && blockIdx.y == gridDim.y - 1) {
    // first pass: the last grid row sums the new columns' squared norms over
    // its rows (warp w: columns w, w + 8, ...), at outputs na nb + q
    const int lane = threadIdx.x & 31;
    for (int q = threadIdx.x >> 5; q < nb; q += BD_T / 32) {
      float h = 0.f, l = 0.f;
      for (int i = rbeg + lane; i < rend; i += 32) {
        const float2 v = wx[(size_t)q * ld + i];
        dot2_step(h, l, v.x, v.y, v.x, v.y);
      }
      const df t = df_lanes<32>(h, l);
      if (lane == 0) out[na * nb + q] = make_float2(t.h, t.l);
    }
    return;
  }
  // columns per chunk: at most one output pair per thread
  const int acl = min(BD_AC, max(1, BD_T / nb));
  const int gy = (MODE == 0 && cgs == 0) ? gridDim.y - 1 : gridDim.y;
  for (int ac = blockIdx.y * acl; ac < na; ac += gy * acl) {
    const int nac = min(acl, na - ac), np = nac * nb;
    float sh[BD_PAIRS], sl[BD_PAIRS];
#pragma unroll
    for (int k = 0; k < BD_PAIRS; ++k) sh[k] = sl[k] = 0.f;
    for (int r0 = rbeg; r0 < rend; r0 += BD_R) {
      const int nr = min(BD_R, rend - r0);
      for (int idx = threadIdx.x; idx < nr * nb; idx += BD_T) {
        const int i = idx % nr, q = idx / nr;
        // MODE 0, 1: the new columns' split copy (written by their producer)
        const float2 v = (MODE == 2) ? split2(Wb[(size_t)q * ld + r0 + i]) : wx[(size_t)q * ld + r0 + i];
        Bs[i * MT_MAX + q] = v;
        if (MODE == 2 && blockIdx.y == 0 && ac == 0) ABx[(size_t)(kpass + q) * ld + r0 + i] = v;
      }
      for (int idx = threadIdx.x; idx < nr * nac; idx += BD_T) {
        const int i = idx % nr, a = idx / nr;
        As[i * (BD_AC + 1) + a] = (MODE == 1) ? wx[(size_t)(ac + a) * ld + r0 + i]
                                              : Bx[(size_t)(ac + a) * ld + r0 + i];
      }
      __syncthreads();
#pragma unroll
      for (int k = 0; k < BD_PAIRS; ++k) {
        const int pr = threadIdx.x + k * BD_T;
        if (pr < np) {
          const int a = pr % nac, q = pr / nac;
          float h = sh[k], l = sl[k];
          for (int i = 0; i < nr; ++i) {
            const float2 x = As[i * (BD_AC + 1) + a], w = Bs[i * MT_MAX + q];
            dot2_step(h, l, x.x, x.y, w.x, w.y);
          }
          sh[k] = h;
          sl[k] = l;
        }
      }
      __syncthreads();
    }
#pragma unroll
    for (int k = 0; k < BD_PAIRS; ++k) {
      const int pr = threadIdx.x + k * BD_T;
      if (pr < np) {
        const df v = two_sum(sh[k], sl[k]);
        out[(ac + pr % nac) * nb + pr / nac] = make_float2(v.h, v.l);
      }
    }
  }
}

// k_bd_sub in split form: B(:, kpass+q) -= Bx(:, 0:kpass) C(:, q). L lanes
// share a row (L = SP for small blocks, whose one-thread-per-row grids leave
// most SMs idle; 1 otherwise), lane p taking basis columns a = p mod L; their
// Dot2 sums are added by a fixed double-float butterfly and column q is
// written by lane q mod L
template <int M, int L>
__global__ void __launch_bounds__(RT) k_bdx_sub(double *__restrict__ B, const float2 *__restrict__ Bx, int64_t ld,
                                                const IterParams *__restrict__ pv, const double *__restrict__ C,
                                                int m, int n, int *__restrict__ bst, int cgs,
                                                float2 *__restrict__ wx) {
  pdl_wait();
  __shared__ float2 Cs[BD_CCH * M];
  if (cgs == 1 && bst[2]) return;
  const int ka = pv[0].c, q0 = blockIdx.y * M;
  if (cgs == 0 && blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x < 32) {
    // "twice is enough" (Kahan, Parlett): the second pass is needed only if
    // the first removed more than half of a column's squared norm; |w - X c|^2
    // = |w|^2 - |c|^2 for the orthonormal basis X. FP32 is enough for the test.
    bool keep = true;
    for (int q = threadIdx.x; q < m; q += 32) {
      float cc = 0.f;
      for (int a = 0; a < ka; ++a) {
        const float c = (float)C[(size_t)a * m + q];
        cc = fmaf(c, c, cc);
      }
      const float w2 = (float)C[(size_t)ka * m + q];
      keep = keep && (w2 - cc >= 0.5f * w2);
    }
    keep = __all_sync(0xffffffffu, keep);
    if (threadIdx.x == 0) bst[2] = keep ? 1 : 0;
  }
  const int part = threadIdx.x % L;
  const int i = blockIdx.x * (RT / L) + threadIdx.x / L;
  float sh[M], sl[M];
#pragma unroll
  for (int q = 0; q < M; ++q) sh[q] = sl[q] = 0.f;
  for (int a0 = 0; a0 < ka; a0 += BD_CCH) {
    const int na = min(BD_CCH, ka - a0);
    __syncthreads();
    for (int idx = threadIdx.x; idx < na * M; idx += RT)
      Cs[idx] = split2(C[(size_t)(a0 + idx / M) * m + q0 + idx % M]);
    __syncthreads();
    if (i < n) {
      // eight basis loads in flight, then their steps
      for (int ab = part; ab < na; ab += 8 * L) {
        float2 xv[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int a = ab + u * L;
          xv[u] = (a < na) ? Bx[(size_t)(a0 + a) * ld + i] : make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int a = ab + u * L;
          if (a < na) {
#pragma unroll
            for (int q = 0; q < M; ++q) {
              const float2 c = Cs[a * M + q];
              dot2_step(sh[q], sl[q], c.x, c.y, xv[u].x, xv[u].y);
            }
          }
        }
      }
    }
  }
#pragma unroll
  for (int q = 0; q < M; ++q) {
    const df acc = df_lanes<L>(sh[q], sl[q]);
    if (i < n && q % L == part) {
      const size_t o = (size_t)(ka + q0 + q) * ld + i;
      const double v = B[o] - ((double)acc.h + (double)acc.l);
      B[o] = v;
      wx[(size_t)(q0 + q) * ld + i] = split2(v);
    }
  }
}

// k_ritz_multi in split form (Bx, ABx for the basis and its products); L
// lanes per row as in k_bdx_sub, target t finished by lane t mod L
template <int NT, int L>
__global__ void __launch_bounds__(RT, 8) k_ritzx_multi(const float2 *__restrict__ Bx, const float2 *__restrict__ ABx,
                                                    int64_t ld, int k, int nt, const double *__restrict__ S,
                                                    const double *__restrict__ lam, double *__restrict__ T, int n,
                                                    double *__restrict__ part, unsigned *__restrict__ counter,
                                                    double *__restrict__ rn2) {
  pdl_wait();
  __shared__ float2 sv[MT_SMEM];
  __shared__ float2 slam[NT];
  __shared__ float fred[RT / 32];
  __shared__ bool last;
  const int t0 = blockIdx.y * NT;
  for (int q = threadIdx.x; q < NT * k; q += RT) sv[q] = split2(S[(size_t)t0 * k + q]);
  if (threadIdx.x < NT) slam[threadIdx.x] = split2(lam[t0 + threadIdx.x]);
  __syncthreads();
  const int lp = threadIdx.x % L;
  const int i = blockIdx.x * (RT / L) + threadIdx.x / L;
  float bh[NT], bl[NT], ah[NT], al[NT];
#pragma unroll
  for (int t = 0; t < NT; ++t) bh[t] = bl[t] = ah[t] = al[t] = 0.f;
  if (i < n) {
#pragma unroll 4
    for (int j = lp; j < k; j += L) {
      const float2 bj = Bx[(size_t)j * ld + i], aj = ABx[(size_t)j * ld + i];
#pragma unroll
      for (int t = 0; t < NT; ++t) {
        const float2 c = sv[t * k + j];
        dot2_step(bh[t], bl[t], c.x, c.y, bj.x, bj.y);
        dot2_step(ah[t], al[t], c.x, c.y, aj.x, aj.y);
      }
    }
  }
  // r = a - lambda b in double-float (FP32 pipes); only the two stores
  // convert to FP64. |r|^2 is summed in FP32 (a norm for NEWVEC's tests, to
  // about 1e-7 relative)
#pragma unroll
  for (int t = 0; t < NT; ++t) {
    const df b2 = df_lanes<L>(bh[t], bl[t]), a2 = df_lanes<L>(ah[t], al[t]);
    float rsq = 0.f;
    if (i < n && t % L == lp) {
      const float2 lm = slam[t];
      const float ph = lm.x * b2.h;
      const float pl = fmaf(lm.x, b2.l, fmaf(lm.y, b2.h, fmaf(lm.x, b2.h, -ph)));
      const df r = df_add(a2, df{-ph, -pl});
      T[(size_t)(2 * (t0 + t)) * ld + i] = (double)b2.h + (double)b2.l;
      T[(size_t)(2 * (t0 + t) + 1) * ld + i] = (double)r.h + (double)r.l;
      rsq = r.h * r.h;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) rsq += __shfl_xor_sync(0xffffffffu, rsq, o);
    if ((threadIdx.x & 31) == 0) fred[threadIdx.x >> 5] = rsq;
    __syncthreads();
    if (threadIdx.x == 0) {
      float sq = 0.f;
#pragma unroll
      for (int q = 0; q < RT / 32; ++q) sq += fred[q];
      part[(size_t)(t0 + t) * gridDim.x + blockIdx.x] = (double)sq;
    }
    __syncthreads();
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = (atomicAdd(counter, 1u) == gridDim.x * gridDim.y - 1);
  __syncthreads();
  if (!last) return;
  // the norms' block partials, one warp per target, summed in FP32
  for (int t = threadIdx.x >> 5; t < nt; t += RT / 32) {
    float u = 0.f;
    for (int q = threadIdx.x & 31; q < (int)gridDim.x; q += 32) u += (float)__ldcg(part + (size_t)t * gridDim.x + q);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) u += __shfl_xor_sync(0xffffffffu, u, o);
    if ((threadIdx.x & 31) == 0) rn2[t] = (double)u;
  }
  if (threadIdx.x == 0) *counter = 0u;
}

// k_multbc in split form: out(:, j) = Xx(:, 0:k) C(:, j) for j in grid row
// blockIdx.y's group of MB_G columns (C column j at C + j k); L lanes per row
// as in k_bdx_sub, column j finished by lane j mod L
constexpr int MB_G = 8, MB_CH = 128;
template <int L>
__global__ void __launch_bounds__(RT) k_multbcx(const float2 *__restrict__ Xx, int64_t ld, int k,
                                                const double *__restrict__ C, int m, double *__restrict__ out,
                                                int n) {
  __shared__ float2 Cs[MB_CH * MB_G];
  const int j0 = blockIdx.y * MB_G;
  const int lp = threadIdx.x % L;
  const int i = blockIdx.x * (RT / L) + threadIdx.x / L;
  float sh[MB_G], sl[MB_G];
#pragma unroll
  for (int u = 0; u < MB_G; ++u) sh[u] = sl[u] = 0.f;
  for (int q0 = 0; q0 < k; q0 += MB_CH) {
    const int nq = min(MB_CH, k - q0);
    __syncthreads();
    for (int idx = threadIdx.x; idx < nq * MB_G; idx += RT) {
      const int q = idx / MB_G, j = j0 + idx % MB_G;
      Cs[idx] = (j < m) ? split2(C[(size_t)j * k + q0 + q]) : make_float2(0.f, 0.f);
    }
    __syncthreads();
    if (i < n) {
#pragma unroll 4
      for (int q = lp; q < nq; q += L) {
        const float2 x = Xx[(size_t)(q0 + q) * ld + i];
#pragma unroll
        for (int u = 0; u < MB_G; ++u) dot2_step(sh[u], sl[u], Cs[q * MB_G + u].x, Cs[q * MB_G + u].y, x.x, x.y);
      }
    }
  }
#pragma unroll
  for (int u = 0; u < MB_G; ++u) {
    const df acc = df_lanes<L>(sh[u], sl[u]);
    if (i < n && j0 + u < m && u % L == lp) out[(size_t)(j0 + u) * ld + i] = (double)acc.h + (double)acc.l;
  }
}

struct Dvd {
  gg_ctx *ctx;
  gg_hmat *h;
  int precision;
  int n, lim;
  int64_t ld;
  cudaStream_t s;
  DBuf<double> B, AB, T, diag, part, small;
  DBuf<double> dots;              // [0, lim + 8) dot products, then SC_N pass scalars
  DBuf<double> dup;               // [0, 8) IterParams, [8, 8 + lim) Ritz coefficients
  DBuf<unsigned> counters;        // last-block counters, one per kernel kind
  int nrow = 0;                   // blocks of the block-pass Ritz kernel (RT rows each)
  int nrow4 = 0;                  // blocks of the split row kernels (RT / SP rows each)
  int nrr = 0;                    // blocks of the row kernels (RR rows each)
  int cd_rows = 0, cd_blocks = 0, kp = 0;  // column-dot layout: rows per block, blocks, partial pitch
  int nmv = 0;
  double mv_ms = 0;
  int mv_count = 0;
  double t_eig = 0, t_wait = 0;   // host seconds: projected eigenproblem, device-to-host waits
  double t_total = 0;             // host seconds in dvdson
  std::vector<cudaEvent_t> evs;   // matvec start/stop pairs, read once at the end
  size_t ev_used = 0;
  char *pinned = nullptr;         // one pinned allocation holding the h* buffers below
  double *hup = nullptr;          // pinned, layout of dup
  double *hdown = nullptr;        // pinned, layout of dots
  DBuf<double> dS;                // staging of new columns of S (packed upper, like S)
  double *hS = nullptr;           // pinned, layout of dS
  DBuf<double> dmt;               // block pass: [MT_MAX lim] coefficients, [MT_MAX] lambda, [MT_MAX] |r|^2
  double *hmt = nullptr;          // pinned, layout of dmt
  cudaGraph_t graph = nullptr;    // single-vector pass (MBLOCK = 1)
  cudaGraphExec_t gexec = nullptr;
  cudaEvent_t gev0 = nullptr, gev1 = nullptr;
  std::vector<cudaEvent_t> bev;    // matvec events of the block passes
  cudaEvent_t pev0 = nullptr, pev1 = nullptr;  // around each single-vector pass
  double pass_ms = 0;             // device ms of the single-vector passes
  int graph_kernels = 0;
  // block pass (MBLOCK > 1): new columns c_v = KPASS + v, v < m, each
  // Gram-Schmidt -> OP -> ADDS, as one graph per m; parameters in dpv[v]
  DBuf<IterParams> dpv;
  // block Gram-Schmidt: CTA partials (bd_G CTAs, pitch bd_ps), coefficients,
  // matvec skip flags, [kept, before] counts, split copies of the new columns
  DBuf<double> bpart, bC, bskip;
  DBuf<int> bst;
  DBuf<float2> bxs;
  DBuf<float2> wx;                // SPLIT: hi + lo copy of the pass's new columns, kept by their producers
  int ensure_wx() {
    if (use_x() && !wx.p) GG_TRY(wx.alloc((size_t)MT_MAX * ld));
    return GG_OK;
  }
  int bd_G = 0, bd_Y = 1, bd_cpc = 0, bd_ps = 0;
  int full_m = 0;                 // MBLOCK: block matvecs over this many columns are timed apart
  double spmm_full_ms = 0;
  int spmm_full_n = 0;
  int cgs_once = 0;               // split block passes whose second Gram-Schmidt pass was skipped
  // SPLIT: hi + lo copies of the basis and its products (split-precision
  // block kernels); columns [0, bx_cols) of both are current
  DBuf<float2> Bx, ABx;
  int bx_cols = 0;
  bool use_x() const { return precision == GG_SPLIT; }
  int sync_split(int k) {
    if (!use_x() || bx_cols >= k) return GG_OK;
    if (!Bx.p) {
      GG_TRY(Bx.alloc((size_t)lim * ld));
      GG_TRY(ABx.alloc((size_t)lim * ld));
    }
    const int nc = k - bx_cols;
    const int grid = std::min<int64_t>(((int64_t)nc * n + TPB - 1) / TPB, 8 * ctx->sms);
    GG_CUDA(launch_pdl(k_split_cols, grid, TPB, 0, s, B.p, ld, bx_cols, nc, n, Bx.p));
    GG_CUDA(launch_pdl(k_split_cols, grid, TPB, 0, s, AB.p, ld, bx_cols, nc, n, ABx.p));
    note_launches(2);
    GG_CUDA(cudaGetLastError());
    bx_cols = k;
    return GG_OK;
  }
  // One block pass moves its inputs in one host-to-device copy and its
  // results in one device-to-host copy:
  //   in:  NvIn | IterParams[MT_MAX] | Ritz coefficients [MT_MAX][lim]
  //   out: NvOut | kept/before counts | the new S columns, packed upper
  //        from offset kpass (kpass + 1) / 2
  DBuf<char> dio_in, dio_out;
  char *hio_in = nullptr, *hio_out = nullptr;  // pinned mirrors
  size_t io_in_bytes = 0, io_out_bytes = 0, io_pv = 0, io_coef = 0, io_bst = 0, io_scol = 0;
  void io_layout() {
    auto a16 = [](size_t b) { return (b + 15) / 16 * 16; };
    io_pv = a16(sizeof(NvIn));
    io_coef = io_pv + a16(MT_MAX * sizeof(IterParams));
    io_in_bytes = io_coef + (size_t)MT_MAX * lim * sizeof(double);
    io_bst = a16(sizeof(NvOut));
    io_scol = io_bst + 16;
    io_out_bytes = io_scol + (size_t)MT_MAX * (lim + MT_MAX) * sizeof(double);
  }
  NvIn *din_nv() { return reinterpret_cast<NvIn *>(dio_in.p); }
  double *din_coef() { return reinterpret_cast<double *>(dio_in.p + io_coef); }
  NvOut *dout_nv() { return reinterpret_cast<NvOut *>(dio_out.p); }
  double *dout_scol() { return reinterpret_cast<double *>(dio_out.p + io_scol); }
  NvOut *hout_nv() { return reinterpret_cast<NvOut *>(hio_out); }
  const int *hout_bst() { return reinterpret_cast<const int *>(hio_out + io_bst); }
  const double *hout_scol() { return reinterpret_cast<const double *>(hio_out + io_scol); }
  std::vector<cudaGraphExec_t> bexec;
  std::vector<int> bkernels;
  std::vector<int> buses;         // block passes run per width
  bool use_graph = true;          // passes replayed as CUDA graphs
  // block passes with NEWVEC's choices on the device (one host wait per
  // pass); more than MT_MAX targets take the host path
  bool use_fused = true;

  double *scal() { return dots.p + lim + 8; }
  IterParams *dpar() { return reinterpret_cast<IterParams *>(dup.p); }
  IterParams *hpar() { return reinterpret_cast<IterParams *>(hup); }
  double *col(DBuf<double> &X, int j) { return X.p + (size_t)j * ld; }

  int init(gg_ctx *c, gg_hmat *hm, int prec, int nn, int lm) {
    static_assert(sizeof(IterParams) <= 8 * sizeof(double), "IterParams slot");
    ctx = c;
    h = hm;
    precision = prec;
    n = nn;
    lim = lm;
    s = c->stream;
    ld = ((int64_t)n + 31) / 32 * 32;
    nrow = (n + RT - 1) / RT;
    nrow4 = (n + RT / SP - 1) / (RT / SP);
    nrr = (n + RR - 1) / RR;
    // about two column-dot blocks per SM, rows a multiple of 32
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
    cd_rows = (int)std::min<int64_t>(CD_MAXR, std::max<int64_t>(32, ((n + 2 * sms - 1) / (2 * sms) + 31) / 32 * 32));
    cd_blocks = (n + cd_rows - 1) / cd_rows;
    kp = lim + 8;
    GG_TRY(B.alloc((size_t)ld * lim));
    GG_TRY(AB.alloc((size_t)ld * lim));
    GG_TRY(T.alloc((size_t)ld * lim));
    GG_TRY(diag.alloc(n));
    GG_TRY(part.alloc((size_t)std::max(std::max(cd_blocks * kp, nrow4 * MT_MAX), nrr) + 1024));
    GG_TRY(dS.alloc((size_t)lim * (lim + 1) / 2));
    GG_TRY(dmt.alloc((size_t)MT_MAX * lim + 2 * MT_MAX));
    {
      // all pinned host buffers of the workspace in one allocation
      auto al = [](size_t b) { return (b + 255) / 256 * 256; };
      const size_t bS = al((size_t)lim * (lim + 1) / 2 * sizeof(double));
      const size_t bmt = al(((size_t)MT_MAX * lim + 2 * MT_MAX) * sizeof(double));
      const size_t bup = al((size_t)(8 + lim) * sizeof(double)), bdown = al((size_t)(lim + 8 + SC_N) * sizeof(double));
      io_layout();
      const size_t bio = al(io_in_bytes) + al(io_out_bytes);
      char *a = nullptr;
      GG_CUDA(cudaMallocHost(&a, bS + bmt + bup + bdown + bio));
      note_alloc();
      pinned = a;
      hS = reinterpret_cast<double *>(a);
      a += bS;
      hmt = reinterpret_cast<double *>(a);
      a += bmt;
      hup = reinterpret_cast<double *>(a);
      a += bup;
      hdown = reinterpret_cast<double *>(a);
      a += bdown;
      hio_in = a;
      a += al(io_in_bytes);
      hio_out = a;
    }
    GG_TRY(dio_in.alloc(io_in_bytes));
    GG_TRY(dio_out.alloc(io_out_bytes));
    GG_TRY(small.alloc(4096));
    GG_TRY(dots.alloc(lim + 8 + SC_N));
    GG_TRY(dup.alloc(8 + lim));
    GG_TRY(counters.alloc(16));
    GG_CUDA(cudaMemsetAsync(counters.p, 0, 16 * sizeof(unsigned), s));
    GG_CUDA(cudaMemsetAsync(dots.p, 0, (lim + 8 + SC_N) * sizeof(double), s));

    std::memset(hup, 0, (size_t)(8 + lim) * sizeof(double));
    GG_CUDA(cudaMemsetAsync(B.p, 0, (size_t)ld * lim * 8, s));
    GG_CUDA(cudaMemsetAsync(AB.p, 0, (size_t)ld * lim * 8, s));
    if (precision == GG_SPLIT) GG_TRY(h->dXs.alloc(n));
    return GG_OK;
  }
  bool reusable(gg_hmat *hm, int prec, int nn, int lm) const {
    return h == hm && precision == prec && n == nn && lim == lm;
  }
  // a reused workspace (same matrix, sizes and precision; allocations and
  // graphs kept) starts a new solve
  int reset() {
    nmv = 0;
    mv_ms = 0;
    mv_count = 0;
    t_eig = t_wait = t_total = 0;
    ev_used = 0;
    pass_ms = 0;
    spmm_full_ms = 0;
    spmm_full_n = 0;
    cgs_once = 0;
    bx_cols = 0;
    full_m = 0;
    GG_CUDA(cudaMemsetAsync(counters.p, 0, 16 * sizeof(unsigned), s));
    GG_CUDA(cudaMemsetAsync(dots.p, 0, (lim + 8 + SC_N) * sizeof(double), s));
    std::memset(hup, 0, (size_t)(8 + lim) * sizeof(double));
    GG_CUDA(cudaMemsetAsync(B.p, 0, (size_t)ld * lim * 8, s));
    GG_CUDA(cudaMemsetAsync(AB.p, 0, (size_t)ld * lim * 8, s));
    return GG_OK;
  }
  ~Dvd() {
    for (cudaEvent_t e : evs) cudaEventDestroy(e);
    if (pinned) cudaFreeHost(pinned);
    if (gexec) cudaGraphExecDestroy(gexec);
    for (cudaGraphExec_t e : bexec)
      if (e) cudaGraphExecDestroy(e);

    if (graph) cudaGraphDestroy(graph);
    if (gev0) cudaEventDestroy(gev0);
    for (auto e : bev)
      if (e) cudaEventDestroy(e);
    if (gev1) cudaEventDestroy(gev1);
    if (pev0) cudaEventDestroy(pev0);
    if (pev1) cudaEventDestroy(pev1);
  }

  // ---- kernel launchers (counters: 0 ritz, 1 column dots, 2 csub) ----
  void launch_ritz(const PSrc &ps) {
    k_ritz<<<nrr, RTH, 0, s>>>(B.p, AB.p, ld, ps, dup.p + 8, n, part.p, counters.p + 0, scal());
    note_launch();
  }
  // column dots (partials per block, then one block per column adds them)
  void launch_dots(bool pre, const PSrc &ps, int kofs, double *W, const double *skip, int fslot,
                   double *out = nullptr, int packed = 0) {
    if (!out) out = dots.p;
    if (pre)
      k_cdots<true><<<cd_blocks, CD_T, 0, s>>>(B.p, ld, ps, kofs, W, AB.p, diag.p, scal(), skip, n, cd_rows,
                                               cd_blocks, part.p);
    else
      k_cdots<false><<<cd_blocks, CD_T, 0, s>>>(B.p, ld, ps, kofs, W, AB.p, diag.p, scal(), skip, n, cd_rows,
                                                cd_blocks, part.p);
    k_colsum<<<lim + 1, CS_T, 0, s>>>(part.p, cd_blocks, cd_blocks, ps, kofs, skip, scal(), fslot, out, packed);
    note_launch();
    note_launch();
  }
  void launch_csub(const PSrc &ps, const double *skip, int fin, int fout) {
    k_csub<<<nrr, RTH, 0, s>>>(B.p, ld, ps, dots.p, skip, fin, fout, n, part.p, counters.p + 2, scal());
    note_launch();
  }
  void launch_cscale(const PSrc &ps, const double *skip, int fslot, float2 *xs) {
    k_cscale<<<std::min((n + TPB - 1) / TPB, 4 * 152), TPB, 0, s>>>(B.p, ld, ps, skip, scal(), fslot, n, xs);
    note_launch();
  }
  // two-pass classical Gram-Schmidt of column ps.c against columns
  // 0..c-1 with normalisation (mgs_nrm, dvdson.f90:1417-1508); the first
  // pass optionally applies the preconditioner to the column first. The
  // normalisation after pass 1 is carried as a factor into pass 2.
  void cgs2(const PSrc &ps, bool pre, const double *skip, float2 *xs) {
    launch_dots(pre, ps, 0, B.p, skip, -1);
    launch_csub(ps, skip, -1, SC_F1);
    launch_dots(false, ps, 0, B.p, skip, SC_F1);
    launch_csub(ps, skip, SC_F1, SC_F2);
    launch_cscale(ps, skip, SC_F2, xs);
  }

  // One single-vector pass (MBLOCK = 1) for target parameters ps, with the
  // Ritz coefficients already in dup: Ritz vector and residual; shift,
  // preconditioner and CGS2 of column c; y = H x; S(0:c, c); results down.
  // Everything after the Ritz kernel is skipped on the device when the
  // target has converged.
  int enqueue_single(const PSrc &ps, const int *dcol, bool in_capture) {
    const double *skip = scal() + SC_CONV;
    GG_CUDA(cudaMemcpyAsync(dup.p, hup, (size_t)(8 + lim) * sizeof(double), cudaMemcpyHostToDevice, s));
    launch_ritz(ps);
    cgs2(ps, true, skip, precision == GG_SPLIT ? h->dXs.p : nullptr);
    if (in_capture) {
      GG_CUDA(cudaEventRecordWithFlags(gev0, s, cudaEventRecordExternal));
    } else {
      GG_CUDA(cudaEventRecord(gev0, s));
    }
    GG_TRY(spmv_col(h, precision, B.p, AB.p, ld, dcol, skip, s));
    if (in_capture) {
      GG_CUDA(cudaEventRecordWithFlags(gev1, s, cudaEventRecordExternal));
    } else {
      GG_CUDA(cudaEventRecord(gev1, s));
    }
    launch_dots(false, ps, 1, AB.p, skip, -1);
    GG_CUDA(cudaMemcpyAsync(hdown, dots.p, (size_t)(lim + 8 + SC_N) * sizeof(double), cudaMemcpyDeviceToHost, s));
    return GG_OK;
  }

  int build_graph() {
    if (!gev0) GG_CUDA(cudaEventCreate(&gev0));
    if (!gev1) GG_CUDA(cudaEventCreate(&gev1));
    PSrc ps{dpar(), IterParams{}};
    const int *dcol = reinterpret_cast<const int *>(reinterpret_cast<const char *>(dup.p) + offsetof(IterParams, c));
    GG_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    const long long before = gg_launch_count();
    const int st = enqueue_single(ps, dcol, true);
    const long long captured = gg_launch_count() - before;
    note_launches(-captured);  // counted per replay instead
    cudaGraph_t gcap = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(s, &gcap);
    if (st != GG_OK) {
      if (gcap) cudaGraphDestroy(gcap);
      return st;
    }
    if (ce != cudaSuccess) return fail(GG_ERR_CUDA, std::string("Davidson graph capture: ") + cudaGetErrorString(ce));
    graph = gcap;
    GG_CUDA(cudaGraphInstantiate(&gexec, graph, 0));
    graph_kernels = (int)captured;
    return GG_OK;
  }

  // Block Gram-Schmidt of the new columns kpass .. kpass+m-1 (two block CGS
  // passes against the basis, two Cholesky QR rounds among themselves), OP of
  // each kept column, the new columns of S into dS at their packed offsets.
  // kpass comes from dpv[0].c, so one graph per m serves every pass.
  int enqueue_block(int m, bool in_capture) {
    const bool split = (precision == GG_SPLIT);
    const int nred = std::max(1, (lim * m + 31) / 32);
    const bool sub_split = (int64_t)nrow * 2 < ctx->sms;  // small blocks: one column per grid row
    // the split kernels' CTA partials are double-float pairs in the same buffer
    float2 *bpx = reinterpret_cast<float2 *>(bpart.p);
    const dim3 gd(bd_G, bd_Y);
    // split dots: chunks of max(1, BD_T / m) columns (one pair per thread)
    const dim3 gdx(bd_G, (lim + std::min(BD_AC, std::max(1, BD_T / m)) - 1) / std::min(BD_AC, std::max(1, BD_T / m)));
    for (int round = 0; round < 2; ++round) {
      if (split) {
        // the first pass's last grid row sums the new columns' squared norms
        const dim3 g0(gdx.x, gdx.y + (round == 0 ? 1 : 0));
        GG_CUDA(launch_pdl(k_bdx_dots<0>, g0, BD_T, 0, s, B.p, AB.p, Bx.p, ABx.p, ld, dpv.p, m, bst.p, n, bd_cpc, bpx,
                           bd_ps, round, wx.p));
        GG_CUDA(launch_pdl(k_bd_reduce<0, float2>, nred, BD_T, 0, s, dpv.p, m, bst.p, bpx, bd_ps, bd_G, bC.p, dS.p,
                           round == 0, round));
      } else {
        GG_CUDA(launch_pdl(k_bd_dots<0>, gd, BD_T, 0, s, B.p, AB.p, ld, dpv.p, m, bst.p, n, bd_cpc, bpart.p, bd_ps));
        GG_CUDA(launch_pdl(k_bd_reduce<0, double>, nred, BD_T, 0, s, dpv.p, m, bst.p, bpart.p, bd_ps, bd_G, bC.p, dS.p,
                           round == 0, -1));
      }
      if (sub_split) {
        if (split)
          GG_CUDA(launch_pdl(k_bdx_sub<1, SP>, dim3(nrow4, m), RT, 0, s, B.p, Bx.p, ld, dpv.p, bC.p, m, n, bst.p, round,
                             wx.p));
        else
          GG_CUDA(launch_pdl(k_bd_sub<1>, dim3(nrow, m), RT, 0, s, B.p, ld, dpv.p, bC.p, m, n));
      } else {
        // an even m as m / 2 grid rows of two columns (more warps in flight;
        // each grid row reads the basis, from L2; all m columns with two
        // lanes per row measured slower)
        const int half = (m % 2 == 0) ? m / 2 : 1;
        switch (m / half) {
#define BD_SUB(K)                                                                           \
  case K:                                                                                   \
    if (split)                                                                              \
      GG_CUDA(launch_pdl(k_bdx_sub<K, 1>, dim3(nrow, half), RT, 0, s, B.p, Bx.p, ld, dpv.p, bC.p, m, n, bst.p,   \
                         round, wx.p));                                                     \
    else                                                                                    \
      GG_CUDA(launch_pdl(k_bd_sub<K>, dim3(nrow, half), RT, 0, s, B.p, ld, dpv.p, bC.p, m, n));              \
    break;
        BD_SUB(1) BD_SUB(2) BD_SUB(3) BD_SUB(4) BD_SUB(5) BD_SUB(6) BD_SUB(7) BD_SUB(8)
        BD_SUB(9) BD_SUB(10) BD_SUB(11) BD_SUB(12) BD_SUB(13) BD_SUB(14) BD_SUB(15) BD_SUB(16)
#undef BD_SUB
          default: return fail(GG_ERR_ARG, "block pass: more new vectors than supported");
        }
      }
      note_launches(3);
    }
    for (int round = 0; round < 2; ++round) {
      if (split) {
        GG_CUDA(launch_pdl(k_bdx_dots<1>, dim3(bd_G, 1), BD_T, 0, s, B.p, AB.p, Bx.p, ABx.p, ld, dpv.p, m, bst.p, n,
                           bd_cpc, bpx, bd_ps, -1, wx.p));
        GG_CUDA(launch_pdl(k_bd_chol<float2>, 1, BD_RED, 0, s, m, bst.p, bpx, bd_ps, bd_G, bC.p, bskip.p, round));
        GG_CUDA(launch_pdl(k_bdx_apply, nrow, RT, 0, s, B.p, ld, dpv.p, bst.p, bC.p, n, round == 1 ? bxs.p : nullptr,
                                        spmm_pitch(m), Bx.p, wx.p));
      } else {
        GG_CUDA(launch_pdl(k_bd_dots<1>, dim3(bd_G, 1), BD_T, 0, s, B.p, AB.p, ld, dpv.p, m, bst.p, n, bd_cpc, bpart.p, bd_ps));
        GG_CUDA(launch_pdl(k_bd_chol<double>, 1, BD_RED, 0, s, m, bst.p, bpart.p, bd_ps, bd_G, bC.p, bskip.p, round));
        GG_CUDA(launch_pdl(k_bd_apply, nrow, RT, 0, s, B.p, ld, dpv.p, bst.p, bC.p, n, nullptr, spmm_pitch(m), Bx.p));
      }
      note_launches(3);
    }
    GG_CUDA(cudaGetLastError());
    if (split) {
      // all m columns in one sweep over the matrix (dropped columns are zero)
      const int *dcol0 = reinterpret_cast<const int *>(reinterpret_cast<const char *>(dpv.p) + offsetof(IterParams, c));
      if (in_capture) {
        GG_CUDA(cudaEventRecordWithFlags(bev[0], s, cudaEventRecordExternal));
      } else {
        GG_CUDA(cudaEventRecord(bev[0], s));
      }
      GG_TRY(spmm_block(h, m, bxs.p, B.p, AB.p, ld, dcol0, s));
      if (in_capture) {
        GG_CUDA(cudaEventRecordWithFlags(bev[1], s, cudaEventRecordExternal));
      } else {
        GG_CUDA(cudaEventRecord(bev[1], s));
      }
    }
    for (int v = 0; v < m && !split; ++v) {
      const int *dcol = reinterpret_cast<const int *>(reinterpret_cast<const char *>(dpv.p + v) +
                                                      offsetof(IterParams, c));
      // each matvec between two events (read after the pass)
      if (in_capture) {
        GG_CUDA(cudaEventRecordWithFlags(bev[2 * v], s, cudaEventRecordExternal));
      } else {
        GG_CUDA(cudaEventRecord(bev[2 * v], s));
      }
      GG_TRY(spmv_col(h, precision, B.p, AB.p, ld, dcol, bskip.p + v, s));
      if (in_capture) {
        GG_CUDA(cudaEventRecordWithFlags(bev[2 * v + 1], s, cudaEventRecordExternal));
      } else {
        GG_CUDA(cudaEventRecord(bev[2 * v + 1], s));
      }
    }
    if (split) {
      GG_CUDA(launch_pdl(k_bdx_dots<2>, gdx, BD_T, 0, s, B.p, AB.p, Bx.p, ABx.p, ld, dpv.p, m, bst.p, n, bd_cpc, bpx,
                         bd_ps, -1, wx.p));
      GG_CUDA(launch_pdl(k_bd_reduce<2, float2>, nred, BD_T, 0, s, dpv.p, m, bst.p, bpx, bd_ps, bd_G, bC.p,
                         dout_scol(), 0, -1));
    } else {
      GG_CUDA(launch_pdl(k_bd_dots<2>, gd, BD_T, 0, s, B.p, AB.p, ld, dpv.p, m, bst.p, n, bd_cpc, bpart.p, bd_ps));
      GG_CUDA(launch_pdl(k_bd_reduce<2, double>, nred, BD_T, 0, s, dpv.p, m, bst.p, bpart.p, bd_ps, bd_G, bC.p,
                         dout_scol(), 0, -1));
    }
    note_launches(2);
    GG_CUDA(cudaGetLastError());
    return GG_OK;
  }
  // the block pass for columns kpass .. kpass+m-1: one graph launch, one copy
  // of the new S columns back
  // staged: the caller copied the pass's IterParams with its inputs
  int block_pass(int kpass, int m, std::vector<double> &S, int *nkept, bool staged = false) {
    *nkept = 0;
    if (m <= 0) return GG_OK;
    if (m > MT_MAX) return fail(GG_ERR_ARG, "block pass: more new vectors than supported");
    if (bev.empty()) {
      bev.resize(2 * MT_MAX, nullptr);
      for (auto &e : bev) GG_CUDA(cudaEventCreate(&e));
    }
    if (!dpv.p) {
      dpv.p = reinterpret_cast<IterParams *>(dio_in.p + io_pv);
      dpv.n = MT_MAX;
      dpv.own = false;

      bexec.assign(MT_MAX + 1, nullptr);
      bkernels.assign(MT_MAX + 1, 0);
      buses.assign(MT_MAX + 1, 0);
      // row ranges of BD_R-row chunks, about two CTAs per SM
      // (grid rows: column chunks of BD_AC, up to LIM / BD_AC of them)
      // (grid rows: the column chunks; about two row ranges per SM, or one
      // CTA per row chunk for small blocks)
      const int nchunk = (n + BD_R - 1) / BD_R;
      bd_Y = std::max(1, (lim + BD_AC - 1) / BD_AC);
      const int want = std::max(1, (nchunk >= 2 * ctx->sms) ? 2 * ctx->sms : (2 * ctx->sms + bd_Y - 1) / bd_Y);
      bd_cpc = (nchunk + want - 1) / want;
      bd_G = (nchunk + bd_cpc - 1) / bd_cpc;

      bd_ps = lim * MT_MAX;
      GG_TRY(bpart.alloc((size_t)bd_G * bd_ps));
      GG_TRY(bC.alloc((size_t)std::max(lim * MT_MAX, MT_MAX * MT_MAX)));
      GG_TRY(bskip.alloc(MT_MAX));
      bst.p = reinterpret_cast<int *>(dio_out.p + io_bst);
      bst.n = 2;
      bst.own = false;

      if (precision == GG_SPLIT) GG_TRY(bxs.alloc((size_t)MT_MAX * ld));
    }
    GG_TRY(ensure_wx());
    GG_TRY(sync_split(kpass));
    if (!staged) {
      // the caller's new columns: their split copy (a staged pass's NEWVEC
      // writes it with the columns)
      if (use_x()) {
        const int64_t tot = (int64_t)m * n;
        const int nb = (int)std::min<int64_t>((tot + TPB - 1) / TPB, 4 * ctx->sms);
        k_split_cols<<<nb, TPB, 0, s>>>(B.p + (size_t)kpass * ld, ld, 0, m, n, wx.p);
        note_launch();
        GG_CUDA(cudaGetLastError());
      }
      IterParams *hp = reinterpret_cast<IterParams *>(hio_in + io_pv);
      for (int v = 0; v < m; ++v) {
        hp[v] = IterParams{};
        hp[v].c = kpass + v;
      }
      GG_CUDA(cudaMemcpyAsync(dpv.p, hp, m * sizeof(IterParams), cudaMemcpyHostToDevice, s));
    }
    // a graph per batch size m, captured at the first pass of the full width
    // or the second pass of another width (a width used once is launched
    // kernel by kernel: cheaper than capturing it)
    ++buses[m];
    if (use_graph && (bexec[m] || m == full_m || buses[m] >= 2)) {
      if (!bexec[m]) {
        GG_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        const long long before = gg_launch_count();
        const int st = enqueue_block(m, true);
        const long long captured = gg_launch_count() - before;
        note_launches(-captured);
        cudaGraph_t g = nullptr;
        const cudaError_t ce = cudaStreamEndCapture(s, &g);
        if (st != GG_OK) {
          if (g) cudaGraphDestroy(g);
          return st;
        }
        if (ce != cudaSuccess) return fail(GG_ERR_CUDA, std::string("block pass capture: ") + cudaGetErrorString(ce));
        const cudaError_t ie = cudaGraphInstantiate(&bexec[m], g, 0);
        cudaGraphDestroy(g);
        if (ie != cudaSuccess) return fail(GG_ERR_CUDA, std::string("block pass graph: ") + cudaGetErrorString(ie));
        bkernels[m] = (int)captured;
      }
      GG_CUDA(cudaGraphLaunch(bexec[m], s));
      note_launches(bkernels[m]);
    } else {
      GG_TRY(enqueue_block(m, false));
    }
    // NEWVEC's results, the column counts and the new S columns in one copy
    const size_t o0 = (size_t)kpass * (kpass + 1) / 2, o1 = (size_t)(kpass + m) * (kpass + m + 1) / 2;
    GG_CUDA(cudaMemcpyAsync(hio_out, dio_out.p, io_scol + (o1 - o0) * sizeof(double), cudaMemcpyDeviceToHost, s));
    const auto t0 = std::chrono::steady_clock::now();
    GG_CUDA(cudaStreamSynchronize(s));
    t_wait += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    const int nk = hout_bst()[0];
    if (nk < 0 || nk > m) return fail(GG_ERR_STATE, "block pass: kept column count out of range");
    if (use_x()) cgs_once += hout_bst()[2];
    std::memcpy(S.data() + o0, hout_scol(), (o1 - o0) * sizeof(double));
    for (int v = 0; v < (use_x() ? 1 : m); ++v) {
      float ms = 0.f;
      GG_CUDA(cudaEventElapsedTime(&ms, bev[2 * v], bev[2 * v + 1]));
      mv_ms += ms;
      if (use_x() && m == full_m) {
        spmm_full_ms += ms;
        ++spmm_full_n;
      }
    }
    nmv += nk;
    mv_count += nk;
    if (use_x()) bx_cols = kpass + nk;  // written by the pass (k_bd_apply, k_bdx_dots<2>)
    *nkept = nk;
    return GG_OK;
  }

  // One single-vector pass for basis size kpass and the target with Ritz
  // coefficients svec. Returns |r|; when |r| >= critr the new column kpass of
  // S is written into S (packed upper).
  int single_pass(int kpass, const double *svec, double lam, double gap, double dl, double critr, double *res,
                  std::vector<double> &S) {
    IterParams &hp = *hpar();
    hp.c = kpass;
    hp.k = kpass;
    hp.lam = lam;
    hp.gap = gap;
    hp.dl = dl;
    hp.critr = critr;
    std::memcpy(hup + 8, svec, (size_t)kpass * sizeof(double));
    if (!pev0) GG_CUDA(cudaEventCreate(&pev0));
    if (!pev1) GG_CUDA(cudaEventCreate(&pev1));
    GG_CUDA(cudaEventRecord(pev0, s));
    if (use_graph && !gexec && build_graph() != GG_OK) {
      // a driver that cannot capture this launch: launch it directly
      cudaGetLastError();
      use_graph = false;
    }
    if (use_graph) {
      GG_CUDA(cudaGraphLaunch(gexec, s));
      note_launches(graph_kernels);
    } else {
      if (!gev0) GG_CUDA(cudaEventCreate(&gev0));
      if (!gev1) GG_CUDA(cudaEventCreate(&gev1));
      PSrc ps{nullptr, hp};
      const int *dcol = reinterpret_cast<const int *>(reinterpret_cast<const char *>(dup.p) + offsetof(IterParams, c));
      GG_TRY(enqueue_single(ps, dcol, false));
    }
    GG_CUDA(cudaEventRecord(pev1, s));
    const auto t0 = std::chrono::steady_clock::now();
    GG_CUDA(cudaStreamSynchronize(s));
    t_wait += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    {
      float pms = 0.f;
      GG_CUDA(cudaEventElapsedTime(&pms, pev0, pev1));
      pass_ms += pms;
    }
    const double *sc = hdown + lim + 8;
    *res = std::sqrt(sc[SC_RN2]);
    if (sc[SC_CONV] == 0.0) {
      const size_t off = (size_t)kpass * (kpass + 1) / 2;
      std::memcpy(S.data() + off, hdown, (size_t)(kpass + 1) * sizeof(double));
      {
        float ms = 0.f;
        GG_CUDA(cudaEventElapsedTime(&ms, gev0, gev1));
        mv_ms += ms;
      }
      ++mv_count;
      ++nmv;
    }
    return GG_OK;
  }

  // OP (gdvd.f90:137-142): AB[:, j0:j0+m) = H BASIS[:, j0:j0+m); each launch
  // is bracketed by events that are read after the solve (no extra sync)
  int op(int j0, int m) {
    if (precision == GG_SPLIT && m >= 2) {  // blocks of up to 16 columns, one sweep each
      for (int v0 = 0; v0 < m; v0 += 16) {
        const int mb = std::min(16, m - v0);
        if (ev_used + 2 > evs.size())
          for (int q = 0; q < 64; ++q) {
            cudaEvent_t e;
            GG_CUDA(cudaEventCreate(&e));
            evs.push_back(e);
          }
        GG_CUDA(cudaEventRecord(evs[ev_used], s));
        if (mb >= 2)
          GG_TRY(spmm_cols(h, col(B, j0 + v0), col(AB, j0 + v0), ld, mb, s));
        else
          GG_TRY(spmv(h, precision, col(B, j0 + v0), col(AB, j0 + v0), 1, s));
        GG_CUDA(cudaEventRecord(evs[ev_used + 1], s));
        ev_used += 2;
        mv_count += mb;
      }
      nmv += m;
      return GG_OK;
    }
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
  static PSrc by_value(int c, int k = 0, double lam = 0, double gap = 0, double dl = 0, double critr = 0) {
    IterParams p{};
    p.c = c;
    p.k = k;
    p.lam = lam;
    p.gap = gap;
    p.dl = dl;
    p.critr = critr;
    return PSrc{nullptr, p};
  }
  // column j orthonormalised against columns 0..j-1
  int orthonormalize(int j) {
    const PSrc ps = by_value(j);
    if (j > 0) {
      cgs2(ps, false, nullptr, nullptr);
    } else {
      launch_csub(ps, nullptr, -1, SC_F2);
      launch_cscale(ps, nullptr, SC_F2, nullptr);
    }
    GG_CUDA(cudaGetLastError());
    return GG_OK;
  }
  // ADDS (dvdson.f90:960-1000): S(1:kp+1, kp+1) for the new columns
  // kp0..kp0+m-1 of AB, staged at their packed offsets and read back with
  // one copy into host S (packed upper)
  int adds(int kp0, int m, std::vector<double> &S) {
    for (int v = 0; v < m; ++v) {
      const int kp_ = kp0 + v;
      launch_dots(false, by_value(kp_), 1, AB.p, nullptr, -1, dS.p + (size_t)kp_ * (kp_ + 1) / 2);
    }
    GG_CUDA(cudaGetLastError());
    const size_t o0 = (size_t)kp0 * (kp0 + 1) / 2, o1 = (size_t)(kp0 + m) * (kp0 + m + 1) / 2;
    GG_CUDA(cudaMemcpyAsync(hS + o0, dS.p + o0, (o1 - o0) * sizeof(double), cudaMemcpyDeviceToHost, s));
    const auto t0 = std::chrono::steady_clock::now();
    GG_CUDA(cudaStreamSynchronize(s));
    t_wait += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    std::memcpy(S.data() + o0, hS + o0, (o1 - o0) * sizeof(double));
    return GG_OK;
  }
  // Block pass: Ritz vectors and residual norms of nt targets (coefficient
  // vectors svec[t], length k; eigenvalues lam[t]) in one sweep; rn2[t] = |r_t|^2
  bool ritz_multi_fits(int k, int nt) const { return nt <= MT_MAX && nt * k <= MT_SMEM && 2 * nt <= lim; }
  int ritz_multi(int k, int nt, const double *const *svec, const double *lam, double *rn2) {
    GG_TRY(launch_ritz_multi(k, nt, svec, lam));
    double *hl = hmt + (size_t)MT_MAX * lim;
    double *drn = dmt.p + (size_t)MT_MAX * lim + MT_MAX;
    GG_CUDA(cudaMemcpyAsync(hl + MT_MAX, drn, nt * sizeof(double), cudaMemcpyDeviceToHost, s));
    const auto t0 = std::chrono::steady_clock::now();
    GG_CUDA(cudaStreamSynchronize(s));
    t_wait += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    for (int t = 0; t < nt; ++t) rn2[t] = hl[MT_MAX + t];
    return GG_OK;
  }
  // the Ritz sweep (residual norms |r_t|^2 left on the device)
  // staged: the coefficients and eigenvalues are already in the pass's
  // input region (din_coef, din_nv()->lam)
  int launch_ritz_multi(int k, int nt, const double *const *svec, const double *lam, bool staged = false) {
    const double *dcoef = dmt.p, *dl = dmt.p + (size_t)MT_MAX * lim;
    if (staged) {
      dcoef = din_coef();
      dl = din_nv()->lam;
    } else {
      for (int t = 0; t < nt; ++t) std::memcpy(hmt + (size_t)t * k, svec[t], k * sizeof(double));
      double *hl = hmt + (size_t)MT_MAX * lim;
      for (int t = 0; t < nt; ++t) hl[t] = lam[t];
      GG_CUDA(cudaMemcpyAsync(dmt.p, hmt, (size_t)nt * k * sizeof(double), cudaMemcpyHostToDevice, s));
      GG_CUDA(cudaMemcpyAsync(dmt.p + (size_t)MT_MAX * lim, hl, nt * sizeof(double), cudaMemcpyHostToDevice, s));
    }
    double *drn = dmt.p + (size_t)MT_MAX * lim + MT_MAX;
    // one group of all targets, or (small blocks) one target per grid row
    const bool per_target = (int64_t)nrow * 2 < ctx->sms;
    if (use_x()) {
      GG_TRY(sync_split(k));
      if (per_target) {
        GG_CUDA(launch_pdl(k_ritzx_multi<1, SP>, dim3(nrow4, nt), RT, 0, s, Bx.p, ABx.p, ld, k, nt, dcoef, dl, T.p, n, part.p,
                                                       counters.p + 3, drn));
      } else {
        // an even nt as two grid rows of nt / 2 targets (twice the warps;
        // one sweep of all targets with one or two lanes per row, and finer
        // splits, measured slower)
        const int half = (nt % 2 == 0) ? 2 : 1;
        switch (nt / half) {
#define RM_CASE(K) \
  case K: GG_CUDA(launch_pdl(k_ritzx_multi<K, 1>, dim3(nrow, half), RT, 0, s, Bx.p, ABx.p, ld, k, nt, dcoef, dl, T.p, n, part.p, counters.p + 3, drn)); break;
          RM_CASE(1) RM_CASE(2) RM_CASE(3) RM_CASE(4) RM_CASE(5) RM_CASE(6) RM_CASE(7) RM_CASE(8)
          RM_CASE(9) RM_CASE(10) RM_CASE(11) RM_CASE(12) RM_CASE(13) RM_CASE(14) RM_CASE(15) RM_CASE(16)
#undef RM_CASE
          default: return fail(GG_ERR_ARG, "ritz_multi: more targets than supported");
        }
      }
    } else if (per_target) {
      GG_CUDA(launch_pdl(k_ritz_multi<1>, dim3(nrow, nt), RT, 0, s, B.p, AB.p, ld, k, nt, dcoef, dl, T.p, n, part.p, counters.p + 3,
                                                    drn));
    } else {
      switch (nt) {
#define RM_CASE(K) \
  case K: GG_CUDA(launch_pdl(k_ritz_multi<K>, nrow, RT, 0, s, B.p, AB.p, ld, k, nt, dcoef, dl, T.p, n, part.p, counters.p + 3, drn)); break;
        RM_CASE(1) RM_CASE(2) RM_CASE(3) RM_CASE(4) RM_CASE(5) RM_CASE(6) RM_CASE(7) RM_CASE(8)
        RM_CASE(9) RM_CASE(10) RM_CASE(11) RM_CASE(12) RM_CASE(13) RM_CASE(14) RM_CASE(15) RM_CASE(16)
#undef RM_CASE
        default: return fail(GG_ERR_ARG, "ritz_multi: more targets than supported");
      }
    }
    note_launch();
    GG_CUDA(cudaGetLastError());
    return GG_OK;
  }
  // One block pass with NEWVEC's choices made on the device: Ritz sweep of
  // the nt candidates, NEWVEC's choices with the preconditioners of the kept ones (the rest
  // of the mg columns zeroed), the block pass graph over mg columns. One
  // host wait, at the end. *nk = columns added, *done = all candidates
  // converged (nothing added).
  int pass_fused(int k, int nt, const double *const *svec, const NvIn &in, int mg, std::vector<double> &S, int *nk,
                 bool *done) {
    if (mg > MT_MAX || nt > MT_MAX) return fail(GG_ERR_ARG, "block pass: more targets than supported");
    // the pass's inputs in one copy: NEWVEC's, the block pass's columns, the
    // Ritz coefficients
    *reinterpret_cast<NvIn *>(hio_in) = in;
    IterParams *hp = reinterpret_cast<IterParams *>(hio_in + io_pv);
    for (int v = 0; v < mg; ++v) {
      hp[v] = IterParams{};
      hp[v].c = k + v;
    }
    double *hc = reinterpret_cast<double *>(hio_in + io_coef);
    for (int t = 0; t < nt; ++t) std::memcpy(hc + (size_t)t * k, svec[t], k * sizeof(double));
    GG_CUDA(cudaMemcpyAsync(dio_in.p, hio_in, io_coef + (size_t)nt * k * sizeof(double), cudaMemcpyHostToDevice, s));
    GG_TRY(launch_ritz_multi(k, nt, svec, in.lam, true));
    const double *drn = dmt.p + (size_t)MT_MAX * lim + MT_MAX;
    // small CTAs for small blocks: the preconditioner is FP64 work, spread
    // over more SMs
    const int tp = (n < 128 * ctx->sms) ? 64 : TPB;
    GG_TRY(ensure_wx());
    GG_CUDA(launch_pdl(k_newvec_precond, (n + tp - 1) / tp, tp, 0, s, din_nv(), drn, dout_nv(), B.p, T.p, ld, diag.p,
                       n, mg, k, use_x() ? wx.p : nullptr));
    note_launch();
    GG_CUDA(cudaGetLastError());
    GG_TRY(block_pass(k, mg, S, nk, true));  // copies NEWVEC's results with its own, waits for the stream
    *done = hout_nv()->done != 0;
    if (*nk > hout_nv()->nadded) return fail(GG_ERR_STATE, "block pass: more columns kept than added");
    return GG_OK;
  }
  int precond_multi(const PrecList &L) {
    k_precond_multi<<<(n + TPB - 1) / TPB, TPB, 0, s>>>(B.p, T.p, ld, L, diag.p, n);
    note_launch();
    GG_CUDA(cudaGetLastError());
    return GG_OK;
  }
  // X[:, 0:m) = X[:, 0:k) C (k x m): computed into T, copied back (BASIS and
  // AB keep their addresses, which the iteration graph holds)
  // (SPLIT: from the split copies, which are made current first)
  int multbc(DBuf<double> &X, DBuf<float2> &Xx, int k, int m, const double *hC) {
    if ((size_t)k * m > small.n) GG_TRY(small.alloc((size_t)k * m));
    GG_CUDA(cudaMemcpyAsync(small.p, hC, (size_t)k * m * sizeof(double), cudaMemcpyHostToDevice, s));
    if (use_x()) {
      GG_TRY(sync_split(k));
      if ((int64_t)nrow * 2 < ctx->sms)
        k_multbcx<SP><<<dim3(nrow4, (m + MB_G - 1) / MB_G), RT, 0, s>>>(Xx.p, ld, k, small.p, m, T.p, n);
      else
        k_multbcx<1><<<dim3(nrow, (m + MB_G - 1) / MB_G), RT, 0, s>>>(Xx.p, ld, k, small.p, m, T.p, n);
    } else {
      k_multbc<<<(n + RC - 1) / RC, TPB, 0, s>>>(X.p, ld, k, small.p, m, T.p, n);
    }
    note_launch();
    GG_CUDA(cudaGetLastError());
    GG_CUDA(cudaMemcpyAsync(X.p, T.p, (size_t)m * ld * sizeof(double), cudaMemcpyDeviceToDevice, s));
    return GG_OK;
  }
  // BASIS and AB both times C (OVFLOW's restart, the final eigenvectors)
  int multbc2(int k, int m, const double *hC) {
    GG_TRY(multbc(B, Bx, k, m, hC));
    GG_TRY(multbc(AB, ABx, k, m, hC));
    bx_cols = 0;  // the split copies no longer match
    return GG_OK;
  }
  // Block pass (MBLOCK > 1): Ritz vector and residual of one target into
  // column c; returns |r| (the preconditioner follows when not converged)
  int ritz(int k, const double *hsvec, double lam, double gap, double dl, double critr, int c, double *res) {
    std::memcpy(hup + 8, hsvec, k * sizeof(double));
    GG_CUDA(cudaMemcpyAsync(dup.p + 8, hup + 8, k * sizeof(double), cudaMemcpyHostToDevice, s));
    launch_ritz(by_value(c, k, lam, gap, dl, critr));
    GG_CUDA(cudaGetLastError());
    GG_CUDA(cudaMemcpyAsync(hdown + lim + 8, scal(), SC_N * sizeof(double), cudaMemcpyDeviceToHost, s));
    const auto t0 = std::chrono::steady_clock::now();
    GG_CUDA(cudaStreamSynchronize(s));
    t_wait += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    *res = std::sqrt(hdown[lim + 8 + SC_RN2]);
    return GG_OK;
  }
  int precond(int c, double lam) {
    k_precond<<<(n + TPB - 1) / TPB, TPB, 0, s>>>(B.p, AB.p, ld, by_value(c, 0, lam), scal(), diag.p, n);
    note_launch();
    GG_CUDA(cudaGetLastError());
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
  const auto t_begin = std::chrono::steady_clock::now();
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
    const int NUME1 = std::min(NUME + 1, LIM);  // no more vectors than the basis holds
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
    GG_TRY(D.adds(0, NIV, S));
  }
  int NLOOPS = 1;
  for (int i = 0; i < NUME; ++i) {
    EIGVAL[i] = 1.0e30;
    ICV[i + 1] = 0;
  }
  D.full_m = MBLOCK;
  int KPASS = NIV, NNCV = KPASS;
  int REST = std::max(LIM / 2, 2 * NUME);
  REST = std::min(REST, LIM - 3);
  bool DONE = false;
  std::vector<double> w, hlo, hhi;
  int kprev = -1, mprev = 0;  // size of S and number of eigenvalues at the previous solve
  for (;;) {
    // with the whole space in the basis every Ritz pair is exact: take all
    const int IFIND = (KPASS == n) ? KPASS : std::min(KPASS, REST);
    for (int i = 0; i < IFIND; ++i) OLDVAL[i] = EIGVAL[i];
    // DSPEVX returns IFIND eigenpairs. Read afterwards are EIGVAL(1:NUME+1)
    // (TSTSEL, NEWVEC's GAP) and the first NUME eigenvectors (TSTSEL,
    // NEWVEC, MULTBC), except when the basis is full: OVFLOW then collapses
    // onto all IFIND = REST pairs. Only those are computed.
    const bool full = (KPASS == LIM);
    const int mneed = full ? IFIND : std::min(IFIND, NUME + 1);
    const int nvecs = full ? IFIND : std::min(IFIND, NUME);
    w.assign(mneed, 0.0);
    // interlacing: S grew by p columns since the last solve (whose leading
    // block had eigenvalues OLDVAL), so lambda_j lies in
    // [OLDVAL(j-p), OLDVAL(j)]
    const double *blo = nullptr, *bhi = nullptr;
    if (kprev > 0 && KPASS > kprev) {
      const int pcols = KPASS - kprev;
      hlo.assign(mneed, -1e300);
      hhi.assign(mneed, 1e300);
      for (int j = 0; j < mneed; ++j) {
        if (j < mprev) hhi[j] = OLDVAL[j];
        if (j - pcols >= 0 && j - pcols < mprev) hlo[j] = OLDVAL[j - pcols];
      }
      blo = hlo.data();
      bhi = hhi.data();
    }
    const auto te0 = std::chrono::steady_clock::now();
    if (sym_eig_lowest(KPASS, S.data(), mneed, nvecs, w.data(), SVEC.data(), blo, bhi) != 0) {
      *ierr_out = -1;
      return fail(GG_ERR_CONVERGE, "DVDSON: projected eigenproblem failed");
    }
    D.t_eig += std::chrono::duration<double>(std::chrono::steady_clock::now() - te0).count();
    for (int i = 0; i < mneed; ++i) EIGVAL[i] = w[i];
    kprev = KPASS;
    mprev = mneed;
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
      GG_TRY(D.multbc2(KPASS, REST, SVEC.data()));
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
      kprev = REST;  // S is now diag(EIGVAL(1:REST)): its eigenvalues are known
    }
    // NEWVEC (dvdson.f90:1002-1172)
    int nadded = 0, icvc = 0;
    // GAP and DL of target indx (dvdson.f90:1128-1138). On the first pass
    // OLDVAL still holds DVDRVR's 1e30 sentinel (dvdson.f90:703): the
    // reference then shifts by RHSEPS ~ 1e13 and its first correction vector
    // carries no new direction, after which the coefficient test (CRITC) can
    // end the iteration early. robust = 1 uses DL = 0 on that pass instead.
    auto gap_dl = [&](int indx, double *gap, double *dl) {
      if (indx == 1) {
        *gap = std::fabs(EIGVAL[1] - EIGVAL[0]);
      } else {
        const double gaplow = std::fabs(EIGVAL[indx - 1] - EIGVAL[indx - 2]);
        const double gapup = std::fabs(EIGVAL[indx] - EIGVAL[indx - 1]);
        *gap = std::min(gaplow, gapup);
      }
      *dl = std::fabs(OLDVAL[indx - 1] - EIGVAL[indx - 1]);
      if (P.robust && OLDVAL[indx - 1] >= 1.0e29) *dl = 0.0;
    };
    if (MBLOCK == 1) {
      // one device pass per target: Ritz vector, shift, preconditioner,
      // Gram-Schmidt, OP and ADDS of column KPASS; a converged target's pass
      // stops after the residual and the next target takes the column
      DONE = false;
      for (int i = 1; i <= NNCV; ++i) {
        const int indx = INCV[i];
        double gap, dl, res = 0.0;
        gap_dl(indx, &gap, &dl);
        GG_TRY(D.single_pass(KPASS, SVEC.data() + (size_t)(indx - 1) * KPASS, EIGVAL[indx - 1], gap, dl, P.critr,
                             &res, S));
        SCRA1[indx - 1] = res;
        if (res < P.critr) {
          ++icvc;
          ICV[indx] = 1;
          if (icvc < NNCV) continue;
          DONE = true;
          break;
        }
        nadded = 1;
        INCV[1] = indx;
        break;
      }
      if (DONE) break;
      NNCV = nadded;
      KPASS += NNCV;
      ++NLOOPS;
      if (NLOOPS <= MAXITER) continue;
      IERR += 2048;
      --NLOOPS;
      KPASS -= NNCV;
      break;
    }
    if (D.use_fused && NNCV <= MT_MAX && D.ritz_multi_fits(KPASS, NNCV)) {
      // NEWVEC on the device: Ritz sweep, choices, preconditioners and the
      // block pass back to back, one host wait
      const int limadd = std::min(LIM, MBLOCK + KPASS);
      const int mg = std::min(NNCV, limadd - KPASS);
      NvIn in{};
      in.nt = NNCV;
      in.kpass = KPASS;
      in.limadd = limadd;
      in.critr = P.critr;
      std::vector<const double *> sv(NNCV);
      for (int t = 0; t < NNCV; ++t) {
        const int indx = INCV[t + 1];
        sv[t] = SVEC.data() + (size_t)(indx - 1) * KPASS;
        in.lam[t] = EIGVAL[indx - 1];
        gap_dl(indx, &in.gap[t], &in.dl[t]);
      }
      int nk = 0;
      bool done = false;
      GG_TRY(D.pass_fused(KPASS, NNCV, sv.data(), in, mg, S, &nk, &done));
      if (done) {
        DONE = true;
        break;
      }
      if (nk == 0) break;  // no direction outside the basis is left
      NNCV = nk;
      KPASS += NNCV;
      ++NLOOPS;
      if (NLOOPS <= MAXITER) continue;
      IERR += 2048;
      --NLOOPS;
      KPASS -= NNCV;
      break;
    }
    if (D.ritz_multi_fits(KPASS, NNCV)) {
      // every candidate target's Ritz vector and residual in one sweep;
      // NEWVEC's sequential decisions then run on the residual norms
      const int limadd = std::min(LIM, MBLOCK + KPASS);
      std::vector<int> tl(INCV.begin() + 1, INCV.begin() + 1 + NNCV);
      std::vector<const double *> sv(NNCV);
      std::vector<double> lam(NNCV), rn2(NNCV);
      for (int t = 0; t < NNCV; ++t) {
        sv[t] = SVEC.data() + (size_t)(tl[t] - 1) * KPASS;
        lam[t] = EIGVAL[tl[t] - 1];
      }
      GG_TRY(D.ritz_multi(KPASS, NNCV, sv.data(), lam.data(), rn2.data()));
      PrecList L{};
      DONE = false;
      for (int i = 1; i <= NNCV; ++i) {
        const int indx = tl[i - 1];
        double gap, dl;
        gap_dl(indx, &gap, &dl);
        const double res = std::sqrt(rn2[i - 1]);
        SCRA1[indx - 1] = res;
        if (res < P.critr) {
          ++icvc;
          ICV[indx] = 1;
          if (icvc < NNCV) continue;
          DONE = true;
          break;
        }
        ++nadded;
        INCV[nadded] = indx;
        L.col[L.m] = KPASS + nadded - 1;
        L.t[L.m] = i - 1;
        L.lam[L.m] = EIGVAL[indx - 1];
        L.rhs[L.m] = (gap > res) ? std::sqrt(dl * res) : std::min(dl, std::sqrt(dl));
        ++L.m;
        if (nadded + KPASS == limadd) break;
      }
      if (DONE) break;
      NNCV = nadded;
      GG_TRY(D.precond_multi(L));
    } else {
      const int limadd = std::min(LIM, MBLOCK + KPASS);
      DONE = false;
      for (int i = 1; i <= NNCV; ++i) {
        const int indx = INCV[i];
        // ICUR = column KPASS + NADDED (a converged target is overwritten)
        double gap, dl, res = 0.0;
        gap_dl(indx, &gap, &dl);
        const int c = KPASS + nadded;
        GG_TRY(D.ritz(KPASS, SVEC.data() + (size_t)(indx - 1) * KPASS, EIGVAL[indx - 1], gap, dl, P.critr, c, &res));
        SCRA1[indx - 1] = res;
        if (res < P.critr) {
          ++icvc;
          ICV[indx] = 1;
          if (icvc < NNCV) continue;
          DONE = true;
          break;
        }
        ++nadded;
        INCV[nadded] = indx;
        // shift + preconditioner for this column now (MBLOCK columns at most)
        GG_TRY(D.precond(c, EIGVAL[indx - 1]));
        if (nadded + KPASS == limadd) break;
      }
      if (DONE) break;
      NNCV = nadded;
    }
    // Gram-Schmidt of the new vectors, OP, ADDS
    if (NNCV <= MT_MAX) {
      int nk = 0;
      GG_TRY(D.block_pass(KPASS, NNCV, S, &nk));
      if (nk == 0) break;  // no direction outside the basis is left
      NNCV = nk;
    } else {
      for (int v = 0; v < NNCV; ++v) GG_TRY(D.orthonormalize(KPASS + v));
      GG_TRY(D.op(KPASS, NNCV));
      GG_TRY(D.adds(KPASS, NNCV, S));
    }
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
  GG_TRY(D.multbc2(KPASS, NUME, SVEC.data()));
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
  D.t_total += std::chrono::duration<double>(std::chrono::steady_clock::now() - t_begin).count();
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
  if (h->host_prec >= 0 && precision != h->host_prec)
    return fail(GG_ERR_ARG, "gg_maneig: p->precision must be the host-resident matrix's precision");
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
  P.mblock = (p && p->mblock > 1) ? std::min(p->mblock, nvec) : 1;
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
  // DVDSON keeps REST = min(max(LIM/2, 2 NUME), LIM - 3) Ritz vectors and
  // reads NUME + 1 of them: LIM >= NUME + 4 unless the basis holds the
  // whole space (LIM = NCF, solved in the full unit basis below)
  if (P.lim < nvec + 4 && P.lim != ncf) return fail(GG_ERR_ARG, "gg_maneig: LIM too small (below NVEC + 4)");
  if (P.lim > 1024) return fail(GG_ERR_ARG, "gg_maneig: LIM above 1024 is not supported");
  using hclock = std::chrono::steady_clock;
  const auto th0 = hclock::now();
  GG_TRY(refresh_sym_values(h));
  std::vector<double> ev, res;
  double mv_ms = 0;
  int mv_count = 0, nmv_total = 0, nl_total = 0;
  // Stage 1 (INIEST2, lib9290/iniest2.f90:49-95): lowest eigenvectors of the
  // leading ns x ns block, here by the same Davidson solver from unit vectors.
  const int ns = std::min(nmax, ncf);
  gg_hmat *blk = h;
  if (ns < ncf) {
    // the leading block is kept with the matrix; its values follow EMT
    if (h->lead && h->lead->ncf != ns) {
      delete h->lead;
      h->lead = nullptr;
    }
    if (!h->lead) {
      GG_TRY(h->host_prec >= 0 ? leading_block_host(h, ns, &h->lead) : leading_block(h, ns, &h->lead));
    } else if (h->host_prec < 0) {
      gg_hmat *b = h->lead;
      GG_CUDA(cudaMemcpyAsync(b->dEmt.p, h->dEmt.p, b->nnz * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
      GG_CUDA(cudaMemcpyAsync(b->dDiag.p, h->dDiag.p, ns * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
      b->sym_vals_valid = false;
    }
    blk = h->lead;
  }
  // device time to here (symmetric structures of the block and of its
  // leading block) is read at the end; host time of the workspaces apart
  if (!ctx->ev_mid) GG_CUDA(cudaEventCreate(&ctx->ev_mid));
  GG_CUDA(cudaEventRecord(ctx->ev_mid, ctx->stream));
  ctx->stats[26] = 1e3 * std::chrono::duration<double>(hclock::now() - th0).count();
  ctx->stats[27] = 0;
  // Davidson workspaces kept with the matrix, by stage and precision
  auto workspace = [&](int stage, gg_hmat *hm, int nn, int lm, Dvd **out) -> int {
    const auto tw0 = hclock::now();
    struct Acc {
      double *dst;
      hclock::time_point t0;
      ~Acc() { *dst += 1e3 * std::chrono::duration<double>(hclock::now() - t0).count(); }
    } acc{&ctx->stats[27], tw0};
    std::shared_ptr<void> &c = h->dvd_cache[2 * stage + (precision == GG_SPLIT ? 1 : 0)];
    Dvd *d = static_cast<Dvd *>(c.get());
    if (d && d->reusable(hm, precision, nn, lm)) {
      GG_TRY(d->reset());
    } else {
      c.reset();
      d = new Dvd;
      c = std::shared_ptr<void>(d, [](void *q) { delete static_cast<Dvd *>(q); });
      const int st = d->init(ctx, hm, precision, nn, lm);
      if (st != GG_OK) {
        c.reset();
        return st;
      }
    }
    *out = d;
    return GG_OK;
  };
  // warm start (rmcdhf90/maneig.f90:116-128): the caller's vectors replace
  // INIEST2's; with a leading block the stage-1 run is skipped
  const int nstart = (p && p->start && p->nstart > 0) ? p->nstart : 0;
  if (nstart > P.lim) return fail(GG_ERR_ARG, "gg_maneig: more start vectors than LIM");
  auto load_start = [&](Dvd &D) -> int {
    GG_CUDA(cudaMemcpy2DAsync(D.B.p, D.ld * 8, p->start, (size_t)ncf * 8, (size_t)ncf * 8, nstart,
                              cudaMemcpyHostToDevice, ctx->stream));
    return GG_OK;
  };
  Dvd *D1p = nullptr, *D2p = nullptr;
  Dvd D1none;  // statistics of a skipped stage 1
  ctx->stats[8] = ctx->stats[9] = ctx->stats[10] = 0;
  if (!(nstart > 0 && ns < ncf)) {
    GG_TRY(refresh_sym_values(blk));
    DvdParams P1 = P;
    // stands in for INIEST2's dense DSPEVX: converge on the residual (no
    // coefficient test) from a sane first shift
    P1.robust = 1;
    P1.critc = 0.0;
    // When a full-block run follows, to a residual of 1e-6 (or CRITR if
    // that is looser): these are only its start vectors. Looser start
    // vectors save passes here (on Fe XV 13 instead of 17 at 1e-4, the
    // full-block run keeping its 25) but let DVDSON's coefficient test
    // (CRITC, with the reference's first-pass shift) stop the full-block
    // run early on other matrices, 1e-6 Eh from the eigenvalues.
    if (ns < ncf) P1.critr = std::max(P.critr, 1e-6);
    // block Davidson: up to NUME correction vectors per pass, so far fewer
    // projected eigenproblems than one vector per pass
    P1.mblock = nvec;
    P1.lim = std::min(ns, P.lim);
    if (ns < ncf && P1.lim < P.nume + 1) P1.lim = ns;
    GG_TRY(tune_prepare(blk, precision, P1.mblock));
    GG_TRY(workspace(0, blk, ns, P1.lim, &D1p));
    Dvd &D1 = *D1p;
    GG_CUDA(cudaMemcpyAsync(D1.diag.p, blk->dDiag.p, ns * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
    // A block too small for DVDSON's restart size (NCF < NVEC + 4; the
    // reference solves such blocks densely, rci90/maneig.f90:157-241,
    // rmcdhf90/maneig.f90:104-120) starts from all NCF unit vectors: S is
    // then the whole matrix and its eigenpairs are exact after one pass.
    if (P1.lim == ns && ns < nvec + 4) P1.niv = ns;
    if (nstart > 0) {
      P1.niv = nstart;
      GG_TRY(load_start(D1));
    } else {
      GG_TRY(unit_start(D1, blk, P1.niv));
    }
    int nl = 0, ie = 0;
    GG_TRY(dvdson(D1, P1, ev, res, &nl, &ie));
    mv_ms += D1.mv_ms;
    mv_count += D1.mv_count;
    nmv_total += D1.nmv;
    nl_total += nl;
    *ierr = ie;
    ctx->stats[8] = nl;  // stage-1 (leading block) loops
    ctx->stats[9] = 0;   // stage-2 loops
    ctx->stats[10] = D1.mv_ms;
  }
  Dvd &D1 = D1p ? *D1p : D1none;
  Dvd *Dout = &D1;
  Dvd D2none;  // statistics of an absent stage 2
  if (ns < ncf) {
    // Stage 2: GDVD on the whole block from the zero-padded estimates
    GG_TRY(tune_prepare(h, precision, P.mblock));
    GG_TRY(workspace(1, h, ncf, P.lim, &D2p));
  }
  Dvd &D2 = D2p ? *D2p : D2none;
  if (ns < ncf) {
    GG_CUDA(cudaMemcpyAsync(D2.diag.p, h->dDiag.p, ncf * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
    DvdParams P2 = P;
    if (nstart > 0) {
      P2.niv = nstart;
      GG_TRY(load_start(D2));
    } else {
      GG_CUDA(cudaMemcpy2DAsync(D2.B.p, D2.ld * 8, D1.B.p, D1.ld * 8, (size_t)ns * 8, nvec, cudaMemcpyDeviceToDevice,
                                ctx->stream));
    }
    int nl = 0, ie = 0;
    GG_TRY(dvdson(D2, P2, ev, res, &nl, &ie));
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
  {
    float f = 0.f;
    GG_CUDA(cudaEventElapsedTime(&f, ctx->ev0, ctx->ev_mid));
    ctx->stats[28] = f;
  }
  ctx->stats[3] = ms;
  ctx->stats[4] = mv_ms;
  ctx->stats[5] = mv_count;
  ctx->stats[13] = 1e3 * (D1.t_eig + D2.t_eig);    // host projected eigenproblem ms
  ctx->stats[14] = 1e3 * (D1.t_wait + D2.t_wait);  // host waits on device results ms
  ctx->stats[15] = 1e3 * (D1.t_total + D2.t_total);  // host ms inside the two Davidson runs
  ctx->stats[16] = D2.pass_ms;
  ctx->stats[17] = 1e3 * D1.t_total;
  ctx->stats[18] = 1e3 * D2.t_total;
  ctx->stats[19] = 1e3 * D2.t_eig;
  ctx->stats[30] = D1.cgs_once + D2.cgs_once;
  ctx->stats[23] = D2.spmm_full_ms;
  ctx->stats[24] = D2.spmm_full_n;
  *nloops = nl_total;
  *nmv = nmv_total;
  if (*ierr & 2048) return fail(GG_ERR_CONVERGE, "DVDSON: maximum number of iterations reached (IERR 2048)");
  return GG_OK;
}
