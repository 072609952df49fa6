// spmv.cu - the Davidson matrix-vector product (SPICMV2, lib9290/spicmv2.f90)
// on the GPU.
//
// The reference keeps the lower triangle by rows (diagonal last) and does,
// row by row, C(i) += H(i,i) B(i) + sum_j H(i,j) B(j) and C(j) += H(i,j) B(i)
// (DMERGE). On the GPU the scattered second update would need atomics, whose
// order (and rounding) changes from run to run. Instead the structure is
// expanded once into a full symmetric CSR (own row, then the transposed
// entries in increasing source row), built by a deterministic chunked
// transpose; each row is then one warp-reduced dot product, so the result is
// reproducible bit for bit.
//
// Precision modes:
//   GG_FP64   y = H x in FP64 (one DFMA per stored entry).
//   GG_SPLIT  off-diagonal H stored as hi + lo FP32 pairs, x split the same
//             way, products and sums in double-float arithmetic on the FP32
//             pipe (about 2^-44 relative), the diagonal term in FP64. GB300's
//             FP64 pipe issues roughly 1/64 of its FP32 rate, so FP64 SpMV is
//             issue-bound at about the HBM rate; the split form is not.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "gg_internal.cuh"

namespace gg {
namespace {

constexpr int NCHUNK = 1024;  // most row chunks of the symmetric structure build

// counts of transposed entries per (chunk, column)
// per chunk of rows, how many of its stored entries fall in each column c
// (entries above the diagonal of the symmetric matrix); warps take rows
__global__ void k_tcount(const int64_t *__restrict__ iendc, const int32_t *__restrict__ irow,
                         const int *__restrict__ chunk_r0, int ncf, int *__restrict__ cnt) {
  const int ch = blockIdx.x;
  const int r0 = chunk_r0[ch], r1 = chunk_r0[ch + 1];
  int *c = cnt + (size_t)ch * ncf;
  const int lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int r = r0 + (threadIdx.x >> 5); r < r1; r += nw) {
    const int64_t lo = iendc[r], hi = iendc[r + 1] - 1;  // last entry is the diagonal
    for (int64_t p = lo + lane; p < hi; p += 32) atomicAdd(&c[irow[p] - 1], 1);
  }
}

// cursor(chunk, col) = start of col's transposed part + entries of earlier chunks
__global__ void k_cursor(const int *__restrict__ cnt, int ncf, int nch, const int64_t *__restrict__ iendc,
                         int *__restrict__ cursor) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < ncf; c += gridDim.x * blockDim.x) {
    int pos = (int)(iendc[c + 1] - iendc[c]);  // the row's own entries come first
#pragma unroll 8
    for (int ch = 0; ch < nch; ++ch) {
      cursor[(size_t)ch * ncf + c] = pos;
      pos += cnt[(size_t)ch * ncf + c];
    }
  }
}

__global__ void k_tcol_total(const int *__restrict__ cnt, int ncf, int nch, const int64_t *__restrict__ iendc,
                             int64_t *__restrict__ rowlen) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < ncf; c += gridDim.x * blockDim.x) {
    int64_t t = iendc[c + 1] - iendc[c];
#pragma unroll 8
    for (int ch = 0; ch < nch; ++ch) t += cnt[(size_t)ch * ncf + c];
    rowlen[c] = t;
  }
}

// transposed placement: rows of a chunk in order; within one row the columns
// are distinct, so the cursors need no atomics
// rows of a chunk in order, the entries of a row in parallel (distinct
// columns): entry (r, c) goes to row c at symptr[c] + cur[c], so each row's
// entries from other rows ascend in r; cursor holds offsets within the row
__global__ void k_tplace(const int64_t *__restrict__ iendc, const int32_t *__restrict__ irow,
                         const int *__restrict__ chunk_r0, int ncf, const int64_t *__restrict__ symptr,
                         int *__restrict__ cursor, int32_t *__restrict__ scol, int64_t *__restrict__ ssrc) {
  const int ch = blockIdx.x;
  const int r0 = chunk_r0[ch], r1 = chunk_r0[ch + 1];
  int *cur = cursor + (size_t)ch * ncf;
  for (int r = r0; r < r1; ++r) {
    const int64_t lo = iendc[r], hi = iendc[r + 1] - 1;
    for (int64_t p = lo + threadIdx.x; p < hi; p += blockDim.x) {
      const int c = irow[p] - 1;
      const int q = cur[c];
      cur[c] = q + 1;
      const int64_t pos = symptr[c] + q;
      scol[pos] = r;
      ssrc[pos] = p;
    }
    __syncthreads();
  }
}
// k_tplace with the chunk's cursor row in shared memory (NCF ints): the
// per-entry read-modify-write of the cursor stays on chip
constexpr int TPLACE_SMEM_MAX = 200 * 1024;
__global__ void k_tplace_smem(const int64_t *__restrict__ iendc, const int32_t *__restrict__ irow,
                              const int *__restrict__ chunk_r0, int ncf, const int64_t *__restrict__ symptr,
                              const int *__restrict__ cursor, int32_t *__restrict__ scol,
                              int64_t *__restrict__ ssrc) {
  extern __shared__ int cur[];
  const int ch = blockIdx.x;
  const int r0 = chunk_r0[ch], r1 = chunk_r0[ch + 1];
  if (r0 == r1) return;
  const int *c0 = cursor + (size_t)ch * ncf;
  for (int c = threadIdx.x; c < ncf; c += blockDim.x) cur[c] = c0[c];
  __syncthreads();
  for (int r = r0; r < r1; ++r) {
    const int64_t lo = iendc[r], hi = iendc[r + 1] - 1;
    for (int64_t p = lo + threadIdx.x; p < hi; p += blockDim.x) {
      const int c = irow[p] - 1;
      const int q = cur[c];
      cur[c] = q + 1;
      const int64_t pos = symptr[c] + q;
      scol[pos] = r;
      ssrc[pos] = p;
    }
    __syncthreads();
  }
}

__global__ void k_own(const int64_t *__restrict__ iendc, const int32_t *__restrict__ irow, int ncf,
                      const int64_t *__restrict__ symptr, int32_t *__restrict__ scol, int64_t *__restrict__ ssrc) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= ncf) return;
  const int64_t lo = iendc[warp], hi = iendc[warp + 1];
  const int64_t base = symptr[warp];
  for (int64_t p = lo + lane; p < hi; p += 32) {
    scol[base + (p - lo)] = irow[p] - 1;
    ssrc[base + (p - lo)] = p;
  }
}

// exclusive scan of the row lengths into ptr[0..n] by one CTA of 1024
// threads: thread t sums its contiguous slice, the slice sums are scanned
// with warp shuffles, then each thread writes its slice's prefix
__global__ void __launch_bounds__(1024) k_rowlen_scan(const int64_t *__restrict__ rowlen, int n,
                                                      int64_t *__restrict__ ptr) {
  __shared__ long long wsum[32];
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  const int per = (n + 1023) / 1024;
  const int i0 = min(n, t * per), i1 = min(n, i0 + per);
  long long my = 0;
  for (int i = i0; i < i1; ++i) my += rowlen[i];
  long long x = my;  // inclusive scan within the warp
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const long long y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) wsum[w] = x;
  __syncthreads();
  if (w == 0) {
    long long v = wsum[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const long long y = __shfl_up_sync(0xffffffffu, v, o);
      if (lane >= o) v += y;
    }
    wsum[lane] = v;  // inclusive over warps
  }
  __syncthreads();
  long long base = x - my + (w > 0 ? wsum[w - 1] : 0);
  for (int i = i0; i < i1; ++i) {
    ptr[i] = base;
    base += rowlen[i];
  }
  if (t == 1023) ptr[n] = x + (w > 0 ? wsum[w - 1] : 0);
}

// values: FP64 copy and the hi/lo split (diagonal excluded from the split)
__global__ void k_symvals(const int64_t *__restrict__ symptr, const int32_t *__restrict__ scol,
                          const int64_t *__restrict__ ssrc, const double *__restrict__ emt, int ncf,
                          double *__restrict__ sval, float *__restrict__ shi, float *__restrict__ slo) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= ncf) return;
  for (int64_t p = symptr[warp] + lane; p < symptr[warp + 1]; p += 32) {
    const double v = emt[ssrc[p]];
    sval[p] = v;
    if (scol[p] == warp) {
      shi[p] = 0.f;
      slo[p] = 0.f;
    } else {
      const float h = __double2float_rn(v);
      shi[p] = h;
      slo[p] = __double2float_rn(v - (double)h);
    }
  }
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// y = H x, FP64, one warp per row
__global__ void __launch_bounds__(256) k_spmv64(const int64_t *__restrict__ ptr, const int32_t *__restrict__ col,
                                                const double *__restrict__ val, const double *__restrict__ x,
                                                double *__restrict__ y, int n) {
  const int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (row >= n) return;
  const int64_t lo = ptr[row], hi = ptr[row + 1];
  double acc = 0.0;
  for (int64_t p = lo + lane; p < hi; p += 32) acc = fma(__ldg(val + p), __ldg(x + __ldg(col + p)), acc);
  acc = warp_sum(acc);
  if (lane == 0) y[row] = acc;
}

// double-float helpers (Dekker / Knuth error-free transformations)
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

__global__ void k_split_x(const double *__restrict__ x, float2 *__restrict__ xs, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double v = x[i];
    const float h = __double2float_rn(v);
    xs[i] = make_float2(h, __double2float_rn(v - (double)h));
  }
}

// y = H x with H_offdiag = hi + lo (FP32 pair), x = xh + xl; double-float
// accumulation; FP64 diagonal. LPR lanes per row (32: a warp; 16: two rows
// per warp), U loads in flight per lane (the autotuner picks both).
template <int LPR>
__device__ __forceinline__ unsigned row_mask() {
  return LPR == 32 ? 0xffffffffu : (0xffffu << (threadIdx.x & 16));
}
template <int LPR>
__device__ __forceinline__ df row_reduce(df acc) {
  const unsigned mk = row_mask<LPR>();
#pragma unroll
  for (int o = LPR / 2; o > 0; o >>= 1) {
    df other;
    other.h = __shfl_xor_sync(mk, acc.h, o);
    other.l = __shfl_xor_sync(mk, acc.l, o);
    acc = df_add(acc, other);
  }
  return acc;
}
template <typename CI, int LPR, int U>
__global__ void __launch_bounds__(256) k_spmv_split(const int64_t *__restrict__ ptr, const CI *__restrict__ col,
                                                    const float *__restrict__ hi, const float *__restrict__ lo,
                                                    const float2 *__restrict__ xs, const double *__restrict__ diag,
                                                    const double *__restrict__ x, double *__restrict__ y, int n) {
  const int row = (blockIdx.x * blockDim.x + threadIdx.x) / LPR, lane = threadIdx.x % LPR;
  if (row >= n) return;  // whole LPR-lane groups leave together
  const int64_t p0 = ptr[row], p1 = ptr[row + 1];
  df acc = {0.f, 0.f};
  // unrolled so that several iterations' loads (and the dependent x gathers)
  // are in flight together; the additions keep their order
#pragma unroll U
  for (int64_t p = p0 + lane; p < p1; p += LPR) {
    const float ah = __ldg(hi + p), al = __ldg(lo + p);
    const float2 xv = __ldg(xs + __ldg(col + p));
    const float ph = ah * xv.x;
    const float pe = fmaf(ah, xv.x, -ph);               // exact low part of ah*xh
    const float cross = fmaf(ah, xv.y, fmaf(al, xv.x, pe));
    acc = df_add(acc, two_sum(ph, cross));
  }
  acc = row_reduce<LPR>(acc);
  if (lane == 0) y[row] = ((double)acc.h + (double)acc.l) + diag[row] * x[row];
}

// Column-indexed forms for the Davidson iteration graph: x = Bbase + c ld,
// y = ABbase + c ld with c read from device memory at run time; nothing is
// done when skip points to a non-zero flag. The split form reads x from its
// hi+lo copy, which the caller prepared.
__global__ void __launch_bounds__(256) k_spmv64_col(const int64_t *__restrict__ ptr, const int32_t *__restrict__ col,
                                                    const double *__restrict__ val, const double *__restrict__ Bbase,
                                                    double *__restrict__ ABbase, int64_t ld,
                                                    const int *__restrict__ pc, const double *skip, int n) {
  if (skip && *skip != 0.0) return;
  const int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (row >= n) return;
  const size_t off = (size_t)(*pc) * ld;
  const double *x = Bbase + off;
  const int64_t lo = ptr[row], hi = ptr[row + 1];
  double acc = 0.0;
  for (int64_t p = lo + lane; p < hi; p += 32) acc = fma(__ldg(val + p), x[__ldg(col + p)], acc);
  acc = warp_sum(acc);
  if (lane == 0) ABbase[off + row] = acc;
}

template <typename CI, int LPR, int U>
__global__ void __launch_bounds__(256) k_spmv_split_col(const int64_t *__restrict__ ptr, const CI *__restrict__ col,
                                                        const float *__restrict__ hi, const float *__restrict__ lo,
                                                        const float2 *__restrict__ xs, const double *__restrict__ diag,
                                                        const double *__restrict__ Bbase, double *__restrict__ ABbase,
                                                        int64_t ld, const int *__restrict__ pc, const double *skip,
                                                        int n) {
  if (skip && *skip != 0.0) return;
  const int row = (blockIdx.x * blockDim.x + threadIdx.x) / LPR, lane = threadIdx.x % LPR;
  if (row >= n) return;
  const size_t off = (size_t)(*pc) * ld;
  const int64_t p0 = ptr[row], p1 = ptr[row + 1];
  df acc = {0.f, 0.f};
#pragma unroll U
  for (int64_t p = p0 + lane; p < p1; p += LPR) {
    const float ah = __ldg(hi + p), al = __ldg(lo + p);
    const float2 xv = xs[__ldg(col + p)];
    const float ph = ah * xv.x;
    const float pe = fmaf(ah, xv.x, -ph);
    const float cross = fmaf(ah, xv.y, fmaf(al, xv.x, pe));
    acc = df_add(acc, two_sum(ph, cross));
  }
  acc = row_reduce<LPR>(acc);
  if (lane == 0) ABbase[off + row] = ((double)acc.h + (double)acc.l) + diag[row] * Bbase[off + row];
}

// Y = H X for the m new columns of a Davidson block pass in one sweep over
// the matrix (SPLIT): X interleaved by row, xb[j MP + v] = hi + lo of x_v[j]
// (MP = spmm_pitch(m)); y_v = ABbase + (kpass + v) ld with kpass = *pc on the
// device (0 when pc is null), the diagonal term from the FP64
// x_v = Bbase + (kpass + v) ld. One warp per row. A stored entry is taken by
// LPE = ceil(m / 2) lanes, lane u reading piece u of the gathered row
// (vectors 2u, 2u + 1), so that a load instruction touches EPW = 32 / LPE
// whole rows of xb instead of 32 scattered ones. Products go into per-vector
// Dot2 sums (Ogita, Rump & Oishi), added over the EPW entry slots by a fixed
// shuffle tree in double-float. U loads in flight per lane; any block size
// that is a multiple of 32 up to 512 (the autotuner picks both).
template <int M, typename CI, int U>
__global__ void __launch_bounds__(512) k_spmm_split(const int64_t *__restrict__ ptr, const CI *__restrict__ col,
                                                    const float *__restrict__ hi, const float *__restrict__ lo,
                                                    const float2 *__restrict__ xb, const double *__restrict__ diag,
                                                    const double *__restrict__ Bbase, double *__restrict__ ABbase,
                                                    int64_t ld, const int *__restrict__ pc, int n) {
  pdl_wait();
  constexpr int MP = spmm_pitch(M), LPE = (M + 1) / 2, EPW = 32 / LPE;
  const int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (row >= n) return;
  const int e = lane / LPE, u = lane % LPE;
  const bool act = e < EPW;
  const int64_t p0 = ptr[row], p1 = ptr[row + 1];
  const float4 *xr = reinterpret_cast<const float4 *>(xb) + u;
  float h0 = 0.f, l0 = 0.f, h1 = 0.f, l1 = 0.f;
  auto step = [&](float &sh, float &sl, float ah, float al, float xh, float xl) {
    const float ph = __fmul_rn(ah, xh);
    const float t = fmaf(ah, xl, fmaf(al, xh, fmaf(ah, xh, -ph)));
    const float sn = __fadd_rn(sh, ph);
    const float bb = __fsub_rn(sn, sh);
    const float err = __fadd_rn(__fsub_rn(sh, __fsub_rn(sn, bb)), __fsub_rn(ph, bb));
    sh = sn;
    sl = __fadd_rn(sl, __fadd_rn(err, t));
  };
  if (act) {
#pragma unroll U
    for (int64_t p = p0 + e; p < p1; p += EPW) {
      const float ah = __ldg(hi + p), al = __ldg(lo + p);
      const float4 x = __ldg(xr + (size_t)__ldg(col + p) * (MP / 2));
      step(h0, l0, ah, al, x.x, x.y);
      if (2 * u + 1 < M) step(h1, l1, ah, al, x.z, x.w);
    }
  }
  df a0 = two_sum(h0, l0), a1 = two_sum(h1, l1);
  // slot e takes slot e + s (s = 1, 2, 4, ...) for e a multiple of 2 s
#pragma unroll
  for (int s = 1; s < EPW; s <<= 1) {
    df o0, o1;
    o0.h = __shfl_down_sync(0xffffffffu, a0.h, s * LPE);
    o0.l = __shfl_down_sync(0xffffffffu, a0.l, s * LPE);
    o1.h = __shfl_down_sync(0xffffffffu, a1.h, s * LPE);
    o1.l = __shfl_down_sync(0xffffffffu, a1.l, s * LPE);
    if (e % (2 * s) == 0 && e + s < EPW) {
      a0 = df_add(a0, o0);
      a1 = df_add(a1, o1);
    }
  }
  if (e != 0) return;
  const size_t off = (pc ? (size_t)(*pc) : 0) * ld + row;
  const double dg = diag[row];
  const size_t o0 = off + (size_t)(2 * u) * ld;
  ABbase[o0] = ((double)a0.h + (double)a0.l) + dg * Bbase[o0];
  if (2 * u + 1 < M) {
    const size_t o1 = o0 + ld;
    ABbase[o1] = ((double)a1.h + (double)a1.l) + dg * Bbase[o1];
  }
}

// xb[i mp + v] = hi + lo of x[v ld + i] for v < m, zero for m <= v < mp
__global__ void k_split_block(const double *__restrict__ x, int64_t ld, int m, int mp, int n, float2 *__restrict__ xb) {
  const int64_t tot = (int64_t)n * mp;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < tot; e += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(e / mp), v = (int)(e % mp);
    float2 r = make_float2(0.f, 0.f);
    if (v < m) {
      const double d = x[(size_t)v * ld + i];
      const float h = __double2float_rn(d);
      r = make_float2(h, __double2float_rn(d - (double)h));
    }
    xb[e] = r;
  }
}

// 16-bit copy of the column indices (blocks of at most 65,536 CSFs): the
// split matvec then reads 10 bytes per stored entry instead of 12
__global__ void k_col16(const int32_t *__restrict__ col, int64_t nnz, unsigned short *__restrict__ c16) {
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < nnz; p += (int64_t)gridDim.x * blockDim.x)
    c16[p] = (unsigned short)col[p];
}

}  // namespace

// ---------------------------------------------------------------------------
// SpMV autotuner. Kernel 0 is the split block matvec over m vectors
// (k_spmm_split<m>): 9 variants, U = 2, 4, 8 loads in flight per lane x
// 128, 256, 512 threads per block. Kernel 1 is the single-vector split
// matvec (k_spmv_split and its column-indexed form for the single-vector
// pass): 6 variants, 32 or 16 lanes per row x U = 2, 4, 8. The first launch
// of a kernel for a matrix shape (device, NCF, stored elements, column width)
// and m that is not inside a stream capture times every variant on a
// scratch input with CUDA events (one warm-up, three timed launches each)
// and keeps the fastest for that shape in this process; inside a capture,
// before any tuning, the default variant runs. gg_hmat_tune_force pins a
// variant for one matrix.
// ---------------------------------------------------------------------------
constexpr int TUNE_NVAR[2] = {9, 6};
constexpr int TUNE_DEFAULT[2] = {4, 1};   // U = 4, 256 threads; 32 lanes per row, U = 4
constexpr int TUNE_REPS = 3;

struct TuneKey {
  int dev, kernel, m, ncf;
  int64_t nnz;
  bool col16;
  bool host;  // the matrix in host memory (read over the host link)
  bool operator<(const TuneKey &o) const {
    return std::tie(dev, kernel, m, ncf, nnz, col16, host) <
           std::tie(o.dev, o.kernel, o.m, o.ncf, o.nnz, o.col16, o.host);
  }
};
struct TuneEntry {
  int variant = -1;
  double ms[16] = {};
};
std::mutex g_tune_mu;
std::map<TuneKey, TuneEntry> g_tune;

TuneKey tune_key(const gg_hmat *h, int kernel, int m) {
  return TuneKey{h->ctx->device, kernel, kernel == 0 ? m : 1, h->ncf, h->sym_nnz, h->sym_col16, h->host_prec >= 0};
}

template <int M, int U>
void launch_spmm_mu(const gg_hmat *h, int tpb, const float2 *xb, const double *Bbase, double *ABbase, int64_t ld,
                    const int *dcol, cudaStream_t s) {
  const int n = h->ncf;
  const unsigned blocks = (unsigned)(((int64_t)n * 32 + tpb - 1) / tpb);
  // a programmatic launch: inside the Davidson block pass it may be
  // scheduled while the pass's previous kernel finishes
  if (h->sym_col16)
    launch_pdl(k_spmm_split<M, unsigned short, U>, blocks, tpb, 0, s, h->dSymPtr.p, h->dSymCol16.p, h->dSymHi.p,
               h->dSymLo.p, xb, h->dDiag.p, Bbase, ABbase, ld, dcol, n);
  else
    launch_pdl(k_spmm_split<M, int32_t, U>, blocks, tpb, 0, s, h->dSymPtr.p, h->dSymCol.p, h->dSymHi.p, h->dSymLo.p,
               xb, h->dDiag.p, Bbase, ABbase, ld, dcol, n);
}
template <int M>
void launch_spmm_m(const gg_hmat *h, int variant, const float2 *xb, const double *Bbase, double *ABbase, int64_t ld,
                   const int *dcol, cudaStream_t s) {
  const int tpb = 128 << (variant % 3);
  switch (variant / 3) {
    case 0: launch_spmm_mu<M, 2>(h, tpb, xb, Bbase, ABbase, ld, dcol, s); break;
    case 1: launch_spmm_mu<M, 4>(h, tpb, xb, Bbase, ABbase, ld, dcol, s); break;
    default: launch_spmm_mu<M, 8>(h, tpb, xb, Bbase, ABbase, ld, dcol, s); break;
  }
}
int launch_spmm(const gg_hmat *h, int m, int variant, const float2 *xb, const double *Bbase, double *ABbase,
                int64_t ld, const int *dcol, cudaStream_t s) {
  switch (m) {
#define SPMM_CASE(K) \
  case K: launch_spmm_m<K>(h, variant, xb, Bbase, ABbase, ld, dcol, s); break;
    SPMM_CASE(1) SPMM_CASE(2) SPMM_CASE(3) SPMM_CASE(4) SPMM_CASE(5) SPMM_CASE(6) SPMM_CASE(7) SPMM_CASE(8)
    SPMM_CASE(9) SPMM_CASE(10) SPMM_CASE(11) SPMM_CASE(12) SPMM_CASE(13) SPMM_CASE(14) SPMM_CASE(15) SPMM_CASE(16)
#undef SPMM_CASE
    default: return fail(GG_ERR_ARG, "spmm_block: 1 to 16 columns");
  }
  ::gg::note_launch();
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

template <int LPR, int U>
void launch_spmv_lu(const gg_hmat *h, const float2 *xs, const double *x, double *y, const double *Bbase,
                    double *ABbase, int64_t ld, const int *dcol, const double *skip, bool colform, cudaStream_t s) {
  const int n = h->ncf;
  const unsigned blocks = (unsigned)(((int64_t)n * LPR + 255) / 256);
  if (colform) {
    if (h->sym_col16)
      k_spmv_split_col<unsigned short, LPR, U><<<blocks, 256, 0, s>>>(
          h->dSymPtr.p, h->dSymCol16.p, h->dSymHi.p, h->dSymLo.p, xs, h->dDiag.p, Bbase, ABbase, ld, dcol, skip, n);
    else
      k_spmv_split_col<int32_t, LPR, U><<<blocks, 256, 0, s>>>(h->dSymPtr.p, h->dSymCol.p, h->dSymHi.p, h->dSymLo.p,
                                                               xs, h->dDiag.p, Bbase, ABbase, ld, dcol, skip, n);
  } else {
    if (h->sym_col16)
      k_spmv_split<unsigned short, LPR, U><<<blocks, 256, 0, s>>>(h->dSymPtr.p, h->dSymCol16.p, h->dSymHi.p,
                                                                  h->dSymLo.p, xs, h->dDiag.p, x, y, n);
    else
      k_spmv_split<int32_t, LPR, U><<<blocks, 256, 0, s>>>(h->dSymPtr.p, h->dSymCol.p, h->dSymHi.p, h->dSymLo.p, xs,
                                                           h->dDiag.p, x, y, n);
  }
}
// the single-vector split matvec, variant v: y = H x (colform false) or the
// column-indexed form
int launch_spmv(const gg_hmat *h, int v, const float2 *xs, const double *x, double *y, const double *Bbase,
                double *ABbase, int64_t ld, const int *dcol, const double *skip, bool colform, cudaStream_t s) {
  switch (v) {
    case 0: launch_spmv_lu<32, 2>(h, xs, x, y, Bbase, ABbase, ld, dcol, skip, colform, s); break;
    case 1: launch_spmv_lu<32, 4>(h, xs, x, y, Bbase, ABbase, ld, dcol, skip, colform, s); break;
    case 2: launch_spmv_lu<32, 8>(h, xs, x, y, Bbase, ABbase, ld, dcol, skip, colform, s); break;
    case 3: launch_spmv_lu<16, 2>(h, xs, x, y, Bbase, ABbase, ld, dcol, skip, colform, s); break;
    case 4: launch_spmv_lu<16, 4>(h, xs, x, y, Bbase, ABbase, ld, dcol, skip, colform, s); break;
    default: launch_spmv_lu<16, 8>(h, xs, x, y, Bbase, ABbase, ld, dcol, skip, colform, s); break;
  }
  ::gg::note_launch();
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

// times every variant of `kernel` for this matrix and m; records the choice
int tune_now(gg_hmat *h, int kernel, int m, TuneEntry *out) {
  cudaStream_t s = h->ctx->stream;
  const int n = h->ncf, mm = kernel == 0 ? m : 1, mp = spmm_pitch(mm);
  DBuf<double> x, y;
  DBuf<float2> xb;
  GG_TRY(x.alloc((size_t)n * mm));
  GG_TRY(y.alloc((size_t)n * mm));
  GG_TRY(xb.alloc((size_t)n * mp));
  std::vector<double> hx((size_t)n * mm);
  for (size_t i = 0; i < hx.size(); ++i) hx[i] = 1.0 / (1.0 + (double)(i % 97));
  GG_CUDA(cudaMemcpyAsync(x.p, hx.data(), hx.size() * 8, cudaMemcpyHostToDevice, s));
  k_split_block<<<(unsigned)std::min<int64_t>(((int64_t)n * mp + 255) / 256, 4096), 256, 0, s>>>(x.p, n, mm, mp, n,
                                                                                                 xb.p);
  ::gg::note_launch();
  cudaEvent_t e0, e1;
  GG_CUDA(cudaEventCreate(&e0));
  GG_CUDA(cudaEventCreate(&e1));
  TuneEntry t;
  double best = 1e300;
  int rc = GG_OK;
  for (int v = 0; v < TUNE_NVAR[kernel] && rc == GG_OK; ++v) {
    auto one = [&]() {
      return kernel == 0 ? launch_spmm(h, mm, v, xb.p, x.p, y.p, n, nullptr, s)
                         : launch_spmv(h, v, xb.p, x.p, y.p, nullptr, nullptr, 0, nullptr, nullptr, false, s);
    };
    rc = one();  // warm-up
    if (rc != GG_OK) break;
    if (cudaEventRecord(e0, s) != cudaSuccess) rc = fail(GG_ERR_CUDA, "tuner: event record");
    for (int r = 0; r < TUNE_REPS && rc == GG_OK; ++r) rc = one();
    if (rc != GG_OK) break;
    if (cudaEventRecord(e1, s) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess) {
      rc = fail(GG_ERR_CUDA, "tuner: event wait");
      break;
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    t.ms[v] = ms / TUNE_REPS;
    if (t.ms[v] < best) {
      best = t.ms[v];
      t.variant = v;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc != GG_OK) return rc;
  *out = t;
  return GG_OK;
}

// the variant to launch: forced for this matrix, else the tuned choice for
// its shape (tuning now when the stream is not being captured), else the
// default
int tune_variant(gg_hmat *h, int kernel, int m, cudaStream_t s, int *variant) {
  const int fm = kernel == 0 ? m : 1;
  if (h->tune_force[kernel][fm] >= 0) {
    *variant = h->tune_force[kernel][fm];
    return GG_OK;
  }
  const TuneKey key = tune_key(h, kernel, m);
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune.find(key);
    if (it != g_tune.end()) {
      *variant = it->second.variant;
      return GG_OK;
    }
  }
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  GG_CUDA(cudaStreamIsCapturing(s, &cs));
  if (cs != cudaStreamCaptureStatusNone) {
    *variant = TUNE_DEFAULT[kernel];
    return GG_OK;
  }
  TuneEntry t;
  GG_TRY(tune_now(h, kernel, m, &t));
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune[key] = t;
  *variant = t.variant;
  return GG_OK;
}

// a host-resident matrix holds the values of one precision only
int check_precision(const gg_hmat *h, int precision) {
  if (h->host_prec >= 0 && precision != h->host_prec)
    return fail(GG_ERR_ARG, "matvec: the host-resident matrix was built for the other precision");
  return GG_OK;
}

// y = H x with x = Bbase + c ld, y = ABbase + c ld, c = *dcol on the device;
// GG_SPLIT reads x from h->dXs (the caller's split copy of the same column)
int spmv_col(gg_hmat *h, int precision, const double *Bbase, double *ABbase, int64_t ld, const int *dcol,
             const double *skip, cudaStream_t s, const float2 *xs) {
  GG_TRY(check_precision(h, precision));
  const int n = h->ncf;
  const unsigned blocks = (unsigned)(((int64_t)n * 32 + 255) / 256);
  if (precision == GG_SPLIT) {
    if (!xs) {
      if (h->dXs.n < (size_t)n) return fail(GG_ERR_STATE, "spmv_col: split copy of x not allocated");
      xs = h->dXs.p;
    }
    int v = 0;
    GG_TRY(tune_variant(h, 1, 1, s, &v));
    return launch_spmv(h, v, xs, nullptr, nullptr, Bbase, ABbase, ld, dcol, skip, true, s);
  } else {
    k_spmv64_col<<<blocks, 256, 0, s>>>(h->dSymPtr.p, h->dSymCol.p, h->dSymVal.p, Bbase, ABbase, ld, dcol, skip, n);
    ::gg::note_launch();
  }
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

int build_sym(gg_hmat *h) {
  if (h->sym_valid) return GG_OK;
  gg_ctx *ctx = h->ctx;
  cudaStream_t s = ctx->stream;
  const int ncf = h->ncf;
  // row chunks balanced by work: about one per 32 rows, at most NCHUNK and
  // as many as the per-chunk count and cursor arrays (8 bytes per chunk and
  // row) allow within 512 MB; k_tplace walks each chunk's rows in order
  const int nch = (int)std::max<int64_t>(
      1, std::min<int64_t>({(int64_t)ncf / 32, (int64_t)NCHUNK, std::max<int64_t>(128, (512ll << 20) / (8ll * ncf))}));
  std::vector<int> r0(nch + 1, ncf);
  r0[0] = 0;
  {
    // a row costs its entries plus a block-wide step (256 entries' worth)
    const double per = ((double)h->nnz + 256.0 * ncf) / nch;
    int c = 1;
    for (int r = 0; r < ncf && c < nch; ++r)
      if ((double)h->hIendc[r + 1] + 256.0 * (r + 1) >= per * c) r0[c++] = r + 1;
    for (; c < nch; ++c) r0[c] = ncf;
    r0[nch] = ncf;
    for (int i = 1; i <= nch; ++i) r0[i] = std::max(r0[i], r0[i - 1]);
  }
  DBuf<int> dr0, cnt, cursor;
  DBuf<int64_t> rowlen;
  GG_TRY(dr0.alloc(nch + 1));
  GG_CUDA(cudaMemcpyAsync(dr0.p, r0.data(), (nch + 1) * sizeof(int), cudaMemcpyHostToDevice, s));
  GG_TRY(cnt.alloc((size_t)nch * ncf));
  GG_CUDA(cudaMemsetAsync(cnt.p, 0, (size_t)nch * ncf * sizeof(int), s));
  k_tcount<<<nch, 256, 0, s>>>(h->dIendc.p, h->dIrow.p, dr0.p, ncf, cnt.p); ::gg::note_launch();
  GG_CUDA(cudaGetLastError());
  GG_TRY(rowlen.alloc(ncf));
  k_tcol_total<<<(ncf + 255) / 256, 256, 0, s>>>(cnt.p, ncf, nch, h->dIendc.p, rowlen.p); ::gg::note_launch();
  GG_TRY(h->dSymPtr.alloc(ncf + 1));
  k_rowlen_scan<<<1, 1024, 0, s>>>(rowlen.p, ncf, h->dSymPtr.p); ::gg::note_launch();
  GG_CUDA(cudaGetLastError());
  int64_t total = 0;
  GG_CUDA(cudaMemcpyAsync(&total, h->dSymPtr.p + ncf, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  GG_CUDA(cudaStreamSynchronize(s));
  if (total != 2 * h->nnz - ncf) return fail(GG_ERR_STATE, "build_sym: inconsistent structure");
  h->sym_nnz = total;
  GG_TRY(h->dSymCol.alloc(total));
  GG_TRY(h->dSymSrc.alloc(total));
  GG_TRY(cursor.alloc((size_t)nch * ncf));
  k_cursor<<<(ncf + 255) / 256, 256, 0, s>>>(cnt.p, ncf, nch, h->dIendc.p, cursor.p); ::gg::note_launch();
  k_own<<<(ncf * 32 + 255) / 256, 256, 0, s>>>(h->dIendc.p, h->dIrow.p, ncf, h->dSymPtr.p, h->dSymCol.p, h->dSymSrc.p); ::gg::note_launch();
  if ((size_t)ncf * sizeof(int) <= (size_t)TPLACE_SMEM_MAX) {
    const int smem = ncf * (int)sizeof(int);
    GG_CUDA(cudaFuncSetAttribute(k_tplace_smem, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    k_tplace_smem<<<nch, 1024, smem, s>>>(h->dIendc.p, h->dIrow.p, dr0.p, ncf, h->dSymPtr.p, cursor.p,
                                           h->dSymCol.p, h->dSymSrc.p);
  } else {
    k_tplace<<<nch, 256, 0, s>>>(h->dIendc.p, h->dIrow.p, dr0.p, ncf, h->dSymPtr.p, cursor.p, h->dSymCol.p,
                                 h->dSymSrc.p);
  }
  ::gg::note_launch();
  GG_CUDA(cudaGetLastError());
  if (ncf <= 65536) {
    GG_TRY(h->dSymCol16.alloc(h->sym_nnz));
    k_col16<<<1024, 256, 0, s>>>(h->dSymCol.p, h->sym_nnz, h->dSymCol16.p);
    ::gg::note_launch();
    h->sym_col16 = true;
  }
  GG_CUDA(cudaGetLastError());
  GG_CUDA(cudaStreamSynchronize(s));
  h->sym_valid = true;
  h->sym_vals_valid = false;
  return GG_OK;
}

int refresh_sym_values(gg_hmat *h) {
  GG_TRY(build_sym(h));
  if (h->sym_vals_valid) return GG_OK;
  cudaStream_t s = h->ctx->stream;
  GG_TRY(h->dSymVal.alloc(h->sym_nnz));
  GG_TRY(h->dSymHi.alloc(h->sym_nnz));
  GG_TRY(h->dSymLo.alloc(h->sym_nnz));
  k_symvals<<<(h->ncf * 32 + 255) / 256, 256, 0, s>>>(h->dSymPtr.p, h->dSymCol.p, h->dSymSrc.p, h->dEmt.p, h->ncf,
                                                      h->dSymVal.p, h->dSymHi.p, h->dSymLo.p); ::gg::note_launch();
  GG_CUDA(cudaGetLastError());
  h->sym_vals_valid = true;
  return GG_OK;
}

// y[:, v] = H x[:, v] for v < m (column-major [ncf x m]); stream-ordered.
// SPLIT with 2 to 16 vectors: one sweep over the matrix for all of them.
int spmv(gg_hmat *h, int precision, const double *dx, double *dy, int m, cudaStream_t s) {
  GG_TRY(check_precision(h, precision));
  const int n = h->ncf;
  const unsigned blocks = (unsigned)(((int64_t)n * 32 + 255) / 256);
  if (precision == GG_SPLIT && m >= 2 && m <= 16) return spmm_cols(h, dx, dy, n, m, s);
  for (int v = 0; v < m; ++v) {
    const double *x = dx + (size_t)v * n;
    double *y = dy + (size_t)v * n;
    if (precision == GG_SPLIT) {
      GG_TRY(h->dXs.alloc(n));
      k_split_x<<<(n + 255) / 256, 256, 0, s>>>(x, h->dXs.p, n); ::gg::note_launch();
      int v = 0;
      GG_TRY(tune_variant(h, 1, 1, s, &v));
      GG_TRY(launch_spmv(h, v, h->dXs.p, x, y, nullptr, nullptr, 0, nullptr, nullptr, false, s));
    } else {
      k_spmv64<<<blocks, 256, 0, s>>>(h->dSymPtr.p, h->dSymCol.p, h->dSymVal.p, x, y, n); ::gg::note_launch();
    }
    GG_CUDA(cudaGetLastError());
  }
  return GG_OK;
}

// Algorithmic bytes of one y = H x in the reference's storage (lower
// triangle once): nnz_l (8 + 4) + (ncf + 1) 8 + 3 ncf 8 m for FP64 (hi+lo is
// the same byte count).
// the block form of spmv_col (SPLIT only): m new columns from kpass = *dcol
int spmm_block(gg_hmat *h, int m, const float2 *xb, const double *Bbase, double *ABbase, int64_t ld,
               const int *dcol, cudaStream_t s) {
  if (m < 1 || m > 16) return fail(GG_ERR_ARG, "spmm_block: 1 to 16 columns");
  GG_TRY(check_precision(h, GG_SPLIT));
  int v = 0;
  GG_TRY(tune_variant(h, 0, m, s, &v));
  return launch_spmm(h, m, v, xb, Bbase, ABbase, ld, dcol, s);
}

// Y = H X for m columns (2 to 16) of leading dimension ld, SPLIT: the split
// copies go to h->dXb, then one block sweep
int spmm_cols(gg_hmat *h, const double *X, double *Y, int64_t ld, int m, cudaStream_t s) {
  const int n = h->ncf, mp = spmm_pitch(m);
  GG_TRY(h->dXb.alloc((size_t)n * mp));
  k_split_block<<<(unsigned)std::min<int64_t>(((int64_t)n * mp + 255) / 256, 4096), 256, 0, s>>>(X, ld, m, mp, n,
                                                                                                 h->dXb.p);
  ::gg::note_launch();
  return spmm_block(h, m, h->dXb.p, X, Y, ld, nullptr, s);
}

// tunes, before any capture, the kernels a solve over this matrix launches
int tune_prepare(gg_hmat *h, int precision, int mblock) {
  if (precision != GG_SPLIT) return GG_OK;
  int v = 0;
  if (mblock > 1) return tune_variant(h, 0, std::min(mblock, 16), h->ctx->stream, &v);
  return tune_variant(h, 1, 1, h->ctx->stream, &v);
}

double spmv_bytes(const gg_hmat *h, int precision, int m) {
  (void)precision;
  return (double)h->nnz * 12.0 + (double)(h->ncf + 1) * 8.0 + 3.0 * h->ncf * 8.0 * m;
}

}  // namespace gg

using namespace gg;

extern "C" int gg_spmm_timing(gg_ctx *ctx, gg_hmat *h, int m, int iters, double *ms_per_launch,
                              double *alg_bytes) {
  if (!ctx || !h || h->ctx != ctx || iters < 1 || m < 1 || m > 16 || !ms_per_launch)
    return fail(GG_ERR_ARG, "gg_spmm_timing: bad args");
  if (!h->emt_valid) return fail(GG_ERR_STATE, "gg_spmm_timing: EMT not set");
  GG_CUDA(cudaSetDevice(ctx->device));
  GG_TRY(refresh_sym_values(h));
  const int n = h->ncf, mp = spmm_pitch(m);
  DBuf<double> x, y;
  DBuf<float2> xb;
  GG_TRY(x.alloc((size_t)n * m));
  GG_TRY(y.alloc((size_t)n * m));
  GG_TRY(xb.alloc((size_t)n * mp));
  std::vector<double> hx((size_t)n * m);
  for (size_t i = 0; i < hx.size(); ++i) hx[i] = 1.0 / (1.0 + (double)(i % 97));
  GG_CUDA(cudaMemcpyAsync(x.p, hx.data(), hx.size() * 8, cudaMemcpyHostToDevice, ctx->stream));
  k_split_block<<<(unsigned)std::min<int64_t>(((int64_t)n * mp + 255) / 256, 4096), 256, 0, ctx->stream>>>(
      x.p, n, m, mp, n, xb.p);
  ::gg::note_launch();
  GG_TRY(spmm_block(h, m, xb.p, x.p, y.p, n, nullptr, ctx->stream));  // warm-up
  GG_TRY(timer_start(ctx));
  for (int it = 0; it < iters; ++it) GG_TRY(spmm_block(h, m, xb.p, x.p, y.p, n, nullptr, ctx->stream));
  double ms = 0;
  GG_TRY(timer_stop(ctx, &ms));
  *ms_per_launch = ms / iters;
  if (alg_bytes) *alg_bytes = spmv_bytes(h, GG_SPLIT, m);
  return GG_OK;
}

extern "C" int gg_matvec_timing(gg_ctx *ctx, gg_hmat *h, int precision, int iters, double *ms_per_launch,
                                double *alg_bytes) {
  if (!ctx || !h || h->ctx != ctx || iters < 1 || !ms_per_launch) return fail(GG_ERR_ARG, "gg_matvec_timing: bad args");
  if (!h->emt_valid) return fail(GG_ERR_STATE, "gg_matvec_timing: EMT not set");
  GG_CUDA(cudaSetDevice(ctx->device));
  GG_TRY(refresh_sym_values(h));
  DBuf<double> x, y;
  const int n = h->ncf;
  GG_TRY(x.alloc(n));
  GG_TRY(y.alloc(n));
  std::vector<double> hx(n);
  for (int i = 0; i < n; ++i) hx[i] = 1.0 / (1.0 + (i % 97));
  GG_CUDA(cudaMemcpyAsync(x.p, hx.data(), n * 8, cudaMemcpyHostToDevice, ctx->stream));
  GG_TRY(spmv(h, precision, x.p, y.p, 1, ctx->stream));  // warm-up
  GG_TRY(timer_start(ctx));
  for (int it = 0; it < iters; ++it) GG_TRY(spmv(h, precision, x.p, y.p, 1, ctx->stream));
  double ms = 0;
  GG_TRY(timer_stop(ctx, &ms));
  *ms_per_launch = ms / iters;
  if (alg_bytes) *alg_bytes = spmv_bytes(h, precision, 1);
  return GG_OK;
}

extern "C" int gg_hmat_tune(gg_hmat *h, int kernel, int m, int *chosen, int *nvariants, double *ms) {
  if (!h || kernel < 0 || kernel > 1 || (kernel == 0 && (m < 1 || m > 16)))
    return fail(GG_ERR_ARG, "gg_hmat_tune: kernel 0 (m = 1..16) or 1");
  if (!h->emt_valid) return fail(GG_ERR_STATE, "gg_hmat_tune: EMT not set");
  GG_TRY(check_precision(h, GG_SPLIT));
  GG_CUDA(cudaSetDevice(h->ctx->device));
  GG_TRY(refresh_sym_values(h));
  int v = 0;
  const int fm = kernel == 0 ? m : 1;
  const int forced = h->tune_force[kernel][fm];
  h->tune_force[kernel][fm] = -1;
  const int st = tune_variant(h, kernel, m, h->ctx->stream, &v);
  h->tune_force[kernel][fm] = forced;
  GG_TRY(st);
  if (chosen) *chosen = forced >= 0 ? forced : v;
  if (nvariants) *nvariants = TUNE_NVAR[kernel];
  if (ms) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    const TuneEntry &t = g_tune[tune_key(h, kernel, m)];
    for (int i = 0; i < TUNE_NVAR[kernel]; ++i) ms[i] = t.ms[i];
  }
  return GG_OK;
}

extern "C" int gg_hmat_tune_force(gg_hmat *h, int kernel, int m, int variant) {
  if (!h || kernel < 0 || kernel > 1 || (kernel == 0 && (m < 1 || m > 16)) || variant < -1 ||
      variant >= TUNE_NVAR[kernel])
    return fail(GG_ERR_ARG, "gg_hmat_tune_force: bad kernel, m or variant");
  h->tune_force[kernel][kernel == 0 ? m : 1] = variant;
  return GG_OK;
}

extern "C" const char *gg_tune_variant_name(int kernel, int variant) {
  static const char *k0[9] = {"U2 T128", "U2 T256", "U2 T512", "U4 T128", "U4 T256",
                              "U4 T512", "U8 T128", "U8 T256", "U8 T512"};
  static const char *k1[6] = {"L32 U2", "L32 U4", "L32 U8", "L16 U2", "L16 U4", "L16 U8"};
  static const char *k2[6] = {"R64 T128", "R64 T256", "R128 T128", "R128 T256", "R256 T128", "R256 T256"};
  if (kernel == 0 && variant >= 0 && variant < 9) return k0[variant];
  if (kernel == 1 && variant >= 0 && variant < 6) return k1[variant];
  if (kernel == 2 && variant >= 0 && variant < 6) return k2[variant];
  return "";
}

extern "C" int gg_spicmv2(gg_ctx *ctx, gg_hmat *h, int m, const double *b, double *c, int precision) {
  if (!ctx || !h || h->ctx != ctx || m < 1 || !b || !c) return fail(GG_ERR_ARG, "gg_spicmv2: bad arguments");
  if (!h->emt_valid) return fail(GG_ERR_STATE, "gg_spicmv2: EMT not set");
  GG_CUDA(cudaSetDevice(ctx->device));
  GG_TRY(refresh_sym_values(h));
  DBuf<double> db, dc;
  const size_t n = (size_t)h->ncf * m;
  GG_TRY(db.alloc(n));
  GG_TRY(dc.alloc(n));
  GG_CUDA(cudaMemcpyAsync(db.p, b, n * 8, cudaMemcpyHostToDevice, ctx->stream));
  GG_TRY(spmv(h, precision, db.p, dc.p, m, ctx->stream));
  GG_CUDA(cudaMemcpyAsync(c, dc.p, n * 8, cudaMemcpyDeviceToHost, ctx->stream));
  GG_CUDA(cudaStreamSynchronize(ctx->stream));
  return GG_OK;
}
