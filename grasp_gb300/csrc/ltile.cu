// ltile.cu - y = H x from the lower triangle read once (hi+lo split values).
//
// The reference's matvec (SPICMV2, lib9290/spicmv2.f90:2-60) walks the
// lower triangle by rows and adds each stored entry twice: a_ij x_j into
// y_i (gather) and a_ij x_i into y_j (scatter). A GPU matvec over a full
// symmetric copy reads every value twice; this one reads each stored value
// once and stays deterministic (no atomics on values):
//
//  - the strict lower triangle is cut into TW x TW tiles (I, J), J <= I;
//  - each tile's rows are grouped into chunks of at most CH entries, stored
//    contiguously: hi[n], lo[n] (FP32), col[n] (u16, column within the
//    tile), perm[n] (u16, the chunk's entries in column order), rowptr
//    (u16), runs (u32: column | first position in perm << 16);
//  - one CTA takes an item (consecutive chunks of one tile), stages each
//    chunk in shared memory with cp.async (double-buffered), and from there
//    (a) sums each row's products with x_J (one warp per row, double-float)
//    into Pg[J][row], and (b) sums each column's products with x_I (one
//    thread per column run, double-float) into its shared y_J, chunk after
//    chunk, written to Ps[item] at the end;
//  - a finishing kernel adds, per row, the FP64 diagonal term, Pg over J in
//    order and Ps over the items of its column tile in order.
//
// HBM bytes per stored entry: 8 (hi+lo) + 2 (col) + 2 (perm) + ~1.3
// (rowptr, runs), against 24 for the full symmetric copy.
#include <algorithm>
#include <cstring>
#include <vector>

#include "gg_internal.cuh"

namespace gg {
namespace {

constexpr int TW = LT_TW;       // tile width (rows and columns)
constexpr int CH = 2048;        // entries per chunk, at most
constexpr int NT = 512;         // threads of the main kernel (two CTAs per SM)
constexpr int ITEM_MIN = 16384; // entries per item, at least (when the tile has them)
constexpr int LONG_RUN = 8;     // column runs longer than this get a warp in the column phase

struct LtChunk {
  long long off;  // byte offset of the chunk in the blob
  int row0;       // first row (0-based)
  int nrows;      // rows covered (some may have no entry in this tile)
  int nent;       // entries
  int nruns;      // columns with entries (written by k_lt_csc)
  int nlong;      // of them, runs longer than LONG_RUN (written by k_lt_csc)
  int tj;
};
struct LtItem {
  int c0, nc;     // chunks [c0, c0 + nc)
  int ti, tj;     // tile (I, J)
  int row0, row1; // rows [row0, row1)
};

__host__ __device__ inline long long a16(long long b) { return (b + 15) & ~15ll; }
// blob layout of a chunk with n entries and r rows (runs sized for the maximum)
struct ChunkLayout {
  long long hi, lo, col, perm, rowptr, runs, size;
};
__host__ __device__ inline ChunkLayout layout(int n, int r) {
  ChunkLayout L;
  L.hi = 0;
  L.lo = L.hi + a16(4ll * n);
  L.col = L.lo + a16(4ll * n);
  L.perm = L.col + a16(2ll * n);
  L.rowptr = L.perm + a16(2ll * n);
  L.runs = L.rowptr + a16(2ll * (r + 1));
  const int maxruns = n < TW ? n : TW;
  L.size = L.runs + a16(4ll * maxruns) + a16(2ll * maxruns);  // runs, then the long-run list
  return L;
}
// bytes of a chunk in use: up to the long-run list after its nruns runs
__host__ __device__ inline long long used_bytes(int n, int r, int nruns, int nlong) {
  return layout(n, r).runs + a16(4ll * nruns) + a16(2ll * nlong);
}
__host__ __device__ inline long long lruns_off(int n, int r, int nruns) { return layout(n, r).runs + a16(4ll * nruns); }
constexpr long long MAXCHUNK =
    4ll * CH + 4ll * CH + 2ll * CH + 2ll * CH + 2ll * (TW + 1) + 16 + 4ll * TW + 16 + 2ll * TW + 16;

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
// (ah + al)(xh + xl) as an unnormalised pair
__device__ __forceinline__ df df_mul(float ah, float al, float2 x) {
  const float ph = ah * x.x;
  const float pe = fmaf(ah, x.x, -ph);
  return two_sum(ph, fmaf(ah, x.y, fmaf(al, x.x, pe)));
}

// ---- structure build --------------------------------------------------------

// per row: entries in each column tile (strict lower part), and whether the
// row's columns ascend (the layout needs it)
__global__ void k_lt_count(const int64_t *__restrict__ iendc, const int32_t *__restrict__ irow, int n, int nj,
                           int *__restrict__ cnt, int *__restrict__ bad) {
  const int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (r >= n) return;
  const int64_t p0 = iendc[r], p1 = iendc[r + 1] - 1;  // last entry is the diagonal
  for (int64_t p = p0 + lane; p < p1; p += 32) {
    const int c = irow[p] - 1;
    if (c >= r || c < 0 || (p > p0 && irow[p - 1] >= irow[p])) atomicOr(bad, 1);
    if (c >= 0 && c < r) atomicAdd(&cnt[(size_t)r * nj + c / TW], 1);
  }
}

// entries into their chunks: column within the tile and EMT source index
__global__ void k_lt_place(const int64_t *__restrict__ iendc, const int32_t *__restrict__ irow, int n, int nj,
                           const int *__restrict__ segstart, const int2 *__restrict__ ent,
                           const LtChunk *__restrict__ ch, const long long *__restrict__ slot0,
                           unsigned char *__restrict__ blob, int64_t *__restrict__ src) {
  const int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (r >= n) return;
  const int64_t p0 = iendc[r], p1 = iendc[r + 1] - 1;
  for (int64_t p = p0 + lane; p < p1; p += 32) {
    const int c = irow[p] - 1;
    const int j = c / TW;
    const int2 e = ent[(size_t)r * nj + j];  // (chunk, position of the row's first entry of tile j)
    const int pos = e.y + (int)(p - p0) - segstart[(size_t)r * nj + j];
    const LtChunk k = ch[e.x];
    const ChunkLayout L = layout(k.nent, k.nrows);
    reinterpret_cast<unsigned short *>(blob + k.off + L.col)[pos] = (unsigned short)(c - j * TW);
    src[slot0[e.x] + pos] = p;
  }
}

// row pointers of each chunk
__global__ void k_lt_rowptr(const LtChunk *__restrict__ ch, const int2 *__restrict__ ent, int nj,
                            unsigned char *__restrict__ blob) {
  const LtChunk k = ch[blockIdx.x];
  const ChunkLayout L = layout(k.nent, k.nrows);
  unsigned short *rp = reinterpret_cast<unsigned short *>(blob + k.off + L.rowptr);
  for (int lr = threadIdx.x; lr < k.nrows; lr += blockDim.x) rp[lr] = (unsigned short)ent[(size_t)(k.row0 + lr) * nj + k.tj].y;
  if (threadIdx.x == 0) rp[k.nrows] = (unsigned short)k.nent;
}

// per chunk: column runs and the column-ordered permutation (stable: rows in
// order, so every column's entries keep their row order)
// launched with TW / 2 threads: two columns (or runs) per thread in the scans
__global__ void __launch_bounds__(TW / 2) k_lt_csc(LtChunk *__restrict__ ch, unsigned char *__restrict__ blob) {
  __shared__ int cntc[TW];
  __shared__ int start[TW];
  __shared__ int wsum[32];
  __shared__ int nruns_s;
  LtChunk &k = ch[blockIdx.x];
  const ChunkLayout L = layout(k.nent, k.nrows);
  const unsigned short *col = reinterpret_cast<const unsigned short *>(blob + k.off + L.col);
  const unsigned short *rp = reinterpret_cast<const unsigned short *>(blob + k.off + L.rowptr);
  unsigned short *perm = reinterpret_cast<unsigned short *>(blob + k.off + L.perm);
  unsigned *runs = reinterpret_cast<unsigned *>(blob + k.off + L.runs);
  for (int c = threadIdx.x; c < TW; c += blockDim.x) cntc[c] = 0;
  if (threadIdx.x < 32) wsum[threadIdx.x] = 0;
  __syncthreads();
  for (int e = threadIdx.x; e < k.nent; e += blockDim.x) atomicAdd(&cntc[col[e]], 1);
  __syncthreads();
  // exclusive scan of the counts (two per thread) and of the non-empty flags
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  const int c0 = 2 * t, c1 = 2 * t + 1;
  const int v0 = cntc[c0], v1 = cntc[c1];
  int s = v0 + v1, f = (v0 > 0) + (v1 > 0);
  // warp inclusive scans of s and f packed into one 32-bit pair of 16-bit halves
  int pk = (s << 16) | f;
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, pk, o);
    if (lane >= o) pk += y;
  }
  if (lane == 31) wsum[w] = pk;
  __syncthreads();
  if (w == 0) {
    int x = wsum[lane];
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    wsum[lane] = x;
  }
  __syncthreads();
  const int before = pk - ((s << 16) | f) + (w > 0 ? wsum[w - 1] : 0);
  const int sb = before >> 16, fb = before & 0xffff;
  start[c0] = sb;
  start[c1] = sb + v0;
  if (v0 > 0) runs[fb] = (unsigned)c0 | ((unsigned)sb << 16);
  if (v1 > 0) runs[fb + (v0 > 0)] = (unsigned)c1 | ((unsigned)(sb + v0) << 16);
  if (t == blockDim.x - 1) nruns_s = (before + ((s << 16) | f)) & 0xffff;
  __syncthreads();
  // stable placement, row after row (a row's columns are distinct)
  for (int lr = 0; lr < k.nrows; ++lr) {
    const int e0 = rp[lr], e1 = rp[lr + 1];
    for (int e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
      const int c = col[e];
      perm[start[c]++] = (unsigned short)e;
    }
    __syncthreads();
  }
  // long runs (more than LONG_RUN entries), in run order
  const int nr = nruns_s;
  const int q0 = 2 * t, q1 = 2 * t + 1;
  auto runlen = [&](int q) {
    const int a = (int)(runs[q] >> 16);
    const int b = (q + 1 < nr) ? (int)(runs[q + 1] >> 16) : k.nent;
    return b - a;
  };
  const int l0 = (q0 < nr && runlen(q0) > LONG_RUN), l1 = (q1 < nr && runlen(q1) > LONG_RUN);
  int x = l0 + l1;
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  __syncthreads();
  if (threadIdx.x < 32) wsum[threadIdx.x] = 0;
  __syncthreads();
  if (lane == 31) wsum[w] = x;
  __syncthreads();
  if (w == 0) {
    int z = wsum[lane];
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, z, o);
      if (lane >= o) z += y;
    }
    wsum[lane] = z;
  }
  __syncthreads();
  const int lb = x - (l0 + l1) + (w > 0 ? wsum[w - 1] : 0);
  unsigned short *lruns = reinterpret_cast<unsigned short *>(blob + k.off + lruns_off(k.nent, k.nrows, nr));
  if (l0) lruns[lb] = (unsigned short)q0;
  if (l1) lruns[lb + l0] = (unsigned short)q1;
  if (threadIdx.x == 0) {
    k.nruns = nr;
    k.nlong = wsum[31];
  }
}

// values: hi/lo split of EMT at each chunk's entries
__global__ void k_lt_vals(const LtChunk *__restrict__ ch, const long long *__restrict__ slot0,
                          const int64_t *__restrict__ src, const double *__restrict__ emt,
                          unsigned char *__restrict__ blob) {
  const LtChunk k = ch[blockIdx.x];
  const ChunkLayout L = layout(k.nent, k.nrows);
  float *hi = reinterpret_cast<float *>(blob + k.off + L.hi);
  float *lo = reinterpret_cast<float *>(blob + k.off + L.lo);
  const int64_t *sp = src + slot0[blockIdx.x];
  for (int e = threadIdx.x; e < k.nent; e += blockDim.x) {
    const double v = emt[sp[e]];
    const float h = __double2float_rn(v);
    hi[e] = h;
    lo[e] = __double2float_rn(v - (double)h);
  }
}

// ---- the matvec ---------------------------------------------------------------

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;\n" ::); }
__device__ __forceinline__ void cp_async_wait0() { asm volatile("cp.async.wait_group 0;\n" ::); }

__device__ __forceinline__ void stage_chunk(unsigned char *dst, const unsigned char *blob, const LtChunk &k) {
  const long long bytes = used_bytes(k.nent, k.nrows, k.nruns, k.nlong);
  const unsigned char *s = blob + k.off;
  for (long long b = (long long)threadIdx.x * 16; b < bytes; b += (long long)NT * 16) cp_async16(dst + b, s + b);
  cp_async_commit();
}

// one CTA per item; dynamic shared memory: x_J, x_I (float2), y_J (h, l),
// rowOf (u16), two chunk buffers
__global__ void __launch_bounds__(NT, 2) k_lt_spmv(const LtItem *__restrict__ items, const LtChunk *__restrict__ ch,
                                                const unsigned char *__restrict__ blob, const float2 *__restrict__ xs,
                                                int n, double *__restrict__ pg, double *__restrict__ ps,
                                                const double *skip) {
  if (skip && *skip != 0.0) return;
  extern __shared__ __align__(16) unsigned char sm[];
  float2 *xj = reinterpret_cast<float2 *>(sm);
  float2 *xi = xj + TW;
  float *yh = reinterpret_cast<float *>(xi + TW);
  float *yl = yh + TW;
  unsigned short *rowof = reinterpret_cast<unsigned short *>(yl + TW);
  unsigned char *buf0 = reinterpret_cast<unsigned char *>(rowof + CH);
  unsigned char *buf1 = buf0 + a16(MAXCHUNK);
  const LtItem it = items[blockIdx.x];
  const int c_lo = it.tj * TW;
  stage_chunk(buf0, blob, ch[it.c0]);
  for (int q = threadIdx.x; q < TW; q += NT) {
    const int c = c_lo + q;
    xj[q] = (c < n) ? xs[c] : make_float2(0.f, 0.f);
    const int r = it.row0 + q;
    xi[q] = (r < it.row1) ? xs[r] : make_float2(0.f, 0.f);
    yh[q] = 0.f;
    yl[q] = 0.f;
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int kc = 0; kc < it.nc; ++kc) {
    const LtChunk k = ch[it.c0 + kc];
    unsigned char *cur = (kc & 1) ? buf1 : buf0;
    if (kc + 1 < it.nc) {
      stage_chunk((kc & 1) ? buf0 : buf1, blob, ch[it.c0 + kc + 1]);
      cp_async_wait1();
    } else {
      cp_async_wait0();
    }
    __syncthreads();
    const ChunkLayout L = layout(k.nent, k.nrows);
    const float *hi = reinterpret_cast<const float *>(cur + L.hi);
    const float *lo = reinterpret_cast<const float *>(cur + L.lo);
    const unsigned short *col = reinterpret_cast<const unsigned short *>(cur + L.col);
    const unsigned short *perm = reinterpret_cast<const unsigned short *>(cur + L.perm);
    const unsigned short *rp = reinterpret_cast<const unsigned short *>(cur + L.rowptr);
    const unsigned *runs = reinterpret_cast<const unsigned *>(cur + L.runs);
    // (a) rows: y_i += sum_j a_ij x_j; four lanes per row (tile rows are
    // short), rows advanced warp-uniformly so that the shuffles see all lanes
    const int sub = lane & 3;
    for (int base = wid * 8; base < k.nrows; base += NT / 4) {
      const int lr = base + (lane >> 2);
      df acc = {0.f, 0.f};
      if (lr < k.nrows) {
        const int e0 = rp[lr], e1 = rp[lr + 1];
        for (int e = e0 + sub; e < e1; e += 4) {
          acc = df_add(acc, df_mul(hi[e], lo[e], xj[col[e]]));
          rowof[e] = (unsigned short)lr;
        }
      }
#pragma unroll
      for (int o = 1; o < 4; o <<= 1) {
        df other;
        other.h = __shfl_xor_sync(0xffffffffu, acc.h, o);
        other.l = __shfl_xor_sync(0xffffffffu, acc.l, o);
        acc = df_add(acc, other);
      }
      if (sub == 0 && lr < k.nrows) pg[(size_t)it.tj * n + k.row0 + lr] = (double)acc.h + (double)acc.l;
    }
    __syncthreads();
    // (b) columns: y_j += sum_i a_ij x_i. Short column runs: one thread
    // each; long ones (listed after the runs): one warp each, lanes striding
    // the run, then a shuffle reduction. A column has one owner per chunk,
    // so its sum has a fixed order.
    const int xoff = k.row0 - it.row0;
    for (int q = threadIdx.x; q < k.nruns; q += NT) {
      const unsigned rq = runs[q];
      const int c = rq & 0xffff, t0 = rq >> 16, t1 = (q + 1 < k.nruns) ? (runs[q + 1] >> 16) : k.nent;
      if (t1 - t0 > LONG_RUN) continue;
      df acc = {0.f, 0.f};
      for (int t = t0; t < t1; ++t) {
        const int e = perm[t];
        acc = df_add(acc, df_mul(hi[e], lo[e], xi[xoff + rowof[e]]));
      }
      const df y = df_add({yh[c], yl[c]}, acc);
      yh[c] = y.h;
      yl[c] = y.l;
    }
    const unsigned short *lruns = reinterpret_cast<const unsigned short *>(cur + lruns_off(k.nent, k.nrows, k.nruns));
    for (int i = wid; i < k.nlong; i += NT / 32) {
      const int q = lruns[i];
      const unsigned rq = runs[q];
      const int c = rq & 0xffff, t0 = rq >> 16, t1 = (q + 1 < k.nruns) ? (runs[q + 1] >> 16) : k.nent;
      df acc = {0.f, 0.f};
      for (int t = t0 + lane; t < t1; t += 32) {
        const int e = perm[t];
        acc = df_add(acc, df_mul(hi[e], lo[e], xi[xoff + rowof[e]]));
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        df other;
        other.h = __shfl_xor_sync(0xffffffffu, acc.h, o);
        other.l = __shfl_xor_sync(0xffffffffu, acc.l, o);
        acc = df_add(acc, other);
      }
      if (lane == 0) {
        const df y = df_add({yh[c], yl[c]}, acc);
        yh[c] = y.h;
        yl[c] = y.l;
      }
    }
    __syncthreads();
  }
  double *out = ps + (size_t)blockIdx.x * TW;
  for (int q = threadIdx.x; q < TW; q += NT) out[q] = (double)yh[q] + (double)yl[q];
}

// y_i = diag_i x_i + sum_{J <= I} Pg[J][i] + sum_{items m of column tile I} Ps[m][i - I TW]
// with x, y = column c of Xbase, Ybase (c = *dcol, or 0)
__global__ void k_lt_finish(int n, const double *__restrict__ diag, const double *__restrict__ Xbase,
                            double *__restrict__ Ybase, int64_t ld, const int *__restrict__ dcol,
                            const double *__restrict__ pg, const double *__restrict__ ps,
                            const int *__restrict__ jptr, const int *__restrict__ jlist, const double *skip) {
  if (skip && *skip != 0.0) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const size_t off = dcol ? (size_t)(*dcol) * ld : 0;
  const int I = i / TW;
  double acc = diag[i] * Xbase[off + i];
  for (int J = 0; J <= I; ++J) acc += pg[(size_t)J * n + i];
  for (int q = jptr[I]; q < jptr[I + 1]; ++q) acc += ps[(size_t)jlist[q] * TW + (i - I * TW)];
  Ybase[off + i] = acc;
}

}  // namespace

// Builds the tiled layout from the structure (once per matrix); leaves
// lt.usable false when the rows' columns do not ascend.
int build_ltile(gg_hmat *h) {
  LTile &T = h->lt;
  if (T.built) return GG_OK;
  T.built = true;
  T.usable = false;
  gg_ctx *ctx = h->ctx;
  cudaStream_t s = ctx->stream;
  const int n = h->ncf;
  const int nj = (n + TW - 1) / TW;
  DBuf<int> cnt, bad;
  GG_TRY(cnt.alloc((size_t)n * nj));
  GG_TRY(bad.alloc(1));
  GG_CUDA(cudaMemsetAsync(cnt.p, 0, (size_t)n * nj * sizeof(int), s));
  GG_CUDA(cudaMemsetAsync(bad.p, 0, sizeof(int), s));
  k_lt_count<<<(unsigned)(((int64_t)n * 32 + 255) / 256), 256, 0, s>>>(h->dIendc.p, h->dIrow.p, n, nj, cnt.p, bad.p);
  note_launch();
  GG_CUDA(cudaGetLastError());
  std::vector<int> hc((size_t)n * nj);
  int hbad = 0;
  GG_CUDA(cudaMemcpyAsync(hc.data(), cnt.p, hc.size() * sizeof(int), cudaMemcpyDeviceToHost, s));
  GG_CUDA(cudaMemcpyAsync(&hbad, bad.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  GG_CUDA(cudaStreamSynchronize(s));
  if (hbad) return GG_OK;  // columns not ascending within rows: keep the full symmetric matvec
  // per (row, tile): offset of the row's tile-j segment within the row
  std::vector<int> seg((size_t)n * nj);
  for (int r = 0; r < n; ++r) {
    int a = 0;
    for (int j = 0; j < nj; ++j) {
      seg[(size_t)r * nj + j] = a;
      a += hc[(size_t)r * nj + j];
    }
  }
  // chunks and items, tile by tile
  int64_t total = 0;
  for (int x : hc) total += x;
  const int sms = std::max(1, ctx->sms);
  const int64_t item_target = std::max<int64_t>(ITEM_MIN, total / (2 * sms) + 1);
  std::vector<LtChunk> chunks;
  std::vector<LtItem> items;
  std::vector<long long> slot0;
  std::vector<int2> ent((size_t)n * nj, make_int2(-1, 0));
  long long off = 0, slots = 0;
  for (int I = 0; I < nj; ++I) {
    const int r0 = I * TW, r1 = std::min(n, r0 + TW);
    for (int J = 0; J <= I; ++J) {
      int64_t tile_n = 0;
      for (int r = r0; r < r1; ++r) tile_n += hc[(size_t)r * nj + J];
      if (tile_n == 0) continue;
      int r = r0;
      LtItem cur{(int)chunks.size(), 0, I, J, r0, r0};
      int64_t cur_n = 0;
      while (r < r1) {
        LtChunk k{};
        k.row0 = r;
        k.tj = J;
        int cn = 0;
        while (r < r1 && cn + hc[(size_t)r * nj + J] <= CH) {
          ent[(size_t)r * nj + J] = make_int2((int)chunks.size(), cn);
          cn += hc[(size_t)r * nj + J];
          ++r;
        }
        k.nrows = r - k.row0;
        k.nent = cn;
        k.off = off;
        off += layout(cn, k.nrows).size;
        slot0.push_back(slots);
        slots += cn;
        if (cur.nc > 0 && cur_n + cn > item_target) {
          items.push_back(cur);
          cur = LtItem{(int)chunks.size(), 0, I, J, k.row0, k.row0};
          cur_n = 0;
        }
        chunks.push_back(k);
        cur.nc += 1;
        cur.row1 = r;
        cur_n += cn;
      }
      items.push_back(cur);
    }
  }
  // items per column tile, in item order
  std::vector<int> jptr(nj + 1, 0), jlist(items.size());
  for (const LtItem &it : items) jptr[it.tj + 1]++;
  for (int j = 0; j < nj; ++j) jptr[j + 1] += jptr[j];
  {
    std::vector<int> fill(jptr.begin(), jptr.end() - 1);
    for (size_t m = 0; m < items.size(); ++m) jlist[fill[items[m].tj]++] = (int)m;
  }
  T.nj = nj;
  T.nchunks = (int)chunks.size();
  T.nitems = (int)items.size();
  T.nslots = slots;
  GG_TRY(T.blob.alloc((size_t)std::max<long long>(off, 16)));
  GG_TRY(T.chunks.alloc(sizeof(LtChunk) * std::max<size_t>(1, chunks.size())));
  GG_TRY(T.items.alloc(sizeof(LtItem) * std::max<size_t>(1, items.size())));
  GG_TRY(T.slot0.alloc(std::max<size_t>(1, slot0.size())));
  GG_TRY(T.src.alloc(std::max<long long>(1, slots)));
  GG_TRY(T.jptr.alloc(nj + 1));
  GG_TRY(T.jlist.alloc(std::max<size_t>(1, jlist.size())));
  GG_TRY(T.pg.alloc((size_t)nj * n));
  GG_TRY(T.ps.alloc((size_t)std::max(1, T.nitems) * TW));
  DBuf<int> dseg;
  DBuf<int2> dent;
  GG_TRY(dseg.alloc(seg.size()));
  GG_TRY(dent.alloc(ent.size()));
  GG_CUDA(cudaMemsetAsync(T.blob.p, 0, T.blob.n, s));
  GG_CUDA(cudaMemsetAsync(T.pg.p, 0, (size_t)nj * n * sizeof(double), s));
  GG_CUDA(cudaMemcpyAsync(T.chunks.p, chunks.data(), sizeof(LtChunk) * chunks.size(), cudaMemcpyHostToDevice, s));
  GG_CUDA(cudaMemcpyAsync(T.items.p, items.data(), sizeof(LtItem) * items.size(), cudaMemcpyHostToDevice, s));
  GG_CUDA(cudaMemcpyAsync(T.slot0.p, slot0.data(), sizeof(long long) * slot0.size(), cudaMemcpyHostToDevice, s));
  GG_CUDA(cudaMemcpyAsync(T.jptr.p, jptr.data(), sizeof(int) * jptr.size(), cudaMemcpyHostToDevice, s));
  GG_CUDA(cudaMemcpyAsync(T.jlist.p, jlist.data(), sizeof(int) * jlist.size(), cudaMemcpyHostToDevice, s));
  GG_CUDA(cudaMemcpyAsync(dseg.p, seg.data(), sizeof(int) * seg.size(), cudaMemcpyHostToDevice, s));
  GG_CUDA(cudaMemcpyAsync(dent.p, ent.data(), sizeof(int2) * ent.size(), cudaMemcpyHostToDevice, s));
  LtChunk *dch = reinterpret_cast<LtChunk *>(T.chunks.p);
  k_lt_place<<<(unsigned)(((int64_t)n * 32 + 255) / 256), 256, 0, s>>>(h->dIendc.p, h->dIrow.p, n, nj, dseg.p, dent.p,
                                                                      dch, T.slot0.p, T.blob.p, T.src.p);
  note_launch();
  if (T.nchunks > 0) {
    k_lt_rowptr<<<T.nchunks, 256, 0, s>>>(dch, dent.p, nj, T.blob.p);
    note_launch();
    k_lt_csc<<<T.nchunks, TW / 2, 0, s>>>(dch, T.blob.p);
    note_launch();
  }
  GG_CUDA(cudaGetLastError());
  GG_CUDA(cudaStreamSynchronize(s));
  T.smem = (size_t)(TW * 8 * 2 + TW * 4 * 2 + CH * 2) + 2 * (size_t)a16(MAXCHUNK);
  GG_CUDA(cudaFuncSetAttribute(k_lt_spmv, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)T.smem));
  T.usable = true;
  T.vals_valid = false;
  return GG_OK;
}

int refresh_ltile_values(gg_hmat *h) {
  LTile &T = h->lt;
  if (!T.usable || T.vals_valid) return GG_OK;
  if (T.nchunks > 0) {
    k_lt_vals<<<T.nchunks, 256, 0, h->ctx->stream>>>(reinterpret_cast<const LtChunk *>(T.chunks.p), T.slot0.p,
                                                      T.src.p, h->dEmt.p, T.blob.p);
    note_launch();
    GG_CUDA(cudaGetLastError());
  }
  T.vals_valid = true;
  return GG_OK;
}

// y = H x for the split precision from the tiled layout: xs is the hi+lo
// copy of x; x and y are column c of Xbase / Ybase (c = *dcol, or 0)
int spmv_ltile(gg_hmat *h, const float2 *xs, const double *Xbase, double *Ybase, int64_t ld, const int *dcol,
               const double *skip, cudaStream_t s) {
  LTile &T = h->lt;
  const int n = h->ncf;
  if (T.nitems > 0) {
    k_lt_spmv<<<T.nitems, NT, T.smem, s>>>(reinterpret_cast<const LtItem *>(T.items.p),
                                           reinterpret_cast<const LtChunk *>(T.chunks.p), T.blob.p, xs, n, T.pg.p,
                                           T.ps.p, skip);
    note_launch();
  }
  k_lt_finish<<<(n + 255) / 256, 256, 0, s>>>(n, h->dDiag.p, Xbase, Ybase, ld, dcol, T.pg.p, T.ps.p, T.jptr.p,
                                              T.jlist.p, skip);
  note_launch();
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

// bytes the tiled matvec reads and writes per launch (for reporting)
double ltile_bytes(const gg_hmat *h) {
  const LTile &T = h->lt;
  return (double)T.blob.n + (double)T.nj * h->ncf * 8.0 * 2 + (double)T.nitems * TW * 8.0 * 2 + h->ncf * 8.0 * 4;
}

}  // namespace gg
