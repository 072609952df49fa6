// radial.cu - R^k table (GENINTRK/SLATER/YZK/QUAD) and one-body I(ab)
// (RINTI/DPBDT) on the GPU.
//
// Compiled with -fmad=false: every multiply and add below is rounded on its
// own, as in the reference's FP64 loops, so that the Y^k functions and the
// per-integral quadratures reproduce the reference's arithmetic step by
// step. The R^k contraction uses explicit fma() and QUAD's head term takes
// the grid's factors per point from a table, so neither is bit-exact.
//
// Layout in HBM (all FP64):
//   Y buffer   [nY][np]  Y^k_bd(r_i) at [f*np + i] (1-based i), zero beyond
//                        the integration limit MTP(b,d) of SLATER.
//   A buffer   [nP][KC]  w(i) * (P_a P_c + Q_a Q_c)(r_i) * RPOR(r_i) for
//                        every pair a <= c, zero outside 2 <= i <= min(MF).
//   VALTEIRK   [N_Rk]    written by the contraction epilogue in GENINTRK order.
#include <cuda_fp16.h>

#include <algorithm>
#include <map>
#include <tuple>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <mutex>

#include "gg_internal.cuh"

namespace gg {

namespace {

constexpr int KC_TILE = 16;  // contraction depth per shared-memory stage
constexpr int BM = 32, BN = 64;

struct YDesc {
  int k, b, d;  // Y^k_{bd}
  int mtp;      // min(MF(b), MF(d)) (YZK's MTP)
  int mtpb;     // last point kept in the Y buffer (N when k == 0 and b == d)
  int cs;       // first function index with the same (k, b)
  int nd;       // number of functions with the same (k, b) = |D(b,k)|
};

struct RkTile {
  int k, a;
  int ncA;        // |C(a,k)|: rows of the (k,a) problem
  int r0;         // first row of this tile
  int rowpair0;   // offset into the row-pair list of the (k,a) problem
  int cs_a;       // first column (Y function) of the (k,a) problem
  int c0, c1;     // column range [c0, c1) of this tile
  long long base; // 0-based VALTEIRK position of the (k,a) problem
};

struct QuadItem {  // one integral evaluated with the general QUAD
  int a, c, f, mtp;
  long long pos;
};

__device__ __forceinline__ double pf(const double *P, int ld, int i, int j) {
  return P[(size_t)(j - 1) * ld + (i - 1)];
}

// QUAD (lib9290/quad.f90:52-103) on a 1-based array TA with room for
// TA(MTP+3). Sequential, in the reference's order.
__device__ double quad_seq(double *TA, int mtp, const double *R, const double *RP, const QuadConst &q) {
  const int mtpm1 = mtp - 1;
  for (int i = 2; i <= mtpm1; ++i) {
    const double tai = TA[i];
    if (fabs(tai) <= 0.0) continue;
    const int ip1 = i + 1;
    const double taip1 = TA[ip1];
    const double quott = taip1 / tai;
    if (quott <= 0.0) continue;
    const double frip1 = taip1 / RP[ip1];
    double fri = tai / RP[i];
    const double ratio = frip1 / fri;
    const double rip1 = R[ip1], ri = R[i];
    const double sigma = log(ratio) / log(rip1 / ri);
    fri = ri * fri;
    double result = fri / (sigma + 1.0);
    TA[mtp + 1] = 0.0;
    TA[mtp + 2] = 0.0;
    TA[mtp + 3] = 0.0;
    result = result + q.C1 * tai;
    double s = 0.0;
    for (int j = ip1; j <= mtp; j += 4) s = s + (q.C2 * (TA[j] + TA[j + 2]) + q.C3 * TA[j + 1] + q.C4 * TA[j + 3]);
    result = result + s;
    if ((mtp - i) % 4 == 0) result = result - q.C1 * TA[mtp];
    return result;
  }
  return 0.0;
}

// ---------------------------------------------------------------------------
// YZK part 1 (yzk.f90:105-126, 190-201): RHOP and the two TEMP arrays.
//   TZ(i) = r^k RHOP(i), TW(i) = RHOP(i) / r^(k+1) on 2 <= i <= MTP, else 0.
// ---------------------------------------------------------------------------
__global__ void k_ytemp(const YDesc *__restrict__ yd, int nf, const double *__restrict__ PF,
                        const double *__restrict__ QF, int ld, const double *__restrict__ RP,
                        const double *__restrict__ pw, int np, double *__restrict__ TZ, double *__restrict__ TW) {
  const int f = blockIdx.y;
  if (f >= nf) return;
  const YDesc y = yd[f];
  const double *RTTK = pw + (size_t)(0 * (KLIMIT + 1) + y.k) * np;
  const double *RTTKM1 = pw + (size_t)(3 * (KLIMIT + 1) + y.k) * np;
  const double *RM = pw;  // row k = 0 of table 0
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < np; i += gridDim.x * blockDim.x) {
    double tz = 0.0, tw = 0.0;
    if (i >= 2 && i <= y.mtp) {
      const double rhop =
          RP[i] * (pf(PF, ld, i, y.b) * pf(PF, ld, i, y.d) + pf(QF, ld, i, y.b) * pf(QF, ld, i, y.d));
      if (y.k == 0) {
        tz = rhop;
        tw = rhop * RM[i];
      } else {
        tz = RTTK[i] * rhop;
        tw = rhop * RTTKM1[i];
      }
    }
    TZ[(size_t)f * np + i] = tz;
    TW[(size_t)f * np + i] = tw;
  }
}

// ---------------------------------------------------------------------------
// YZK part 2 (yzk.f90:128-224): the four interleaved stride-4 Newton-Cotes
// recurrences for Z (forward) and W (backward). One thread per (function,
// residue class mod 4); the four threads of a function are adjacent lanes.
// ---------------------------------------------------------------------------
__global__ void k_ychain(const YDesc *__restrict__ yd, int nf, const double *__restrict__ TZ,
                         const double *__restrict__ TW, const double *__restrict__ R,
                         const double *__restrict__ pw, int np, QuadConst q, double *__restrict__ Y) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int f = t >> 2, c = t & 3;
  const bool active = f < nf;
  YDesc y = active ? yd[f] : yd[0];
  const int K = y.k, MTP = y.mtp, MTPP3 = MTP + 3, N = q.n;
  const double *T = TZ + (size_t)(active ? f : 0) * np;
  const double *Tw = TW + (size_t)(active ? f : 0) * np;
  double *Yf = Y + (size_t)(active ? f : 0) * np;
  const int s = c + 2;  // chain start: 2, 3, 4, 5
  double z = 0.0;
  if (active) {
    if (s <= 4) {
      double sum = 0.0;
      for (int kk = 2; kk <= 5; ++kk) sum = sum + q.CNC5C[kk - 2][s - 2] * T[kk];
      z = sum;
    } else {  // ZK(5) = ZK(1) + RTMP(5), ZK(1) = 0
      const double rtmp = q.C1 * (T[1] + T[5]) + q.C2 * (T[2] + T[4]) + q.C3 * T[3];
      z = 0.0 + rtmp;
    }
    Yf[s] = z;
    for (int i = s + 4; i <= MTPP3; i += 4) {
      const double rtmp = q.C1 * (T[i - 4] + T[i]) + q.C2 * (T[i - 3] + T[i - 1]) + q.C3 * T[i - 2];
      z = z + rtmp;
      Yf[i] = z;
    }
  }
  // asymptotic value (yzk.f90:150-171)
  const int owner = (MTPP3 - 2) & 3;
  const double z_top = __shfl_sync(0xffffffffu, z, (threadIdx.x & ~3) + owner);
  if (!active) return;
  double zklim, dif = 0.0;
  if (K == 0) {
    zklim = (y.b == y.d) ? 1.0 : 0.0;
    const double d0 = z - zklim;  // this chain's value at its last point (in [MTP, MTP+3])
    if (fabs(d0) > q.accy) dif = d0;
  } else {
    zklim = z_top;
  }
  const double *RTTKM = pw + (size_t)(1 * (KLIMIT + 1) + K) * np;
  const double *RTTK1 = pw + (size_t)(2 * (KLIMIT + 1) + K) * np;
  // backward pass: W recurrence on i <= MTP, assembly of Y = Z + W on 2..N
  int top = s;
  while (top + 4 < np) top += 4;
  double wk_next = 0.0;
  for (int i = top; i >= s; i -= 4) {
    if (i > N) {
      Yf[i] = 0.0;
      continue;
    }
    double zf;
    if (K == 0) {
      if (i <= MTPP3)
        zf = (dif != 0.0) ? Yf[i] - dif : Yf[i];
      else
        zf = zklim;
    } else {
      zf = (i <= MTPP3) ? Yf[i] * RTTKM[i] : zklim * RTTKM[i];
    }
    double wkf = 0.0;
    if (i <= MTP) {
      const double wk = wk_next + q.C1 * (Tw[i] + Tw[i + 4]) + q.C2 * (Tw[i + 1] + Tw[i + 3]) + q.C3 * Tw[i + 2];
      wk_next = wk;
      wkf = (K == 0) ? wk * R[i] : wk * RTTK1[i];
    }
    double yv = zf + wkf;
    if (i > y.mtpb) yv = 0.0;
    Yf[i] = yv;
  }
}

// A rows: w(i) (P_a P_c + Q_a Q_c) RPOR on 2 <= i <= min(MF(a), MF(c)).
// w is the closed Newton-Cotes weight pattern of QUAD started at i = 2:
// C1 at 2, then C2, C3, C2, C4 repeating.
__global__ void k_apairs(const int2 *__restrict__ pairs, int npairs, const double *__restrict__ PF,
                         const double *__restrict__ QF, int ld, const int *__restrict__ MF,
                         const double *__restrict__ RPOR, int KC, QuadConst q, double *__restrict__ A) {
  const int p = blockIdx.y;
  if (p >= npairs) return;
  const int a = pairs[p].x, c = pairs[p].y;
  const int m = min(MF[a], MF[c]);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < KC; i += gridDim.x * blockDim.x) {
    double v = 0.0;
    if (i >= 2 && i <= m) {
      const double rho = (pf(PF, ld, i, a) * pf(PF, ld, i, c) + pf(QF, ld, i, a) * pf(QF, ld, i, c)) * RPOR[i];
      const int ph = (i - 2) & 3;
      const double w = (i == 2) ? q.C1 : (ph == 1 || ph == 3) ? q.C2 : (ph == 2) ? q.C3 : q.C4;
      v = w * rho;
    }
    A[(size_t)p * KC + i] = v;
  }
}

// Completes one R^k(ab;cd) from its contraction sum: QUAD's power-law head
// term at i = 2 and the end-panel correction at MTP (quad.f90), written at
// its GENINTRK position; entries whose QUAD head index is not 2 go to the
// general per-integral QUAD instead.
// QUAD's power-law head term and end-panel correction (quad.f90:52-103) for
// integral (a, c; f) of order k whose GEMM part (grid points 3.., the
// Newton-Cotes weights folded into A) is `sum`, stored at VALTEIRK position
// pos; an integral whose head index is not 2 goes to the general QUAD list.
__device__ __forceinline__ void rk_head_store(int k, int a, int c, int f, long long pos, double sum,
                                              const YDesc *__restrict__ yd, const double *__restrict__ Y, int np,
                                              const double *__restrict__ PF, const double *__restrict__ QF, int ld,
                                              const int *__restrict__ MF, const double *__restrict__ R,
                                              const double *__restrict__ RP, const double *__restrict__ RPOR,
                                              const double *__restrict__ HD, const QuadConst &q,
                                              double *__restrict__ val, QuadItem *__restrict__ fb,
                                              int *__restrict__ nfb) {
  const YDesc y = yd[f];
  int mtp;
  if (k == 0 && y.b == y.d)
    mtp = min(MF[a], MF[c]);
  else
    mtp = min(min(y.mtp, MF[a]), MF[c]);
  const double *Yf = Y + (size_t)f * np;
  auto ta = [&](int i) {
    return ((pf(PF, ld, i, a) * pf(PF, ld, i, c) + pf(QF, ld, i, a) * pf(QF, ld, i, c)) * RPOR[i]) * Yf[i];
  };
  bool ok = mtp >= 3;
  double res = 0.0;
  if (ok) {
    const double tai = ta(2), taip1 = ta(3);
    const double t = taip1 / tai;
    ok = !(fabs(tai) <= 0.0) && (t > 0.0);
    if (ok) {
      // QUAD's head term with the grid's factors per point (HD): the ratio
      // (TA(3)/RP(3)) / (TA(2)/RP(2)), sigma = log(ratio) / log(R(3)/R(2)),
      // R(2) TA(2)/RP(2) / (sigma + 1); equal to quad.f90's to rounding
      const double sigma = log(t * HD[np + 2]) * HD[2];
      const double fri = tai * HD[2 * np + 2];
      res = fri / (sigma + 1.0) + sum;
      if ((mtp - 2) % 4 == 0) res = res - q.C1 * ta(mtp);
    }
  }
  if (ok) {
    val[pos] = res;
  } else {
    const int slot = atomicAdd(nfb, 1);
    fb[slot] = QuadItem{a, c, f, mtp, pos};
  }
}

// the GEMM part `sum` of canonical entry (p = (a, c), f) of tile T: its
// GENINTRK position, then the head term
__device__ __forceinline__ void rk_finish(const RkTile &T, int p, int idx_c, int f, double sum,
                                          const int2 *__restrict__ pairs, const YDesc *__restrict__ yd,
                                          const double *__restrict__ Y, int np, const double *__restrict__ PF,
                                          const double *__restrict__ QF, int ld, const int *__restrict__ MF,
                                          const double *__restrict__ R, const double *__restrict__ RP,
                                          const double *__restrict__ RPOR, const double *__restrict__ HD,
                                          const QuadConst &q, double *__restrict__ val, long long nval,
                                          QuadItem *__restrict__ fb, int *__restrict__ nfb) {
  const YDesc y = yd[f];
  const long long pos = T.base + (long long)T.ncA * (y.cs - T.cs_a) + (long long)idx_c * y.nd + (long long)(f - y.cs);
  if (pos < 0 || pos >= nval) {  // position outside the table: report, never write
    atomicExch(nfb + 1, 1);
    return;
  }
  rk_head_store(T.k, T.a, pairs[p].y, f, pos, sum, yd, Y, np, PF, QF, ld, MF, R, RP, RPOR, HD, q, val, fb, nfb);
}

// ---------------------------------------------------------------------------
// R^k contraction: for each (k, a) the GEMM  O[c, f] = sum_i A[(a,c), i] Y[f, i]
// over the rows c in C(a,k) and the Y functions f = (b,d) with b >= a, then
// QUAD's power-law head term and end-panel correction per entry. Output
// positions follow GENINTRK's loop order (k, a, b, c, d).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_rk_gemm(const RkTile *__restrict__ tiles, const int *__restrict__ rowpair,
                                                 const int2 *__restrict__ pairs, const double *__restrict__ A,
                                                 const double *__restrict__ Y, const YDesc *__restrict__ yd, int KC,
                                                 int np, const double *__restrict__ PF, const double *__restrict__ QF,
                                                 int ld, const int *__restrict__ MF, const double *__restrict__ R,
                                                 const double *__restrict__ RP, const double *__restrict__ RPOR,
                                                 const double *__restrict__ HD, QuadConst q,
                                                 double *__restrict__ val, long long nval,
                                                 QuadItem *__restrict__ fb, int *__restrict__ nfb) {
  __shared__ double As[2][KC_TILE][BM];
  __shared__ double Bs[2][KC_TILE][BN + 1];
  __shared__ int rowp[BM];
  const RkTile T = tiles[blockIdx.x];
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  const int nrow = min(BM, T.ncA - T.r0);
  const int ncol = T.c1 - T.c0;
  if (tid < BM) rowp[tid] = (tid < nrow) ? rowpair[T.rowpair0 + T.r0 + tid] : -1;
  __syncthreads();
  double acc[2][4];
#pragma unroll
  for (int u = 0; u < 2; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) acc[u][v] = 0.0;

  auto load = [&](int buf, int k0) {
    // A: BM rows x KC_TILE ; 256 threads -> 2 elements each
    for (int e = tid; e < BM * KC_TILE; e += 256) {
      const int r = e / KC_TILE, kk = e % KC_TILE;
      const int p = rowp[r];
      As[buf][kk][r] = (p >= 0) ? A[(size_t)p * KC + k0 + kk] : 0.0;
    }
    for (int e = tid; e < BN * KC_TILE; e += 256) {
      const int j = e / KC_TILE, kk = e % KC_TILE;
      Bs[buf][kk][j] = (j < ncol) ? Y[(size_t)(T.c0 + j) * np + k0 + kk] : 0.0;
    }
  };
  const int nk = KC / KC_TILE;
  load(0, 0);
  __syncthreads();
  for (int s = 0; s < nk; ++s) {
    const int buf = s & 1;
    if (s + 1 < nk) load(buf ^ 1, (s + 1) * KC_TILE);
#pragma unroll
    for (int kk = 0; kk < KC_TILE; ++kk) {
      const double a0 = As[buf][kk][ty * 2 + 0], a1 = As[buf][kk][ty * 2 + 1];
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const double b = Bs[buf][kk][tx * 4 + v];
        acc[0][v] = fma(a0, b, acc[0][v]);
        acc[1][v] = fma(a1, b, acc[1][v]);
      }
    }
    __syncthreads();
  }
  // epilogue
#pragma unroll
  for (int u = 0; u < 2; ++u) {
    const int r = ty * 2 + u;
    if (r >= nrow) continue;
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int j = tx * 4 + v;
      if (j >= ncol) continue;
      rk_finish(T, rowp[r], T.r0 + r, T.c0 + j, acc[u][v], pairs, yd, Y, np, PF, QF, ld, MF, R, RP, RPOR, HD, q,
                val, nval, fb, nfb);
    }
  }
}

// ---------------------------------------------------------------------------
// The same contraction on the tensor cores, split-precision (Ozaki): each row
// of A and of Y is scaled by a power of two 2^e (|row| < 2^(e-1)) and cut
// into OZ_S slices of 7 bits, x = 2^e sum_s q_s 2^(-7(s+1)), each q_s the
// nearest integer to the remainder, so |q_s| <= 64 (every step is exact in
// FP64). Products of slice pairs (s, t) with s + t < OZ_S are exact integer
// tensor products (|q_s q_t| <= 4096); pairs with the same q = s + t share one
// FP32 accumulator in tensor memory, where at most 10 pairs x 256 grid points
// x 4096 < 2^24 keeps every partial sum an exact integer between flushes. The sum over q is then
// sum_q acc_q 2^(eA + eY - 7(q + 2)). With OZ_S = 10 the result agrees with
// the FP64 contraction to a few 1e-13 relative on R^k data.
// ---------------------------------------------------------------------------
constexpr int OZ_S = 10;

// General per-integral QUAD: TA(i) = ((P_a P_c + Q_a Q_c) RPOR) Y_f(i),
// one warp per integral, sequential reference-order sum on lane 0.
// ---------------------------------------------------------------------------
// The Ozaki contraction on GB300's fifth-generation tensor cores (tcgen05).
//
// For each k the rows of all (k, a) problems (the (a, c) pairs with a <= c
// and TRIANGRK(l_a, k, l_c), in GENINTRK's order) and all Y functions of k
// form one GEMM, cut into tiles of TC_M = 128 functions (the MMA's M) x
// TC_N = 48 rows (N); tiles that hold no needed entry (b < a for all) are
// skipped. k_oz_tile writes the int8-range slices (|q| <= 64) as fp16, which
// holds them exactly, straight into per-tile blocks laid out as the MMA reads
// them from shared memory (no-swizzle K-major core matrices: 8 rows x 16 B,
// neighbours in K 128 B apart, in M/N 256 B apart), one block per 32 grid
// points: 80 KB of Y slices, 30 KB of A slices.
//
// k_rk_tc, one CTA per tile, is warp-specialised. Warp 4 streams the blocks
// into two shared-memory stages with cp.async.bulk (completion counted in
// bytes on a per-stage "full" mbarrier) and issues, per K = 16 step, the 55
// slice-pair MMAs tcgen05.mma.cta_group::1.kind::f16 into the FP32 tensor-
// memory accumulator of their group q = s + t (OZ_S x TC_N columns); a
// tcgen05.commit to the stage's "empty" mbarrier frees the stage. Every
// TC_FLUSH stages (256 grid points, while every group sum is still an exact
// integer below 2^24) warps 0-3 read their 32 lanes of each group
// (tcgen05.ld) and fold group q, scaled by 2^(-7q), into double-float sums;
// the next MMA of each group overwrites. The raw sum 2^(eA+eY-14) (h + l) is
// stored at the entry's GENINTRK position; k_rk_finish_all adds the head
// term. Every wait is bounded: on a timeout the CTA records it, waits
// (bounded) for what it issued, frees its tensor memory and writes nothing.
// ---------------------------------------------------------------------------
constexpr int TC_M = 128, TC_N = 48, TC_KC = 32, TC_FLUSH = 8;
constexpr int TC_YBLK = OZ_S * 2 * (TC_M / 8) * 2 * 64;  // fp16 elements per Y block (80 KB)
constexpr int TC_ABLK = OZ_S * 2 * (TC_N / 8) * 2 * 64;  // fp16 elements per A block (30 KB)
constexpr size_t TC_SMEM = (size_t)2 * (TC_YBLK + TC_ABLK) * sizeof(__half) + 128;
constexpr uint32_t TC_TMEM_COLS = 512;  // >= OZ_S * TC_N, a power of two
constexpr int TC_SPIN = 1 << 24;
constexpr int TC_THREADS = 160;  // warps 0-3: accumulators; warp 4: copies and MMAs

struct TcRow {  // one row of a k: its pair, problem and position data
  int p, a, ic, ncA, cs_a;
  long long base;
};
struct TcTile {
  int k, fg, pg;  // k; global indices of the Y block column and the A block column
  int f0, fn;     // first Y function and how many are valid
  int r0, rn;     // first row (TcRow index) and how many are valid
  int c0, c1, s;  // grid chunks [c0, c1) of this split of the tile, split index
};

}  // namespace

// GENINTRK's orbital-set-dependent structure and its work buffers, kept on
// the context between calls (gg_genintrk rebuilds it when the orbitals' l, j
// or kmax change)
struct RkCache {
  std::vector<int> key;
  int nf = 0, npairs = 0;
  std::vector<YDesc> yd;
  std::vector<int> kend, rowpair, yslot, aslot, fidx;
  std::vector<int2> pairs;
  std::vector<RkTile> tiles;
  std::vector<TcRow> tcrows;
  std::vector<TcTile> tct;
  DBuf<YDesc> dYd;
  DBuf<int2> dPairs;
  DBuf<RkTile> dTiles;
  DBuf<int> dRowpair, dYslot, dAslot, dFidx, dNfb, dEA, dEY;
  DBuf<int32_t> dKst;
  DBuf<TcTile> dTct;
  // split-K form of tct (each tile's grid chunks over nsplit CTAs) for the
  // chunk count it was made for, and the partial sums it writes
  std::vector<TcTile> tcs;
  int tcs_nch = -1, tcs_split = 0;
  DBuf<TcTile> dTcs;
  DBuf<double> dParts;
  DBuf<TcRow> dTcr;
  DBuf<double> dY, dA, scratch;
  DBuf<QuadItem> dFb;
  DBuf<__half> dYt, dAt;
};

void rk_cache_free(RkCache *c) { delete c; }

const std::vector<int> *rk_structure_key(const gg_ctx *ctx) {
  return (ctx->rk.cache && ctx->rk.valid) ? &ctx->rk.cache->key : nullptr;
}

namespace {

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: start address, leading (K) byte offset
// 128, stride (M/N) byte offset 256, descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t tc_desc(uint32_t addr) {
  return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)(128 >> 4) << 16) | ((uint64_t)(256 >> 4) << 32) |
         ((uint64_t)1 << 46);
}

__device__ __forceinline__ bool tc_wait(uint32_t mbar, uint32_t parity, int spin = TC_SPIN) {
  uint32_t done = 0;
  for (int it = 0; it < spin && !done; ++it)
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(mbar), "r"(parity)
        : "memory");
  return done != 0;
}

// Slices of rows into their tile blocks: one CTA per row slot (slot = tile
// block column g, row m < R); src_row[slot] < 0 pads with zeros. The row's
// exponent goes to exps[src_row] (the same row always gets the same value).
template <int R>
__global__ void k_oz_tile(const double *__restrict__ M, int pitch, int K, int nch, const int *__restrict__ src_row,
                          int *__restrict__ exps, __half *__restrict__ dst) {
  constexpr int BLK = OZ_S * 2 * (R / 8) * 2 * 64;
  const int slot = blockIdx.x, g = slot / R, m = slot % R;
  const int row = src_row[slot];
  __shared__ double red[128];
  double mx = 0.0;
  if (row >= 0)
    for (int i = threadIdx.x; i < K; i += blockDim.x) mx = fmax(mx, fabs(M[(size_t)row * pitch + i]));
  red[threadIdx.x] = mx;
  __syncthreads();
  for (int st = 64; st > 0; st >>= 1) {
    if ((int)threadIdx.x < st) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + st]);
    __syncthreads();
  }
  mx = red[0];
  const int e = (mx > 0.0) ? ilogb(mx) + 2 : 0;  // mx < 2^(e-1)
  if (threadIdx.x == 0 && row >= 0) exps[row] = e;
  __half *base = dst + (size_t)g * nch * BLK;
  const int KP = nch * TC_KC;
  for (int i = threadIdx.x; i < KP; i += blockDim.x) {
    // x 2^35 = X1 + d exactly with X1 = rint(x 2^35), |d| <= 1/2 (|x| < 1/2);
    // X2 = rint(d 2^35); x = (X1 + X2 2^-35) 2^-35 to 2^-71, |X1|, |X2| <= 2^34.
    // Each of X1 and X2 gives five balanced base-128 digits (|digit| <= 64)
    // in integer arithmetic: only the two roundings use the FP64 pipe, which
    // GB300 issues slowly.
    const double xs = (row >= 0 && i < K) ? scalbn(M[(size_t)row * pitch + i], 35 - e) : 0.0;
    const double x1 = rint(xs);
    long long X[2] = {(long long)x1, (long long)rint((xs - x1) * 34359738368.0)};  // 2^35
    int dg[OZ_S];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      long long v = X[h];
#pragma unroll
      for (int u = 4; u >= 1; --u) {
        const int r = (int)(((v + 64) & 127) - 64);  // balanced remainder in [-64, 63]
        dg[h * 5 + u] = r;
        v = (v - r) >> 7;
      }
      dg[h * 5] = (int)v;  // |v| <= 64
    }
    const int c = i / TC_KC, kk = i % TC_KC, j = kk / 16, k8 = (kk / 8) % 2, el = kk % 8;
    __half *blk = base + (size_t)c * BLK + ((size_t)(m / 8) * 2 + k8) * 64 + (m % 8) * 8 + el;
#pragma unroll
    for (int q = 0; q < OZ_S; ++q) blk[(size_t)(q * 2 + j) * (R / 8) * 2 * 64] = __int2half_rn(dg[q]);
  }
}

__global__ void __launch_bounds__(TC_THREADS, 1) k_rk_tc(const TcTile *__restrict__ tiles,
                                                         const TcRow *__restrict__ rows,
                                                         const __half *__restrict__ Yt,
                                                         const __half *__restrict__ At, int nch,
                                                         const int *__restrict__ eA, const int *__restrict__ eY,
                                                         const YDesc *__restrict__ yd, double *__restrict__ val,
                                                         long long nval, int *__restrict__ flags, int stall_tile) {
  extern __shared__ __align__(1024) unsigned char tsm[];
  __half *Ysm = reinterpret_cast<__half *>(tsm);
  __half *Asm = Ysm + 2 * TC_YBLK;
  uint64_t *full = reinterpret_cast<uint64_t *>(Asm + 2 * TC_ABLK);
  uint64_t *empty = full + 2;
  uint32_t *tslot = reinterpret_cast<uint32_t *>(empty + 2);
  int *okflag = reinterpret_cast<int *>(tslot + 1);
  __shared__ TcRow trow[TC_N];
  const TcTile T = tiles[blockIdx.x];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid < TC_N) trow[tid] = (tid < T.rn) ? rows[T.r0 + tid] : TcRow{-1, 0, 0, 0, 0, 0};
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tslot)),
                 "r"(TC_TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    for (int st = 0; st < 2; ++st) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(&full[st])), "r"(1));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(&empty[st])), "r"(1));
    }
    *okflag = 1;
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = *tslot;
  const int nloc = T.c1 - T.c0;  // chunks of this split
  const int nflush = (nloc + TC_FLUSH - 1) / TC_FLUSH;
  if (warp == 4) {
    // copies and MMAs (lane 0 issues; the warp stays converged). A tile
    // named by stall_tile (a test of the bounded waits) withholds its first
    // copy and polls briefly: its first wait runs out with nothing in flight.
    const bool stall = (int)blockIdx.x == stall_tile;
    const int spin = stall ? (1 << 12) : TC_SPIN;
    const uint32_t idesc = (1u << 4) | ((uint32_t)(TC_N >> 3) << 17) | ((uint32_t)(TC_M >> 4) << 24);
    const char *ysrc = reinterpret_cast<const char *>(Yt + (size_t)T.fg * nch * TC_YBLK);
    const char *asrc = reinterpret_cast<const char *>(At + (size_t)T.pg * nch * TC_ABLK);
    constexpr uint32_t YB = TC_YBLK * sizeof(__half), AB = TC_ABLK * sizeof(__half);
    // local chunk j of the split is grid chunk T.c0 + j
    auto copy = [&](int j) {
      const int st = j & 1;
      if (lane == 0) {
        const uint32_t fb = smem_addr(&full[st]);
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(fb), "r"(YB + AB) : "memory");
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                smem_addr(Ysm + st * TC_YBLK)),
            "l"(ysrc + (size_t)(T.c0 + j) * YB), "r"(YB), "r"(fb)
            : "memory");
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                smem_addr(Asm + st * TC_ABLK)),
            "l"(asrc + (size_t)(T.c0 + j) * AB), "r"(AB), "r"(fb)
            : "memory");
      }
      __syncwarp();
    };
    bool ok = true;
    uint32_t fresh = (1u << OZ_S) - 1;
    int issued = -1;  // last chunk whose MMAs were committed
    int copied = -1;  // last chunk whose copy was issued
    if (!stall) {
      copy(0);
      copied = 0;
    }
    int fl = 0;
    for (int j = 0; j < nloc; ++j) {
      const int st = j & 1;
      if (ok) ok = __all_sync(0xffffffffu, tc_wait(smem_addr(&full[st]), (j >> 1) & 1, spin));
      if (ok) {
        asm volatile("tcgen05.fence::after_thread_sync;");
        if (lane == 0) {
          const uint32_t yb = smem_addr(Ysm + st * TC_YBLK), ab = smem_addr(Asm + st * TC_ABLK);
#pragma unroll 1
          for (int ks = 0; ks < 2; ++ks)
#pragma unroll 1
            for (int sa = 0; sa < OZ_S; ++sa) {
              const uint64_t bdesc = tc_desc(ab + (uint32_t)(sa * 2 + ks) * ((TC_N / 8) * 2 * 64 * 2));
#pragma unroll 1
              for (int t = 0; t < OZ_S - sa; ++t) {
                const int qg = sa + t;
                const uint64_t adesc = tc_desc(yb + (uint32_t)(t * 2 + ks) * ((TC_M / 8) * 2 * 64 * 2));
                const uint32_t accum = ((fresh >> qg) & 1u) ? 0u : 1u;
                fresh &= ~(1u << qg);
                asm volatile(
                    "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                    " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(
                        tmem + (uint32_t)(qg * TC_N)),
                    "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accum));
              }
            }
          asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                           smem_addr(&empty[st]))
                       : "memory");
        }
        __syncwarp();
        issued = j;
        // refill the other stage with chunk j + 1 once chunk j - 1's MMAs are done
        if (j + 1 < nloc) {
          if (j >= 1)
            ok = __all_sync(0xffffffffu, tc_wait(smem_addr(&empty[(j - 1) & 1]), ((j - 1) >> 1) & 1, spin));
          if (ok) {
            copy(j + 1);
            copied = j + 1;
          }
        }
      }
      if ((j + 1) % TC_FLUSH == 0 || j == nloc - 1) {
        if (ok) ok = __all_sync(0xffffffffu, tc_wait(smem_addr(&empty[st]), (j >> 1) & 1, spin));  // MMAs done
        if (!ok && lane == 0) *okflag = 0;
        asm volatile("tcgen05.fence::before_thread_sync;");
        __syncthreads();  // A: the accumulators are ready (or the flag says no)
        __syncthreads();  // B: warps 0-3 have read them
        asm volatile("tcgen05.fence::after_thread_sync;");
        fresh = (1u << OZ_S) - 1;
        ++fl;
      }
    }
    for (; fl < nflush; ++fl) {  // a failed wait leaves the loop early: meet the remaining barriers
      __syncthreads();
      __syncthreads();
    }
    if (!ok && lane == 0) {
      // timed out: before the tensor memory is freed and the CTA leaves,
      // wait (bounded) for the last copy issued to land in shared memory and
      // for the last committed MMAs to finish; 2 records a failed drain
      bool drained = true;
      if (copied >= 0) drained = tc_wait(smem_addr(&full[copied & 1]), (copied >> 1) & 1);
      if (issued >= 0) drained = tc_wait(smem_addr(&empty[issued & 1]), (issued >> 1) & 1) && drained;
      atomicMax(flags + 1, drained ? 1 : 2);
    }
  } else {
    // warps 0-3: lane quadrant `warp` of each group accumulator
    float ah[TC_N], al[TC_N];
#pragma unroll
    for (int n = 0; n < TC_N; ++n) ah[n] = al[n] = 0.f;
    for (int fl = 0; fl < nflush; ++fl) {
      __syncthreads();  // A
      asm volatile("tcgen05.fence::after_thread_sync;");
      if (*okflag) {
#pragma unroll 1
        for (int qg = 0; qg < OZ_S; ++qg) {
          const float scale = __int_as_float((127 - 7 * qg) << 23);  // 2^(-7 qg)
#pragma unroll
          for (int h = 0; h < TC_N / 16; ++h) {
            uint32_t r[16];
            const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(qg * TC_N + h * 16);
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
                "[%16];"
                : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                  "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                  "=r"(r[15])
                : "r"(taddr));
            asm volatile("tcgen05.wait::ld.sync.aligned;");
#pragma unroll
            for (int u = 0; u < 16; ++u) {
              // (ah, al) += v: TwoSum into the high part, the error into al
              const int n = h * 16 + u;
              const float v = __uint_as_float(r[u]) * scale;
              const float sv = ah[n] + v;
              const float bb = sv - ah[n];
              const float e = (ah[n] - (sv - bb)) + (v - bb);
              ah[n] = sv;
              al[n] = al[n] + e;
            }
          }
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;");
      __syncthreads();  // B
    }
    const int m = warp * 32 + lane;
    if (*okflag && m < T.fn) {
      const int f = T.f0 + m;
      const YDesc y = yd[f];
      const int ey = eY[f];
#pragma unroll
      for (int n = 0; n < TC_N; ++n) {
        const TcRow rw = trow[n];
        if (n >= T.rn || f < rw.cs_a) continue;  // padding, or b < a: not a GENINTRK entry
        const long long pos =
            rw.base + (long long)rw.ncA * (y.cs - rw.cs_a) + (long long)rw.ic * y.nd + (long long)(f - y.cs);
        if (pos < 0 || pos >= nval) {
          atomicExch(flags, 1);  // position outside the table
          continue;
        }
        // split s of the contraction: its partial sum (val + s nval)
        val[(long long)T.s * nval + pos] = scalbn((double)ah[n] + (double)al[n], eA[rw.p] + ey - 14);
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_TMEM_COLS));
}

// QUAD head term for every table entry, one thread per entry: (a, b, c, d)
// from INDTEIRK, k from KSTART, the Y function from fidx[(k KEY + b) KEY + d];
// the entry's GEMM part is the sum, in split order, of parts[s n + i] for
// s < nsplit (parts == val when the contraction was not split).
__global__ void k_rk_finish_all(const int32_t *__restrict__ ind, long long n, const int32_t *__restrict__ kstart,
                                int kloop, int KEY, const int *__restrict__ fidx, const YDesc *__restrict__ yd,
                                const double *__restrict__ Y, int np, const double *__restrict__ PF,
                                const double *__restrict__ QF, int ld, const int *__restrict__ MF,
                                const double *__restrict__ R, const double *__restrict__ RP,
                                const double *__restrict__ RPOR, const double *__restrict__ HD, QuadConst q,
                                double *__restrict__ val, QuadItem *__restrict__ fb, int *__restrict__ nfb,
                                const double *__restrict__ parts, int nsplit) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    int p = ind[i];
    const int d = p % KEY;
    p /= KEY;
    const int c = p % KEY;
    p /= KEY;
    const int b = p % KEY, a = p / KEY;
    int k = 0;
    while (k < kloop && (long long)kstart[k + 1] - 1 <= i) ++k;
    const int f = fidx[((size_t)k * KEY + b) * KEY + d];
    if (f < 0) {
      atomicExch(nfb + 1, 1);
      continue;
    }
    double gemm = parts[i];
    for (int t = 1; t < nsplit; ++t) gemm += parts[(long long)t * n + i];
    rk_head_store(k, a, c, f, i, gemm, yd, Y, np, PF, QF, ld, MF, R, RP, RPOR, HD, q, val, fb, nfb);
  }
}

__global__ void k_quad_items(const QuadItem *__restrict__ items, const int *__restrict__ nitems_p, int nitems_max,
                             const double *__restrict__ Y, int np, const double *__restrict__ PF,
                             const double *__restrict__ QF, int ld, const double *__restrict__ R,
                             const double *__restrict__ RP, const double *__restrict__ RPOR, QuadConst q,
                             double *__restrict__ out) {
  extern __shared__ double sm[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int wpb = blockDim.x >> 5;
  double *TA = sm + (size_t)warp * np;
  const int nitems = nitems_p ? min(*nitems_p, nitems_max) : nitems_max;
  for (int it = blockIdx.x * wpb + warp; it < nitems; it += gridDim.x * wpb) {
    const QuadItem w = items[it];
    const double *Yf = Y + (size_t)w.f * np;
    for (int i = lane; i < np; i += 32) {
      double v = 0.0;
      if (i >= 2 && i <= w.mtp)
        v = ((pf(PF, ld, i, w.a) * pf(PF, ld, i, w.c) + pf(QF, ld, i, w.a) * pf(QF, ld, i, w.c)) * RPOR[i]) * Yf[i];
      TA[i] = v;
    }
    __syncwarp();
    if (lane == 0) out[w.pos] = quad_seq(TA, w.mtp, R, RP, q);
    __syncwarp();
  }
}

// The same QUAD for the table's items, one warp per integral with the work
// spread over the lanes: the head index (first i in [2, MTP-1] with
// TA(i) != 0 and TA(i+1)/TA(i) > 0) by ballot, the 4-point panel sums
// (quad.f90:94-99) split over the lanes and combined by a fixed butterfly,
// so the result is deterministic. Only the order of the panel sum differs
// from quad_seq (a few ulps of the sum of |terms|). TA values are formed
// where they are used, so no grid size limit comes from shared memory.
__global__ void k_quad_table(const QuadItem *__restrict__ items, const int *__restrict__ nitems_p, int nitems_max,
                             const double *__restrict__ Y, int np, const double *__restrict__ PF,
                             const double *__restrict__ QF, int ld, const double *__restrict__ R,
                             const double *__restrict__ RP, const double *__restrict__ RPOR,
                             const double *__restrict__ HD, QuadConst q, double *__restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int wpb = blockDim.x >> 5;
  const int nitems = min(*nitems_p, nitems_max);
  // TA(i) of quad.f90 for item w, zero outside [2, MTP] (the pads TA(MTP+1..MTP+3))
  auto ta = [&](const QuadItem &w, int i) -> double {
    if (i < 2 || i > w.mtp) return 0.0;
    const double *Pa = PF + (size_t)(w.a - 1) * ld, *Pc = PF + (size_t)(w.c - 1) * ld;
    const double *Qa = QF + (size_t)(w.a - 1) * ld, *Qc = QF + (size_t)(w.c - 1) * ld;
    return ((Pa[i - 1] * Pc[i - 1] + Qa[i - 1] * Qc[i - 1]) * RPOR[i]) * Y[(size_t)w.f * np + i];
  };
  // One item per warp for the head index and the panel sum; the block's
  // items then get their head terms (a logarithm and divisions: serial FP64
  // work that would otherwise occupy a warp per item) from the lanes of
  // warp 0, one item each
  __shared__ int sh_head[32];
  __shared__ double sh_s[32];
  for (int base = blockIdx.x * wpb; base < nitems; base += gridDim.x * wpb) {
    const int it = base + (threadIdx.x >> 5);
    if (it < nitems) {
      const QuadItem w = items[it];
      int head = -1;
      for (int i0 = 2; i0 <= w.mtp - 1 && head < 0; i0 += 32) {
        const int i = i0 + lane;
        bool hit = false;
        if (i <= w.mtp - 1) {
          const double tai = ta(w, i);
          hit = !(fabs(tai) <= 0.0) && (ta(w, i + 1) / tai > 0.0);
        }
        const unsigned bal = __ballot_sync(0xffffffffu, hit);
        if (bal) head = i0 + __ffs(bal) - 1;
      }
      double sp = 0.0;
      if (head >= 0)
        for (int j = head + 1 + 4 * lane; j <= w.mtp; j += 128)
          sp += q.C2 * (ta(w, j) + ta(w, j + 2)) + q.C3 * ta(w, j + 1) + q.C4 * ta(w, j + 3);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) sp += __shfl_xor_sync(0xffffffffu, sp, o);
      if (lane == 0) {
        sh_head[threadIdx.x >> 5] = head;
        sh_s[threadIdx.x >> 5] = sp;
      }
    }
    __syncthreads();
    if (threadIdx.x < wpb && base + (int)threadIdx.x < nitems) {
      const QuadItem w = items[base + threadIdx.x];
      const int i = sh_head[threadIdx.x];
      double result = 0.0;
      if (i >= 0) {
        // quad.f90:61-103 with the grid's factors per point (HD)
        const double tai = ta(w, i), taip1 = ta(w, i + 1);
        const double sigma = log((taip1 / tai) * HD[np + i]) * HD[i];
        result = (tai * HD[2 * np + i]) / (sigma + 1.0);
        result = result + q.C1 * tai;
        result = result + sh_s[threadIdx.x];
        if ((w.mtp - i) % 4 == 0) result = result - q.C1 * ta(w, w.mtp);
      }
      out[w.pos] = result;
    }
    __syncthreads();
  }
}

// YPOT / XPOT (rmcdhf90/ypot.f90:35-49, xpot.f90:31-54): one thread per grid
// point combines the list's Y functions in the list's order (the reference's
// per-point operations: YP = YP - COEFF*TB; CTB = COEFF*TB, XP += CTB*QF,
// XQ -= CTB*PF, with COEFF = XA/C). One launch takes the lists of several
// jobs (blockIdx.y); each thread loads the next group of terms (index,
// coefficient, Y value, orbital values; 16 for YPOT, 8 for XPOT) before it
// combines the current ones, so the loads do not wait on the chain.
struct PotSeg {
  const int *fidx, *iorb;
  const double *coef;
  double *out0, *out1;
  int ncof;
};
template <int MODE>
__global__ void k_potential(const PotSeg *__restrict__ segs, const double *__restrict__ Y, int np,
                            const double *__restrict__ ZZ, const double *__restrict__ PF,
                            const double *__restrict__ QF, int ld, int n) {
  constexpr int A = MODE == 0 ? 16 : 8;  // terms loaded ahead
  const PotSeg g = segs[blockIdx.y];
  const int i = 1 + blockIdx.x * blockDim.x + threadIdx.x;
  if (i > n) return;
  const int nc = g.ncof;
  double cy[A], cc[A], cq[A], cp[A];
  double ny[A], nc_[A], nq[A], npf[A];
  // terms t0 .. t0 + A - 1 (those below nc when `guard`)
  auto load = [&](int t0, bool guard, double *y, double *c, double *qv, double *pv) {
#pragma unroll
    for (int u = 0; u < A; ++u) {
      const int t = t0 + u;
      y[u] = c[u] = qv[u] = pv[u] = 0.0;
      if (!guard || t < nc) {
        c[u] = g.coef[t];
        y[u] = Y[(size_t)g.fidx[t] * np + i];
        if (MODE == 1) {
          const int io = g.iorb[t];
          qv[u] = pf(QF, ld, i, io);
          pv[u] = pf(PF, ld, i, io);
        }
      }
    }
  };
  double a0 = (MODE == 0) ? ZZ[i] : 0.0, a1 = 0.0;
  auto combine = [&](int t0, const double *y, const double *c, const double *qv, const double *pv) {
#pragma unroll
    for (int u = 0; u < A; ++u)
      if (t0 + u < nc) {
        if (MODE == 0) {
          a0 = a0 - c[u] * y[u];
        } else {
          const double ctb = c[u] * y[u];
          a0 = a0 + ctb * qv[u];
          a1 = a1 - ctb * pv[u];
        }
      }
  };
  load(0, true, cy, cc, cq, cp);
  int t = 0;
  // while the next group is complete its loads need no bounds test
  for (; t + 2 * A <= nc; t += A) {
    load(t + A, false, ny, nc_, nq, npf);
    combine(t, cy, cc, cq, cp);
#pragma unroll
    for (int u = 0; u < A; ++u) {
      cy[u] = ny[u];
      cc[u] = nc_[u];
      cq[u] = nq[u];
      cp[u] = npf[u];
    }
  }
  if (t + A <= nc) {  // cur is complete; fewer than A terms follow it
    load(t + A, true, ny, nc_, nq, npf);
    combine(t, cy, cc, cq, cp);
    combine(t + A, ny, nc_, nq, npf);
  } else {
    combine(t, cy, cc, cq, cp);
  }
  g.out0[i - 1] = a0;
  if (MODE == 1) g.out1[i - 1] = a1;
}

// XPOT in two passes for long lists: the products of a segment of terms at
// every grid point (CTB = COEFF TB, CTB QF and CTB PF) by all SMs, then per
// grid point the sums XP = XP + CTB QF, XQ = XQ - CTB PF in list order (the
// same operations as k_potential; only the additions stay sequential). A
// segment is terms t0 .. t0+nt of one job's list; one launch takes the
// segments of several jobs (blockIdx.y / blockIdx.z).
struct XSeg {
  const int *fidx, *iorb;
  const double *coef;
  double *P1, *P2;  // nt * n products each
  double *xp, *xq;
  int nt;
};
__global__ void k_xprod(const XSeg *__restrict__ segs, const double *__restrict__ Y, int np,
                        const double *__restrict__ PF, const double *__restrict__ QF, int ld, int n) {
  const XSeg g = segs[blockIdx.y];
  const int tot = g.nt * n;  // the caller keeps nt * n below 2^26
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += gridDim.x * blockDim.x) {
    const int t = e / n, i = e % n + 1;
    const double ctb = g.coef[t] * Y[(size_t)g.fidx[t] * np + i];
    g.P1[e] = ctb * pf(QF, ld, i, g.iorb[t]);
    g.P2[e] = ctb * pf(PF, ld, i, g.iorb[t]);
  }
}
// k_xsum: 32 grid points of segment blockIdx.z per block; blockIdx.y = 0
// sums XP = XP + P1, blockIdx.y = 1 sums XQ = XQ - P2. The loads run XSUM_AHEAD terms ahead of
// the additions (register double buffer) so that the chain of dependent
// FP64 additions, not the load latency, sets the time.
constexpr int XSUM_AHEAD = 48;
template <bool SUB>
__device__ __forceinline__ double xsum_chain(double acc, const double *__restrict__ P, int nt, int n) {
  constexpr int A = XSUM_AHEAD;
  double cur[A], nxt[A];
#pragma unroll
  for (int u = 0; u < A; ++u) cur[u] = (u < nt) ? P[(size_t)u * n] : 0.0;
  int t = 0;
  // while the next group is complete its loads need no bounds test
  for (; t + 2 * A <= nt; t += A) {
    const double *q = P + (size_t)(t + A) * n;
#pragma unroll
    for (int u = 0; u < A; ++u) nxt[u] = q[(size_t)u * n];
#pragma unroll
    for (int u = 0; u < A; ++u) acc = SUB ? acc - cur[u] : acc + cur[u];
#pragma unroll
    for (int u = 0; u < A; ++u) cur[u] = nxt[u];
  }
  if (t + A <= nt) {  // cur is a complete group; fewer than A terms follow it
    const int t1 = t + A;
#pragma unroll
    for (int u = 0; u < A; ++u) nxt[u] = (t1 + u < nt) ? P[(size_t)(t1 + u) * n] : 0.0;
#pragma unroll
    for (int u = 0; u < A; ++u) acc = SUB ? acc - cur[u] : acc + cur[u];
#pragma unroll
    for (int u = 0; u < A; ++u)
      if (t1 + u < nt) acc = SUB ? acc - nxt[u] : acc + nxt[u];
  } else {  // fewer than A terms in all
#pragma unroll
    for (int u = 0; u < A; ++u)
      if (t + u < nt) acc = SUB ? acc - cur[u] : acc + cur[u];
  }
  return acc;
}
__global__ void k_xsum(const XSeg *__restrict__ segs, int n) {
  const XSeg g = segs[blockIdx.z];
  const int i = blockIdx.x * 32 + threadIdx.x;
  if (i >= n) return;
  if (blockIdx.y == 0)
    g.xp[i] = xsum_chain<false>(g.xp[i], g.P1 + i, g.nt, n);
  else
    g.xq[i] = xsum_chain<true>(g.xq[i], g.P2 + i, g.nt, n);
}

// The lists' labels decoded on the device, one thread per term (mode 0:
// YPOT labels, 1: XPOT labels): the term's (K, a, b) key into a dense table
// over K <= KLIMIT and the orbital pairs, marked present; the orbital it
// multiplies (XPOT) and COEFF (XPOT: XA/C, as the reference forms it). A
// label outside the orbital set or with K above KLIMIT sets *err.
__global__ void k_parse_terms(int mode, int64_t nt, const int32_t *__restrict__ lab, const double *__restrict__ co,
                              int nw, double c, int *__restrict__ tab, int *__restrict__ key,
                              int *__restrict__ iorb, double *__restrict__ coef, int *__restrict__ err) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nt; e += (int64_t)gridDim.x * blockDim.x) {
    const int32_t l0 = lab[e];
    int64_t l = l0;
    const int k = (int)(l % KEYORB);
    l /= KEYORB;
    const int a = (int)(l % KEYORB);
    l /= KEYORB;
    const int64_t b = mode == 0 ? l : l % KEYORB;
    const int64_t io = mode == 0 ? 1 : l / KEYORB;
    if (l0 < 0 || k > KLIMIT || a < 1 || a > nw || b < 1 || b > nw || io < 1 || io > nw) {
      atomicOr(err, 1);
      key[e] = 0;
      iorb[e] = 1;
      coef[e] = 0.0;
      continue;
    }
    const int kk = (k * nw + (a - 1)) * nw + (int)(b - 1);
    tab[kk] = 1;
    key[e] = kk;
    iorb[e] = (int)io;
    coef[e] = mode == 0 ? co[e] : co[e] / c;
  }
}

// numbers the table's present (K, a, b) in table order (one block): the
// entry becomes its function index + 1, the function's YZK descriptor is
// written there, info[0] = the number of functions
__global__ void __launch_bounds__(1024) k_number_functions(int *__restrict__ tab, int size, int nw,
                                                            const int *__restrict__ MF, int n,
                                                            YDesc *__restrict__ yd, int *__restrict__ info) {
  __shared__ int part[1024];
  const int per = (size + 1023) / 1024, lo = threadIdx.x * per, hi = min(size, lo + per);
  int cnt = 0;
  for (int e = lo; e < hi; ++e) cnt += tab[e] != 0;
  part[threadIdx.x] = cnt;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {  // inclusive scan of the counts
    const int v = threadIdx.x >= (unsigned)off ? part[threadIdx.x - off] : 0;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  int f = part[threadIdx.x] - cnt;
  for (int e = lo; e < hi; ++e)
    if (tab[e]) {
      const int k = e / (nw * nw), a = (e / nw) % nw + 1, b = e % nw + 1;
      yd[f] = YDesc{k, a, b, min(MF[a], MF[b]), n, 0, 1};
      tab[e] = ++f;
    }
  if (threadIdx.x == 1023) info[0] = part[1023];
}

__global__ void k_term_functions(int64_t nt, const int *__restrict__ key, const int *__restrict__ tab,
                                 int *__restrict__ fidx) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nt; e += (int64_t)gridDim.x * blockDim.x)
    fidx[e] = tab[key[e]] - 1;
}

// DPBDT (lib9290/dpbdt.f90:39-99): 13-point derivative of orbital J at grid
// index i (1-based): the end rows from the 13 x 13 table, the interior by the
// antisymmetric 12-neighbour formula.
__device__ __forceinline__ void dpbdt_point(const double *PF, const double *QF, int ld, int J, const QuadConst &q,
                                            int i, double &hp, double &hq) {
  const int N = q.n;
  hp = 0.0;
  hq = 0.0;
  if (i <= 6) {
    for (int k = 1; k <= 13; ++k) hp = hp + q.A13[i - 1][k - 1] * pf(PF, ld, k, J);
    for (int k = 1; k <= 13; ++k) hq = hq + q.A13[i - 1][k - 1] * pf(QF, ld, k, J);
  } else if (i <= N - 6) {
    const double A1 = q.A13[6][0], A2 = q.A13[6][1], A3 = q.A13[6][2], A4 = q.A13[6][3], A5 = q.A13[6][4],
                 A6 = q.A13[6][5];
    hp = A1 * (pf(PF, ld, i - 6, J) - pf(PF, ld, i + 6, J)) + A2 * (pf(PF, ld, i - 5, J) - pf(PF, ld, i + 5, J)) +
         A3 * (pf(PF, ld, i - 4, J) - pf(PF, ld, i + 4, J)) + A4 * (pf(PF, ld, i - 3, J) - pf(PF, ld, i + 3, J)) +
         A5 * (pf(PF, ld, i - 2, J) - pf(PF, ld, i + 2, J)) + A6 * (pf(PF, ld, i - 1, J) - pf(PF, ld, i + 1, J));
    hq = A1 * (pf(QF, ld, i - 6, J) - pf(QF, ld, i + 6, J)) + A2 * (pf(QF, ld, i - 5, J) - pf(QF, ld, i + 5, J)) +
         A3 * (pf(QF, ld, i - 4, J) - pf(QF, ld, i + 4, J)) + A4 * (pf(QF, ld, i - 3, J) - pf(QF, ld, i + 3, J)) +
         A5 * (pf(QF, ld, i - 2, J) - pf(QF, ld, i + 2, J)) + A6 * (pf(QF, ld, i - 1, J) - pf(QF, ld, i + 1, J));
  } else {
    const int irow = i - N + 13;
    for (int k = 1; k <= 13; ++k) hp = hp + q.A13[irow - 1][k - 1] * pf(PF, ld, N - 13 + k, J);
    for (int k = 1; k <= 13; ++k) hq = hq + q.A13[irow - 1][k - 1] * pf(QF, ld, N - 13 + k, J);
  }
}

// DPBDT of orbital J at every grid index into dP, dQ (1-based), by the lanes
// of a warp
__device__ void dpbdt_warp(const double *PF, const double *QF, int ld, int J, const QuadConst &q, double *dP,
                           double *dQ, int lane) {
  for (int i = 1 + lane; i <= q.n; i += 32) {
    double hp, hq;
    dpbdt_point(PF, QF, ld, J, q, i, hp, hq);
    dP[i] = hp;
    dQ[i] = hq;
  }
}

// LAGCON (rmcdhf90/lagcon.f90:46-55): per multiplier in list order,
// XP(I) = XP(I) + WARI QF(I,M), XQ(I) = XQ(I) - WARI PF(I,M), WARI = WA R(I),
// I = 1..MF(M); mo[t] = M and wa[t] = ECV WB of the multipliers the host kept
// (those of pairs with this orbital, |WA| >= EPS). xp, xq 0-based.
// One job's LAGCON or DACON list (blockIdx.y selects the job): the entries'
// orbitals and weights, and the job's XP, XQ.
struct TermSeg {
  const int *idx;
  const double *w;
  double *xp, *xq;
  int nt;
};
__global__ void k_lagcon(const TermSeg *__restrict__ segs, int n, const int *__restrict__ MF,
                         const double *__restrict__ R, const double *__restrict__ PF, const double *__restrict__ QF,
                         int ld) {
  const TermSeg g = segs[blockIdx.y];
  const int nt = g.nt, *mo = g.idx;
  const double *wa = g.w;
  double *xp = g.xp, *xq = g.xq;
  for (int i = 1 + blockIdx.x * blockDim.x + threadIdx.x; i <= n; i += gridDim.x * blockDim.x) {
    double p = xp[i - 1], qv = xq[i - 1];
    for (int t = 0; t < nt; ++t) {
      const int M = mo[t];
      if (i > MF[M]) continue;
      const double wari = wa[t] * R[i];
      p = p + wari * pf(QF, ld, i, M);
      qv = qv - wari * pf(PF, ld, i, M);
    }
    xp[i - 1] = p;
    xq[i - 1] = qv;
  }
}

// DACON (rmcdhf90/dacon.f90:25-46): per entry of the list in order, with TA,
// TB = DPBDT(IORB) at the point, for I = 2..MF(IORB):
//   XP(I) += COEFF (TA RPORII + FK PFI - (2C R(I) + ZBCI) QFI),
//   XQ(I) += COEFF (TB RPORII - FK QFI + ZBCI PFI),
// RPORII = 1/(H RPOR(I)), ZBCI = ZZ(I)/C, FK = kappa(IORB). xp, xq 0-based.
__global__ void k_dacon(const TermSeg *__restrict__ segs, int n, const int *__restrict__ NAK,
                        const int *__restrict__ MF, const double *__restrict__ R, const double *__restrict__ RPOR,
                        const double *__restrict__ ZZ, const double *__restrict__ PF, const double *__restrict__ QF,
                        int ld, QuadConst q) {
  const TermSeg g = segs[blockIdx.y];
  const int nd = g.nt, *nda = g.idx;
  const double *da = g.w;
  double *xp = g.xp, *xq = g.xq;
  const double twoc = q.c + q.c;
  for (int i = 2 + blockIdx.x * blockDim.x + threadIdx.x; i <= n; i += gridDim.x * blockDim.x) {
    double p = xp[i - 1], qv = xq[i - 1];
    for (int t = 0; t < nd; ++t) {
      const int io = nda[t];
      if (i > MF[io]) continue;
      double ta, tb;
      dpbdt_point(PF, QF, ld, io, q, i, ta, tb);
      const double coeff = da[t], fk = (double)NAK[io];
      const double rporii = 1.0 / (q.h * RPOR[i]);
      const double pfi = pf(PF, ld, i, io), qfi = pf(QF, ld, i, io);
      const double zbci = ZZ[i] / q.c;
      p = p + coeff * (ta * rporii + fk * pfi - (twoc * R[i] + zbci) * qfi);
      qv = qv + coeff * (tb * rporii - fk * qfi + zbci * pfi);
    }
    xp[i - 1] = p;
    xq[i - 1] = qv;
  }
}

// SETLAG's quadrature (rmcdhf90/setlag.f90:177-219), one block per pair
// {J, M, case, MTP}: TA(I), I = 2..MTP, from the two orbitals' potentials
// (pot + 3 n slot: YP, XP, XQ, 0-based), then QUAD by thread 0. case 0: M
// fixed; 1: J fixed; 2: occupations more than 10 % apart; 3: otherwise.
__global__ void k_setlag_quad(const int4 *__restrict__ pj, const int2 *__restrict__ slots,
                              const double *__restrict__ pot, int n, const double *__restrict__ PF,
                              const double *__restrict__ QF, int ld, const double *__restrict__ R,
                              const double *__restrict__ RP, const double *__restrict__ RPOR, QuadConst q, int np,
                              double *__restrict__ TAall, double *__restrict__ result) {
  const int4 w = pj[blockIdx.x];
  const int J = w.x, M = w.y, cs = w.z, mtp = w.w;
  const double *ypj = pot + (size_t)3 * n * slots[blockIdx.x].x, *xpj = ypj + n, *xqj = xpj + n;
  const double *ypm = pot + (size_t)3 * n * slots[blockIdx.x].y, *xpm = ypm + n, *xqm = xpm + n;
  double *TA = TAall + (size_t)blockIdx.x * np;
  const double C = q.c;
  for (int i = threadIdx.x; i < np; i += blockDim.x) {
    double v = 0.0;
    if (i >= 2 && i <= mtp) {
      const double pj_ = pf(PF, ld, i, J), qj = pf(QF, ld, i, J), pm = pf(PF, ld, i, M), qm = pf(QF, ld, i, M);
      if (cs == 0)
        v = RPOR[i] * ((pm * xqj[i - 1] - qm * xpj[i - 1]) * C + (pm * pj_ + qm * qj) * ypj[i - 1]);
      else if (cs == 1)
        v = RPOR[i] * ((pj_ * xqm[i - 1] - qj * xpm[i - 1]) * C + (pj_ * pm + qj * qm) * ypm[i - 1]);
      else if (cs == 2)
        v = RPOR[i] * ((pm * xqj[i - 1] - qm * xpj[i - 1] - pj_ * xqm[i - 1] + qj * xpm[i - 1]) * C +
                       (ypj[i - 1] - ypm[i - 1]) * (pm * pj_ + qm * qj));
      else
        v = RPOR[i] * ((pm * xqj[i - 1] - qm * xpj[i - 1] + pj_ * xqm[i - 1] - qj * xpm[i - 1]) * C +
                       (ypj[i - 1] + ypm[i - 1]) * (pm * pj_ + qm * qj));
    }
    TA[i] = v;
  }
  __syncthreads();
  if (threadIdx.x == 0) result[blockIdx.x] = quad_seq(TA, mtp, R, RP, q);
}

// ECV from the pair's quadrature and RINTI (setlag.f90:184, 194, 205, 218)
__global__ void k_setlag_final(int np_, const int4 *__restrict__ pj, const double2 *__restrict__ ucf,
                               const double *__restrict__ result, const double *__restrict__ rijm,
                               double *__restrict__ ecv) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= np_) return;
  const double uj = ucf[t].x, um = ucf[t].y;
  switch (pj[t].z) {
    case 0: ecv[t] = (result[t] - rijm[t]) * uj; break;
    case 1: ecv[t] = (result[t] - rijm[t]) * um; break;
    case 2: ecv[t] = result[t] / (1.0 / uj - 1.0 / um); break;
    default: ecv[t] = (result[t] - 2.0 * rijm[t]) / (1.0 / uj + 1.0 / um); break;
  }
}

// RINTI (lib9290/rinti.f90:53-100) for a list of (J, K) pairs: one warp each.
__global__ void k_rinti(const int2 *__restrict__ jk, int npairs, int mode, const double *__restrict__ PF,
                        const double *__restrict__ QF, int ld, const int *__restrict__ MF,
                        const int *__restrict__ NAK, const double *__restrict__ R, const double *__restrict__ RP,
                        const double *__restrict__ RPOR, const double *__restrict__ ZZ, int np, QuadConst q,
                        double *__restrict__ out, const int *__restrict__ outidx) {
  extern __shared__ double sm[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int wpb = blockDim.x >> 5;
  double *dP = sm + (size_t)warp * 3 * np;
  double *dQ = dP + np;
  double *TA = dQ + np;
  for (int it = blockIdx.x * wpb + warp; it < npairs; it += gridDim.x * wpb) {
    const int J = jk[it].x, K = jk[it].y;
    const int mtp = max(MF[J], MF[K]);
    const double C = q.c;
    dpbdt_warp(PF, QF, ld, K, q, dP, dQ, lane);
    __syncwarp();
    for (int i = lane; i < np; i += 32) TA[i] = (i >= 2 && i <= mtp) ? pf(QF, ld, i, J) * dP[i] - pf(PF, ld, i, J) * dQ[i] : 0.0;
    __syncwarp();
    double piece1 = 0.0, piece2 = 0.0, piece3 = 0.0, piece4 = 0.0;
    if (lane == 0) {
      piece1 = quad_seq(TA, mtp, R, RP, q);
      piece1 = C * piece1 / q.h;
    }
    __syncwarp();
    for (int i = lane; i < np; i += 32)
      TA[i] = (i >= 2 && i <= mtp) ? RP[i] * pf(QF, ld, i, J) * pf(QF, ld, i, K) : 0.0;
    __syncwarp();
    if (lane == 0) {
      piece2 = quad_seq(TA, mtp, R, RP, q);
      piece2 = -2.0 * C * C * piece2;
    }
    __syncwarp();
    for (int i = lane; i < np; i += 32)
      TA[i] = (i >= 2 && i <= mtp)
                  ? RPOR[i] * (pf(PF, ld, i, J) * pf(QF, ld, i, K) + pf(QF, ld, i, J) * pf(PF, ld, i, K))
                  : 0.0;
    __syncwarp();
    if (lane == 0) {
      piece3 = quad_seq(TA, mtp, R, RP, q);
      piece3 = piece3 * C * (double)NAK[K];
    }
    __syncwarp();
    if (mode == 0) {
      for (int i = lane; i < np; i += 32)
        TA[i] = (i >= 2 && i <= mtp)
                    ? RPOR[i] * ZZ[i] * (pf(PF, ld, i, J) * pf(PF, ld, i, K) + pf(QF, ld, i, J) * pf(QF, ld, i, K))
                    : 0.0;
      __syncwarp();
      if (lane == 0) {
        piece4 = quad_seq(TA, mtp, R, RP, q);
        piece4 = -piece4;
      }
      __syncwarp();
    }
    if (lane == 0) out[outidx ? outidx[it] : it] = piece1 + piece2 + piece3 + piece4;
    __syncwarp();
  }
}

__global__ void k_fill(double *p, size_t n, double v) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) p[i] = v;
}

bool triangrk(int la, int k, int lb) {  // rci90/triangrk.f90:27-37
  if ((k + la + lb) % 2 != 0) return false;
  if (std::abs(la - lb) > k) return false;
  if (la + lb < k) return false;
  return true;
}

// The same YZK part 2 in three passes for many functions. Each step of
// k_ychain's recurrences adds an increment that does not depend on the
// chain, so the increments are formed by all SMs (k_yincr), the chains run
// only the dependent additions (k_ychain_sum), and Y = Z r^-k + W r^(k+1)
// is assembled per point (k_yassemble). The operations and their order are
// k_ychain's: the functions come out identical.
//   RZ(i) = C1 (T(i-4) + T(i)) + C2 (T(i-3) + T(i-1)) + C3 T(i-2), i >= 5,
//     added to Z as one term (Z = Z + RTMP);
//   RW(i) = the three terms C1 (TW(i) + TW(i+4)), C2 (TW(i+1) + TW(i+3)),
//     C3 TW(i+2), 2 <= i <= MTP, added to W one after the other
//     (WK = ((WK + t1) + t2) + t3, k_ychain's left-to-right sum).
__global__ void k_yincr(const YDesc *__restrict__ yd, int nf, const double *__restrict__ TZ,
                        const double *__restrict__ TW, int np, QuadConst q, double *__restrict__ RZ,
                        double *__restrict__ RW) {
  const int f = blockIdx.y;
  if (f >= nf) return;
  const int MTP = yd[f].mtp;
  const double *T = TZ + (size_t)f * np, *Tw = TW + (size_t)f * np;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < np; i += gridDim.x * blockDim.x) {
    double rz = 0.0, w1 = 0.0, w2 = 0.0, w3 = 0.0;
    if (i >= 5) rz = q.C1 * (T[i - 4] + T[i]) + q.C2 * (T[i - 3] + T[i - 1]) + q.C3 * T[i - 2];
    if (i >= 2 && i <= MTP) {
      w1 = q.C1 * (Tw[i] + Tw[i + 4]);
      w2 = q.C2 * (Tw[i + 1] + Tw[i + 3]);
      w3 = q.C3 * Tw[i + 2];
    }
    RZ[(size_t)f * np + i] = rz;
    double *rw = RW + ((size_t)f * np + i) * 3;
    rw[0] = w1;
    rw[1] = w2;
    rw[2] = w3;
  }
}

// acc = acc + P(o_j, 0) + ... + P(o_j, NT-1) (left to right), O(o_j) = acc
// for j = 0 .. cnt-1 in order, o_j = start + step j, P holding NT terms per
// point; the loads of group g + 1 are issued before the additions of group g
template <int NT, int A>
__device__ __forceinline__ double ychain_run(double acc, const double *__restrict__ P, double *__restrict__ O,
                                             int start, int step, int cnt) {
  double cur[A][NT], nxt[A][NT];
#pragma unroll
  for (int u = 0; u < A; ++u)
#pragma unroll
    for (int v = 0; v < NT; ++v) cur[u][v] = (u < cnt) ? P[(size_t)(start + step * u) * NT + v] : 0.0;
  int j = 0;
  for (; j + A <= cnt; j += A) {
    const int j1 = j + A;
#pragma unroll
    for (int u = 0; u < A; ++u)
#pragma unroll
      for (int v = 0; v < NT; ++v) nxt[u][v] = (j1 + u < cnt) ? P[(size_t)(start + step * (j1 + u)) * NT + v] : 0.0;
#pragma unroll
    for (int u = 0; u < A; ++u) {
#pragma unroll
      for (int v = 0; v < NT; ++v) acc = acc + cur[u][v];
      O[start + step * (j + u)] = acc;
    }
#pragma unroll
    for (int u = 0; u < A; ++u)
#pragma unroll
      for (int v = 0; v < NT; ++v) cur[u][v] = nxt[u][v];
  }
#pragma unroll
  for (int u = 0; u < A; ++u)
    if (j + u < cnt) {
#pragma unroll
      for (int v = 0; v < NT; ++v) acc = acc + cur[u][v];
      O[start + step * (j + u)] = acc;
    }
  return acc;
}
// the chains' additions (Z: 16 points loaded ahead, W: 8); writes Z into Y,
// W into W, each chain's K = 0 correction DIF and the function's asymptotic
// value ZKLIM
__global__ void k_ychain_sum(const YDesc *__restrict__ yd, int nf, const double *__restrict__ TZ,
                             const double *__restrict__ RZ, const double *__restrict__ RW, int np, QuadConst q,
                             double *__restrict__ Y, double *__restrict__ W, double *__restrict__ dif_out,
                             double *__restrict__ zk_out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int f = t >> 2, c = t & 3;
  const bool active = f < nf;
  const YDesc y = active ? yd[f] : yd[0];
  const int K = y.k, MTP = y.mtp, MTPP3 = MTP + 3, N = q.n;
  const size_t base = (size_t)(active ? f : 0) * np;
  const double *T = TZ + base, *Rz = RZ + base, *Rw = RW + 3 * base;
  double *Yf = Y + base, *Wf = W + base;
  const int s = c + 2;  // chain start: 2, 3, 4, 5
  double z = 0.0;
  if (active) {
    if (s <= 4) {
      double sum = 0.0;
      for (int kk = 2; kk <= 5; ++kk) sum = sum + q.CNC5C[kk - 2][s - 2] * T[kk];
      z = sum;
    } else {  // ZK(5) = ZK(1) + RTMP(5), ZK(1) = 0
      z = 0.0 + Rz[5];
    }
    Yf[s] = z;
    // the points s + 4, s + 8, ... <= MTP + 3
    const int cnt = (MTPP3 >= s + 4) ? (MTPP3 - s - 4) / 4 + 1 : 0;
    z = ychain_run<1, 16>(z, Rz, Yf, s + 4, 4, cnt);
  }
  const int owner = (MTPP3 - 2) & 3;
  const double z_top = __shfl_sync(0xffffffffu, z, (threadIdx.x & ~3) + owner);
  if (!active) return;
  double zklim, dif = 0.0;
  if (K == 0) {
    zklim = (y.b == y.d) ? 1.0 : 0.0;
    const double d0 = z - zklim;
    if (fabs(d0) > q.accy) dif = d0;
  } else {
    zklim = z_top;
  }
  dif_out[(size_t)f * 4 + c] = dif;
  if (c == 0) zk_out[f] = zklim;
  // W from the top of this chain's points with i <= min(N, MTP) down to s
  const int lim = min(N, MTP);
  if (lim < s) return;
  const int cnt = (lim - s) / 4 + 1;  // the points s + 4 (cnt - 1), ..., s + 4, s
  ychain_run<3, 8>(0.0, Rw, Wf, s + 4 * (cnt - 1), -4, cnt);
}

__global__ void k_yassemble(const YDesc *__restrict__ yd, int nf, const double *__restrict__ R,
                            const double *__restrict__ pw, int np, QuadConst q, const double *__restrict__ dif,
                            const double *__restrict__ zk, const double *__restrict__ W, double *__restrict__ Y) {
  const int f = blockIdx.y;
  if (f >= nf) return;
  const YDesc y = yd[f];
  const int K = y.k, MTP = y.mtp, MTPP3 = MTP + 3, N = q.n;
  const double zklim = zk[f];
  const double *RTTKM = pw + (size_t)(1 * (KLIMIT + 1) + K) * np;
  const double *RTTK1 = pw + (size_t)(2 * (KLIMIT + 1) + K) * np;
  const double *Wf = W + (size_t)f * np;
  double *Yf = Y + (size_t)f * np;
  for (int i = 2 + blockIdx.x * blockDim.x + threadIdx.x; i < np; i += gridDim.x * blockDim.x) {
    double yv = 0.0;
    if (i <= N) {
      double zf;
      if (K == 0) {
        if (i <= MTPP3) {
          const double d = dif[(size_t)f * 4 + ((i - 2) & 3)];
          zf = (d != 0.0) ? Yf[i] - d : Yf[i];
        } else {
          zf = zklim;
        }
      } else {
        zf = (i <= MTPP3) ? Yf[i] * RTTKM[i] : zklim * RTTKM[i];
      }
      double wkf = 0.0;
      if (i <= MTP) {
        const double wk = Wf[i];
        wkf = (K == 0) ? wk * R[i] : wk * RTTK1[i];
      }
      yv = zf + wkf;
      if (i > y.mtpb) yv = 0.0;
    }
    Yf[i] = yv;
  }
}

// build_y takes the three-pass form from this many functions on
constexpr int YSPLIT_MIN = 32;

// Builds Y functions for the descriptor list on the device: TZ/TW scratch
// then the chains. Y must hold nf * np doubles.
int build_y(gg_ctx *ctx, const YDesc *d_yd, int nf, double *dY, DBuf<double> &scratch) {
  Grid &g = ctx->grid;
  Orbitals &o = ctx->orb;
  const int np = g.np;
  const bool split = nf >= YSPLIT_MIN;
  GG_TRY(scratch.alloc(split ? (size_t)6 * nf * np + (size_t)5 * nf : (size_t)2 * nf * np));
  double *TZ = scratch.p, *TW = scratch.p + (size_t)nf * np;
  dim3 grid1((np + 127) / 128, nf);
  k_ytemp<<<grid1, 128, 0, ctx->stream>>>(d_yd, nf, o.dPF.p, o.dQF.p, o.ld, g.dRP.p, g.dPow.p, np, TZ, TW); ::gg::note_launch();
  GG_CUDA(cudaGetLastError());
  GG_CUDA(cudaMemsetAsync(dY, 0, (size_t)nf * np * sizeof(double), ctx->stream));
  const int nthr = nf * 4;
  if (!split) {
    k_ychain<<<(nthr + 127) / 128, 128, 0, ctx->stream>>>(d_yd, nf, TZ, TW, g.dR.p, g.dPow.p, np, g.q, dY);
    ::gg::note_launch();
  } else {
    // RZ: one term per point; RW: three terms per point; DIF per chain; ZKLIM
    double *RZ = TW + (size_t)nf * np, *RW = RZ + (size_t)nf * np, *dif = RW + (size_t)3 * nf * np;
    double *zk = dif + 4 * nf;
    k_yincr<<<grid1, 128, 0, ctx->stream>>>(d_yd, nf, TZ, TW, np, g.q, RZ, RW);
    // W goes where TW was: k_yincr was its last reader
    k_ychain_sum<<<(nthr + 127) / 128, 128, 0, ctx->stream>>>(d_yd, nf, TZ, RZ, RW, np, g.q, dY, TW, dif, zk);
    k_yassemble<<<grid1, 128, 0, ctx->stream>>>(d_yd, nf, g.dR.p, g.dPow.p, np, g.q, dif, zk, TW, dY);
    ::gg::note_launch();
    ::gg::note_launch();
    ::gg::note_launch();
  }
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

template <class T> int upload(DBuf<T> &b, const std::vector<T> &h, cudaStream_t s) {
  GG_TRY(b.alloc(h.size()));
  if (!h.empty()) GG_CUDA(cudaMemcpyAsync(b.p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, s));
  return GG_OK;
}

}  // namespace

}  // namespace gg

using namespace gg;

extern "C" {

// The part of GENINTRK that depends only on the orbitals' l and j and on
// kmax: Y functions, pairs, INDTEIRK and KSTART, the contraction tiles of
// both forms, and their device copies. Built once per orbital set.
static int rk_build_structure(gg_ctx *ctx, int kloop, RkCache &C) {
  Grid &g = ctx->grid;
  Orbitals &o = ctx->orb;
  RkTable &rk = ctx->rk;
  const int NW = o.nw, KEY = NW + 1;
  // Y functions, ordered (k, b, d): D(b,k) = {d >= b : TRIANGRK(l_b, k, l_d)}
  std::vector<YDesc> &yd = C.yd;
  yd.clear();
  std::vector<std::vector<int>> cs(kloop + 1, std::vector<int>(NW + 2, -1)), nd(kloop + 1, std::vector<int>(NW + 2, 0));
  std::vector<int> &kend = C.kend;
  kend.assign(kloop + 1, 0);
  for (int k = 0; k <= kloop; ++k) {
    for (int b = 1; b <= NW; ++b) {
      cs[k][b] = (int)yd.size();
      for (int d = b; d <= NW; ++d)
        if (triangrk(o.nkl[b], k, o.nkl[d])) {
          YDesc y;
          y.k = k;
          y.b = b;
          y.d = d;
          y.mtp = std::min(o.mf[b], o.mf[d]);
          y.mtpb = (k == 0 && b == d) ? g.n : y.mtp;
          y.cs = cs[k][b];
          y.nd = 0;
          yd.push_back(y);
        }
      nd[k][b] = (int)yd.size() - cs[k][b];
      for (int f = cs[k][b]; f < (int)yd.size(); ++f) yd[f].nd = nd[k][b];
    }
    kend[k] = (int)yd.size();
  }
  // pair list for the A rows (a <= c), k-independent
  std::vector<int2> &pairs = C.pairs;
  pairs.clear();
  std::vector<int> pidx((size_t)(NW + 1) * (NW + 1), -1);
  for (int a = 1; a <= NW; ++a)
    for (int c = a; c <= NW; ++c) {
      pidx[(size_t)a * (NW + 1) + c] = (int)pairs.size();
      pairs.push_back(make_int2(a, c));
    }
  // INDTEIRK and KSTART in GENINTRK order (rci90/genintrk.f90:64-86) and the
  // contraction problems (k, a); each problem's entries are contiguous.
  rk.kstart.assign(kloop + 2, 0);
  rk.hInd.clear();
  std::vector<RkTile> &tiles = C.tiles;
  std::vector<int> &rowpair = C.rowpair;
  std::vector<TcRow> &tcrows = C.tcrows;
  tiles.clear();
  rowpair.clear();
  tcrows.clear();
  std::vector<int> tcr0(kloop + 2, 0);  // first tcrows entry of each k
  int64_t N = 0;
  rk.kstart[0] = 1;
  for (int k = 0; k <= kloop; ++k) {
    tcr0[k] = (int)tcrows.size();
    for (int a = 1; a <= NW; ++a) {
      const int ncA = nd[k][a];
      if (ncA == 0) continue;
      const int c0 = cs[k][a], c1 = kend[k];
      const long long base = N;
      // integer index list in reference order
      for (int b = a; b <= NW; ++b)
        for (int ic = 0; ic < ncA; ++ic) {
          const int c = yd[cs[k][a] + ic].d;
          for (int id = 0; id < nd[k][b]; ++id) {
            const int d = yd[cs[k][b] + id].d;
            rk.hInd.push_back(((a * KEY + b) * KEY + c) * KEY + d);
          }
        }
      N = (int64_t)rk.hInd.size();
      const int rp0 = (int)rowpair.size();
      for (int ic = 0; ic < ncA; ++ic) rowpair.push_back(pidx[(size_t)a * (NW + 1) + yd[cs[k][a] + ic].d]);
      for (int r0 = 0; r0 < ncA; r0 += BM)
        for (int cc = c0; cc < c1; cc += BN) {
          RkTile t;
          t.k = k;
          t.a = a;
          t.ncA = ncA;
          t.r0 = r0;
          t.rowpair0 = rp0;
          t.cs_a = c0;
          t.c0 = cc;
          t.c1 = std::min(c1, cc + BN);
          t.base = base;
          tiles.push_back(t);
        }
      // rows of the tcgen05 form (all problems of one k, in order)
      for (int ic = 0; ic < ncA; ++ic) tcrows.push_back(TcRow{rowpair[rp0 + ic], a, ic, ncA, c0, base});
    }
    rk.kstart[k + 1] = (int32_t)(N + 1);
  }
  tcr0[kloop + 1] = (int)tcrows.size();
  if (N > INT32_MAX) return fail(GG_ERR_RANGE, "genintrk: table too large");
  rk.n = N;
  C.nf = (int)yd.size();
  C.npairs = (int)pairs.size();
  const int nf = C.nf;
  {
  std::vector<int> fg0(kloop + 1), pg0(kloop + 1), kbeg(kloop + 1);
  std::vector<int> &yslot = C.yslot, &aslot = C.aslot;
  std::vector<TcTile> &tct = C.tct;
  yslot.clear();
  aslot.clear();
  tct.clear();
  C.tcs_nch = -1;  // the split-K list follows tct
  for (int k = 0; k <= kloop; ++k) {
    kbeg[k] = (k == 0) ? 0 : kend[k - 1];
    const int F = kend[k] - kbeg[k], Rk = tcr0[k + 1] - tcr0[k];
    const int nft = (F + TC_M - 1) / TC_M, npt = (Rk + TC_N - 1) / TC_N;
    fg0[k] = (int)(yslot.size() / TC_M);
    pg0[k] = (int)(aslot.size() / TC_N);
    for (int ft = 0; ft < nft; ++ft)
      for (int m = 0; m < TC_M; ++m) {
        const int f = kbeg[k] + ft * TC_M + m;
        yslot.push_back(f < kend[k] ? f : -1);
      }
    for (int pt = 0; pt < npt; ++pt)
      for (int n = 0; n < TC_N; ++n) {
        const int r = tcr0[k] + pt * TC_N + n;
        aslot.push_back(r < tcr0[k + 1] ? tcrows[r].p : -1);
      }
    for (int pt = 0; pt < npt; ++pt)
      for (int ft = 0; ft < nft; ++ft) {
        TcTile t;
        t.k = k;
        t.fg = fg0[k] + ft;
        t.pg = pg0[k] + pt;
        t.f0 = kbeg[k] + ft * TC_M;
        t.fn = std::min(TC_M, F - ft * TC_M);
        t.r0 = tcr0[k] + pt * TC_N;
        t.rn = std::min(TC_N, Rk - pt * TC_N);
        // rows are ordered by a, so the first row has the smallest cs_a:
        // no needed entry when every function of the tile is below it
        if (t.f0 + t.fn - 1 < tcrows[t.r0].cs_a) continue;
        tct.push_back(t);
      }
  }
    std::vector<int> &fidx = C.fidx;
    fidx.assign((size_t)(kloop + 1) * KEY * KEY, -1);
    for (int f = 0; f < nf; ++f) fidx[((size_t)yd[f].k * KEY + yd[f].b) * KEY + yd[f].d] = f;
  }
  GG_TRY(upload(C.dPairs, pairs, ctx->stream));
  GG_TRY(upload(C.dTiles, tiles, ctx->stream));
  GG_TRY(upload(C.dRowpair, rowpair, ctx->stream));
  GG_TRY(upload(C.dTct, C.tct, ctx->stream));
  GG_TRY(upload(C.dTcr, tcrows, ctx->stream));
  GG_TRY(upload(C.dYslot, C.yslot, ctx->stream));
  GG_TRY(upload(C.dAslot, C.aslot, ctx->stream));
  GG_TRY(upload(C.dFidx, C.fidx, ctx->stream));
  GG_TRY(upload(C.dKst, rk.kstart, ctx->stream));
  GG_TRY(rk.dInd.alloc(std::max<int64_t>(N, 1)));
  if (N > 0)
    GG_CUDA(cudaMemcpyAsync(rk.dInd.p, rk.hInd.data(), N * sizeof(int32_t), cudaMemcpyHostToDevice, ctx->stream));
  GG_CUDA(cudaStreamSynchronize(ctx->stream));
  return GG_OK;
}

int gg_genintrk(gg_ctx *ctx, int kmax, int precision, int64_t *n_out, int *j2max_out) {
  GG_TRY(ensure_orbitals(ctx));
  if (precision != GG_FP64 && precision != GG_SPLIT) return fail(GG_ERR_ARG, "gg_genintrk: unknown precision");
  GG_CUDA(cudaSetDevice(ctx->device));
  Grid &g = ctx->grid;
  Orbitals &o = ctx->orb;
  RkTable &rk = ctx->rk;
  const int NW = o.nw, KEY = NW + 1;
  int j2max = o.nkj[1];
  for (int i = 2; i <= NW; ++i) j2max = std::max(j2max, o.nkj[i]);
  if (j2max > KLIMIT) return fail(GG_ERR_ARG, "genintrk: KMAX too small");
  const int kloop = kmax < 0 ? j2max : kmax;
  if (kloop > KLIMIT) return fail(GG_ERR_ARG, "genintrk: k beyond KLIMIT = 20");
  GG_TRY(timer_start(ctx));
  // the index structure is rebuilt only when the orbital set's l, j or kmax change
  std::vector<int> key{NW, kloop};
  for (int i = 1; i <= NW; ++i) {
    key.push_back(o.nkl[i]);
    key.push_back(o.nkj[i]);
  }
  if (!rk.cache) rk.cache = new RkCache();
  RkCache &C = *rk.cache;
  if (C.key != key) {
    C.key.clear();  // not valid until built
    rk.valid = false;
    GG_TRY(rk_build_structure(ctx, kloop, C));
    C.key = key;
  }
  const int64_t N = rk.n;
  rk.valid = false;  // until this call's table is complete
  rk.kloop = kloop;
  rk.j2max = j2max;
  // per call: each Y function's MTP from the current orbital extents
  for (YDesc &y : C.yd) {
    y.mtp = std::min(o.mf[y.b], o.mf[y.d]);
    y.mtpb = (y.k == 0 && y.b == y.d) ? g.n : y.mtp;
  }
  GG_TRY(upload(C.dYd, C.yd, ctx->stream));
  const int nf = C.nf, npairs = C.npairs;
  const int np = g.np;
  const int KC = ((g.n + 1 + KC_TILE - 1) / KC_TILE) * KC_TILE;
  if (KC > np) return fail(GG_ERR_ARG, "genintrk: grid padding too small");
  const std::vector<RkTile> &tiles = C.tiles;
  GG_TRY(rk.dVal.alloc(std::max<int64_t>(N, 1)));
  GG_TRY(C.dY.alloc((size_t)std::max(nf, 1) * np));
  if (nf > 0) GG_TRY(build_y(ctx, C.dYd.p, nf, C.dY.p, C.scratch));
  GG_TRY(C.dA.alloc((size_t)std::max(npairs, 1) * KC));
  if (npairs > 0) {
    dim3 gr((KC + 127) / 128, npairs);
    k_apairs<<<gr, 128, 0, ctx->stream>>>(C.dPairs.p, npairs, o.dPF.p, o.dQF.p, o.ld, o.dMF.p, g.dRPOR.p, KC, g.q,
                                          C.dA.p);
    ::gg::note_launch();
    GG_CUDA(cudaGetLastError());
  }
  GG_TRY(C.dFb.alloc(std::max<int64_t>(N, 1)));
  GG_TRY(C.dNfb.alloc(3));  // [0] fallback count, [1] position error flag, [2] tensor-core wait timed out
  GG_CUDA(cudaMemsetAsync(C.dNfb.p, 0, 3 * sizeof(int), ctx->stream));
  if (!tiles.empty() && precision == GG_SPLIT) {
    // tensor-core contraction on Ozaki slices of A and Y
    const int KP = (KC + 31) / 32 * 32;
    GG_TRY(C.dEA.alloc(npairs + 1));
    GG_TRY(C.dEY.alloc(nf + 1));
    {
      // tcgen05: the slices written into the tile blocks, the raw GEMM parts
      // at their positions, then the head terms
      const int nch = KP / TC_KC;
      GG_TRY(C.dYt.alloc(std::max<size_t>(1, C.yslot.size() / TC_M * nch * TC_YBLK)));
      GG_TRY(C.dAt.alloc(std::max<size_t>(1, C.aslot.size() / TC_N * nch * TC_ABLK)));
      if (!C.yslot.empty()) {
        k_oz_tile<TC_M><<<(unsigned)C.yslot.size(), 128, 0, ctx->stream>>>(C.dY.p, np, KC, nch, C.dYslot.p, C.dEY.p,
                                                                          C.dYt.p);
        ::gg::note_launch();
      }
      if (!C.aslot.empty()) {
        k_oz_tile<TC_N><<<(unsigned)C.aslot.size(), 128, 0, ctx->stream>>>(C.dA.p, KC, KC, nch, C.dAslot.p, C.dEA.p,
                                                                          C.dAt.p);
        ::gg::note_launch();
      }
      static bool attr = false;
      if (!attr) {
        GG_CUDA(cudaFuncSetAttribute(k_rk_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TC_SMEM));
        attr = true;
      }
      // split-K: one CTA per SM holds a tile (shared memory), so with
      // fewer tiles than SMs each tile's grid chunks are cut into nsplit
      // ranges of at least TC_FLUSH chunks, whose partial sums
      // k_rk_finish_all adds in order
      int nsplit = 1;
      if (!C.tct.empty()) {
        const int want = (ctx->sms + (int)C.tct.size() - 1) / (int)C.tct.size();
        nsplit = std::max(1, std::min(want, nch / TC_FLUSH));
      }
      if (C.tcs_nch != nch || C.tcs_split != nsplit) {
        C.tcs.clear();
        for (const TcTile &t : C.tct)
          for (int sp = 0; sp < nsplit; ++sp) {
            TcTile u = t;
            u.c0 = (int)((long long)nch * sp / nsplit);
            u.c1 = (int)((long long)nch * (sp + 1) / nsplit);
            u.s = sp;
            C.tcs.push_back(u);
          }
        GG_TRY(upload(C.dTcs, C.tcs, ctx->stream));
        C.tcs_nch = nch;
        C.tcs_split = nsplit;
      }
      double *parts = rk.dVal.p;
      if (nsplit > 1) {
        GG_TRY(C.dParts.alloc((size_t)nsplit * std::max<int64_t>(N, 1)));
        parts = C.dParts.p;
      }
      if (!C.tcs.empty()) {
        k_rk_tc<<<(unsigned)C.tcs.size(), TC_THREADS, TC_SMEM, ctx->stream>>>(
            C.dTcs.p, C.dTcr.p, C.dYt.p, C.dAt.p, nch, C.dEA.p, C.dEY.p, C.dYd.p, parts, (long long)N,
            C.dNfb.p + 1, ctx->test_stall_tile);
        ctx->test_stall_tile = -1;  // one call only
        ::gg::note_launch();
      }
      ctx->stats[25] = nsplit;
      GG_CUDA(cudaGetLastError());
      const unsigned fb_blocks = (unsigned)std::min<long long>((N + 255) / 256, 8LL * ctx->sms);
      k_rk_finish_all<<<std::max(1u, fb_blocks), 256, 0, ctx->stream>>>(
          rk.dInd.p, (long long)N, C.dKst.p, kloop, KEY, C.dFidx.p, C.dYd.p, C.dY.p, np, o.dPF.p, o.dQF.p, o.ld,
          o.dMF.p, g.dR.p, g.dRP.p, g.dRPOR.p, g.dHead.p, g.q, rk.dVal.p, C.dFb.p, C.dNfb.p, parts, nsplit);
      ::gg::note_launch();
    }
    GG_CUDA(cudaGetLastError());
  } else if (!tiles.empty()) {
    k_rk_gemm<<<(unsigned)tiles.size(), 256, 0, ctx->stream>>>(C.dTiles.p, C.dRowpair.p, C.dPairs.p, C.dA.p, C.dY.p,
                                                              C.dYd.p, KC, np, o.dPF.p, o.dQF.p, o.ld, o.dMF.p,
                                                              g.dR.p, g.dRP.p, g.dRPOR.p, g.dHead.p, g.q, rk.dVal.p,
                                                              (long long)N, C.dFb.p, C.dNfb.p);
    ::gg::note_launch();
    GG_CUDA(cudaGetLastError());
  }
  int hfb[3] = {0, 0, 0};
  GG_CUDA(cudaMemcpyAsync(hfb, C.dNfb.p, 3 * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  GG_CUDA(cudaStreamSynchronize(ctx->stream));
  if (hfb[1]) return fail(GG_ERR_STATE, "genintrk: contraction produced a table position out of range");
  if (hfb[2] == 1)
    return fail(GG_ERR_TIMEOUT, "genintrk: a tensor-core tile timed out waiting for its copies or MMAs (drained; "
                                "the table is not valid)");
  if (hfb[2] > 1)
    return fail(GG_ERR_TIMEOUT, "genintrk: a tensor-core tile timed out and its copies or MMAs did not drain");
  const int nfb = hfb[0];
  ctx->stats[20] = nfb;
  if (nfb > 0) {
    const int wpb = 16;  // warps per block: an item each, their head terms by warp 0
    const int blocks = std::min((nfb + wpb - 1) / wpb, 4 * ctx->sms);
    k_quad_table<<<blocks, 32 * wpb, 0, ctx->stream>>>(C.dFb.p, C.dNfb.p, nfb, C.dY.p, np, o.dPF.p, o.dQF.p, o.ld,
                                                       g.dR.p, g.dRP.p, g.dRPOR.p, g.dHead.p, g.q, rk.dVal.p);
    ::gg::note_launch();
    GG_CUDA(cudaGetLastError());
  }
  double ms = 0;
  GG_TRY(timer_stop(ctx, &ms));
  ctx->stats[0] = ms;
  rk.valid = true;
  if (n_out) *n_out = N;
  if (j2max_out) *j2max_out = j2max;
  return GG_OK;
}

int gg_get_rk_table(gg_ctx *ctx, int32_t *indteirk, double *valteirk, int32_t *kstart) {
  if (!ctx || !ctx->rk.valid) return fail(GG_ERR_STATE, "gg_get_rk_table: no table (call gg_genintrk)");
  GG_CUDA(cudaSetDevice(ctx->device));
  const RkTable &rk = ctx->rk;
  if (indteirk && rk.n) std::memcpy(indteirk, rk.hInd.data(), rk.n * sizeof(int32_t));
  if (valteirk && rk.n) {
    GG_CUDA(cudaMemcpyAsync(valteirk, rk.dVal.p, rk.n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    GG_CUDA(cudaStreamSynchronize(ctx->stream));
  }
  if (kstart) std::memcpy(kstart, rk.kstart.data(), rk.kstart.size() * sizeof(int32_t));
  return GG_OK;
}

int gg_rkintc(gg_ctx *ctx, int ia, int ib, int ic, int id, int k, double *tegral) {
  if (!ctx || !ctx->rk.valid) return fail(GG_ERR_STATE, "gg_rkintc: no table");
  const RkTable &rk = ctx->rk;
  const int nw = ctx->orb.nw, KEY = nw + 1;
  if (k < 0 || k > rk.kloop || ia < 1 || ib < 1 || ic < 1 || id < 1 || ia > nw || ib > nw || ic > nw || id > nw)
    return fail(GG_ERR_ARG, "gg_rkintc: index out of range");
  // canonical order (rci90/rkintc.f90:45-62)
  if (ia > ic) std::swap(ia, ic);
  if (ib > id) std::swap(ib, id);
  if (ia > ib) {
    std::swap(ia, ib);
    std::swap(ic, id);
  }
  const int32_t index = ((ia * KEY + ib) * KEY + ic) * KEY + id;
  int64_t jl = rk.kstart[k], ju = rk.kstart[k + 1] - 1;
  if (ju < jl || index < rk.hInd[jl - 1] || index > rk.hInd[ju - 1])
    return fail(GG_ERR_NOTFOUND, "Something wrong in rkintc");
  while (ju - jl > 1) {
    const int64_t jm = (ju + jl) / 2;
    if (rk.hInd[jm - 1] > index)
      ju = jm;
    else
      jl = jm;
  }
  int64_t loc;
  if (index == rk.hInd[ju - 1])
    loc = ju;
  else if (index == rk.hInd[jl - 1])
    loc = jl;
  else
    return fail(GG_ERR_NOTFOUND, "Rkintc Integral not found");
  GG_CUDA(cudaSetDevice(ctx->device));
  GG_CUDA(cudaMemcpyAsync(tegral, rk.dVal.p + (loc - 1), sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  GG_CUDA(cudaStreamSynchronize(ctx->stream));
  return GG_OK;
}

int gg_slater(gg_ctx *ctx, int ia, int ib, int ic, int id, int k, double *out) {
  GG_TRY(ensure_orbitals(ctx));
  Orbitals &o = ctx->orb;
  Grid &g = ctx->grid;
  const int nw = o.nw;
  if (!out || k < 0 || k > KLIMIT || ia < 1 || ib < 1 || ic < 1 || id < 1 || ia > nw || ib > nw || ic > nw ||
      id > nw)
    return fail(GG_ERR_ARG, "gg_slater: bad arguments");
  GG_CUDA(cudaSetDevice(ctx->device));
  YDesc y;
  y.k = k;
  y.b = ib;
  y.d = id;
  y.mtp = std::min(o.mf[ib], o.mf[id]);
  y.mtpb = (k == 0 && ib == id) ? g.n : y.mtp;
  y.cs = 0;
  y.nd = 1;
  // SLATER's integration limit (slater.f90:56-60)
  QuadItem it;
  it.a = ia;
  it.c = ic;
  it.f = 0;
  it.mtp = (k == 0 && ib == id) ? std::min(o.mf[ia], o.mf[ic]) : std::min(std::min(y.mtp, o.mf[ia]), o.mf[ic]);
  it.pos = 0;
  std::vector<YDesc> hy{y};
  std::vector<QuadItem> hi{it};
  DBuf<YDesc> dy;
  DBuf<QuadItem> di;
  DBuf<double> dY, scratch, dout;
  GG_TRY(upload(dy, hy, ctx->stream));
  GG_TRY(upload(di, hi, ctx->stream));
  GG_TRY(dY.alloc(g.np));
  GG_TRY(dout.alloc(1));
  GG_TRY(build_y(ctx, dy.p, 1, dY.p, scratch));
  k_quad_items<<<1, 32, g.np * sizeof(double), ctx->stream>>>(di.p, nullptr, 1, dY.p, g.np, o.dPF.p, o.dQF.p, o.ld,
                                                             g.dR.p, g.dRP.p, g.dRPOR.p, g.q, dout.p); ::gg::note_launch();
  GG_CUDA(cudaGetLastError());
  GG_CUDA(cudaMemcpyAsync(out, dout.p, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  GG_CUDA(cudaStreamSynchronize(ctx->stream));
  return GG_OK;
}

}  // extern "C"


extern "C" {
static int run_rinti(gg_ctx *ctx, const std::vector<int2> &jk, int mode, double *dOut, const std::vector<int> *outidx);
}

// YPOT / XPOT on the device: the list's distinct Y^k_ab (every grid point,
// YZK's TB), then k_potential. A list as the caller passed it: YPOT labels
// NYA = (IOY2 KEY + IOY1) KEY + K, XPOT labels NXA = ((IORB KEY + IOY2) KEY +
// IOY1) KEY + K, and their coefficients.
struct RawList {
  const int32_t *lab = nullptr;
  const double *co = nullptr;
  int n = 0;
};

static int raw_list(int ncof, const int32_t *lab, const double *co, RawList &r) {
  if (ncof < 0 || (ncof > 0 && (!lab || !co))) return fail(GG_ERR_ARG, "potential: bad coefficient list");
  r = RawList{lab, co, ncof};
  return GG_OK;
}

// XPOT lists at least this long take the two-pass form (products by all
// SMs, then the per-point sums, all such lists of one call together)
constexpr int XPOT_SPLIT = 512;

// One orbital's potentials on the device: YP, XP, XQ (N each, 0-based) at
// out, out + n, out + 2 n.
struct PotJob {
  RawList y, x;
  std::vector<int> nda;
  std::vector<double> da;
  std::vector<int> lag_m;      // LAGCON: the pairs' other orbitals
  std::vector<double> lag_wa;  // and their weights ECV WB
};

// the jobs' YPOT, XPOT, then LAGCON and DACON, into dPot (3 n per job): all
// Y functions of all lists built once
static int run_potentials(gg_ctx *ctx, const std::vector<PotJob> &jobs, DBuf<double> &dPot) {
  Orbitals &o = ctx->orb;
  Grid &g = ctx->grid;
  cudaStream_t s = ctx->stream;
  const int n = g.n, nw = o.nw;
  // every job's YPOT list, then every job's XPOT list, as the caller passed
  // them, staged in pinned memory and copied to the device in one transfer
  std::vector<size_t> oy(jobs.size()), ox(jobs.size());
  size_t T = 0;
  for (size_t j = 0; j < jobs.size(); ++j) oy[j] = T, T += (size_t)jobs[j].y.n;
  const size_t TY = T;
  for (size_t j = 0; j < jobs.size(); ++j) ox[j] = T, T += (size_t)jobs[j].x.n;
  const size_t lab_bytes = (T * sizeof(int32_t) + 15) / 16 * 16, need = lab_bytes + T * sizeof(double);
  if (need > ctx->pot_stage_bytes) {
    void *hp = nullptr;
    GG_CUDA(cudaHostAlloc(&hp, need + need / 4, cudaHostAllocDefault));
    note_alloc();
    ctx->pot_stage = std::shared_ptr<void>(hp, [](void *q) { cudaFreeHost(q); });
    ctx->pot_stage_bytes = need + need / 4;
  }
  char *stage = static_cast<char *>(ctx->pot_stage.get());
  int32_t *hlab = reinterpret_cast<int32_t *>(stage);
  double *hco = reinterpret_cast<double *>(stage + lab_bytes);
  for (size_t j = 0; j < jobs.size(); ++j) {
    const RawList *L[2] = {&jobs[j].y, &jobs[j].x};
    const size_t at[2] = {oy[j], ox[j]};
    for (int m = 0; m < 2; ++m)
      if (L[m]->n > 0) {
        std::memcpy(hlab + at[m], L[m]->lab, (size_t)L[m]->n * sizeof(int32_t));
        std::memcpy(hco + at[m], L[m]->co, (size_t)L[m]->n * sizeof(double));
      }
  }
  const size_t tsize = (size_t)(KLIMIT + 1) * nw * nw;
  DBuf<char> draw;
  DBuf<int> dterm, dtab, dinfo;  // dterm: key, orbital, function index per term
  DBuf<double> dcoef;
  DBuf<YDesc> dy;
  GG_TRY(draw.alloc(std::max<size_t>(need, 16)));
  GG_TRY(dterm.alloc(3 * std::max<size_t>(T, 1)));
  GG_TRY(dcoef.alloc(std::max<size_t>(T, 1)));
  GG_TRY(dtab.alloc(tsize));
  GG_TRY(dinfo.alloc(2));
  GG_TRY(dy.alloc(std::max<size_t>(1, std::min(T, tsize))));
  int *dkey = dterm.p, *diorb = dkey + std::max<size_t>(T, 1), *dfidx = diorb + std::max<size_t>(T, 1);
  const int32_t *dlab = reinterpret_cast<const int32_t *>(draw.p);
  const double *dco = reinterpret_cast<const double *>(draw.p + lab_bytes);
  if (T > 0) GG_CUDA(cudaMemcpyAsync(draw.p, stage, need, cudaMemcpyHostToDevice, s));
  GG_CUDA(cudaMemsetAsync(dtab.p, 0, tsize * sizeof(int), s));
  GG_CUDA(cudaMemsetAsync(dinfo.p, 0, 2 * sizeof(int), s));
  const unsigned pgrid = (unsigned)std::max<size_t>(1, std::min<size_t>((T + 255) / 256, (size_t)8 * ctx->sms));
  for (int m = 0; m < 2; ++m) {
    const size_t a = m == 0 ? 0 : TY, cnt = m == 0 ? TY : T - TY;
    if (cnt == 0) continue;
    k_parse_terms<<<pgrid, 256, 0, s>>>(m, (int64_t)cnt, dlab + a, dco + a, nw, g.c, dtab.p, dkey + a, diorb + a,
                                        dcoef.p + a, dinfo.p + 1);
    ::gg::note_launch();
  }
  k_number_functions<<<1, 1024, 0, s>>>(dtab.p, (int)tsize, nw, o.dMF.p, n, dy.p, dinfo.p);
  ::gg::note_launch();
  int info[2] = {0, 0};
  GG_CUDA(cudaMemcpyAsync(info, dinfo.p, sizeof(info), cudaMemcpyDeviceToHost, s));
  GG_CUDA(cudaStreamSynchronize(s));
  if (info[1]) return fail(GG_ERR_ARG, "potential: label outside the orbital set or K above 20");
  if (T > 0) {
    k_term_functions<<<pgrid, 256, 0, s>>>((int64_t)T, dkey, dtab.p, dfidx);
    ::gg::note_launch();
  }
  const int nf = std::max(1, info[0]);
  DBuf<double> dY, scratch;
  GG_TRY(dY.alloc((size_t)nf * g.np));
  if (info[0] > 0) GG_TRY(build_y(ctx, dy.p, nf, dY.p, scratch));  // no terms: no function is read
  GG_TRY(dPot.alloc((size_t)3 * n * std::max<size_t>(1, jobs.size())));
  // the DACON and LAGCON lists (a few entries per job) in one upload each
  std::vector<int> ih;
  std::vector<double> dh;
  struct Off { size_t dn, dd, lm, lw; };
  std::vector<Off> off(jobs.size());
  for (size_t j = 0; j < jobs.size(); ++j) {
    const PotJob &J = jobs[j];
    auto pi = [&](const std::vector<int> &v) { size_t at = ih.size(); ih.insert(ih.end(), v.begin(), v.end()); ih.push_back(0); return at; };
    auto pd = [&](const std::vector<double> &v) { size_t at = dh.size(); dh.insert(dh.end(), v.begin(), v.end()); dh.push_back(0.0); return at; };
    off[j] = Off{pi(J.nda), pd(J.da), pi(J.lag_m), pd(J.lag_wa)};
  }
  DBuf<int> di;
  DBuf<double> dd, prod;
  GG_TRY(upload(di, ih, s));
  GG_TRY(upload(dd, dh, s));
  const unsigned blocks = (unsigned)((n + 127) / 128);
  GG_CUDA(cudaMemsetAsync(dPot.p, 0, (size_t)3 * n * jobs.size() * sizeof(double), s));
  // YPOT of every job and the short XPOT lists: one launch each
  std::vector<int> longj;  // jobs whose XPOT takes the two-pass form
  std::vector<PotSeg> hp;
  for (size_t j = 0; j < jobs.size(); ++j) {
    double *yp = dPot.p + (size_t)3 * n * j;
    hp.push_back(PotSeg{dfidx + oy[j], nullptr, dcoef.p + oy[j], yp, nullptr, jobs[j].y.n});
  }
  const size_t nyseg = hp.size();
  for (size_t j = 0; j < jobs.size(); ++j) {
    const int nx = jobs[j].x.n;
    double *xp = dPot.p + (size_t)3 * n * j + n;
    if (nx >= XPOT_SPLIT)
      longj.push_back((int)j);
    else
      hp.push_back(PotSeg{dfidx + ox[j], diorb + ox[j], dcoef.p + ox[j], xp, xp + n, nx});
  }
  DBuf<PotSeg> dpseg;
  if (!hp.empty()) {
    GG_TRY(upload(dpseg, hp, s));
    for (size_t a = 0; a < hp.size(); a += 65535) {  // gridDim.y limit
      const size_t b = std::min(hp.size(), a + 65535);
      if (a < nyseg) {
        const size_t e = std::min(b, nyseg);
        k_potential<0><<<dim3(blocks, (unsigned)(e - a)), 128, 0, s>>>(dpseg.p + a, dY.p, g.np, g.dZZ.p, o.dPF.p,
                                                                        o.dQF.p, o.ld, n);
        ::gg::note_launch();
      }
      if (b > nyseg) {
        const size_t a1 = std::max(a, nyseg);
        k_potential<1><<<dim3(blocks, (unsigned)(b - a1)), 128, 0, s>>>(dpseg.p + a1, dY.p, g.np, g.dZZ.p, o.dPF.p,
                                                                         o.dQF.p, o.ld, n);
        ::gg::note_launch();
      }
    }
  }
  // the long lists of all jobs together, in rounds of at most `per` terms of
  // each job (a job's rounds run in its list's order), each round one
  // product launch and one sum launch over its segments
  DBuf<XSeg> dseg;
  std::vector<size_t> rstart;
  if (!longj.empty()) {
    const int64_t round_terms = std::max<int64_t>(1, (512ll << 20) / (16ll * n));
    const int per = (int)std::max<int64_t>(1, std::min<int64_t>(round_terms / (int64_t)longj.size(), (1 << 26) / n));
    std::vector<XSeg> hs;
    std::vector<size_t> poff;
    size_t maxprod = 0;
    for (int t0 = 0;; t0 += per) {
      const size_t r0 = hs.size();
      size_t po = 0;
      for (int j : longj) {
        const int nx = jobs[j].x.n;
        if (t0 >= nx) continue;
        const int nt = std::min(per, nx - t0);
        double *yp = dPot.p + (size_t)3 * n * j;
        hs.push_back(XSeg{dfidx + ox[j] + t0, diorb + ox[j] + t0, dcoef.p + ox[j] + t0, nullptr, nullptr, yp + n,
                          yp + 2 * n, nt});
        poff.push_back(po);
        po += (size_t)2 * nt * n;
      }
      if (hs.size() == r0) break;
      rstart.push_back(r0);
      maxprod = std::max(maxprod, po);
    }
    rstart.push_back(hs.size());
    GG_TRY(prod.alloc(maxprod));
    for (size_t e = 0; e < hs.size(); ++e) {
      hs[e].P1 = prod.p + poff[e];
      hs[e].P2 = hs[e].P1 + (size_t)hs[e].nt * n;
    }
    GG_TRY(upload(dseg, hs, s));
    for (size_t r = 0; r + 1 < rstart.size(); ++r) {
      const unsigned nseg = (unsigned)(rstart[r + 1] - rstart[r]);
      const unsigned bx = std::max(1u, (unsigned)(4 * ctx->sms) / nseg);
      k_xprod<<<dim3(bx, nseg), 256, 0, s>>>(dseg.p + rstart[r], dY.p, g.np, o.dPF.p, o.dQF.p, o.ld, n);
      k_xsum<<<dim3((n + 31) / 32, 2, nseg), 32, 0, s>>>(dseg.p + rstart[r], n);
      ::gg::note_launch();
      ::gg::note_launch();
    }
  }
  // then every job's LAGCON terms (one launch) and DACON terms (one launch),
  // in that order per job as in COFPOT
  std::vector<TermSeg> ht;
  size_t nlag = 0;
  for (int pass = 0; pass < 2; ++pass) {
    for (size_t j = 0; j < jobs.size(); ++j) {
      const PotJob &J = jobs[j];
      double *xp = dPot.p + (size_t)3 * n * j + n;
      if (pass == 0 && !J.lag_m.empty())
        ht.push_back(TermSeg{di.p + off[j].lm, dd.p + off[j].lw, xp, xp + n, (int)J.lag_m.size()});
      if (pass == 1 && !J.nda.empty())
        ht.push_back(TermSeg{di.p + off[j].dn, dd.p + off[j].dd, xp, xp + n, (int)J.nda.size()});
    }
    if (pass == 0) nlag = ht.size();
  }
  DBuf<TermSeg> dtseg;
  if (!ht.empty()) {
    GG_TRY(upload(dtseg, ht, s));
    for (size_t a = 0; a < nlag; a += 65535) {  // gridDim.y limit
      const unsigned c = (unsigned)std::min<size_t>(65535, nlag - a);
      k_lagcon<<<dim3(blocks, c), 128, 0, s>>>(dtseg.p + a, n, o.dMF.p, g.dR.p, o.dPF.p, o.dQF.p, o.ld);
      ::gg::note_launch();
    }
    for (size_t a = nlag; a < ht.size(); a += 65535) {
      const unsigned c = (unsigned)std::min<size_t>(65535, ht.size() - a);
      k_dacon<<<dim3(blocks, c), 128, 0, s>>>(dtseg.p + a, n, o.dNAK.p, o.dMF.p, g.dR.p, g.dRPOR.p, g.dZZ.p, o.dPF.p,
                                              o.dQF.p, o.ld, g.q);
      ::gg::note_launch();
    }
  }
  GG_CUDA(cudaGetLastError());
  GG_CUDA(cudaStreamSynchronize(s));  // the uploads and scratch are freed on return
  return GG_OK;
}

static int potential(gg_ctx *ctx, int mode, int ncof, const int32_t *lab, const double *co, double *out0,
                     double *out1) {
  GG_TRY(ensure_orbitals(ctx));
  if (!out0 || (mode == 1 && !out1)) return fail(GG_ERR_ARG, "gg_ypot/gg_xpot: bad arguments");
  GG_CUDA(cudaSetDevice(ctx->device));
  std::vector<PotJob> jobs(1);
  GG_TRY(raw_list(ncof, lab, co, mode == 0 ? jobs[0].y : jobs[0].x));
  DBuf<double> pot;
  GG_TRY(run_potentials(ctx, jobs, pot));
  const int n = ctx->grid.n;
  if (mode == 0) {
    GG_CUDA(cudaMemcpy(out0, pot.p, n * sizeof(double), cudaMemcpyDeviceToHost));
  } else {
    GG_CUDA(cudaMemcpy(out0, pot.p + n, n * sizeof(double), cudaMemcpyDeviceToHost));
    GG_CUDA(cudaMemcpy(out1, pot.p + 2 * n, n * sizeof(double), cudaMemcpyDeviceToHost));
  }
  return GG_OK;
}

// one orbital's SETCOF lists as a job (DACON's list checked here)
static int cof_job(gg_ctx *ctx, const gg_cof *c, PotJob &J) {
  if (!c) return fail(GG_ERR_ARG, "potential: missing coefficient lists");
  GG_TRY(raw_list(c->ny, c->nya, c->ya, J.y));
  GG_TRY(raw_list(c->nx, c->nxa, c->xa, J.x));
  if (c->nd < 0 || (c->nd > 0 && (!c->nda || !c->da))) return fail(GG_ERR_ARG, "potential: bad DACON list");
  J.nda.assign(c->nda, c->nda + std::max(0, c->nd));
  J.da.assign(c->da, c->da + std::max(0, c->nd));
  for (int io : J.nda)
    if (io < 1 || io > ctx->orb.nw) return fail(GG_ERR_ARG, "potential: DACON orbital outside the orbital set");
  return GG_OK;
}

extern "C" {

int gg_ypot(gg_ctx *ctx, int ncof, const int32_t *nya, const double *ya, double *yp) {
  if (!ctx) return fail(GG_ERR_ARG, "gg_ypot: no context");
  return potential(ctx, 0, ncof, nya, ya, yp, nullptr);
}

int gg_xpot(gg_ctx *ctx, int ncof, const int32_t *nxa, const double *xa, double *xp, double *xq) {
  if (!ctx) return fail(GG_ERR_ARG, "gg_xpot: no context");
  return potential(ctx, 1, ncof, nxa, xa, xp, xq);
}

int gg_cofpot(gg_ctx *ctx, int j, double ucfj, const gg_cof *cof, int nec, const int32_t *iecc, const double *ecv,
              double accy, double *yp, double *xp, double *xq) {
  if (!ctx || !cof || !yp || !xp || !xq || nec < 0 || (nec > 0 && (!iecc || !ecv)))
    return fail(GG_ERR_ARG, "gg_cofpot: bad arguments");
  GG_TRY(ensure_orbitals(ctx));
  const int nw = ctx->orb.nw;
  if (j < 1 || j > nw) return fail(GG_ERR_ARG, "gg_cofpot: orbital outside the orbital set");
  GG_CUDA(cudaSetDevice(ctx->device));
  std::vector<PotJob> jobs(1);
  GG_TRY(cof_job(ctx, cof, jobs[0]));
  // LAGCON's host part (lagcon.f90:32-45): the pairs with J and their weights
  if (nec > 0) {
    const double eps = (accy > 0 ? accy : std::pow(ctx->grid.h, 6)) * 0.01;
    const double wb = 1.0 / (ucfj * ctx->grid.c) / 1.0;
    for (int k = 0; k < nec; ++k) {
      const int l1 = iecc[k] / KEYORB, l2 = iecc[k] - KEYORB * l1;
      int m;
      if (j == l1)
        m = l2;
      else if (j == l2)
        m = l1;
      else
        continue;
      if (m < 1 || m > nw) return fail(GG_ERR_ARG, "gg_cofpot: multiplier pair outside the orbital set");
      const double wa = ecv[k] * wb;
      if (std::fabs(wa) < eps) continue;
      jobs[0].lag_m.push_back(m);
      jobs[0].lag_wa.push_back(wa);
    }
  }
  DBuf<double> pot;
  GG_TRY(run_potentials(ctx, jobs, pot));
  const int n = ctx->grid.n;
  std::vector<double> h((size_t)3 * n);  // one read-back of YP, XP, XQ
  GG_CUDA(cudaMemcpy(h.data(), pot.p, h.size() * sizeof(double), cudaMemcpyDeviceToHost));
  std::copy(h.begin(), h.begin() + n, yp);
  std::copy(h.begin() + n, h.begin() + 2 * n, xp);
  std::copy(h.begin() + 2 * n, h.end(), xq);
  return GG_OK;
}

int gg_setlag(gg_ctx *ctx, int nec, const int32_t *iecc, const double *ucf, const int *lfix, const gg_cof *cof,
              double *ecv) {
  if (!ctx || nec < 0 || (nec > 0 && (!iecc || !ucf || !lfix || !cof || !ecv)))
    return fail(GG_ERR_ARG, "gg_setlag: bad arguments");
  if (nec == 0) return GG_OK;
  GG_TRY(ensure_orbitals(ctx));
  const Orbitals &o = ctx->orb;
  Grid &g = ctx->grid;
  const int nw = o.nw;
  GG_CUDA(cudaSetDevice(ctx->device));
  // the pairs (setlag.f90:146-149: M = IECC / KEY, J = IECC - KEY M), one
  // potential job per orbital named in a pair
  std::vector<int> slot(nw + 1, -1), orbs;
  std::vector<int4> pj(nec);
  std::vector<int2> ps(nec);
  std::vector<double2> uc(nec);
  std::vector<int2> rjk;
  std::vector<int> ridx;
  for (int k = 0; k < nec; ++k) {
    const int M = iecc[k] / KEYORB, J = iecc[k] - KEYORB * M;
    if (J < 1 || J > nw || M < 1 || M > nw) return fail(GG_ERR_ARG, "gg_setlag: pair outside the orbital set");
    if (o.nak[J] != o.nak[M]) return fail(GG_ERR_KAPPA, "gg_setlag: pair with different kappa (RINTI)");
    for (int x : {J, M})
      if (slot[x] < 0) {
        slot[x] = (int)orbs.size();
        orbs.push_back(x);
      }
    const double uj = ucf[J - 1], um = ucf[M - 1];
    int cs;
    if (lfix[M - 1]) {
      cs = 0;
    } else if (lfix[J - 1]) {
      cs = 1;
    } else {
      const double qdif = std::fabs((uj - um) / std::max(uj, um));
      cs = (qdif > 1.0e-01) ? 2 : 3;
    }
    pj[k] = make_int4(J, M, cs, std::max(o.mf[J], o.mf[M]));
    ps[k] = make_int2(slot[J], slot[M]);
    uc[k] = make_double2(uj, um);
    if (cs != 2) {  // RINTI(M, J, 1), or RINTI(J, M, 1) when J is fixed
      rjk.push_back(cs == 1 ? make_int2(J, M) : make_int2(M, J));
      ridx.push_back(k);
    }
  }
  std::vector<PotJob> jobs(orbs.size());
  for (size_t i = 0; i < orbs.size(); ++i) GG_TRY(cof_job(ctx, &cof[orbs[i] - 1], jobs[i]));
  DBuf<double> pot;
  GG_TRY(run_potentials(ctx, jobs, pot));
  cudaStream_t s = ctx->stream;
  DBuf<int4> dpj;
  DBuf<int2> dps;
  DBuf<double2> duc;
  DBuf<double> dTA, dres, drij, decv;
  GG_TRY(upload(dpj, pj, s));
  GG_TRY(upload(dps, ps, s));
  GG_TRY(upload(duc, uc, s));
  GG_TRY(dTA.alloc((size_t)nec * g.np));
  GG_TRY(dres.alloc(nec));
  GG_TRY(drij.alloc(nec));
  GG_TRY(decv.alloc(nec));
  GG_CUDA(cudaMemsetAsync(drij.p, 0, nec * sizeof(double), s));
  k_setlag_quad<<<nec, 128, 0, s>>>(dpj.p, dps.p, pot.p, g.n, o.dPF.p, o.dQF.p, o.ld, g.dR.p, g.dRP.p, g.dRPOR.p,
                                    g.q, g.np, dTA.p, dres.p);
  ::gg::note_launch();
  GG_CUDA(cudaGetLastError());
  if (!rjk.empty()) GG_TRY(run_rinti(ctx, rjk, 1, drij.p, &ridx));
  k_setlag_final<<<(nec + 127) / 128, 128, 0, s>>>(nec, dpj.p, duc.p, dres.p, drij.p, decv.p);
  ::gg::note_launch();
  GG_CUDA(cudaGetLastError());
  GG_CUDA(cudaMemcpyAsync(ecv, decv.p, nec * sizeof(double), cudaMemcpyDeviceToHost, s));
  GG_CUDA(cudaStreamSynchronize(s));
  return GG_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// gg_slater_noalloc: SLATER without any device allocation.
//
// Some callers cannot allocate device memory when they need one integral: a
// host code that has handed the whole device to a memory pool or to the
// Hamiltonian and Davidson basis of a large block (where a cudaMalloc would
// fail or fragment the pool), or code whose error handling cannot recover
// from an allocation failure in the middle of a loop (the Fortran callers
// STOP). For them this entry point evaluates R^k(ab;cd) exactly like
// gg_slater, but its working arrays (the two TEMP arrays and Y^k of YZK, the
// integral's descriptors and its result) live in one file-scope device array
// of fixed size, reserved when the library is loaded and held by every GPU
// that loads it until the process exits.
//
// Limit: the grid must satisfy N + 26 <= NOALLOC_NP (N <= 2022 points; GRASP
// uses 590). The first call on a device looks up the array's device address
// (cudaGetSymbolAddress) with that device current; make that first call
// before any stream capture. All calls share the array and it keeps the last
// call's contents (Y^k is cleared at the start of each call): calls that can
// overlap on the GPU -- several host threads, or several contexts on one
// device -- race on it and must be serialised by the caller.
// ---------------------------------------------------------------------------
namespace gg {
namespace {
constexpr int NOALLOC_NP = 2048;              // doubles per working array
constexpr int NOALLOC_DESC = 64;              // doubles reserved for descriptors and the result
static __device__ __align__(256) double g_noalloc_scratch[3 * NOALLOC_NP + NOALLOC_DESC];

struct NoallocAddr {
  std::mutex mu;
  double *ptr[64] = {};
};
NoallocAddr &noalloc_addr() {
  static NoallocAddr a;
  return a;
}
}  // namespace
}  // namespace gg

extern "C" int gg_slater_noalloc(gg_ctx *ctx, int ia, int ib, int ic, int id, int k, double *out) {
  GG_TRY(ensure_orbitals(ctx));
  Orbitals &o = ctx->orb;
  Grid &g = ctx->grid;
  const int nw = o.nw;
  if (!out || k < 0 || k > KLIMIT || ia < 1 || ib < 1 || ic < 1 || id < 1 || ia > nw || ib > nw || ic > nw ||
      id > nw)
    return fail(GG_ERR_ARG, "gg_slater_noalloc: bad arguments");
  if (g.np > NOALLOC_NP)
    return fail(GG_ERR_ARG, "gg_slater_noalloc: grid of " + std::to_string(g.n) +
                                " points exceeds the fixed scratch (at most " + std::to_string(NOALLOC_NP - GPAD - 10) +
                                " points); use gg_slater");
  if (ctx->device < 0 || ctx->device >= 64) return fail(GG_ERR_ARG, "gg_slater_noalloc: device index above 63");
  GG_CUDA(cudaSetDevice(ctx->device));
  double *base = nullptr;
  {
    NoallocAddr &A = noalloc_addr();
    std::lock_guard<std::mutex> lock(A.mu);
    if (!A.ptr[ctx->device]) {
      void *p = nullptr;
      GG_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
      A.ptr[ctx->device] = static_cast<double *>(p);
    }
    base = A.ptr[ctx->device];
  }
  double *TZ = base, *TW = base + NOALLOC_NP, *Y = base + 2 * NOALLOC_NP;
  double *tail = base + 3 * NOALLOC_NP;  // 256-byte aligned: 3 * 2048 doubles = 192 * 256 bytes
  YDesc *dyd = reinterpret_cast<YDesc *>(tail);
  QuadItem *ditem = reinterpret_cast<QuadItem *>(tail + 8);
  double *dout = tail + 16;
  YDesc y;
  y.k = k;
  y.b = ib;
  y.d = id;
  y.mtp = std::min(o.mf[ib], o.mf[id]);
  y.mtpb = (k == 0 && ib == id) ? g.n : y.mtp;
  y.cs = 0;
  y.nd = 1;
  QuadItem it;
  it.a = ia;
  it.c = ic;
  it.f = 0;
  it.mtp = (k == 0 && ib == id) ? std::min(o.mf[ia], o.mf[ic]) : std::min(std::min(y.mtp, o.mf[ia]), o.mf[ic]);
  it.pos = 0;
  const int np = g.np;
  GG_CUDA(cudaMemcpyAsync(dyd, &y, sizeof(YDesc), cudaMemcpyHostToDevice, ctx->stream));
  GG_CUDA(cudaMemcpyAsync(ditem, &it, sizeof(QuadItem), cudaMemcpyHostToDevice, ctx->stream));
  dim3 grid1((np + 127) / 128, 1);
  k_ytemp<<<grid1, 128, 0, ctx->stream>>>(dyd, 1, o.dPF.p, o.dQF.p, o.ld, g.dRP.p, g.dPow.p, np, TZ, TW);
  ::gg::note_launch();
  GG_CUDA(cudaMemsetAsync(Y, 0, (size_t)np * sizeof(double), ctx->stream));
  k_ychain<<<1, 128, 0, ctx->stream>>>(dyd, 1, TZ, TW, g.dR.p, g.dPow.p, np, g.q, Y);
  ::gg::note_launch();
  k_quad_items<<<1, 32, np * sizeof(double), ctx->stream>>>(ditem, nullptr, 1, Y, np, o.dPF.p, o.dQF.p, o.ld, g.dR.p,
                                                            g.dRP.p, g.dRPOR.p, g.q, dout);
  ::gg::note_launch();
  GG_CUDA(cudaGetLastError());
  GG_CUDA(cudaMemcpyAsync(out, dout, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  GG_CUDA(cudaStreamSynchronize(ctx->stream));
  return GG_OK;
}

extern "C" {

static int run_rinti(gg_ctx *ctx, const std::vector<int2> &jk, int mode, double *dOut, const std::vector<int> *outidx) {
  Orbitals &o = ctx->orb;
  Grid &g = ctx->grid;
  DBuf<int2> djk;
  DBuf<int> didx;
  GG_TRY(upload(djk, jk, ctx->stream));
  if (outidx) GG_TRY(upload(didx, *outidx, ctx->stream));
  const int wpb = 2;
  const size_t smem = (size_t)wpb * 3 * g.np * sizeof(double);
  const int blocks = std::max(1, std::min(((int)jk.size() + wpb - 1) / wpb, 2048));
  k_rinti<<<blocks, 32 * wpb, smem, ctx->stream>>>(djk.p, (int)jk.size(), mode, o.dPF.p, o.dQF.p, o.ld, o.dMF.p,
                                                   o.dNAK.p, g.dR.p, g.dRP.p, g.dRPOR.p, g.dZZ.p, g.np, g.q, dOut,
                                                   outidx ? didx.p : nullptr); ::gg::note_launch();
  GG_CUDA(cudaGetLastError());
  GG_CUDA(cudaStreamSynchronize(ctx->stream));
  return GG_OK;
}

int gg_rinti(gg_ctx *ctx, int j, int k, int mode, double *out) {
  GG_TRY(ensure_orbitals(ctx));
  const Orbitals &o = ctx->orb;
  if (!out || j < 1 || k < 1 || j > o.nw || k > o.nw) return fail(GG_ERR_ARG, "gg_rinti: bad arguments");
  if (o.nak[j] != o.nak[k]) return fail(GG_ERR_KAPPA, "RINTI: Attempt to calculate I(a,b) with kappa(a) != kappa(b)");
  GG_CUDA(cudaSetDevice(ctx->device));
  DBuf<double> d;
  GG_TRY(d.alloc(1));
  GG_TRY(run_rinti(ctx, {make_int2(j, k)}, mode, d.p, nullptr));
  GG_CUDA(cudaMemcpy(out, d.p, sizeof(double), cudaMemcpyDeviceToHost));
  return GG_OK;
}

int gg_iabint_table(gg_ctx *ctx, double *iab) {
  GG_TRY(ensure_orbitals(ctx));
  GG_CUDA(cudaSetDevice(ctx->device));
  const Orbitals &o = ctx->orb;
  const int nw = o.nw;
  GG_TRY(timer_start(ctx));
  GG_TRY(ctx->dIab.alloc((size_t)nw * nw));
  k_fill<<<64, 256, 0, ctx->stream>>>(ctx->dIab.p, (size_t)nw * nw, nan("")); ::gg::note_launch();
  GG_CUDA(cudaGetLastError());
  std::vector<int2> jk;
  std::vector<int> idx;
  for (int a = 1; a <= nw; ++a)
    for (int b = 1; b <= nw; ++b)
      if (o.nak[a] == o.nak[b]) {
        jk.push_back(make_int2(a, b));
        idx.push_back((a - 1) * nw + (b - 1));
      }
  if (!jk.empty()) GG_TRY(run_rinti(ctx, jk, 0, ctx->dIab.p, &idx));
  double ms = 0;
  GG_TRY(timer_stop(ctx, &ms));
  ctx->stats[1] = ms;
  ctx->iab_valid = true;
  if (iab) GG_CUDA(cudaMemcpy(iab, ctx->dIab.p, (size_t)nw * nw * sizeof(double), cudaMemcpyDeviceToHost));
  return GG_OK;
}

}  // extern "C"
