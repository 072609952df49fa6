// setham.cu - Hamiltonian assembly from rangular's T/V lists on the GPU
// (rmcdhf90/setham.f90:3-352, the EAV shift of rmcdhf90/matrix.f90:178-203).
//
// Compiled with -fmad=false: EMT(LOC) = EMT(LOC) + TEGRAL*COEFF is rounded
// twice, as the reference does.
//
// Method. The reference scatters, label by label, EMT(LOC) += I * COEFF.
// Here every contribution is first given the slot of its integral in one
// device array [VALTEIRK | I(ab) table]; the contributions are then
// transposed into per-element segments (a counting sort by LOC whose
// segments are sorted back into list order), so that one thread per matrix
// element adds its contributions in exactly the reference's order (T list,
// then V^0 .. V^kmaxf, labels in file order). No floating-point atomics: the
// result is deterministic and equals the reference's sequence of roundings
// given the same integrals.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "gg_internal.cuh"

namespace gg {
namespace {

struct DiagTerm {
  int type;    // 0 I(aa) IQ ; 1 F0(aa) ; 2 Fk(aa) ; 3 F0(ab) ; 4 Gk(ab)
  int a, b;    // 0-based orbital indices
  int full_a, full_b;  // 2j+1 of a, b
  double fac;  // CLRX(...) for types 2 and 4
  long long slot;
};

// GAM(I) = log((I-1)!) (lib9290/factt.f90)
struct Gam {
  double g[512];
  Gam() {
    g[0] = 0.0;
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

// CLRX (lib9290/clrx.f90): the 3j symbol (ja k jb; 1/2 0 -1/2) up to sign
// conventions, from log-factorials.
double clrx(int kappaa, int k, int kappab) {
  static const Gam G;
  const double *GAM = G.g;
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

// canonical RKINTC position of R^k(abcd) in the device table; -1 if absent
__device__ long long rk_lookup(const int32_t *ind, const int32_t *kstart, int kloop, int key, int ia, int ib, int ic,
                               int id, int k) {
  if (k < 0 || k > kloop) return -1;
  if (ia > ic) {
    const int t = ia;
    ia = ic;
    ic = t;
  }
  if (ib > id) {
    const int t = ib;
    ib = id;
    id = t;
  }
  if (ia > ib) {
    int t = ia;
    ia = ib;
    ib = t;
    t = ic;
    ic = id;
    id = t;
  }
  const int32_t index = ((ia * key + ib) * key + ic) * key + id;
  long long jl = kstart[k], ju = (long long)kstart[k + 1] - 1;
  if (ju < jl) return -1;
  if (index < ind[jl - 1] || index > ind[ju - 1]) return -1;
  while (ju - jl > 1) {
    const long long jm = (ju + jl) / 2;
    if (ind[jm - 1] > index)
      ju = jm;
    else
      jl = jm;
  }
  if (index == ind[ju - 1]) return ju - 1;
  if (index == ind[jl - 1]) return jl - 1;
  return -1;
}

// Label -> integral slot, and the slot of each contribution (one warp per label).
__global__ void k_label_slots(const int32_t *__restrict__ lab, const int64_t *__restrict__ start, int64_t nlab,
                              const int64_t *__restrict__ list_lab0, int nlists, int nw, const int *__restrict__ nak,
                              const int32_t *__restrict__ ind, const int32_t *__restrict__ kstart, int kloop,
                              long long nrk, int32_t *__restrict__ cslot, int *__restrict__ err) {
  const int lane = threadIdx.x & 31;
  const long long wid = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long l = wid; l < nlab; l += nwarps) {
    int list = 0;
    while (list + 1 < nlists && l >= list_lab0[list + 1]) ++list;
    int32_t L = lab[l];
    long long slot = -1;
    if (list == 0) {  // T list: IA = MOD(LAB,KEY), IB = LAB/KEY (setham.f90:244-245)
      const int ia = L % KEYORB, ib = L / KEYORB;
      if (ia >= 1 && ib >= 1 && ia <= nw && ib <= nw && nak[ia] == nak[ib]) slot = nrk + (long long)(ia - 1) * nw + (ib - 1);
    } else {  // V^k list (setham.f90:305-310)
      const int k = list - 1;
      const int id = L % KEYORB;
      L = L / KEYORB;
      const int ib = L % KEYORB;
      L = L / KEYORB;
      const int ic = L % KEYORB;
      const int ia = L / KEYORB;
      if (ia >= 1 && ib >= 1 && ic >= 1 && id >= 1 && ia <= nw && ib <= nw && ic <= nw && id <= nw)
        slot = rk_lookup(ind, kstart, kloop, nw + 1, ia, ib, ic, id, k);
    }
    if (slot < 0) {
      if (lane == 0) atomicExch(err, 1);
      slot = 0;
    }
    for (long long j = start[l] + lane; j < start[l + 1]; j += 32) cslot[j] = (int32_t)slot;
  }
}

__global__ void k_count_loc(const int32_t *__restrict__ loc, int64_t n, int64_t nnz, int *__restrict__ cnt,
                            int *__restrict__ err) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
    const int32_t L = loc[j];
    if (L < 1 || (int64_t)L > nnz) {
      atomicExch(err, 2);
      continue;
    }
    atomicAdd(&cnt[L - 1], 1);
  }
}

// exclusive scan of cnt[n] into off[n+1] (int64), three phases
__global__ void k_scan_blocks(const int *__restrict__ cnt, int64_t n, int64_t *__restrict__ part, int64_t chunk) {
  __shared__ long long s[1024];
  const int64_t b = blockIdx.x;
  const int64_t lo = b * chunk, hi = min(n, lo + chunk);
  long long acc = 0;
  for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) acc += cnt[i];
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[b] = s[0];
}
__global__ void k_scan_parts(int64_t *part, int64_t nparts) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    long long acc = 0;
    for (int64_t i = 0; i < nparts; ++i) {
      const long long v = part[i];
      part[i] = acc;
      acc += v;
    }
    part[nparts] = acc;
  }
}
__global__ void k_scan_final(const int *__restrict__ cnt, int64_t n, const int64_t *__restrict__ part, int64_t chunk,
                             int64_t *__restrict__ off) {
  // one block per chunk; serial over warps-sized pieces with a block scan
  __shared__ long long s[1024];
  const int64_t b = blockIdx.x;
  const int64_t lo = b * chunk, hi = min(n, lo + chunk);
  long long base = part[b];
  for (int64_t i0 = lo; i0 < hi; i0 += blockDim.x) {
    const int64_t i = i0 + threadIdx.x;
    const long long v = (i < hi) ? cnt[i] : 0;
    s[threadIdx.x] = v;
    __syncthreads();
    for (int w = 1; w < (int)blockDim.x; w <<= 1) {
      long long t = ((int)threadIdx.x >= w) ? s[threadIdx.x - w] : 0;
      __syncthreads();
      s[threadIdx.x] += t;
      __syncthreads();
    }
    if (i < hi) off[i] = base + s[threadIdx.x] - v;
    const long long tot = s[blockDim.x - 1];
    __syncthreads();
    base += tot;
  }
  if (b == gridDim.x - 1 && threadIdx.x == 0) off[n] = part[gridDim.x];
}

__global__ void k_scatter_perm(const int32_t *__restrict__ loc, int64_t n, const int64_t *__restrict__ off,
                               int *__restrict__ fill, int32_t *__restrict__ perm) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
    const int32_t L = loc[j];
    const int r = atomicAdd(&fill[L - 1], 1);
    perm[off[L - 1] + r] = (int32_t)j;
  }
}

// sort each element's segment back into list order, then gather the
// coefficient and integral slot of each contribution
// Each element's contributions back into list order (insertion sort of its
// short segment of perm, one lane per element), then the coefficients and
// integral slots gathered in that order: the 32 elements of a warp own one
// contiguous range, which the warp writes with coalesced stores.
__global__ void __launch_bounds__(256) k_sort_gather(const int64_t *__restrict__ off, int64_t nnz,
                                                     int32_t *__restrict__ perm, const double *__restrict__ coeff,
                                                     const int32_t *__restrict__ cslot, double *__restrict__ coeff_s,
                                                     int32_t *__restrict__ slot_s) {
  const int lane = threadIdx.x & 31;
  const int64_t e0 = ((int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * 32;
  if (e0 >= nnz) return;
  const int ne = (int)min((int64_t)32, nnz - e0);
  if (lane < ne) {
    const int64_t lo = off[e0 + lane], hi = off[e0 + lane + 1];
    for (int64_t i = lo + 1; i < hi; ++i) {
      const int32_t v = perm[i];
      int64_t j = i - 1;
      while (j >= lo && perm[j] > v) {
        perm[j + 1] = perm[j];
        --j;
      }
      perm[j + 1] = v;
    }
  }
  __syncwarp();
  const int64_t c0 = off[e0], c1 = off[e0 + ne];
  for (int64_t i = c0 + lane; i < c1; i += 32) {
    const int32_t p = perm[i];
    coeff_s[i] = coeff[p];
    slot_s[i] = cslot[p];
  }
}

// Diagonal pieces without MCP coefficients (setham.f90:83-219), one thread
// per CSF, terms in the reference's loop order, zero coefficients skipped.
// The diagonal pieces of EMT per run of equal occupations (a configuration),
// one warp per run: lane l takes the terms t = l, l + 32, ...; the lane sums
// are added by a fixed shuffle tree (the order of the reference's sum
// differs only by rounding); k_diag_scatter copies them to the CSFs
__global__ void k_diag_terms(const DiagTerm *__restrict__ terms, int nterms, const uint8_t *__restrict__ iq, int nw,
                             int nconf, const double *__restrict__ integ, double *__restrict__ cdiag) {
  const int ir = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (ir >= nconf) return;
  const uint8_t *q = iq + (size_t)ir * nw;
  double acc = 0.0;
  for (int t = lane; t < nterms; t += 32) {
    const DiagTerm T = terms[t];
    const int qa = q[T.a];
    double coef = 0.0;
    switch (T.type) {
      case 0:  // IQ(a) I(aa)
        if (qa <= 0) continue;
        coef = (double)qa;
        break;
      case 1:  // FCO(0,a,a) = (q(q-1))/2 (fco.f90)
        coef = (double)((qa * (qa - 1)) / 2);
        break;
      case 2:  // FCO(k,a,a) for a full subshell
        if (qa == T.full_a) {
          const double fac = T.fac * (double)qa;
          coef = -0.5 * fac * fac;
        }
        break;
      case 3:  // FCO(0,a,b) = q_a q_b
        coef = (double)(qa * (int)q[T.b]);
        break;
      case 4: {  // GCO(k,a,b) (gco.f90)
        const int qb = q[T.b];
        if (qa == T.full_a || qb == T.full_b) coef = -(double)(qa * qb) * T.fac * T.fac;
        break;
      }
    }
    if (coef == 0.0) continue;
    acc = fma(coef, integ[T.slot], acc);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) cdiag[ir] = acc;
}
__global__ void k_diag_scatter(const int32_t *__restrict__ conf, const double *__restrict__ cdiag, int ncf,
                               const int64_t *__restrict__ iendc, double *__restrict__ emt) {
  const int ir = blockIdx.x * blockDim.x + threadIdx.x;
  if (ir < ncf) emt[iendc[ir + 1] - 1] = cdiag[conf[ir]];
}

// EMT(LOC) = EMT(LOC) + I * COEFF over the element's contributions, in order
// One EMT element per lane, its contributions added in list order. The 32
// elements of a warp own one contiguous range of contributions: the warp
// forms the products integ[slot] coeff of that range with coalesced loads
// into shared memory, then each lane adds its own segment in order (the
// same sums as a lane walking its segment alone, which is what a range
// longer than the staging buffer does).
constexpr int AS_WARPS = 8, AS_MAX = 256;
__global__ void __launch_bounds__(AS_WARPS * 32) k_assemble(const int64_t *__restrict__ off, int64_t nnz,
                                                            const double *__restrict__ coeff_s,
                                                            const int32_t *__restrict__ slot_s,
                                                            const double *__restrict__ integ,
                                                            double *__restrict__ emt) {
  __shared__ double sv[AS_WARPS][AS_MAX];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t e0 = ((int64_t)blockIdx.x * AS_WARPS + warp) * 32;
  if (e0 >= nnz) return;
  const int ne = (int)min((int64_t)32, nnz - e0);
  const int64_t e = e0 + lane;
  const int64_t c0 = off[e0], c1 = off[e0 + ne];
  const int64_t lo = (lane < ne) ? off[e] : 0, hi = (lane < ne) ? off[e + 1] : 0;
  if (c1 - c0 <= AS_MAX) {
    for (int64_t i = c0 + lane; i < c1; i += 32) sv[warp][i - c0] = integ[slot_s[i]] * coeff_s[i];
    __syncwarp();
    if (lo < hi) {
      double acc = emt[e];
      for (int64_t i = lo; i < hi; ++i) acc = acc + sv[warp][i - c0];
      emt[e] = acc;
    }
  } else if (lo < hi) {
    double acc = emt[e];
    for (int64_t i = lo; i < hi; ++i) acc = acc + integ[slot_s[i]] * coeff_s[i];
    emt[e] = acc;
  }
}

// EAV = sum of diagonals / NCF (deterministic tree), then H - EAV I
// EAV = mean of the diagonal, subtracted from it (matrix.f90:123-203): CTA
// partial sums over contiguous row ranges (EAV_CTAS of them, each in a fixed
// order), their sum by one CTA in CTA order, then the shift in parallel
constexpr int EAV_CTAS = 64;
__global__ void __launch_bounds__(256) k_eav_part(const int64_t *__restrict__ iendc, int ncf,
                                                  const double *__restrict__ emt, double *__restrict__ part) {
  __shared__ double s[256];
  const int per = (ncf + EAV_CTAS - 1) / EAV_CTAS;
  const int r0 = blockIdx.x * per, r1 = min(ncf, r0 + per);
  double acc = 0.0;
  for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) acc = acc + emt[iendc[i + 1] - 1];
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) s[threadIdx.x] = s[threadIdx.x] + s[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = s[0];
}
__global__ void k_eav_fin(const double *__restrict__ part, int ncf, double *__restrict__ eav_out) {
  if (threadIdx.x != 0) return;
  double sum = 0.0;
  for (int b = 0; b < EAV_CTAS; ++b) sum = sum + part[b];
  *eav_out = sum / (double)ncf;
}
__global__ void k_eav_sub(const int64_t *__restrict__ iendc, int ncf, const double *__restrict__ eav,
                          double *__restrict__ emt, double *__restrict__ diag) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ncf) return;
  const int64_t p = iendc[i + 1] - 1;
  const double v = emt[p] - *eav;
  emt[p] = v;
  diag[i] = v;
}

// IROW checks of gg_hmat_create, one warp per row: each row ends with its
// diagonal (IROW = row, 1-based) and its other entries lie in 1 .. row - 1.
// bad = min over offending rows of (row << 2 | kind), kind 1 for a missing
// diagonal, 2 for an entry outside the lower triangle.
__global__ void k_check_irow(const int64_t *__restrict__ iendc, const int32_t *__restrict__ irow, int ncf,
                             unsigned long long *__restrict__ bad) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= ncf) return;
  const int i = warp + 1;
  const int64_t p0 = iendc[warp], p1 = iendc[warp + 1];
  int kind = 0;
  if (lane == 0 && irow[p1 - 1] != i) kind = 1;
  for (int64_t p = p0 + lane; p < p1 - 1; p += 32)
    if (irow[p] < 1 || irow[p] >= i) kind = 2;
  kind = __reduce_max_sync(0xffffffffu, kind);
  if (lane == 0 && kind) atomicMin(bad, ((unsigned long long)i << 2) | (unsigned long long)kind);
}

template <class T> int upload(DBuf<T> &b, const T *h, size_t n, cudaStream_t s) {
  GG_TRY(b.alloc(n));
  if (n) GG_CUDA(cudaMemcpyAsync(b.p, h, n * sizeof(T), cudaMemcpyHostToDevice, s));
  return GG_OK;
}

// host-side RKINTC position (0-based) in the context table, -1 if absent
long long host_rk_pos(const RkTable &rk, int nw, int ia, int ib, int ic, int id, int k) {
  if (k > rk.kloop) return -1;
  const int KEY = nw + 1;
  if (ia > ic) std::swap(ia, ic);
  if (ib > id) std::swap(ib, id);
  if (ia > ib) {
    std::swap(ia, ib);
    std::swap(ic, id);
  }
  const int32_t index = ((ia * KEY + ib) * KEY + ic) * KEY + id;
  const int32_t *b = rk.hInd.data() + (rk.kstart[k] - 1);
  const int32_t *e = rk.hInd.data() + (rk.kstart[k + 1] - 1);
  const int32_t *p = std::lower_bound(b, e, index);
  if (p == e || *p != index) return -1;
  return p - rk.hInd.data();
}

}  // namespace

double clrx_host(int kappaa, int k, int kappab) { return clrx(kappaa, k, kappab); }

}  // namespace gg

using namespace gg;

extern "C" {

int gg_hmat_create(gg_ctx *ctx, int ncf, int64_t nnz, const int64_t *iendc, const int32_t *irow, gg_hmat **out) {
  if (!ctx || !out || !iendc || !irow || ncf < 1 || nnz < ncf) return fail(GG_ERR_ARG, "gg_hmat_create: bad arguments");
  *out = nullptr;
  if (iendc[0] != 0 || iendc[ncf] != nnz) return fail(GG_ERR_ARG, "gg_hmat_create: IENDC(0) must be 0, IENDC(NCF) = NNZ");
  for (int i = 1; i <= ncf; ++i)
    if (iendc[i] <= iendc[i - 1]) return fail(GG_ERR_ARG, "gg_hmat_create: empty row (the diagonal is required)");
  GG_CUDA(cudaSetDevice(ctx->device));
  gg_hmat *h = new gg_hmat;
  h->ctx = ctx;
  h->ncf = ncf;
  h->nnz = nnz;
  h->hIendc.assign(iendc, iendc + ncf + 1);
  int s = upload(h->dIendc, iendc, (size_t)ncf + 1, ctx->stream);
  if (s == GG_OK) s = upload(h->dIrow, irow, (size_t)nnz, ctx->stream);
  if (s == GG_OK) s = h->dEmt.alloc(nnz);
  if (s == GG_OK) s = h->dDiag.alloc(ncf);
  // IROW checked on the device (diagonal last in each row: the
  // lower-triangle-by-rows mode of spicmv2.f90), the result read back here
  DBuf<unsigned long long> dbad;
  unsigned long long hbad[1] = {~0ull};
  if (s == GG_OK) s = upload(dbad, hbad, 1, ctx->stream);
  if (s == GG_OK) {
    k_check_irow<<<(unsigned)(((int64_t)ncf * 32 + 255) / 256), 256, 0, ctx->stream>>>(h->dIendc.p, h->dIrow.p, ncf,
                                                                                       dbad.p);
    ::gg::note_launch();
    if (cudaMemcpyAsync(hbad, dbad.p, sizeof(hbad), cudaMemcpyDeviceToHost, ctx->stream) != cudaSuccess ||
        cudaStreamSynchronize(ctx->stream) != cudaSuccess)
      s = fail(GG_ERR_CUDA, "gg_hmat_create: copy failed");
  }
  if (s == GG_OK && hbad[0] != ~0ull)
    s = fail(GG_ERR_ARG, (hbad[0] & 3) == 1 ? "gg_hmat_create: row does not end with its diagonal"
                                            : "gg_hmat_create: IROW outside the lower triangle");
  if (s != GG_OK) {
    delete h;
    return s;
  }
  *out = h;
  return GG_OK;
}

int gg_hmat_destroy(gg_hmat *h) {
  if (!h) return GG_OK;
  cudaSetDevice(h->ctx->device);
  cudaStreamSynchronize(h->ctx->stream);
  if (gg_hmat *root = h->base) {  // a view: its borrowed buffers are not freed with it
    delete h;
    if (--root->views == 0 && root->dead) delete root;
    return GG_OK;
  }
  if (h->views > 0) {  // freed with its last view
    h->dead = true;
    return GG_OK;
  }
  delete h;
  return GG_OK;
}

int gg_hmat_create_view(gg_ctx *ctx, gg_hmat *src, gg_hmat **out) {
  if (!ctx || !src || !out) return fail(GG_ERR_ARG, "gg_hmat_create_view: bad arguments");
  *out = nullptr;
  gg_hmat *root = src->base ? src->base : src;
  if (root->dead) return fail(GG_ERR_STATE, "gg_hmat_create_view: the source was destroyed");
  if (root->host_prec >= 0) return fail(GG_ERR_ARG, "gg_hmat_create_view: the source is a host-resident matrix");
  if (ctx->device != root->ctx->device) return fail(GG_ERR_ARG, "gg_hmat_create_view: source on another device");
  // the source's symmetric structure is built once and shared
  GG_TRY(build_sym(root));
  GG_CUDA(cudaStreamSynchronize(root->ctx->stream));
  GG_CUDA(cudaSetDevice(ctx->device));
  gg_hmat *h = new gg_hmat;
  h->ctx = ctx;
  h->ncf = root->ncf;
  h->nnz = root->nnz;
  h->hIendc = root->hIendc;
  h->dIendc.borrow(root->dIendc);
  h->dIrow.borrow(root->dIrow);
  h->lists = root->lists;
  h->sym_valid = root->sym_valid;
  h->sym_nnz = root->sym_nnz;
  h->sym_col16 = root->sym_col16;
  h->dSymPtr.borrow(root->dSymPtr);
  h->dSymCol.borrow(root->dSymCol);
  h->dSymCol16.borrow(root->dSymCol16);
  h->dSymSrc.borrow(root->dSymSrc);
  int s = h->dEmt.alloc(h->nnz);
  if (s == GG_OK) s = h->dDiag.alloc(h->ncf);
  if (s != GG_OK) {
    delete h;
    return s;
  }
  h->base = root;
  ++root->views;
  *out = h;
  return GG_OK;
}

static int build_plan(gg_ctx *ctx, gg_hmat *h, Lists &L, cudaEvent_t coeff_ready);

int gg_setham_upload(gg_ctx *ctx, gg_hmat *h, const uint8_t *iq, const gg_list *tlist, int kmaxf,
                     const gg_list *vlists) {
  if (!ctx || !h || h->ctx != ctx || !iq || !tlist || kmaxf < -1 || (kmaxf >= 0 && !vlists))
    return fail(GG_ERR_ARG, "gg_setham_upload: bad arguments");
  if (h->host_prec >= 0) return fail(GG_ERR_ARG, "gg_setham_upload: a host-resident matrix is not assembled here");
  GG_TRY(ensure_orbitals(ctx));
  GG_CUDA(cudaSetDevice(ctx->device));
  GG_TRY(timer_start(ctx));
  if (h->base) return fail(GG_ERR_STATE, "gg_setham_upload: a view shares its source's lists (upload to the source)");
  Lists &L = *h->lists;
  L.plan_key.clear();  // new lists: the assembly plan is rebuilt
  const int nlists = kmaxf + 2;
  std::vector<const gg_list *> ls;
  ls.push_back(tlist);
  for (int k = 0; k <= kmaxf; ++k) ls.push_back(&vlists[k]);
  int64_t nlab = 0, ncontr = 0;
  L.list_lab0.assign(nlists + 1, 0);
  for (int i = 0; i < nlists; ++i) {
    const gg_list *x = ls[i];
    if (x->nlab < 0 || (x->nlab > 0 && (!x->lab || !x->start || !x->loc || !x->coeff)))
      return fail(GG_ERR_ARG, "gg_setham_upload: bad list");
    if (x->nlab > 0 && x->start[0] != 0) return fail(GG_ERR_ARG, "gg_setham_upload: start[0] must be 0");
    for (int64_t l = 0; l < x->nlab; ++l)
      if (x->start[l + 1] < x->start[l]) return fail(GG_ERR_ARG, "gg_setham_upload: decreasing start[]");
    L.list_lab0[i] = nlab;
    nlab += x->nlab;
    ncontr += x->nlab ? x->start[x->nlab] : 0;
  }
  L.list_lab0[nlists] = nlab;
  if (ncontr > INT32_MAX) return fail(GG_ERR_RANGE, "gg_setham_upload: more than 2^31-1 contributions in one block");
  L.kmaxf = kmaxf;
  L.nlab = nlab;
  L.ncontr = ncontr;
  const int nw = ctx->orb.nw;
  {
    // runs of equal IQ rows (GRASP lists a configuration's CSFs together):
    // the diagonal pieces depend on the occupations only, so they are
    // evaluated once per run
    std::vector<int32_t> conf(h->ncf);
    std::vector<uint8_t> rows;
    rows.reserve((size_t)h->ncf * nw);
    int nc = 0;
    for (int ir = 0; ir < h->ncf; ++ir) {
      const uint8_t *q = iq + (size_t)ir * nw;
      if (ir == 0 || std::memcmp(q, q - nw, nw) != 0) {
        rows.insert(rows.end(), q, q + nw);
        ++nc;
      }
      conf[ir] = nc - 1;
    }
    L.nconf = nc;
    GG_TRY(L.dIq.alloc((size_t)nc * nw));
    GG_TRY(L.dConf.alloc(h->ncf));
    GG_TRY(L.dConfDiag.alloc(nc));
    GG_CUDA(cudaMemcpyAsync(L.dIq.p, rows.data(), rows.size(), cudaMemcpyHostToDevice, ctx->stream));
    GG_CUDA(cudaMemcpyAsync(L.dConf.p, conf.data(), conf.size() * sizeof(int32_t), cudaMemcpyHostToDevice,
                            ctx->stream));
    GG_CUDA(cudaStreamSynchronize(ctx->stream));  // rows and conf are host temporaries
  }
  GG_TRY(L.dLab.alloc(nlab));
  GG_TRY(L.dStart.alloc(nlab + 1));
  GG_TRY(L.dLoc.alloc(ncontr));
  GG_TRY(L.dCoeff.alloc(ncontr));
  // the coefficients (two thirds of the bytes) travel on the second stream
  // while the assembly plan, which reads them only in its last step, is
  // built from the labels and LOC on the context stream
  if (!ctx->aux) GG_CUDA(cudaStreamCreate(&ctx->aux));
  if (!ctx->aux_done) GG_CUDA(cudaEventCreateWithFlags(&ctx->aux_done, cudaEventDisableTiming));
  // concatenate lists; label starts are shifted to global contribution offsets
  std::vector<int64_t> st;
  st.reserve(nlab + 1);
  int64_t c0 = 0, l0 = 0;
  for (int i = 0; i < nlists; ++i) {
    const gg_list *x = ls[i];
    if (x->nlab == 0) continue;
    const int64_t nc = x->start[x->nlab];
    for (int64_t l = 0; l < x->nlab; ++l) st.push_back(c0 + x->start[l]);
    GG_CUDA(cudaMemcpyAsync(L.dLab.p + l0, x->lab, x->nlab * sizeof(int32_t), cudaMemcpyHostToDevice, ctx->stream));
    if (nc) {
      GG_CUDA(cudaMemcpyAsync(L.dLoc.p + c0, x->loc, nc * sizeof(int32_t), cudaMemcpyHostToDevice, ctx->stream));
      GG_CUDA(cudaMemcpyAsync(L.dCoeff.p + c0, x->coeff, nc * sizeof(double), cudaMemcpyHostToDevice, ctx->aux));
    }
    c0 += nc;
    l0 += x->nlab;
  }
  GG_CUDA(cudaEventRecord(ctx->aux_done, ctx->aux));
  st.push_back(c0);
  GG_CUDA(cudaMemcpyAsync(L.dStart.p, st.data(), st.size() * sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream));
  L.valid = true;
  h->emt_valid = false;
  h->sym_vals_valid = false;
  int st_plan = GG_OK;
  const std::vector<int> *key = rk_structure_key(ctx);
  ctx->stats[29] = 0;
  if (key && ctx->rk.valid && L.kmaxf <= ctx->rk.kloop) {
    if (!ctx->ev_mid) GG_CUDA(cudaEventCreate(&ctx->ev_mid));
    GG_CUDA(cudaEventRecord(ctx->ev_mid, ctx->stream));
    st_plan = build_plan(ctx, h, L, ctx->aux_done);
    if (st_plan != GG_OK) L.plan_key.clear();
  }
  // the coefficients and the host arrays' copies are done before returning
  GG_CUDA(cudaStreamWaitEvent(ctx->stream, ctx->aux_done, 0));
  GG_CUDA(cudaStreamSynchronize(ctx->aux));
  if (st_plan != GG_OK) {
    L.valid = false;
    return st_plan;
  }
  double ms = 0;
  GG_TRY(timer_stop(ctx, &ms));  // synchronises: the host vector st may go
  ctx->stats[7] = ms;
  if (!L.plan_key.empty()) {
    float f = 0.f;  // the plan, from its first kernel to the end of the call
    GG_CUDA(cudaEventElapsedTime(&f, ctx->ev_mid, ctx->ev1));
    ctx->stats[29] = f;
  }
  return GG_OK;
}

// The assembly plan of lists L for the current R^k table: integral slots of
// every label (k_label_slots), a counting transpose of the contributions by
// LOC (k_count_loc, scans, k_scatter_perm) and a per-segment sort back into
// list order (k_sort_gather), plus the diagonal term list in the loop order
// of setham.f90:83-219. Kept in L until the lists or the table's index
// structure change.
// coeff_ready (may be null): an event after the upload of L.dCoeff, which
// only the last step (k_sort_gather) reads.
static int build_plan(gg_ctx *ctx, gg_hmat *h, Lists &L, cudaEvent_t coeff_ready) {
  cudaStream_t s = ctx->stream;
  const Orbitals &o = ctx->orb;
  const RkTable &rk = ctx->rk;
  const int nw = o.nw;
  const int64_t nnz = h->nnz, ncontr = L.ncontr;
  const long long nrk = rk.n;
  std::vector<DiagTerm> terms;
  auto iab_slot = [&](int a) { return (long long)nrk + (long long)(a - 1) * nw + (a - 1); };
  auto add = [&](int type, int a, int b, int k, double fac) -> int {
    DiagTerm t;
    t.type = type;
    t.a = a - 1;
    t.b = b - 1;
    t.full_a = o.nkj[a] + 1;
    t.full_b = o.nkj[b] + 1;
    t.fac = fac;
    if (type == 0)
      t.slot = iab_slot(a);
    else if (type == 1 || type == 2)
      t.slot = host_rk_pos(rk, nw, a, a, a, a, k);
    else if (type == 3)
      t.slot = host_rk_pos(rk, nw, a, b, a, b, 0);
    else
      t.slot = host_rk_pos(rk, nw, a, b, b, a, k);
    if (t.slot < 0) return fail(GG_ERR_STATE, "setham: diagonal integral missing from the R^k table");
    terms.push_back(t);
    return GG_OK;
  };
  for (int a = 1; a <= nw; ++a) GG_TRY(add(0, a, a, 0, 0.0));
  for (int a = 1; a <= nw; ++a) GG_TRY(add(1, a, a, 0, 0.0));
  {
    int km = 0, K = 0;
    do {
      K = K + 2;
      for (int a = 1; a <= nw; ++a) {
        const int k0 = o.nkj[a] - 1;
        km = std::max(k0, km);
        if (K > k0) continue;
        GG_TRY(add(2, a, a, K, clrx(o.nak[a], K, o.nak[a])));
      }
    } while (K < km);
  }
  for (int a = 1; a <= nw - 1; ++a)
    for (int b = a + 1; b <= nw; ++b) GG_TRY(add(3, a, b, 0, 0.0));
  {
    int km = 0, K = -1;
    do {
      K = K + 1;
      for (int a = 1; a <= nw - 1; ++a)
        for (int b = a + 1; b <= nw; ++b) {
          const int nja = o.nkj[a], njb = o.nkj[b];
          const int kmin = (o.nak[a] * o.nak[b] > 0) ? std::abs((nja - njb) / 2) : std::abs((nja - njb) / 2) + 1;
          if ((K - kmin) % 2 != 0) continue;
          const int kmx = (nja + njb) / 2;
          km = std::max(kmx, km);
          if (K < kmin || K > kmx) continue;
          GG_TRY(add(4, a, b, K, clrx(o.nak[a], K, o.nak[b])));
        }
    } while (K < km);
  }
  GG_TRY(L.pTerms.alloc(std::max<size_t>(1, terms.size() * sizeof(DiagTerm))));
  if (!terms.empty())
    GG_CUDA(cudaMemcpyAsync(L.pTerms.p, terms.data(), terms.size() * sizeof(DiagTerm), cudaMemcpyHostToDevice, s));
  L.nterms = (int)terms.size();
  DBuf<int32_t> cslot, perm;
  DBuf<int> cnt, fill, err;
  DBuf<int64_t> part;
  GG_TRY(cslot.alloc(ncontr));
  GG_TRY(perm.alloc(ncontr));
  GG_TRY(L.pSlot.alloc(ncontr));
  GG_TRY(L.pCoeff.alloc(ncontr));
  GG_TRY(cnt.alloc(nnz));
  GG_TRY(fill.alloc(nnz));
  GG_TRY(L.pOff.alloc(nnz + 1));
  GG_TRY(err.alloc(1));
  GG_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), s));
  GG_CUDA(cudaMemsetAsync(cnt.p, 0, nnz * sizeof(int), s));
  GG_CUDA(cudaMemsetAsync(fill.p, 0, nnz * sizeof(int), s));
  DBuf<int64_t> dLab0;
  GG_TRY(upload(dLab0, L.list_lab0.data(), L.list_lab0.size(), s));
  DBuf<int32_t> dKstart;
  GG_TRY(upload(dKstart, rk.kstart.data(), rk.kstart.size(), s));
  const int nlists = L.kmaxf + 2;
  if (L.nlab) {
    const int blocks = (int)std::min<int64_t>((L.nlab * 32 + 255) / 256, 65535);
    k_label_slots<<<blocks, 256, 0, s>>>(L.dLab.p, L.dStart.p, L.nlab, dLab0.p, nlists, nw, o.dNAK.p, rk.dInd.p,
                                         dKstart.p, rk.kloop, nrk, cslot.p, err.p); ::gg::note_launch();
    GG_CUDA(cudaGetLastError());
  }
  const int gblocks = ctx->sms * 8;
  if (ncontr) {
    k_count_loc<<<gblocks, 256, 0, s>>>(L.dLoc.p, ncontr, nnz, cnt.p, err.p); ::gg::note_launch();
    GG_CUDA(cudaGetLastError());
  }
  int herr = 0;
  GG_CUDA(cudaMemcpyAsync(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  GG_CUDA(cudaStreamSynchronize(s));
  if (herr == 1) return fail(GG_ERR_RANGE, "SETHAM: a list label has no integral (bad label or R^k not in the table)");
  if (herr == 2) return fail(GG_ERR_RANGE, "SETHAM: Error in computing contribution: LOC > NELMNT");
  {
    const int64_t chunk = 1 << 16;
    const int64_t nparts = (nnz + chunk - 1) / chunk;
    GG_TRY(part.alloc(nparts + 1));
    k_scan_blocks<<<(unsigned)nparts, 1024, 0, s>>>(cnt.p, nnz, part.p, chunk); ::gg::note_launch();
    k_scan_parts<<<1, 32, 0, s>>>(part.p, nparts); ::gg::note_launch();
    k_scan_final<<<(unsigned)nparts, 1024, 0, s>>>(cnt.p, nnz, part.p, chunk, L.pOff.p); ::gg::note_launch();
    GG_CUDA(cudaGetLastError());
  }
  if (coeff_ready) GG_CUDA(cudaStreamWaitEvent(s, coeff_ready, 0));
  if (ncontr) {
    k_scatter_perm<<<gblocks, 256, 0, s>>>(L.dLoc.p, ncontr, L.pOff.p, fill.p, perm.p); ::gg::note_launch();
    k_sort_gather<<<(unsigned)((nnz + 255) / 256), 256, 0, s>>>(L.pOff.p, nnz, perm.p, L.dCoeff.p, cslot.p,
                                                                L.pCoeff.p, L.pSlot.p);
    ::gg::note_launch();
    GG_CUDA(cudaGetLastError());
  }
  GG_CUDA(cudaStreamSynchronize(s));  // the temporaries are freed on return
  L.plan_key = *rk_structure_key(ctx);
  L.plan_nrk = nrk;
  return GG_OK;
}

int gg_setham_assemble(gg_ctx *ctx, gg_hmat *h, double *eav_out) {
  if (!ctx || !h || h->ctx != ctx) return fail(GG_ERR_ARG, "gg_setham_assemble: bad arguments");
  Lists &L = *h->lists;
  if (!L.valid) return fail(GG_ERR_STATE, "gg_setham_assemble: no lists (call gg_setham_upload)");
  if (!ctx->rk.valid) return fail(GG_ERR_STATE, "gg_setham_assemble: no R^k table (call gg_genintrk)");
  if (!ctx->iab_valid) return fail(GG_ERR_STATE, "gg_setham_assemble: no I(ab) table (call gg_iabint_table)");
  if (L.kmaxf > ctx->rk.kloop) return fail(GG_ERR_STATE, "gg_setham_assemble: R^k table does not reach KMAXF");
  GG_CUDA(cudaSetDevice(ctx->device));
  cudaStream_t s = ctx->stream;
  const Orbitals &o = ctx->orb;
  const RkTable &rk = ctx->rk;
  const int nw = o.nw, ncf = h->ncf;
  const int64_t nnz = h->nnz;
  GG_TRY(timer_start(ctx));
  const std::vector<int> *key = rk_structure_key(ctx);
  if (!key || L.plan_key != *key || L.plan_nrk != rk.n) {
    L.plan_key.clear();
    GG_TRY(build_plan(ctx, h, L, nullptr));
  }
  // combined integral array [VALTEIRK | I(ab)]
  const long long nrk = rk.n;
  GG_TRY(L.integ.alloc((size_t)nrk + (size_t)nw * nw));
  if (nrk) GG_CUDA(cudaMemcpyAsync(L.integ.p, rk.dVal.p, nrk * sizeof(double), cudaMemcpyDeviceToDevice, s));
  GG_CUDA(cudaMemcpyAsync(L.integ.p + nrk, ctx->dIab.p, (size_t)nw * nw * sizeof(double), cudaMemcpyDeviceToDevice,
                          s));
  // EMT = 0 ; diagonal pieces ; list contributions ; EAV shift
  GG_CUDA(cudaMemsetAsync(h->dEmt.p, 0, nnz * sizeof(double), s));
  k_diag_terms<<<(unsigned)(((int64_t)L.nconf * 32 + 255) / 256), 256, 0, s>>>(
      reinterpret_cast<const DiagTerm *>(L.pTerms.p), L.nterms, L.dIq.p, nw, L.nconf, L.integ.p, L.dConfDiag.p);
  k_diag_scatter<<<(ncf + 255) / 256, 256, 0, s>>>(L.dConf.p, L.dConfDiag.p, ncf, h->dIendc.p, h->dEmt.p);
  ::gg::note_launches(2);
  GG_CUDA(cudaGetLastError());
  k_assemble<<<(unsigned)((nnz + AS_WARPS * 32 - 1) / (AS_WARPS * 32)), AS_WARPS * 32, 0, s>>>(
      L.pOff.p, nnz, L.pCoeff.p, L.pSlot.p, L.integ.p, h->dEmt.p);
  ::gg::note_launch();
  GG_CUDA(cudaGetLastError());
  GG_TRY(h->dEav.alloc(1 + EAV_CTAS));
  k_eav_part<<<EAV_CTAS, 256, 0, s>>>(h->dIendc.p, ncf, h->dEmt.p, h->dEav.p + 1);
  k_eav_fin<<<1, 32, 0, s>>>(h->dEav.p + 1, ncf, h->dEav.p);
  k_eav_sub<<<(ncf + 255) / 256, 256, 0, s>>>(h->dIendc.p, ncf, h->dEav.p, h->dEmt.p, h->dDiag.p);
  ::gg::note_launches(3);
  GG_CUDA(cudaGetLastError());
  double eav = 0;
  GG_CUDA(cudaMemcpyAsync(&eav, h->dEav.p, sizeof(double), cudaMemcpyDeviceToHost, s));
  double ms = 0;
  GG_TRY(timer_stop(ctx, &ms));
  ctx->stats[2] = ms;
  h->eav = eav;
  h->emt_valid = true;
  h->sym_vals_valid = false;
  if (eav_out) *eav_out = eav;
  return GG_OK;
}

int gg_setham(gg_ctx *ctx, gg_hmat *h, const uint8_t *iq, const gg_list *tlist, int kmaxf, const gg_list *vlists,
              double *eav_out) {
  GG_TRY(gg_setham_upload(ctx, h, iq, tlist, kmaxf, vlists));
  return gg_setham_assemble(ctx, h, eav_out);
}

int gg_hmat_get_emt(gg_hmat *h, double *emt) {
  if (!h || !emt) return fail(GG_ERR_ARG, "gg_hmat_get_emt: bad arguments");
  if (!h->emt_valid) return fail(GG_ERR_STATE, "gg_hmat_get_emt: EMT not assembled");
  if (h->host_prec >= 0) return fail(GG_ERR_ARG, "gg_hmat_get_emt: a host-resident matrix keeps no EMT");
  GG_CUDA(cudaSetDevice(h->ctx->device));
  GG_CUDA(cudaMemcpyAsync(emt, h->dEmt.p, h->nnz * sizeof(double), cudaMemcpyDeviceToHost, h->ctx->stream));
  GG_CUDA(cudaStreamSynchronize(h->ctx->stream));
  return GG_OK;
}

int gg_hmat_set_emt(gg_hmat *h, const double *emt) {
  if (!h || !emt) return fail(GG_ERR_ARG, "gg_hmat_set_emt: bad arguments");
  if (h->host_prec >= 0) return fail(GG_ERR_ARG, "gg_hmat_set_emt: a host-resident matrix keeps no EMT");
  GG_CUDA(cudaSetDevice(h->ctx->device));
  GG_CUDA(cudaMemcpyAsync(h->dEmt.p, emt, h->nnz * sizeof(double), cudaMemcpyHostToDevice, h->ctx->stream));
  std::vector<double> d(h->ncf);
  for (int i = 0; i < h->ncf; ++i) d[i] = emt[h->hIendc[i + 1] - 1];
  GG_CUDA(cudaMemcpyAsync(h->dDiag.p, d.data(), h->ncf * sizeof(double), cudaMemcpyHostToDevice, h->ctx->stream));
  GG_CUDA(cudaStreamSynchronize(h->ctx->stream));
  h->emt_valid = true;
  h->sym_vals_valid = false;
  h->eav = 0.0;
  return GG_OK;
}

}  // extern "C"
