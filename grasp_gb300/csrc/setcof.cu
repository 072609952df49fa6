// setcof.cu - SETCOF (rmcdhf90/setcof.f90) on the device: the coefficient
// lists of the direct (YPOT), exchange (XPOT) and one-body (DACON)
// potentials of an orbital, from the blocks' T/V lists and the mixing
// coefficients.
//
// The reference reads mcp.30/31/32+k from disk once per orbital and SCF
// iteration and, for each label that involves the orbital, adds its
// contributions' DSUBRS(IR, IC) COEFF (dsubrs.f90: the generalized weight of
// the CSF pair). Those label sums do not depend on the orbital except
// through the final 1/UCF(J), so here one pass computes them for every label
// of every block (one thread per label, contributions added in list order,
// as the reference does), together with the diagonal FCO/GCO sums of every
// (J, IB, K) (one thread each, CSFs in block and row order). A call for
// orbital J then only filters and merges the labels on the host, in the
// reference's order (FCO, GCO, the T list by block, the V^k lists by k and
// block), so its lists are the reference's entry for entry.
#include <algorithm>
#include <cstring>
#include <memory>
#include <tuple>
#include <utility>
#include <vector>

#include "gg_internal.cuh"

namespace gg {

// the prepared sums of the last gg_setcof_prepare
struct SetcofState {
  int nblocks = 0, eol = 0;
  int kmaxf = -1;                             // largest over the blocks
  std::vector<int> bkmaxf;                    // per block
  std::vector<std::vector<int64_t>> lab0;     // per block: first label of each list (T, V0..)
  std::vector<std::vector<int32_t>> labs;     // per block: the labels of all its lists
  std::vector<std::vector<double>> sums;      // per block: each label's sum of DSUBRS COEFF (x2 off the diagonal)
  std::vector<double> fco, gco;               // [J][IB][K] diagonal sums (index below)
  int kdim = 0;
  size_t idx(int j, int ib, int k) const { return ((size_t)(j - 1) * nw + (ib - 1)) * kdim + k; }
  int nw = 0;
  // per orbital, the labels that name it: T labels as (block, label), V
  // labels as (k, block, label), each in the order SETCOF visits them
  std::vector<std::vector<std::pair<int, int64_t>>> tref;
  std::vector<std::vector<std::tuple<int, int, int64_t>>> vref;
};

namespace {

// DSUBRS (rmcdhf90/dsubrs.f90:20-33): EOL, sum over the block's levels of
// EVEC(I) EVEC(J) WT(level); otherwise WT(I) on the diagonal, 0 elsewhere.
// ev holds the levels' coefficients by CSF ([ncf][nev]: one CSF's nev
// values contiguous), the same products in the same order.
__device__ __forceinline__ double dsubrs(int eol, int i, int j, int nev, const double *ev, const double *wt) {
  if (eol) {
    const double *a = ev + (size_t)(i - 1) * nev, *b = ev + (size_t)(j - 1) * nev;
    double d = 0.0;
    for (int k = 0; k < nev; ++k) d = d + a[k] * b[k] * wt[k];
    return d;
  }
  return i == j ? wt[i - 1] : 0.0;
}

// the levels' coefficients by CSF: evr[r][k] = evec[k][r]
__global__ void k_by_csf(const double *__restrict__ evec, int ncf, int nev, double *__restrict__ evr) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < (int64_t)ncf * nev;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(e / nev), k = (int)(e % nev);
    evr[e] = evec[(size_t)k * ncf + r];
  }
}

// DSUBRS(IR, IR) of every CSF
__global__ void k_dsubrs_diag(int eol, int ncf, int nev, const double *__restrict__ ev, const double *__restrict__ wt,
                              double *__restrict__ d) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r < ncf) d[r] = dsubrs(eol, r + 1, r + 1, nev, ev, wt);
}

// the column owning each EMT position (ICLMN of the mcp records, 1-based)
__global__ void k_owner(const int64_t *__restrict__ iendc, int ncf, int32_t *__restrict__ owner) {
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (w >= ncf) return;
  for (int64_t p = iendc[w] + lane; p < iendc[w + 1]; p += 32) owner[p] = w + 1;
}

// SUM over a label's contributions (setcof.f90:242-251 for the T list,
// :302-311 for the V lists): CONTR = DSUBRS(IR, IC) COEFF, doubled when
// IR != IC, added in list order; IR = IROW(INDX), IC = ICLMN. One warp per
// label: the lanes form 32 consecutive CONTR at a time (their gathers in
// flight together) into shared memory, lane 0 adds them in order.
constexpr int LS_WARPS = 4;
__global__ void __launch_bounds__(LS_WARPS * 32) k_label_sums(int64_t nlab, const int64_t *__restrict__ start,
                                                              const int32_t *__restrict__ loc,
                                                              const double *__restrict__ coeff,
                                                              const int32_t *__restrict__ irow,
                                                              const int32_t *__restrict__ owner, int eol, int nev,
                                                              const double *__restrict__ ev,
                                                              const double *__restrict__ wt,
                                                              double *__restrict__ out) {
  __shared__ double cs[LS_WARPS][32];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t l = blockIdx.x * (int64_t)LS_WARPS + w;
  if (l >= nlab) return;
  double sum = 0.0;
  const int64_t i0 = start[l], i1 = start[l + 1];
  for (int64_t c = i0; c < i1; c += 32) {
    const int64_t i = c + lane;
    double contr = 0.0;
    if (i < i1) {
      const int p = loc[i] - 1;
      const int ir = irow[p], ic = owner[p];
      contr = dsubrs(eol, ir, ic, nev, ev, wt) * coeff[i];
      if (ir != ic) contr = contr + contr;
    }
    cs[w][lane] = contr;
    __syncwarp();
    if (lane == 0) {
      const int n = (int)min((int64_t)32, i1 - c);
      for (int t = 0; t < n; ++t) sum = sum + cs[w][t];
    }
    __syncwarp();
  }
  if (lane == 0) out[l] = sum;
}

// one block's CSFs for the diagonal sums
struct DiagBlock {
  int ncf;
  const double *d;        // DSUBRS(IR, IR)
  const uint8_t *iq;      // [nconf][nw]
  const int32_t *conf;    // [ncf]
};

// one diagonal sum: kind 0 FCO(K, IR, J, IB) (fco.f90), 1 GCO(K, IR, J, IB)
// (gco.f90); c = CLRX of the item
struct DiagItem {
  int kind, j, ib, k;
  int fullj, fullb;  // 2j + 1 of J and IB (a full subshell)
  double c;
};

// SUMR = sum over blocks and CSFs of DSUBRS(IR, IR) FCO/GCO (setcof.f90:82-90,
// 121-129), CSFs in block and row order. One warp per sum: the lanes form
// 32 consecutive terms, lane 0 adds them in order.
__global__ void __launch_bounds__(LS_WARPS * 32) k_diag_sums(const DiagItem *__restrict__ items, int nitems,
                                                             const DiagBlock *__restrict__ blocks, int nblocks,
                                                             int nw, double *__restrict__ out) {
  __shared__ double cs[LS_WARPS][32];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int t = blockIdx.x * LS_WARPS + w;
  if (t >= nitems) return;
  const DiagItem it = items[t];
  double sumr = 0.0;
  for (int b = 0; b < nblocks; ++b) {
    const DiagBlock B = blocks[b];
    for (int r0 = 1; r0 <= B.ncf; r0 += 32) {
      const int ir = r0 + lane;
      double term = 0.0;
      if (ir <= B.ncf) {
      const uint8_t *q = B.iq + (size_t)B.conf[ir - 1] * nw;
      const int qa = q[it.j - 1], qb = q[it.ib - 1];
      double f = 0.0;
      if (it.kind == 0) {
        if (it.j == it.ib) {
          if (it.k == 0) {
            f = (double)((qa * (qa - 1)) / 2);
          } else if (qa == it.fullj) {
            const double fac = it.c * (double)qa;
            f = -0.5 * fac * fac;
          }
        } else if (it.k == 0) {
          f = (double)(qa * qb);
        }
      } else if (qa == it.fullj || qb == it.fullb) {
        f = -(double)(qa * qb) * it.c * it.c;
      }
      term = B.d[ir - 1] * f;
      }
      cs[w][lane] = term;
      __syncwarp();
      if (lane == 0) {
        const int n = min(32, B.ncf - r0 + 1);
        for (int u = 0; u < n; ++u) sumr = sumr + cs[w][u];
      }
      __syncwarp();
    }
  }
  if (lane == 0) out[t] = sumr;
}

template <class T> int upv(DBuf<T> &b, const std::vector<T> &h, cudaStream_t s) {
  GG_TRY(b.alloc(std::max<size_t>(1, h.size())));
  if (!h.empty()) GG_CUDA(cudaMemcpyAsync(b.p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, s));
  return GG_OK;
}

// appends (label, value) or, when merge and the label is already listed,
// adds to its value (the reference's "check it against the previously
// recorded" search: the first entry with that label)
void put(std::vector<int32_t> &lab, std::vector<double> &val, int32_t l, double v, bool merge) {
  if (merge)
    for (size_t i = 0; i < lab.size(); ++i)
      if (lab[i] == l) {
        val[i] = val[i] + v;
        return;
      }
  lab.push_back(l);
  val.push_back(v);
}

}  // namespace
}  // namespace gg

using namespace gg;

extern "C" {

int gg_setcof_prepare(gg_ctx *ctx, int nblocks, gg_hmat *const *h, const int *nev, const double *const *evec,
                      const double *const *wt, int eol) {
  if (!ctx || nblocks < 1 || !h || !wt || (eol && (!nev || !evec)))
    return fail(GG_ERR_ARG, "gg_setcof_prepare: bad arguments");
  GG_TRY(ensure_orbitals(ctx));
  GG_CUDA(cudaSetDevice(ctx->device));
  const Orbitals &o = ctx->orb;
  const int nw = o.nw;
  cudaStream_t s = ctx->stream;
  auto st = std::make_shared<SetcofState>();
  st->nblocks = nblocks;
  st->eol = eol ? 1 : 0;
  st->nw = nw;
  std::vector<DBuf<double>> devec(nblocks), dwt(nblocks), ddiag(nblocks);
  std::vector<DiagBlock> hb(nblocks);
  for (int b = 0; b < nblocks; ++b) {
    gg_hmat *m = h[b];
    if (!m || m->ctx->device != ctx->device) return fail(GG_ERR_ARG, "gg_setcof_prepare: bad block");
    Lists &L = *m->lists;
    if (!L.valid) return fail(GG_ERR_STATE, "gg_setcof_prepare: a block has no lists (gg_setham_upload)");
    if (m->host_prec >= 0) return fail(GG_ERR_ARG, "gg_setcof_prepare: a host-resident block has no lists");
    const int ncf = m->ncf, ne = eol ? nev[b] : 0;
    if (eol && (ne < 1 || !evec[b] || !wt[b])) return fail(GG_ERR_ARG, "gg_setcof_prepare: missing levels");
    if (!eol && !wt[b]) return fail(GG_ERR_ARG, "gg_setcof_prepare: missing CSF weights");
    if (eol) {
      DBuf<double> tmp;
      GG_TRY(tmp.alloc((size_t)ncf * ne));
      GG_TRY(devec[b].alloc((size_t)ncf * ne));
      GG_CUDA(cudaMemcpyAsync(tmp.p, evec[b], (size_t)ncf * ne * sizeof(double), cudaMemcpyHostToDevice, s));
      k_by_csf<<<std::max(1, std::min(4 * ctx->sms, (int)(((int64_t)ncf * ne + 255) / 256))), 256, 0, s>>>(
          tmp.p, ncf, ne, devec[b].p);
      ::gg::note_launch();
      GG_CUDA(cudaStreamSynchronize(s));  // tmp is freed here
      GG_TRY(dwt[b].alloc(ne));
      GG_CUDA(cudaMemcpyAsync(dwt[b].p, wt[b], ne * sizeof(double), cudaMemcpyHostToDevice, s));
    } else {
      GG_TRY(dwt[b].alloc(ncf));
      GG_CUDA(cudaMemcpyAsync(dwt[b].p, wt[b], ncf * sizeof(double), cudaMemcpyHostToDevice, s));
    }
    // every label's sum
    DBuf<int32_t> owner;
    DBuf<double> dsum;
    GG_TRY(owner.alloc(std::max<int64_t>(1, m->nnz)));
    k_owner<<<(unsigned)(((int64_t)ncf * 32 + 255) / 256), 256, 0, s>>>(m->dIendc.p, ncf, owner.p);
    ::gg::note_launch();
    GG_TRY(dsum.alloc(std::max<int64_t>(1, L.nlab)));
    if (L.nlab > 0) {
      k_label_sums<<<(unsigned)((L.nlab + LS_WARPS - 1) / LS_WARPS), LS_WARPS * 32, 0, s>>>(
          L.nlab, L.dStart.p, L.dLoc.p, L.dCoeff.p,
                                                                   m->dIrow.p, owner.p, st->eol, ne, devec[b].p,
                                                                   dwt[b].p, dsum.p);
      ::gg::note_launch();
    }
    GG_CUDA(cudaGetLastError());
    st->labs.emplace_back(L.nlab);
    st->sums.emplace_back(L.nlab);
    if (L.nlab > 0) {
      GG_CUDA(cudaMemcpyAsync(st->labs.back().data(), L.dLab.p, L.nlab * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
      GG_CUDA(cudaMemcpyAsync(st->sums.back().data(), dsum.p, L.nlab * sizeof(double), cudaMemcpyDeviceToHost, s));
    }
    GG_CUDA(cudaStreamSynchronize(s));  // owner and dsum are freed here
    st->lab0.push_back(L.list_lab0);
    st->bkmaxf.push_back(L.kmaxf);
    st->kmaxf = std::max(st->kmaxf, L.kmaxf);
    GG_TRY(ddiag[b].alloc(ncf));
    k_dsubrs_diag<<<(ncf + 255) / 256, 256, 0, s>>>(st->eol, ncf, ne, devec[b].p, dwt[b].p, ddiag[b].p);
    ::gg::note_launch();
    hb[b] = DiagBlock{ncf, ddiag[b].p, L.dIq.p, L.dConf.p};
  }
  // the diagonal sums of every (J, IB, K) SETCOF asks for
  int jmax = 0;
  for (int a = 1; a <= nw; ++a) jmax = std::max(jmax, o.nkj[a]);
  st->kdim = jmax + 2;
  std::vector<DiagItem> items;
  std::vector<size_t> where;
  for (int j = 1; j <= nw; ++j)
    for (int ib = 1; ib <= nw; ++ib) {
      const int kmax = (ib == j) ? o.nkj[j] - 1 : 0;
      for (int k = 0; k <= kmax; k += 2) {
        items.push_back(DiagItem{0, j, ib, k, o.nkj[j] + 1, o.nkj[ib] + 1, k > 0 ? clrx_host(o.nak[j], k, o.nak[j]) : 0.0});
        where.push_back(st->idx(j, ib, k) * 2);
      }
      if (ib == j) continue;
      const int kmin = (o.nak[j] * o.nak[ib] > 0) ? std::abs((o.nkj[j] - o.nkj[ib]) / 2)
                                                   : std::abs((o.nkj[j] - o.nkj[ib]) / 2) + 1;
      for (int k = kmin; k <= (o.nkj[j] + o.nkj[ib]) / 2; k += 2) {
        items.push_back(DiagItem{1, j, ib, k, o.nkj[j] + 1, o.nkj[ib] + 1, clrx_host(o.nak[j], k, o.nak[ib])});
        where.push_back(st->idx(j, ib, k) * 2 + 1);
      }
    }
  DBuf<DiagItem> ditems;
  DBuf<DiagBlock> dblocks;
  DBuf<double> dout;
  GG_TRY(upv(ditems, items, s));
  GG_TRY(upv(dblocks, hb, s));
  GG_TRY(dout.alloc(std::max<size_t>(1, items.size())));
  if (!items.empty()) {
    k_diag_sums<<<(unsigned)((items.size() + LS_WARPS - 1) / LS_WARPS), LS_WARPS * 32, 0, s>>>(
        ditems.p, (int)items.size(), dblocks.p, nblocks, nw, dout.p);
    ::gg::note_launch();
  }
  GG_CUDA(cudaGetLastError());
  std::vector<double> hv(items.size());
  if (!items.empty()) GG_CUDA(cudaMemcpyAsync(hv.data(), dout.p, hv.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
  GG_CUDA(cudaStreamSynchronize(s));
  st->fco.assign((size_t)nw * nw * st->kdim, 0.0);
  st->gco.assign((size_t)nw * nw * st->kdim, 0.0);
  for (size_t t = 0; t < items.size(); ++t) (where[t] % 2 ? st->gco : st->fco)[where[t] / 2] = hv[t];
  // the labels of each orbital, in visiting order
  st->tref.assign(nw + 1, {});
  st->vref.assign(nw + 1, {});
  for (int b = 0; b < nblocks; ++b)
    for (int64_t l = st->lab0[b][0]; l < st->lab0[b][1]; ++l) {
      const int32_t lab = st->labs[b][l];
      const int ia = lab % KEYORB, ib = lab / KEYORB;
      if (ia >= 1 && ia <= nw) st->tref[ia].push_back({b, l});
      if (ib != ia && ib >= 1 && ib <= nw) st->tref[ib].push_back({b, l});
    }
  for (int k = 0; k <= st->kmaxf; ++k)
    for (int b = 0; b < nblocks; ++b) {
      if (k > st->bkmaxf[b]) continue;
      for (int64_t l = st->lab0[b][k + 1]; l < st->lab0[b][k + 2]; ++l) {
        int32_t lab = st->labs[b][l];
        int ix[4];
        for (int t = 0; t < 4; ++t) {
          ix[t] = lab % KEYORB;
          lab /= KEYORB;
        }
        for (int t = 0; t < 4; ++t) {
          bool seen = false;
          for (int u = 0; u < t; ++u) seen = seen || ix[u] == ix[t];
          if (!seen && ix[t] >= 1 && ix[t] <= nw) st->vref[ix[t]].push_back(std::make_tuple(k, b, l));
        }
      }
    }
  ctx->setcof = st;
  return GG_OK;
}

int gg_setcof(gg_ctx *ctx, int j, double ucfj, int cap, int *ny, int32_t *nya, double *ya, int *nx, int32_t *nxa,
              double *xa, int *nd, int32_t *nda, double *da) {
  if (!ctx || !ny || !nx || !nd || cap < 0 || (cap > 0 && (!nya || !ya || !nxa || !xa || !nda || !da)))
    return fail(GG_ERR_ARG, "gg_setcof: bad arguments");
  const auto st = std::static_pointer_cast<SetcofState>(ctx->setcof);
  if (!st) return fail(GG_ERR_STATE, "gg_setcof: call gg_setcof_prepare first");
  const Orbitals &o = ctx->orb;
  const int nw = st->nw, KEY = KEYORB;
  if (j < 1 || j > nw || o.nw != nw) return fail(GG_ERR_ARG, "gg_setcof: orbital outside the orbital set");
  std::vector<int32_t> ly, lx, ld;
  std::vector<double> vy, vx, vd;
  // Y from FCO (setcof.f90:73-105): NYA = K + IB KEY (KEY + 1)
  {
    int64_t ilabel = 0;
    const int64_t nwterm = (int64_t)KEY * (KEY + 1);
    for (int ib = 1; ib <= nw; ++ib) {
      ilabel += nwterm;
      const int kmax = (ib == j) ? o.nkj[j] - 1 : 0;
      for (int k = 0; k <= kmax; k += 2) {
        const double sumr = st->fco[st->idx(j, ib, k)];
        const double ykab = (ib == j) ? 2.0 * sumr / ucfj : sumr / ucfj;
        ly.push_back((int32_t)(k + ilabel));
        vy.push_back(ykab);
      }
    }
  }
  // X from GCO (:107-147): NXA = K + KEY J + IB KEY^2 (KEY + 1)
  {
    int64_t ilabel = (int64_t)KEY * j;
    const int64_t nwterm = (int64_t)KEY * KEY * (KEY + 1);
    for (int ib = 1; ib <= nw; ++ib) {
      ilabel += nwterm;
      if (ib == j) continue;
      const int kmin = (o.nak[j] * o.nak[ib] > 0) ? std::abs((o.nkj[j] - o.nkj[ib]) / 2)
                                                   : std::abs((o.nkj[j] - o.nkj[ib]) / 2) + 1;
      for (int k = kmin; k <= (o.nkj[j] + o.nkj[ib]) / 2; k += 2) {
        lx.push_back((int32_t)(k + ilabel));
        vx.push_back(st->gco[st->idx(j, ib, k)] / ucfj);
      }
    }
  }
  // DA from the T lists, block by block (:188-285)
  for (const auto &r : st->tref[j]) {
    const int b = r.first;
    const int64_t l = r.second;
    const int32_t lab = st->labs[b][l];
    const int ia = lab % KEY, ibb = lab / KEY;
    const double sum = 0.5 * st->sums[b][l] / ucfj;
    put(ld, vd, ia == j ? ibb : ia, sum, b > 0);
  }
  // the V^k lists, k by k and block by block (:287-515)
  for (const auto &r : st->vref[j]) {
      const int k = std::get<0>(r), b = std::get<1>(r);
      const bool merge = b > 0;
      {
        const int64_t l = std::get<2>(r);
        int32_t lab = st->labs[b][l];
        int ix[4];
        ix[3] = lab % KEY;
        lab /= KEY;
        ix[1] = lab % KEY;
        lab /= KEY;
        ix[2] = lab % KEY;
        ix[0] = lab / KEY;
        int irank = 0;
        for (int t = 0; t < 4; ++t) irank += (ix[t] == j);
        if (irank == 0) continue;
        const double sum = 0.5 * st->sums[b][l] / ucfj;
        auto at = [&](int p) { return ix[(p - 1) % 4]; };  // INDEXS(IL), IL wrapped into 1..4
        if (irank == 1) {
          int ithis = 0;
          for (int iind = 1; iind <= 4; ++iind) {
            if (ix[iind - 1] != j) continue;
            ithis = ((at(iind + 2) * KEY + at(iind + 3)) * KEY + at(iind + 1)) * KEY + k;
            break;
          }
          put(lx, vx, ithis, sum, merge);
        } else if (irank == 2) {
          int loc1 = 0, loc2 = 0, found = 0;
          for (int iind = 1; iind <= 4; ++iind) {
            if (ix[iind - 1] != j) continue;
            if (found == 0) {
              loc1 = iind;
              found = 1;
            } else {
              loc2 = iind;
              break;
            }
          }
          if (loc2 - loc1 == 2) {
            const int ithis = (at(loc1 + 3) * KEY + at(loc1 + 1)) * KEY + k;
            put(ly, vy, ithis, sum + sum, merge);
          } else {
            const int ithis = ((at(loc1 + 2) * KEY + at(loc1 + 3)) * KEY + at(loc1 + 1)) * KEY + k;
            put(lx, vx, ithis, sum + sum, merge);
          }
        } else if (irank == 3) {
          int ithis = 0, ithis2 = 0;
          for (int iind = 1; iind <= 4; ++iind) {
            if (ix[iind - 1] == j) continue;
            const int other = ix[iind - 1];
            ithis = (other * KEY + j) * KEY + k;
            ithis2 = ((other * KEY + j) * KEY + j) * KEY + k;
          }
          put(ly, vy, ithis, sum + sum, merge);
          put(lx, vx, ithis2, sum, merge);
        } else {
          put(ly, vy, (j * KEY + j) * KEY + k, 4.0 * sum, merge);
        }
      }
    }
  *ny = (int)ly.size();
  *nx = (int)lx.size();
  *nd = (int)ld.size();
  if ((int)ly.size() > cap || (int)lx.size() > cap || (int)ld.size() > cap)
    return fail(GG_ERR_RANGE, "gg_setcof: a list is longer than cap (the counts are set)");
  std::copy(ly.begin(), ly.end(), nya);
  std::copy(vy.begin(), vy.end(), ya);
  std::copy(lx.begin(), lx.end(), nxa);
  std::copy(vx.begin(), vx.end(), xa);
  std::copy(ld.begin(), ld.end(), nda);
  std::copy(vd.begin(), vd.end(), da);
  return GG_OK;
}

}  // extern "C"
