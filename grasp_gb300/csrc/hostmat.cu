// hostmat.cu - blocks whose matrix is not on the device, and the packed
// dense form.
//
// SPODMV (rci90/spodmv.f90:3) is rci's product for a block too large to keep
// in memory (rci90/maneig.f90:262-279): every product re-reads the lower
// triangle from rci.res. On GB300 the counterpart of "too large for memory"
// is "too large for HBM", and the next tier is the Grace host memory behind
// NVLink-C2C. gg_hmat_create_host builds the block's full symmetric matrix
// once, in pinned host memory, in exactly the form and entry order the
// device-resident matvec reads (spmv.cu: own row with the diagonal last,
// then the transposed entries in increasing source row), and points the
// matrix's symmetric arrays at it: the same kernels then read the entries
// over the link (coalesced row by row) while the vectors, their split copies
// and the diagonal stay in HBM. The sums are the resident ones, so a product
// is bit for bit the product of the same matrix kept on the device.
//
// DNICMV (rci90/dnicmv.f90:3) is the product with a dense lower triangle
// packed by rows (EMT(IBEG..IEND), IEND = IEND + ICOL). gg_hmat_create_packed
// gives that triangle the sparse structure with every entry present, so the
// SPICMV2 path computes DNICMV's product.
#include <algorithm>
#include <cstring>
#include <vector>

#include "gg_internal.cuh"

namespace gg {
namespace {

// rows kept for MANEIG's leading block (INIEST2's sub-matrix: 2000 rows for
// rci, 4000 for rmcdhf)
constexpr int LEAD_ROWS = 4000;

// pinned, mapped host array owned by h; *dev is its device address
template <class T>
int host_array(gg_hmat *h, size_t count, T **host, DBuf<T> &dev) {
  void *p = nullptr;
  const cudaError_t e = cudaHostAlloc(&p, std::max<size_t>(count, 1) * sizeof(T), cudaHostAllocMapped);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(GG_ERR_NOMEM, std::string("cudaHostAlloc: ") + cudaGetErrorString(e));
  }
  h->host_bufs.push_back(p);
  void *dp = nullptr;
  GG_CUDA(cudaHostGetDevicePointer(&dp, p, 0));
  *host = static_cast<T *>(p);
  dev.release();
  dev.p = static_cast<T *>(dp);
  dev.n = count;
  dev.own = false;
  return GG_OK;
}

// the checks of gg_hmat_create, on the host
int check_structure(const char *who, int ncf, int64_t nnz, const int64_t *iendc, const int32_t *irow) {
  if (iendc[0] != 0 || iendc[ncf] != nnz) return fail(GG_ERR_ARG, std::string(who) + ": IENDC(0) must be 0, IENDC(NCF) = NNZ");
  for (int i = 1; i <= ncf; ++i)
    if (iendc[i] <= iendc[i - 1]) return fail(GG_ERR_ARG, std::string(who) + ": empty row (the diagonal is required)");
  for (int r = 0; r < ncf; ++r) {
    const int64_t p1 = iendc[r + 1] - 1;
    if (irow[p1] != r + 1) return fail(GG_ERR_ARG, std::string(who) + ": row does not end with its diagonal");
    for (int64_t p = iendc[r]; p < p1; ++p)
      if (irow[p] < 1 || irow[p] > r) return fail(GG_ERR_ARG, std::string(who) + ": IROW outside the lower triangle");
  }
  return GG_OK;
}

// The full symmetric CSR of the block in pinned host memory: row c holds its
// own entries in stored order (diagonal last, value EMT - eav), then entry
// (r, c) of every later row r in increasing r (the order of spmv.cu's
// device build). GG_FP64 keeps FP64 values and int32 columns; GG_SPLIT keeps
// hi + lo FP32 values (zero at the diagonal, whose FP64 term is added apart)
// and 16-bit columns for NCF <= 65536.
int build_host_sym(gg_hmat *h, const int64_t *iendc, const int32_t *irow, const double *emt, double eav,
                   int precision) {
  const int ncf = h->ncf;
  const int64_t total = 2 * h->nnz - ncf;
  std::vector<int64_t> cnt(ncf, 0);
  for (int r = 0; r < ncf; ++r)
    for (int64_t p = iendc[r]; p < iendc[r + 1] - 1; ++p) ++cnt[irow[p] - 1];
  int64_t *ptr = nullptr;
  GG_TRY(host_array(h, (size_t)ncf + 1, &ptr, h->dSymPtr));
  ptr[0] = 0;
  for (int c = 0; c < ncf; ++c) ptr[c + 1] = ptr[c] + (iendc[c + 1] - iendc[c]) + cnt[c];
  if (ptr[ncf] != total) return fail(GG_ERR_STATE, "gg_hmat_create_host: inconsistent structure");
  const bool split = (precision == GG_SPLIT);
  const bool c16 = split && ncf <= 65536;
  int32_t *col = nullptr;
  unsigned short *col16 = nullptr;
  double *val = nullptr;
  float *hi = nullptr, *lo = nullptr;
  if (c16)
    GG_TRY(host_array(h, (size_t)total, &col16, h->dSymCol16));
  else
    GG_TRY(host_array(h, (size_t)total, &col, h->dSymCol));
  if (split) {
    GG_TRY(host_array(h, (size_t)total, &hi, h->dSymHi));
    GG_TRY(host_array(h, (size_t)total, &lo, h->dSymLo));
  } else {
    GG_TRY(host_array(h, (size_t)total, &val, h->dSymVal));
  }
  auto put = [&](int64_t pos, int c, double v, bool diagonal) {
    if (c16)
      col16[pos] = (unsigned short)c;
    else
      col[pos] = c;
    if (!split) {
      val[pos] = v;
    } else if (diagonal) {
      hi[pos] = 0.f;
      lo[pos] = 0.f;
    } else {
      const float fh = (float)v;
      hi[pos] = fh;
      lo[pos] = (float)(v - (double)fh);
    }
  };
  std::vector<int64_t> cur(ncf);
  for (int c = 0; c < ncf; ++c) {
    const int64_t p0 = iendc[c], p1 = iendc[c + 1];
    for (int64_t p = p0; p < p1; ++p) {
      const bool diagonal = (p == p1 - 1);
      put(ptr[c] + (p - p0), irow[p] - 1, diagonal ? emt[p] - eav : emt[p], diagonal);
    }
    cur[c] = ptr[c] + (p1 - p0);
  }
  for (int r = 0; r < ncf; ++r)
    for (int64_t p = iendc[r]; p < iendc[r + 1] - 1; ++p) {
      const int c = irow[p] - 1;
      put(cur[c]++, r, emt[p], false);
    }
  h->sym_nnz = total;
  h->sym_col16 = c16;
  return GG_OK;
}

// streaming read of n float4 from (host) memory, U loads in flight per
// thread; one sum per block keeps the loads
__global__ void __launch_bounds__(256) k_stream_read(const float4 *__restrict__ src, int64_t n,
                                                     float *__restrict__ sink) {
  constexpr int U = 4;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  float acc = 0.f;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += U * stride) {
    float4 v[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t j = i + u * stride;
      v[u] = j < n ? src[j] : make_float4(0.f, 0.f, 0.f, 0.f);
    }
#pragma unroll
    for (int u = 0; u < U; ++u) acc += v[u].x + v[u].y + v[u].z + v[u].w;
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(sink + blockIdx.x, acc);
}

}  // namespace

int leading_block_host(gg_hmat *h, int ns, gg_hmat **out) {
  if (ns > (int)h->hIendc.size() - 1 || h->hIendc[ns] > (int64_t)h->hLeadIrow.size())
    return fail(GG_ERR_ARG, "leading block: more rows than kept with the host matrix");
  gg_ctx *ctx = h->ctx;
  cudaStream_t s = ctx->stream;
  const int64_t nnz = h->hIendc[ns];
  gg_hmat *b = new gg_hmat;
  b->ctx = ctx;
  b->ncf = ns;
  b->nnz = nnz;
  b->hIendc.assign(h->hIendc.begin(), h->hIendc.begin() + ns + 1);
  std::vector<double> d(ns);
  for (int i = 0; i < ns; ++i) d[i] = h->hLeadEmt[b->hIendc[i + 1] - 1];
  int st = b->dIendc.alloc(ns + 1);
  if (!st) st = b->dIrow.alloc(nnz);
  if (!st) st = b->dEmt.alloc(nnz);
  if (!st) st = b->dDiag.alloc(ns);
  if (!st && (cudaMemcpyAsync(b->dIendc.p, b->hIendc.data(), (ns + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, s) ||
              cudaMemcpyAsync(b->dIrow.p, h->hLeadIrow.data(), nnz * sizeof(int32_t), cudaMemcpyHostToDevice, s) ||
              cudaMemcpyAsync(b->dEmt.p, h->hLeadEmt.data(), nnz * sizeof(double), cudaMemcpyHostToDevice, s) ||
              cudaMemcpyAsync(b->dDiag.p, d.data(), ns * sizeof(double), cudaMemcpyHostToDevice, s) ||
              cudaStreamSynchronize(s)))
    st = fail(GG_ERR_CUDA, "leading block: copy failed");
  if (st) {
    delete b;
    return st;
  }
  b->emt_valid = true;
  *out = b;
  return GG_OK;
}

}  // namespace gg

using namespace gg;

extern "C" {

int gg_hmat_create_host(gg_ctx *ctx, int ncf, int64_t nnz, const int64_t *iendc, const int32_t *irow,
                        const double *emt, double eav, int precision, gg_hmat **out) {
  if (!ctx || !out || !iendc || !irow || !emt || ncf < 1 || nnz < ncf)
    return fail(GG_ERR_ARG, "gg_hmat_create_host: bad arguments");
  if (precision != GG_FP64 && precision != GG_SPLIT) return fail(GG_ERR_ARG, "gg_hmat_create_host: bad precision");
  *out = nullptr;
  GG_TRY(check_structure("gg_hmat_create_host", ncf, nnz, iendc, irow));
  GG_CUDA(cudaSetDevice(ctx->device));
  gg_hmat *h = new gg_hmat;
  h->ctx = ctx;
  h->ncf = ncf;
  h->nnz = nnz;
  h->host_prec = precision;
  h->hIendc.assign(iendc, iendc + ncf + 1);
  const int nl = std::min(ncf, LEAD_ROWS);
  h->hLeadIrow.assign(irow, irow + iendc[nl]);
  h->hLeadEmt.assign(emt, emt + iendc[nl]);
  for (int i = 0; i < nl; ++i) h->hLeadEmt[iendc[i + 1] - 1] -= eav;
  std::vector<double> d(ncf);
  for (int i = 0; i < ncf; ++i) d[i] = emt[iendc[i + 1] - 1] - eav;
  int s = build_host_sym(h, iendc, irow, emt, eav, precision);
  if (s == GG_OK) s = h->dDiag.alloc(ncf);
  if (s == GG_OK &&
      (cudaMemcpyAsync(h->dDiag.p, d.data(), ncf * sizeof(double), cudaMemcpyHostToDevice, ctx->stream) ||
       cudaStreamSynchronize(ctx->stream)))
    s = fail(GG_ERR_CUDA, "gg_hmat_create_host: copy failed");
  if (s != GG_OK) {
    delete h;
    return s;
  }
  h->eav = eav;
  h->emt_valid = true;
  h->sym_valid = true;
  h->sym_vals_valid = true;
  *out = h;
  return GG_OK;
}

int gg_hmat_host_precision(gg_hmat *h) {
  if (!h) return fail(GG_ERR_ARG, "gg_hmat_host_precision: null matrix");
  return h->host_prec;
}

int gg_spodmv(gg_ctx *ctx, gg_hmat *h, int m, const double *b, double *c) {
  if (!h || h->host_prec < 0) return fail(GG_ERR_ARG, "gg_spodmv: not a host-resident matrix");
  return gg_spicmv2(ctx, h, m, b, c, h->host_prec);
}

int gg_host_read_timing(gg_ctx *ctx, size_t bytes, int mode, int iters, double *ms_per_pass) {
  if (!ctx || bytes < 16 || iters < 1 || (mode != 0 && mode != 1) || !ms_per_pass)
    return fail(GG_ERR_ARG, "gg_host_read_timing: bad arguments");
  GG_CUDA(cudaSetDevice(ctx->device));
  bytes &= ~(size_t)15;
  void *hp = nullptr;
  GG_CUDA(cudaHostAlloc(&hp, bytes, cudaHostAllocMapped));
  std::memset(hp, 0, bytes);
  void *dp = nullptr;
  int st = GG_OK;
  if (cudaHostGetDevicePointer(&dp, hp, 0) != cudaSuccess) st = fail(GG_ERR_CUDA, "gg_host_read_timing: mapping");
  DBuf<float> sink;
  DBuf<char> dst;
  const int blocks = 4 * ctx->sms;
  if (st == GG_OK) st = sink.alloc(blocks);
  if (st == GG_OK && mode == 1) st = dst.alloc(bytes);
  auto pass = [&]() -> int {
    if (mode == 0) {
      k_stream_read<<<blocks, 256, 0, ctx->stream>>>(static_cast<const float4 *>(dp), (int64_t)(bytes / 16),
                                                      sink.p);
      ::gg::note_launch();
    } else {
      GG_CUDA(cudaMemcpyAsync(dst.p, hp, bytes, cudaMemcpyHostToDevice, ctx->stream));
    }
    GG_CUDA(cudaGetLastError());
    return GG_OK;
  };
  if (st == GG_OK && sink.p) st = cudaMemsetAsync(sink.p, 0, blocks * sizeof(float), ctx->stream) == cudaSuccess
                                      ? GG_OK : fail(GG_ERR_CUDA, "gg_host_read_timing: memset");
  if (st == GG_OK) st = pass();  // warm-up
  if (st == GG_OK) st = timer_start(ctx);
  for (int it = 0; it < iters && st == GG_OK; ++it) st = pass();
  double ms = 0;
  if (st == GG_OK) st = timer_stop(ctx, &ms);
  cudaStreamSynchronize(ctx->stream);
  cudaFreeHost(hp);
  if (st != GG_OK) return st;
  *ms_per_pass = ms / iters;
  return GG_OK;
}

int gg_hmat_create_packed(gg_ctx *ctx, int ncf, const double *ap, gg_hmat **out) {
  if (!ctx || !out || !ap || ncf < 1) return fail(GG_ERR_ARG, "gg_hmat_create_packed: bad arguments");
  *out = nullptr;
  const int64_t nnz = (int64_t)ncf * (ncf + 1) / 2;
  std::vector<int64_t> iendc((size_t)ncf + 1);
  std::vector<int32_t> irow((size_t)nnz);
  iendc[0] = 0;
  for (int r = 0; r < ncf; ++r) {
    iendc[r + 1] = iendc[r] + r + 1;
    for (int j = 0; j <= r; ++j) irow[iendc[r] + j] = j + 1;
  }
  gg_hmat *h = nullptr;
  GG_TRY(gg_hmat_create(ctx, ncf, nnz, iendc.data(), irow.data(), &h));
  const int st = gg_hmat_set_emt(h, ap);
  if (st != GG_OK) {
    gg_hmat_destroy(h);
    return st;
  }
  *out = h;
  return GG_OK;
}

}  // extern "C"
