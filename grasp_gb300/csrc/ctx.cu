// ctx.cu - context, grid (RADGRD/SETQIC) and orbital state of libgraspgpu.
#include <atomic>
#include <cmath>
#include <cstring>

#include "gg_internal.cuh"

namespace gg {

static thread_local std::string g_last_error;
static std::atomic<long long> g_launches{0};
static std::atomic<long long> g_allocs{0};

void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
void note_launches(long long m) { g_launches.fetch_add(m, std::memory_order_relaxed); }
void note_alloc() { g_allocs.fetch_add(1, std::memory_order_relaxed); }
void set_error(const std::string &msg) { g_last_error = msg; }
int fail(int status, const std::string &msg) {
  g_last_error = msg;
  return status;
}

int timer_start(gg_ctx *ctx) {
  GG_CUDA(cudaEventRecord(ctx->ev0, ctx->stream));
  return GG_OK;
}
int timer_stop(gg_ctx *ctx, double *ms) {
  GG_CUDA(cudaEventRecord(ctx->ev1, ctx->stream));
  GG_CUDA(cudaEventSynchronize(ctx->ev1));
  float f = 0.f;
  GG_CUDA(cudaEventElapsedTime(&f, ctx->ev0, ctx->ev1));
  *ms = f;
  return GG_OK;
}

// libgcc's __powidf2 algorithm: the value gfortran computes for
// R(2:N)**K with a run-time integer K (yzk.f90:76).
static double powi(double x, int m) {
  unsigned n = m < 0 ? -(unsigned)m : (unsigned)m;
  double y = (n % 2) ? x : 1.0;
  while (n >>= 1) {
    x = x * x;
    if (n % 2) y = y * x;
  }
  return m < 0 ? 1.0 / y : y;
}

}  // namespace gg

using namespace gg;

extern "C" {

const char *gg_last_error(void) { return g_last_error.c_str(); }
int gg_version(void) { return 1; }

int gg_ctx_create(int device, gg_ctx **out) {
  if (!out) return fail(GG_ERR_ARG, "gg_ctx_create: out is NULL");
  *out = nullptr;
  int ndev = 0;
  GG_CUDA(cudaGetDeviceCount(&ndev));
  if (device < 0 || device >= ndev) return fail(GG_ERR_ARG, "gg_ctx_create: no such device");
  GG_CUDA(cudaSetDevice(device));
  {
    // device buffers come from the default pool, which keeps what is freed
    cudaMemPool_t pool = nullptr;
    GG_CUDA(cudaDeviceGetDefaultMemPool(&pool, device));
    uint64_t keep = UINT64_MAX;
    GG_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
  }
  gg_ctx *c = new gg_ctx;
  c->device = device;
  cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, device);
  // a blocking stream: the legacy stream on which device buffers are
  // allocated and freed (gg_internal.cuh, DBuf) is ordered with it
  cudaError_t e = cudaStreamCreate(&c->stream);
  if (e == cudaSuccess) e = cudaEventCreate(&c->ev0);
  if (e == cudaSuccess) e = cudaEventCreate(&c->ev1);
  if (e != cudaSuccess) {
    delete c;
    return fail(GG_ERR_CUDA, std::string("gg_ctx_create: ") + cudaGetErrorString(e));
  }
  *out = c;
  return GG_OK;
}

int gg_ctx_destroy(gg_ctx *ctx) {
  if (!ctx) return GG_OK;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  for (cudaEvent_t &e : ctx->marks)
    if (e) cudaEventDestroy(e);
  if (ctx->ev0) cudaEventDestroy(ctx->ev0);
  if (ctx->ev1) cudaEventDestroy(ctx->ev1);
  if (ctx->ev_mid) cudaEventDestroy(ctx->ev_mid);
  if (ctx->aux) {
    cudaStreamSynchronize(ctx->aux);
    cudaStreamDestroy(ctx->aux);
  }
  if (ctx->aux_done) cudaEventDestroy(ctx->aux_done);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  gg::rk_cache_free(ctx->rk.cache);
  delete ctx;
  return GG_OK;
}

int gg_release_memory(int device) {
  int ndev = 0;
  GG_CUDA(cudaGetDeviceCount(&ndev));
  if (device < 0 || device >= ndev) return fail(GG_ERR_ARG, "gg_release_memory: no such device");
  GG_CUDA(cudaSetDevice(device));
  GG_CUDA(cudaDeviceSynchronize());
  cudaMemPool_t pool = nullptr;
  GG_CUDA(cudaDeviceGetDefaultMemPool(&pool, device));
  GG_CUDA(cudaMemPoolTrimTo(pool, 0));
  return GG_OK;
}

int gg_ctx_synchronize(gg_ctx *ctx) {
  if (!ctx) return fail(GG_ERR_ARG, "null context");
  GG_CUDA(cudaStreamSynchronize(ctx->stream));
  return GG_OK;
}

int gg_set_grid(gg_ctx *ctx, int n, double rnt, double h, double c, const double *r, const double *rp,
                const double *rpor, const double *zz) {
  if (!ctx) return fail(GG_ERR_ARG, "null context");
  if (n < 20 || n > 100000 || !(h > 0) || !(rnt > 0) || !(c > 0))
    return fail(GG_ERR_ARG, "gg_set_grid: bad n/rnt/h/c");
  GG_CUDA(cudaSetDevice(ctx->device));
  Grid &g = ctx->grid;
  g.n = n;
  g.rnt = rnt;
  g.h = h;
  g.c = c;
  const size_t sz = (size_t)n + GPAD + 10;
  g.R.assign(sz, 0.0);
  g.RP.assign(sz, 0.0);
  g.RPOR.assign(sz, 0.0);
  g.ZZ.assign(sz, 0.0);
  const int np10 = n + 10;
  if (r && rp && rpor) {
    for (int i = 1; i <= np10; ++i) {
      g.R[i] = r[i - 1];
      g.RP[i] = rp[i - 1];
      g.RPOR[i] = rpor[i - 1];
    }
  } else {
    // RADGRD, HP = 0 branch (lib9290/radgrd.f90:38-60)
    g.R[1] = 0.0;
    g.RPOR[1] = 0.0;
    g.RP[1] = rnt;
    const double eph = std::exp(h);
    double ett = 1.0;
    for (int i = 2; i <= np10; ++i) {
      ett = eph * ett;
      const double ettm1 = ett - 1.0;
      g.R[i] = rnt * ettm1;
      g.RP[i] = rnt * ett;
      g.RPOR[i] = ett / ettm1;
    }
  }
  if (zz)
    for (int i = 1; i <= n; ++i) g.ZZ[i] = zz[i - 1];
  // SETQIC (lib9290/setqic.f90:157-188): the 13-point derivative weights are
  // the rationals of the 13-point Lagrange first-derivative formula over the
  // common denominator 12! = 479001600; computed here from their definition
  // (exact in double) rather than tabulated.
  QuadConst &q = g.q;
  {
    // d/dx of the Lagrange basis l_j at node i on nodes 0..12, times 12!.
    // l_j'(x_i) = prod_{m != j} (i - m) / prod_{m != j} (j - m) for i != j,
    //           = sum_{m != i} 1/(i - m) for i == j.
    const double fact12 = 479001600.0;
    for (int i = 0; i < 13; ++i)
      for (int j = 0; j < 13; ++j) {
        double v;
        if (i != j) {
          double num = 1.0, den = 1.0;
          for (int m = 0; m < 13; ++m) {
            if (m == j) continue;
            den *= (double)(j - m);
            if (m != i) num *= (double)(i - m);
          }
          v = num / den * fact12;
        } else {
          double s = 0.0;
          for (int m = 0; m < 13; ++m)
            if (m != i) s += fact12 / (double)(i - m);
          v = s;
        }
        q.A13[i][j] = std::nearbyint(v) * (1.0 / fact12);
      }
  }
  const double factor = h / 720.0;
  // Five-point Newton-Cotes numerators over 720 (setqic.f90 C5NUM(I, J),
  // rows I = 2..5, columns J = 2..4: the semi-open starting formulae used for
  // ZK(2:4) in YZK) and the closed formula 224, 1024, 384, 1024, 224.
  const double c5num[4][3] = {{646.0, 992.0, 918.0}, {-264.0, 192.0, 648.0}, {106.0, 32.0, 378.0},
                              {-19.0, -8.0, -27.0}};
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < 4; ++i) q.CNC5C[i][j] = factor * c5num[i][j];
  q.C1 = factor * 224.0;
  q.C2 = factor * 1024.0;
  q.C3 = factor * 384.0;
  q.C4 = q.C1 + q.C1;
  {
    const double h2 = h * h, h3 = h2 * h;  // ACCY = H**6 (getcid.f90:262)
    q.accy = h3 * h3;
  }
  q.h = h;
  q.c = c;
  q.n = n;
  // device copies
  GG_TRY(g.dR.alloc(sz));
  GG_TRY(g.dRP.alloc(sz));
  GG_TRY(g.dRPOR.alloc(sz));
  GG_TRY(g.dZZ.alloc(sz));
  GG_CUDA(cudaMemcpy(g.dR.p, g.R.data(), sz * 8, cudaMemcpyHostToDevice));
  GG_CUDA(cudaMemcpy(g.dRP.p, g.RP.data(), sz * 8, cudaMemcpyHostToDevice));
  GG_CUDA(cudaMemcpy(g.dRPOR.p, g.RPOR.data(), sz * 8, cudaMemcpyHostToDevice));
  GG_CUDA(cudaMemcpy(g.dZZ.p, g.ZZ.data(), sz * 8, cudaMemcpyHostToDevice));
  // YZK's power tables (yzk.f90:70-95), rows k = 1..KLIMIT; row 0 of RTTK
  // holds RM = 1/R.
  g.np = (int)sz;
  std::vector<double> pw((size_t)4 * (KLIMIT + 1) * g.np, 0.0);
  auto P = [&](int t, int k, int i) -> double & { return pw[((size_t)t * (KLIMIT + 1) + k) * g.np + i]; };
  for (int i = 2; i <= n; ++i) P(0, 0, i) = 1.0 / g.R[i];
  for (int k = 1; k <= KLIMIT; ++k)
    for (int i = 2; i <= n; ++i) {
      const double t = powi(g.R[i], k);
      P(0, k, i) = t;
      P(1, k, i) = 1.0 / t;
      P(2, k, i) = t * g.R[i];
      P(3, k, i) = 1.0 / (t * g.R[i]);
    }
  GG_TRY(g.dPow.alloc(pw.size()));
  GG_CUDA(cudaMemcpy(g.dPow.p, pw.data(), pw.size() * 8, cudaMemcpyHostToDevice));
  {
    std::vector<double> hd((size_t)3 * g.np, 0.0);
    for (int i = 2; i + 1 < g.np && i + 1 <= n + 9; ++i) {
      hd[i] = 1.0 / std::log(g.R[i + 1] / g.R[i]);
      hd[(size_t)g.np + i] = g.RP[i] / g.RP[i + 1];
      hd[(size_t)2 * g.np + i] = g.R[i] / g.RP[i];
    }
    GG_TRY(g.dHead.alloc(hd.size()));
    GG_CUDA(cudaMemcpy(g.dHead.p, hd.data(), hd.size() * 8, cudaMemcpyHostToDevice));
  }
  // a new grid invalidates everything computed on the old one
  ctx->rk.valid = false;
  ctx->iab_valid = false;
  return GG_OK;
}

int gg_get_grid(gg_ctx *ctx, double *r, double *rp, double *rpor) {
  if (!ctx || ctx->grid.n == 0) return fail(GG_ERR_STATE, "gg_get_grid: no grid");
  const Grid &g = ctx->grid;
  for (int i = 1; i <= g.n + 10; ++i) {
    if (r) r[i - 1] = g.R[i];
    if (rp) rp[i - 1] = g.RP[i];
    if (rpor) rpor[i - 1] = g.RPOR[i];
  }
  return GG_OK;
}

int gg_set_orbitals(gg_ctx *ctx, int nw, int ld, const int *nak, const int *mf, const double *pf,
                    const double *qf) {
  if (!ctx) return fail(GG_ERR_ARG, "null context");
  if (ctx->grid.n == 0) return fail(GG_ERR_STATE, "gg_set_orbitals: set the grid first");
  const int n = ctx->grid.n;
  if (nw <= 0 || nw >= KEYORB || ld < n || !nak || !mf || !pf || !qf)
    return fail(GG_ERR_ARG, "gg_set_orbitals: bad arguments");
  GG_CUDA(cudaSetDevice(ctx->device));
  Orbitals &o = ctx->orb;
  o.nw = nw;
  o.ld = ld;
  o.nak.assign(nw + 1, 0);
  o.mf.assign(nw + 1, 0);
  o.nkl.assign(nw + 1, 0);
  o.nkj.assign(nw + 1, 0);
  for (int j = 1; j <= nw; ++j) {
    const int kap = nak[j - 1];
    if (kap == 0 || std::abs(kap) > KLIMIT) return fail(GG_ERR_ARG, "gg_set_orbitals: bad kappa");
    if (mf[j - 1] < 3 || mf[j - 1] > n) return fail(GG_ERR_ARG, "gg_set_orbitals: MF out of range");
    o.nak[j] = kap;
    o.mf[j] = mf[j - 1];
    o.nkl[j] = kap > 0 ? kap : -kap - 1;
    o.nkj[j] = 2 * std::abs(kap) - 1;
  }
  // device copies with ld rounded up so that each orbital starts 64-byte aligned
  const int ldd = (n + GPAD + 7) / 8 * 8;
  std::vector<double> hp((size_t)nw * ldd, 0.0), hq((size_t)nw * ldd, 0.0);
  for (int j = 0; j < nw; ++j)
    for (int i = 0; i < n; ++i) {
      hp[(size_t)j * ldd + i] = pf[(size_t)j * ld + i];
      hq[(size_t)j * ldd + i] = qf[(size_t)j * ld + i];
    }
  o.ld = ldd;
  GG_TRY(o.dPF.alloc(hp.size()));
  GG_TRY(o.dQF.alloc(hq.size()));
  GG_CUDA(cudaMemcpy(o.dPF.p, hp.data(), hp.size() * 8, cudaMemcpyHostToDevice));
  GG_CUDA(cudaMemcpy(o.dQF.p, hq.data(), hq.size() * 8, cudaMemcpyHostToDevice));
  GG_TRY(o.dMF.alloc(nw + 1));
  GG_TRY(o.dNAK.alloc(nw + 1));
  GG_CUDA(cudaMemcpy(o.dMF.p, o.mf.data(), (nw + 1) * sizeof(int), cudaMemcpyHostToDevice));
  GG_CUDA(cudaMemcpy(o.dNAK.p, o.nak.data(), (nw + 1) * sizeof(int), cudaMemcpyHostToDevice));
  ctx->rk.valid = false;
  ctx->iab_valid = false;
  return GG_OK;
}

double gg_stage_stat(gg_ctx *ctx, int which) {
  if (!ctx || which < 0 || which >= 34) return -1.0;
  return ctx->stats[which];
}

long long gg_launch_count(void) { return g_launches.load(); }
long long gg_alloc_count(void) { return g_allocs.load(); }

int gg_batched_tune_info(gg_ctx *ctx, int *chosen, int *nvariants, double *ms) {
  if (!ctx) return fail(GG_ERR_ARG, "gg_batched_tune_info: no context");
  if (ctx->btune_var < 0) return fail(GG_ERR_STATE, "gg_batched_tune_info: no batched solve on this context yet");
  if (chosen) *chosen = ctx->btune_var;
  if (nvariants) *nvariants = 6;
  if (ms)
    for (int i = 0; i < 6; ++i) ms[i] = ctx->btune_ms[i];
  return GG_OK;
}

int gg_test_stall_rk_tile(gg_ctx *ctx, int tile) {
  if (!ctx) return fail(GG_ERR_ARG, "gg_test_stall_rk_tile: no context");
  ctx->test_stall_tile = tile < 0 ? -1 : tile;
  return GG_OK;
}

int gg_projected_eig(int n, const double *ap, int m, int mvec, double *w, double *z) {
  if (n < 1 || !ap || m < 1 || m > n || mvec < 0 || mvec > m || !w || (mvec > 0 && !z))
    return fail(GG_ERR_ARG, "gg_projected_eig: bad arguments");
  const int st = gg::sym_eig_lowest(n, ap, m, mvec, w, z);
  if (st == -1) return fail(GG_ERR_ARG, "gg_projected_eig: bad arguments");
  if (st != 0) return fail(GG_ERR_CONVERGE, "gg_projected_eig: eigenvalue search did not finish");
  return GG_OK;
}

int gg_host_register(void *p, size_t bytes) {
  if (!p || bytes == 0) return fail(GG_ERR_ARG, "gg_host_register: bad arguments");
  GG_CUDA(cudaHostRegister(p, bytes, cudaHostRegisterDefault));
  return GG_OK;
}

int gg_host_unregister(void *p) {
  if (!p) return fail(GG_ERR_ARG, "gg_host_unregister: null pointer");
  GG_CUDA(cudaHostUnregister(p));
  return GG_OK;
}

int gg_event_record(gg_ctx *ctx, int slot) {
  if (!ctx || slot < 0 || slot >= 8) return fail(GG_ERR_ARG, "gg_event_record: bad slot");
  GG_CUDA(cudaSetDevice(ctx->device));
  if (!ctx->marks[slot]) GG_CUDA(cudaEventCreate(&ctx->marks[slot]));
  GG_CUDA(cudaEventRecord(ctx->marks[slot], ctx->stream));
  return GG_OK;
}

int gg_event_elapsed(gg_ctx *ctx, int a, int b, double *ms) {
  if (!ctx || a < 0 || a >= 8 || b < 0 || b >= 8 || !ctx->marks[a] || !ctx->marks[b] || !ms)
    return fail(GG_ERR_ARG, "gg_event_elapsed: bad slots");
  GG_CUDA(cudaEventSynchronize(ctx->marks[b]));
  float f = 0.f;
  GG_CUDA(cudaEventElapsedTime(&f, ctx->marks[a], ctx->marks[b]));
  *ms = f;
  return GG_OK;
}

}  // extern "C"

namespace gg {
int ensure_grid(gg_ctx *ctx) {
  if (!ctx) return fail(GG_ERR_ARG, "null context");
  if (ctx->grid.n == 0) return fail(GG_ERR_STATE, "no grid: call gg_set_grid first");
  return GG_OK;
}
int ensure_orbitals(gg_ctx *ctx) {
  GG_TRY(ensure_grid(ctx));
  if (ctx->orb.nw == 0) return fail(GG_ERR_STATE, "no orbitals: call gg_set_orbitals first");
  return GG_OK;
}
}  // namespace gg
