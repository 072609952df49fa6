// gg_internal.cuh - shared state and helpers of libgraspgpu (not part of the ABI).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <memory>
#include <string>
#include <utility>
#include <vector>

#include "../../include/grasp_gpu.h"

namespace gg {

void set_error(const std::string &msg);
int fail(int status, const std::string &msg);
// counts this library's kernel launches (reported by gg_launch_count)
void note_launch();
// adds m (possibly negative: launches recorded while a graph was captured)
void note_launches(long long m);
// counts this library's device and pinned-host allocations (gg_alloc_count)
void note_alloc();

#define GG_CUDA(call)                                                                   \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess)                                                              \
      return ::gg::fail(GG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

#define GG_TRY(call)             \
  do {                           \
    int s_ = (call);             \
    if (s_ != GG_OK) return s_;  \
  } while (0)

// Programmatic dependent launch. A kernel launched by launch_pdl may be
// scheduled while the kernel before it on the stream is still running, so
// that its launch overlaps that kernel's last wave; it must call pdl_wait()
// before it touches memory (griddepcontrol.wait returns once every
// prerequisite grid has completed and its writes are visible). pdl_trigger()
// lets the next such kernel be scheduled (it only starts waiting: the
// ordering is kept by its own pdl_wait). In a stream capture the launches
// become programmatic graph edges.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*k)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                              Args &&...args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k, std::forward<Args>(args)...);
}

constexpr int KLIMIT = 20;   // yzk.f90:54 (KLIMIT), kkstart_C KMAX
constexpr int KEYORB = 215;  // parameter_def_M.f90:22
constexpr int GPAD = 16;     // padding slots after NNN1 in device grid arrays

// Device buffer with RAII. Memory comes from the device's default memory
// pool in the order of the legacy stream (cudaMallocAsync/cudaFreeAsync on
// stream 0): the contexts' streams are blocking streams, so a free is
// ordered after all work issued before it and an allocation before all
// work issued after it. The pool keeps freed memory (gg_ctx_create sets no
// release threshold), so a new matrix or workspace of a size seen before
// maps nothing; gg_release_memory hands it back to the driver.
template <class T> struct DBuf {
  T *p = nullptr;
  size_t n = 0;
  bool own = true;  // false: borrowed from another buffer, never freed here
  DBuf() = default;
  DBuf(const DBuf &) = delete;
  DBuf &operator=(const DBuf &) = delete;
  ~DBuf() { release(); }
  void release() {
    if (p && own) cudaFreeAsync(p, 0);
    p = nullptr;
    n = 0;
    own = true;
  }
  // refer to o's memory without owning it (o must outlive this buffer)
  void borrow(const DBuf &o) {
    release();
    p = o.p;
    n = o.n;
    own = false;
  }
  int alloc(size_t count) {
    if (count <= n && p) return GG_OK;
    release();
    if (count == 0) count = 1;
    cudaError_t e = cudaMallocAsync(reinterpret_cast<void **>(&p), count * sizeof(T), 0);
    note_alloc();
    if (e != cudaSuccess) {
      p = nullptr;
      cudaGetLastError();
      return fail(GG_ERR_NOMEM, std::string("cudaMallocAsync: ") + cudaGetErrorString(e));
    }
    n = count;
    return GG_OK;
  }
};

// Grid constants passed by value to kernels (SETQIC results, DEF_C values).
struct QuadConst {
  double C1, C2, C3, C4;
  double CNC5C[4][3];  // CNC5C(i=2..5, j=2..4) -> [i-2][j-2]
  double A13[13][13];  // LIC13_C A(13,13), row-major [i-1][j-1]
  double accy;         // ACCY = H**6
  double h, c;         // H, speed of light C
  int n;               // N
};

struct Grid {
  int n = 0;
  double rnt = 0, h = 0, c = 0;
  std::vector<double> R, RP, RPOR, ZZ;  // host, 1-based, size n + GPAD + 10
  QuadConst q{};
  DBuf<double> dR, dRP, dRPOR, dZZ;     // device, 1-based like the host copies
  DBuf<double> dPow;                    // [4][KLIMIT+1][np]: RTTK, RTTKM, RTTK1, RTTKM1 ; k = 0 row holds RM
  // QUAD's power-law head term at point i (quad.f90:61-75) needs
  // log(R(i+1)/R(i)), RP(i)/RP(i+1) and R(i)/RP(i): [3][np] per point
  // (1 / the logarithm, the two ratios), 0 below i = 2
  DBuf<double> dHead;
  int np = 0;                           // row pitch of dPow (>= n + GPAD)
};

struct Orbitals {
  int nw = 0, ld = 0;
  std::vector<int> nak, mf, nkl, nkj;   // 1-based host copies
  DBuf<double> dPF, dQF;                // [nw][ld]
  DBuf<int> dMF, dNAK;                  // 1-based
};

// GENINTBREIT1/2's tables (breit.cu): type 1 and type 2
struct BreitTable {
  bool valid = false;
  int j2max = 0;
  int64_t n = 0;
  std::vector<int32_t> kstart;          // KSTARTBREIT(0:j2max+1), 1-based positions
  std::vector<int32_t> hInd;            // INDTP
  std::vector<double> hVal;             // VALTP
};

struct RkCache;  // radial.cu: GENINTRK's orbital-set structure, reused between calls
void rk_cache_free(RkCache *c);

struct RkTable {
  RkCache *cache = nullptr;
  int kloop = -1, j2max = 0;
  int64_t n = 0;
  std::vector<int32_t> kstart;          // KSTART(0:kloop+1)
  std::vector<int32_t> hInd;            // host copy of INDTEIRK
  DBuf<int32_t> dInd;
  DBuf<double> dVal;
  bool valid = false;
};

struct Lists {  // device copies of one block's T/V lists, concatenated in SETHAM order
  int kmaxf = -1;
  int64_t nlab = 0, ncontr = 0;
  std::vector<int64_t> list_lab0;       // first label of each list (T, V0..Vkmaxf), size kmaxf + 3
  DBuf<int32_t> dLab;                   // [nlab]
  DBuf<int64_t> dStart;                 // [nlab + 1], global contribution offsets
  DBuf<int32_t> dLoc;                   // [ncontr]
  DBuf<double> dCoeff;                  // [ncontr]
  DBuf<uint8_t> dIq;                    // [nconf][nw] occupations of each run of equal IQ rows
  DBuf<int32_t> dConf;                  // [ncf] the run of each CSF
  DBuf<double> dConfDiag;               // [nconf] diagonal pieces per run, last assembly
  int nconf = 0;
  bool valid = false;
  // assembly plan (setham.cu): the contributions sorted by LOC with their
  // integral slots, and the diagonal terms; it depends only on these lists
  // and on the R^k table's index structure, whose key it records
  std::vector<int> plan_key;
  int64_t plan_nrk = -1;
  DBuf<int64_t> pOff;                   // [nnz + 1] contribution offsets per EMT position
  DBuf<int32_t> pSlot;                  // [ncontr] integral slot, sorted order
  DBuf<double> pCoeff;                  // [ncontr] coefficient, sorted order
  DBuf<unsigned char> pTerms;           // diagonal terms (setham.cu's DiagTerm records)
  int nterms = 0;
  DBuf<double> integ;                   // [VALTEIRK | I(ab)] of the last assembly
};

}  // namespace gg

struct gg_ctx {
  int device = 0;
  int sms = 152;                        // multiprocessors of the device
  cudaStream_t stream = nullptr;
  gg::Grid grid;
  gg::Orbitals orb;
  gg::RkTable rk;
  gg::DBuf<double> dIab;                // [nw * nw]
  bool iab_valid = false;
  double stats[40] = {};
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  cudaEvent_t ev_mid = nullptr;  // a point inside a timed call (gg_maneig: after its structures)
  cudaEvent_t marks[8] = {};  // gg_event_record slots
  int test_stall_tile = -1;     // gg_test_stall_rk_tile: one tensor-core tile withholds a copy, once
  int btune_var = -1;           // the last gg_maneig_batched's matvec variant and the
  double btune_ms[6] = {};      // tuner's times of its variants (ms)
  cudaStream_t aux = nullptr;   // second blocking stream: uploads that overlap work on `stream`
  cudaEvent_t aux_done = nullptr;
  gg::BreitTable breit[2];      // GENINTBREIT1, GENINTBREIT2
  std::shared_ptr<void> setcof; // setcof.cu: the sums of the last gg_setcof_prepare
  std::shared_ptr<void> pot_stage;  // radial.cu: pinned staging of the potentials' coefficient lists
  size_t pot_stage_bytes = 0;
};

struct gg_hmat {
  gg_ctx *ctx = nullptr;
  int ncf = 0;
  int64_t nnz = 0;
  std::vector<int64_t> hIendc;          // IENDC(0:ncf)
  gg::DBuf<int64_t> dIendc;             // [ncf + 1]
  gg::DBuf<int32_t> dIrow;              // [nnz]
  gg::DBuf<double> dEmt;                // [nnz]
  gg::DBuf<double> dDiag;               // [ncf]
  gg::DBuf<double> dEav;                // EAV of the last assembly
  bool emt_valid = false;
  double eav = 0.0;
  std::shared_ptr<gg::Lists> lists = std::make_shared<gg::Lists>();  // shared with views
  gg_hmat *base = nullptr;              // a view's source (views borrow its structure)
  int views = 0;                        // views of this matrix still alive
  bool dead = false;                    // destroyed while views were alive
  // full symmetric CSR used by the matvec (both triangles, diagonal first)
  bool sym_valid = false;
  int64_t sym_nnz = 0;
  gg::DBuf<int64_t> dSymPtr;            // [ncf + 1]
  gg::DBuf<int32_t> dSymCol;            // [sym_nnz]
  gg::DBuf<unsigned short> dSymCol16;   // [sym_nnz] when ncf <= 65536
  bool sym_col16 = false;
  gg::DBuf<int64_t> dSymSrc;            // [sym_nnz] index into EMT
  gg::DBuf<double> dSymVal;             // [sym_nnz] FP64 values
  gg::DBuf<float> dSymHi, dSymLo;       // [sym_nnz] split values
  gg::DBuf<float2> dXs;                 // [ncf] split copy of the input vector
  gg::DBuf<float2> dXb;                 // [ncf][m even] split copies of m input vectors, by row
  bool sym_vals_valid = false;
  // autotuner overrides (spmv.cu): variant per kernel (0 block, 1 single) and
  // m, -1 = the tuned choice
  int tune_force[2][17];
  gg_hmat() {
    for (auto &r : tune_force)
      for (int &v : r) v = -1;
  }
  // kept between gg_maneig calls (davidson.cu): the leading block of the
  // INIEST2 stage (its structure and symmetric matvec structure; values
  // recopied per call) and the Davidson workspaces with their CUDA graphs,
  // by stage and precision
  gg_hmat *lead = nullptr;
  std::shared_ptr<void> dvd_cache[4];
  // a matrix kept in host memory (gg_hmat_create_host): the precision its
  // symmetric form was built for (-1: the matrix is on the device), the
  // pinned host arrays the dSym* buffers borrow, and the leading rows
  // (lower triangle by rows, diagonal shifted) for MANEIG's leading block
  int host_prec = -1;
  std::vector<void *> host_bufs;
  std::vector<int32_t> hLeadIrow;
  std::vector<double> hLeadEmt;
  ~gg_hmat() {
    for (auto &c : dvd_cache) c.reset();
    delete lead;
    for (void *p : host_bufs) cudaFreeHost(p);
  }
};

namespace gg {
// radial.cu
int ensure_grid(gg_ctx *ctx);
// key of the R^k table's index structure (null before the first table)
const std::vector<int> *rk_structure_key(const gg_ctx *ctx);
int ensure_orbitals(gg_ctx *ctx);
// timing helpers (ctx.cu)
int timer_start(gg_ctx *ctx);
int timer_stop(gg_ctx *ctx, double *ms);
// spmv.cu
int build_sym(gg_hmat *h);
// setham.cu: CLRX (lib9290/clrx.f90) on the host
double clrx_host(int kappaa, int k, int kappab);
// hostmat.cu: the leading ns x ns block of a host-resident matrix as a
// device matrix
int leading_block_host(gg_hmat *h, int ns, gg_hmat **out);
int refresh_sym_values(gg_hmat *h);
int spmv(gg_hmat *h, int precision, const double *dx, double *dy, int m, cudaStream_t s);
// xs: the split (hi + lo FP32) copy of x to read; null = the matrix's dXs
int spmv_col(gg_hmat *h, int precision, const double *Bbase, double *ABbase, int64_t ld, const int *dcol,
             const double *skip, cudaStream_t s, const float2 *xs = nullptr);
// Row pitch (in float2) of the interleaved split copies of m vectors that the
// block matvec reads: m rounded up to a power of two (at least 2), so that a
// row is whole 16-byte pieces and never straddles a 128-byte line.
__host__ __device__ constexpr int spmm_pitch(int m) { return m <= 2 ? 2 : m <= 4 ? 4 : m <= 8 ? 8 : 16; }
// block form (SPLIT): columns kpass .. kpass+m-1, kpass = *dcol (0 when dcol is
// null); xb holds their
// hi + lo values interleaved by row (row j at xb + j spmm_pitch(m))
int spmm_block(gg_hmat *h, int m, const float2 *xb, const double *Bbase, double *ABbase, int64_t ld,
               const int *dcol, cudaStream_t s);
int spmm_cols(gg_hmat *h, const double *X, double *Y, int64_t ld, int m, cudaStream_t s);
double spmv_bytes(const gg_hmat *h, int precision, int m);
// tunes the split matvec a solve with this MBLOCK launches (outside capture)
int tune_prepare(gg_hmat *h, int precision, int mblock);
// hosteig.cpp: lowest m eigenvalues of a packed-upper symmetric matrix and
// the eigenvectors of the lowest mvec <= m of them; blo/bhi (may be null)
// bound eigenvalue j from below/above
int sym_eig_lowest(int n, const double *ap, int m, int mvec, double *w, double *z, const double *blo = nullptr,
                   const double *bhi = nullptr);
}  // namespace gg
