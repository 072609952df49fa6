/*
 * grasp_gpu.h - C ABI of the GB300 (sm_103a) CI hot path for GRASP.
 *
 * This library replaces one stage of GRASP's rci / rmcdhf: the radial
 * integral tables (GENINTRK / SLATER / RINTI), the Hamiltonian assembly from
 * rangular's T/V angular-coefficient lists (SETHAM) and the Davidson
 * eigensolver (MANEIG -> GDVD/DVDSON with SPICMV2 as the matrix-vector
 * product). Everything runs on one GPU; there is no CPU fallback.
 *
 * Conventions (the reference's own):
 *  - orbital, CSF and sparse-position indices are 1-based;
 *  - PF/QF are column-major [ld x nw] (PF(NNNP, NW), wave_C);
 *  - the Hamiltonian is the lower triangle stored by rows with the diagonal
 *    last in each row: IENDC(0:NCF) row ends, IROW column indices, EMT values
 *    (hmat_C; mcp.30 record layout). IENDC is int64 here so that blocks above
 *    2^31-1 non-zeros are representable; IROW stays int32.
 *  - every entry point returns 0 on success and a negative gg_status on
 *    failure; gg_last_error() gives the message. No entry point aborts the
 *    process (the reference STOPs; the caller decides what to do).
 *
 * Device memory is owned by the context and its handles. All work is issued
 * on the context's CUDA stream (a blocking stream); calls are synchronous
 * unless documented. Device buffers come from the device's default memory
 * pool, which keeps memory the library frees for its later allocations;
 * gg_release_memory returns it to the driver.
 */
#ifndef GRASP_GPU_H
#define GRASP_GPU_H
#include <stddef.h>
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct gg_ctx gg_ctx;
typedef struct gg_hmat gg_hmat;

enum gg_status {
  GG_OK = 0,
  GG_ERR_ARG = -1,       /* invalid argument */
  GG_ERR_CUDA = -2,      /* CUDA runtime error */
  GG_ERR_STATE = -3,     /* call order (e.g. no orbitals yet) */
  GG_ERR_NOTFOUND = -4,  /* RKINTC: integral not in the table */
  GG_ERR_RANGE = -5,     /* SETHAM: LOC beyond NELMNT, label out of range */
  GG_ERR_KAPPA = -6,     /* RINTI: orbitals with different kappa */
  GG_ERR_CONVERGE = -7,  /* DVDSON: MAXITER reached (ierr has bit 2048) */
  GG_ERR_NOMEM = -8,
  GG_ERR_TIMEOUT = -9    /* a bounded device wait ran out; the call's result
                            is not valid, the context stays usable */
};

/* Precision of the R^k contraction and of the Davidson matvec. */
enum gg_precision {
  GG_FP64 = 0,       /* FP64 everywhere */
  GG_SPLIT = 1       /* hi+lo FP32 split of the off-diagonal matvec; FP64
                        diagonal, Rayleigh-Ritz, Gram-Schmidt and residuals */
};

const char *gg_last_error(void);
int gg_version(void);

/* ---- context --------------------------------------------------------- */
int gg_ctx_create(int device, gg_ctx **out);
int gg_ctx_destroy(gg_ctx *ctx);
/* Blocks until all work on the context's stream has finished. */
int gg_ctx_synchronize(gg_ctx *ctx);
/* Waits for the device, then returns the memory the library's freed
 * buffers left in the device's default memory pool to the driver. */
int gg_release_memory(int device);

/* ---- grid (grid_C, npot_C, def_C) ---------------------------------------
 * Replaces RADGRD (lib9290/radgrd.f90:3) + SETQIC (lib9290/setqic.f90:3) as
 * called from GETCID (rci90/getcid.f90:233-237). r/rp/rpor may be NULL: the
 * exponential grid (HP = 0) is then generated as RADGRD does. zz[n] is the
 * nuclear potential r*V(r) (ZZ). c is the speed of light (C).            */
int gg_set_grid(gg_ctx *ctx, int n, double rnt, double h, double c, const double *r, const double *rp,
                const double *rpor, const double *zz);
/* Copies of R, RP, RPOR (n + 10 values each). */
int gg_get_grid(gg_ctx *ctx, double *r, double *rp, double *rpor);

/* ---- orbitals (wave_C: PF, QF, MF; orb_C: NAK) ----------------------------
 * Replaces the state LODRWF (lib9290/lodrwf.f90:100-134) leaves behind.
 * Values beyond MF(j) must be zero, as LODRWF leaves them.               */
int gg_set_orbitals(gg_ctx *ctx, int nw, int ld, const int *nak, const int *mf, const double *pf,
                    const double *qf);

/* ---- R^k table ------------------------------------------------------------
 * GENINTRK (rci90/genintrk.f90:3, loop :67-86): all R^k(ab;cd) with
 * a<=b, a<=c, b<=d and TRIANGRK(l_a,k,l_c) & TRIANGRK(l_b,k,l_d), for
 * k = 0..J2MAX (kmax < 0) or k = 0..kmax. The table stays on the device.
 * precision: GG_FP64: FP64 contraction on the CUDA cores; GG_SPLIT: the
 * contraction on the tensor cores (tcgen05.mma kind::f16), A and Y each
 * split into 10 balanced 7-bit digits under a per-row power-of-two scale
 * (Ozaki scheme), exact products and exact FP32 group sums in tensor memory,
 * folded in double-float (relative error ~1e-13 of the row scales'
 * product); the QUAD head term and end correction stay FP64. The index
 * structure is kept between calls with the same orbital l, j and kmax.     */
int gg_genintrk(gg_ctx *ctx, int kmax, int precision, int64_t *n_out, int *j2max_out);
/* Copies INDTEIRK (int32, packed ((a*KEY+b)*KEY+c)*KEY+d, KEY = NW+1),
 * VALTEIRK (double) and KSTART(0:kloop+1) (1-based positions). Any pointer
 * may be NULL.                                                              */
int gg_get_rk_table(gg_ctx *ctx, int32_t *indteirk, double *valteirk, int32_t *kstart);
/* RKINTC (rci90/rkintc.f90:3): canonicalise, then look the integral up in
 * the device table. Returns GG_ERR_NOTFOUND where the reference STOPs.     */
int gg_rkintc(gg_ctx *ctx, int ia, int ib, int ic, int id, int k, double *tegral);
/* SLATER (lib9290/slater.f90:3): one R^k(ab;cd) evaluated on the device. */
int gg_slater(gg_ctx *ctx, int ia, int ib, int ic, int id, int k, double *out);
/* ---- SCF potentials from the Y^k functions (rmcdhf) ------------------------
 * The Y^k_ab functions of YZK (lib9290/yzk.f90:3: TB(1:N), every grid point),
 * built on the device for a coefficient list of SETCOF and combined in the
 * list's order, each grid point's operations those of the reference loop.
 * gg_ypot: YPOT(J) (rmcdhf90/ypot.f90:35-49), the direct potential
 *   yp[i-1] = ZZ(i) - sum_t ya[t] Y^K_{IOY1 IOY2}(r_i), i = 1..N;
 *   nya[t] = (IOY2 * 215 + IOY1) * 215 + K (rmcdhf's NYA, KEY = KEYORB).
 * gg_xpot: XPOT(J) (rmcdhf90/xpot.f90:31-54), the exchange potential
 *   xp[i-1] = sum_t (xa[t] / C) Y^K_{IOY1 IOY2}(r_i) QF(i, IORB),
 *   xq[i-1] = -sum_t (xa[t] / C) Y^K_{IOY1 IOY2}(r_i) PF(i, IORB);
 *   nxa[t] = ((IORB * 215 + IOY2) * 215 + IOY1) * 215 + K (NXA).
 * Orbital indices are 1-based in the context's orbital order; yp, xp and xq
 * hold N doubles. GG_ERR_ARG for a label outside the orbital set or
 * K > 20 (YZK's KLIMIT).                                                    */
int gg_ypot(gg_ctx *ctx, int ncof, const int32_t *nya, const double *ya, double *yp);
int gg_xpot(gg_ctx *ctx, int ncof, const int32_t *nxa, const double *xa, double *xp, double *xq);
/* The three coefficient lists SETCOF (rmcdhf90/setcof.f90) leaves in scf_C
 * for one orbital: YPOT's (NYCOF, NYA, YA), XPOT's (NXCOF, NXA, XA) and
 * DACON's (NDCOF, NDA, DA; NDA = orbital index, 1-based).                  */
typedef struct {
  int ny;
  const int32_t *nya;
  const double *ya;
  int nx;
  const int32_t *nxa;
  const double *xa;
  int nd;
  const int32_t *nda;
  const double *da;
} gg_cof;
/* gg_cofpot: COFPOT (rmcdhf90/cofpot.f90:29-33) after its SETCOF: YPOT,
 * XPOT, LAGCON (lagcon.f90:32-56, one process) and DACON (dacon.f90:25-46)
 * for orbital j (1-based) with UCF(J) = ucfj. The Lagrange multipliers are
 * lagr_C's: nec pairs iecc[k] = LI + 215 LJ with values ecv[k] (nec = 0: no
 * LAGCON term). accy: def_C's ACCY (<= 0: H^6, its default); LAGCON skips a
 * multiplier whose weight is below 0.01 ACCY. yp, xp, xq: N doubles each.
 * gg_setlag: SETLAG's multipliers (rmcdhf90/setlag.f90:127-223) for the nec
 * pairs of iecc (as above; the orbitals of a pair have the same kappa): each
 * orbital named in a pair gets its potentials (YPOT, XPOT, DACON) from its
 * lists cof[orbital - 1] once, then ecv[k] from the pair's quadrature and
 * RINTI, by the reference's three cases (a fixed orbital, occupation numbers
 * more than 10 % apart, close occupations). ucf[nw], lfix[nw] (0/1): UCF and
 * LFIX of every orbital. Entries of cof for orbitals in no pair are not read. */
/* SETCOF (rmcdhf90/setcof.f90:3) from the blocks' T/V lists on the device.
 * gg_setcof_prepare: the sums SETCOF forms from the mixing coefficients, for
 * every orbital at once: each label's sum over its contributions of
 * DSUBRS(IR, IC) COEFF, doubled off the diagonal (setcof.f90:242-251,
 * 302-311), and every diagonal FCO/GCO sum over the CSFs (:82-90, :121-129).
 * h[nblocks]: the blocks in rmcdhf's order, their lists uploaded with
 * gg_setham_upload (which also gave their IQ). eol != 0 (EOL): DSUBRS from
 * the levels (dsubrs.f90:20-28), evec[b] the block's nev[b] eigenvectors
 * (NCF_b x nev[b], column-major) and wt[b] their weights; eol = 0: wt[b] the
 * NCF_b weights DSUBRS(IR, IR) = WT(IR) reads, evec and nev unused. The sums
 * stay with the context until the next call.
 * gg_setcof: SETCOF(EOL, J)'s lists for orbital j with UCF(J) = ucfj, from
 * the prepared sums: YPOT's (*ny, nya, ya), XPOT's (*nx, nxa, xa) and
 * DACON's (*nd, nda, da), entry for entry the reference's (its order and
 * its merging of repeated labels across blocks). Each output array holds
 * cap entries; GG_ERR_RANGE (with the counts set) when a list is longer.   */
int gg_setcof_prepare(gg_ctx *ctx, int nblocks, gg_hmat *const *h, const int *nev, const double *const *evec,
                      const double *const *wt, int eol);
int gg_setcof(gg_ctx *ctx, int j, double ucfj, int cap, int *ny, int32_t *nya, double *ya, int *nx, int32_t *nxa,
              double *xa, int *nd, int32_t *nda, double *da);
int gg_cofpot(gg_ctx *ctx, int j, double ucfj, const gg_cof *cof, int nec, const int32_t *iecc, const double *ecv,
              double accy, double *yp, double *xp, double *xq);
int gg_setlag(gg_ctx *ctx, int nec, const int32_t *iecc, const double *ucf, const int *lfix, const gg_cof *cof,
              double *ecv);
/* ---- Breit (transverse photon) integrals -----------------------------------
 * gg_genintbreit: GENINTBREIT1 / GENINTBREIT2 (rci90/genintbreit1.f90:3,
 * genintbreit2.f90:3) on the device: BRINTF(type, ia, ib, ic, id, k)
 * (rci90/brintf.f90:3) for every k = 0..J2MAX and orbitals ia, ib, ic, id
 * (1..NW) that TRIANGBREIT1 / TRIANGBREIT2 admits, in the reference's loop
 * order (k, then ia, ib, ic, id). The photon frequencies are W = wfact
 * |E(a) - E(b)| / C (bessel.f90:88) from the orbital energies e[nw] (orb_C's
 * E) and WFACT (bess_C; 1 is rci's default, 0 the zero-frequency limit);
 * accy: ACCY (<= 0: H^6). *nb_out = NB, *j2max_out = J2MAX. The table stays
 * with the context (one per type).
 * BRINTF is evaluated from its arguments alone: where the reference skips a
 * BESSEL call for two equal orbitals and reads its slot's earlier content
 * (brintf.f90:47-48), the zero-frequency function (zero) is used.
 * gg_get_breit_table: INDTP = ((ia KEY + ib) KEY + ic) KEY + id (KEY = NW +
 * 1), VALTP and KSTARTBREIT(0:J2MAX+1) (1-based); any pointer may be NULL.
 * gg_brint: BRINT1 / BRINT2 (rci90/brint1.f90:3, brint2.f90:3), a value of
 * the context's table of that type; GG_ERR_NOTFOUND where the reference
 * STOPs.
 * gg_brintf: BRINTF for n integrals of any type 1..6 (those BRINT3-6
 * evaluate on demand and cache, brint3.f90:111-153, in one call):
 * items[6 t .. 6 t + 5] = type, ia, ib, ic, id, k; out[n].                  */
int gg_genintbreit(gg_ctx *ctx, int type, double wfact, const double *e, double accy, int64_t *nb_out,
                   int *j2max_out);
int gg_get_breit_table(gg_ctx *ctx, int type, int32_t *indtp, double *valtp, int32_t *kstart);
int gg_brint(gg_ctx *ctx, int type, int ia, int ib, int ic, int id, int k, double *tegral);
int gg_brintf(gg_ctx *ctx, int n, const int32_t *items, double wfact, const double *e, double accy, double *out);
/* gg_slater without any device allocation. No counterpart in the reference:
 * for callers that cannot allocate device memory at the point where they
 * need an integral (device memory fully handed to a pool or to a large
 * block's Hamiltonian and basis; callers that cannot recover from a failed
 * allocation inside a loop). Same result as gg_slater. Its working arrays
 * sit in one fixed device array that every GPU loading this library holds
 * until exit; grids up to 2022 points (N + 26 <= 2048), larger ones are
 * rejected with GG_ERR_ARG. The first call on a device looks up that
 * array's address with the device current: make it before any stream
 * capture. Calls share the array: calls that overlap on the GPU race.      */
int gg_slater_noalloc(gg_ctx *ctx, int ia, int ib, int ic, int id, int k, double *out);

/* ---- one-body integrals ----------------------------------------------------
 * RINTI (lib9290/rinti.f90:3) with DPBDT (dpbdt.f90:3): I(ab), mode 0
 * includes the nuclear potential. GG_ERR_KAPPA where NAK(a) != NAK(b).      */
int gg_rinti(gg_ctx *ctx, int j, int k, int mode, double *out);
/* IABINT's cache (rci90/iabint.f90:3) as a dense table: iab[(a-1)*nw+(b-1)]
 * = I(ab) for NAK(a) == NAK(b), NaN otherwise. iab may be NULL (the table
 * is kept on the device for SETHAM).                                         */
int gg_iabint_table(gg_ctx *ctx, double *iab);

/* ---- Hamiltonian block (hmat_C) -------------------------------------------
 * Structure of one block as MATRIX reads it from mcp.30
 * (rmcdhf90/matrix.f90:123-140): iendc[0..ncf] (IENDC(0) = 0), irow[nnz]. */
int gg_hmat_create(gg_ctx *ctx, int ncf, int64_t nnz, const int64_t *iendc, const int32_t *irow,
                   gg_hmat **out);
int gg_hmat_destroy(gg_hmat *h);
/* A matrix with src's structure (IENDC/IROW, the symmetric matvec structure)
 * and src's T/V lists and assembly plan, shared, but its own EMT: for the
 * same J/parity block of another ion (other orbitals, same CSFs). Assemble it
 * with gg_setham_assemble on ctx (any context of src's device) after that
 * context's gg_genintrk and gg_iabint_table; gg_setham_upload on a view is an
 * error. src may be destroyed before its views (its memory is released with
 * the last view).                                                           */
int gg_hmat_create_view(gg_ctx *ctx, gg_hmat *src, gg_hmat **out);

/* One rangular coefficient list (mcp.31 or mcp.32+k, one block), as
 * SORTMEM writes it (rangular90/sortmem.f90:232-284): nlab labels; label l
 * owns contributions start[l] .. start[l+1]-1 of loc[] (the sparse INDEX,
 * 1-based into EMT) and coeff[]. T labels pack min(a,b)*215+max(a,b);
 * V labels pack ((a*215+c)*215+b)*215+d (rmcdhf90/setham.f90:244, 305-310). */
typedef struct {
  int64_t nlab;
  const int32_t *lab;
  const int64_t *start; /* nlab + 1 entries, start[0] = 0 */
  const int32_t *loc;
  const double *coeff;
} gg_list;

/* SETHAM (rmcdhf90/setham.f90:3) for one block, followed by the average
 * energy shift of MATRIX (rmcdhf90/matrix.f90:178-203).
 * iq[(ir-1)*nw + (a-1)] = IQ(a, ir), the subshell occupations of the block's
 * CSFs (used for the diagonal FCO/GCO pieces, setham.f90:83-219).
 * vlists has kmaxf + 1 entries (k = 0..kmaxf). Needs gg_genintrk (with
 * kloop >= kmaxf) and gg_iabint_table first. On return EMT holds H - EAV*I
 * on the device and *eav_out = EAV.
 * gg_setham_upload copies the lists to the device; gg_setham_assemble
 * builds the per-element gather index and assembles EMT from the device
 * copies. gg_setham does both.                                              */
int gg_setham_upload(gg_ctx *ctx, gg_hmat *h, const uint8_t *iq, const gg_list *tlist, int kmaxf,
                     const gg_list *vlists);
int gg_setham_assemble(gg_ctx *ctx, gg_hmat *h, double *eav_out);
int gg_setham(gg_ctx *ctx, gg_hmat *h, const uint8_t *iq, const gg_list *tlist, int kmaxf,
              const gg_list *vlists, double *eav_out);
/* Copies EMT (nnz values) back to the host. */
int gg_hmat_get_emt(gg_hmat *h, double *emt);
/* Replaces EMT by caller values (for a matrix assembled elsewhere, e.g. the
 * rows rci writes to rci.res, setham_gg.f90:378). */
int gg_hmat_set_emt(gg_hmat *h, const double *emt);

/* SPICMV2 (lib9290/spicmv2.f90:2): C = H B for m host vectors [ncf x m]. */
int gg_spicmv2(gg_ctx *ctx, gg_hmat *h, int m, const double *b, double *c, int precision);

/* ---- blocks whose matrix stays off the device (SPODMV, DNICMV) -------------
 * SPODMV (rci90/spodmv.f90:3): rci's product for a block too large to keep in
 * memory, which re-reads the lower triangle from rci.res for every product
 * (rci90/maneig.f90:262-279). gg_hmat_create_host keeps such a block in
 * pinned host memory instead of HBM: its full symmetric matrix is built once
 * there, in the form the given precision's product reads (GG_FP64: FP64
 * values and int32 columns, 12 bytes per stored entry of either triangle;
 * GG_SPLIT: hi + lo FP32 values and 16-bit columns when NCF <= 65536, 10
 * bytes), and every product reads it over the host link while the vectors
 * and the diagonal stay on the device. Results are bit for bit those of the
 * same matrix on the device (gg_hmat_create + gg_hmat_set_emt with the
 * shifted diagonal).
 * iendc/irow as gg_hmat_create; emt[nnz]: the block's values as rci writes
 * them to rci.res (setham_gg.f90:378), diagonal unshifted; the diagonal used
 * is EMT(IENDC(i)) - eav, SPODMV's DIAG (spodmv.f90:77). The caller's arrays
 * are not referenced after the call.
 * The matrix works with gg_spicmv2 and gg_spodmv, gg_maneig (whose
 * p->precision must be the matrix's; the leading-block stage runs on a device
 * copy of the leading rows), gg_matvec_timing, gg_spmm_timing and
 * gg_hmat_tune in its precision; SETHAM, gg_hmat_get_emt/set_emt,
 * gg_hmat_create_view and gg_maneig_batched refuse it with GG_ERR_ARG.
 * gg_hmat_host_precision: the precision a host-resident matrix was built for,
 * -1 for a matrix on the device.
 * gg_spodmv: C = (H - EAV) B for m host vectors [ncf x m], in the matrix's
 * precision (GG_ERR_ARG for a matrix on the device).                        */
int gg_hmat_create_host(gg_ctx *ctx, int ncf, int64_t nnz, const int64_t *iendc, const int32_t *irow,
                        const double *emt, double eav, int precision, gg_hmat **out);
int gg_hmat_host_precision(gg_hmat *h);
int gg_spodmv(gg_ctx *ctx, gg_hmat *h, int m, const double *b, double *c);
/* DNICMV (rci90/dnicmv.f90:3): the product with a dense lower triangle packed
 * by rows, ap[i(i-1)/2 + j - 1] = A(i, j) for 1 <= j <= i <= ncf (the EMT of
 * hmat_C with IEND = IEND + ICOL, diagonal last in each row). The matrix gets
 * the sparse structure with every entry present; gg_spicmv2 on it is
 * DNICMV's C = A B and gg_maneig solves it like any block.                 */
int gg_hmat_create_packed(gg_ctx *ctx, int ncf, const double *ap, gg_hmat **out);

/* ---- eigen-solve ------------------------------------------------------------
 * MANEIG (rci90/maneig.f90:3 when flavour = 0, rmcdhf90/maneig.f90:3 when
 * flavour = 1): lowest nvec eigenpairs of the block's H - EAV, dominant
 * component of each eigenvector made positive (rci90/maneig.f90:532-555).
 * The Davidson solver follows GDVD/DVDSON (libdvd90/gdvd.f90:4,
 * dvdson.f90:1) with the reference's constants: CRITE 1e-17, CRITC = CRITR
 * = 1e-9, MBLOCK 1, LIM/MAXITR per flavour. Where the reference uses dense
 * DSPEVX (rci, ncf <= 2000), this library runs the same Davidson to the
 * same tolerances; a block with NCF < NVEC + 4 is solved in its full unit
 * basis (one projected eigenproblem of the whole matrix). Initial estimates
 * follow INIEST2
 * (lib9290/iniest2.f90:3): the lowest eigenvectors of the leading
 * min(nmax, ncf) block.
 * eval[nvec] (relative to EAV), evec[ncf x nvec] column-major.             */
typedef struct {
  int flavour;    /* 0 = rci, 1 = rmcdhf */
  int precision;  /* gg_precision of the matvec */
  int lim;        /* <= 0: reference default; else NCF or at least NVEC + 4
                     (DVDSON's restart keeps min(max(LIM/2, 2 NVEC), LIM - 3)
                     vectors and needs NVEC + 1 of them) */
  int maxiter;    /* <= 0: reference default */
  double critr;   /* <= 0: 1e-9 */
  double critc;   /* <= 0: 1e-9 */
  double crite;   /* <= 0: 1e-17 */
  int robust;     /* 0: DVDSON exactly. 1: the first pass's robust shift uses
                     DL = 0 where the reference uses |1e30 - lambda| (its
                     OLDVAL sentinel, dvdson.f90:703), which otherwise wastes
                     the first correction vector and can let the coefficient
                     test stop the solver early. */
  int mblock;     /* DVDSON's MBLOCK for the full block: <= 0 or 1 keeps the
                     reference's single-vector passes; up to nvec adds that
                     many correction vectors per pass (one matvec pass over
                     the matrix for all of them, one projected eigenproblem
                     per pass) */
  int nstart;     /* > 0: DVDSON starts from the nstart (<= LIM) vectors in
                     start instead of INIEST2's estimates: rmcdhf's repeated
                     solves, which start from the previous SCF iteration's
                     eigenvectors (rmcdhf90/maneig.f90:116-128; the
                     reference does so for NCF > 4000, this library for any
                     NCF). Like DVDSON's initial vectors they must be
                     orthonormal (libdvd90/dvdson.f90:228); the previous
                     call's evec is. 0: INIEST2. */
  const double *start; /* [ncf x nstart] column-major, host memory */
} gg_dvd_params;

int gg_maneig(gg_ctx *ctx, gg_hmat *h, int nvec, const gg_dvd_params *p, double *eval, double *evec,
              int *nloops, int *nmv, int *ierr);

/* ---- MANEIG over many blocks ---------------------------------------------
 * Replaces the per-block MANEIG calls of rci's block loop
 * (rci90/matrix.f90:177-187 -> rci90/maneig.f90:3) for nblocks blocks at
 * once: all blocks run one batched Davidson on the device (every step of the
 * iteration, including the projected eigenproblems, is a GPU kernel over all
 * blocks; the iteration is one CUDA graph). Block b asks for its lowest
 * nvec[b] (1..16, <= NCF) eigenpairs of its assembled matrix (EMT - EAV, as
 * MANEIG). p (may be NULL): precision (GG_FP64 / GG_SPLIT matvec), lim (LIM,
 * default min(NCF, 2 NVEC + 60), at most 128), maxiter (default
 * max(200 NVEC, NCF/10)), critr (residual norm, default 1e-9); flavour,
 * critc, crite and robust are not used. Blocks may come from different
 * contexts of the same device.
 * eval: all blocks' eigenvalues, concatenated (sum of nvec). evec (may be
 * NULL): all blocks' eigenvectors, concatenated, block b column-major
 * NCF_b x nvec[b], dominant component positive (rci90/maneig.f90:532-555).
 * nloops, nmv, ierr (may be NULL): per block; ierr bit 2048 = MAXITER
 * reached, then GG_ERR_CONVERGE is returned (results are still written).
 * Blocks with NCF <= LIM are solved exactly in the full unit basis.         */
int gg_maneig_batched(gg_ctx *ctx, int nblocks, gg_hmat *const *h, const int *nvec, const gg_dvd_params *p,
                      double *eval, double *evec, int *nloops, int *nmv, int *ierr);

/* ---- timing --------------------------------------------------------------
 * Device time (ms, CUDA events on the context stream) of the named stage of
 * the last call: 0 genintrk, 1 iabint, 2 setham assemble, 3 maneig total,
 * 4 matvec (sum over the last maneig), 5 number of matvec launches,
 * 6 bytes moved by one matvec (algorithmic), 7 setham upload,
 * 8 / 9 Davidson loops of the leading-block (INIEST2) / full-block stage,
 * 10 / 11 their matvec ms, 12 full-block matvec launches, 13 host ms in the
 * projected eigenproblems, 14 host ms waiting for device results, 15 host ms
 * inside both Davidson runs, 16 device ms of the full-block single-vector
 * passes, 17 / 18 host ms of the leading-block / full-block Davidson run,
 * 19 host ms of the full-block projected eigenproblems, 20 number of R^k
 * table entries the last genintrk evaluated with the general QUAD (head
 * index above 2), 21 iterations of the last gg_maneig_batched (all blocks
 * together), 22 kernels per batched iteration (stage 3 is the batched
 * solve's total ms), 23 / 24 device ms / number of the full-block block
 * matvecs (split SpMM) over MBLOCK columns of the last gg_maneig, 25 the
 * number of grid-point ranges (split-K) of the last tensor-core
 * gg_genintrk's contraction tiles, 26 / 27 host ms of the last gg_maneig's
 * structure set-up (symmetric matvec structures of the block and of its
 * leading block) / Davidson workspaces, 28 device ms from the start of that
 * gg_maneig to the end of its structure set-up, 29 device ms of the
 * assembly plan built by the last gg_setham_upload (0 when it built none),
 * 30 block passes of the last split gg_maneig whose second Gram-Schmidt
 * pass was skipped (the first kept at least half of every new column's
 * squared norm), 31 device and host ms of the last gg_genintbreit, 32 / 33
 * its host ms enumerating the integrals and their terms / its device ms of
 * the Bessel, term and combination kernels.                                                            */
double gg_stage_stat(gg_ctx *ctx, int which);

/* gg_projected_eig: DVDSON's projected eigenproblem, CALL DSPEVX('Vectors
 * also', 'In a range', 'Upper triangular', KPASS, S, ...) at
 * libdvd90/dvdson.f90:724, on the host (no GPU): the lowest m eigenvalues
 * (ascending) of the symmetric n x n matrix in packed upper storage
 * ap[i + j(j+1)/2] = A(i, j), 0 <= i <= j < n, into w[m], and the eigenvectors
 * of the lowest mvec <= m of them into z (n x mvec, column-major, unit norm,
 * sign unspecified). The Davidson iteration calls the same routine once per
 * pass. Returns GG_ERR_ARG for bad sizes, GG_ERR_CONVERGE if the
 * eigenvalue search does not finish.                                       */
int gg_projected_eig(int n, const double *ap, int m, int mvec, double *w, double *z);

/* ---- SpMV autotuner (no counterpart in the reference) ---------------------
 * The split-precision matvec kernels come in variants: kernel 0, the block
 * matvec over m = 1..16 vectors (Davidson block passes; gg_spicmv2 with
 * m >= 2), 9 variants = 2, 4 or 8 loads in flight per lane x 128, 256 or
 * 512 threads per block; kernel 1, the single-vector matvec (MBLOCK = 1
 * passes), 6 variants = 32 or 16 lanes per row x 2, 4 or 8 loads in flight.
 * The first launch for a matrix shape (device, NCF, stored elements) and m
 * outside a stream capture times every variant (CUDA events; one warm-up
 * and three timed launches each) and keeps the fastest for that shape for
 * the rest of the process; gg_maneig tunes the widths it will use before
 * it captures its graphs. Every variant computes the same products and
 * sums in double-float; their results differ only by the order of the
 * partial sums.
 * gg_hmat_tune: tunes if needed, then reports the variant the solver
 * launches (*chosen), the number of variants and their mean times per
 * launch (ms[nvariants]).
 * gg_hmat_tune_force: launch `variant` for this matrix (-1: the tuned one).
 * Kernel 2 is the batched matvec of gg_maneig_batched (k_b_spmm), 6
 * variants = 64, 128 or 256 rows per CTA x 128 or 256 threads: all of them
 * run on the first start-up expansion of a batch shape (device, blocks,
 * rows, stored elements, precision), each computing the same columns, and
 * the fastest is kept for the shape in this process; gg_batched_tune_info
 * reports the last batched solve's choice on the context and the variants'
 * times from the run that tuned the shape.
 * gg_tune_variant_name: a short name of a variant ("U4 T256", "L16 U8",
 * "R128 T256").                                                           */
int gg_hmat_tune(gg_hmat *h, int kernel, int m, int *chosen, int *nvariants, double *ms);
int gg_hmat_tune_force(gg_hmat *h, int kernel, int m, int variant);
int gg_batched_tune_info(gg_ctx *ctx, int *chosen, int *nvariants, double *ms);
const char *gg_tune_variant_name(int kernel, int variant);

/* ---- measurement helpers (no counterpart in the reference) ------------------
 * gg_launch_count: kernels this library has launched in this process.
 * gg_alloc_count: device (cudaMalloc) and pinned host (cudaMallocHost)
 * allocations this library has made in this process.
 * gg_event_record / gg_event_elapsed: CUDA events (8 slots) on the context
 * stream; elapsed synchronises on slot b.
 * gg_matvec_timing: average device time of one y = H x launch (after a
 * warm-up) over iters launches, and its algorithmic bytes.
 * gg_spmm_timing: the same for one split-precision Y = H X launch over m
 * vectors (1 <= m <= 16; the Davidson block pass's matvec), algorithmic
 * bytes = the matrix in the reference's storage once + 3 m NCF doubles.     */
long long gg_launch_count(void);
/* Test hook of the bounded device waits: in the next tensor-core
 * gg_genintrk (GG_SPLIT) on ctx, tile `tile` of the contraction withholds
 * its first copy and polls its barrier only briefly, so that wait runs out
 * with nothing in flight. The call then returns GG_ERR_TIMEOUT and leaves
 * no valid table; the context stays usable. tile < 0 cancels.             */
int gg_test_stall_rk_tile(gg_ctx *ctx, int tile);
long long gg_alloc_count(void);
/* Page-locks (pins) caller memory so that uploads from it run at full link
 * rate; unregister before freeing it. */
int gg_host_register(void *p, size_t bytes);
int gg_host_unregister(void *p);
int gg_event_record(gg_ctx *ctx, int slot);
int gg_event_elapsed(gg_ctx *ctx, int a, int b, double *ms);
int gg_matvec_timing(gg_ctx *ctx, gg_hmat *h, int precision, int iters, double *ms_per_launch, double *alg_bytes);
int gg_spmm_timing(gg_ctx *ctx, gg_hmat *h, int m, int iters, double *ms_per_launch, double *alg_bytes);
/* The host link's read rate, the bound of a host-resident matrix's product:
 * ms per pass over a pinned host buffer of `bytes` (rounded down to 16),
 * mode 0: read by a streaming kernel (16-byte loads, as the matvec's entries
 * are read), mode 1: copied to the device by cudaMemcpyAsync.             */
int gg_host_read_timing(gg_ctx *ctx, size_t bytes, int mode, int iters, double *ms_per_pass);

#ifdef __cplusplus
}
#endif
#endif
