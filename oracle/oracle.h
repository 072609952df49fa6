/*
 * oracle.h - CPU FP64 restatement of GRASP's CI hot path.
 *
 * TEST INFRASTRUCTURE ONLY. This library is the checker for the CUDA path in
 * grasp_gb300/csrc. Only tests/, __graft_entry__.smoke() and the CPU-baseline
 * legs of bench.py may load it. It is never part of the product path.
 *
 * Every routine restates one reference subroutine, loop by loop, in FP64.
 * The reference (GRASP2018, Fortran 90) cannot be compiled in this
 * environment (no Fortran compiler), so parity is pinned by the reference's
 * own QUAD known-answer test (test/lib9290_quad.f90:22-33) and by analytic
 * hydrogenic known answers; see tests/test_oracle_kat.py.
 *
 * Conventions: arrays follow the Fortran layout. Orbital tables PF/QF are
 * column-major [ld x nw]; grid arrays have NNN1 = n + 10 entries; orbital
 * and CSF indices in the API are 1-based exactly as in the reference.
 */
#ifndef GRASP_ORACLE_H
#define GRASP_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct or_ctx or_ctx;

/* RADGRD (lib9290/radgrd.f90:38-60, HP = 0 branch) + SETQIC (setqic.f90:157-195).
 * c is the speed of light (DEF_C C), zz[n] the nuclear potential r*V (NPOT_C ZZ). */
or_ctx *or_create(int n, double rnt, double h, double c, const double *zz);
void or_destroy(or_ctx *);
/* copies of R, RP, RPOR (n + 10 values each) */
void or_get_grid(const or_ctx *, double *r, double *rp, double *rpor);
/* C1..C4 (4 values) and CNC5C(2:5, 2:4) column-major (12 values) */
void or_get_qic(const or_ctx *, double *c1234, double *cnc5c);

/* wave_C: PF, QF [ld x nw] column-major, MF[nw], NAK[nw] (kappa). */
int or_set_orbitals(or_ctx *, int nw, int ld, const int *nak, const int *mf,
                    const double *pf, const double *qf);

/* QUAD (lib9290/quad.f90:52-103). ta has >= mtp + 3 entries, 1-based
 * (ta[0] = TA(1)); the tail TA(MTP+1:MTP+3) is zeroed as in the reference. */
double or_quad(const or_ctx *, int mtp, double *ta);

/* YZK (lib9290/yzk.f90:58-224): writes YK = TB (n values, 1-based) and returns MTP. */
int or_yzk(or_ctx *, int k, int i, int j, double *yk_out);
/* SLATER (lib9290/slater.f90:52-67) */
double or_slater(or_ctx *, int ia, int ib, int ic, int id, int k);
/* RINTI (lib9290/rinti.f90:53-100) with DPBDT (dpbdt.f90:39-99).
 * Returns 0 and sets *err = 1 when NAK(J) != NAK(K) (the reference STOPs). */
double or_rinti(or_ctx *, int j, int k, int mode, int *err);

/* TRIANGRK (rci90/triangrk.f90:27-37) */
int or_triangrk(int la, int k, int lb);
/* GENINTRK (rci90/genintrk.f90:64-106). kmax < 0: loop to J2MAX as the
 * reference does; otherwise loop k = 0..kmax. Two-pass: call with ind = val
 * = NULL to count, then with buffers. kstart has kloop + 2 entries
 * (KSTART(0:kloop+1)), 1-based positions as in the reference. Returns N. */
int64_t or_genintrk(or_ctx *, int kmax, int32_t *indteirk, double *valteirk,
                    int32_t *kstart, int *j2max_out, int nthreads);
/* RKINTC (rci90/rkintc.f90:38-104): canonicalise + binary search.
 * Returns 0 on success, -1 when the integral is not in the table. */
int or_rkintc(int nw, const int32_t *indteirk, const double *valteirk,
              const int32_t *kstart, int ia, int ib, int ic, int id, int k,
              double *tegral);

/* CLRX (lib9290/clrx.f90) with GAM from FACTT (factt.f90) */
double or_clrx(int kappaa, int k, int kappab);

/* ---------------------------------------------------------------------
 * SETHAM from rangular's T/V lists (rmcdhf90/setham.f90:77-342).
 *
 * One block. iq holds the subshell occupations IQ(IA, IR) of the block's
 * CSFs as [nw x ncf] column-major bytes: iq[(ir-1)*nw + (ia-1)].
 * nkj: 2j of each orbital is derived from NAK.
 * iendc[0..ncf] (IENDC(0:NCF), 1-based positions, diagonal last per row).
 * The T list and each V^k list are given as label groups (or_list):
 *   nlab labels; lab[l]; start[l]..start[l+1]-1 index the contribution arrays
 *   loc[] (1-based INDEX into EMT) and coeff[].
 * vlists has kmaxf + 1 entries (k = 0..kmaxf).
 * emt[nelmnt] is accumulated (the caller zeroes it, as MATRIX does).
 * Returns 0, or -1 when a LOC exceeds nelmnt (the reference ERROR STOPs).
 * ------------------------------------------------------------------- */
typedef struct {
  int64_t nlab;
  const int32_t *lab;
  const int64_t *start; /* nlab + 1 */
  const int32_t *loc;
  const double *coeff;
} or_list;

int or_setham(or_ctx *, int ncf, int64_t nelmnt, const int64_t *iendc,
              const uint8_t *iq, const or_list *tlist, int kmaxf,
              const or_list *vlists, double *emt);

/* SETCOF (rmcdhf90/setcof.f90:48-524) for orbital j: one block's data as
 * SETCOF reads it (its mcp.30 structure, its T/V lists, its IQ) and the
 * mixing coefficients DSUBRS reads (dsubrs.f90): eol != 0: nev levels,
 * evec [ncf x nev] column-major, wt[nev]; eol == 0: wt[ncf] CSF weights. */
typedef struct {
  int ncf;
  const int64_t *iendc;
  const int32_t *irow;
  const uint8_t *iq;
  or_list tlist;
  int kmaxf;
  const or_list *vlists;
  int nev;
  const double *evec;
  const double *wt;
} or_block;
/* the lists (NYA/YA, NXA/XA, NDA/DA), cap entries each; -2 when a list is
 * longer (counts set) */
int or_setcof(or_ctx *, int nblocks, const or_block *blocks, int eol, int j, double ucfj, int cap, int *ny,
              int32_t *nya, double *ya, int *nx, int32_t *nxa, double *xa, int *nd, int32_t *nda, double *da);

/* EAV and its subtraction from the diagonal (rmcdhf90/matrix.f90:178-203). */
double or_shift_eav(int ncf, const int64_t *iendc, double *emt);

/* SPICMV2 + DMERGE (lib9290/spicmv2.f90:42-57, dmerge.f90:36-40).
 * b, c are [n x m] column-major. */
void or_spicmv2(int n, int m, const int64_t *iendc, const int32_t *irow,
                const double *emt, const double *b, double *c);

/* Restatement of LAPACK DSPEVX('V','I','U') for the lowest eigenpairs
 * il..iu of a packed-upper symmetric matrix (the algorithm DSPEVX uses:
 * Householder tridiagonalisation, bisection, inverse iteration, back
 * transformation). w[iu-il+1], z[n x (iu-il+1)]. Returns 0 on success. */
int or_dspevx(int n, const double *ap, int il, int iu, double *w, double *z);

/* DVDSON parameters (libdvd90/dvdson.f90:1, gdvd.f90:4) */
typedef struct {
  int lim, ilow, ihigh, niv, mblock, maxiter;
  double crite, critc, critr, ortho;
  int robust; /* 0: the reference exactly; 1: first-pass shift DL = 0 */
} or_dvd_params;

/* GDVD + DVDSON with SPICMV2 as OP. work has length
 * 2*n*lim + lim*lim*2 + 11*lim + nume (MANEIG's LWORK); on entry
 * work[0 .. n*niv) holds the initial estimates. On exit work holds
 * eigenvectors, then eigenvalues, as DVDSON documents (dvdson.f90:472-474).
 * diag[n] is the matrix diagonal (modified in place as GDVD does). */
int or_gdvd(int n, const int64_t *iendc, const int32_t *irow, const double *emt,
            double *diag, const or_dvd_params *p, double *work, int64_t lwork,
            int *nloops, int *nmv, int *ierr, int nthreads);

/* INIEST2 (lib9290/iniest2.f90:49-95) */
int or_iniest2(int nmax, int ncf, int niv, double *basis, const double *emt,
               const int64_t *iendc, const int32_t *irow);

/* MANEIG. flavour 0 = rci (rci90/maneig.f90), 1 = rmcdhf (rmcdhf90/maneig.f90).
 * The matrix already has EAV subtracted from its diagonal. Computes the
 * lowest nvec eigenpairs (IVEC = 1..nvec) with the reference's dispatch
 * (dense DSPEVX or Davidson), and the reference's sign convention.
 * eval[nvec], evec[ncf x nvec]. maxiter_override > 0 replaces MAXITR (for
 * timing a bounded number of Davidson loops); seconds (may be NULL) gets
 * [INIEST2 wall time, DVDSON wall time]. */
int or_maneig(int flavour, int ncf, int nvec, const int64_t *iendc,
              const int32_t *irow, const double *emt, double *eval,
              double *evec, int *nloops, int *nmv, int *ierr, int nthreads,
              int robust, int maxiter_override, double *seconds);

#ifdef __cplusplus
}
#endif
#endif
