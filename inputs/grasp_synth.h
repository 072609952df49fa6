/*
 * grasp_synth.h - input producers for the CI hot path (host C++, libgraspsynth).
 *
 * Not part of the drop-in boundary: in GRASP these inputs come from
 * rwfnestimate (screened hydrogenic orbitals, rwfnestimate90/frmhyd.f90:68-72
 * with lib9290/dcbsrw.f90:3 and screenpar.f90:33-43), rcsfgenerate (the CSF
 * list) and rangular (the T/V angular-coefficient lists, mcp.3x files).
 * This library makes seeded synthetic stand-ins with the reference's formats:
 *  - orbitals: DCBSRW Dirac-Coulomb hydrogenic spinors at Z - sigma, exact;
 *  - CSF space: relativistic configurations reached by single and double
 *    excitations from reference configurations, each contributing the number
 *    of jj-coupled CSFs with the requested J (counted exactly, M-scheme);
 *  - H structure: all CSF pairs whose configurations differ by at most two
 *    electrons (optionally thinned to a target density), stored as the
 *    lower triangle by rows with the diagonal last (mcp.30 layout);
 *  - T/V lists: for each stored element, labels of the radial integrals the
 *    excitation can involve (one-body I(ab) for kappa_a = kappa_b, R^k with
 *    the triangle and parity rules) with seeded coefficients, grouped by
 *    label as SORTMEM writes them. The coefficients are NOT angular
 *    coefficients; computing those needs the recoupling engine.
 */
#ifndef GRASP_SYNTH_H
#define GRASP_SYNTH_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

/* DCBSRW (lib9290/dcbsrw.f90:3): hydrogenic Dirac-Coulomb P, Q for (n, kappa)
 * at nuclear charge z on the grid r[0..ntp-1] (R(1..NTP)); accy = ACCY.
 * Returns 0; p, q [ntp] (zero beyond MTP), *mtp, *e (binding energy
 * (1-eps) c^2), *pz (RG0). Negative on invalid (n, kappa, z).             */
int gs_dcbsrw(int n, int kappa, double z, double c, const double *r, int ntp, double accy, double *e, double *pz,
              double *p, double *q, int *mtp);

/* SCREENPAR (rwfnestimate90/screenpar.f90:33-43): sigma for the first ncore
 * orbitals = electrons inside + (2j+1)/2, the rest = all core electrons. */
int gs_screenpar(int nw, const int *nak, int ncore, double *sigma);

typedef struct gs_block gs_block;

typedef struct {
  int nw;
  const int *np;          /* principal quantum numbers */
  const int *nak;         /* kappa */
  const uint8_t *frozen;  /* 1 = inactive (electrons may not leave) */
  int nref;
  const uint8_t *refs;    /* nref x nw occupations */
  int max_rank;           /* 1 = singles, 2 = singles and doubles */
  int two_j;              /* 2J of the block */
  int parity;             /* 0 even, 1 odd */
  int kmaxf;              /* largest k in the V lists (<= J2MAX of the orbital set) */
  int64_t max_ncf;        /* cap on CSFs (configurations are kept in order) */
  double density;         /* target lower-triangle density; <= 0 keeps every pair */
  double coeff_scale;     /* scale of off-diagonal coefficients */
  uint64_t seed;
} gs_block_spec;

int gs_block_generate(const gs_block_spec *spec, gs_block **out);
void gs_block_free(gs_block *b);
/* sizes: ncf, nnz, number of configurations, kmaxf, total labels and
 * contributions of the T list (index 0) and V^k lists (index 1 + k) */
int gs_block_sizes(const gs_block *b, int *ncf, int64_t *nnz, int *nconf, int *kmaxf, int64_t *nlab,
                   int64_t *ncontr);
/* structure and occupations: iendc[ncf+1], irow[nnz], iq[ncf*nw] */
int gs_block_structure(const gs_block *b, int64_t *iendc, int32_t *irow, uint8_t *iq);
/* one list (0 = T, 1 + k = V^k): lab[nlab], start[nlab+1], iclmn/loc[ncontr], coeff[ncontr] */
int gs_block_list(const gs_block *b, int list, int32_t *lab, int64_t *start, int32_t *iclmn, int32_t *loc,
                  double *coeff);

/* A seeded synthetic symmetric H in GRASP's lower-triangle-by-rows storage
 * (mcp.30's IENDC / IROW, diagonal last in each row, 1-based IROW) with
 * off-diagonal density p: row r holds each column c < r with probability p
 * (independent draws, taken in ascending order by geometric skips), then its
 * diagonal. EMT: diagonal -1000 + 30 sqrt(r / ncf) + N(0, 1e-3) Eh,
 * off-diagonal N(0, 2e-3) Eh. Every row draws from its own counter-based
 * stream, so the result does not depend on the thread count. Call with
 * irow = emt = NULL to get IENDC(0:ncf) (sizes), then again with all three. */
int gs_synthetic_h(int ncf, double p, uint64_t seed, int64_t *iendc, int32_t *irow, double *emt);

#ifdef __cplusplus
}
#endif
#endif
