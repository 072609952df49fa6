/*
 * grasp_angular.h - angular coefficients of the Dirac-Coulomb Hamiltonian
 * between jj-coupled CSFs (host C++, libgraspangular). The producer of the
 * T/V lists that SETHAM consumes (include/grasp_gpu.h, gg_setham).
 *
 * In GRASP the lists come from rangular (rangular90/mcp_gg.f90:143-313 with
 * librang90's ONESCALAR and RKCO_GG, sorted by sortmem.f90:232-284). This
 * library computes the same expansion
 *     H_rs = sum_ab T_rs(ab) I(ab) + sum_k sum_abcd V^k_rs(abcd) R^k(ab;cd)
 * by another route: each CSF is built as a vector of Slater determinants
 * (subshell states |j^w nu J M> from the lowering operator and the
 * seniority operator, coupled subshell by subshell with Clebsch-Gordan
 * coefficients, as the CSF list's couplings say), the Slater-Condon rules
 * give the determinant matrix elements with
 *   <a m_a|C^k_q|c m_c> = (-1)^(j_a-m_a) (j_a k j_c; -m_a q m_c) <k_a||C^k||k_c>,
 * and the CSF coefficients follow by transforming each integral's
 * determinant coefficients with the CSF vectors. The coefficient of every
 * radial integral is exact up to rounding. The CSFs carry the reference's
 * phases (Clebsch-Gordan coupling of the subshell states in list order, the
 * subshell states' own signs fixed by their parents): for a GRASP-written
 * list with up to three electrons in an open subshell the mixing
 * coefficients agree with rmcdhf's in sign, so the off-diagonal
 * coefficients have rangular's signs too.
 *
 * Output per block: the CSR-lower structure (IENDC/IROW, rows in CSF order,
 * diagonal last; mcp.30) and the lists in SETHAM's layout: the T list
 * (labels min(a,b)*215 + max(a,b)), then V^0..V^kmaxf (labels
 * ((a*215+c)*215+b)*215+d with a <= c, b <= d, (a,c) <= (b,d)), each grouped
 * by label with (column, 1-based position in EMT, coefficient) per element.
 * With average_split = 0 the lists hold the whole Hamiltonian: pass zero
 * occupations (IQ) to gg_setham so that it adds no diagonal pieces. With
 * average_split = 1 they follow rangular's convention for rmcdhf: the
 * diagonal pieces that SETHAM adds from the occupations
 * (rmcdhf90/setham.f90:75-209 with FCO/GCO, fco.f90, gco.f90: I(aa) times
 * IQ(a), F^0 of every pair, F^k of closed subshells, G^k with a closed
 * subshell) are left out of the lists; pass the CSFs' occupations to
 * gg_setham.
 */
#ifndef GRASP_ANGULAR_H
#define GRASP_ANGULAR_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct ga_block ga_block;

/* One J/parity block of a CSF list in the arrays LODCSH2 fills
 * (lib9290/lodcsh2.f90:150-330). Per CSF r and subshell a (row-major
 * [ncsf][nw]): iq electrons; jqs 2J of an open subshell (0 otherwise);
 * nu seniority where the list names it (0: the only state of that J, or
 * the lowest seniority); xj 2X, the coupling of all open subshells up to
 * and including a (X of the first open subshell is its J; -1 for subshells
 * that are not open). two_j is the block's 2J. Coefficients with
 * |value| <= cutoff are dropped (cutoff < 0: 1e-12).                       */
typedef struct {
  int nw;
  const int *nak;     /* kappa of each subshell */
  int ncsf;
  const uint8_t *iq;
  const int *jqs;
  const int *nu;
  const int *xj;
  int two_j;
  double cutoff;
  int nthreads;       /* <= 0: all hardware threads */
  int average_split;  /* 1: leave SETHAM's occupation-driven diagonal pieces out */
} ga_block_spec;

int ga_block_generate(const ga_block_spec *spec, ga_block **out);
void ga_block_free(ga_block *b);
/* ncf, stored elements, kmaxf, and per list (T, V^0..V^kmaxf: kmaxf + 2
 * entries) the number of labels and of contributions.                     */
int ga_block_sizes(const ga_block *b, int *ncf, int64_t *nnz, int *kmaxf, int64_t *nlab, int64_t *ncontr);
int ga_block_structure(const ga_block *b, int64_t *iendc, int32_t *irow);
/* which = 0: T list; which = 1 + k: V^k list. start has nlab + 1 entries. */
int ga_block_list(const ga_block *b, int which, int32_t *lab, int64_t *start, int32_t *iclmn, int32_t *loc,
                  double *coeff);
const char *ga_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
