/*
 * sbd_oracle: CPU restatement of the reference's tensor-product-basis (TPB)
 * selected-CI path at MPI size 1.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA product
 * (tests/, __graft_entry__.smoke(), and the CPU-baseline leg of bench.py are
 * its only users).  The product library never links, loads or calls it.
 *
 * Parity is pinned against the reference itself: oracle/_ref/sbdref (the
 * reference's own headers compiled in place by oracle/Makefile) produced the
 * golden fixtures under tests/golden/ that this restatement must match
 * bit-for-bit (tables) and to 1e-12 (hii, sigma, energies).
 *
 * Data conventions follow the reference exactly:
 *   - a spin string is `words` machine words, `bit_length` orbital bits per
 *     word, orbital p in word p/bit_length, bit p%bit_length
 *     (framework/bit_manipulation.h:195-233);
 *   - spin-orbital index: alpha orbital p -> 2p, beta orbital p -> 2p+1
 *     (chemistry/basic/determinants.h:105-150);
 *   - one-body integrals in spin-orbital form (2L)^2 row-major
 *     (chemistry/basic/integrals.h:13-25, makeintegrals.h:150-154);
 *   - two-body integrals 8-fold packed, B = L(L+1)/2 pair index, B(B+1)/2
 *     entries (integrals.h:94-102, makeintegrals.h:143-145).
 */
#ifndef SBD_ORACLE_H
#define SBD_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_ints orc_ints;

/* Builds the integral tables of SetupIntegrals (makeintegrals.h:123-174) from
 * spatial h1 (L*L, row-major) and the 8-fold packed ERI (B(B+1)/2 doubles). */
orc_ints *orc_ints_create(int L, double I0, const double *h1, const double *eri_packed);
void orc_ints_destroy(orc_ints *ints);

/* Threads of the following parallel loops (omp_set_num_threads); n <= 0 keeps
 * the current setting.  A launcher may export OMP_NUM_THREADS=1 before the
 * OpenMP runtime starts; the timed CPU baseline sets its own count here. */
void orc_set_threads(int n);

/* Excitation lists of one spin (helper.h:185-342, GenerateExcitation with
 * bra = ket = the whole list, i.e. MPI size 1).  spin = 0 (alpha) stores
 * spin-orbital indices 2p, spin = 1 (beta) stores 2p+1.
 * Two calls: with offsets only (others NULL) to count; then with all
 * arrays allocated from the counts (off_s[n], off_d[n] = totals). */
int orc_excitations(const uint64_t *strs, size_t n, int words, int bit_length, int L, int spin,
                    size_t *off_s, size_t *off_d, uint64_t *ket_s, int32_t *cran_s, uint64_t *ket_d,
                    int32_t *cran_d);

/* Diagonal hii[ia*nb+ib] (qcham.h:289-340 -> determinants.h:451-474) for the
 * bra alpha rows [row_begin, row_end). */
void orc_hii(const orc_ints *ints, const uint64_t *astr, size_t na, const uint64_t *bstr, size_t nb,
             int words, int bit_length, double *hii, size_t row_begin, size_t row_end);

/* Matrix-free sigma, Wb += H*Wk (TRADMODE mult, chemistry/tpb/mult.h:114-621,
 * CPU loop :440-558, the three tasks of size-1 MakeHelpers, helper.h:752-767).
 * Tables are the CSR lists from orc_excitations for alpha (a*) and beta (b*).
 * row_begin/row_end restrict the bra alpha rows that are computed (the full
 * product is row_begin=0,row_end=na); used to time a bounded sample. */
void orc_mult(const orc_ints *ints, const uint64_t *astr, size_t na, const uint64_t *bstr, size_t nb,
              int words, int bit_length, const size_t *aoff_s, const uint64_t *aket_s, const int32_t *acran_s,
              const size_t *aoff_d, const uint64_t *aket_d, const int32_t *acran_d, const size_t *boff_s,
              const uint64_t *bket_s, const int32_t *bcran_s, const size_t *boff_d, const uint64_t *bket_d,
              const int32_t *bcran_d, const double *hii, const double *Wk, double *Wb, size_t row_begin,
              size_t row_end);

/* Explicit Hamiltonian off-diagonal triplets (same element formulas as
 * orc_mult; the stored-H idea of chemistry/tpb/qcham.h:10-287).  With rows ==
 * NULL it only counts.  Returns the count. */
size_t orc_hamiltonian_offdiag(const orc_ints *ints, const uint64_t *astr, size_t na, const uint64_t *bstr,
                               size_t nb, int words, int bit_length, const size_t *aoff_s,
                               const uint64_t *aket_s, const int32_t *acran_s, const size_t *aoff_d,
                               const uint64_t *aket_d, const int32_t *acran_d, const size_t *boff_s,
                               const uint64_t *bket_s, const int32_t *bcran_s, const size_t *boff_d,
                               const uint64_t *bket_d, const int32_t *bcran_d, int64_t *rows, int64_t *cols,
                               double *vals);

/* Single-root Davidson of chemistry/tpb/davidson.h:707-970 (restart every
 * max_nb steps with C0 = W, diagonal preconditioner with the 1e-12 guard,
 * modified Gram-Schmidt, Kahan-summed inner products).  The projected
 * eigenproblem is solved by a sorted cyclic Jacobi in place of LAPACK dsyev.
 * W holds the initial vector on entry and the normalized Ritz vector on exit.
 * Returns the number of sigma products used; *energy receives E0. */
int orc_davidson(const orc_ints *ints, const uint64_t *astr, size_t na, const uint64_t *bstr, size_t nb,
                 int words, int bit_length, const size_t *aoff_s, const uint64_t *aket_s, const int32_t *acran_s,
                 const size_t *aoff_d, const uint64_t *aket_d, const int32_t *acran_d, const size_t *boff_s,
                 const uint64_t *bket_s, const int32_t *bcran_s, const size_t *boff_d, const uint64_t *bket_d,
                 const int32_t *bcran_d, const double *hii, double *W, int max_it, int max_nb, double eps,
                 double *energy, double *resid);

/* Occupation density of W (OccupationDensity, chemistry/tpb/occupation.h:
 * 11-95): res[2p] = sum |W|^2 over determinants with alpha orbital p
 * occupied, res[2p+1] the same for beta. */
void orc_density(const uint64_t *astr, size_t na, const uint64_t *bstr, size_t nb, int words, int bit_length,
                 int L, const double *W, double *res);

/* One- and two-particle RDMs of W (Correlation at MPI size 1, chemistry/tpb/
 * correlation.h:379-640, element rules chemistry/basic/correlation.h:17-299).
 * one: 2 blocks of L*L (spin s at s*L*L), two: 4 blocks of L^4 (spin pair
 * s1 + 2*s2), indexed as in the reference.  Serial, fixed order. */
void orc_correlation(const uint64_t *astr, size_t na, const uint64_t *bstr, size_t nb, int words, int bit_length,
                     int L, const size_t *aoff_s, const uint64_t *aket_s, const int32_t *acran_s,
                     const size_t *aoff_d, const uint64_t *aket_d, const int32_t *acran_d, const size_t *boff_s,
                     const uint64_t *bket_s, const int32_t *bcran_s, const size_t *boff_d, const uint64_t *bket_d,
                     const int32_t *bcran_d, const double *W, double *one, double *two);

/* Kahan-compensated inner product (framework/dm_vector.h:23-51). */
double orc_inner(const double *x, const double *y, size_t n);
/* The vector algebra of one Davidson step at subspace position ib on n
 * elements (timing only; C: ib+2 vectors, HC: ib+1). */
void orc_algebra_step(double *C, const double *HC, double *W, double *R, const double *hii, size_t n, int ib);

/* Symmetric eigensolver for the small projected matrix: cyclic Jacobi with
 * eigenvalues sorted ascending (stands in for hp_numeric.h:503-520 dsyev).
 * A is n x n column-major with leading dimension lda; on exit its first n
 * columns hold the eigenvectors. */
void orc_symeig(int n, double *A, int lda, double *w);

#ifdef __cplusplus
}
#endif
#endif
