/*
 * sbd_oracle.c -- CPU restatement of the reference's TPB selected-CI path at
 * MPI size 1.  TEST INFRASTRUCTURE ONLY (see sbd_oracle.h): the checker for
 * the CUDA product and the "port" CPU baseline; never part of the product.
 *
 * Every function follows the cited reference lines step for step, including
 * the per-element evaluation strategy (interleaved determinant rebuilt per
 * bra element, Slater-Condon rules evaluated per matrix element, bit-by-bit
 * scans), so its run time is representative of the reference CPU path.
 */
#define _GNU_SOURCE
#include "sbd_oracle.h"

#include <math.h>
#include <omp.h>
#include <stdlib.h>
#include <string.h>

#define ORC_MAXW 16 /* max words of an interleaved determinant */

struct orc_ints {
  int L;
  int n2; /* 2L spin orbitals */
  double I0;
  double *I1; /* (2L)^2 row-major, integrals.h:13-25 */
  double *I2; /* 8-fold packed, integrals.h:67-110 */
  double *D;  /* direct (2L)^2 column-major, integrals.h:103-105 */
  double *X;  /* exchange (2L)^2 column-major, integrals.h:106-108 */
};

/* ---- integrals: chemistry/basic/integrals.h, makeintegrals.h ---------- */

static inline size_t orc_pair(int I, int J) {
  int a = I > J ? I : J, b = I > J ? J : I;
  return (size_t)a * (size_t)(a + 1) / 2 + (size_t)b;
}

/* twoInt::Value (integrals.h:94-102): zero unless the two spin pairs match. */
static inline double orc_I2(const orc_ints *t, int i, int j, int k, int l) {
  if (!((i % 2 == j % 2) && (k % 2 == l % 2))) return 0.0;
  size_t ij = orc_pair(i / 2, j / 2), kl = orc_pair(k / 2, l / 2);
  size_t a = ij > kl ? ij : kl, b = ij > kl ? kl : ij;
  return t->I2[a * (a + 1) / 2 + b];
}

orc_ints *orc_ints_create(int L, double I0, const double *h1, const double *eri_packed) {
  orc_ints *t = (orc_ints *)calloc(1, sizeof(orc_ints));
  int n2 = 2 * L;
  size_t B = (size_t)L * (size_t)(L + 1) / 2;
  size_t nI2 = B * (B + 1) / 2;
  t->L = L;
  t->n2 = n2;
  t->I0 = I0;
  t->I1 = (double *)calloc((size_t)n2 * n2, sizeof(double));
  t->I2 = (double *)malloc(nI2 * sizeof(double));
  t->D = (double *)calloc((size_t)n2 * n2, sizeof(double));
  t->X = (double *)calloc((size_t)n2 * n2, sizeof(double));
  memcpy(t->I2, eri_packed, nI2 * sizeof(double));
  /* makeintegrals.h:150-154: same-spin blocks only */
  for (int i = 0; i < L; ++i)
    for (int j = 0; j < L; ++j) {
      t->I1[(size_t)(2 * i) * n2 + 2 * j] = h1[i * L + j];
      t->I1[(size_t)(2 * i + 1) * n2 + 2 * j + 1] = h1[i * L + j];
    }
  /* makeintegrals.h:160-173 */
  for (int i = 0; i < L; ++i)
    for (int j = 0; j < L; ++j) {
      for (int si = 0; si < 2; ++si)
        for (int sj = 0; sj < 2; ++sj) {
          int p = 2 * i + si, q = 2 * j + sj;
          t->D[p + (size_t)n2 * q] = orc_I2(t, p, p, q, q);
          t->X[p + (size_t)n2 * q] = orc_I2(t, p, q, q, p);
        }
    }
  return t;
}

void orc_set_threads(int n) {
  if (n > 0) omp_set_num_threads(n);
}

void orc_ints_destroy(orc_ints *t) {
  if (!t) return;
  free(t->I1);
  free(t->I2);
  free(t->D);
  free(t->X);
  free(t);
}

/* ---- bit strings: chemistry/basic/determinants.h ---------------------- */

static inline int orc_getocc(const uint64_t *det, int bl, int x) {
  return (int)((det[x / bl] >> (x % bl)) & 1u);
}

/* DetFromAlphaBeta (determinants.h:129-150): alpha orbital i -> bit 2i,
 * beta orbital i -> bit 2i+1 of the interleaved determinant. */
static void orc_det(const uint64_t *A, const uint64_t *B, int bl, int L, uint64_t *D, int dwords) {
  for (int w = 0; w < dwords; ++w) D[w] = 0;
  for (int i = 0; i < L; ++i) {
    int blk = i / bl, pos = i % bl;
    if (A[blk] & ((uint64_t)1 << pos)) D[(2 * i) / bl] |= (uint64_t)1 << ((2 * i) % bl);
    if (B[blk] & ((uint64_t)1 << pos)) D[(2 * i + 1) / bl] |= (uint64_t)1 << ((2 * i + 1) % bl);
  }
}

/* parity (determinants.h:242-294): sign of the set bits in [start, end),
 * flipped again when the start bit itself is set. */
static inline void orc_parity(const uint64_t *det, int bl, int start, int end, double *sgn) {
  int bs = start / bl, os = start % bl, be = end / bl, oe = end % bl;
  int cnt = 0;
  if (bs == be) {
    uint64_t m = (((uint64_t)1 << oe) - 1) ^ (((uint64_t)1 << os) - 1);
    cnt += __builtin_popcountll(det[bs] & m);
  } else {
    if (os != 0) {
      cnt += __builtin_popcountll(det[bs] & ~(((uint64_t)1 << os) - 1));
      bs++;
    }
    for (int w = bs; w < be; ++w) cnt += __builtin_popcountll(det[w]);
    if (oe != 0) cnt += __builtin_popcountll(det[be] & (((uint64_t)1 << oe) - 1));
  }
  *sgn *= (cnt % 2) ? -1.0 : 1.0;
  if ((det[start / bl] >> (start % bl)) & 1u) *sgn *= -1.0;
}

/* ZeroExcite (determinants.h:451-474). */
static double orc_zero(const orc_ints *t, const uint64_t *det, int bl) {
  double e = 0.0;
  for (int i = 0; i < t->n2; ++i) {
    if (!orc_getocc(det, bl, i)) continue;
    e += t->I1[(size_t)i * t->n2 + i];
    for (int j = i + 1; j < t->n2; ++j) {
      if (!orc_getocc(det, bl, j)) continue;
      e += t->D[i + (size_t)t->n2 * j];
      if ((i % 2) == (j % 2)) e -= t->X[i + (size_t)t->n2 * j];
    }
  }
  return e + t->I0;
}

/* OneExcite (determinants.h:476-498): i occupied in det, a empty. */
static double orc_one(const orc_ints *t, const uint64_t *det, int dwords, int bl, int i, int a) {
  double sgn = 1.0;
  orc_parity(det, bl, i < a ? i : a, i < a ? a : i, &sgn);
  double e = t->I1[(size_t)a * t->n2 + i];
  for (int x = 0; x < dwords; ++x) {
    uint64_t bits = det[x];
    for (int pos = 0; pos < bl; ++pos) {
      if (bits & 1u) {
        int j = x * bl + pos;
        e += orc_I2(t, a, i, j, j) - orc_I2(t, a, j, j, i);
      }
      bits >>= 1;
    }
  }
  return e * sgn;
}

/* TwoExcite (determinants.h:500-518): i, j occupied in det; a, b empty. */
static double orc_two(const orc_ints *t, const uint64_t *det, int bl, int i, int j, int a, int b) {
  double sgn = 1.0;
  int I = i < j ? i : j, J = i < j ? j : i, A = a < b ? a : b, B = a < b ? b : a;
  orc_parity(det, bl, I < A ? I : A, I < A ? A : I, &sgn);
  orc_parity(det, bl, J < B ? J : B, J < B ? B : J, &sgn);
  if (A > J || B < I) sgn *= -1.0;
  return sgn * (orc_I2(t, A, I, B, J) - orc_I2(t, A, J, B, I));
}

/* difference (determinants.h:380-402) */
static inline int orc_diff(const uint64_t *a, const uint64_t *b, int bl, int L) {
  int full = L / bl, rem = L % bl, c = 0;
  for (int w = 0; w < full; ++w) c += __builtin_popcountll(a[w] ^ b[w]);
  if (rem > 0) c += __builtin_popcountll((a[full] ^ b[full]) & (((uint64_t)1 << rem) - 1));
  return c;
}

/* OrbitalDifference (determinants.h:404-449): x = in a not in b, y = in b
 * not in a, each ascending.  Returns counts through nx, ny. */
static void orc_orbdiff(const uint64_t *a, const uint64_t *b, int bl, int L, int *x, int *nx, int *y, int *ny) {
  int full = L / bl, rem = L % bl;
  *nx = 0;
  *ny = 0;
  for (int w = 0; w <= full; ++w) {
    int nbits = (w < full) ? bl : rem;
    if (nbits == 0) break;
    uint64_t m = (nbits >= 64) ? ~(uint64_t)0 : (((uint64_t)1 << nbits) - 1);
    uint64_t da = (a[w] & ~b[w]) & m, db = (b[w] & ~a[w]) & m;
    for (int p = 0; p < nbits; ++p) {
      if (da & ((uint64_t)1 << p)) {
        if (*nx < 4) x[*nx] = w * bl + p;
        (*nx)++;
      }
      if (db & ((uint64_t)1 << p)) {
        if (*ny < 4) y[*ny] = w * bl + p;
        (*ny)++;
      }
    }
  }
}

/* ---- excitation lists: chemistry/tpb/helper.h:185-342 ----------------- */

int orc_excitations(const uint64_t *strs, size_t n, int words, int bit_length, int L, int spin,
                    size_t *off_s, size_t *off_d, uint64_t *ket_s, int32_t *cran_s, uint64_t *ket_d,
                    int32_t *cran_d) {
  const int bl = bit_length;
  if (ket_s == NULL) {
    /* counting pass (helper.h:226-233, 256-263) */
#pragma omp parallel for schedule(dynamic, 16)
    for (size_t ia = 0; ia < n; ++ia) {
      size_t cs = 0, cd = 0;
      for (size_t ja = 0; ja < n; ++ja) {
        int d = orc_diff(strs + ia * words, strs + ja * words, bl, L);
        if (d == 2) cs++;
        if (d == 4) cd++;
      }
      off_s[ia + 1] = cs;
      off_d[ia + 1] = cd;
    }
    off_s[0] = 0;
    off_d[0] = 0;
    for (size_t i = 0; i < n; ++i) {
      off_s[i + 1] += off_s[i];
      off_d[i + 1] += off_d[i];
    }
    return 0;
  }
  int bad = 0;
  /* fill pass in ascending ket order (helper.h:235-243, 265-275, 297-305, 327-337) */
#pragma omp parallel for schedule(dynamic, 16) reduction(| : bad)
  for (size_t ia = 0; ia < n; ++ia) {
    size_t ps = off_s[ia], pd = off_d[ia];
    int cr[4], an[4], ncr, nan;
    for (size_t ja = 0; ja < n; ++ja) {
      const uint64_t *a = strs + ia * words, *b = strs + ja * words;
      int d = orc_diff(a, b, bl, L);
      if (d == 2) {
        orc_orbdiff(a, b, bl, L, cr, &ncr, an, &nan);
        if (ncr != 1 || nan != 1) bad = 1;
        ket_s[ps] = ja;
        cran_s[2 * ps + 0] = 2 * cr[0] + spin;
        cran_s[2 * ps + 1] = 2 * an[0] + spin;
        ps++;
      } else if (d == 4) {
        orc_orbdiff(a, b, bl, L, cr, &ncr, an, &nan);
        if (ncr != 2 || nan != 2) bad = 1;
        ket_d[pd] = ja;
        cran_d[4 * pd + 0] = 2 * cr[0] + spin;
        cran_d[4 * pd + 1] = 2 * cr[1] + spin;
        cran_d[4 * pd + 2] = 2 * an[0] + spin;
        cran_d[4 * pd + 3] = 2 * an[1] + spin;
        pd++;
      }
    }
  }
  return bad ? -1 : 0;
}

/* ---- diagonal: chemistry/tpb/qcham.h:289-340 --------------------------- */

void orc_hii(const orc_ints *t, const uint64_t *astr, size_t na, const uint64_t *bstr, size_t nb, int words,
             int bit_length, double *hii, size_t row_begin, size_t row_end) {
  const int bl = bit_length, L = t->L;
  const int dwords = (2 * L + bl - 1) / bl;
  if (row_end > na) row_end = na;
#pragma omp parallel
  {
    uint64_t det[ORC_MAXW];
#pragma omp for
    for (size_t ia = row_begin; ia < row_end; ++ia)
      for (size_t ib = 0; ib < nb; ++ib) {
        orc_det(astr + ia * words, bstr + ib * words, bl, L, det, dwords);
        hii[ia * nb + ib] = orc_zero(t, det, bl);
      }
  }
}

/* ---- sigma: chemistry/tpb/mult.h:114-621 (TRADMODE) --------------------- */

void orc_mult(const orc_ints *t, const uint64_t *astr, size_t na, const uint64_t *bstr, size_t nb, int words,
              int bit_length, const size_t *aoff_s, const uint64_t *aket_s, const int32_t *acran_s,
              const size_t *aoff_d, const uint64_t *aket_d, const int32_t *acran_d, const size_t *boff_s,
              const uint64_t *bket_s, const int32_t *bcran_s, const size_t *boff_d, const uint64_t *bket_d,
              const int32_t *bcran_d, const double *hii, const double *Wk, double *Wb, size_t row_begin,
              size_t row_end) {
  const int bl = bit_length, L = t->L;
  const int dwords = (2 * L + bl - 1) / bl;
  if (row_end > na) row_end = na;
  /* diagonal term (mult.h:169-174) */
#pragma omp parallel for
  for (size_t i = row_begin * nb; i < row_end * nb; ++i) Wb[i] += hii[i] * Wk[i];

  /* task type 2: alpha singles and doubles (mult.h:450-488) */
#pragma omp parallel
  {
    uint64_t det[ORC_MAXW];
#pragma omp for schedule(dynamic)
    for (size_t ia = row_begin; ia < row_end; ++ia)
      for (size_t ib = 0; ib < nb; ++ib) {
        size_t bra = ia * nb + ib;
        orc_det(astr + ia * words, bstr + ib * words, bl, L, det, dwords);
        for (size_t j = aoff_s[ia]; j < aoff_s[ia + 1]; ++j) {
          size_t ket = (size_t)aket_s[j] * nb + ib;
          Wb[bra] += orc_one(t, det, dwords, bl, acran_s[2 * j], acran_s[2 * j + 1]) * Wk[ket];
        }
        for (size_t j = aoff_d[ia]; j < aoff_d[ia + 1]; ++j) {
          size_t ket = (size_t)aket_d[j] * nb + ib;
          Wb[bra] += orc_two(t, det, bl, acran_d[4 * j], acran_d[4 * j + 1], acran_d[4 * j + 2], acran_d[4 * j + 3]) *
                     Wk[ket];
        }
      }
  }
  /* task type 1: beta singles and doubles (mult.h:489-525) */
#pragma omp parallel
  {
    uint64_t det[ORC_MAXW];
#pragma omp for schedule(dynamic)
    for (size_t ia = row_begin; ia < row_end; ++ia)
      for (size_t ib = 0; ib < nb; ++ib) {
        size_t bra = ia * nb + ib;
        orc_det(astr + ia * words, bstr + ib * words, bl, L, det, dwords);
        for (size_t j = boff_s[ib]; j < boff_s[ib + 1]; ++j) {
          size_t ket = ia * nb + (size_t)bket_s[j];
          Wb[bra] += orc_one(t, det, dwords, bl, bcran_s[2 * j], bcran_s[2 * j + 1]) * Wk[ket];
        }
        for (size_t j = boff_d[ib]; j < boff_d[ib + 1]; ++j) {
          size_t ket = ia * nb + (size_t)bket_d[j];
          Wb[bra] += orc_two(t, det, bl, bcran_d[4 * j], bcran_d[4 * j + 1], bcran_d[4 * j + 2], bcran_d[4 * j + 3]) *
                     Wk[ket];
        }
      }
  }
  /* task type 0: alpha single x beta single (mult.h:527-557) */
#pragma omp parallel
  {
    uint64_t det[ORC_MAXW];
#pragma omp for schedule(dynamic)
    for (size_t ia = row_begin; ia < row_end; ++ia)
      for (size_t ib = 0; ib < nb; ++ib) {
        size_t bra = ia * nb + ib;
        orc_det(astr + ia * words, bstr + ib * words, bl, L, det, dwords);
        for (size_t j = aoff_s[ia]; j < aoff_s[ia + 1]; ++j) {
          size_t ja = (size_t)aket_s[j];
          for (size_t k = boff_s[ib]; k < boff_s[ib + 1]; ++k) {
            size_t ket = ja * nb + (size_t)bket_s[k];
            Wb[bra] += orc_two(t, det, bl, acran_s[2 * j], bcran_s[2 * k], acran_s[2 * j + 1], bcran_s[2 * k + 1]) *
                       Wk[ket];
          }
        }
      }
  }
}

size_t orc_hamiltonian_offdiag(const orc_ints *t, const uint64_t *astr, size_t na, const uint64_t *bstr, size_t nb,
                               int words, int bit_length, const size_t *aoff_s, const uint64_t *aket_s,
                               const int32_t *acran_s, const size_t *aoff_d, const uint64_t *aket_d,
                               const int32_t *acran_d, const size_t *boff_s, const uint64_t *bket_s,
                               const int32_t *bcran_s, const size_t *boff_d, const uint64_t *bket_d,
                               const int32_t *bcran_d, int64_t *rows, int64_t *cols, double *vals) {
  const int bl = bit_length, L = t->L;
  const int dwords = (2 * L + bl - 1) / bl;
  uint64_t det[ORC_MAXW];
  size_t k = 0;
#define ORC_EMIT(r, c, v)                  \
  do {                                     \
    if (rows) {                            \
      rows[k] = (int64_t)(r);              \
      cols[k] = (int64_t)(c);              \
      vals[k] = (v);                       \
    }                                      \
    k++;                                   \
  } while (0)
  for (size_t ia = 0; ia < na; ++ia)
    for (size_t ib = 0; ib < nb; ++ib) {
      size_t bra = ia * nb + ib;
      orc_det(astr + ia * words, bstr + ib * words, bl, L, det, dwords);
      for (size_t j = aoff_s[ia]; j < aoff_s[ia + 1]; ++j)
        ORC_EMIT(bra, (size_t)aket_s[j] * nb + ib, rows ? orc_one(t, det, dwords, bl, acran_s[2 * j], acran_s[2 * j + 1]) : 0.0);
      for (size_t j = aoff_d[ia]; j < aoff_d[ia + 1]; ++j)
        ORC_EMIT(bra, (size_t)aket_d[j] * nb + ib,
                 rows ? orc_two(t, det, bl, acran_d[4 * j], acran_d[4 * j + 1], acran_d[4 * j + 2], acran_d[4 * j + 3])
                      : 0.0);
      for (size_t j = boff_s[ib]; j < boff_s[ib + 1]; ++j)
        ORC_EMIT(bra, ia * nb + (size_t)bket_s[j], rows ? orc_one(t, det, dwords, bl, bcran_s[2 * j], bcran_s[2 * j + 1]) : 0.0);
      for (size_t j = boff_d[ib]; j < boff_d[ib + 1]; ++j)
        ORC_EMIT(bra, ia * nb + (size_t)bket_d[j],
                 rows ? orc_two(t, det, bl, bcran_d[4 * j], bcran_d[4 * j + 1], bcran_d[4 * j + 2], bcran_d[4 * j + 3])
                      : 0.0);
      for (size_t j = aoff_s[ia]; j < aoff_s[ia + 1]; ++j)
        for (size_t q = boff_s[ib]; q < boff_s[ib + 1]; ++q)
          ORC_EMIT(bra, (size_t)aket_s[j] * nb + (size_t)bket_s[q],
                   rows ? orc_two(t, det, bl, acran_s[2 * j], bcran_s[2 * q], acran_s[2 * j + 1], bcran_s[2 * q + 1])
                        : 0.0);
    }
#undef ORC_EMIT
  return k;
}

/* ---- vector algebra: framework/dm_vector.h:23-87 ------------------------ */

#define ORC_CHUNKS 64

double orc_inner(const double *x, const double *y, size_t n) {
  double part[ORC_CHUNKS];
#pragma omp parallel for schedule(static, 1)
  for (int c = 0; c < ORC_CHUNKS; ++c) {
    size_t lo = n * (size_t)c / ORC_CHUNKS, hi = n * (size_t)(c + 1) / ORC_CHUNKS;
    double s = 0.0, comp = 0.0;
    for (size_t i = lo; i < hi; ++i) {
      double v = x[i] * y[i] - comp;
      double tt = s + v;
      comp = (tt - s) - v;
      s = tt;
    }
    part[c] = s;
  }
  double sum = 0.0;
  for (int c = 0; c < ORC_CHUNKS; ++c) sum += part[c];
  return sum;
}

static double orc_normalize(double *x, size_t n) {
  double r = sqrt(orc_inner(x, x, n));
  double f = 1.0 / r;
#pragma omp parallel for
  for (size_t i = 0; i < n; ++i) x[i] *= f;
  return r;
}

void orc_symeig(int n, double *A, int lda, double *w) {
  double *V = (double *)calloc((size_t)n * n, sizeof(double));
  for (int i = 0; i < n; ++i) V[i + (size_t)n * i] = 1.0;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0, diag = 0.0;
    for (int q = 0; q < n; ++q)
      for (int p = 0; p < n; ++p) {
        double v = A[p + (size_t)lda * q];
        if (p != q) off += v * v;
        else diag += v * v;
      }
    if (off <= 1e-30 * (diag + 1e-300)) break;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        double apq = A[p + (size_t)lda * q];
        if (fabs(apq) < 1e-300) continue;
        double app = A[p + (size_t)lda * p], aqq = A[q + (size_t)lda * q];
        double theta = (aqq - app) / (2.0 * apq);
        double tt = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        double c = 1.0 / sqrt(tt * tt + 1.0), s = tt * c;
        for (int k = 0; k < n; ++k) { /* columns p, q */
          double akp = A[k + (size_t)lda * p], akq = A[k + (size_t)lda * q];
          A[k + (size_t)lda * p] = c * akp - s * akq;
          A[k + (size_t)lda * q] = s * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) { /* rows p, q */
          double apk = A[p + (size_t)lda * k], aqk = A[q + (size_t)lda * k];
          A[p + (size_t)lda * k] = c * apk - s * aqk;
          A[q + (size_t)lda * k] = s * apk + c * aqk;
        }
        for (int k = 0; k < n; ++k) {
          double vkp = V[k + (size_t)n * p], vkq = V[k + (size_t)n * q];
          V[k + (size_t)n * p] = c * vkp - s * vkq;
          V[k + (size_t)n * q] = s * vkp + c * vkq;
        }
      }
  }
  int *idx = (int *)malloc(sizeof(int) * n);
  for (int i = 0; i < n; ++i) idx[i] = i;
  for (int i = 1; i < n; ++i) { /* insertion sort by eigenvalue */
    int v = idx[i], j = i - 1;
    while (j >= 0 && A[idx[j] + (size_t)lda * idx[j]] > A[v + (size_t)lda * v]) {
      idx[j + 1] = idx[j];
      j--;
    }
    idx[j + 1] = v;
  }
  for (int i = 0; i < n; ++i) w[i] = A[idx[i] + (size_t)lda * idx[i]];
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) A[i + (size_t)lda * j] = V[i + (size_t)n * idx[j]];
  free(idx);
  free(V);
}

/* ---- Davidson: chemistry/tpb/davidson.h:707-970 ------------------------ */

/* The vector algebra of one step of the reference's Davidson
 * (chemistry/tpb/davidson.h:778-923) at subspace position ib, on n elements,
 * without the sigma product: the ib+1 projections <C_j|HC_ib> (:802-805),
 * the Ritz vector and residual over the ib+1 basis vectors (:818-843), their
 * normalisations, the preconditioner (:899-908) and the modified Gram-Schmidt
 * of the new direction (:909-923).  The Ritz coefficients are fixed (the
 * operation count does not depend on them), so this times the reference's
 * per-step vector work on a slice of a vector.  C holds ib+2 vectors of n
 * (C[ib+1] receives the new direction), HC ib+1, W and R one each. */
void orc_algebra_step(double *C, const double *HC, double *W, double *R, const double *hii, size_t n, int ib) {
  const double eps_reg = 1.0e-12;
  double *U = (double *)malloc(sizeof(double) * (size_t)(ib + 1));
  volatile double sink = 0.0;
  for (int jb = 0; jb <= ib; ++jb) sink += orc_inner(C + (size_t)jb * n, HC + (size_t)ib * n, n);
  for (int kb = 0; kb <= ib; ++kb) U[kb] = 1.0 / sqrt((double)(ib + 1));
  const double E0 = -1.0;
#pragma omp parallel for
  for (size_t s = 0; s < n; ++s) {
    double w = C[s] * U[0], r = HC[s] * (-U[0]);
    for (int kb = 1; kb <= ib; ++kb) {
      w += C[(size_t)kb * n + s] * U[kb];
      r += HC[(size_t)kb * n + s] * (-U[kb]);
    }
    W[s] = w;
    R[s] = r + E0 * w;
  }
  sink += orc_normalize(W, n);
  sink += orc_normalize(R, n);
  double *cn = C + (size_t)(ib + 1) * n;
#pragma omp parallel for
  for (size_t s = 0; s < n; ++s) {
    double den = E0 - hii[s];
    cn[s] = (fabs(den) > eps_reg) ? R[s] / den : R[s] / (den - eps_reg);
  }
  for (int kb = 0; kb < ib + 1; ++kb) {
    double olap = -orc_inner(C + (size_t)kb * n, cn, n);
    const double *ck = C + (size_t)kb * n;
#pragma omp parallel for
    for (size_t s = 0; s < n; ++s) cn[s] += ck[s] * olap;
  }
  sink += orc_normalize(cn, n);
  free(U);
  (void)sink;
}

int orc_davidson(const orc_ints *t, const uint64_t *astr, size_t na, const uint64_t *bstr, size_t nb, int words,
                 int bit_length, const size_t *aoff_s, const uint64_t *aket_s, const int32_t *acran_s,
                 const size_t *aoff_d, const uint64_t *aket_d, const int32_t *acran_d, const size_t *boff_s,
                 const uint64_t *bket_s, const int32_t *bcran_s, const size_t *boff_d, const uint64_t *bket_d,
                 const int32_t *bcran_d, const double *hii, double *W, int max_it, int max_nb, double eps,
                 double *energy, double *resid) {
  const size_t N = na * nb;
  const int nbk = max_nb;
  const double eps_reg = 1.0e-12;
  double *C = (double *)malloc(sizeof(double) * N * nbk);
  double *HC = (double *)malloc(sizeof(double) * N * nbk);
  double *R = (double *)malloc(sizeof(double) * N);
  double *H = (double *)calloc((size_t)nbk * nbk, sizeof(double));
  double *U = (double *)calloc((size_t)nbk * nbk, sizeof(double));
  double *E = (double *)calloc((size_t)nbk, sizeof(double));
  int nsigma = 0;
  double normR = 0.0;
  int done = 0;
  for (int it = 0; it < max_it && !done; ++it) {
    memcpy(C, W, sizeof(double) * N); /* C[0] = W (davidson.h:769-772, 959-962) */
    for (int ib = 0; ib < nbk; ++ib) {
      double *ci = C + (size_t)ib * N, *hci = HC + (size_t)ib * N;
      memset(hci, 0, sizeof(double) * N);
      orc_mult(t, astr, na, bstr, nb, words, bit_length, aoff_s, aket_s, acran_s, aoff_d, aket_d, acran_d, boff_s,
               bket_s, bcran_s, boff_d, bket_d, bcran_d, hii, ci, hci, 0, na);
      nsigma++;
      for (int jb = 0; jb <= ib; ++jb) { /* davidson.h:802-805 */
        H[jb + nbk * ib] = orc_inner(C + (size_t)jb * N, hci, N);
        H[ib + nbk * jb] = H[jb + nbk * ib];
      }
      for (int jb = 0; jb <= ib; ++jb)
        for (int kb = 0; kb <= ib; ++kb) U[jb + nbk * kb] = H[jb + nbk * kb];
      orc_symeig(ib + 1, U, nbk, E);
      /* Ritz vector and residual (davidson.h:818-843) */
#pragma omp parallel for
      for (size_t s = 0; s < N; ++s) {
        double w = C[s] * U[0], r = HC[s] * (-U[0]);
        for (int kb = 1; kb <= ib; ++kb) {
          w += C[(size_t)kb * N + s] * U[kb];
          r += HC[(size_t)kb * N + s] * (-U[kb]);
        }
        W[s] = w;
        R[s] = r + E[0] * w;
      }
      orc_normalize(W, N);
      normR = orc_normalize(R, N);
      if (normR < eps) {
        done = 1;
        break;
      }
      if (ib < nbk - 1) { /* preconditioner and MGS (davidson.h:899-923) */
        double *cn = C + (size_t)(ib + 1) * N;
#pragma omp parallel for
        for (size_t s = 0; s < N; ++s) {
          double den = E[0] - hii[s];
          cn[s] = (fabs(den) > eps_reg) ? R[s] / den : R[s] / (den - eps_reg);
        }
        for (int kb = 0; kb < ib + 1; ++kb) {
          double olap = -orc_inner(C + (size_t)kb * N, cn, N);
          const double *ck = C + (size_t)kb * N;
#pragma omp parallel for
          for (size_t s = 0; s < N; ++s) cn[s] += ck[s] * olap;
        }
        orc_normalize(cn, N);
      }
    }
  }
  *energy = E[0];
  if (resid) *resid = normR;
  free(C);
  free(HC);
  free(R);
  free(H);
  free(U);
  free(E);
  return nsigma;
}

/* ---- occupation density: chemistry/tpb/occupation.h:11-95 --------------- */

void orc_density(const uint64_t *astr, size_t na, const uint64_t *bstr, size_t nb, int words, int bit_length,
                 int L, const double *W, double *res) {
  for (int k = 0; k < 2 * L; ++k) res[k] = 0.0;
  for (size_t ia = 0; ia < na; ++ia)
    for (size_t ib = 0; ib < nb; ++ib) {
      const double w2 = W[ia * nb + ib] * W[ia * nb + ib];
      for (int p = 0; p < L; ++p) {
        if (orc_getocc(astr + ia * words, bit_length, p)) res[2 * p] += w2;
        if (orc_getocc(bstr + ib * words, bit_length, p)) res[2 * p + 1] += w2;
      }
    }
}

/* ---- one- and two-particle RDMs: chemistry/tpb/correlation.h:379-640 with
 * the element rules of chemistry/basic/correlation.h:17-299.
 * one[s*L*L + i + L*j], two[(s1 + 2*s2)*L^4 + index as in the reference]. */

static void orc_rdm_zero(const uint64_t *det, int dwords, int bl, int L, double w, double *one, double *two) {
  const size_t L2 = (size_t)L * L, L3 = L2 * L, L4 = L3 * L;
  int closed[256], nc = 0;
  for (int x = 0; x < 2 * L; ++x)
    if (orc_getocc(det, bl, x)) closed[nc++] = x;
  (void)dwords;
  for (int i = 0; i < nc; ++i) {
    const int oi = closed[i] / 2, si = closed[i] % 2;
    one[si * L2 + oi + (size_t)L * oi] += w;
    for (int j = i + 1; j < nc; ++j) {
      const int oj = closed[j] / 2, sj = closed[j] % 2;
      two[(si + 2 * sj) * L4 + oi + L * oj + L2 * oi + L3 * oj] += w;
      two[(sj + 2 * si) * L4 + oj + L * oi + L2 * oj + L3 * oi] += w;
      if (si == sj) {
        two[(si + 2 * sj) * L4 + oi + L * oj + L2 * oj + L3 * oi] -= w;
        two[(sj + 2 * si) * L4 + oj + L * oi + L2 * oi + L3 * oj] -= w;
      }
    }
  }
}

static void orc_rdm_one(const uint64_t *det, int dwords, int bl, int L, double v, int i, int a, double *one,
                        double *two) {
  const size_t L2 = (size_t)L * L, L3 = L2 * L, L4 = L3 * L;
  double sgn = 1.0;
  orc_parity(det, bl, i < a ? i : a, i < a ? a : i, &sgn);
  const int oi = i / 2, si = i % 2, oa = a / 2;
  const double x = v * sgn;
  one[si * L2 + oi + (size_t)L * oa] += x;
  for (int w = 0; w < dwords; ++w)
    for (int pos = 0; pos < bl; ++pos) {
      if (!((det[w] >> pos) & 1u)) continue;
      const int soj = w * bl + pos, oj = soj / 2, sj = soj % 2;
      two[(si + 2 * sj) * L4 + oa + oj * L + oi * L2 + oj * L3] += x;
      two[(sj + 2 * si) * L4 + oj + oa * L + oj * L2 + oi * L3] += x;
      if (si == sj) {
        two[(si + 2 * sj) * L4 + oa + oj * L + oj * L2 + oi * L3] -= x;
        two[(sj + 2 * si) * L4 + oj + oa * L + oi * L2 + oj * L3] -= x;
      }
    }
}

static void orc_rdm_two(const uint64_t *det, int bl, int L, double v, int i, int j, int a, int b, double *two) {
  const size_t L2 = (size_t)L * L, L4 = L2 * L2;
  double sgn = 1.0;
  const int I = i < j ? i : j, J = i < j ? j : i, A = a < b ? a : b, B = a < b ? b : a;
  orc_parity(det, bl, I < A ? I : A, I < A ? A : I, &sgn);
  orc_parity(det, bl, J < B ? J : B, J < B ? B : J, &sgn);
  if (A > J || B < I) sgn = -sgn;
  const int oi = I / 2, si = I % 2, oa = A / 2, sa = A % 2, oj = J / 2, sj = J % 2, ob = B / 2, sb = B % 2;
  const double x = sgn * v;
  if (si == sa) {
    two[(si + 2 * sj) * L4 + oa + (size_t)L * ob + L2 * (oi + (size_t)L * oj)] += x;
    two[(sj + 2 * si) * L4 + ob + (size_t)L * oa + L2 * (oj + (size_t)L * oi)] += x;
  }
  if (si == sb) {
    two[(si + 2 * sj) * L4 + oa + (size_t)L * ob + L2 * (oj + (size_t)L * oi)] -= x;
    two[(sj + 2 * si) * L4 + ob + (size_t)L * oa + L2 * (oi + (size_t)L * oj)] -= x;
  }
}

void orc_correlation(const uint64_t *astr, size_t na, const uint64_t *bstr, size_t nb, int words, int bit_length,
                     int L, const size_t *aoff_s, const uint64_t *aket_s, const int32_t *acran_s,
                     const size_t *aoff_d, const uint64_t *aket_d, const int32_t *acran_d, const size_t *boff_s,
                     const uint64_t *bket_s, const int32_t *bcran_s, const size_t *boff_d, const uint64_t *bket_d,
                     const int32_t *bcran_d, const double *W, double *one, double *two) {
  const int bl = bit_length, dwords = (2 * L + bl - 1) / bl;
  const size_t L2 = (size_t)L * L;
  memset(one, 0, sizeof(double) * 2 * L2);
  memset(two, 0, sizeof(double) * 4 * L2 * L2);
  uint64_t det[ORC_MAXW];
  for (size_t ia = 0; ia < na; ++ia)
    for (size_t ib = 0; ib < nb; ++ib) {
      const size_t bra = ia * nb + ib;
      orc_det(astr + ia * words, bstr + ib * words, bl, L, det, dwords);
      orc_rdm_zero(det, dwords, bl, L, W[bra] * W[bra], one, two);
      /* task type 2 */
      for (size_t j = aoff_s[ia]; j < aoff_s[ia + 1]; ++j)
        orc_rdm_one(det, dwords, bl, L, W[bra] * W[aket_s[j] * nb + ib], acran_s[2 * j], acran_s[2 * j + 1], one,
                    two);
      for (size_t j = aoff_d[ia]; j < aoff_d[ia + 1]; ++j)
        orc_rdm_two(det, bl, L, W[bra] * W[aket_d[j] * nb + ib], acran_d[4 * j], acran_d[4 * j + 1],
                    acran_d[4 * j + 2], acran_d[4 * j + 3], two);
      /* task type 1 */
      for (size_t j = boff_s[ib]; j < boff_s[ib + 1]; ++j)
        orc_rdm_one(det, dwords, bl, L, W[bra] * W[ia * nb + bket_s[j]], bcran_s[2 * j], bcran_s[2 * j + 1], one,
                    two);
      for (size_t j = boff_d[ib]; j < boff_d[ib + 1]; ++j)
        orc_rdm_two(det, bl, L, W[bra] * W[ia * nb + bket_d[j]], bcran_d[4 * j], bcran_d[4 * j + 1],
                    bcran_d[4 * j + 2], bcran_d[4 * j + 3], two);
      /* task type 0 */
      for (size_t j = aoff_s[ia]; j < aoff_s[ia + 1]; ++j)
        for (size_t k = boff_s[ib]; k < boff_s[ib + 1]; ++k)
          orc_rdm_two(det, bl, L, W[bra] * W[aket_s[j] * nb + bket_s[k]], acran_s[2 * j], bcran_s[2 * k],
                      acran_s[2 * j + 1], bcran_s[2 * k + 1], two);
    }
}
