// Device helpers shared by the sigma kernels (sigma.cu) and the batched
// small-problem solver (batch.cu): phase words, sign flips, the argument
// block of a product and the same-spin row sweep.
#pragma once

#include <type_traits>

#include "common.cuh"
#include "df.cuh"

namespace sbdgb {
namespace sdev {

__device__ __forceinline__ double flip(double x, uint32_t ph) {
  return __longlong_as_double(__double_as_longlong(x) ^ ((unsigned long long)ph << 63));
}
__device__ __forceinline__ float flip(float x, uint32_t ph) {
  return __int_as_float(__float_as_int(x) ^ (int)(ph << 31));
}
__device__ __forceinline__ dfloat flip(dfloat x, uint32_t ph) { return dfloat(flip(x.hi, ph), flip(x.lo, ph)); }

// Float-float accumulator of the mixed form: an FP32 sum hi and the rounding
// errors of the additions into it in lo (Knuth's TwoSum), so hi + lo keeps
// FP32 partial sums to about 48 bits, as an FP64 accumulator would, with FP32
// instructions only.  The FP64 pipe of this GPU issues at 1/64 of the FP32
// rate; FP64 adds and conversions per element bounded the FP32 kernels.
struct FF {
  float hi, lo;
};
__device__ __forceinline__ void ff_add(FF &a, float x) {
  const float s = a.hi + x;
  const float bb = s - a.hi;
  a.lo += (a.hi - (s - bb)) + (x - bb);
  a.hi = s;
}
__device__ __forceinline__ void ff_add(FF &a, const FF &b) {
  ff_add(a, b.hi);
  a.lo += b.lo;
}
__device__ __forceinline__ float ff_value(const FF &a) { return a.hi + a.lo; }
// (h_hi + h_lo - s_hi - s_lo) * x as a float-float: the two differences are
// exact or nearly so when the shift is close to the diagonal (the case the
// shift is for), their sum is split by TwoSum, and fmaf recovers the rounding
// error of the leading product.
__device__ __forceinline__ FF ff_diag(float h_hi, float h_lo, float s_hi, float s_lo, float x) {
  const float a = h_hi - s_hi, b = h_lo - s_lo;
  const float dh = a + b;
  const float bb = dh - a;
  const float dl = (a - (dh - bb)) + (b - bb);
  const float p = dh * x;
  return FF{p, fmaf(dl, x, fmaf(dh, x, -p))};
}

// x * h as a float-float (the product's rounding error by one FMA): the
// diagonal term of an unshifted FP32 product.
__device__ __forceinline__ FF ff_prod(float h, float x) {
  const float p = h * x;
  return FF{p, fmaf(h, x, -p)};
}
__device__ __forceinline__ void acc_diag_f(FF &acc, float h, float x) { acc = ff_prod(h, x); }
template <typename A, typename X>
__device__ __forceinline__ void acc_diag_f(A &, float, X) {}  // only FP32 kernels read the FP32 diagonal

// Per-element accumulator: FP64 in the FP64 form, float-float in the FP32
// kernels of the mixed form, double-float (the vectors' own format) in its
// double-float phase.
template <typename T>
using AccT = typename std::conditional<std::is_same<T, float>::value, FF, T>::type;
__device__ __forceinline__ void acc_zero(double &a) { a = 0.0; }
__device__ __forceinline__ void acc_zero(FF &a) { a = FF{0.f, 0.f}; }
__device__ __forceinline__ void acc_zero(dfloat &a) { a = dfloat(0.f, 0.f); }
__device__ __forceinline__ void acc_add_part(double &, double) {}
__device__ __forceinline__ void acc_add_part(dfloat &, dfloat) {}
__device__ __forceinline__ void acc_add_part(FF &a, float part) { ff_add(a, part); }
__device__ __forceinline__ double acc_value(double a) { return a; }
__device__ __forceinline__ dfloat acc_value(dfloat a) { return a; }
__device__ __forceinline__ float acc_value(const FF &a) { return ff_value(a); }

// Precision index of an element type: 0 FP64, 1 FP32 (mixed form), 2 double-float.
template <typename T>
constexpr int prec_of() {
  return std::is_same<T, double>::value ? 0 : std::is_same<T, float>::value ? 1 : 2;
}

template <typename T>
struct Args {
  const uint64_t *astr, *bstr;
  uint32_t na, nb;
  const double *hii;
  const dfloat *hii_df;  // FP32 and double-float kernels: hii as hi + lo (no FP64 instruction in them)
  dfloat shift_df;       // the shift split the same way
  // FP32 kernels with no shift: hii rounded to FP32 (4 bytes a determinant
  // instead of 8; its rounding, 2^-24 relative, is that of the FP32 result)
  const float *hii_f;
  const T *C;   // N, row-major [ia][ib]
  const T *CT;  // N, transposed [ib][ia]
  T *S;
  int accumulate;
  SpinTables A, B;
  const T *val_sa, *val_da, *val_sb, *val_db;  // table values in storage precision
  const T *Jb;  // [npair][nb]
  const T *Ja;  // [npair][na]
  const T *Kp;  // [npair][npair]
  int npair;
  const uint32_t *tile_start, *tile_order;  // row tiles of the kernel's row spin
  double shift;  // sigma = (H - shift) C in the FP32 and double-float forms; the FP64 form has none
  int skip_ab = 0;  // 1: leave the alpha x beta single pairs to k_sigma_ab (sigma_ab.cu)
};

// Strings and phase masks as 32-bit words when norb <= 32 (half the integer
// work per element: one AND and one POPC instead of two each), 64-bit otherwise.
template <typename Wd>
__device__ __forceinline__ Wd word(const uint64_t *a, size_t i) {
  if constexpr (sizeof(Wd) == 4)
    return ldg(reinterpret_cast<const uint32_t *>(a) + 2 * i);  // low half (little endian)
  else
    return ldg(a + i);
}
__device__ __forceinline__ uint32_t parity(uint32_t x) { return __popc(x) & 1u; }
__device__ __forceinline__ uint32_t parity(unsigned long long x) { return __popcll(x) & 1u; }

// Phase conventions.  With interleaved determinants (the reference's, kB =
// false) an element's phase has an opposite-spin part: the parity of the
// opposite-spin string under the table entry's mask.  In the block ordering
// (all alpha creators before all beta ones, kB = true) it has none: every
// phase is the table entry's same-spin sign.  The two conventions differ by
// the sign eta(ia, ib) of each determinant (H_interleaved = eta H_block eta),
// so a solver can keep its vectors multiplied by eta and skip the
// opposite-spin parities; tests/test_sign_factorisation.py checks the
// identity exhaustively.
template <bool kB, typename Wd>
__device__ __forceinline__ Wd mask_of(const uint64_t *masks, size_t i) {
  if constexpr (kB)
    return Wd(0);
  else
    return word<Wd>(masks, i);
}
template <bool kB, typename Wd>
__device__ __forceinline__ uint32_t par(Wd x) {
  if constexpr (kB)
    return 0u;
  else
    return parity(x);
}
// eta(alpha, beta) as a parity: one transposition per (alpha p, beta q) pair
// with q < p, i.e. the parity of alpha AND the prefix parity of beta.
__device__ __forceinline__ uint32_t eta_parity(unsigned long long alpha, unsigned long long beta) {
  unsigned long long x = beta << 1;
  x ^= x << 1;
  x ^= x << 2;
  x ^= x << 4;
  x ^= x << 8;
  x ^= x << 16;
  x ^= x << 32;
  return __popcll(x & alpha) & 1u;
}

// One term v*x: into the FP64 accumulator directly, or into the FP32 partial
// sum of the current pair list (merged into the float-float accumulator once
// per list).
__device__ __forceinline__ void madd(double &acc, double &, double v, double x) { acc = fma(v, x, acc); }
__device__ __forceinline__ void madd(dfloat &acc, dfloat &, dfloat v, dfloat x) { acc = fma(v, x, acc); }
__device__ __forceinline__ void madd(FF &, float &part, float v, float x) { part = fmaf(v, x, part); }

// Vector loads and stores of VW consecutive elements (8, 16 or 32 bytes).
template <int VW, typename T>
__device__ __forceinline__ void load_v(const T *__restrict__ p, T (&x)[VW]) {
  static_assert(VW == 1 || sizeof(T) * VW == 8 || sizeof(T) * VW == 16 || sizeof(T) * VW == 32,
                "vector loads of 8, 16 or 32 bytes");
  if constexpr (VW == 1) {
    x[0] = ldg(p);
  } else if constexpr (sizeof(T) * VW == 32) {  // the double-float diagonal of four FP32 columns
    const uint4 u0 = ldg(reinterpret_cast<const uint4 *>(p)), u1 = ldg(reinterpret_cast<const uint4 *>(p) + 1);
    memcpy(x, &u0, 16);
    memcpy(reinterpret_cast<char *>(x) + 16, &u1, 16);
  } else if constexpr (sizeof(T) * VW == 16) {
    const uint4 u = ldg(reinterpret_cast<const uint4 *>(p));
    memcpy(x, &u, 16);
  } else {
    const uint2 u = ldg(reinterpret_cast<const uint2 *>(p));
    memcpy(x, &u, 8);
  }
}
template <int VW, typename T>
__device__ __forceinline__ void store_v(T *__restrict__ p, const T (&x)[VW]) {
  static_assert(VW == 1 || sizeof(T) * VW == 8 || sizeof(T) * VW == 16, "vector stores of 8 or 16 bytes");
  if constexpr (VW == 1) {
    *p = x[0];
  } else if constexpr (sizeof(T) * VW == 16) {
    uint4 u;
    memcpy(&u, x, 16);
    *reinterpret_cast<uint4 *>(p) = u;
  } else {
    uint2 u;
    memcpy(&u, x, 8);
    *reinterpret_cast<uint2 *>(p) = u;
  }
}

// Same-spin excitations of one row applied to this thread's CPT columns.
// In: ket-major input rows (ld = ldin); Jo: opposite-spin Coulomb table
// [npair][ldj] for the single excitations.  Element offsets are 32-bit
// (problems have fewer than 2^32 determinants): the address of a gather is
// one 32-bit multiply-add and one widening add.
template <int CPT, typename T, typename Wd, bool kB>
__device__ __forceinline__ void same_spin_row(const SpinTables &Tb, const T *__restrict__ vs,
                                              const T *__restrict__ vd, const T *__restrict__ Jo, uint32_t ldj,
                                              const T *__restrict__ In, uint32_t ldin, uint32_t row,
                                              const uint32_t (&col)[CPT], const bool (&ok)[CPT],
                                              const Wd (&opp)[CPT], AccT<T> (&acc)[CPT]) {
  T part[CPT];
#pragma unroll
  for (int c = 0; c < CPT; ++c) part[c] = T(0);
  // singles, two at a time
  const uint32_t p0 = ldg(Tb.off_s + row), p1 = ldg(Tb.off_s + row + 1);
  uint32_t p = p0;
  for (; p + 2 <= p1; p += 2) {
    uint32_t ket[2], code[2];
    T v[2];
    Wd m[2];
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      ket[u] = ldg(Tb.ket_s + p + u);
      code[u] = ldg(Tb.code_s + p + u);
      v[u] = ldg(vs + p + u);
      m[u] = mask_of<kB, Wd>(Tb.mask_s, p + u);
    }
#pragma unroll
    for (int c = 0; c < CPT; ++c)
      if (ok[c]) {
        T x[2], j[2];
#pragma unroll
        for (int u = 0; u < 2; ++u) {
          x[u] = ldg(In + (ket[u] * ldin + col[c]));
          j[u] = ldg(Jo + (((code[u] >> 16) & 0x7fffu) * ldj + col[c]));
        }
#pragma unroll
        for (int u = 0; u < 2; ++u) {
          const uint32_t ph = par<kB>(opp[c] & m[u]) ^ (code[u] >> 31);
          madd(acc[c], part[c], flip(v[u] + j[u], ph), x[u]);
        }
      }
  }
  if (p < p1) {
    const uint32_t ket = ldg(Tb.ket_s + p), code = ldg(Tb.code_s + p);
    const T v = ldg(vs + p);
    const Wd m = mask_of<kB, Wd>(Tb.mask_s, p);
#pragma unroll
    for (int c = 0; c < CPT; ++c)
      if (ok[c]) {
        const uint32_t ph = par<kB>(opp[c] & m) ^ (code >> 31);
        const T j = ldg(Jo + (((code >> 16) & 0x7fffu) * ldj + col[c]));
        madd(acc[c], part[c], flip(v + j, ph), ldg(In + (ket * ldin + col[c])));
      }
  }
  // doubles, four at a time
  const uint32_t d0 = ldg(Tb.off_d + row), d1 = ldg(Tb.off_d + row + 1);
  p = d0;
  for (; p + 4 <= d1; p += 4) {
    uint32_t ket[4];
    T v[4];
    Wd m[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      ket[u] = ldg(Tb.ket_d + p + u);
      v[u] = ldg(vd + p + u);
      m[u] = mask_of<kB, Wd>(Tb.mask_d, p + u);
    }
#pragma unroll
    for (int c = 0; c < CPT; ++c)
      if (ok[c]) {
        T x[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) x[u] = ldg(In + (ket[u] * ldin + col[c]));
#pragma unroll
        for (int u = 0; u < 4; ++u) madd(acc[c], part[c], flip(v[u], par<kB>(opp[c] & m[u])), x[u]);
      }
  }
  for (; p < d1; ++p) {
    const uint32_t ket = ldg(Tb.ket_d + p);
    const T v = ldg(vd + p);
    const Wd m = mask_of<kB, Wd>(Tb.mask_d, p);
#pragma unroll
    for (int c = 0; c < CPT; ++c)
      if (ok[c]) madd(acc[c], part[c], flip(v, par<kB>(opp[c] & m)), ldg(In + (ket * ldin + col[c])));
  }
#pragma unroll
  for (int c = 0; c < CPT; ++c) acc_add_part(acc[c], part[c]);
}


}  // namespace sdev

// sigma_ab.cu: the alpha x beta single pairs in a kernel of their own, added
// into a.S (block: the block ordering's phases).
template <typename T>
void launch_ab(const Problem &p, const sdev::Args<T> &a, bool block, cudaStream_t s);
// sigma_stream.cu: the streaming kernel for problems with few nonzeros per row
// (every task type in one pass; variant 0/1 = row tiles of 8/16 rows).
template <typename T, bool kB>
void launch_stream(const Problem &p, const sdev::Args<T> &a, int variant, cudaStream_t s);

}  // namespace sbdgb
