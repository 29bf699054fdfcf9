// Device helpers shared by the sigma kernels (sigma.cu) and the batched
// small-problem solver (batch.cu): phase words, sign flips, the argument
// block of a product and the same-spin row sweep.
#pragma once

#include <type_traits>

#include "common.cuh"

namespace sbdgb {
namespace sdev {

__device__ __forceinline__ double flip(double x, uint32_t ph) {
  return __longlong_as_double(__double_as_longlong(x) ^ ((unsigned long long)ph << 63));
}
__device__ __forceinline__ float flip(float x, uint32_t ph) {
  return __int_as_float(__float_as_int(x) ^ (int)(ph << 31));
}

template <typename T>
struct Args {
  const uint64_t *astr, *bstr;
  uint32_t na, nb;
  const double *hii;
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
  double shift;  // sigma = (H - shift) C; 0 except in the mixed solver's inner products
};

// Strings and phase masks as 32-bit words when norb <= 32 (half the integer
// work per element: one AND and one POPC instead of two each), 64-bit otherwise.
template <typename Wd>
__device__ __forceinline__ Wd word(const uint64_t *a, size_t i) {
  if constexpr (sizeof(Wd) == 4)
    return __ldg(reinterpret_cast<const uint32_t *>(a) + 2 * i);  // low half (little endian)
  else
    return __ldg(a + i);
}
__device__ __forceinline__ uint32_t parity(uint32_t x) { return __popc(x) & 1u; }
__device__ __forceinline__ uint32_t parity(unsigned long long x) { return __popcll(x) & 1u; }

template <typename T>
__device__ __forceinline__ void madd(double &acc, T &part, T v, T x) {
  if constexpr (std::is_same<T, double>::value)
    acc = fma(v, x, acc);
  else
    part = fmaf(v, x, part);
}

// Same-spin excitations of one row applied to this thread's CPT columns.
// In: ket-major input rows (ld = ldin); Jo: opposite-spin Coulomb table
// [npair][ldj] for the single excitations.  Element offsets are 32-bit
// (problems have fewer than 2^32 determinants): the address of a gather is
// one 32-bit multiply-add and one widening add.
template <int CPT, typename T, typename Wd>
__device__ __forceinline__ void same_spin_row(const SpinTables &Tb, const T *__restrict__ vs,
                                              const T *__restrict__ vd, const T *__restrict__ Jo, uint32_t ldj,
                                              const T *__restrict__ In, uint32_t ldin, uint32_t row,
                                              const uint32_t (&col)[CPT], const bool (&ok)[CPT],
                                              const Wd (&opp)[CPT], double (&acc)[CPT]) {
  T part[CPT];
#pragma unroll
  for (int c = 0; c < CPT; ++c) part[c] = T(0);
  // singles, two at a time
  const uint32_t p0 = __ldg(Tb.off_s + row), p1 = __ldg(Tb.off_s + row + 1);
  uint32_t p = p0;
  for (; p + 2 <= p1; p += 2) {
    uint32_t ket[2], code[2];
    T v[2];
    Wd m[2];
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      ket[u] = __ldg(Tb.ket_s + p + u);
      code[u] = __ldg(Tb.code_s + p + u);
      v[u] = __ldg(vs + p + u);
      m[u] = word<Wd>(Tb.mask_s, p + u);
    }
#pragma unroll
    for (int c = 0; c < CPT; ++c)
      if (ok[c]) {
        T x[2], j[2];
#pragma unroll
        for (int u = 0; u < 2; ++u) {
          x[u] = __ldg(In + (ket[u] * ldin + col[c]));
          j[u] = __ldg(Jo + (((code[u] >> 16) & 0x7fffu) * ldj + col[c]));
        }
#pragma unroll
        for (int u = 0; u < 2; ++u) {
          const uint32_t ph = parity(opp[c] & m[u]) ^ (code[u] >> 31);
          madd<T>(acc[c], part[c], flip(v[u] + j[u], ph), x[u]);
        }
      }
  }
  if (p < p1) {
    const uint32_t ket = __ldg(Tb.ket_s + p), code = __ldg(Tb.code_s + p);
    const T v = __ldg(vs + p);
    const Wd m = word<Wd>(Tb.mask_s, p);
#pragma unroll
    for (int c = 0; c < CPT; ++c)
      if (ok[c]) {
        const uint32_t ph = parity(opp[c] & m) ^ (code >> 31);
        const T j = __ldg(Jo + (((code >> 16) & 0x7fffu) * ldj + col[c]));
        madd<T>(acc[c], part[c], flip(v + j, ph), __ldg(In + (ket * ldin + col[c])));
      }
  }
  // doubles, four at a time
  const uint32_t d0 = __ldg(Tb.off_d + row), d1 = __ldg(Tb.off_d + row + 1);
  p = d0;
  for (; p + 4 <= d1; p += 4) {
    uint32_t ket[4];
    T v[4];
    Wd m[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      ket[u] = __ldg(Tb.ket_d + p + u);
      v[u] = __ldg(vd + p + u);
      m[u] = word<Wd>(Tb.mask_d, p + u);
    }
#pragma unroll
    for (int c = 0; c < CPT; ++c)
      if (ok[c]) {
        T x[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) x[u] = __ldg(In + (ket[u] * ldin + col[c]));
#pragma unroll
        for (int u = 0; u < 4; ++u) madd<T>(acc[c], part[c], flip(v[u], parity(opp[c] & m[u])), x[u]);
      }
  }
  for (; p < d1; ++p) {
    const uint32_t ket = __ldg(Tb.ket_d + p);
    const T v = __ldg(vd + p);
    const Wd m = word<Wd>(Tb.mask_d, p);
#pragma unroll
    for (int c = 0; c < CPT; ++c)
      if (ok[c]) madd<T>(acc[c], part[c], flip(v, parity(opp[c] & m)), __ldg(In + (ket * ldin + col[c])));
  }
  if constexpr (!std::is_same<T, double>::value) {
#pragma unroll
    for (int c = 0; c < CPT; ++c) acc[c] += (double)part[c];
  }
}


}  // namespace sdev
}  // namespace sbdgb
