// Double-float arithmetic: a value is an unevaluated sum hi + lo of two FP32
// numbers (|lo| <= ulp(hi)/2), which carries 48 significand bits, with every
// operation done on the FP32 pipe.  On this GPU the FP64 pipe issues at 1/64
// of the FP32 rate, so a double-float multiply-add (about 15 FP32 operations)
// is several times cheaper than one FP64 FMA.  The mixed-precision solver runs
// its second phase in this format (relative rounding about 2^-47 per
// operation) before one final FP64 check of the result.
//
// The algorithms are the classical error-free transformations: TwoSum
// (Knuth), Fast2Sum (Dekker), and the product error from one fused
// multiply-add; addition renormalises through both error terms.
#pragma once

#include <cuda_runtime.h>

namespace sbdgb {

// The overloads below are for dfloat; keep the FP32/FP64 math functions
// visible to unqualified calls inside the namespace.
using ::fabs;
using ::fma;

struct __align__(8) dfloat {
  float hi, lo;
  dfloat() = default;
  __host__ __device__ constexpr dfloat(float h, float l) : hi(h), lo(l) {}
  __host__ __device__ explicit dfloat(double x) : hi((float)x), lo((float)(x - (double)(float)x)) {}
  __host__ __device__ explicit dfloat(float x) : hi(x), lo(0.f) {}
  __host__ __device__ explicit dfloat(int x) : dfloat((double)x) {}
  __host__ __device__ explicit operator double() const { return (double)hi + (double)lo; }
  __host__ __device__ explicit operator float() const { return hi + lo; }
};

namespace dfimpl {
__host__ __device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}
__host__ __device__ __forceinline__ void fast_two_sum(float a, float b, float &s, float &e) {
  s = a + b;
  e = b - (s - a);
}
}  // namespace dfimpl

__host__ __device__ __forceinline__ dfloat operator+(dfloat a, dfloat b) {
  float s, e, t, f;
  dfimpl::two_sum(a.hi, b.hi, s, e);
  dfimpl::two_sum(a.lo, b.lo, t, f);
  e += t;
  dfimpl::fast_two_sum(s, e, s, e);
  e += f;
  dfimpl::fast_two_sum(s, e, s, e);
  return dfloat(s, e);
}
__host__ __device__ __forceinline__ dfloat operator-(dfloat a) { return dfloat(-a.hi, -a.lo); }
__host__ __device__ __forceinline__ dfloat operator-(dfloat a, dfloat b) { return a + (-b); }
__host__ __device__ __forceinline__ dfloat operator*(dfloat a, dfloat b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  float s;
  dfimpl::fast_two_sum(p, e, s, e);
  return dfloat(s, e);
}
__host__ __device__ __forceinline__ dfloat operator/(dfloat a, dfloat b) {
  const float q1 = a.hi / b.hi;
  const dfloat r = a - b * dfloat(q1, 0.f);
  const float q2 = r.hi / b.hi;
  float s, e;
  dfimpl::fast_two_sum(q1, q2, s, e);
  return dfloat(s, e);
}
__host__ __device__ __forceinline__ dfloat &operator+=(dfloat &a, dfloat b) { return a = a + b; }
__host__ __device__ __forceinline__ dfloat &operator-=(dfloat &a, dfloat b) { return a = a - b; }
// a*b + c with the product's rounding error kept.
__host__ __device__ __forceinline__ dfloat fma(dfloat a, dfloat b, dfloat c) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  float s, t;
  dfimpl::two_sum(p, c.hi, s, t);
  t += e + c.lo;
  dfimpl::fast_two_sum(s, t, s, t);
  return dfloat(s, t);
}
__host__ __device__ __forceinline__ dfloat fabs(dfloat a) { return a.hi < 0.f ? -a : a; }
__host__ __device__ __forceinline__ bool operator<=(dfloat a, dfloat b) {
  return a.hi < b.hi || (a.hi == b.hi && a.lo <= b.lo);
}
__host__ __device__ __forceinline__ bool operator<(dfloat a, dfloat b) {
  return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo);
}

// Read-only cached load of any element type (dfloat as one 8-byte load).
template <typename T>
__device__ __forceinline__ T ldg(const T *p) {
  return __ldg(p);
}
__device__ __forceinline__ dfloat ldg(const dfloat *p) {
  const float2 v = __ldg(reinterpret_cast<const float2 *>(p));
  return dfloat(v.x, v.y);
}

}  // namespace sbdgb
