// Davidson eigensolvers on the device (replace sbd::Davidson,
// chemistry/tpb/davidson.h:707-970, and its GPU form chemistry/basic/
// davidson_thrust.h:97-385 / :389-675).
//
// The reference solves one root with a single-vector Davidson: subspace up to
// max_nb, Ritz pair from the projected matrix, residual R = E0 W - H W,
// diagonal preconditioner R/(E0 - d) with a 1e-12 guard, modified
// Gram-Schmidt, restart C0 = W (which recomputes sigma(W)).
//
// FP64 solver: the same steps generalised to nroots.  Each step adds the
// corrected directions of the unconverged roots as one block: one pass of
// dots against the basis, one fused projection, a Gram matrix, and a
// Cholesky-style orthonormalisation written straight into the basis (a second
// projection pass only when a norm drops below 1/sqrt(2), the "twice is
// enough" rule).  Restarts keep the nroots Ritz vectors together with their
// sigma vectors, formed from the stored H*V instead of a new sigma product;
// Ritz vectors are materialised only at a restart and at the end.  Vectors
// stay resident in HBM; only the projected (<= max_nb)^2 matrix and a few
// norms cross to the host per step.
//
// Mixed solver: each root keeps an FP64 vector x (and its FP64 sigma) that is
// never rounded to FP32.  Corrections live in an FP32 subspace W with FP32
// sigma products.  Rayleigh-Ritz runs on span{x, W} as a generalised
// symmetric problem whose x-W overlaps are computed in FP64 (W is only
// orthogonal to x to FP32 accuracy); every refine_every steps the Ritz vectors
// are assembled in FP64, their FP64 sigma and FP64 residual are recomputed
// (iterative refinement), and convergence is judged on that FP64 residual.
// The FP32 subspace is kept across refinements and dropped only when full.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <numeric>
#include <type_traits>

#include "common.cuh"
#include "small_eig.h"

namespace sbdgb {

namespace {

constexpr int kRed = 256;  // threads per reduction block
constexpr int kMaxV = 8;   // basis columns per dots pass
constexpr int kMaxW = 4;   // right-hand columns per dots pass
constexpr int kMaxCoef = 64 * 16;
constexpr int kMaxBlock = 8;  // new directions per step
constexpr int kMaxChunks = 16;  // dots passes batched behind one host read-back

// Small coefficient sets travel as kernel parameters (no host-to-device copy,
// no staging buffer to protect between launches).
template <int M>
struct Vals {
  double v[M];
};
template <int M>
struct FVals {
  float v[M];
};

template <typename T, int M>
struct Ptrs {
  const T *p[M];
};

// partial[b][i*NW+j] = sum over this block's elements of V_i * W_j.  FP32 x
// FP32 uses FP32 products with per-thread Kahan compensation; anything with an
// FP64 operand accumulates with FP64 FMAs.
template <typename TV, typename TW, int NV, int NW>
__global__ void __launch_bounds__(kRed) k_dots(Ptrs<TV, kMaxV> V, Ptrs<TW, kMaxW> W, size_t N,
                                               double *__restrict__ partial) {
  constexpr bool kF32 = std::is_same<TV, float>::value && std::is_same<TW, float>::value;
  constexpr bool kDF = std::is_same<TV, dfloat>::value || std::is_same<TW, dfloat>::value;
  using Acc = typename std::conditional<kF32, float, typename std::conditional<kDF, dfloat, double>::type>::type;
  Acc acc[NV][NW], cmp[NV][NW];
#pragma unroll
  for (int i = 0; i < NV; ++i)
#pragma unroll
    for (int j = 0; j < NW; ++j) {
      acc[i][j] = Acc(0);
      cmp[i][j] = Acc(0);
    }
  for (size_t e = blockIdx.x * (size_t)kRed + threadIdx.x; e < N; e += (size_t)gridDim.x * kRed) {
    Acc w[NW];
#pragma unroll
    for (int j = 0; j < NW; ++j) w[j] = (Acc)ldg(W.p[j] + e);
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      const Acc v = (Acc)ldg(V.p[i] + e);
#pragma unroll
      for (int j = 0; j < NW; ++j) {
        if constexpr (kF32) {
          const float y = v * w[j] - cmp[i][j];
          const float t = acc[i][j] + y;
          cmp[i][j] = (t - acc[i][j]) - y;
          acc[i][j] = t;
        } else {
          acc[i][j] = fma(v, w[j], acc[i][j]);
        }
      }
    }
  }
  __shared__ double red[kRed / 32][NV * NW];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < NV; ++i)
#pragma unroll
    for (int j = 0; j < NW; ++j) {
      double x = (double)acc[i][j] - (double)cmp[i][j];
      for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
      if (lane == 0) red[warp][i * NW + j] = x;
    }
  __syncthreads();
  for (int t = threadIdx.x; t < NV * NW; t += kRed) {
    double x = 0.0;
    for (int w2 = 0; w2 < kRed / 32; ++w2) x += red[w2][t];
    partial[(size_t)blockIdx.x * NV * NW + t] = x;
  }
}

// Sums the per-block partials in block order (deterministic).
__global__ void k_sum_partials(const double *__restrict__ partial, int nblocks, int width, double *__restrict__ out) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= width) return;
  double s = 0.0;
  for (int b = 0; b < nblocks; ++b) s += partial[(size_t)b * width + t];
  out[t] = s;
}

template <typename F>
struct CombineArgs {
  const F *V;
  const F *HV;
  size_t N;
  int nv;
  int k;
  const double *hii;
  const dfloat *hii_df;  // hii as double-float (read instead of hii by the FP32 and double-float forms)
  F *X;             // k x N or null
  F *HX;            // k x N or null
  F *T;             // k x N or null: preconditioned residual
  F *U;             // k x N or null: X / (theta - d), for the Olsen correction of T
  double *partial;  // blocks x k residual norm^2 partials (x 3k with U: norm^2, x.T, x.U)
  Vals<kMaxCoef> coef;  // nv x k column-major (coef[j + nv*r])
  Vals<16> theta;       // k
  const double *coef_dev;   // or these on the device (the Rayleigh-Ritz result), when not null
  const double *theta_dev;
};

// 1/x.  FP64: the correctly rounded FP32 reciprocal refined by one
// Newton-Raphson step, r <- r + r (1 - x r), which squares its relative error
// (2^-24 -> 2^-48, then FP64 rounding): two FP64 FMAs and two conversions in
// place of an FP64 division, whose instruction sequence on this GPU's 1/64-rate
// FP64 pipe cost more than the combine's multiply-adds.  |x| >= 1e-12 here
// (the preconditioner's guard), well inside the FP32 range.  FP32 and
// double-float: their own division.
__device__ __forceinline__ double recip(double x) {
  if (!(fabs(x) < 1e30)) return 1.0 / x;  // outside the FP32 range of the seed
  const double r = (double)(1.0f / (float)x);
  return fma(r, fma(-x, r, 1.0), r);
}
__device__ __forceinline__ float recip(float x) { return 1.0f / x; }
__device__ __forceinline__ dfloat recip(dfloat x) { return dfloat(1.0f, 0.0f) / x; }

// X_r = V c_r, HX_r = HV c_r, R_r = HX_r - theta_r X_r, T_r = R_r / (theta_r - d)
// (davidson.h:818-843 and the preconditioner :899-908, 1e-12 guard).  With U
// it also writes U_r = X_r / (theta_r - d) and sums x.T and x.U, from which
// the host forms Olsen's correction T_r - eps_r U_r (eps_r = x.T / x.U), the
// component of the preconditioned residual orthogonal to the Ritz vector.
// Where the diagonal is nearly exact (weakly coupled determinants) the plain
// correction is almost parallel to X and the subspace stops growing.
// F is the storage and arithmetic precision (FP64, or FP32 in the first phase
// of the two-phase mixed form); the block sums are FP64.
template <int K, typename F>
__global__ void __launch_bounds__(kRed) k_combine(CombineArgs<F> a) {
  __shared__ F cs[kMaxCoef];
  __shared__ F th[16];
  for (int t = threadIdx.x; t < a.nv * K; t += kRed) cs[t] = (F)(a.coef_dev ? a.coef_dev[t] : a.coef.v[t]);
  if (threadIdx.x < K) th[threadIdx.x] = (F)(a.theta_dev ? a.theta_dev[threadIdx.x] : a.theta.v[threadIdx.x]);
  __syncthreads();
  F rn[K], xt[K], xu[K];
#pragma unroll
  for (int r = 0; r < K; ++r) rn[r] = xt[r] = xu[r] = F(0);
  for (size_t e = blockIdx.x * (size_t)kRed + threadIdx.x; e < a.N; e += (size_t)gridDim.x * kRed) {
    F x[K], h[K];
#pragma unroll
    for (int r = 0; r < K; ++r) {
      x[r] = F(0);
      h[r] = F(0);
    }
    for (int j = 0; j < a.nv; ++j) {
      const F v = ldg(a.V + (size_t)j * a.N + e);
      const F hv = ldg(a.HV + (size_t)j * a.N + e);
#pragma unroll
      for (int r = 0; r < K; ++r) {
        x[r] = fma(v, cs[j + a.nv * r], x[r]);
        h[r] = fma(hv, cs[j + a.nv * r], h[r]);
      }
    }
    F d = F(0);
    if constexpr (std::is_same<F, double>::value) {
      if (a.hii) d = ldg(a.hii + e);
    } else if constexpr (std::is_same<F, float>::value) {
      if (a.hii_df) d = ldg(a.hii_df + e).hi;
    } else {
      if (a.hii_df) d = ldg(a.hii_df + e);
    }
#pragma unroll
    for (int r = 0; r < K; ++r) {
      const F res = h[r] - th[r] * x[r];
      rn[r] = fma(res, res, rn[r]);
      if (a.X) a.X[(size_t)r * a.N + e] = x[r];
      if (a.HX) a.HX[(size_t)r * a.N + e] = h[r];
      if (a.T) {
        F den = th[r] - d;
        if (fabs(den) <= F(1.0e-12)) den -= F(1.0e-12);
        const F inv = recip(den);  // one reciprocal for both quotients
        const F t = res * inv;
        a.T[(size_t)r * a.N + e] = t;
        if (a.U) {
          const F u = x[r] * inv;
          a.U[(size_t)r * a.N + e] = u;
          xt[r] = fma(x[r], t, xt[r]);
          xu[r] = fma(x[r], u, xu[r]);
        }
      }
    }
  }
  constexpr int W3 = 3 * K;
  __shared__ double red[kRed / 32][W3];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int width = a.U ? W3 : K;
#pragma unroll
  for (int r = 0; r < W3; ++r) {
    double x = (double)(r < K ? rn[r] : (r < 2 * K ? xt[r - K] : xu[r - 2 * K]));
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if (lane == 0) red[warp][r] = x;
  }
  __syncthreads();
  if (threadIdx.x < width) {
    double x = 0.0;
    for (int w2 = 0; w2 < kRed / 32; ++w2) x += red[w2][threadIdx.x];
    a.partial[(size_t)blockIdx.x * width + threadIdx.x] = x;
  }
}

// T_r -= eps_r U_r (Olsen's correction, eps on the device).
template <typename T>
__global__ void __launch_bounds__(kRed) k_olsen(T *__restrict__ Tv, const T *__restrict__ U, const Vals<kMaxBlock> eps,
                                                 int k, size_t N) {
  for (size_t e = blockIdx.x * (size_t)kRed + threadIdx.x; e < N; e += (size_t)gridDim.x * kRed)
    for (int r = 0; r < k; ++r) {
      const T ep = (T)eps.v[r];
      Tv[(size_t)r * N + e] = fma(-ep, U[(size_t)r * N + e], Tv[(size_t)r * N + e]);
    }
}

// T_r -= sum_j V_j G[j][r]  (G column-major, ld = nv), in the vectors' precision.
template <typename T, int K>
__global__ void __launch_bounds__(kRed) k_project_out(const T *__restrict__ V, int nv, size_t N,
                                                       const Vals<kMaxCoef> G, T *__restrict__ Tv) {
  __shared__ T gs[kMaxCoef];
  for (int t = threadIdx.x; t < nv * K; t += kRed) gs[t] = (T)G.v[t];
  __syncthreads();
  for (size_t e = blockIdx.x * (size_t)kRed + threadIdx.x; e < N; e += (size_t)gridDim.x * kRed) {
    T t[K];
#pragma unroll
    for (int r = 0; r < K; ++r) t[r] = Tv[(size_t)r * N + e];
    for (int j = 0; j < nv; ++j) {
      const T v = ldg(V + (size_t)j * N + e);
#pragma unroll
      for (int r = 0; r < K; ++r) t[r] = fma(-v, gs[j + nv * r], t[r]);
    }
#pragma unroll
    for (int r = 0; r < K; ++r) Tv[(size_t)r * N + e] = t[r];
  }
}

// Y_q = sum_j X_j M[j + nx*q], q < ny (a small basis change, written to Y).
template <typename T>
__global__ void __launch_bounds__(kRed) k_lincomb(const T *__restrict__ X, int nx, size_t N,
                                                   const Vals<kMaxBlock * kMaxBlock> M, int ny, T *__restrict__ Y) {
  __shared__ T ms[kMaxBlock * kMaxBlock];
  for (int t = threadIdx.x; t < nx * ny; t += kRed) ms[t] = (T)M.v[t];
  __syncthreads();
  for (size_t e = blockIdx.x * (size_t)kRed + threadIdx.x; e < N; e += (size_t)gridDim.x * kRed) {
    T x[kMaxBlock];
    for (int j = 0; j < nx; ++j) x[j] = ldg(X + (size_t)j * N + e);
    for (int q = 0; q < ny; ++q) {
      T y = T(0);
      for (int j = 0; j < nx; ++j) y = fma(x[j], ms[j + nx * q], y);
      Y[(size_t)q * N + e] = y;
    }
  }
}

// Unit vector on `pos`, plus (amp > 0) a small deterministic pseudo-random
// component on every entry.  The lowest-diagonal guess can lie in one sector of
// an exact symmetry of H (e.g. alpha/beta exchange when both lists are equal);
// an FP64 Davidson started there never leaves that sector, so the guess gets a
// component along every direction (splitmix64 of the index, in [-amp, amp]).
__global__ void k_fill_unit(double *__restrict__ y, size_t N, size_t pos, double amp, uint64_t seed) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < N; e += (size_t)gridDim.x * blockDim.x) {
    double v = (e == pos) ? 1.0 : 0.0;
    if (amp > 0.0) {
      uint64_t x = (uint64_t)e * 0x9E3779B97F4A7C15ull + seed;
      x ^= x >> 30;
      x *= 0xBF58476D1CE4E5B9ull;
      x ^= x >> 27;
      x *= 0x94D049BB133111EBull;
      x ^= x >> 31;
      v += amp * ((double)(x >> 11) * (2.0 / 9007199254740992.0) - 1.0);
    }
    y[e] = v;
  }
}

// Block-wise argmin over hii skipping already chosen positions.
__global__ void k_argmin(const double *__restrict__ h, size_t N, const unsigned long long *__restrict__ skip,
                         int nskip, double *__restrict__ bval, unsigned long long *__restrict__ bidx) {
  double best = INFINITY;
  unsigned long long bi = ~0ull;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < N; e += (size_t)gridDim.x * blockDim.x) {
    bool sk = false;
    for (int q = 0; q < nskip; ++q) sk |= (skip[q] == e);
    const double v = h[e];
    if (!sk && (v < best || (v == best && e < bi))) {
      best = v;
      bi = e;
    }
  }
  __shared__ double sv[256];
  __shared__ unsigned long long si[256];
  sv[threadIdx.x] = best;
  si[threadIdx.x] = bi;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      double v2 = sv[threadIdx.x + o];
      unsigned long long i2 = si[threadIdx.x + o];
      if (v2 < sv[threadIdx.x] || (v2 == sv[threadIdx.x] && i2 < si[threadIdx.x])) {
        sv[threadIdx.x] = v2;
        si[threadIdx.x] = i2;
      }
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    bval[blockIdx.x] = sv[0];
    bidx[blockIdx.x] = si[0];
  }
}

// ---- mixed-solver kernels ----------------------------------------------------

// Xf_j = fp32(X_j), Rf_j = fp32(S_j - theta_j X_j): the anchors and their FP64
// residuals rounded once per refinement (the residual is small, so its FP32
// copy keeps FP32 relative accuracy of a small vector).
__global__ void k_make_anchor_f32(const double *__restrict__ X, const double *__restrict__ S,
                                  const Vals<kMaxBlock> theta, int k, size_t N, float *__restrict__ Xf,
                                  float *__restrict__ Rf) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < N; e += (size_t)gridDim.x * blockDim.x)
    for (int j = 0; j < k; ++j) {
      const double x = X[(size_t)j * N + e];
      Xf[(size_t)j * N + e] = (float)x;
      Rf[(size_t)j * N + e] = (float)fma(-theta.v[j], x, S[(size_t)j * N + e]);
    }
}

struct MixedResArgs {
  const float *Xf, *Rf, *W, *HW;
  int k, m, nq;
  size_t N;
  const double *hii;
  float *T;            // out: nq preconditioned residuals
  float *U;            // out: nq Ritz vectors / (theta - d), for Olsen's correction
  double *partial;     // blocks x 3nq: residual norm^2, x.T, x.U
  FVals<kMaxBlock * 3 * 64> coef;  // per root q: [k cx | k dth | m cw], stride 3*64
  FVals<kMaxBlock> thw;            // nq Ritz values minus the shift of HW
  Vals<kMaxBlock> theta;           // nq Ritz values (preconditioner)
};

// For each root q of the block:
//   r_q = sum_j (Rf_j + dth_jq Xf_j) cx_jq + sum_l (HW_l - theta_q W_l) cw_lq
//   T_q = r_q / (theta_q - d) with the reference's 1e-12 guard,
//   U_q = x_q / (theta_q - d), x_q = sum_j Xf_j cx_jq + sum_l W_l cw_lq,
// and the sums x.T and x.U of Olsen's correction (see k_combine).
// FP32 arithmetic with compensated sums; Xf, Rf, W, HW are read once for all roots.
__device__ __forceinline__ void kahan_add(float &s, float &c, float v) {
  const float y = v - c;
  const float t = s + y;
  c = (t - s) - y;
  s = t;
}

template <int K>
__global__ void __launch_bounds__(kRed) k_mixed_residual(MixedResArgs a) {
  __shared__ float c[K][3 * 64];
  __shared__ float th[K];
  for (int t = threadIdx.x; t < K * 3 * 64; t += kRed) c[t / (3 * 64)][t % (3 * 64)] = a.coef.v[t];
  if (threadIdx.x < K) th[threadIdx.x] = a.thw.v[threadIdx.x];
  __syncthreads();
  float s[3 * K], comp[3 * K];
#pragma unroll
  for (int q = 0; q < 3 * K; ++q) {
    s[q] = 0.f;
    comp[q] = 0.f;
  }
  for (size_t e = blockIdx.x * (size_t)kRed + threadIdx.x; e < a.N; e += (size_t)gridDim.x * kRed) {
    float r[K], x[K];
#pragma unroll
    for (int q = 0; q < K; ++q) r[q] = x[q] = 0.f;
    for (int j = 0; j < a.k; ++j) {
      const float xf = ldg(a.Xf + (size_t)j * a.N + e), rf = ldg(a.Rf + (size_t)j * a.N + e);
#pragma unroll
      for (int q = 0; q < K; ++q) {
        r[q] = fmaf(fmaf(c[q][64 + j], xf, rf), c[q][j], r[q]);
        x[q] = fmaf(xf, c[q][j], x[q]);
      }
    }
    for (int l = 0; l < a.m; ++l) {
      const float w = ldg(a.W + (size_t)l * a.N + e), hw = ldg(a.HW + (size_t)l * a.N + e);
#pragma unroll
      for (int q = 0; q < K; ++q) {
        r[q] = fmaf(fmaf(-th[q], w, hw), c[q][128 + l], r[q]);
        x[q] = fmaf(w, c[q][128 + l], x[q]);
      }
    }
    const double d = ldg(a.hii + e);
#pragma unroll
    for (int q = 0; q < K; ++q) {
      kahan_add(s[q], comp[q], r[q] * r[q]);
      double den = a.theta.v[q] - d;
      if (fabs(den) <= 1.0e-12) den -= 1.0e-12;
      const float t = (float)((double)r[q] / den), u = (float)((double)x[q] / den);
      a.T[(size_t)q * a.N + e] = t;
      a.U[(size_t)q * a.N + e] = u;
      kahan_add(s[K + q], comp[K + q], x[q] * t);
      kahan_add(s[2 * K + q], comp[2 * K + q], x[q] * u);
    }
  }
  __shared__ double red[kRed / 32][3 * K];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < 3 * K; ++q) {
    double v = (double)s[q] - (double)comp[q];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[warp][q] = v;
  }
  __syncthreads();
  if (threadIdx.x < 3 * K) {
    double t = 0.0;
    for (int w2 = 0; w2 < kRed / 32; ++w2) t += red[w2][threadIdx.x];
    a.partial[(size_t)blockIdx.x * 3 * K + threadIdx.x] = t;
  }
}

// D_j = fp32(X_j) - Xf_j: the step of the anchors over one refinement (the
// search direction kept when the FP32 subspace is dropped).
__global__ void k_anchor_step_f32(const double *__restrict__ X, const float *__restrict__ Xf, int k, size_t N,
                                  float *__restrict__ D) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < N; e += (size_t)gridDim.x * blockDim.x)
    for (int j = 0; j < k; ++j) D[(size_t)j * N + e] = (float)X[(size_t)j * N + e] - Xf[(size_t)j * N + e];
}

// y = sum_j X_j cx_j (FP64) + fp64(sum_l W_l cw_l) (FP32): the refined Ritz vector.
__global__ void __launch_bounds__(kRed) k_mixed_assemble(const double *__restrict__ X, int k, const float *__restrict__ W,
                                                         int m, size_t N, const Vals<64> cx, const FVals<64> cw,
                                                         double *__restrict__ y) {
  __shared__ double sx[64];
  __shared__ float sw[64];
  for (int t = threadIdx.x; t < k; t += kRed) sx[t] = cx.v[t];
  for (int t = threadIdx.x; t < m; t += kRed) sw[t] = cw.v[t];
  __syncthreads();
  for (size_t e = blockIdx.x * (size_t)kRed + threadIdx.x; e < N; e += (size_t)gridDim.x * kRed) {
    double v = 0.0;
    for (int j = 0; j < k; ++j) v = fma(ldg(X + (size_t)j * N + e), sx[j], v);
    float w = 0.f;
    for (int l = 0; l < m; ++l) w = fmaf(ldg(W + (size_t)l * N + e), sw[l], w);
    y[e] = v + (double)w;
  }
}

// ---- Lanczos kernels ------------------------------------------------------------

// HC -= alpha C; next = HC; partial sums of |HC|^2 (one Lanczos step's
// three-term update, lanczos.h:244-261).
__global__ void __launch_bounds__(kRed) k_lz_update(double *__restrict__ HC, const double *__restrict__ Cb,
                                                     double *__restrict__ next, const double a, size_t N,
                                                     double *__restrict__ partial) {
  double s = 0.0;
  for (size_t e = blockIdx.x * (size_t)kRed + threadIdx.x; e < N; e += (size_t)gridDim.x * kRed) {
    const double h = fma(-a, ldg(Cb + e), HC[e]);
    HC[e] = h;
    next[e] = h;
    s = fma(h, h, s);
  }
  __shared__ double red[kRed / 32];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < kRed / 32; ++w) t += red[w];
    partial[blockIdx.x] = t;
  }
}

// next /= beta; HC = -beta * C (lanczos.h:263, 281-291 at communicator size 1).
__global__ void __launch_bounds__(kRed) k_lz_scale(double *__restrict__ next, double *__restrict__ HC,
                                                    const double *__restrict__ Cb, const double b, size_t N) {
  const double ib = 1.0 / b;
  for (size_t e = blockIdx.x * (size_t)kRed + threadIdx.x; e < N; e += (size_t)gridDim.x * kRed) {
    next[e] *= ib;
    HC[e] = -b * ldg(Cb + e);
  }
}

// W = sum_j u_j C_j over the n Krylov vectors (lanczos.h:300-312).
__global__ void __launch_bounds__(kRed) k_lz_ritz(const double *__restrict__ C, int n, size_t N, const Vals<64> u,
                                                   double *__restrict__ W) {
  __shared__ double us[64];
  for (int t = threadIdx.x; t < n; t += kRed) us[t] = u.v[t];
  __syncthreads();
  for (size_t e = blockIdx.x * (size_t)kRed + threadIdx.x; e < N; e += (size_t)gridDim.x * kRed) {
    double w = 0.0;
    for (int j = 0; j < n; ++j) w = fma(us[j], ldg(C + (size_t)j * N + e), w);
    W[e] = w;
  }
}

// ---- Rayleigh-Ritz on the device ------------------------------------------------

// M[(i0 + i) + ld (j0 + j)] = sum over blocks of partial[b][i * mw + j] (and the
// transposed entry when sym): a dots pass written into the projected matrix.
__global__ void k_sum_partials_mat(const double *__restrict__ partial, int nblocks, int mv, int mw,
                                   double *__restrict__ M, int ld, int i0, int j0, int sym) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= mv * mw) return;
  double x = 0.0;
  for (int b = 0; b < nblocks; ++b) x += partial[(size_t)b * mv * mw + t];
  const int i = i0 + t / mw, j = j0 + t % mw;
  M[i + (size_t)ld * j] = x;
  if (sym) M[j + (size_t)ld * i] = x;
}

constexpr int kRR = 64;          // largest projected matrix (max_nb <= 64)
constexpr int kRRThreads = 1024;  // one element of the n x n matrices per thread (n <= 32)

// Sum over the block (kRRThreads threads) of one value per thread.
__device__ __forceinline__ double rr_block_sum(double v, double *tmp) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) tmp[threadIdx.x >> 5] = v;
  __syncthreads();
  double r = 0.0;
  for (int w = 0; w < kRRThreads / 32; ++w) r += tmp[w];
  __syncthreads();
  return r;
}

// Eigenvalues (ascending) and eigenvectors of the symmetric part of the n x n
// leading block of Hs (ld), n <= 64, by one block: out[0..n) the eigenvalues,
// out[n + i + n j] the eigenvector matrix (column j).  The reference solves
// this with LAPACK dsyev on the host (framework/hp_numeric.h:503-520).
//
// Parallel-order Jacobi: each sweep is n' - 1 rounds (n' = n rounded up to
// even) of the round-robin pairing; the n'/2 rotations of a round act on
// disjoint index pairs, so n'/2 threads compute them at once and every
// element of A <- J^T A J and of V <- V J is then formed by its own thread
// from four (two) elements of the previous round.
//
// Warm start: when the first nw basis columns are unchanged since the
// previous call (the subspace only grew), that call's eigenvectors, still in
// out (n = nw), diagonalise their block.  The iteration then starts from
// Y^T A Y with Y = diag(those eigenvectors, identity): diagonal but for the
// new rows and columns, so a few sweeps converge it.
__global__ void __launch_bounds__(kRRThreads) k_rr(const double *__restrict__ Hs, int ld, int n, int nw,
                                                   double *__restrict__ out) {
  extern __shared__ double sm[];
  const int nn = n * n;
  double *Acur = sm, *Anext = sm + nn, *Vcur = sm + 2 * nn, *Vnext = sm + 3 * nn;
  __shared__ double ca[kRR], cb[kRR], tmp[kRRThreads / 32];
  __shared__ int partner[kRR];
  const int tid = threadIdx.x;
  for (int t = tid; t < nn; t += kRRThreads) {
    const int i = t % n, j = t / n;
    Anext[t] = 0.5 * (Hs[i + (size_t)ld * j] + Hs[j + (size_t)ld * i]);
    Vcur[t] = (i < nw && j < nw) ? out[nw + i + nw * j] : (i == j ? 1.0 : 0.0);
  }
  __syncthreads();
  if (nw > 0) {
    // Vnext = A Y, then Acur = Y^T (A Y); Y is block diagonal (Y_old, I)
    for (int t = tid; t < nn; t += kRRThreads) {
      const int i = t % n, j = t / n;
      double x = 0.0;
      if (j < nw)
        for (int k = 0; k < nw; ++k) x = fma(Anext[i + n * k], Vcur[k + n * j], x);
      else
        x = Anext[i + n * j];
      Vnext[t] = x;
    }
    __syncthreads();
    for (int t = tid; t < nn; t += kRRThreads) {
      const int i = t % n, j = t / n;
      double x = 0.0;
      if (i < nw)
        for (int k = 0; k < nw; ++k) x = fma(Vcur[k + n * i], Vnext[k + n * j], x);
      else
        x = Vnext[i + n * j];
      Acur[t] = x;
    }
  } else {
    for (int t = tid; t < nn; t += kRRThreads) Acur[t] = Anext[t];
  }
  __syncthreads();
  const int n2 = (n + 1) & ~1, np = n2 / 2;
  auto idx = [&](int pos, int r) { return pos == 0 ? 0 : 1 + (pos - 1 + r) % (n2 - 1); };
  for (int sweep = 0; sweep < 60 && n > 1; ++sweep) {
    double off = 0.0, dg = 0.0;
    for (int t = tid; t < nn; t += kRRThreads) {
      const double x = Acur[t];
      if (t % n == t / n) dg += x * x; else off += x * x;
    }
    off = rr_block_sum(off, tmp);
    dg = rr_block_sum(dg, tmp);
    if (off <= 1e-30 * (dg + 1e-300)) break;
    for (int r = 0; r < n2 - 1; ++r) {
      if (tid < np) {
        const int a = idx(tid, r), b = idx(n2 - 1 - tid, r);
        const int pp = min(a, b), q = max(a, b);
        double c = 1.0, sn = 0.0;
        if (q < n) {  // q == n is the padding index of odd n
          const double apq = Acur[pp + n * q];
          if (fabs(apq) >= 1e-300) {
            const double th = (Acur[q + n * q] - Acur[pp + n * pp]) / (2.0 * apq);
            const double tt = (th >= 0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1.0));
            c = 1.0 / sqrt(tt * tt + 1.0);
            sn = tt * c;
          }
          // new column p = c col_p - s col_q, new column q = s col_p + c col_q
          partner[q] = pp;
          ca[q] = c;
          cb[q] = sn;
        }
        partner[pp] = q < n ? q : pp;
        ca[pp] = c;
        cb[pp] = q < n ? -sn : 0.0;
      }
      __syncthreads();
      for (int t = tid; t < nn; t += kRRThreads) {
        const int i = t % n, j = t / n, pi = partner[i], pj = partner[j];
        const double ci = ca[i], si = cb[i], cj = ca[j], sj = cb[j];
        Anext[t] = ci * (cj * Acur[i + n * j] + sj * Acur[i + n * pj]) + si * (cj * Acur[pi + n * j] + sj * Acur[pi + n * pj]);
        Vnext[t] = cj * Vcur[i + n * j] + sj * Vcur[i + n * pj];
      }
      __syncthreads();
      double *x = Acur;
      Acur = Anext;
      Anext = x;
      x = Vcur;
      Vcur = Vnext;
      Vnext = x;
    }
  }
  // ascending order: rank of each eigenvalue (ties by index), then scatter
  if (tid < n) {
    const double e = Acur[tid + n * tid];
    int rank = 0;
    for (int j = 0; j < n; ++j) {
      const double f = Acur[j + n * j];
      rank += (f < e) || (f == e && j < tid);
    }
    out[rank] = e;
    for (int i = 0; i < n; ++i) out[n + i + (size_t)n * rank] = Vcur[i + n * tid];
  }
}

// ---- host-side helper ----------------------------------------------------------

struct Solver {
  Problem &p;
  cudaStream_t s;
  size_t N;
  int blocks;
  double *partial = nullptr;  // blocks * kMaxV*kMaxW per batched dots pass
  double *red = nullptr;      // reduced results (device)
  double *hs = nullptr;       // projected matrix on the device (kRR x kRR, ld kRR)
  double *rr = nullptr;       // Rayleigh-Ritz result on the device: n eigenvalues, n x n eigenvectors
  double *host = nullptr;     // pinned read-back buffer of the context

  Solver(Problem &pp, cudaStream_t ss) : p(pp), s(ss), N(pp.N) {
    int dev = p.ctx->device, sms = 0;
    SBDGB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    size_t want = (N + kRed - 1) / kRed;
    blocks = (int)std::max<size_t>(1, std::min<size_t>(want, (size_t)sms * 4));
    partial = (double *)workspace(p, WS_PARTIAL,
                                  sizeof(double) * ((size_t)blocks * kMaxV * kMaxW * kMaxChunks + 64));
    red = (double *)workspace(p, WS_RED, sizeof(double) * (4096 + kRR * kRR + kRR + kRR * kRR));
    hs = red + 4096;
    rr = hs + kRR * kRR;
    host = pinned_buffer(p.ctx);
  }

  // The projected matrix columns [j0, j0 + nw) = V^T W written on the device
  // (rows 0..nv, and the transposed entries): no read-back.
  template <typename TV, typename TW>
  void dots_into_hs(const TV *V0, int nv, const TW *W0, int nw, int j0) {
    int batch = 0;
    for (int jb = 0; jb < nw; jb += kMaxW) {
      const int mw = std::min(kMaxW, nw - jb);
      Ptrs<TW, kMaxW> wp{};
      for (int j = 0; j < kMaxW; ++j) wp.p[j] = W0 + (size_t)(jb + std::min(j, mw - 1)) * N;
      for (int i0 = 0; i0 < nv; i0 += kMaxV) {
        const int mv = std::min(kMaxV, nv - i0);
        Ptrs<TV, kMaxV> vp{};
        for (int i = 0; i < kMaxV; ++i) vp.p[i] = V0 + (size_t)(i0 + std::min(i, mv - 1)) * N;
        double *part = partial + (size_t)(batch % kMaxChunks) * blocks * kMaxV * kMaxW;
        launch_dots<TV, TW>(vp, wp, mv, mw, part);
        k_sum_partials_mat<<<(mv * mw + 63) / 64, 64, 0, s>>>(part, blocks, mv, mw, hs, kRR, i0, j0 + jb, 1);
        count_launch(p.ctx);
        ++batch;
      }
    }
    SBDGB_CUDA(cudaGetLastError());
  }

  // Rayleigh-Ritz of the leading n x n block of the device projected matrix,
  // on the device (k_rr); the result stays in rr until read back.
  // nw > 0: the first nw basis columns are those of the previous call (no
  // change of basis since), whose eigenvectors are still in rr.
  void rayleigh_ritz(int n, int nw = 0) {
    SBDGB_REQUIRE(n >= 1 && n <= kRR, SBDGB_E_UNSUPPORTED, "projected matrix larger than 64");
    if (nw > n) nw = 0;
    const size_t smem = sizeof(double) * 4 * (size_t)n * n;
    ensure_dynamic_smem((const void *)k_rr, smem);
    k_rr<<<1, kRRThreads, smem, s>>>(hs, kRR, n, nw, rr);
    count_launch(p.ctx);
    SBDGB_CUDA(cudaGetLastError());
  }

  // The device projected matrix's leading n x n block (column-major, ld ld) to the host.
  void read_hs(int n, std::vector<double> &H, int ld) {
    SBDGB_CUDA(cudaMemcpy2DAsync(host, sizeof(double) * n, hs, sizeof(double) * kRR, sizeof(double) * n, n,
                                 cudaMemcpyDeviceToHost, s));
    SBDGB_CUDA(cudaStreamSynchronize(s));
    std::fill(H.begin(), H.end(), 0.0);
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) H[i + (size_t)ld * j] = host[i + (size_t)n * j];
  }
  // Replaces the device projected matrix by the n x n matrix H (column-major, ld ld).
  void write_hs(int n, const std::vector<double> &H, int ld) {
    double *stage = host + kPinnedDoubles / 2;
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) stage[i + (size_t)n * j] = H[i + (size_t)ld * j];
    SBDGB_CUDA(cudaMemcpy2DAsync(hs, sizeof(double) * kRR, stage, sizeof(double) * n, sizeof(double) * n, n,
                                 cudaMemcpyHostToDevice, s));
    SBDGB_CUDA(cudaStreamSynchronize(s));  // the staging area is reused
  }

  // Copies n reduced values from red to the pinned buffer and waits for them.
  const double *read_back(int n) {
    SBDGB_CUDA(cudaMemcpyAsync(host, red, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    SBDGB_CUDA(cudaStreamSynchronize(s));
    return host;
  }

  // G (column-major nv x nw) = V^T W, V columns at V0 + j*N.  All passes
  // (at most kMaxV x kMaxW each) are launched first and read back together.
  template <typename TV, typename TW>
  void dots(const TV *V0, int nv, const TW *const *W, int nw, std::vector<double> &G) {
    G.assign((size_t)nv * nw, 0.0);
    struct Pass {
      int i0, j0, mv, mw, off;
    };
    std::vector<Pass> batch;
    int width = 0;
    auto flush = [&]() {
      if (batch.empty()) return;
      const double *h = read_back(width);
      for (const Pass &q : batch)
        for (int i = 0; i < q.mv; ++i)
          for (int j = 0; j < q.mw; ++j) G[(size_t)(q.i0 + i) + (size_t)nv * (q.j0 + j)] = h[q.off + i * q.mw + j];
      batch.clear();
      width = 0;
    };
    for (int j0 = 0; j0 < nw; j0 += kMaxW) {
      const int mw = std::min(kMaxW, nw - j0);
      Ptrs<TW, kMaxW> wp{};
      for (int j = 0; j < kMaxW; ++j) wp.p[j] = W[j0 + std::min(j, mw - 1)];
      for (int i0 = 0; i0 < nv; i0 += kMaxV) {
        const int mv = std::min(kMaxV, nv - i0);
        Ptrs<TV, kMaxV> vp{};
        for (int i = 0; i < kMaxV; ++i) vp.p[i] = V0 + (size_t)(i0 + std::min(i, mv - 1)) * N;
        double *part = partial + (size_t)batch.size() * blocks * kMaxV * kMaxW;
        launch_dots<TV, TW>(vp, wp, mv, mw, part);
        k_sum_partials<<<(mv * mw + 63) / 64, 64, 0, s>>>(part, blocks, mv * mw, red + width);
        count_launch(p.ctx);
        batch.push_back({i0, j0, mv, mw, width});
        width += mv * mw;
        if ((int)batch.size() == kMaxChunks) flush();
      }
    }
    flush();
  }
  // G = V^T W for W contiguous too.
  template <typename TV, typename TW>
  void dots_c(const TV *V0, int nv, const TW *W0, int nw, std::vector<double> &G) {
    std::vector<const TW *> w(nw);
    for (int j = 0; j < nw; ++j) w[j] = W0 + (size_t)j * N;
    dots<TV, TW>(V0, nv, w.data(), nw, G);
  }

  template <typename TV, typename TW, int NV>
  void launch_dots_w(Ptrs<TV, kMaxV> vp, Ptrs<TW, kMaxW> wp, int mw, double *part) {
    switch (mw) {
      case 1: k_dots<TV, TW, NV, 1><<<blocks, kRed, 0, s>>>(vp, wp, N, part); break;
      case 2: k_dots<TV, TW, NV, 2><<<blocks, kRed, 0, s>>>(vp, wp, N, part); break;
      case 3: k_dots<TV, TW, NV, 3><<<blocks, kRed, 0, s>>>(vp, wp, N, part); break;
      default: k_dots<TV, TW, NV, 4><<<blocks, kRed, 0, s>>>(vp, wp, N, part); break;
    }
  }
  template <typename TV, typename TW>
  void launch_dots(Ptrs<TV, kMaxV> vp, Ptrs<TW, kMaxW> wp, int mv, int mw, double *part) {
    switch (mv) {
      case 1: launch_dots_w<TV, TW, 1>(vp, wp, mw, part); break;
      case 2: launch_dots_w<TV, TW, 2>(vp, wp, mw, part); break;
      case 3: launch_dots_w<TV, TW, 3>(vp, wp, mw, part); break;
      case 4: launch_dots_w<TV, TW, 4>(vp, wp, mw, part); break;
      case 5: launch_dots_w<TV, TW, 5>(vp, wp, mw, part); break;
      case 6: launch_dots_w<TV, TW, 6>(vp, wp, mw, part); break;
      case 7: launch_dots_w<TV, TW, 7>(vp, wp, mw, part); break;
      default: launch_dots_w<TV, TW, 8>(vp, wp, mw, part); break;
    }
    count_launch(p.ctx);
    SBDGB_CUDA(cudaGetLastError());
  }

  // Ritz vectors (optional), their sigma (optional) and the preconditioned
  // residuals (optional) of the combination c; returns the residual norms.
  //
  // With dev_rr, the coefficients and theta are the device Rayleigh-Ritz result
  // (rr: eigenvalues, then the eigenvector matrix) and come back to the host,
  // with the residual norms, in *rr_host (n eigenvalues, n x n eigenvectors).
  template <typename F>
  std::vector<double> combine(const F *V, const F *HV, int nv, int k, const std::vector<double> &c,
                              const std::vector<double> &theta, F *X, F *HX, F *T, F *U = nullptr,
                              std::vector<double> *rr_host = nullptr) {
    SBDGB_REQUIRE((size_t)nv * k <= (size_t)kMaxCoef && k <= 16, SBDGB_E_UNSUPPORTED, "subspace too large");
    if (!T) U = nullptr;
    CombineArgs<F> a{V, HV, N, nv, k, p.hii, p.hii_df, X, HX, T, U, partial, {}, {}, nullptr, nullptr};
    if (rr_host) {
      a.coef_dev = rr + nv;
      a.theta_dev = rr;
    } else {
      std::copy(c.begin(), c.begin() + (size_t)nv * k, a.coef.v);
      for (int r = 0; r < k; ++r) a.theta.v[r] = r < (int)theta.size() ? theta[r] : 0.0;
    }
    switch (k) {
#define SBDGB_K(KK) \
  case KK: k_combine<KK, F><<<blocks, kRed, 0, s>>>(a); break;
      SBDGB_K(1) SBDGB_K(2) SBDGB_K(3) SBDGB_K(4) SBDGB_K(5) SBDGB_K(6) SBDGB_K(7) SBDGB_K(8)
      SBDGB_K(9) SBDGB_K(10) SBDGB_K(11) SBDGB_K(12) SBDGB_K(13) SBDGB_K(14) SBDGB_K(15) SBDGB_K(16)
#undef SBDGB_K
      default: throw Error(SBDGB_E_UNSUPPORTED, "at most 16 roots");
    }
    const int width = U ? 3 * k : k;
    k_sum_partials<<<1, 64, 0, s>>>(partial, blocks, width, red);
    count_launch(p.ctx, 2);
    SBDGB_CUDA(cudaGetLastError());
    const int nrr = rr_host ? nv + nv * nv : 0;
    if (nrr) SBDGB_CUDA(cudaMemcpyAsync(host + width, rr, sizeof(double) * nrr, cudaMemcpyDeviceToHost, s));
    const double *h = read_back(width);
    if (rr_host) rr_host->assign(h + width, h + width + nrr);
    std::vector<double> v(h, h + width);
    std::vector<double> rn(v.begin(), v.begin() + k);
    for (auto &x : rn) x = std::sqrt(std::max(0.0, x));
    if (U) olsen<F>(T, U, k, std::vector<double>(v.begin() + k, v.begin() + 2 * k),
                    std::vector<double>(v.begin() + 2 * k, v.end()));
    return rn;
  }

  // T_r -= (x.T_r / x.U_r) U_r for every root whose ratio is finite.
  template <typename T>
  void olsen(T *Tv, const T *U, int k, const std::vector<double> &xt, const std::vector<double> &xu) {
    Vals<kMaxBlock> e{};
    bool any = false;
    for (int r = 0; r < k && r < kMaxBlock; ++r) {
      const double q = xt[r] / xu[r];
      if (std::isfinite(q) && xu[r] != 0.0) {
        e.v[r] = q;
        any = true;
      }
    }
    if (!any) return;
    k_olsen<T><<<blocks, kRed, 0, s>>>(Tv, U, e, k, N);
    count_launch(p.ctx);
    SBDGB_CUDA(cudaGetLastError());
  }

  template <typename T>
  void project_out(const T *V, int nv, const std::vector<double> &G, T *Tv, int k) {
    if (nv == 0) return;
    for (int j0 = 0; j0 < nv; j0 += kMaxCoef / std::max(k, 1)) {
      const int mv = std::min(nv - j0, kMaxCoef / std::max(k, 1));
      Vals<kMaxCoef> g;
      for (int r = 0; r < k; ++r)
        for (int j = 0; j < mv; ++j) g.v[j + (size_t)mv * r] = G[(j0 + j) + (size_t)nv * r];
      const T *Vj = V + (size_t)j0 * N;
      switch (k) {
#define SBDGB_K(KK) \
  case KK: k_project_out<T, KK><<<blocks, kRed, 0, s>>>(Vj, mv, N, g, Tv); break;
        SBDGB_K(1) SBDGB_K(2) SBDGB_K(3) SBDGB_K(4) SBDGB_K(5) SBDGB_K(6) SBDGB_K(7) SBDGB_K(8)
#undef SBDGB_K
        default: throw Error(SBDGB_E_UNSUPPORTED, "at most 8 vectors per projection");
      }
      count_launch(p.ctx);
      SBDGB_CUDA(cudaGetLastError());
    }
  }

  template <typename T>
  void lincomb(const T *X, int nx, const std::vector<double> &M, int ny, T *Y) {
    SBDGB_REQUIRE(nx <= kMaxBlock && ny <= kMaxBlock, SBDGB_E_UNSUPPORTED, "block too large");
    Vals<kMaxBlock * kMaxBlock> m;
    std::copy(M.begin(), M.begin() + (size_t)nx * ny, m.v);
    k_lincomb<T><<<blocks, kRed, 0, s>>>(X, nx, N, m, ny, Y);
    count_launch(p.ctx);
    SBDGB_CUDA(cudaGetLastError());
  }

  double reduce_partials(int width, std::vector<double> *out = nullptr) {
    k_sum_partials<<<1, 64, 0, s>>>(partial, blocks, width, red);
    count_launch(p.ctx);
    const double *h = read_back(width);
    if (out) out->assign(h, h + width);
    return h[0];
  }

  // Orthonormalises the nt vectors Tb against the first nv columns of V and
  // among themselves, writing the kept directions to Vout (which may follow V).
  // Classical Gram-Schmidt for the block with a second pass when a squared norm
  // falls below half of its value before the pass; the block itself is
  // orthonormalised through its Gram matrix (Cholesky with dropping of
  // directions whose remaining norm is below `drop` of the original).
  template <typename T>
  int orthonormalize_block(T *Tb, int nt, const T *V, int nv, T *Vout, double drop) {
    if (nt <= 0) return 0;
    SBDGB_REQUIRE(nt <= kMaxBlock, SBDGB_E_UNSUPPORTED, "block too large");
    std::vector<double> G0;
    dots_c<T, T>(Tb, nt, Tb, nt, G0);
    std::vector<double> n0(nt);
    for (int q = 0; q < nt; ++q) n0[q] = G0[q + (size_t)nt * q];
    std::vector<double> Gm = G0, prev = n0;
    for (int pass = 0; pass < 2 && nv > 0; ++pass) {
      std::vector<double> G;
      dots_c<T, T>(V, nv, Tb, nt, G);
      project_out<T>(V, nv, G, Tb, nt);
      dots_c<T, T>(Tb, nt, Tb, nt, Gm);
      bool again = false;
      for (int q = 0; q < nt; ++q) again = again || (Gm[q + (size_t)nt * q] < 0.5 * prev[q]);
      for (int q = 0; q < nt; ++q) prev[q] = Gm[q + (size_t)nt * q];
      if (!again) break;
    }
    // orthonormal combinations u_q of the block (u^T Gm u = 1), dropping
    // directions that are numerically dependent
    std::vector<std::vector<double>> us;
    for (int q = 0; q < nt; ++q) {
      if (!(n0[q] > 0.0) || !std::isfinite(n0[q])) continue;
      std::vector<double> v(nt, 0.0);
      v[q] = 1.0;
      for (int pass = 0; pass < 2; ++pass)
        for (const auto &u : us) {
          double pr = 0.0;
          for (int i = 0; i < nt; ++i)
            for (int j = 0; j < nt; ++j) pr += u[i] * Gm[i + (size_t)nt * j] * v[j];
          for (int i = 0; i < nt; ++i) v[i] -= pr * u[i];
        }
      double nn = 0.0;
      for (int i = 0; i < nt; ++i)
        for (int j = 0; j < nt; ++j) nn += v[i] * Gm[i + (size_t)nt * j] * v[j];
      if (!(nn > drop * drop * n0[q])) continue;
      const double f = 1.0 / std::sqrt(nn);
      for (auto &x : v) x *= f;
      us.push_back(v);
    }
    const int kept = (int)us.size();
    if (kept == 0) return 0;
    std::vector<double> M((size_t)nt * kept);
    for (int c = 0; c < kept; ++c)
      for (int i = 0; i < nt; ++i) M[i + (size_t)nt * c] = us[c][i];
    lincomb<T>(Tb, nt, M, kept, Vout);
    return kept;
  }

  std::vector<size_t> lowest_diagonal(int k) {
    std::vector<size_t> out;
    unsigned long long *skip = (unsigned long long *)(red + 1024);
    double *bval = partial;
    unsigned long long *bidx = (unsigned long long *)(partial + blocks);
    std::vector<double> hv(blocks);
    std::vector<unsigned long long> hi(blocks);
    std::vector<unsigned long long> chosen;
    for (int r = 0; r < k && (size_t)r < N; ++r) {
      if (!chosen.empty())
        SBDGB_CUDA(cudaMemcpyAsync(skip, chosen.data(), sizeof(unsigned long long) * chosen.size(),
                                   cudaMemcpyHostToDevice, s));
      k_argmin<<<blocks, 256, 0, s>>>(p.hii, N, skip, (int)chosen.size(), bval, bidx);
      count_launch(p.ctx);
      SBDGB_CUDA(cudaMemcpyAsync(hv.data(), bval, sizeof(double) * blocks, cudaMemcpyDeviceToHost, s));
      SBDGB_CUDA(cudaMemcpyAsync(hi.data(), bidx, sizeof(unsigned long long) * blocks, cudaMemcpyDeviceToHost, s));
      SBDGB_CUDA(cudaStreamSynchronize(s));
      double best = INFINITY;
      unsigned long long bi = ~0ull;
      for (int b = 0; b < blocks; ++b)
        if (hi[b] != ~0ull && (hv[b] < best || (hv[b] == best && hi[b] < bi))) {
          best = hv[b];
          bi = hi[b];
        }
      chosen.push_back(bi);
      out.push_back((size_t)bi);
    }
    return out;
  }

  // Starting vectors (BasisInitVector, davidson.h:144-184) into T (k x N).
  void start_vectors(const sbdgb_davidson_opts &o, int k, double *T, const double *Xin) {
    if (o.init == 2) {
      SBDGB_REQUIRE(Xin != nullptr, SBDGB_E_INPUT, "init 2 needs starting vectors in X");
      SBDGB_CUDA(cudaMemcpyAsync(T, Xin, sizeof(double) * N * k, cudaMemcpyHostToDevice, s));
      apply_eta<double>(p, T, k, s);  // the solvers work in the block ordering
      return;
    }
    std::vector<size_t> pos;
    if (o.init == 0) {
      pos.push_back(0);
      if (k > 1) {
        auto low = lowest_diagonal(k + 1);
        for (size_t q : low)
          if (q != 0 && (int)pos.size() < k) pos.push_back(q);
      }
    } else {
      pos = lowest_diagonal(k);
    }
    // init 0 is the reference's exact unit vector; init 1 gets a 1e-3 total
    // perturbation spread over all entries
    const double amp = o.init == 1 ? 1e-3 * std::sqrt(3.0 / (double)N) : 0.0;
    for (int q = 0; q < k; ++q) {
      k_fill_unit<<<blocks, kRed, 0, s>>>(T + (size_t)q * N, N, pos[q], amp, 0x5BD1E995ull * (uint64_t)(q + 1));
      count_launch(p.ctx);
    }
  }
};

void print_iter(const char *tag, int iter, const std::vector<double> &resid, const std::vector<double> &th, int kk) {
  printf(" Davidson%s iteration %d (tol=%.6g):", tag, iter, *std::max_element(resid.begin(), resid.end()));
  for (int q = 0; q < std::min(kk, 4); ++q) printf(" %.12f", th[q]);
  printf("\n");
  fflush(stdout);
}

// ---- FP64 solver and the two-phase mixed form ----------------------------------------

// y = (D)x for n elements (precision conversion of a vector block).
template <typename S, typename D>
__global__ void __launch_bounds__(kRed) k_convert(const S *__restrict__ x, D *__restrict__ y, size_t n) {
  for (size_t e = blockIdx.x * (size_t)kRed + threadIdx.x; e < n; e += (size_t)gridDim.x * kRed) y[e] = (D)x[e];
}

// What a run of the Davidson core does besides the options: its convergence
// test (every residual below max(eps, eps_rel |theta|)), an iteration cap,
// start vectors given on the device (FP64, replacing the options' init), and
// the lowest Ritz vectors written out in FP64 at the end.
struct CorePhase {
  double eps_rel = 0.0;
  int step_cap = 0;               // 0: max_it * max_nb
  double *seed = nullptr;         // nseed FP64 start vectors (overwritten)
  int nseed = 0;
  double *seed_out = nullptr;     // the lowest min(nseed_out, available) Ritz vectors
  int nseed_out = 0;
  int *nseed_written = nullptr;
  int max_nb_cap = 0;             // > 0: subspace at most this large (the final FP64 check)
};

// The Davidson iteration in storage precision F: FP64 (the plain solver),
// FP32 (the first phase of the mixed form: FP32 vectors, the FP32 sigma of the
// mixed kernels, FP32 vector algebra with FP64 block sums) or double-float (its
// second phase: double-float vectors, sigma and vector algebra on the FP32
// pipe).  The projected matrix and Rayleigh-Ritz stay FP64 in every form.
template <typename F>
void davidson_core(Problem &p, const sbdgb_davidson_opts &o, const CorePhase &ph, double *E, double *Xout,
                   sbdgb_report &r) {
  using clock = std::chrono::steady_clock;
  constexpr bool kF64 = std::is_same<F, double>::value;
  constexpr bool kDF = std::is_same<F, dfloat>::value;
  auto slot = [](int f64, int f32, int df) { return kF64 ? f64 : kDF ? df : f32; };
  const auto t0 = clock::now();
  const int k = o.nroots;
  const size_t N = p.N;
  SBDGB_REQUIRE(k <= kMaxBlock, SBDGB_E_UNSUPPORTED, "at most 8 roots");
  int max_nb = std::max(o.max_nb, 2 * k);
  if (ph.max_nb_cap > 0) max_nb = std::min(max_nb, std::max(ph.max_nb_cap, 2 * k));
  max_nb = (int)std::min<size_t>((size_t)max_nb, N);
  SBDGB_REQUIRE(max_nb <= 64, SBDGB_E_INPUT, "max_nb must be <= 64");
  cudaStream_t s = p.ctx->stream;
  Solver sv(p, s);
  const int nstart = ph.seed ? ph.nseed : k;
  F *V = (F *)workspace(p, slot(WS_V, WS_VF, WS_VD), sizeof(F) * N * max_nb);
  F *HV = (F *)workspace(p, slot(WS_HV, WS_HVF, WS_HVD), sizeof(F) * N * max_nb);
  F *X = (F *)workspace(p, slot(WS_X, WS_CF, WS_XD), sizeof(F) * N * 3 * k);  // restart basis (<= 3k)
  F *HX = (F *)workspace(p, slot(WS_HX, WS_SF, WS_HXD), sizeof(F) * N * 3 * k);
  F *T = (F *)workspace(p, slot(WS_T, WS_RES64, WS_TD), sizeof(F) * N * std::max(k, nstart));
  F *U = (F *)workspace(p, slot(WS_U, WS_UF, WS_UD), sizeof(F) * N * k);
  // relative norm below which a new direction is dropped
  const double drop = kF64 ? 1e-8 : kDF ? 1e-7 : 1e-5;

  int nv = 0;
  if (ph.seed && kF64) {
    nv = sv.orthonormalize_block<double>(ph.seed, ph.nseed, (const double *)V, 0, (double *)V, drop);
  } else if (ph.seed) {
    k_convert<double, F><<<sv.blocks, kRed, 0, s>>>(ph.seed, T, N * (size_t)ph.nseed);
    count_launch(p.ctx);
    nv = sv.orthonormalize_block<F>(T, ph.nseed, V, 0, V, drop);
  } else if (kF64) {
    sv.start_vectors(o, k, (double *)T, Xout);
    nv = sv.orthonormalize_block<double>((double *)T, k, (const double *)V, 0, (double *)V, drop);
  } else {
    double *T64 = (double *)workspace(p, WS_C64, sizeof(double) * N * k);
    sv.start_vectors(o, k, T64, Xout);
    k_convert<double, F><<<sv.blocks, kRed, 0, s>>>(T64, T, N * k);
    count_launch(p.ctx);
    nv = sv.orthonormalize_block<F>(T, k, V, 0, V, drop);
  }
  SBDGB_REQUIRE(nv >= 1, SBDGB_E_INPUT, "starting vectors are zero");
  std::vector<double> Hs((size_t)max_nb * max_nb, 0.0);  // projected matrix, column-major ld max_nb
  // sigma of V[from, to) and the new columns of the projected matrix
  auto extend = [&](int from, int to) {
    if constexpr (kF64) {
      for (int j = from; j < to; ++j) {
        sigma_fp64(p, V + (size_t)j * N, HV + (size_t)j * N, 0, s, true);
        r.sigma_fp64++;
      }
    } else if constexpr (kDF) {
      for (int j = from; j < to; ++j) sigma_df(p, V + (size_t)j * N, HV + (size_t)j * N, 0, s, 0.0, true);
    } else {
      for (int j = from; j < to; j += 4)
        sigma_mixed_multi(p, V + (size_t)j * N, HV + (size_t)j * N, std::min(4, to - j), s, 0.0, true);
    }
    r.sigma_calls += to - from;
    // the new columns of the projected matrix, written on the device
    sv.dots_into_hs<F, F>(V, to, HV + (size_t)from * N, to - from, from);
  };
  extend(0, nv);

  std::vector<double> theta, Y, resid(k, 0.0), c, th;
  std::vector<double> cprev;  // previous step's Ritz coefficients in the current basis (nvprev x kk)
  int nvprev = 0, kprev = 0;
  bool converged = false, rotated = false;  // rotated: the basis changed since the last Rayleigh-Ritz
  int nv_rr = 0;  // basis size at the last Rayleigh-Ritz (its eigenvectors warm-start the next)
  int iter = 0, kk = 0;
  int max_steps = std::max(1, o.max_it) * max_nb;
  if (ph.step_cap > 0) max_steps = std::min(max_steps, ph.step_cap);
  auto tol = [&](int q) { return std::max(o.eps, ph.eps_rel * std::fabs(th[q])); };
  while (true) {
    // Rayleigh-Ritz on the device projected matrix (FP64, on the GPU), then
    // the residual norms and preconditioned corrections from its result
    // (Ritz vectors not materialised); the eigenpairs come back with the norms
    sv.rayleigh_ritz(nv, rotated ? 0 : nv_rr);
    nv_rr = nv;
    rotated = false;
    kk = std::min(k, nv);
    std::vector<double> rrh;
    resid = sv.combine<F>(V, HV, nv, kk, c, th, nullptr, nullptr, T, U, &rrh);
    theta.assign(rrh.begin(), rrh.begin() + nv);
    Y.assign(rrh.begin() + nv, rrh.end());
    c.assign((size_t)nv * kk, 0.0);
    for (int q = 0; q < kk; ++q)
      for (int i = 0; i < nv; ++i) c[i + (size_t)nv * q] = Y[i + (size_t)nv * q];
    th.assign(theta.begin(), theta.begin() + kk);
    iter++;
    r.iterations++;
    if (o.verbose) print_iter(kF64 ? "" : kDF ? " (double-float phase)" : " (FP32 phase)", iter, resid, th, kk);
    converged = kk == k;
    for (int q = 0; q < kk; ++q) converged = converged && (resid[q] < tol(q));
    const double elapsed = std::chrono::duration<double>(clock::now() - t0).count();
    if (converged || iter >= max_steps || (o.max_time > 0 && elapsed > o.max_time)) break;
    int nnew = 0;
    for (int q = 0; q < kk; ++q) nnew += (resid[q] >= tol(q));
    if (nv + nnew > max_nb) {
      // Thick restart on span{Ritz vectors, previous step's Ritz vectors}
      // (the second set keeps the search direction, as in locally optimal
      // methods).  The new basis is V Q for Q orthonormal in coefficient
      // space, so its sigma vectors are HV Q and its projected matrix
      // Q^T A Q: no sigma product and no dot product is needed.
      // Keeping 2k Ritz vectors (not only the k wanted) retains the next
      // part of the spectrum and saves 5-20% of the sigma products on
      // Hamiltonians that are not diagonally dominant.
      std::vector<std::vector<double>> cols;
      const int keep = std::max(kk, std::min(std::min(2 * k, nv), max_nb - nnew));
      for (int q = 0; q < keep; ++q) cols.emplace_back(Y.begin() + (size_t)nv * q, Y.begin() + (size_t)nv * (q + 1));
      const int nkeep = std::min(kprev, max_nb - keep - nnew);
      for (int q = 0; q < nkeep; ++q) {
        std::vector<double> v(nv, 0.0);
        for (int i = 0; i < nvprev && i < nv; ++i) v[i] = cprev[i + (size_t)nvprev * q];
        cols.push_back(v);
      }
      std::vector<double> Q;  // nv x m, orthonormal columns
      int m = 0;
      for (auto &v : cols) {
        const double n0 = std::sqrt(std::inner_product(v.begin(), v.end(), v.begin(), 0.0));
        for (int pass = 0; pass < 2; ++pass)
          for (int j = 0; j < m; ++j) {
            double pr = 0.0;
            for (int i = 0; i < nv; ++i) pr += Q[i + (size_t)nv * j] * v[i];
            for (int i = 0; i < nv; ++i) v[i] -= pr * Q[i + (size_t)nv * j];
          }
        const double nn = std::sqrt(std::inner_product(v.begin(), v.end(), v.begin(), 0.0));
        if (!(nn > 1e-8 * n0)) continue;
        for (double &x : v) x /= nn;
        Q.insert(Q.end(), v.begin(), v.end());
        ++m;
      }
      // V Q and HV Q (m <= 3k columns) in blocks of at most 16 columns
      for (int b0 = 0; b0 < m; b0 += 16) {
        const int mb = std::min(16, m - b0);
        const std::vector<double> Qb(Q.begin() + (size_t)nv * b0, Q.begin() + (size_t)nv * (b0 + mb));
        sv.combine<F>(V, HV, nv, mb, Qb, std::vector<double>(mb, 0.0), X + (size_t)b0 * N, HX + (size_t)b0 * N,
                      nullptr);
      }
      SBDGB_CUDA(cudaMemcpyAsync(V, X, sizeof(F) * N * m, cudaMemcpyDeviceToDevice, s));
      SBDGB_CUDA(cudaMemcpyAsync(HV, HX, sizeof(F) * N * m, cudaMemcpyDeviceToDevice, s));
      sv.read_hs(nv, Hs, max_nb);  // the projected matrix, for its basis change
      std::vector<double> A((size_t)nv * nv), AQ((size_t)nv * m, 0.0), Hn((size_t)m * m, 0.0), cn((size_t)m * kk, 0.0);
      for (int j = 0; j < nv; ++j)
        for (int i = 0; i < nv; ++i)
          A[i + (size_t)nv * j] = 0.5 * (Hs[i + (size_t)max_nb * j] + Hs[j + (size_t)max_nb * i]);
      for (int b = 0; b < m; ++b)
        for (int j = 0; j < nv; ++j)
          for (int i = 0; i < nv; ++i) AQ[i + (size_t)nv * b] += A[i + (size_t)nv * j] * Q[j + (size_t)nv * b];
      for (int b = 0; b < m; ++b)
        for (int a2 = 0; a2 < m; ++a2)
          for (int i = 0; i < nv; ++i) Hn[a2 + (size_t)m * b] += Q[i + (size_t)nv * a2] * AQ[i + (size_t)nv * b];
      for (int q = 0; q < kk; ++q)
        for (int a2 = 0; a2 < m; ++a2)
          for (int i = 0; i < nv; ++i) cn[a2 + (size_t)m * q] += Q[i + (size_t)nv * a2] * c[i + (size_t)nv * q];
      std::fill(Hs.begin(), Hs.end(), 0.0);
      for (int b = 0; b < m; ++b)
        for (int a2 = 0; a2 < m; ++a2) Hs[a2 + (size_t)max_nb * b] = Hn[a2 + (size_t)m * b];
      sv.write_hs(m, Hs, max_nb);
      c = cn;
      nv = m;
      rotated = true;
      r.restarts++;
      // T still holds the preconditioned residuals of these Ritz vectors
    }
    cprev = c;
    nvprev = nv;
    kprev = kk;
    // corrections of the unconverged roots, packed at the front of T
    int nt = 0;
    for (int q = 0; q < kk; ++q)
      if (resid[q] >= tol(q)) {
        if (nt != q)
          SBDGB_CUDA(cudaMemcpyAsync(T + (size_t)nt * N, T + (size_t)q * N, sizeof(F) * N, cudaMemcpyDeviceToDevice, s));
        nt++;
      }
    // the subspace never exceeds max_nb (= N when 2k > N, where the restart
    // keeps k Ritz vectors and only N - k directions are left)
    nt = std::min(nt, max_nb - nv);
    const int added = nt > 0 ? sv.orthonormalize_block<F>(T, nt, V, nv, V + (size_t)nv * N, drop) : 0;
    if (added == 0) break;  // no new direction: the subspace is invariant
    extend(nv, nv + added);
    nv += added;
  }
  r.converged = converged ? 1 : 0;
  for (int q = 0; q < k && q < 16; ++q) r.resid[q] = q < (int)resid.size() ? resid[q] : 0.0;
  for (int q = 0; q < k; ++q) E[q] = q < (int)theta.size() ? theta[q] : NAN;
  if (Xout && kF64) {
    sv.combine<F>(V, HV, nv, kk, c, th, X, nullptr, nullptr);
    apply_eta<F>(p, X, kk, s);  // back to the interleaved convention
    SBDGB_CUDA(cudaMemcpyAsync(Xout, X, sizeof(double) * N * kk, cudaMemcpyDeviceToHost, s));
  }
  if (ph.seed_out) {
    // the lowest Ritz vectors of the last Rayleigh-Ritz (only the kk of c if
    // the basis was rotated after it), in FP64
    std::vector<double> cs;
    int ns;
    if (!rotated) {
      ns = std::min(std::min(ph.nseed_out, nv), 3 * k);
      cs.assign(Y.begin(), Y.begin() + (size_t)nv * ns);
    } else {
      ns = std::min(kk, ph.nseed_out);
      cs.assign(c.begin(), c.begin() + (size_t)nv * ns);
    }
    sv.combine<F>(V, HV, nv, ns, cs, std::vector<double>(ns, 0.0), X, nullptr, nullptr);
    k_convert<F, double><<<sv.blocks, kRed, 0, s>>>(X, ph.seed_out, N * (size_t)ns);
    count_launch(p.ctx);
    SBDGB_CUDA(cudaGetLastError());
    if (ph.nseed_written) *ph.nseed_written = ns;
  }
  SBDGB_CUDA(cudaStreamSynchronize(s));
  r.seconds += std::chrono::duration<double>(clock::now() - t0).count();
}

void davidson_fp64(Problem &p, const sbdgb_davidson_opts &o, double *E, double *Xout, sbdgb_report *rep) {
  sbdgb_report r{};
  davidson_core<double>(p, o, CorePhase{}, E, Xout, r);
  if (rep) *rep = r;
}

// Mixed form (precision MIXED with refine_every 0), in three phases:
//  1. FP32: the Davidson iteration on FP32 vectors with the FP32 sigma until
//     every residual is below 5e-7 |theta| (at most 4 max_nb iterations);
//  2. double-float: the same iteration on double-float vectors (48-bit
//     values, sigma and vector algebra on the FP32 pipe) from the lowest 2k
//     Ritz vectors of phase 1 (at most 8) to the full tolerance;
//  3. FP64: the lowest k Ritz vectors of phase 2 as the start of the FP64
//     iteration, whose first step recomputes their FP64 sigma, Rayleigh-Ritz
//     and residuals and stops there when those meet the tolerance (it goes on
//     in FP64, in a subspace of at most 4k, when they do not).
// FP64 runs at 1/64 of the FP32 rate on this GPU: phases 1 and 2 take the
// iterations, and the energies, vectors and residuals reported are FP64.
void davidson_two_phase(Problem &p, const sbdgb_davidson_opts &o, double *E, double *Xout, sbdgb_report *rep) {
  const int k = o.nroots;
  const size_t N = p.N;
  cudaStream_t s = p.ctx->stream;
  prepare_mixed(p, s);
  prepare_df(p, s);
  const int max_nb = (int)std::min<size_t>((size_t)std::max(o.max_nb, 2 * k), N);
  const int nseed = std::max(k, std::min(std::min(2 * k, kMaxBlock), max_nb));
  double *seeds = (double *)workspace(p, WS_C64, sizeof(double) * N * std::max(nseed, k));
  int written = 0;
  CorePhase p32;
  p32.eps_rel = 5e-7;
  p32.step_cap = 4 * max_nb;
  p32.seed_out = seeds;
  p32.nseed_out = nseed;
  p32.nseed_written = &written;
  sbdgb_report r32{};
  std::vector<double> E32(k);
  davidson_core<float>(p, o, p32, E32.data(), Xout, r32);  // Xout: start vectors of init 2 (not written)
  CorePhase pdf;
  pdf.seed = seeds;
  pdf.nseed = written;
  pdf.eps_rel = 2e-14;  // the double-float rounding floor: FP64 finishes below it
  pdf.seed_out = seeds;
  pdf.nseed_out = k;
  pdf.nseed_written = &written;
  sbdgb_report rdf{};
  std::vector<double> Edf(k);
  davidson_core<dfloat>(p, o, pdf, Edf.data(), nullptr, rdf);
  release_workspace(p, WS_VD);
  release_workspace(p, WS_HVD);
  CorePhase p64;
  p64.seed = seeds;
  p64.nseed = written;
  p64.max_nb_cap = 4 * k;
  sbdgb_report r{};
  davidson_core<double>(p, o, p64, E, Xout, r);
  r.iterations += r32.iterations + rdf.iterations;
  r.sigma_calls += r32.sigma_calls + rdf.sigma_calls;
  r.restarts += r32.restarts + rdf.restarts;
  r.seconds += r32.seconds + rdf.seconds;
  if (rep) *rep = r;
}

// ---- mixed solver ------------------------------------------------------------------

void davidson_mixed(Problem &p, const sbdgb_davidson_opts &o, double *E, double *Xout, sbdgb_report *rep) {
  using clock = std::chrono::steady_clock;
  const auto t0 = clock::now();
  const int k = o.nroots;
  const size_t N = p.N;
  SBDGB_REQUIRE(k <= kMaxBlock, SBDGB_E_UNSUPPORTED, "the mixed solver supports up to 8 roots");
  const int mmax = std::max(std::min(o.max_nb, 64) - k, 2 * k);  // FP32 correction vectors
  SBDGB_REQUIRE(k + mmax <= 64, SBDGB_E_INPUT, "max_nb must be <= 64");
  const int refine_every = std::max(1, o.refine_every);
  cudaStream_t s = p.ctx->stream;
  prepare_mixed(p, s);
  Solver sv(p, s);
  double *X = (double *)workspace(p, WS_X, sizeof(double) * N * k);    // FP64 anchors
  double *S = (double *)workspace(p, WS_HX, sizeof(double) * N * k);   // their FP64 sigma
  double *T = (double *)workspace(p, WS_T, sizeof(double) * N * k);    // FP64 scratch
  double *Y = (double *)workspace(p, WS_C64, sizeof(double) * N * k);  // FP64 scratch
  // [Xf | W]: rounded anchors followed by the FP32 subspace, so that new
  // directions are orthogonalised against both in one pass
  float *XW = (float *)workspace(p, WS_VF, sizeof(float) * N * (k + mmax));
  float *Xf = XW, *W = XW + (size_t)k * N;
  float *HW = (float *)workspace(p, WS_HVF, sizeof(float) * N * mmax);
  float *Rf = (float *)workspace(p, WS_SF, sizeof(float) * N * k);
  float *Tf = (float *)workspace(p, WS_CF, sizeof(float) * N * k);
  float *Uf = (float *)workspace(p, WS_UF, sizeof(float) * N * k);

  sbdgb_report r{};
  // anchors: starting vectors orthonormalised in FP64
  sv.start_vectors(o, k, T, Xout);
  SBDGB_REQUIRE(sv.orthonormalize_block<double>(T, k, X, 0, X, 1e-8) == k, SBDGB_E_INPUT,
                "starting vectors are linearly dependent");
  std::vector<double> theta(k), resid(k, 0.0);
  // FP64 sigma of the anchors, Rayleigh-Ritz among them, FP64 residual norms
  auto refine_rr = [&]() {
    for (int j = 0; j < k; ++j) {
      sigma_fp64(p, X + (size_t)j * N, S + (size_t)j * N, 0, s, true);
      r.sigma_calls++;
      r.sigma_fp64++;
    }
    std::vector<double> G, th, Yv;
    sv.dots_c<double, double>(X, k, S, k, G);
    for (int j = 0; j < k; ++j)
      for (int i = 0; i < j; ++i)
        G[i + (size_t)k * j] = G[j + (size_t)k * i] = 0.5 * (G[i + (size_t)k * j] + G[j + (size_t)k * i]);
    jacobi_eig(k, G, th, Yv);
    resid = sv.combine<double>(X, S, k, k, Yv, th, T, Y, nullptr);
    SBDGB_CUDA(cudaMemcpyAsync(X, T, sizeof(double) * N * k, cudaMemcpyDeviceToDevice, s));
    SBDGB_CUDA(cudaMemcpyAsync(S, Y, sizeof(double) * N * k, cudaMemcpyDeviceToDevice, s));
    theta = th;
  };
  refine_rr();
  // FP32 sigma products are taken of H - shift with the first Ritz value as
  // the shift: H W is then of the size of the spread of the spectrum rather
  // than of the energy, and HW - theta W loses no FP32 digits to cancellation
  const double shift = theta[0];

  // projected quantities of the basis [anchors, W]
  std::vector<double> Sxw((size_t)k * mmax), Hxw((size_t)k * mmax), Sww((size_t)mmax * mmax),
      Hww((size_t)mmax * mmax);
  std::vector<double> cX((size_t)k * k, 0.0), cW, thc(k);  // current Ritz vectors: cX[j + k*q], cW[l + m*q]
  int m = 0, seed = 0;
  // Rayleigh-Ritz on span{anchors, W}: generalised problem with the exact overlaps
  auto rayleigh_ritz = [&]() -> bool {
    const int n = k + m;
    std::vector<double> A((size_t)n * n, 0.0), B((size_t)n * n, 0.0), w, V;
    for (int j = 0; j < k; ++j) {
      A[j + (size_t)n * j] = theta[j];
      B[j + (size_t)n * j] = 1.0;
    }
    for (int l = 0; l < m; ++l)
      for (int j = 0; j < k; ++j) {
        A[j + (size_t)n * (k + l)] = A[(k + l) + (size_t)n * j] = Hxw[j + (size_t)k * l];
        B[j + (size_t)n * (k + l)] = B[(k + l) + (size_t)n * j] = Sxw[j + (size_t)k * l];
      }
    for (int l = 0; l < m; ++l)
      for (int l2 = 0; l2 < m; ++l2) {
        A[(k + l) + (size_t)n * (k + l2)] = Hww[l + (size_t)mmax * l2];
        B[(k + l) + (size_t)n * (k + l2)] = Sww[l + (size_t)mmax * l2];
      }
    if (!gen_sym_eig(n, A, B, w, V)) return false;
    cW.assign((size_t)m * k, 0.0);
    for (int q = 0; q < k; ++q) {
      thc[q] = w[q];
      for (int j = 0; j < k; ++j) cX[j + (size_t)k * q] = V[j + (size_t)n * q];
      for (int l = 0; l < m; ++l) cW[l + (size_t)m * q] = V[(k + l) + (size_t)n * q];
    }
    return true;
  };
  // couplings of the anchors to W columns [from, to)
  auto couple = [&](int from, int to) {
    if (to <= from) return;
    std::vector<double> g1, g2;
    sv.dots_c<double, float>(X, k, W + (size_t)from * N, to - from, g1);  // X^T w, FP64
    sv.dots_c<float, float>(Rf, k, W + (size_t)from * N, to - from, g2);  // R^T w, FP32 products
    for (int l = from; l < to; ++l)
      for (int j = 0; j < k; ++j) {
        const double x = g1[j + (size_t)k * (l - from)];
        Sxw[j + (size_t)k * l] = x;
        Hxw[j + (size_t)k * l] = g2[j + (size_t)k * (l - from)] + theta[j] * x;  // S_j = R_j + theta_j X_j
      }
  };

  bool converged = false;
  int iter = 0;
  const int max_steps = std::max(1, o.max_it) * std::max(o.max_nb, 2 * k);
  while (true) {
    converged = true;
    for (int q = 0; q < k; ++q) converged = converged && (resid[q] < o.eps);
    if (o.verbose) print_iter(" (mixed, FP64 residual)", iter, resid, theta, k);
    double elapsed = std::chrono::duration<double>(clock::now() - t0).count();
    if (converged || iter >= max_steps || (o.max_time > 0 && elapsed > o.max_time)) break;
    // rounded anchors and residuals for the FP32 inner steps
    {
      Vals<kMaxBlock> th{};
      for (int j = 0; j < k; ++j) th.v[j] = theta[j];
      k_make_anchor_f32<<<sv.blocks, kRed, 0, s>>>(X, S, th, k, N, Xf, Rf);
    }
    count_launch(p.ctx);
    if (seed > 0) {
      // the FP32 subspace was dropped: restart it with the anchors' last step
      // (locally optimal restart), orthonormalised against the new anchors
      const int added = sv.orthonormalize_block<float>(Tf, seed, XW, k, W, 1e-3);
      for (int j = 0; j < added; j += 4) {
        const int nv = std::min(4, added - j);
        sigma_mixed_multi(p, W + (size_t)j * N, HW + (size_t)j * N, nv, s, shift, true);
        r.sigma_calls += nv;
      }
      if (added > 0) {
        std::vector<double> g3, g4;
        sv.dots_c<float, float>(W, added, W, added, g3);
        sv.dots_c<float, float>(W, added, HW, added, g4);
        for (int c2 = 0; c2 < added; ++c2)
          for (int l = 0; l < added; ++l) {
            Sww[l + (size_t)mmax * c2] = g3[l + (size_t)added * c2];
            Hww[l + (size_t)mmax * c2] = 0.5 * (g4[l + (size_t)added * c2] + g4[c2 + (size_t)added * l]) +
                                         shift * g3[l + (size_t)added * c2];
          }
      }
      m = added;
      seed = 0;
    }
    couple(0, m);
    bool stalled = false;
    if (m > 0) {
      stalled = !rayleigh_ritz();
    } else {
      std::fill(cX.begin(), cX.end(), 0.0);
      for (int q = 0; q < k; ++q) cX[q + (size_t)k * q] = 1.0;
      cW.clear();
      thc = theta;
    }
    std::vector<double> res_est = resid;
    for (int inner = 0; inner < refine_every && !stalled; ++inner) {
      std::vector<int> roots;
      for (int q = 0; q < k; ++q)
        if (res_est[q] >= o.eps) roots.push_back(q);
      const int nq = (int)roots.size();
      if (nq == 0 || m + nq > mmax) break;
      // preconditioned residuals of the unconverged roots, FP32, one pass
      MixedResArgs ma{Xf, Rf, W, HW, k, m, nq, N, p.hii, Tf, Uf, sv.partial, {}, {}};
      for (int i = 0; i < nq; ++i) {
        const int q = roots[i];
        for (int j = 0; j < k; ++j) {
          ma.coef.v[(size_t)i * 192 + j] = (float)cX[j + (size_t)k * q];
          ma.coef.v[(size_t)i * 192 + 64 + j] = (float)(theta[j] - thc[q]);
        }
        for (int l = 0; l < m; ++l) ma.coef.v[(size_t)i * 192 + 128 + l] = (float)cW[l + (size_t)m * q];
        ma.thw.v[i] = (float)(thc[q] - shift);
        ma.theta.v[i] = thc[q];
      }
      switch (nq) {
#define SBDGB_K(KK) \
  case KK: k_mixed_residual<KK><<<sv.blocks, kRed, 0, s>>>(ma); break;
        SBDGB_K(1) SBDGB_K(2) SBDGB_K(3) SBDGB_K(4) SBDGB_K(5) SBDGB_K(6) SBDGB_K(7) SBDGB_K(8)
#undef SBDGB_K
        default: throw Error(SBDGB_E_UNSUPPORTED, "block too large");
      }
      count_launch(p.ctx);
      SBDGB_CUDA(cudaGetLastError());
      std::vector<double> rn;
      sv.reduce_partials(3 * nq, &rn);
      for (int i = 0; i < nq; ++i) res_est[roots[i]] = std::sqrt(std::max(0.0, rn[i]));
      sv.olsen<float>(Tf, Uf, nq, std::vector<double>(rn.begin() + nq, rn.begin() + 2 * nq),
                      std::vector<double>(rn.begin() + 2 * nq, rn.end()));
      // orthonormalise the block against [Xf, W] and itself, into W[m..]
      const int added = sv.orthonormalize_block<float>(Tf, nq, XW, k + m, W + (size_t)m * N, 1e-3);
      if (added == 0) {
        stalled = true;
        break;
      }
      for (int j = m; j < m + added; j += 4) {
        const int nv = std::min(4, m + added - j);
        sigma_mixed_multi(p, W + (size_t)j * N, HW + (size_t)j * N, nv, s, shift, true);
        r.sigma_calls += nv;
      }
      // projected quantities of the new columns
      couple(m, m + added);
      std::vector<double> g3, g4;
      sv.dots_c<float, float>(W, m + added, W + (size_t)m * N, added, g3);   // W^T w
      sv.dots_c<float, float>(W, m + added, HW + (size_t)m * N, added, g4);  // W^T Hw
      for (int jj = 0; jj < added; ++jj)
        for (int l = 0; l < m + added; ++l) {
          const int c2 = m + jj;
          const double sw = g3[l + (size_t)(m + added) * jj];
          const double hw = g4[l + (size_t)(m + added) * jj] + shift * sw;  // W^T H W from W^T (H - shift) W
          Sww[l + (size_t)mmax * c2] = Sww[c2 + (size_t)mmax * l] = sw;
          if (l < c2 || l == c2) {
            Hww[l + (size_t)mmax * c2] = Hww[c2 + (size_t)mmax * l] = hw;
          }
        }
      m += added;
      if (!rayleigh_ritz()) {
        stalled = true;
        break;
      }
      iter++;
      r.iterations = iter;
      if (iter >= max_steps) break;
    }
    // refinement: assemble the Ritz vectors in FP64, orthonormalise, FP64 sigma
    for (int q = 0; q < k; ++q) {
      Vals<64> cx{};
      FVals<64> cw{};
      for (int j = 0; j < k; ++j) cx.v[j] = cX[j + (size_t)k * q];
      for (int l = 0; l < m; ++l) cw.v[l] = (float)cW[l + (size_t)m * q];
      k_mixed_assemble<<<sv.blocks, kRed, 0, s>>>(X, k, W, m, N, cx, cw, T + (size_t)q * N);
      count_launch(p.ctx);
    }
    SBDGB_REQUIRE(sv.orthonormalize_block<double>(T, k, X, 0, X, 1e-8) == k, SBDGB_E_STATE,
                  "mixed Davidson lost a root");
    r.restarts++;
    refine_rr();
    bool full = m + k > mmax;
    if (full) {
      // subspace full: the anchors carry its information on, together with
      // their step over this refinement (Xf still holds the previous anchors)
      k_anchor_step_f32<<<sv.blocks, kRed, 0, s>>>(X, Xf, k, N, Tf);
      count_launch(p.ctx);
      seed = k;
      m = 0;
    }
    if (stalled) {
      bool ok = true;
      for (int q = 0; q < k; ++q) ok = ok && resid[q] < o.eps;
      if (!ok) {
        if (m == 0 && !full) {
          if (o.verbose) printf(" mixed Davidson: no new FP32 direction\n");
          break;
        }
        m = 0;  // start a fresh FP32 subspace from the refined anchors
      }
    }
  }
  converged = true;
  for (int q = 0; q < k; ++q) converged = converged && (resid[q] < o.eps);
  r.converged = converged ? 1 : 0;
  r.iterations = std::max(r.iterations, iter);
  for (int q = 0; q < k && q < 16; ++q) r.resid[q] = resid[q];
  for (int q = 0; q < k; ++q) E[q] = theta[q];
  if (Xout) {
    apply_eta<double>(p, X, k, s);  // back to the interleaved convention
    SBDGB_CUDA(cudaMemcpyAsync(Xout, X, sizeof(double) * N * k, cudaMemcpyDeviceToHost, s));
  }
  SBDGB_CUDA(cudaStreamSynchronize(s));
  r.seconds = std::chrono::duration<double>(clock::now() - t0).count();
  if (rep) *rep = r;
}

// ---- Lanczos (chemistry/tpb/lanczos.h:169-320) --------------------------------------

// Restarted Lanczos without reorthogonalisation, as the reference runs it for
// --method 2: each cycle builds up to max_nb Krylov vectors from W with the
// three-term recurrence (sigma accumulated into HC, which holds -beta C_{j-1}),
// stops when the lowest eigenvalue of the tridiagonal matrix moves by less
// than eps or the off-diagonal falls below eps, and restarts from the Ritz
// vector W = sum_j U[j][0] C_j.
void lanczos_fp64(Problem &p, const sbdgb_davidson_opts &o, double *E, double *Xout, sbdgb_report *rep) {
  using clock = std::chrono::steady_clock;
  const auto t0 = clock::now();
  const size_t N = p.N;
  const int nb = std::max(2, std::min(o.max_nb, 64));
  cudaStream_t s = p.ctx->stream;
  Solver sv(p, s);
  double *Cv = (double *)workspace(p, WS_V, sizeof(double) * N * nb);
  double *HC = (double *)workspace(p, WS_HV, sizeof(double) * N);
  double *W = (double *)workspace(p, WS_X, sizeof(double) * N);
  sv.start_vectors(o, 1, W, Xout);
  {
    // a caller's vector (init 2) is normalised; the unit-vector guesses already are
    std::vector<double> g;
    sv.dots_c<double, double>(W, 1, W, 1, g);
    SBDGB_REQUIRE(g[0] > 0.0 && std::isfinite(g[0]), SBDGB_E_INPUT, "starting vector is zero");
    if (std::fabs(g[0] - 1.0) > 1e-14) {
      std::vector<double> m{1.0 / std::sqrt(g[0])};
      sv.lincomb<double>(W, 1, m, 1, Cv);
      SBDGB_CUDA(cudaMemcpyAsync(W, Cv, sizeof(double) * N, cudaMemcpyDeviceToDevice, s));
    }
  }
  sbdgb_report r{};
  double E0 = 0.0, change = 0.0;
  bool stop = false;
  std::vector<double> A((size_t)nb * nb), theta, Y;
  for (int it = 0; it < std::max(1, o.max_it) && !stop; ++it) {
    SBDGB_CUDA(cudaMemcpyAsync(Cv, W, sizeof(double) * N, cudaMemcpyDeviceToDevice, s));
    SBDGB_CUDA(cudaMemsetAsync(HC, 0, sizeof(double) * N, s));
    std::fill(A.begin(), A.end(), 0.0);
    int n = 0;
    double E_old = 1.0e8;
    for (int ib = 0; ib < nb; ++ib) {
      ++n;
      double *Cb = Cv + (size_t)ib * N;
      sigma_fp64(p, Cb, HC, 1, s, true);
      r.sigma_calls++;
      r.sigma_fp64++;
      r.iterations++;
      std::vector<double> g;
      sv.dots_c<double, double>(Cb, 1, HC, 1, g);
      const double alpha = g[0];
      A[ib + (size_t)nb * ib] = alpha;
      std::vector<double> T((size_t)n * n);
      for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) T[i + (size_t)n * j] = A[i + (size_t)nb * j];
      jacobi_eig(n, T, theta, Y);
      change = std::fabs(theta[0] - E_old);
      if (o.verbose) printf(" Lanczos iteration %d, step %d: (A,B)=(%.12g) %.12f\n", it, ib, alpha, theta[0]);
      if (change < o.eps) {
        stop = true;
        break;
      }
      E_old = theta[0];
      if (ib + 1 == nb) break;
      double *next = Cv + (size_t)(ib + 1) * N;
      k_lz_update<<<sv.blocks, kRed, 0, s>>>(HC, Cb, next, alpha, N, sv.partial);
      count_launch(p.ctx);
      const double beta = std::sqrt(std::max(0.0, sv.reduce_partials(1)));
      A[ib + (size_t)nb * (ib + 1)] = A[(ib + 1) + (size_t)nb * ib] = beta;
      if (std::fabs(beta) < o.eps) break;  // invariant subspace (the new vector is not used)
      k_lz_scale<<<sv.blocks, kRed, 0, s>>>(next, HC, Cb, beta, N);
      count_launch(p.ctx);
      SBDGB_CUDA(cudaGetLastError());
    }
    std::vector<double> T((size_t)n * n);
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) T[i + (size_t)n * j] = A[i + (size_t)nb * j];
    jacobi_eig(n, T, theta, Y);
    E0 = theta[0];
    Vals<64> u{};
    std::copy(Y.begin(), Y.begin() + n, u.v);
    k_lz_ritz<<<sv.blocks, kRed, 0, s>>>(Cv, n, N, u, W);
    count_launch(p.ctx);
    SBDGB_CUDA(cudaGetLastError());
    r.restarts++;
    const double elapsed = std::chrono::duration<double>(clock::now() - t0).count();
    if (o.max_time > 0 && elapsed > o.max_time) break;
  }
  r.converged = stop ? 1 : 0;
  r.resid[0] = change;
  E[0] = E0;
  if (Xout) {
    apply_eta<double>(p, W, 1, s);  // back to the interleaved convention
    SBDGB_CUDA(cudaMemcpyAsync(Xout, W, sizeof(double) * N, cudaMemcpyDeviceToHost, s));
  }
  SBDGB_CUDA(cudaStreamSynchronize(s));
  r.seconds = std::chrono::duration<double>(clock::now() - t0).count();
  if (rep) *rep = r;
}

}  // namespace

void lanczos(Problem &p, const sbdgb_davidson_opts &o, double *E, double *Xout, sbdgb_report *rep) {
  if (!p.tables || !p.diag) throw Error(SBDGB_E_STATE, "Lanczos needs tables and diagonal");
  SBDGB_REQUIRE(o.nroots == 1, SBDGB_E_UNSUPPORTED, "Lanczos solves one root");
  SBDGB_REQUIRE(o.precision == SBDGB_FP64, SBDGB_E_UNSUPPORTED, "Lanczos runs in FP64");
  lanczos_fp64(p, o, E, Xout, rep);
}

void davidson(Problem &p, const sbdgb_davidson_opts &o, double *E, double *Xout, sbdgb_report *rep) {
  if (!p.tables || !p.diag) throw Error(SBDGB_E_STATE, "Davidson needs tables and diagonal");
  SBDGB_REQUIRE(o.nroots >= 1 && o.nroots <= kMaxBlock, SBDGB_E_INPUT, "nroots must be in [1, 8]");
  SBDGB_REQUIRE((size_t)o.nroots <= p.N, SBDGB_E_INPUT, "more roots than determinants");
  if (o.precision == SBDGB_MIXED && o.refine_every == 0)
    davidson_two_phase(p, o, E, Xout, rep);
  else if (o.precision == SBDGB_MIXED)
    davidson_mixed(p, o, E, Xout, rep);
  else
    davidson_fp64(p, o, E, Xout, rep);
}

}  // namespace sbdgb
