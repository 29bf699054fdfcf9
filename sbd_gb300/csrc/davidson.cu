// Davidson eigensolvers on the device (replace sbd::Davidson,
// chemistry/tpb/davidson.h:707-970, and its GPU form chemistry/basic/
// davidson_thrust.h:97-385 / :389-675).
//
// The reference solves one root with a single-vector Davidson: subspace up to
// max_nb, Ritz pair from the projected matrix, residual R = E0 W - H W,
// diagonal preconditioner R/(E0 - d) with a 1e-12 guard, modified
// Gram-Schmidt, restart C0 = W (which recomputes sigma(W)).
//
// FP64 solver: the same steps generalised to nroots.  Each step adds one
// corrected direction per unconverged root, orthogonalises it against the
// basis with classical Gram-Schmidt plus a second pass when the norm drops
// (the "twice is enough" rule), and restarts from the nroots Ritz vectors
// together with their sigma vectors, which are formed from the stored H*V
// instead of a new sigma product.  Vectors stay resident in HBM; only the
// projected (<= max_nb)^2 matrix and a few norms cross to the host per step.
//
// Mixed solver: each root keeps an FP64 vector x (and its FP64 sigma) that is
// never rounded to FP32.  Corrections live in an FP32 subspace W with FP32
// sigma products.  Rayleigh-Ritz runs on span{x, W} as a generalised
// symmetric problem whose x-W couplings are computed in FP64 (W is only
// orthogonal to x to FP32 accuracy); every refine_every steps the Ritz vectors
// are assembled in FP64, their FP64 sigma and FP64 residual are recomputed
// (iterative refinement), and convergence is judged on that FP64 residual.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <type_traits>

#include "common.cuh"
#include "small_eig.h"

namespace sbdgb {

namespace {

constexpr int kRed = 256;  // threads per reduction block
constexpr int kMaxV = 8;   // basis columns per dots pass
constexpr int kMaxW = 4;   // right-hand columns per dots pass
constexpr int kMaxCoef = 64 * 16;

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
  using Acc = typename std::conditional<kF32, float, double>::type;
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
    for (int j = 0; j < NW; ++j) w[j] = (Acc)__ldg(W.p[j] + e);
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      const Acc v = (Acc)__ldg(V.p[i] + e);
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

struct CombineArgs {
  const double *V;
  const double *HV;
  size_t N;
  int nv;
  int k;
  const double *coef;   // nv x k column-major (coef[j + nv*r])
  const double *theta;  // k
  const double *hii;
  double *X;        // k x N or null
  double *HX;       // k x N or null
  double *T;        // k x N or null: preconditioned residual
  double *partial;  // blocks x k residual norm^2 partials
};

// X_r = V c_r, HX_r = HV c_r, R_r = HX_r - theta_r X_r, T_r = R_r / (theta_r - d)
// (davidson.h:818-843 and the preconditioner :899-908, 1e-12 guard).
template <int K>
__global__ void __launch_bounds__(kRed) k_combine(CombineArgs a) {
  __shared__ double cs[kMaxCoef];
  __shared__ double th[16];
  for (int t = threadIdx.x; t < a.nv * K; t += kRed) cs[t] = a.coef[t];
  if (threadIdx.x < K) th[threadIdx.x] = a.theta[threadIdx.x];
  __syncthreads();
  double rn[K];
#pragma unroll
  for (int r = 0; r < K; ++r) rn[r] = 0.0;
  for (size_t e = blockIdx.x * (size_t)kRed + threadIdx.x; e < a.N; e += (size_t)gridDim.x * kRed) {
    double x[K], h[K];
#pragma unroll
    for (int r = 0; r < K; ++r) {
      x[r] = 0.0;
      h[r] = 0.0;
    }
    for (int j = 0; j < a.nv; ++j) {
      const double v = __ldg(a.V + (size_t)j * a.N + e);
      const double hv = __ldg(a.HV + (size_t)j * a.N + e);
#pragma unroll
      for (int r = 0; r < K; ++r) {
        x[r] = fma(v, cs[j + a.nv * r], x[r]);
        h[r] = fma(hv, cs[j + a.nv * r], h[r]);
      }
    }
    const double d = a.hii ? __ldg(a.hii + e) : 0.0;
#pragma unroll
    for (int r = 0; r < K; ++r) {
      const double res = h[r] - th[r] * x[r];
      rn[r] = fma(res, res, rn[r]);
      if (a.X) a.X[(size_t)r * a.N + e] = x[r];
      if (a.HX) a.HX[(size_t)r * a.N + e] = h[r];
      if (a.T) {
        double den = th[r] - d;
        if (fabs(den) <= 1.0e-12) den -= 1.0e-12;
        a.T[(size_t)r * a.N + e] = res / den;
      }
    }
  }
  __shared__ double red[kRed / 32][16];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int r = 0; r < K; ++r) {
    double x = rn[r];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if (lane == 0) red[warp][r] = x;
  }
  __syncthreads();
  if (threadIdx.x < K) {
    double x = 0.0;
    for (int w2 = 0; w2 < kRed / 32; ++w2) x += red[w2][threadIdx.x];
    a.partial[(size_t)blockIdx.x * K + threadIdx.x] = x;
  }
}

// T_r -= sum_j V_j G[j][r]  (G column-major, ld = nv), in the vectors' precision.
template <typename T, int K>
__global__ void __launch_bounds__(kRed) k_project_out(const T *__restrict__ V, int nv, size_t N,
                                                       const double *__restrict__ G, T *__restrict__ Tv) {
  __shared__ T gs[kMaxCoef];
  for (int t = threadIdx.x; t < nv * K; t += kRed) gs[t] = (T)G[t];
  __syncthreads();
  for (size_t e = blockIdx.x * (size_t)kRed + threadIdx.x; e < N; e += (size_t)gridDim.x * kRed) {
    T t[K];
#pragma unroll
    for (int r = 0; r < K; ++r) t[r] = Tv[(size_t)r * N + e];
    for (int j = 0; j < nv; ++j) {
      const T v = __ldg(V + (size_t)j * N + e);
#pragma unroll
      for (int r = 0; r < K; ++r) t[r] = fma(-v, gs[j + nv * r], t[r]);
    }
#pragma unroll
    for (int r = 0; r < K; ++r) Tv[(size_t)r * N + e] = t[r];
  }
}

template <typename TI, typename TO>
__global__ void k_scale_copy(const TI *x, TO *y, size_t N, double f) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < N; e += (size_t)gridDim.x * blockDim.x)
    y[e] = (TO)((double)x[e] * f);
}

__global__ void k_fill_unit(double *__restrict__ y, size_t N, size_t pos) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < N; e += (size_t)gridDim.x * blockDim.x)
    y[e] = (e == pos) ? 1.0 : 0.0;
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
                                  const double *__restrict__ theta, int k, size_t N, float *__restrict__ Xf,
                                  float *__restrict__ Rf) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < N; e += (size_t)gridDim.x * blockDim.x)
    for (int j = 0; j < k; ++j) {
      const double x = X[(size_t)j * N + e];
      Xf[(size_t)j * N + e] = (float)x;
      Rf[(size_t)j * N + e] = (float)fma(-theta[j], x, S[(size_t)j * N + e]);
    }
}

struct MixedResArgs {
  const float *Xf, *Rf, *W, *HW;
  int k, m;
  size_t N;
  const float *cx;   // k: anchor coefficients of this Ritz vector
  const float *dth;  // k: theta_j - theta (anchor Ritz values minus current value)
  const float *cw;   // m: subspace coefficients
  float theta;
  const double *hii;
  float *T;          // out: preconditioned residual
  double *partial;   // blocks: residual norm^2
};

// r = sum_j (Rf_j + dth_j Xf_j) cx_j + sum_l (HW_l - theta W_l) cw_l, then
// T = r / (theta - d) with the reference's 1e-12 guard.  FP32 arithmetic.
__global__ void __launch_bounds__(kRed) k_mixed_residual(MixedResArgs a) {
  __shared__ float c[3 * 64];
  for (int t = threadIdx.x; t < a.k; t += kRed) {
    c[t] = a.cx[t];
    c[64 + t] = a.dth[t];
  }
  for (int t = threadIdx.x; t < a.m; t += kRed) c[128 + t] = a.cw[t];
  __syncthreads();
  float s = 0.f, comp = 0.f;
  for (size_t e = blockIdx.x * (size_t)kRed + threadIdx.x; e < a.N; e += (size_t)gridDim.x * kRed) {
    float r = 0.f;
    for (int j = 0; j < a.k; ++j)
      r = fmaf(fmaf(c[64 + j], __ldg(a.Xf + (size_t)j * a.N + e), __ldg(a.Rf + (size_t)j * a.N + e)), c[j], r);
    for (int l = 0; l < a.m; ++l)
      r = fmaf(fmaf(-a.theta, __ldg(a.W + (size_t)l * a.N + e), __ldg(a.HW + (size_t)l * a.N + e)), c[128 + l], r);
    const float y = r * r - comp;
    const float t = s + y;
    comp = (t - s) - y;
    s = t;
    double den = (double)a.theta - __ldg(a.hii + e);
    if (fabs(den) <= 1.0e-12) den -= 1.0e-12;
    a.T[e] = (float)((double)r / den);
  }
  __shared__ double red[kRed / 32];
  double x = (double)s - (double)comp;
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = x;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w2 = 0; w2 < kRed / 32; ++w2) t += red[w2];
    a.partial[blockIdx.x] = t;
  }
}

// y = sum_j X_j cx_j (FP64) + fp64(sum_l W_l cw_l) (FP32): the refined Ritz vector.
__global__ void __launch_bounds__(kRed) k_mixed_assemble(const double *__restrict__ X, int k, const float *__restrict__ W,
                                                         int m, size_t N, const double *__restrict__ cx,
                                                         const float *__restrict__ cw, double *__restrict__ y) {
  __shared__ double sx[64];
  __shared__ float sw[64];
  for (int t = threadIdx.x; t < k; t += kRed) sx[t] = cx[t];
  for (int t = threadIdx.x; t < m; t += kRed) sw[t] = cw[t];
  __syncthreads();
  for (size_t e = blockIdx.x * (size_t)kRed + threadIdx.x; e < N; e += (size_t)gridDim.x * kRed) {
    double v = 0.0;
    for (int j = 0; j < k; ++j) v = fma(__ldg(X + (size_t)j * N + e), sx[j], v);
    float w = 0.f;
    for (int l = 0; l < m; ++l) w = fmaf(__ldg(W + (size_t)l * N + e), sw[l], w);
    y[e] = v + (double)w;
  }
}

// ---- host-side helper ----------------------------------------------------------

struct Solver {
  Problem &p;
  cudaStream_t s;
  size_t N;
  int blocks;
  double *partial = nullptr;  // blocks * kMaxV*kMaxW
  double *red = nullptr;      // reduced results (device)
  double *coef = nullptr;     // device coefficient staging
  std::vector<double> hbuf;

  Solver(Problem &pp, cudaStream_t ss) : p(pp), s(ss), N(pp.N) {
    int dev = p.ctx->device, sms = 0;
    SBDGB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    size_t want = (N + kRed - 1) / kRed;
    blocks = (int)std::max<size_t>(1, std::min<size_t>(want, (size_t)sms * 4));
    partial = (double *)workspace(p, WS_PARTIAL, sizeof(double) * ((size_t)blocks * kMaxV * kMaxW + 64));
    red = (double *)workspace(p, WS_RED, sizeof(double) * 4096);
    coef = (double *)workspace(p, WS_COEF, sizeof(double) * (kMaxCoef + 64));
  }

  // G (column-major nv x nw) = V^T W, V columns at V0 + j*N.
  template <typename TV, typename TW>
  void dots(const TV *V0, int nv, const TW *const *W, int nw, std::vector<double> &G) {
    G.assign((size_t)nv * nw, 0.0);
    for (int j0 = 0; j0 < nw; j0 += kMaxW) {
      const int mw = std::min(kMaxW, nw - j0);
      Ptrs<TW, kMaxW> wp{};
      for (int j = 0; j < kMaxW; ++j) wp.p[j] = W[j0 + std::min(j, mw - 1)];
      for (int i0 = 0; i0 < nv; i0 += kMaxV) {
        const int mv = std::min(kMaxV, nv - i0);
        Ptrs<TV, kMaxV> vp{};
        for (int i = 0; i < kMaxV; ++i) vp.p[i] = V0 + (size_t)(i0 + std::min(i, mv - 1)) * N;
        launch_dots<TV, TW>(vp, wp, mv, mw);
        const int width = mv * mw;
        k_sum_partials<<<(width + 63) / 64, 64, 0, s>>>(partial, blocks, width, red);
        count_launch(p.ctx);
        hbuf.resize(width);
        SBDGB_CUDA(cudaMemcpyAsync(hbuf.data(), red, sizeof(double) * width, cudaMemcpyDeviceToHost, s));
        SBDGB_CUDA(cudaStreamSynchronize(s));
        for (int i = 0; i < mv; ++i)
          for (int j = 0; j < mw; ++j) G[(size_t)(i0 + i) + (size_t)nv * (j0 + j)] = hbuf[i * mw + j];
      }
    }
  }

  template <typename TV, typename TW, int NV>
  void launch_dots_w(Ptrs<TV, kMaxV> vp, Ptrs<TW, kMaxW> wp, int mw) {
    switch (mw) {
      case 1: k_dots<TV, TW, NV, 1><<<blocks, kRed, 0, s>>>(vp, wp, N, partial); break;
      case 2: k_dots<TV, TW, NV, 2><<<blocks, kRed, 0, s>>>(vp, wp, N, partial); break;
      case 3: k_dots<TV, TW, NV, 3><<<blocks, kRed, 0, s>>>(vp, wp, N, partial); break;
      default: k_dots<TV, TW, NV, 4><<<blocks, kRed, 0, s>>>(vp, wp, N, partial); break;
    }
  }
  template <typename TV, typename TW>
  void launch_dots(Ptrs<TV, kMaxV> vp, Ptrs<TW, kMaxW> wp, int mv, int mw) {
    switch (mv) {
      case 1: launch_dots_w<TV, TW, 1>(vp, wp, mw); break;
      case 2: launch_dots_w<TV, TW, 2>(vp, wp, mw); break;
      case 3: launch_dots_w<TV, TW, 3>(vp, wp, mw); break;
      case 4: launch_dots_w<TV, TW, 4>(vp, wp, mw); break;
      case 5: launch_dots_w<TV, TW, 5>(vp, wp, mw); break;
      case 6: launch_dots_w<TV, TW, 6>(vp, wp, mw); break;
      case 7: launch_dots_w<TV, TW, 7>(vp, wp, mw); break;
      default: launch_dots_w<TV, TW, 8>(vp, wp, mw); break;
    }
    count_launch(p.ctx);
    SBDGB_CUDA(cudaGetLastError());
  }

  // Returns the residual norms.
  std::vector<double> combine(const double *V, const double *HV, int nv, int k, const std::vector<double> &c,
                              const std::vector<double> &theta, double *X, double *HX, double *T) {
    std::vector<double> hc((size_t)nv * k + 16, 0.0);
    std::copy(c.begin(), c.end(), hc.begin());
    SBDGB_CUDA(cudaMemcpyAsync(coef, hc.data(), sizeof(double) * nv * k, cudaMemcpyHostToDevice, s));
    SBDGB_CUDA(cudaMemcpyAsync(red + 2048, theta.data(), sizeof(double) * k, cudaMemcpyHostToDevice, s));
    CombineArgs a{V, HV, N, nv, k, coef, red + 2048, p.hii, X, HX, T, partial};
    switch (k) {
#define SBDGB_K(KK) \
  case KK: k_combine<KK><<<blocks, kRed, 0, s>>>(a); break;
      SBDGB_K(1) SBDGB_K(2) SBDGB_K(3) SBDGB_K(4) SBDGB_K(5) SBDGB_K(6) SBDGB_K(7) SBDGB_K(8)
      SBDGB_K(9) SBDGB_K(10) SBDGB_K(11) SBDGB_K(12) SBDGB_K(13) SBDGB_K(14) SBDGB_K(15) SBDGB_K(16)
#undef SBDGB_K
      default: throw Error(SBDGB_E_UNSUPPORTED, "at most 16 roots");
    }
    k_sum_partials<<<1, 64, 0, s>>>(partial, blocks, k, red);
    count_launch(p.ctx, 2);
    SBDGB_CUDA(cudaGetLastError());
    std::vector<double> rn(k);
    SBDGB_CUDA(cudaMemcpyAsync(rn.data(), red, sizeof(double) * k, cudaMemcpyDeviceToHost, s));
    SBDGB_CUDA(cudaStreamSynchronize(s));
    for (auto &x : rn) x = std::sqrt(std::max(0.0, x));
    return rn;
  }

  template <typename T>
  void project_out(const T *V, int nv, const std::vector<double> &G, T *Tv, int k) {
    if (nv == 0) return;
    SBDGB_CUDA(cudaMemcpyAsync(coef, G.data(), sizeof(double) * nv * k, cudaMemcpyHostToDevice, s));
    switch (k) {
#define SBDGB_K(KK) \
  case KK: k_project_out<T, KK><<<blocks, kRed, 0, s>>>(V, nv, N, coef, Tv); break;
      SBDGB_K(1) SBDGB_K(2) SBDGB_K(3) SBDGB_K(4) SBDGB_K(5) SBDGB_K(6) SBDGB_K(7) SBDGB_K(8)
#undef SBDGB_K
      default: throw Error(SBDGB_E_UNSUPPORTED, "at most 8 vectors per projection");
    }
    count_launch(p.ctx);
    SBDGB_CUDA(cudaGetLastError());
  }

  template <typename TI, typename TO>
  void scale_copy(const TI *x, TO *y, double f) {
    k_scale_copy<TI, TO><<<blocks, kRed, 0, s>>>(x, y, N, f);
    count_launch(p.ctx);
  }
  template <typename T>
  double norm(const T *x) {
    std::vector<double> g;
    const T *w[1] = {x};
    dots<T, T>(x, 1, w, 1, g);
    return std::sqrt(std::max(0.0, g[0]));
  }
  double reduce_partials(int width) {
    k_sum_partials<<<1, 64, 0, s>>>(partial, blocks, width, red);
    count_launch(p.ctx);
    double out = 0.0;
    SBDGB_CUDA(cudaMemcpyAsync(&out, red, sizeof(double), cudaMemcpyDeviceToHost, s));
    SBDGB_CUDA(cudaStreamSynchronize(s));
    return out;
  }

  // Orthonormalises t against the first nv columns of V (two passes of
  // classical Gram-Schmidt when the norm drops), in the vectors' precision.
  // Returns the norm left relative to the unit-normalised input (0 if t was 0).
  template <typename T>
  double orthonormalize(T *t, const T *V, int nv) {
    double n0 = norm(t);
    if (!(n0 > 0.0) || !std::isfinite(n0)) return 0.0;
    scale_copy<T, T>(t, t, 1.0 / n0);
    n0 = 1.0;
    for (int pass = 0; pass < 2 && nv > 0; ++pass) {
      for (int j0 = 0; j0 < nv; j0 += kMaxV) {
        const int mv = std::min(kMaxV, nv - j0);
        std::vector<double> G;
        const T *w[1] = {t};
        dots<T, T>(V + (size_t)j0 * N, mv, w, 1, G);
        project_out<T>(V + (size_t)j0 * N, mv, G, t, 1);
      }
      const double n1 = norm(t);
      const bool enough = n1 > 0.7071 * n0;
      n0 = n1;
      if (enough) break;
    }
    if (n0 > 0.0) scale_copy<T, T>(t, t, 1.0 / n0);
    return n0;
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
    for (int q = 0; q < k; ++q) {
      k_fill_unit<<<blocks, kRed, 0, s>>>(T + (size_t)q * N, N, pos[q]);
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

// ---- FP64 solver ------------------------------------------------------------------

void davidson_fp64(Problem &p, const sbdgb_davidson_opts &o, double *E, double *Xout, sbdgb_report *rep) {
  using clock = std::chrono::steady_clock;
  const auto t0 = clock::now();
  const int k = o.nroots;
  const size_t N = p.N;
  int max_nb = std::max(o.max_nb, 2 * k);
  max_nb = (int)std::min<size_t>((size_t)max_nb, N);
  SBDGB_REQUIRE(max_nb <= 64, SBDGB_E_INPUT, "max_nb must be <= 64");
  cudaStream_t s = p.ctx->stream;
  Solver sv(p, s);
  double *V = (double *)workspace(p, WS_V, sizeof(double) * N * max_nb);
  double *HV = (double *)workspace(p, WS_HV, sizeof(double) * N * max_nb);
  double *X = (double *)workspace(p, WS_X, sizeof(double) * N * k);
  double *HX = (double *)workspace(p, WS_HX, sizeof(double) * N * k);
  double *T = (double *)workspace(p, WS_T, sizeof(double) * N * k);

  sbdgb_report r{};
  sv.start_vectors(o, k, T, Xout);
  int nv = 0;
  auto append = [&](double *Tin, int nt) -> int {
    int added = 0;
    for (int q = 0; q < nt && nv < max_nb; ++q) {
      double *t = Tin + (size_t)q * N;
      const double left = sv.orthonormalize<double>(t, V, nv);
      if (!(left > 1e-8)) continue;  // linearly dependent direction: dropped
      SBDGB_CUDA(cudaMemcpyAsync(V + (size_t)nv * N, t, sizeof(double) * N, cudaMemcpyDeviceToDevice, s));
      nv++;
      added++;
    }
    return added;
  };
  auto sigma_range = [&](int from) {
    for (int j = from; j < nv; ++j) {
      sigma_fp64(p, V + (size_t)j * N, HV + (size_t)j * N, 0, s);
      r.sigma_calls++;
      r.sigma_fp64++;
    }
  };
  append(T, k);
  SBDGB_REQUIRE(nv >= 1, SBDGB_E_INPUT, "starting vectors are zero");
  sigma_range(0);
  std::vector<double> Hs((size_t)max_nb * max_nb, 0.0);  // projected matrix, column-major ld max_nb
  auto update_projection = [&](int from) {
    std::vector<const double *> w;
    for (int j = from; j < nv; ++j) w.push_back(HV + (size_t)j * N);
    std::vector<double> G;
    sv.dots<double, double>(V, nv, w.data(), (int)w.size(), G);
    for (int jj = 0; jj < (int)w.size(); ++jj)
      for (int i = 0; i < nv; ++i) {
        const double g = G[(size_t)i + (size_t)nv * jj];
        Hs[(size_t)i + (size_t)max_nb * (from + jj)] = g;
        Hs[(size_t)(from + jj) + (size_t)max_nb * i] = g;
      }
  };
  update_projection(0);

  std::vector<double> theta, Y, resid(k, 0.0);
  bool converged = false;
  int iter = 0;
  const int max_steps = std::max(1, o.max_it) * max_nb;
  while (true) {
    // Rayleigh-Ritz on the projected matrix
    std::vector<double> A((size_t)nv * nv);
    for (int j = 0; j < nv; ++j)
      for (int i = 0; i < nv; ++i)
        A[i + (size_t)nv * j] = 0.5 * (Hs[i + (size_t)max_nb * j] + Hs[j + (size_t)max_nb * i]);
    jacobi_eig(nv, A, theta, Y);
    const int kk = std::min(k, nv);
    std::vector<double> c((size_t)nv * kk);
    for (int q = 0; q < kk; ++q)
      for (int i = 0; i < nv; ++i) c[i + (size_t)nv * q] = Y[i + (size_t)nv * q];
    std::vector<double> th(theta.begin(), theta.begin() + kk);
    resid = sv.combine(V, HV, nv, kk, c, th, X, HX, T);
    iter++;
    r.iterations = iter;
    if (o.verbose) print_iter("", iter, resid, th, kk);
    converged = kk == k;
    for (int q = 0; q < kk; ++q) converged = converged && (resid[q] < o.eps);
    const double elapsed = std::chrono::duration<double>(clock::now() - t0).count();
    if (converged || iter >= max_steps || (o.max_time > 0 && elapsed > o.max_time)) break;
    // restart when the new directions would not fit (thick restart with the Ritz vectors)
    int nnew = 0;
    for (int q = 0; q < kk; ++q) nnew += (resid[q] >= o.eps);
    if (nv + nnew > max_nb) {
      SBDGB_CUDA(cudaMemcpyAsync(V, X, sizeof(double) * N * kk, cudaMemcpyDeviceToDevice, s));
      SBDGB_CUDA(cudaMemcpyAsync(HV, HX, sizeof(double) * N * kk, cudaMemcpyDeviceToDevice, s));
      nv = kk;
      std::fill(Hs.begin(), Hs.end(), 0.0);
      for (int q = 0; q < kk; ++q) Hs[q + (size_t)max_nb * q] = th[q];
      r.restarts++;
      // T still holds the preconditioned residuals of these Ritz vectors
    }
    // keep the corrections of the unconverged roots, packed at the front of T
    int nt = 0;
    for (int q = 0; q < kk; ++q)
      if (resid[q] >= o.eps) {
        if (nt != q)
          SBDGB_CUDA(cudaMemcpyAsync(T + (size_t)nt * N, T + (size_t)q * N, sizeof(double) * N,
                                     cudaMemcpyDeviceToDevice, s));
        nt++;
      }
    const int from = nv;
    const int added = append(T, nt);
    if (added == 0) break;  // no new direction: the subspace is invariant
    sigma_range(from);
    update_projection(from);
  }
  r.converged = converged ? 1 : 0;
  for (int q = 0; q < k && q < 16; ++q) r.resid[q] = q < (int)resid.size() ? resid[q] : 0.0;
  for (int q = 0; q < k; ++q) E[q] = q < (int)theta.size() ? theta[q] : NAN;
  if (Xout) SBDGB_CUDA(cudaMemcpyAsync(Xout, X, sizeof(double) * N * k, cudaMemcpyDeviceToHost, s));
  SBDGB_CUDA(cudaStreamSynchronize(s));
  r.seconds = std::chrono::duration<double>(clock::now() - t0).count();
  if (rep) *rep = r;
}

// ---- mixed solver ------------------------------------------------------------------

void davidson_mixed(Problem &p, const sbdgb_davidson_opts &o, double *E, double *Xout, sbdgb_report *rep) {
  using clock = std::chrono::steady_clock;
  const auto t0 = clock::now();
  const int k = o.nroots;
  const size_t N = p.N;
  SBDGB_REQUIRE(k <= 8, SBDGB_E_UNSUPPORTED, "the mixed solver supports up to 8 roots");
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
  float *W = (float *)workspace(p, WS_VF, sizeof(float) * N * mmax);
  float *HW = (float *)workspace(p, WS_HVF, sizeof(float) * N * mmax);
  float *Xf = (float *)workspace(p, WS_CF, sizeof(float) * N * k);
  float *Rf = (float *)workspace(p, WS_SF, sizeof(float) * N * k);
  float *Tf = (float *)workspace(p, WS_RES64, sizeof(float) * N);
  float *dcoef = (float *)workspace(p, WS_DIAG1, sizeof(float) * 256);

  sbdgb_report r{};
  // anchors: starting vectors orthonormalised in FP64
  sv.start_vectors(o, k, T, Xout);
  for (int q = 0; q < k; ++q) {
    double *t = T + (size_t)q * N;
    const double left = sv.orthonormalize<double>(t, X, q);
    SBDGB_REQUIRE(left > 1e-8, SBDGB_E_INPUT, "starting vectors are linearly dependent");
    SBDGB_CUDA(cudaMemcpyAsync(X + (size_t)q * N, t, sizeof(double) * N, cudaMemcpyDeviceToDevice, s));
  }
  std::vector<double> theta(k), resid(k, 0.0);
  // FP64 sigma of the anchors, Rayleigh-Ritz among them, FP64 residual norms
  auto refine_rr = [&]() {
    for (int j = 0; j < k; ++j) {
      sigma_fp64(p, X + (size_t)j * N, S + (size_t)j * N, 0, s);
      r.sigma_calls++;
      r.sigma_fp64++;
    }
    std::vector<const double *> w;
    for (int j = 0; j < k; ++j) w.push_back(S + (size_t)j * N);
    std::vector<double> G, th, Yv;
    sv.dots<double, double>(X, k, w.data(), k, G);
    for (int j = 0; j < k; ++j)
      for (int i = 0; i < j; ++i)
        G[i + (size_t)k * j] = G[j + (size_t)k * i] = 0.5 * (G[i + (size_t)k * j] + G[j + (size_t)k * i]);
    jacobi_eig(k, G, th, Yv);
    resid = sv.combine(X, S, k, k, Yv, th, T, Y, nullptr);
    SBDGB_CUDA(cudaMemcpyAsync(X, T, sizeof(double) * N * k, cudaMemcpyDeviceToDevice, s));
    SBDGB_CUDA(cudaMemcpyAsync(S, Y, sizeof(double) * N * k, cudaMemcpyDeviceToDevice, s));
    theta = th;
  };
  refine_rr();

  // projected quantities of the basis [anchors, W]
  std::vector<double> Sxw((size_t)k * mmax), Hxw((size_t)k * mmax), Sww((size_t)mmax * mmax),
      Hww((size_t)mmax * mmax);
  std::vector<double> cX((size_t)k * k, 0.0), cW, thc(k);  // current Ritz vectors: cX[j + k*q], cW[l + m*q]
  int m = 0;
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
  // couplings of the (new) anchors to the kept W columns
  auto recouple = [&]() {
    for (int l = 0; l < m; ++l) {
      const float *wl[1] = {W + (size_t)l * N};
      std::vector<double> g1, g2;
      sv.dots<double, float>(X, k, wl, 1, g1);  // X^T w, FP64
      sv.dots<float, float>(Rf, k, wl, 1, g2);  // R^T w, FP32 products
      for (int j = 0; j < k; ++j) {
        Sxw[j + (size_t)k * l] = g1[j];
        Hxw[j + (size_t)k * l] = g2[j] + theta[j] * g1[j];  // S_j = R_j + theta_j X_j
      }
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
    SBDGB_CUDA(cudaMemcpyAsync(sv.red + 2048, theta.data(), sizeof(double) * k, cudaMemcpyHostToDevice, s));
    k_make_anchor_f32<<<sv.blocks, kRed, 0, s>>>(X, S, sv.red + 2048, k, N, Xf, Rf);
    count_launch(p.ctx);
    recouple();
    bool ok_rr = true;
    if (m > 0) {
      ok_rr = rayleigh_ritz();
    } else {
      std::fill(cX.begin(), cX.end(), 0.0);
      for (int q = 0; q < k; ++q) cX[q + (size_t)k * q] = 1.0;
      cW.clear();
      thc = theta;
    }
    std::vector<double> res_est = resid;
    bool stalled = !ok_rr;
    for (int inner = 0; inner < refine_every && !stalled; ++inner) {
      if (m + k > mmax) break;
      const int m0 = m;
      for (int q = 0; q < k && m < mmax; ++q) {
        if (res_est[q] < o.eps) continue;
        // preconditioned residual of root q in FP32
        std::vector<float> hc(3 * 64, 0.f);
        for (int j = 0; j < k; ++j) {
          hc[j] = (float)cX[j + (size_t)k * q];
          hc[64 + j] = (float)(theta[j] - thc[q]);
        }
        for (int l = 0; l < m0; ++l) hc[128 + l] = (float)cW[l + (size_t)m0 * q];
        SBDGB_CUDA(cudaMemcpyAsync(dcoef, hc.data(), sizeof(float) * 3 * 64, cudaMemcpyHostToDevice, s));
        MixedResArgs ma{Xf, Rf, W, HW, k, m0, N, dcoef, dcoef + 64, dcoef + 128, (float)thc[q], p.hii, Tf, sv.partial};
        k_mixed_residual<<<sv.blocks, kRed, 0, s>>>(ma);
        count_launch(p.ctx);
        res_est[q] = std::sqrt(std::max(0.0, sv.reduce_partials(1)));
        // orthogonalise against the rounded anchors, then against W, in FP32
        double n0 = sv.norm<float>(Tf);
        if (!(n0 > 0.0) || !std::isfinite(n0)) continue;
        sv.scale_copy<float, float>(Tf, Tf, 1.0 / n0);
        for (int pass = 0; pass < 2; ++pass) {
          std::vector<double> G;
          const float *w[1] = {Tf};
          sv.dots<float, float>(Xf, k, w, 1, G);
          sv.project_out<float>(Xf, k, G, Tf, 1);
        }
        const double left = sv.orthonormalize<float>(Tf, W, m);
        if (!(left > 1e-3)) continue;  // no new direction in FP32
        SBDGB_CUDA(cudaMemcpyAsync(W + (size_t)m * N, Tf, sizeof(float) * N, cudaMemcpyDeviceToDevice, s));
        sigma_mixed(p, W + (size_t)m * N, HW + (size_t)m * N, s);
        r.sigma_calls++;
        // projected quantities of the new column: anchor couplings in FP64
        const float *wn[1] = {W + (size_t)m * N};
        const float *hwn[1] = {HW + (size_t)m * N};
        std::vector<double> g1, g2, g3, g4, g5;
        sv.dots<double, float>(X, k, wn, 1, g1);     // X^T w
        sv.dots<float, float>(Rf, k, wn, 1, g2);     // R^T w
        sv.dots<float, float>(W, m + 1, wn, 1, g3);  // W^T w
        sv.dots<float, float>(W, m + 1, hwn, 1, g4); // W^T Hw
        sv.dots<float, float>(HW, m + 1, wn, 1, g5); // (HW)^T w
        for (int j = 0; j < k; ++j) {
          Sxw[j + (size_t)k * m] = g1[j];
          Hxw[j + (size_t)k * m] = g2[j] + theta[j] * g1[j];
        }
        for (int l = 0; l <= m; ++l) {
          Sww[l + (size_t)mmax * m] = Sww[m + (size_t)mmax * l] = g3[l];
          const double h = 0.5 * (g4[l] + g5[l]);
          Hww[l + (size_t)mmax * m] = Hww[m + (size_t)mmax * l] = h;
        }
        m++;
      }
      if (m == m0) {
        stalled = true;
        break;
      }
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
      std::vector<double> cx(k);
      std::vector<float> cw(m);
      for (int j = 0; j < k; ++j) cx[j] = cX[j + (size_t)k * q];
      for (int l = 0; l < m; ++l) cw[l] = (float)cW[l + (size_t)m * q];
      SBDGB_CUDA(cudaMemcpyAsync(sv.red + 3000, cx.data(), sizeof(double) * k, cudaMemcpyHostToDevice, s));
      if (m) SBDGB_CUDA(cudaMemcpyAsync(dcoef, cw.data(), sizeof(float) * m, cudaMemcpyHostToDevice, s));
      k_mixed_assemble<<<sv.blocks, kRed, 0, s>>>(X, k, W, m, N, sv.red + 3000, dcoef, T + (size_t)q * N);
      count_launch(p.ctx);
    }
    for (int q = 0; q < k; ++q) {
      double *t = T + (size_t)q * N;
      const double left = sv.orthonormalize<double>(t, T, q);
      SBDGB_REQUIRE(left > 1e-8, SBDGB_E_STATE, "mixed Davidson lost a root");
    }
    SBDGB_CUDA(cudaMemcpyAsync(X, T, sizeof(double) * N * k, cudaMemcpyDeviceToDevice, s));
    r.restarts++;
    refine_rr();
    if (m + k > mmax) m = 0;  // subspace full: the anchors carry its information on
    if (stalled) {
      bool ok = true;
      for (int q = 0; q < k; ++q) ok = ok && resid[q] < o.eps;
      if (!ok) {
        if (m == 0) {
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
  if (Xout) SBDGB_CUDA(cudaMemcpyAsync(Xout, X, sizeof(double) * N * k, cudaMemcpyDeviceToHost, s));
  SBDGB_CUDA(cudaStreamSynchronize(s));
  r.seconds = std::chrono::duration<double>(clock::now() - t0).count();
  if (rep) *rep = r;
}

}  // namespace

void davidson(Problem &p, const sbdgb_davidson_opts &o, double *E, double *Xout, sbdgb_report *rep) {
  if (!p.tables || !p.diag) throw Error(SBDGB_E_STATE, "Davidson needs tables and diagonal");
  SBDGB_REQUIRE(o.nroots >= 1 && o.nroots <= 16, SBDGB_E_INPUT, "nroots must be in [1, 16]");
  SBDGB_REQUIRE((size_t)o.nroots <= p.N, SBDGB_E_INPUT, "more roots than determinants");
  if (o.precision == SBDGB_MIXED)
    davidson_mixed(p, o, E, Xout, rep);
  else
    davidson_fp64(p, o, E, Xout, rep);
}

}  // namespace sbdgb
