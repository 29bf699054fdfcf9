// Davidson eigensolver on the device (replaces sbd::Davidson,
// chemistry/tpb/davidson.h:707-970, and its GPU form chemistry/basic/
// davidson_thrust.h:97-385 / :389-675).
//
// The reference solves one root with a single-vector Davidson: subspace up to
// max_nb, Ritz pair from the projected matrix, residual R = E0 W - H W,
// diagonal preconditioner R/(E0 - d) with a 1e-12 guard, modified
// Gram-Schmidt, restart C0 = W (which recomputes sigma(W)).  This solver keeps
// those steps and generalises them to nroots: each step adds one corrected
// direction per unconverged root, orthogonalises it against the basis with
// classical Gram-Schmidt plus a second pass when the norm drops (the
// "twice is enough" rule), and restarts from the nroots Ritz vectors together
// with their sigma vectors, which are formed from the stored H*V instead of a
// new sigma product.  Vectors stay resident in HBM; only the projected
// (<= max_nb)^2 matrix and a few norms cross to the host per step.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>

#include "common.cuh"

namespace sbdgb {

void transpose_fp64(Problem &p, const double *in, double *out, uint32_t R, uint32_t Cn, cudaStream_t s);

namespace {

constexpr int kRed = 256;   // threads per reduction block
constexpr int kMaxV = 8;    // basis columns per dots pass
constexpr int kMaxW = 4;    // right-hand columns per dots pass
constexpr int kMaxCoef = 64 * 16;

struct ColPtrs {
  const double *p[kMaxV];
};
struct WPtrs {
  const double *p[kMaxW];
};

// partial[b][i*nw+j] = sum over this block's elements of V_i * W_j.
template <int NV, int NW>
__global__ void __launch_bounds__(kRed) k_dots(ColPtrs V, WPtrs W, size_t N, double *__restrict__ partial) {
  double acc[NV][NW];
#pragma unroll
  for (int i = 0; i < NV; ++i)
#pragma unroll
    for (int j = 0; j < NW; ++j) acc[i][j] = 0.0;
  for (size_t e = blockIdx.x * (size_t)kRed + threadIdx.x; e < N; e += (size_t)gridDim.x * kRed) {
    double w[NW];
#pragma unroll
    for (int j = 0; j < NW; ++j) w[j] = __ldg(W.p[j] + e);
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      const double v = __ldg(V.p[i] + e);
#pragma unroll
      for (int j = 0; j < NW; ++j) acc[i][j] = fma(v, w[j], acc[i][j]);
    }
  }
  __shared__ double red[kRed / 32][NV * NW];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < NV; ++i)
#pragma unroll
    for (int j = 0; j < NW; ++j) {
      double x = acc[i][j];
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
  double *X;    // k x N or null
  double *HX;   // k x N or null
  double *T;    // k x N or null: preconditioned residual
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

// T_r -= sum_j V_j G[j][r]  (G column-major, ld = nv), then optional scale.
template <int K>
__global__ void __launch_bounds__(kRed) k_project_out(const double *__restrict__ V, int nv, size_t N,
                                                       const double *__restrict__ G, double *__restrict__ T) {
  __shared__ double gs[kMaxCoef];
  for (int t = threadIdx.x; t < nv * K; t += kRed) gs[t] = G[t];
  __syncthreads();
  for (size_t e = blockIdx.x * (size_t)kRed + threadIdx.x; e < N; e += (size_t)gridDim.x * kRed) {
    double t[K];
#pragma unroll
    for (int r = 0; r < K; ++r) t[r] = T[(size_t)r * N + e];
    for (int j = 0; j < nv; ++j) {
      const double v = __ldg(V + (size_t)j * N + e);
#pragma unroll
      for (int r = 0; r < K; ++r) t[r] = fma(-v, gs[j + nv * r], t[r]);
    }
#pragma unroll
    for (int r = 0; r < K; ++r) T[(size_t)r * N + e] = t[r];
  }
}

__global__ void k_scale_copy(const double *__restrict__ x, double *__restrict__ y, size_t N, double f) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < N; e += (size_t)gridDim.x * blockDim.x)
    y[e] = x[e] * f;
}

__global__ void k_axpy(double *__restrict__ y, const double *__restrict__ x, size_t N, double f) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < N; e += (size_t)gridDim.x * blockDim.x)
    y[e] = fma(f, x[e], y[e]);
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

// Symmetric eigensolver for the projected matrix: cyclic Jacobi, eigenvalues
// ascending (stands in for LAPACK dsyev, framework/hp_numeric.h:503-520).
void jacobi_eig(int n, std::vector<double> A, std::vector<double> &w, std::vector<double> &Vout) {
  std::vector<double> V((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) V[i + (size_t)n * i] = 1.0;
  auto a = [&](int i, int j) -> double & { return A[i + (size_t)n * j]; };
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0, dg = 0.0;
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) (i == j ? dg : off) += a(i, j) * a(i, j);
    if (off <= 1e-30 * (dg + 1e-300)) break;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        const double apq = a(p, q);
        if (std::fabs(apq) < 1e-300) continue;
        const double theta = (a(q, q) - a(p, p)) / (2.0 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < n; ++k) {
          const double akp = a(k, p), akq = a(k, q);
          a(k, p) = c * akp - s * akq;
          a(k, q) = s * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) {
          const double apk = a(p, k), aqk = a(q, k);
          a(p, k) = c * apk - s * aqk;
          a(q, k) = s * apk + c * aqk;
        }
        for (int k = 0; k < n; ++k) {
          const double vkp = V[k + (size_t)n * p], vkq = V[k + (size_t)n * q];
          V[k + (size_t)n * p] = c * vkp - s * vkq;
          V[k + (size_t)n * q] = s * vkp + c * vkq;
        }
      }
  }
  std::vector<int> idx(n);
  for (int i = 0; i < n; ++i) idx[i] = i;
  std::stable_sort(idx.begin(), idx.end(), [&](int x, int y) { return a(x, x) < a(y, y); });
  w.resize(n);
  Vout.assign((size_t)n * n, 0.0);
  for (int j = 0; j < n; ++j) {
    w[j] = a(idx[j], idx[j]);
    for (int i = 0; i < n; ++i) Vout[i + (size_t)n * j] = V[i + (size_t)n * idx[j]];
  }
}

struct Solver {
  Problem &p;
  cudaStream_t s;
  size_t N;
  int blocks;
  double *partial = nullptr;   // blocks * kMaxV*kMaxW
  double *red = nullptr;       // reduced results (device)
  double *coef = nullptr;      // device coefficient staging
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
  void dots(const double *V0, int nv, const double *const *W, int nw, std::vector<double> &G) {
    G.assign((size_t)nv * nw, 0.0);
    for (int j0 = 0; j0 < nw; j0 += kMaxW) {
      const int mw = std::min(kMaxW, nw - j0);
      WPtrs wp{};
      for (int j = 0; j < kMaxW; ++j) wp.p[j] = W[j0 + std::min(j, mw - 1)];
      for (int i0 = 0; i0 < nv; i0 += kMaxV) {
        const int mv = std::min(kMaxV, nv - i0);
        ColPtrs vp{};
        for (int i = 0; i < kMaxV; ++i) vp.p[i] = V0 + (size_t)(i0 + std::min(i, mv - 1)) * N;
        launch_dots(vp, wp, mv, mw);
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

  template <int NV>
  void launch_dots_w(ColPtrs vp, WPtrs wp, int mw) {
    switch (mw) {
      case 1: k_dots<NV, 1><<<blocks, kRed, 0, s>>>(vp, wp, N, partial); break;
      case 2: k_dots<NV, 2><<<blocks, kRed, 0, s>>>(vp, wp, N, partial); break;
      case 3: k_dots<NV, 3><<<blocks, kRed, 0, s>>>(vp, wp, N, partial); break;
      default: k_dots<NV, 4><<<blocks, kRed, 0, s>>>(vp, wp, N, partial); break;
    }
  }
  void launch_dots(ColPtrs vp, WPtrs wp, int mv, int mw) {
    switch (mv) {
      case 1: launch_dots_w<1>(vp, wp, mw); break;
      case 2: launch_dots_w<2>(vp, wp, mw); break;
      case 3: launch_dots_w<3>(vp, wp, mw); break;
      case 4: launch_dots_w<4>(vp, wp, mw); break;
      case 5: launch_dots_w<5>(vp, wp, mw); break;
      case 6: launch_dots_w<6>(vp, wp, mw); break;
      case 7: launch_dots_w<7>(vp, wp, mw); break;
      default: launch_dots_w<8>(vp, wp, mw); break;
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

  void project_out(const double *V, int nv, const std::vector<double> &G, double *T, int k) {
    if (nv == 0) return;
    SBDGB_CUDA(cudaMemcpyAsync(coef, G.data(), sizeof(double) * nv * k, cudaMemcpyHostToDevice, s));
    switch (k) {
#define SBDGB_K(KK) \
  case KK: k_project_out<KK><<<blocks, kRed, 0, s>>>(V, nv, N, coef, T); break;
      SBDGB_K(1) SBDGB_K(2) SBDGB_K(3) SBDGB_K(4) SBDGB_K(5) SBDGB_K(6) SBDGB_K(7) SBDGB_K(8)
      SBDGB_K(9) SBDGB_K(10) SBDGB_K(11) SBDGB_K(12) SBDGB_K(13) SBDGB_K(14) SBDGB_K(15) SBDGB_K(16)
#undef SBDGB_K
      default: throw Error(SBDGB_E_UNSUPPORTED, "at most 16 roots");
    }
    count_launch(p.ctx);
    SBDGB_CUDA(cudaGetLastError());
  }

  void scale_copy(const double *x, double *y, double f) {
    k_scale_copy<<<blocks, kRed, 0, s>>>(x, y, N, f);
    count_launch(p.ctx);
  }
  void axpy(double *y, const double *x, double f) {
    k_axpy<<<blocks, kRed, 0, s>>>(y, x, N, f);
    count_launch(p.ctx);
  }
  double norm(const double *x) {
    std::vector<double> g;
    const double *w[1] = {x};
    dots(x, 1, w, 1, g);
    return std::sqrt(std::max(0.0, g[0]));
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
};

}  // namespace

void davidson(Problem &p, const sbdgb_davidson_opts &o, double *E, double *Xout, sbdgb_report *rep) {
  using clock = std::chrono::steady_clock;
  const auto t0 = clock::now();
  if (!p.tables || !p.diag) throw Error(SBDGB_E_STATE, "Davidson needs tables and diagonal");
  const int k = o.nroots;
  const size_t N = p.N;
  SBDGB_REQUIRE(k >= 1 && k <= 16, SBDGB_E_INPUT, "nroots must be in [1, 16]");
  SBDGB_REQUIRE((size_t)k <= N, SBDGB_E_INPUT, "more roots than determinants");
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
  // ---- initial vectors (BasisInitVector, davidson.h:144-184) ----
  int nv = 0;
  if (o.init == 2) {
    SBDGB_REQUIRE(Xout != nullptr, SBDGB_E_INPUT, "init 2 needs starting vectors in X");
    SBDGB_CUDA(cudaMemcpyAsync(T, Xout, sizeof(double) * N * k, cudaMemcpyHostToDevice, s));
  } else {
    std::vector<size_t> pos;
    if (o.init == 0) {
      pos.push_back(0);
      if (k > 1) {
        auto low = sv.lowest_diagonal(k + 1);
        for (size_t q : low)
          if (q != 0 && (int)pos.size() < k) pos.push_back(q);
      }
    } else {
      pos = sv.lowest_diagonal(k);
    }
    for (int q = 0; q < k; ++q) {
      k_fill_unit<<<sv.blocks, kRed, 0, s>>>(T + (size_t)q * N, N, pos[q]);
      count_launch(p.ctx);
    }
  }
  // orthonormalise the starting block into V
  auto append = [&](double *Tin, int nt) -> int {
    int added = 0;
    for (int q = 0; q < nt; ++q) {
      double *t = Tin + (size_t)q * N;
      double n0 = sv.norm(t);
      if (!(n0 > 0.0)) continue;
      for (int pass = 0; pass < 2; ++pass) {
        if (nv == 0) break;
        std::vector<double> G;
        const double *w[1] = {t};
        sv.dots(V, nv, w, 1, G);
        sv.project_out(V, nv, G, t, 1);
        double n1 = sv.norm(t);
        if (n1 > 0.7071 * n0) {
          n0 = n1;
          break;
        }
        n0 = n1;
      }
      if (!(n0 > 1e-10)) continue;  // linearly dependent direction: dropped
      sv.scale_copy(t, V + (size_t)nv * N, 1.0 / n0);
      nv++;
      added++;
      if (nv >= max_nb) break;
    }
    return added;
  };
  // sigma of the vectors V[from .. nv)
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
    sv.dots(V, nv, w.data(), (int)w.size(), G);
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
      for (int i = 0; i < nv; ++i) A[i + (size_t)nv * j] = 0.5 * (Hs[i + (size_t)max_nb * j] + Hs[j + (size_t)max_nb * i]);
    jacobi_eig(nv, A, theta, Y);
    const int kk = std::min(k, nv);
    std::vector<double> c((size_t)nv * kk);
    for (int q = 0; q < kk; ++q)
      for (int i = 0; i < nv; ++i) c[i + (size_t)nv * q] = Y[i + (size_t)nv * q];
    std::vector<double> th(theta.begin(), theta.begin() + kk);
    resid = sv.combine(V, HV, nv, kk, c, th, X, HX, T);
    iter++;
    r.iterations = iter;
    if (o.verbose) {
      printf(" Davidson iteration %d (tol=%.6g):", iter, *std::max_element(resid.begin(), resid.end()));
      for (int q = 0; q < std::min(kk, 4); ++q) printf(" %.12f", th[q]);
      printf("\n");
      fflush(stdout);
    }
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

}  // namespace sbdgb
