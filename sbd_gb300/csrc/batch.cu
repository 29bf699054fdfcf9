// Many small Davidson solves in one launch: one CTA runs the whole FP64 solve
// of one problem (sigma products, projections, Rayleigh-Ritz, corrections and
// restarts) with no host round trip, so thousands of tiny problems cost one
// kernel launch instead of tens of launches and synchronisations per
// iteration each.
//
// The algorithm is the device solver's (davidson.cu, the reference's
// chemistry/tpb/davidson.h:707-970 generalised to nroots): lowest-diagonal
// start vectors with the deterministic perturbation, Olsen-corrected diagonal
// preconditioner with the reference's 1e-12 guard, classical Gram-Schmidt
// with a second pass, thick restart on the Ritz vectors and the previous
// step's Ritz vectors, convergence on every residual norm below eps.
//
// Inside a CTA:
//   - sigma: one element per thread at a time, the fused form (diagonal,
//     alpha pairs of the row with the sigma kernels' same-spin sweep, alpha x
//     beta singles, beta pairs of the column read from the same row);
//   - dot products: up to 8 x 4 per pass in registers, one block reduction;
//   - the projected eigenproblem (n <= 32): cyclic Jacobi by one warp in
//     shared memory; coefficient-space Gram-Schmidt by one thread.
#include <algorithm>
#include <chrono>
#include <cmath>

#include "common.cuh"
#include "sigma_dev.cuh"

namespace sbdgb {

namespace {

using namespace sdev;

constexpr int kBT = 256;      // threads per problem
constexpr int kBMaxNb = 32;   // subspace cap of the batched solver
constexpr int kBMaxK = 8;     // roots

struct SmallProb {
  Args<double> a;  // strings, tables, integrals, diagonal (C, CT, S unused)
  uint32_t N;
  int norb;
  double *V, *HV, *X, *HX, *T, *U;  // N x kBMaxNb, N x kBMaxNb, N x 2k, N x 2k, N x k, N x k
  double *Xout;                      // N x k Ritz vectors, or null
  double *out;                       // k energies, k residuals, then [iterations, sigma calls, converged, restarts]
};

struct SmallOpts {
  int k, max_nb, max_steps;
  double eps;
};

struct Smem {
  double A[kBMaxNb * kBMaxNb];   // projected matrix (column-major, ld kBMaxNb)
  double W[kBMaxNb * kBMaxNb];   // scratch matrix (eigenvectors, Q, Gram)
  double E[kBMaxNb];             // eigenvalues
  double c[kBMaxNb * kBMaxK];    // Ritz coefficients (nv x kk)
  double cprev[kBMaxNb * kBMaxK];
  double G[kBMaxNb * kBMaxK];    // dots
  double red[kBT / 32][32];
  double th[kBMaxK], res[kBMaxK], eo[kBMaxK];
  double M[kBMaxK * kBMaxK];
  double dv[kBT / 32];
  unsigned long long di[kBT / 32];
  unsigned long long pos[kBMaxK];
  int ival[8];
};

// ---- block primitives ------------------------------------------------------------

// Sum of one value over the block; every thread gets it.
__device__ double block_sum(double v, Smem &sm) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) sm.dv[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.0;
  for (int w = 0; w < kBT / 32; ++w) t += sm.dv[w];
  return t;
}

// G[i + ldg*j] = V_i . W_j for i < nv, j < nw (columns at stride N).
__device__ void block_dots(const double *V, int nv, const double *W, int nw, uint32_t N, double *G, int ldg,
                           Smem &sm) {
  for (int j0 = 0; j0 < nw; j0 += 4)
    for (int i0 = 0; i0 < nv; i0 += 8) {
      const int mw = min(4, nw - j0), mv = min(8, nv - i0);
      double acc[8][4];
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0.0;
      for (uint32_t e = threadIdx.x; e < N; e += kBT) {
        double w[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) w[j] = j < mw ? W[(size_t)(j0 + j) * N + e] : 0.0;
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          if (i >= mv) break;
          const double v = V[(size_t)(i0 + i) * N + e];
#pragma unroll
          for (int j = 0; j < 4; ++j) acc[i][j] = fma(v, w[j], acc[i][j]);
        }
      }
      __syncthreads();
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          double x = acc[i][j];
          for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
          if ((threadIdx.x & 31) == 0) sm.red[threadIdx.x >> 5][i * 4 + j] = x;
        }
      __syncthreads();
      if (threadIdx.x < 32) {
        const int i = threadIdx.x / 4, j = threadIdx.x % 4;
        if (i < mv && j < mw) {
          double t = 0.0;
          for (int w2 = 0; w2 < kBT / 32; ++w2) t += sm.red[w2][threadIdx.x];
          G[(i0 + i) + (size_t)ldg * (j0 + j)] = t;
        }
      }
      __syncthreads();
    }
}

// Symmetric eigenproblem of the n x n leading block of sm.A (ld kBMaxNb), by
// warp 0: eigenvalues ascending in sm.E, eigenvectors in the columns of sm.W.
__device__ void block_eig(int n, Smem &sm, double *Aw) {
  // Aw: a working copy (shared), ld kBMaxNb
  for (int t = threadIdx.x; t < kBMaxNb * kBMaxNb; t += kBT) {
    const int i = t % kBMaxNb, j = t / kBMaxNb;
    Aw[t] = (i < n && j < n) ? 0.5 * (sm.A[i + kBMaxNb * j] + sm.A[j + kBMaxNb * i]) : 0.0;
    sm.W[t] = (i == j) ? 1.0 : 0.0;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    const int l = threadIdx.x;
    for (int sweep = 0; sweep < 60; ++sweep) {
      double off = 0.0, dg = 0.0;
      for (int j = 0; j < n; ++j)
        if (l < n) {
          const double x = Aw[l + kBMaxNb * j];
          if (l == j) dg += x * x; else off += x * x;
        }
      for (int o = 16; o > 0; o >>= 1) {
        off += __shfl_xor_sync(0xffffffffu, off, o);
        dg += __shfl_xor_sync(0xffffffffu, dg, o);
      }
      if (off <= 1e-30 * (dg + 1e-300)) break;
      for (int p = 0; p < n - 1; ++p)
        for (int q = p + 1; q < n; ++q) {
          const double apq = Aw[p + kBMaxNb * q];
          if (fabs(apq) < 1e-300) continue;
          const double theta = (Aw[q + kBMaxNb * q] - Aw[p + kBMaxNb * p]) / (2.0 * apq);
          const double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
          const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
          __syncwarp();
          if (l < n) {  // columns p, q
            const double akp = Aw[l + kBMaxNb * p], akq = Aw[l + kBMaxNb * q];
            Aw[l + kBMaxNb * p] = c * akp - s * akq;
            Aw[l + kBMaxNb * q] = s * akp + c * akq;
          }
          __syncwarp();
          if (l < n) {  // rows p, q
            const double apk = Aw[p + kBMaxNb * l], aqk = Aw[q + kBMaxNb * l];
            Aw[p + kBMaxNb * l] = c * apk - s * aqk;
            Aw[q + kBMaxNb * l] = s * apk + c * aqk;
            const double vkp = sm.W[l + kBMaxNb * p], vkq = sm.W[l + kBMaxNb * q];
            sm.W[l + kBMaxNb * p] = c * vkp - s * vkq;
            sm.W[l + kBMaxNb * q] = s * vkp + c * vkq;
          }
          __syncwarp();
        }
    }
    if (l == 0) {  // sort ascending (selection), permuting the eigenvector columns
      for (int i = 0; i < n; ++i) sm.E[i] = Aw[i + kBMaxNb * i];
      for (int i = 0; i < n; ++i) {
        int b = i;
        for (int j = i + 1; j < n; ++j)
          if (sm.E[j] < sm.E[b]) b = j;
        if (b != i) {
          const double e = sm.E[i];
          sm.E[i] = sm.E[b];
          sm.E[b] = e;
          for (int r = 0; r < n; ++r) {
            const double x = sm.W[r + kBMaxNb * i];
            sm.W[r + kBMaxNb * i] = sm.W[r + kBMaxNb * b];
            sm.W[r + kBMaxNb * b] = x;
          }
        }
      }
    }
  }
  __syncthreads();
}

// One sigma element, fused form (as k_sigma_alpha<..., kFused>).
template <typename Wd>
__device__ double sigma_element(const Args<double> &a, const double *__restrict__ x, uint32_t ia, uint32_t ib) {
  const uint32_t col[1] = {ib};
  const bool ok[1] = {true};
  const Wd beta[1] = {word<Wd>(a.bstr, ib)};
  double acc[1] = {a.hii[(size_t)ia * a.nb + ib] * x[(size_t)ia * a.nb + ib]};
  same_spin_row<1, double, Wd>(a.A, a.val_sa, a.val_da, a.Jb, a.nb, x, a.nb, ia, col, ok, beta, acc);
  double part = 0.0;
  const uint32_t q0 = a.B.off_s[ib], q1 = a.B.off_s[ib + 1];
  for (uint32_t p = a.A.off_s[ia]; p < a.A.off_s[ia + 1]; ++p) {
    const uint32_t ja = a.A.ket_s[p], ca = a.A.code_s[p];
    const Wd alpha_ket = word<Wd>(a.astr, ja);
    const double *krow = a.Kp + (size_t)((ca >> 16) & 0x7fffu) * a.npair;
    const uint32_t pa = parity(beta[0] & word<Wd>(a.A.mask_s, p)) ^ (ca >> 31);
    for (uint32_t q = q0; q < q1; ++q) {
      const uint32_t jb = a.B.ket_s[q], cb = a.B.code_s[q];
      const uint32_t ph = (pa ^ parity(alpha_ket & word<Wd>(a.B.mask_s, q)) ^ (cb >> 31)) & 1u;
      part = fma(flip(krow[(cb >> 16) & 0x7fffu], ph), x[(size_t)ja * a.nb + jb], part);
    }
  }
  const Wd arow = word<Wd>(a.astr, ia);
  const double *row = x + (size_t)ia * a.nb;
  for (uint32_t q = q0; q < q1; ++q) {
    const uint32_t jb = a.B.ket_s[q], cb = a.B.code_s[q];
    const uint32_t ph = parity(arow & word<Wd>(a.B.mask_s, q)) ^ (cb >> 31);
    part = fma(flip(a.val_sb[q] + a.Ja[(size_t)((cb >> 16) & 0x7fffu) * a.na + ia], ph), row[jb], part);
  }
  for (uint32_t q = a.B.off_d[ib]; q < a.B.off_d[ib + 1]; ++q)
    part = fma(flip(a.val_db[q], parity(arow & word<Wd>(a.B.mask_d, q))), row[a.B.ket_d[q]], part);
  return acc[0] + part;
}

template <typename Wd>
__device__ void block_sigma(const SmallProb &P, const double *x, double *y) {
  for (uint32_t e = threadIdx.x; e < P.N; e += kBT) y[e] = sigma_element<Wd>(P.a, x, e / P.a.nb, e % P.a.nb);
  __syncthreads();
}

// Orthonormalises the nt columns of T (stride N) against V[0, nv) and among
// themselves (CGS with a second pass when a norm falls below half, then
// coefficient-space Gram-Schmidt with dropping below `drop` of the original
// norm); writes the kept directions to V[nv, nv + kept).  Returns kept.
__device__ int block_orthonormalize(double *T, int nt, double *V, int nv, uint32_t N, double drop, Smem &sm) {
  double n0[kBMaxK], prev[kBMaxK];
  block_dots(T, nt, T, nt, N, sm.W, kBMaxNb, sm);
  for (int q = 0; q < nt; ++q) n0[q] = prev[q] = sm.W[q + kBMaxNb * q];
  for (int pass = 0; pass < 2 && nv > 0; ++pass) {
    block_dots(V, nv, T, nt, N, sm.G, kBMaxNb, sm);
    for (uint32_t e = threadIdx.x; e < N; e += kBT)
      for (int q = 0; q < nt; ++q) {
        double t = T[(size_t)q * N + e];
        for (int j = 0; j < nv; ++j) t = fma(-V[(size_t)j * N + e], sm.G[j + kBMaxNb * q], t);
        T[(size_t)q * N + e] = t;
      }
    __syncthreads();
    block_dots(T, nt, T, nt, N, sm.W, kBMaxNb, sm);
    bool again = false;
    for (int q = 0; q < nt; ++q) {
      const double g = sm.W[q + kBMaxNb * q];
      again = again || (g < 0.5 * prev[q]);
      prev[q] = g;
    }
    if (!again) break;
  }
  // coefficient-space Gram-Schmidt on the Gram matrix sm.W (thread 0)
  if (threadIdx.x == 0) {
    int kept = 0;
    for (int q = 0; q < nt; ++q) {
      if (!(n0[q] > 0.0)) continue;
      double v[kBMaxK];
      for (int i = 0; i < nt; ++i) v[i] = (i == q) ? 1.0 : 0.0;
      for (int pass = 0; pass < 2; ++pass)
        for (int u = 0; u < kept; ++u) {
          double pr = 0.0;
          for (int i = 0; i < nt; ++i)
            for (int j = 0; j < nt; ++j) pr += sm.M[i + kBMaxK * u] * sm.W[i + kBMaxNb * j] * v[j];
          for (int i = 0; i < nt; ++i) v[i] -= pr * sm.M[i + kBMaxK * u];
        }
      double nn = 0.0;
      for (int i = 0; i < nt; ++i)
        for (int j = 0; j < nt; ++j) nn += v[i] * sm.W[i + kBMaxNb * j] * v[j];
      if (!(nn > drop * drop * n0[q])) continue;
      const double f = 1.0 / sqrt(nn);
      for (int i = 0; i < nt; ++i) sm.M[i + kBMaxK * kept] = v[i] * f;
      ++kept;
    }
    sm.ival[0] = kept;
  }
  __syncthreads();
  const int kept = sm.ival[0];
  for (uint32_t e = threadIdx.x; e < N; e += kBT) {
    double t[kBMaxK];
    for (int q = 0; q < nt; ++q) t[q] = T[(size_t)q * N + e];
    for (int c = 0; c < kept; ++c) {
      double y = 0.0;
      for (int q = 0; q < nt; ++q) y = fma(t[q], sm.M[q + kBMaxK * c], y);
      V[(size_t)(nv + c) * N + e] = y;
    }
  }
  __syncthreads();
  return kept;
}

template <typename Wd>
__device__ void solve_one(const SmallProb &P, const SmallOpts o, Smem &sm, double *Aw) {
  const uint32_t N = P.N;
  const int k = min(o.k, (int)N);
  const int max_nb = min(min(max(o.max_nb, 2 * k), kBMaxNb), (int)N);
  double *V = P.V, *HV = P.HV, *T = P.T, *U = P.U;
  // start vectors: unit vectors on the k lowest diagonal entries (ties by
  // index) plus a deterministic splitmix64 component of total size 1e-3
  for (int q = 0; q < k; ++q) {
    double best = INFINITY;
    unsigned long long bi = ~0ull;
    for (uint32_t e = threadIdx.x; e < N; e += kBT) {
      bool skip = false;
      for (int r = 0; r < q; ++r) skip |= (sm.pos[r] == e);
      const double h = P.a.hii[e];
      if (!skip && (h < best || (h == best && e < bi))) {
        best = h;
        bi = e;
      }
    }
    for (int off = 16; off > 0; off >>= 1) {
      const double b2 = __shfl_xor_sync(0xffffffffu, best, off);
      const unsigned long long i2 = __shfl_xor_sync(0xffffffffu, bi, off);
      if (b2 < best || (b2 == best && i2 < bi)) {
        best = b2;
        bi = i2;
      }
    }
    if ((threadIdx.x & 31) == 0) {
      sm.dv[threadIdx.x >> 5] = best;
      sm.di[threadIdx.x >> 5] = bi;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      double b = INFINITY;
      unsigned long long ix = ~0ull;
      for (int w = 0; w < kBT / 32; ++w)
        if (sm.dv[w] < b || (sm.dv[w] == b && sm.di[w] < ix)) {
          b = sm.dv[w];
          ix = sm.di[w];
        }
      sm.pos[q] = ix;
    }
    __syncthreads();
  }
  const double amp = 1e-3 * sqrt(3.0 / (double)N);
  for (uint32_t e = threadIdx.x; e < N; e += kBT)
    for (int q = 0; q < k; ++q) {
      uint64_t z = (uint64_t)e * 0x9E3779B97F4A7C15ull + 0x5BD1E995ull * (uint64_t)(q + 1);
      z ^= z >> 30;
      z *= 0xBF58476D1CE4E5B9ull;
      z ^= z >> 27;
      z *= 0x94D049BB133111EBull;
      z ^= z >> 31;
      T[(size_t)q * N + e] = (e == sm.pos[q] ? 1.0 : 0.0) + amp * ((double)(z >> 11) * (2.0 / 9007199254740992.0) - 1.0);
    }
  __syncthreads();
  int nv = block_orthonormalize(T, k, V, 0, N, 1e-8, sm);
  int sigma_calls = 0, restarts = 0, iter = 0, kk = 0, nvprev = 0, kprev = 0;
  for (int j = 0; j < nv; ++j) block_sigma<Wd>(P, V + (size_t)j * N, HV + (size_t)j * N);
  sigma_calls += nv;
  block_dots(V, nv, HV, nv, N, sm.A, kBMaxNb, sm);
  bool converged = false;
  while (true) {
    block_eig(nv, sm, Aw);
    kk = min(k, nv);
    for (int t = threadIdx.x; t < nv * kk; t += kBT) sm.c[t] = sm.W[(t % nv) + kBMaxNb * (t / nv)];
    if (threadIdx.x < kk) sm.th[threadIdx.x] = sm.E[threadIdx.x];
    __syncthreads();
    // residuals and Olsen-corrected preconditioned corrections
    double rn[kBMaxK], xt[kBMaxK], xu[kBMaxK];
    for (int q = 0; q < kk; ++q) rn[q] = xt[q] = xu[q] = 0.0;
    for (uint32_t e = threadIdx.x; e < N; e += kBT) {
      const double d = P.a.hii[e];
      for (int q = 0; q < kk; ++q) {
        double xv = 0.0, hv = 0.0;
        for (int j = 0; j < nv; ++j) {
          const double cq = sm.c[j + nv * q];
          xv = fma(V[(size_t)j * N + e], cq, xv);
          hv = fma(HV[(size_t)j * N + e], cq, hv);
        }
        const double r = hv - sm.th[q] * xv;
        rn[q] = fma(r, r, rn[q]);
        double den = sm.th[q] - d;
        if (fabs(den) <= 1.0e-12) den -= 1.0e-12;
        const double t = r / den, u = xv / den;
        T[(size_t)q * N + e] = t;
        U[(size_t)q * N + e] = u;
        xt[q] = fma(xv, t, xt[q]);
        xu[q] = fma(xv, u, xu[q]);
      }
    }
    for (int q = 0; q < kk; ++q) {
      const double rq = sqrt(fmax(0.0, block_sum(rn[q], sm)));
      const double a1 = block_sum(xt[q], sm), a2 = block_sum(xu[q], sm);
      if (threadIdx.x == 0) {
        sm.res[q] = rq;
        sm.eo[q] = (a2 != 0.0 && isfinite(a1 / a2)) ? a1 / a2 : 0.0;
      }
    }
    __syncthreads();
    for (uint32_t e = threadIdx.x; e < N; e += kBT)
      for (int q = 0; q < kk; ++q) T[(size_t)q * N + e] = fma(-sm.eo[q], U[(size_t)q * N + e], T[(size_t)q * N + e]);
    __syncthreads();
    ++iter;
    converged = kk == k;
    int nnew = 0;
    for (int q = 0; q < kk; ++q) {
      converged = converged && (sm.res[q] < o.eps);
      nnew += (sm.res[q] >= o.eps);
    }
    if (converged || iter >= o.max_steps) break;
    if (nv + nnew > max_nb) {
      // thick restart on span{Ritz vectors, previous Ritz vectors}: V Q, HV Q, Q^T A Q
      if (threadIdx.x == 0) {
        int m = 0;
        const int nkeep = min(kprev, max_nb - kk - nnew);
        for (int col = 0; col < kk + nkeep; ++col) {
          double v[kBMaxNb];
          for (int i = 0; i < nv; ++i)
            v[i] = col < kk ? sm.c[i + nv * col] : (i < nvprev ? sm.cprev[i + nvprev * (col - kk)] : 0.0);
          double n0 = 0.0;
          for (int i = 0; i < nv; ++i) n0 += v[i] * v[i];
          n0 = sqrt(n0);
          for (int pass = 0; pass < 2; ++pass)
            for (int j = 0; j < m; ++j) {
              double pr = 0.0;
              for (int i = 0; i < nv; ++i) pr += sm.W[i + kBMaxNb * j] * v[i];
              for (int i = 0; i < nv; ++i) v[i] -= pr * sm.W[i + kBMaxNb * j];
            }
          double nn = 0.0;
          for (int i = 0; i < nv; ++i) nn += v[i] * v[i];
          nn = sqrt(nn);
          if (!(nn > 1e-8 * n0)) continue;
          for (int i = 0; i < nv; ++i) sm.W[i + kBMaxNb * m] = v[i] / nn;
          ++m;
        }
        sm.ival[1] = m;
      }
      __syncthreads();
      const int m = sm.ival[1];
      for (uint32_t e = threadIdx.x; e < N; e += kBT)
        for (int b = 0; b < m; ++b) {
          double xv = 0.0, hv = 0.0;
          for (int j = 0; j < nv; ++j) {
            xv = fma(V[(size_t)j * N + e], sm.W[j + kBMaxNb * b], xv);
            hv = fma(HV[(size_t)j * N + e], sm.W[j + kBMaxNb * b], hv);
          }
          P.X[(size_t)b * N + e] = xv;
          P.HX[(size_t)b * N + e] = hv;
        }
      __syncthreads();
      for (uint32_t e = threadIdx.x; e < N; e += kBT)
        for (int b = 0; b < m; ++b) {
          V[(size_t)b * N + e] = P.X[(size_t)b * N + e];
          HV[(size_t)b * N + e] = P.HX[(size_t)b * N + e];
        }
      // projected matrix Q^T A Q and the Ritz coefficients Q^T c (thread 0)
      if (threadIdx.x == 0) {
        // A Q into Aw (nv x m), then Q^T (A Q) (m x m) into a local block
        for (int b = 0; b < m; ++b)
          for (int j = 0; j < nv; ++j) {
            double aq = 0.0;
            for (int i = 0; i < nv; ++i)
              aq += 0.5 * (sm.A[j + kBMaxNb * i] + sm.A[i + kBMaxNb * j]) * sm.W[i + kBMaxNb * b];
            Aw[j + kBMaxNb * b] = aq;
          }
        double hn[2 * kBMaxK * 2 * kBMaxK];
        for (int b = 0; b < m; ++b)
          for (int a2 = 0; a2 < m; ++a2) {
            double t = 0.0;
            for (int j = 0; j < nv; ++j) t += sm.W[j + kBMaxNb * a2] * Aw[j + kBMaxNb * b];
            hn[a2 + m * b] = t;
          }
        for (int t = 0; t < kBMaxNb * kBMaxNb; ++t) sm.A[t] = 0.0;
        for (int b = 0; b < m; ++b)
          for (int a2 = 0; a2 < m; ++a2) sm.A[a2 + kBMaxNb * b] = hn[a2 + m * b];
        double cn[kBMaxNb * kBMaxK];
        for (int q = 0; q < kk; ++q)
          for (int a2 = 0; a2 < m; ++a2) {
            double t = 0.0;
            for (int i = 0; i < nv; ++i) t += sm.W[i + kBMaxNb * a2] * sm.c[i + nv * q];
            cn[a2 + m * q] = t;
          }
        for (int t = 0; t < m * kk; ++t) sm.c[t] = cn[t];
      }
      __syncthreads();
      nv = m;
      ++restarts;
    }
    for (int t = threadIdx.x; t < nv * kk; t += kBT) sm.cprev[t] = sm.c[t];
    nvprev = nv;
    kprev = kk;
    __syncthreads();
    // corrections of the unconverged roots, packed at the front of T
    int nt = 0;
    for (int q = 0; q < kk; ++q)
      if (sm.res[q] >= o.eps) {
        if (nt != q)
          for (uint32_t e = threadIdx.x; e < N; e += kBT) T[(size_t)nt * N + e] = T[(size_t)q * N + e];
        ++nt;
      }
    __syncthreads();
    const int added = block_orthonormalize(T, nt, V, nv, N, 1e-8, sm);
    if (added == 0) break;
    for (int j = nv; j < nv + added; ++j) block_sigma<Wd>(P, V + (size_t)j * N, HV + (size_t)j * N);
    sigma_calls += added;
    // new columns of the projected matrix
    block_dots(V, nv + added, HV + (size_t)nv * N, added, N, sm.G, kBMaxNb, sm);
    for (int t = threadIdx.x; t < (nv + added) * added; t += kBT) {
      const int i = t % (nv + added), jj = t / (nv + added);
      const double g = sm.G[i + kBMaxNb * jj];
      sm.A[i + kBMaxNb * (nv + jj)] = g;
      sm.A[(nv + jj) + kBMaxNb * i] = g;
    }
    __syncthreads();
    nv += added;
  }
  // outputs
  if (P.Xout)
    for (uint32_t e = threadIdx.x; e < N; e += kBT)
      for (int q = 0; q < kk; ++q) {
        double xv = 0.0;
        for (int j = 0; j < nv; ++j) xv = fma(V[(size_t)j * N + e], sm.c[j + nv * q], xv);
        P.Xout[(size_t)q * N + e] = xv;
      }
  if (threadIdx.x == 0) {
    for (int q = 0; q < o.k; ++q) {
      P.out[q] = q < kk ? sm.th[q] : NAN;
      P.out[o.k + q] = q < kk ? sm.res[q] : NAN;
    }
    P.out[2 * o.k + 0] = iter;
    P.out[2 * o.k + 1] = sigma_calls;
    P.out[2 * o.k + 2] = converged ? 1.0 : 0.0;
    P.out[2 * o.k + 3] = restarts;
  }
}

__global__ void __launch_bounds__(kBT) k_batch_davidson(const SmallProb *__restrict__ probs, SmallOpts o) {
  extern __shared__ double smem_raw[];
  Smem &sm = *reinterpret_cast<Smem *>(smem_raw);
  double *Aw = smem_raw + (sizeof(Smem) + 7) / 8;  // kBMaxNb^2 working copy for the eigensolver
  const SmallProb &P = probs[blockIdx.x];
  if (P.norb <= 32)
    solve_one<uint32_t>(P, o, sm, Aw);
  else
    solve_one<unsigned long long>(P, o, sm, Aw);
}

}  // namespace

// Solves every problem of the batch with the same options in one launch.
// Problems must belong to one context; tables and diagonals are built here if
// missing.  E: count x nroots energies; reps: count reports (may be null);
// X: count pointers to host buffers of nroots x N (entries may be null).
void batch_davidson(Ctx &c, Problem **ps, int count, const sbdgb_davidson_opts &o, double *E, sbdgb_report *reps,
                    double **X) {
  using clock = std::chrono::steady_clock;
  const auto t0 = clock::now();
  SBDGB_REQUIRE(count >= 0, SBDGB_E_INPUT, "negative batch size");
  if (count == 0) return;
  SBDGB_REQUIRE(o.nroots >= 1 && o.nroots <= kBMaxK, SBDGB_E_UNSUPPORTED, "the batched solver takes 1..8 roots");
  SBDGB_REQUIRE(o.precision == SBDGB_FP64, SBDGB_E_UNSUPPORTED, "the batched solver runs in FP64");
  SBDGB_REQUIRE(o.init == 1, SBDGB_E_UNSUPPORTED, "the batched solver starts on the lowest diagonal (init 1)");
  cudaStream_t s = c.stream;
  const int k = o.nroots, nb = std::min(std::max(o.max_nb, 2 * k), kBMaxNb);
  std::vector<SmallProb> hp(count);
  for (int i = 0; i < count; ++i) {
    Problem &p = *ps[i];
    SBDGB_REQUIRE(p.ctx == &c, SBDGB_E_INPUT, "batch problems must belong to the context");
    SBDGB_REQUIRE(p.N >= (uint64_t)k, SBDGB_E_INPUT, "more roots than determinants");
    if (!p.tables) build_tables(p, s);
    if (!p.diag) build_diag(p, s);
    const size_t N = p.N;
    double *w = (double *)workspace(p, WS_V, sizeof(double) * N * ((size_t)2 * nb + 6 * k) + 8 * (3 * k + 8));
    SmallProb &q = hp[i];
    q = SmallProb{};
    q.a.astr = p.astr;
    q.a.bstr = p.bstr;
    q.a.na = p.na;
    q.a.nb = p.nb;
    q.a.hii = p.hii;
    q.a.A = p.A;
    q.a.B = p.B;
    q.a.val_sa = p.A.val_s;
    q.a.val_da = p.A.val_d;
    q.a.val_sb = p.B.val_s;
    q.a.val_db = p.B.val_d;
    q.a.Jb = p.Jb;
    q.a.Ja = p.Ja;
    q.a.Kp = p.Kp;
    q.a.npair = p.npair;
    q.N = (uint32_t)N;
    q.norb = p.norb;
    q.V = w;
    q.HV = q.V + N * nb;
    q.X = q.HV + N * nb;
    q.HX = q.X + N * 2 * k;
    q.T = q.HX + N * 2 * k;
    q.U = q.T + N * k;
    q.out = q.U + N * k;
    q.Xout = (X && X[i]) ? (double *)workspace(p, WS_C64, sizeof(double) * N * k) : nullptr;
  }
  SmallProb *dp = (SmallProb *)tmp_alloc(&c, sizeof(SmallProb) * count);
  SBDGB_CUDA(cudaMemcpyAsync(dp, hp.data(), sizeof(SmallProb) * count, cudaMemcpyHostToDevice, s));
  SmallOpts so{k, nb, std::max(1, o.max_it) * nb, o.eps};
  const size_t smem = sizeof(Smem) + 8 * kBMaxNb * kBMaxNb + 8;
  SBDGB_CUDA(cudaFuncSetAttribute(k_batch_davidson, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  k_batch_davidson<<<count, kBT, smem, s>>>(dp, so);
  count_launch(&c);
  SBDGB_CUDA(cudaGetLastError());
  std::vector<double> out(3 * k + 8);
  for (int i = 0; i < count; ++i) {
    SBDGB_CUDA(cudaMemcpyAsync(out.data(), hp[i].out, sizeof(double) * (2 * k + 4), cudaMemcpyDeviceToHost, s));
    if (hp[i].Xout) SBDGB_CUDA(cudaMemcpyAsync(X[i], hp[i].Xout, sizeof(double) * hp[i].N * k, cudaMemcpyDeviceToHost, s));
    SBDGB_CUDA(cudaStreamSynchronize(s));
    for (int q = 0; q < k; ++q) E[(size_t)i * k + q] = out[q];
    if (reps) {
      sbdgb_report &r = reps[i];
      r = sbdgb_report{};
      for (int q = 0; q < k && q < 16; ++q) r.resid[q] = out[k + q];
      r.iterations = (int)out[2 * k];
      r.sigma_calls = r.sigma_fp64 = (int)out[2 * k + 1];
      r.converged = (int)out[2 * k + 2];
      r.restarts = (int)out[2 * k + 3];
    }
  }
  tmp_free(&c, dp);
  const double secs = std::chrono::duration<double>(clock::now() - t0).count();
  if (reps)
    for (int i = 0; i < count; ++i) reps[i].seconds = secs;
}

}  // namespace sbdgb

extern "C" int sbdgb_batch_davidson(sbdgb_ctx *ctx, sbdgb_problem **problems, int count,
                                    const sbdgb_davidson_opts *o, double *E, sbdgb_report *reps, double **X) {
  if (!ctx || (count > 0 && (!problems || !E)) || !o) return SBDGB_E_INPUT;
  sbdgb::Ctx &c = ctx->c;
  try {
    SBDGB_CUDA(cudaSetDevice(c.device));
    std::vector<sbdgb::Problem *> ps(count);
    for (int i = 0; i < count; ++i) {
      SBDGB_REQUIRE(problems[i] != nullptr, SBDGB_E_INPUT, "null problem in batch");
      ps[i] = &problems[i]->p;
    }
    sbdgb::batch_davidson(c, ps.data(), count, *o, E, reps, X);
    c.last_error.clear();
    return SBDGB_OK;
  } catch (const sbdgb::Error &e) {
    c.last_error = e.what();
    return e.status;
  } catch (const std::exception &e) {
    c.last_error = e.what();
    return SBDGB_E_INPUT;
  }
}
