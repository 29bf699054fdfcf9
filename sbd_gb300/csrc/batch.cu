// Many small Davidson solves advanced in lock step: every step of the solver
// is one kernel launch over ALL problems of the batch, and one whole Davidson
// iteration (twelve launches) is captured once in a CUDA graph and replayed,
// so thousands of small problems cost a few graph launches per iteration
// instead of tens of launches and host synchronisations per problem.
//
// The algorithm is the device solver's (davidson.cu, the reference's
// chemistry/tpb/davidson.h:707-970 generalised to nroots): lowest-diagonal
// start vectors with a deterministic perturbation, Olsen-corrected diagonal
// preconditioner with the reference's 1e-12 guard, classical Gram-Schmidt
// (two passes) with coefficient-space dropping, thick restart on the lowest
// 2k Ritz vectors and the previous step's Ritz vectors, convergence on every
// residual norm below eps.  Each problem stops on its own; its blocks then
// return at once.
//
// Work decomposition:
//   - element work runs on chunks of kCH consecutive elements of one problem;
//     the chunks of every problem form one grid.  Kernels that leave partial
//     sums (dots, residuals) take one 256-thread block per chunk; the others
//     (sigma, projections, restart and correction updates) take kSubPer
//     blocks per chunk, so that the last few problems still fill the GPU;
//   - dot products leave one partial per chunk (no atomics) that a
//     per-problem warp sums in chunk order, so results are deterministic;
//   - the projected eigenproblem (n <= 32) is a parallel-order Jacobi by one
//     warp per problem, which also does the small coefficient-space work;
//   - sigma is the fused per-element form (diagonal, alpha pairs of the row,
//     alpha x beta singles, beta pairs of the column) for up to 8 vectors at
//     once, sharing the index, value and phase work between the vectors; the
//     (P|Q) table sits in shared memory when it fits.
//
// Mixed form (precision MIXED): FP64 arithmetic runs at 1/64 of the FP32 rate
// on this GPU and the FP64 sigma above keeps the FP64 pipe ~97% busy, so the
// mixed form runs the same iteration first on FP32 vectors (FP32 sigma from
// FP32 table values, FP32 vector algebra; partial sums, projected matrix,
// Rayleigh-Ritz and control stay FP64) until every residual is below
// kMixedRel * |theta|, then polishes in FP64 from the lowest 2k Ritz vectors
// of that phase (at most 8).  The FP64 phase applies the full tolerance, so
// the energies and vectors are those of the FP64 solver; the FP32 phase only
// removes FP64 iterations (about 60% of the FP64 sigma products on the
// norb-12 batch).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <type_traits>

#include "common.cuh"
#include "sigma_dev.cuh"

namespace sbdgb {

namespace {

using namespace sdev;

constexpr int kNB = 32;    // subspace cap of the batched solver
constexpr int kK = 8;      // roots
constexpr int kR = 3 * kK; // restart basis: 2k Ritz vectors and k previous directions
constexpr int kCH = 4096;  // elements per chunk (the unit of the partial sums)
constexpr int kSub = 512;  // elements per block of the kernels without partial sums
constexpr int kSubPer = kCH / kSub;
constexpr int kT = 256;    // threads per element block
constexpr int kStepLaunches = 12;
constexpr double kMixedRel = 5e-7;  // FP32 phase: residual below this times |theta|
constexpr size_t kKpSmem = 48 * 1024;  // largest (P|Q) table staged in shared memory by sigma

struct Chunk {
  uint32_t prob, e0, e1;
};

struct BProb {
  Args<double> a;  // strings, tables, integrals, diagonal (C, CT, S unused)
  Args<float> af;  // the same with FP32 table values (mixed form)
  uint32_t N;
  int norb, max_nb, max_steps;
  double *V, *HV, *T, *U;  // nb, nb, k, k columns at stride N
  float *Vf, *HVf, *Tf, *Uf;  // FP32 phase: the same shapes, in the first half of the region
  uint32_t c0, c1;         // chunk range of the problem
};

// Control state of one problem (device).
struct BState {
  int active, converged, iter, sigma_calls, restarts;
  int iter32, sigma32;  // FP32-phase iterations and sigma products (mixed form)
  int nv, kk, kc, nvprev, kprev, restart, nv_old, m, nt, from, to;
  int roots[kK];
  double th[kK], res[kK], eo[kK], n0[kK];
  double A[kNB * kNB];     // projected matrix, ld kNB (its symmetric part is used)
  double c[kNB * 2 * kK];  // coefficients of the lowest kc = min(2k, nv) Ritz vectors (ld nv)
  double cprev[kNB * kK];  // previous step's Ritz coefficients (nvprev x kprev)
  double Q[kNB * kR];      // restart basis in coefficient space (nv_old x m, ld nv_old)
  double G[kNB * kK];      // V^T T (nv x nt, ld nv)
  double M[kK * kK];       // orthonormal combinations of the corrections (nt x kept, ld nt)
};

struct BCommon {
  const BProb *P;
  BState *S;
  const Chunk *ch;
  double *part;  // per-chunk partial sums, pstride doubles each
  int pstride;
  int k;
  double eps;      // convergence: every residual below max(eps, eps_rel * |theta|)
  double eps_rel;
  int step_cap;    // iteration cap of the phase (0: the problem's max_steps)
  int kp_smem;     // sigma reads (P|Q) from shared memory
};

template <typename T>
struct Buf {
  T *V, *HV, *T_, *U;
};
template <typename T>
__device__ __forceinline__ Buf<T> buf(const BProb &P) {
  if constexpr (std::is_same<T, float>::value)
    return Buf<float>{P.Vf, P.HVf, P.Tf, P.Uf};
  else
    return Buf<double>{P.V, P.HV, P.T, P.U};
}
template <typename T>
__device__ __forceinline__ const Args<T> &args_of(const BProb &P) {
  if constexpr (std::is_same<T, float>::value)
    return P.af;
  else
    return P.a;
}
__device__ __forceinline__ float fmx(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double fmx(double a, double b, double c) { return fma(a, b, c); }

// ---- block and warp primitives ----------------------------------------------------

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Sums NV <= 32 per-thread values over the block into out[0, NV).
template <int NV>
__device__ void block_reduce(const double (&v)[NV], double (*red)[32], double *out) {
  static_assert(NV <= 32, "at most 32 values");
  __syncthreads();
#pragma unroll
  for (int i = 0; i < NV; ++i) {
    const double x = warp_sum(v[i]);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5][i] = x;
  }
  __syncthreads();
  if (threadIdx.x < NV) {
    double t = 0.0;
    for (int w = 0; w < kT / 32; ++w) t += red[w][threadIdx.x];
    out[threadIdx.x] = t;
  }
  __syncthreads();
}

// out[i + ldo * j] = L_i . R_j over the elements [e0, e1), columns at stride N
// (per-thread sums in the storage precision, block sums in FP64).
template <typename T>
__device__ void chunk_dots(const T *__restrict__ L, int nl, const T *__restrict__ R, int nr, uint32_t N,
                           uint32_t e0, uint32_t e1, double *out, int ldo, double (*red)[32]) {
  for (int j0 = 0; j0 < nr; j0 += 4)
    for (int i0 = 0; i0 < nl; i0 += 8) {
      const int mw = min(4, nr - j0), mv = min(8, nl - i0);
      T acc[8][4];
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = T(0);
      for (uint32_t e = e0 + threadIdx.x; e < e1; e += kT) {
        T w[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) w[j] = j < mw ? R[(size_t)(j0 + j) * N + e] : T(0);
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          if (i >= mv) break;
          const T v = L[(size_t)(i0 + i) * N + e];
#pragma unroll
          for (int j = 0; j < 4; ++j) acc[i][j] = fmx(v, w[j], acc[i][j]);
        }
      }
      __syncthreads();
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const double x = warp_sum((double)acc[i][j]);
          if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5][i * 4 + j] = x;
        }
      __syncthreads();
      if (threadIdx.x < 32) {
        const int i = threadIdx.x / 4, j = threadIdx.x % 4;
        if (i < mv && j < mw) {
          double t = 0.0;
          for (int w2 = 0; w2 < kT / 32; ++w2) t += red[w2][threadIdx.x];
          out[(i0 + i) + (size_t)ldo * (j0 + j)] = t;
        }
      }
    }
  __syncthreads();
}

// Sum over the problem's chunks (in chunk order) of partial value v.
__device__ __forceinline__ double chunk_total(const BCommon &g, const BProb &P, int v) {
  double t = 0.0;
  for (uint32_t c = P.c0; c < P.c1; ++c) t += g.part[(size_t)c * g.pstride + v];
  return t;
}

// The element range of this block in a kernel launched with kSubPer blocks per
// chunk; false when the range is empty (the last chunk of a problem).
__device__ __forceinline__ bool sub_range(const BCommon &g, Chunk &ch, uint32_t &e0, uint32_t &e1) {
  ch = g.ch[blockIdx.x / kSubPer];
  e0 = ch.e0 + (blockIdx.x % kSubPer) * kSub;
  e1 = min(ch.e1, e0 + kSub);
  return e0 < e1;
}

// Symmetric eigenproblem of the n x n leading block of A (ld kNB, symmetric
// part) by one warp: eigenvalues ascending in E, eigenvectors in the columns
// of Wv (ld kNB).  Aw, Wv, E: shared.
//
// Parallel-order Jacobi: each sweep is n' - 1 rounds (n' = n rounded up to
// even) of the round-robin pairing, and the n'/2 rotations of a round act on
// disjoint index pairs, so their parameters are computed by n'/2 lanes at once
// and applied together (A <- J^T A J zeroes every pair of the round).  FP64
// division and square root dominate a rotation on this GPU; the parallel
// order takes them once per round instead of once per pair.
__device__ void warp_eig(int n, const double *A, double *Aw, double *Wv, double *E) {
  __shared__ double rc[kNB / 2], rs[kNB / 2];
  __shared__ int rp[kNB / 2], rq[kNB / 2];
  const int l = threadIdx.x & 31;
  for (int t = l; t < kNB * kNB; t += 32) {
    const int i = t % kNB, j = t / kNB;
    Aw[t] = (i < n && j < n) ? 0.5 * (A[i + kNB * j] + A[j + kNB * i]) : 0.0;
    Wv[t] = (i == j) ? 1.0 : 0.0;
  }
  __syncwarp();
  const int n2 = (n + 1) & ~1, np = n2 / 2;
  // position -> index in round r of the circle method (position 0 fixed)
  auto idx = [&](int pos, int r) { return pos == 0 ? 0 : 1 + (pos - 1 + r) % (n2 - 1); };
  for (int sweep = 0; sweep < 60 && n > 1; ++sweep) {
    double off = 0.0, dg = 0.0;
    if (l < n)
      for (int j = 0; j < n; ++j) {
        const double x = Aw[l + kNB * j];
        if (l == j) dg += x * x; else off += x * x;
      }
    off = warp_sum(off);
    dg = warp_sum(dg);
    if (off <= 1e-30 * (dg + 1e-300)) break;
    for (int r = 0; r < n2 - 1; ++r) {
      if (l < np) {
        const int a = idx(l, r), b = idx(n2 - 1 - l, r);
        const int p = min(a, b), q = max(a, b);
        double c = 1.0, sn = 0.0;
        if (q < n) {  // q == n is the padding index of odd n
          const double apq = Aw[p + kNB * q];
          if (fabs(apq) >= 1e-300) {
            const double theta = (Aw[q + kNB * q] - Aw[p + kNB * p]) / (2.0 * apq);
            const double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
            c = 1.0 / sqrt(t * t + 1.0);
            sn = t * c;
          }
        }
        rp[l] = p;
        rq[l] = q;
        rc[l] = c;
        rs[l] = sn;
      }
      __syncwarp();
      if (l < n)  // columns p, q of every pair: row l
        for (int i = 0; i < np; ++i) {
          const int p = rp[i], q = rq[i];
          if (q >= n || rs[i] == 0.0) continue;
          const double c = rc[i], sn = rs[i];
          const double akp = Aw[l + kNB * p], akq = Aw[l + kNB * q];
          Aw[l + kNB * p] = c * akp - sn * akq;
          Aw[l + kNB * q] = sn * akp + c * akq;
        }
      __syncwarp();
      if (l < n)  // rows p, q of every pair: column l; and the eigenvectors: row l
        for (int i = 0; i < np; ++i) {
          const int p = rp[i], q = rq[i];
          if (q >= n || rs[i] == 0.0) continue;
          const double c = rc[i], sn = rs[i];
          const double apk = Aw[p + kNB * l], aqk = Aw[q + kNB * l];
          Aw[p + kNB * l] = c * apk - sn * aqk;
          Aw[q + kNB * l] = sn * apk + c * aqk;
          const double vkp = Wv[l + kNB * p], vkq = Wv[l + kNB * q];
          Wv[l + kNB * p] = c * vkp - sn * vkq;
          Wv[l + kNB * q] = sn * vkp + c * vkq;
        }
      __syncwarp();
    }
  }
  if (l == 0) {  // ascending order (selection sort), permuting the eigenvector columns
    for (int i = 0; i < n; ++i) E[i] = Aw[i + kNB * i];
    for (int i = 0; i < n; ++i) {
      int b = i;
      for (int j = i + 1; j < n; ++j)
        if (E[j] < E[b]) b = j;
      if (b != i) {
        const double e = E[i];
        E[i] = E[b];
        E[b] = e;
        for (int r = 0; r < n; ++r) {
          const double x = Wv[r + kNB * i];
          Wv[r + kNB * i] = Wv[r + kNB * b];
          Wv[r + kNB * b] = x;
        }
      }
    }
  }
  __syncwarp();
}

// ---- sigma ---------------------------------------------------------------------------

// sigma of NV vectors (columns of x at stride N) at element (ia, ib), fused
// form, in the storage precision T (table values of that precision).
template <int NV, typename Wd, typename T>
__device__ __forceinline__ void sigma_element_mv(const Args<T> &a, const T *__restrict__ Kp, const T *__restrict__ x,
                                                 uint32_t N, uint32_t ia, uint32_t ib, T (&acc)[NV]) {
  const uint32_t nb = a.nb, e = ia * nb + ib;
  const T h = (T)__ldg(a.hii + e);
#pragma unroll
  for (int n = 0; n < NV; ++n) acc[n] = h * __ldg(x + (size_t)n * N + e);
  const Wd beta = word<Wd>(a.bstr, ib);
  // alpha singles and doubles of row ia, this column
  for (uint32_t p = __ldg(a.A.off_s + ia), p1 = __ldg(a.A.off_s + ia + 1); p < p1; ++p) {
    const uint32_t ja = __ldg(a.A.ket_s + p), code = __ldg(a.A.code_s + p);
    const T v = __ldg(a.val_sa + p) + __ldg(a.Jb + ((code >> 16) & 0x7fffu) * nb + ib);
    const T sv = flip(v, parity(beta & word<Wd>(a.A.mask_s, p)) ^ (code >> 31));
    const uint32_t off = ja * nb + ib;
#pragma unroll
    for (int n = 0; n < NV; ++n) acc[n] = fmx(sv, __ldg(x + (size_t)n * N + off), acc[n]);
  }
  for (uint32_t p = __ldg(a.A.off_d + ia), p1 = __ldg(a.A.off_d + ia + 1); p < p1; ++p) {
    const uint32_t off = __ldg(a.A.ket_d + p) * nb + ib;
    const T sv = flip(__ldg(a.val_da + p), parity(beta & word<Wd>(a.A.mask_d, p)));
#pragma unroll
    for (int n = 0; n < NV; ++n) acc[n] = fmx(sv, __ldg(x + (size_t)n * N + off), acc[n]);
  }
  // alpha x beta singles: the beta singles of this column outside (their
  // table entries are read once per thread), the alpha singles of the row
  // inside (the same entries for the threads of one row: broadcast loads);
  // Kp is the (P|Q) table, in shared memory when it fits
  const uint32_t q0 = __ldg(a.B.off_s + ib), q1 = __ldg(a.B.off_s + ib + 1);
  const uint32_t pa0 = __ldg(a.A.off_s + ia), pa1 = __ldg(a.A.off_s + ia + 1);
  for (uint32_t q = q0; q < q1; ++q) {
    const uint32_t jb = __ldg(a.B.ket_s + q), cb = __ldg(a.B.code_s + q);
    const Wd mb = word<Wd>(a.B.mask_s, q);
    const uint32_t kb = (cb >> 16) & 0x7fffu, sb = cb >> 31;
    for (uint32_t p = pa0; p < pa1; ++p) {
      const uint32_t ja = __ldg(a.A.ket_s + p), ca = __ldg(a.A.code_s + p);
      const uint32_t ph =
          (parity(beta & word<Wd>(a.A.mask_s, p)) ^ parity(word<Wd>(a.astr, ja) & mb) ^ (ca >> 31) ^ sb) & 1u;
      const T kv = flip(Kp[((ca >> 16) & 0x7fffu) * a.npair + kb], ph);
      const uint32_t off = ja * nb + jb;
#pragma unroll
      for (int n = 0; n < NV; ++n) acc[n] = fmx(kv, __ldg(x + (size_t)n * N + off), acc[n]);
    }
  }
  // beta singles and doubles of column ib, this row
  const Wd arow = word<Wd>(a.astr, ia);
  const uint32_t rowoff = ia * nb;
  for (uint32_t q = q0; q < q1; ++q) {
    const uint32_t jb = __ldg(a.B.ket_s + q), cb = __ldg(a.B.code_s + q);
    const T sv = flip(__ldg(a.val_sb + q) + __ldg(a.Ja + (size_t)((cb >> 16) & 0x7fffu) * a.na + ia),
                      parity(arow & word<Wd>(a.B.mask_s, q)) ^ (cb >> 31));
#pragma unroll
    for (int n = 0; n < NV; ++n) acc[n] = fmx(sv, __ldg(x + (size_t)n * N + rowoff + jb), acc[n]);
  }
  for (uint32_t q = __ldg(a.B.off_d + ib), q1d = __ldg(a.B.off_d + ib + 1); q < q1d; ++q) {
    const uint32_t jb = __ldg(a.B.ket_d + q);
    const T sv = flip(__ldg(a.val_db + q), parity(arow & word<Wd>(a.B.mask_d, q)));
#pragma unroll
    for (int n = 0; n < NV; ++n) acc[n] = fmx(sv, __ldg(x + (size_t)n * N + rowoff + jb), acc[n]);
  }
}

template <int NV, typename Wd, typename T>
__device__ void chunk_sigma(const BProb &P, const T *Kp, const T *x, T *y, uint32_t e0, uint32_t e1) {
  const Args<T> &a = args_of<T>(P);
  const uint32_t nb = a.nb;
  for (uint32_t e = e0 + threadIdx.x; e < e1; e += kT) {
    T acc[NV];
    sigma_element_mv<NV, Wd, T>(a, Kp, x, P.N, e / nb, e % nb, acc);
#pragma unroll
    for (int n = 0; n < NV; ++n) y[(size_t)n * P.N + e] = acc[n];
  }
}

template <typename Wd, typename T>
__device__ void chunk_sigma_any(const BProb &P, int nvec, const T *Kp, const T *x, T *y, uint32_t e0, uint32_t e1) {
  switch (nvec) {
    case 1: chunk_sigma<1, Wd, T>(P, Kp, x, y, e0, e1); break;
    case 2: chunk_sigma<2, Wd, T>(P, Kp, x, y, e0, e1); break;
    case 3: chunk_sigma<3, Wd, T>(P, Kp, x, y, e0, e1); break;
    case 4: chunk_sigma<4, Wd, T>(P, Kp, x, y, e0, e1); break;
    case 5: chunk_sigma<5, Wd, T>(P, Kp, x, y, e0, e1); break;
    case 6: chunk_sigma<6, Wd, T>(P, Kp, x, y, e0, e1); break;
    case 7: chunk_sigma<7, Wd, T>(P, Kp, x, y, e0, e1); break;
    default: chunk_sigma<8, Wd, T>(P, Kp, x, y, e0, e1); break;
  }
}

// ---- kernels ---------------------------------------------------------------------------

// Start vectors (one block per problem): unit vectors on the k lowest diagonal
// entries (ties by index) plus a deterministic splitmix64 component of total
// size 1e-3, in T; the state is set for the first orthonormalisation.
template <typename T>
__global__ void __launch_bounds__(kT) k_b_init(BCommon g) {
  __shared__ double dv[kT / 32];
  __shared__ unsigned long long di[kT / 32], pos[kK];
  const BProb &P = g.P[blockIdx.x];
  BState &S = g.S[blockIdx.x];
  T *Tb = buf<T>(P).T_;
  const uint32_t N = P.N;
  const int k = g.k;
  for (int q = 0; q < k; ++q) {
    double best = INFINITY;
    unsigned long long bi = ~0ull;
    for (uint32_t e = threadIdx.x; e < N; e += kT) {
      bool skip = false;
      for (int r = 0; r < q; ++r) skip |= (pos[r] == e);
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
      dv[threadIdx.x >> 5] = best;
      di[threadIdx.x >> 5] = bi;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      double b = INFINITY;
      unsigned long long ix = ~0ull;
      for (int w = 0; w < kT / 32; ++w)
        if (dv[w] < b || (dv[w] == b && di[w] < ix)) {
          b = dv[w];
          ix = di[w];
        }
      pos[q] = ix;
    }
    __syncthreads();
  }
  const double amp = 1e-3 * sqrt(3.0 / (double)N);
  for (uint32_t e = threadIdx.x; e < N; e += kT)
    for (int q = 0; q < k; ++q) {
      uint64_t z = (uint64_t)e * 0x9E3779B97F4A7C15ull + 0x5BD1E995ull * (uint64_t)(q + 1);
      z ^= z >> 30;
      z *= 0xBF58476D1CE4E5B9ull;
      z ^= z >> 27;
      z *= 0x94D049BB133111EBull;
      z ^= z >> 31;
      Tb[(size_t)q * N + e] =
          (T)((e == pos[q] ? 1.0 : 0.0) + amp * ((double)(z >> 11) * (2.0 / 9007199254740992.0) - 1.0));
    }
  if (threadIdx.x == 0) {
    S.active = 1;
    S.converged = S.iter = S.sigma_calls = S.restarts = 0;
    S.iter32 = S.sigma32 = 0;
    S.nv = S.kk = S.kc = S.nvprev = S.kprev = S.restart = S.nv_old = S.m = S.from = S.to = 0;
    S.nt = k;
    for (int q = 0; q < kK; ++q) {
      S.roots[q] = q;
      S.th[q] = S.res[q] = S.eo[q] = S.n0[q] = 0.0;
    }
  }
}

// Mixed form, between the phases (one thread per problem): the FP32 phase's
// counters are kept aside and the state is set to orthonormalise the seed
// vectors (the lowest kc Ritz vectors of the FP32 phase, at most 8, written to
// the FP64 correction block by k_b_ritz) for the FP64 phase.
__global__ void k_b_seed_state(BCommon g, int count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const BProb &P = g.P[i];
  BState &S = g.S[i];
  S.iter32 = S.iter;
  S.sigma32 = S.sigma_calls;
  S.active = 1;
  S.converged = S.iter = S.sigma_calls = S.restarts = 0;
  S.nt = min(min(S.kc, P.max_nb), kK);
  S.nv = S.kk = S.kc = S.nvprev = S.kprev = S.restart = S.nv_old = S.m = S.from = S.to = 0;
  for (int q = 0; q < kK; ++q) {
    S.roots[q] = q;
    S.th[q] = S.res[q] = S.eo[q] = S.n0[q] = 0.0;
  }
}

// Partial dot products of one chunk.  mode 0: V[0, to)^T HV[from, to) (the new
// columns of the projected matrix); mode 1: V[0, nv)^T T[0, nt) followed by the
// Gram matrix T^T T.
template <typename T>
__global__ void __launch_bounds__(kT) k_b_dots(BCommon g, int mode) {
  __shared__ double red[kT / 32][32];
  const Chunk ch = g.ch[blockIdx.x];
  const BState &S = g.S[ch.prob];
  if (!S.active) return;
  const BProb &P = g.P[ch.prob];
  const Buf<T> b = buf<T>(P);
  double *out = g.part + (size_t)blockIdx.x * g.pstride;
  if (mode == 0) {
    const int nl = S.to, nr = S.to - S.from;
    chunk_dots<T>(b.V, nl, b.HV + (size_t)S.from * P.N, nr, P.N, ch.e0, ch.e1, out, nl, red);
  } else {
    const int nl = S.nv, nr = S.nt;
    chunk_dots<T>(b.V, nl, b.T_, nr, P.N, ch.e0, ch.e1, out, nl, red);
    chunk_dots<T>(b.T_, nr, b.T_, nr, P.N, ch.e0, ch.e1, out + nl * nr, nr, red);
  }
}

// Rayleigh-Ritz (one warp per problem): the new columns of the projected
// matrix from the mode-0 partials, then its eigenpairs; the coefficients of
// the lowest kc = min(2k, nv) Ritz vectors are kept.
__global__ void __launch_bounds__(32) k_b_rr(BCommon g) {
  __shared__ double Aw[kNB * kNB], Wv[kNB * kNB], E[kNB];
  const BProb &P = g.P[blockIdx.x];
  BState &S = g.S[blockIdx.x];
  if (!S.active) return;
  const int l = threadIdx.x, from = S.from, to = S.to, nr = to - from;
  for (int v = l; v < to * nr; v += 32) {
    const double t = chunk_total(g, P, v);
    const int i = v % to, j = from + v / to;
    S.A[i + kNB * j] = t;
    if (i < from) S.A[j + kNB * i] = t;
  }
  __syncwarp();
  const int nv = to, kk = min(g.k, nv), kc = min(2 * g.k, nv);
  warp_eig(nv, S.A, Aw, Wv, E);
  for (int t = l; t < nv * kc; t += 32) S.c[t] = Wv[(t % nv) + kNB * (t / nv)];
  if (l < kk) S.th[l] = E[l];
  if (l == 0) {
    S.nv = nv;
    S.kk = kk;
    S.kc = kc;
    S.iter++;
  }
}

// Residuals and Olsen-corrected preconditioned corrections of the kk Ritz
// pairs: T = r / (theta - d), U = x / (theta - d); partials of |r|^2, x.T, x.U.
template <typename T>
__global__ void __launch_bounds__(kT) k_b_combine(BCommon g) {
  __shared__ double red[kT / 32][32];
  __shared__ T cs[kNB * kK], th[kK];
  const Chunk ch = g.ch[blockIdx.x];
  const BState &S = g.S[ch.prob];
  if (!S.active) return;
  const BProb &P = g.P[ch.prob];
  const Buf<T> b = buf<T>(P);
  const int nv = S.nv, kk = S.kk;
  const uint32_t N = P.N;
  for (int t = threadIdx.x; t < nv * kk; t += kT) cs[t] = (T)S.c[t];
  if (threadIdx.x < kk) th[threadIdx.x] = (T)S.th[threadIdx.x];
  __syncthreads();
  T acc[3 * kK];
#pragma unroll
  for (int i = 0; i < 3 * kK; ++i) acc[i] = T(0);
  for (uint32_t e = ch.e0 + threadIdx.x; e < ch.e1; e += kT) {
    T xv[kK], hv[kK];
#pragma unroll
    for (int q = 0; q < kK; ++q) xv[q] = hv[q] = T(0);
    for (int j = 0; j < nv; ++j) {
      const T vj = b.V[(size_t)j * N + e], hj = b.HV[(size_t)j * N + e];
#pragma unroll
      for (int q = 0; q < kK; ++q)
        if (q < kk) {
          xv[q] = fmx(vj, cs[j + nv * q], xv[q]);
          hv[q] = fmx(hj, cs[j + nv * q], hv[q]);
        }
    }
    const T d = (T)P.a.hii[e];
#pragma unroll
    for (int q = 0; q < kK; ++q)
      if (q < kk) {
        const T r = hv[q] - th[q] * xv[q];
        T den = th[q] - d;
        if (fabs(den) <= T(1.0e-12)) den -= T(1.0e-12);
        const T t = r / den, u = xv[q] / den;
        b.T_[(size_t)q * N + e] = t;
        b.U[(size_t)q * N + e] = u;
        acc[q] = fmx(r, r, acc[q]);
        acc[kK + q] = fmx(xv[q], t, acc[kK + q]);
        acc[2 * kK + q] = fmx(xv[q], u, acc[2 * kK + q]);
      }
  }
  double accd[3 * kK];
#pragma unroll
  for (int i = 0; i < 3 * kK; ++i) accd[i] = (double)acc[i];
  block_reduce<3 * kK>(accd, red, g.part + (size_t)blockIdx.x * g.pstride);
}

// Control after the residuals (one warp per problem): residual norms, Olsen
// coefficients, convergence, and the thick restart in coefficient space.
__global__ void __launch_bounds__(32) k_b_ctl(BCommon g) {
  __shared__ double sums[3 * kK];
  __shared__ double Aw[kNB * kR];
  __shared__ int flag[2];
  const BProb &P = g.P[blockIdx.x];
  BState &S = g.S[blockIdx.x];
  if (!S.active) return;
  const int l = threadIdx.x, kk = S.kk, nv = S.nv;
  if (l < 3 * kK) sums[l] = chunk_total(g, P, l);
  __syncwarp();
  if (l == 0) {
    int nnew = 0;
    bool conv = kk == g.k;
    for (int q = 0; q < kk; ++q) {
      const double a1 = sums[kK + q], a2 = sums[2 * kK + q];
      S.res[q] = sqrt(fmax(0.0, sums[q]));
      S.eo[q] = (a2 != 0.0 && isfinite(a1 / a2)) ? a1 / a2 : 0.0;
      const bool ok = S.res[q] < fmax(g.eps, g.eps_rel * fabs(S.th[q]));
      conv = conv && ok;
      nnew += !ok;
    }
    S.restart = 0;
    flag[0] = 0;
    const int cap = g.step_cap > 0 ? min(g.step_cap, P.max_steps) : P.max_steps;
    if (conv || S.iter >= cap) {
      S.converged = conv;
      S.active = 0;
      flag[0] = 1;
    } else if (nv + nnew > P.max_nb) {
      // orthonormal Q (nv x m) spanning the lowest 2k Ritz coefficient
      // vectors (room permitting) and the previous step's Ritz coefficients
      const int keep = max(kk, min(S.kc, P.max_nb - nnew));
      const int nkeep = max(0, min(S.kprev, P.max_nb - keep - nnew));
      int m = 0;
      for (int col = 0; col < keep + nkeep; ++col) {
        double v[kNB];
        for (int i = 0; i < nv; ++i)
          v[i] = col < keep ? S.c[i + nv * col] : (i < S.nvprev ? S.cprev[i + S.nvprev * (col - keep)] : 0.0);
        double n0 = 0.0;
        for (int i = 0; i < nv; ++i) n0 += v[i] * v[i];
        n0 = sqrt(n0);
        for (int pass = 0; pass < 2; ++pass)
          for (int j = 0; j < m; ++j) {
            double pr = 0.0;
            for (int i = 0; i < nv; ++i) pr += S.Q[i + nv * j] * v[i];
            for (int i = 0; i < nv; ++i) v[i] -= pr * S.Q[i + nv * j];
          }
        double nn = 0.0;
        for (int i = 0; i < nv; ++i) nn += v[i] * v[i];
        nn = sqrt(nn);
        if (!(nn > 1e-8 * n0)) continue;
        for (int i = 0; i < nv; ++i) S.Q[i + nv * m] = v[i] / nn;
        ++m;
      }
      S.m = m;
      S.restart = 1;
    }
    if (!flag[0]) {
      int nt = 0;
      for (int q = 0; q < kk; ++q)
        if (!(S.res[q] < fmax(g.eps, g.eps_rel * fabs(S.th[q])))) S.roots[nt++] = q;
      nt = min(nt, P.max_nb - (S.restart ? S.m : nv));
      if (nt <= 0) {  // no room for a new direction: the subspace is the whole space
        S.converged = 0;
        S.active = 0;
        S.restart = 0;
        flag[0] = 1;
      }
      S.nt = nt;
    }
    flag[1] = S.restart;
  }
  __syncwarp();
  if (flag[0]) return;
  if (flag[1]) {
    // A <- Q^T A Q, c <- Q^T c (lanes over the columns of Q; m <= 24)
    const int m = S.m;
    for (int b = l; b < m; b += 32)
      for (int j = 0; j < nv; ++j) {
        double aq = 0.0;
        for (int i = 0; i < nv; ++i) aq += 0.5 * (S.A[j + kNB * i] + S.A[i + kNB * j]) * S.Q[i + nv * b];
        Aw[j + kNB * b] = aq;
      }
    __syncwarp();
    double hn[kR], cn[kK];
    if (l < m) {
      for (int a2 = 0; a2 < m; ++a2) {
        double t = 0.0;
        for (int j = 0; j < nv; ++j) t += S.Q[j + nv * a2] * Aw[j + kNB * l];
        hn[a2] = t;
      }
      for (int q = 0; q < kk; ++q) {
        double t = 0.0;
        for (int i = 0; i < nv; ++i) t += S.Q[i + nv * l] * S.c[i + nv * q];
        cn[q] = t;
      }
    }
    __syncwarp();
    if (l < m) {
      for (int a2 = 0; a2 < m; ++a2) S.A[a2 + kNB * l] = hn[a2];
      for (int q = 0; q < kk; ++q) S.c[l + m * q] = cn[q];
    }
    __syncwarp();
    if (l == 0) {
      S.nv_old = nv;
      S.nv = m;
      S.kc = kk;  // only the kk Ritz coefficient vectors follow the restart
      S.restarts++;
    }
    __syncwarp();
  }
  const int nvn = flag[1] ? S.m : nv;
  for (int t = l; t < nvn * kk; t += 32) S.cprev[t] = S.c[t];
  if (l == 0) {
    S.nvprev = nvn;
    S.kprev = kk;
  }
}

// Element updates after the control step: the restart V <- V Q, HV <- HV Q
// (per element, in registers), then the Olsen update T - eo U of the
// unconverged roots, packed at the front of T.
template <typename T>
__global__ void __launch_bounds__(kT) k_b_apply(BCommon g) {
  __shared__ T Qs[kNB * kR], eo[kK];
  __shared__ int roots[kK];
  Chunk ch;
  uint32_t e0, e1;
  if (!sub_range(g, ch, e0, e1)) return;
  const BState &S = g.S[ch.prob];
  if (!S.active) return;
  const BProb &P = g.P[ch.prob];
  const Buf<T> bf = buf<T>(P);
  const uint32_t N = P.N;
  const int restart = S.restart, nvo = S.nv_old, m = S.m, nt = S.nt;
  if (restart)
    for (int t = threadIdx.x; t < nvo * m; t += kT) Qs[t] = (T)S.Q[t];
  if (threadIdx.x < kK) {
    eo[threadIdx.x] = (T)S.eo[threadIdx.x];
    roots[threadIdx.x] = S.roots[threadIdx.x];
  }
  __syncthreads();
  for (uint32_t e = e0 + threadIdx.x; e < e1; e += kT) {
    if (restart) {
      for (int pass = 0; pass < 2; ++pass) {
        T *B = pass == 0 ? bf.V : bf.HV;
        T vin[kNB];
#pragma unroll
        for (int j = 0; j < kNB; ++j) vin[j] = j < nvo ? B[(size_t)j * N + e] : T(0);
        for (int b = 0; b < m; ++b) {
          T y = T(0);
#pragma unroll
          for (int j = 0; j < kNB; ++j)
            if (j < nvo) y = fmx(vin[j], Qs[j + nvo * b], y);
          B[(size_t)b * N + e] = y;
        }
      }
    }
    T t[kK];
#pragma unroll
    for (int i = 0; i < kK; ++i)
      if (i < nt) {
        const int r = roots[i];
        t[i] = fmx(-eo[r], bf.U[(size_t)r * N + e], bf.T_[(size_t)r * N + e]);
      }
#pragma unroll
    for (int i = 0; i < kK; ++i)
      if (i < nt) bf.T_[(size_t)i * N + e] = t[i];
  }
}

// First Gram-Schmidt pass, control (one warp per problem): G = V^T T and the
// original correction norms.
__global__ void __launch_bounds__(32) k_b_gs1(BCommon g) {
  const BProb &P = g.P[blockIdx.x];
  BState &S = g.S[blockIdx.x];
  if (!S.active) return;
  const int nv = S.nv, nt = S.nt;
  for (int v = threadIdx.x; v < nv * nt; v += 32) S.G[v] = chunk_total(g, P, v);
  if ((int)threadIdx.x < nt) S.n0[threadIdx.x] = chunk_total(g, P, nv * nt + threadIdx.x * (nt + 1));
}

// T <- T - V G.
template <typename T>
__global__ void __launch_bounds__(kT) k_b_project(BCommon g) {
  __shared__ T Gs[kNB * kK];
  Chunk ch;
  uint32_t e0, e1;
  if (!sub_range(g, ch, e0, e1)) return;
  const BState &S = g.S[ch.prob];
  if (!S.active) return;
  const BProb &P = g.P[ch.prob];
  const Buf<T> bf = buf<T>(P);
  const uint32_t N = P.N;
  const int nv = S.nv, nt = S.nt;
  if (nv == 0) return;
  for (int t = threadIdx.x; t < nv * nt; t += kT) Gs[t] = (T)S.G[t];
  __syncthreads();
  for (uint32_t e = e0 + threadIdx.x; e < e1; e += kT) {
    T t[kK];
#pragma unroll
    for (int q = 0; q < kK; ++q) t[q] = q < nt ? bf.T_[(size_t)q * N + e] : T(0);
    for (int j = 0; j < nv; ++j) {
      const T vj = bf.V[(size_t)j * N + e];
#pragma unroll
      for (int q = 0; q < kK; ++q)
        if (q < nt) t[q] = fmx(-vj, Gs[j + nv * q], t[q]);
    }
#pragma unroll
    for (int q = 0; q < kK; ++q)
      if (q < nt) bf.T_[(size_t)q * N + e] = t[q];
  }
}

// Second Gram-Schmidt pass, control (one warp per problem): G = V^T T (the
// second projection, applied with the new columns), the Gram matrix of the
// projected block (T^T T - G^T G) and its coefficient-space Gram-Schmidt with
// dropping below 1e-8 of the original norm.
__global__ void __launch_bounds__(32) k_b_gs2(BCommon g) {
  __shared__ double Gm[kK * kK];
  const BProb &P = g.P[blockIdx.x];
  BState &S = g.S[blockIdx.x];
  if (!S.active) return;
  const int nv = S.nv, nt = S.nt, l = threadIdx.x;
  for (int v = l; v < nv * nt; v += 32) S.G[v] = chunk_total(g, P, v);
  for (int v = l; v < nt * nt; v += 32) Gm[v] = chunk_total(g, P, nv * nt + v);
  __syncwarp();
  for (int v = l; v < nt * nt; v += 32) {
    const int i = v % nt, j = v / nt;
    double s = Gm[v];
    for (int r = 0; r < nv; ++r) s -= S.G[r + nv * i] * S.G[r + nv * j];
    Gm[v] = s;
  }
  __syncwarp();
  if (l == 0) {
    int kept = 0;
    for (int q = 0; q < nt; ++q) {
      const double n0 = S.n0[q];
      if (!(n0 > 0.0) || !isfinite(n0)) continue;
      double v[kK];
      for (int i = 0; i < nt; ++i) v[i] = (i == q) ? 1.0 : 0.0;
      for (int pass = 0; pass < 2; ++pass)
        for (int u = 0; u < kept; ++u) {
          double pr = 0.0;
          for (int i = 0; i < nt; ++i)
            for (int j = 0; j < nt; ++j) pr += S.M[i + nt * u] * Gm[i + nt * j] * v[j];
          for (int i = 0; i < nt; ++i) v[i] -= pr * S.M[i + nt * u];
        }
      double nn = 0.0;
      for (int i = 0; i < nt; ++i)
        for (int j = 0; j < nt; ++j) nn += v[i] * Gm[i + nt * j] * v[j];
      if (!(nn > 1e-16 * n0)) continue;
      const double f = 1.0 / sqrt(nn);
      for (int i = 0; i < nt; ++i) S.M[i + nt * kept] = v[i] * f;
      ++kept;
    }
    if (kept == 0) {  // no new direction: the subspace is invariant
      S.active = 0;
      S.converged = 0;
    } else {
      S.from = nv;
      S.to = nv + kept;
      S.sigma_calls += kept;
    }
  }
}

// New basis columns V[nv + c] = (T - V G) M.
template <typename T>
__global__ void __launch_bounds__(kT) k_b_newcols(BCommon g) {
  __shared__ T Gs[kNB * kK], Ms[kK * kK];
  Chunk ch;
  uint32_t e0, e1;
  if (!sub_range(g, ch, e0, e1)) return;
  const BState &S = g.S[ch.prob];
  if (!S.active) return;
  const BProb &P = g.P[ch.prob];
  const Buf<T> bf = buf<T>(P);
  const uint32_t N = P.N;
  const int nv = S.nv, nt = S.nt, kept = S.to - S.from;
  for (int t = threadIdx.x; t < nv * nt; t += kT) Gs[t] = (T)S.G[t];
  for (int t = threadIdx.x; t < nt * kept; t += kT) Ms[t] = (T)S.M[t];
  __syncthreads();
  for (uint32_t e = e0 + threadIdx.x; e < e1; e += kT) {
    T t[kK];
#pragma unroll
    for (int q = 0; q < kK; ++q) t[q] = q < nt ? bf.T_[(size_t)q * N + e] : T(0);
    for (int j = 0; j < nv; ++j) {
      const T vj = bf.V[(size_t)j * N + e];
#pragma unroll
      for (int q = 0; q < kK; ++q)
        if (q < nt) t[q] = fmx(-vj, Gs[j + nv * q], t[q]);
    }
    for (int c = 0; c < kept; ++c) {
      T y = T(0);
#pragma unroll
      for (int q = 0; q < kK; ++q)
        if (q < nt) y = fmx(t[q], Ms[q + nt * c], y);
      bf.V[(size_t)(nv + c) * N + e] = y;
    }
  }
}

// HV[from, to) = H V[from, to).  With g.kp_smem the block first copies the
// problem's (P|Q) table into shared memory (launched with npair^2 elements of
// dynamic shared memory for the largest npair of the batch).
template <typename T>
__global__ void __launch_bounds__(kT) k_b_sigma(BCommon g) {
  extern __shared__ __align__(16) unsigned char kp_raw[];
  Chunk ch;
  uint32_t e0, e1;
  if (!sub_range(g, ch, e0, e1)) return;
  const BState &S = g.S[ch.prob];
  if (!S.active) return;
  const BProb &P = g.P[ch.prob];
  const Args<T> &a = args_of<T>(P);
  const T *Kp = a.Kp;
  if (g.kp_smem) {
    T *ks = reinterpret_cast<T *>(kp_raw);
    const int npp = a.npair * a.npair;
    for (int t = threadIdx.x; t < npp; t += kT) ks[t] = __ldg(a.Kp + t);
    __syncthreads();
    Kp = ks;
  }
  const Buf<T> bf = buf<T>(P);
  const int from = S.from, nvec = S.to - S.from;
  const T *x = bf.V + (size_t)from * P.N;
  T *y = bf.HV + (size_t)from * P.N;
  if (P.norb <= 32)
    chunk_sigma_any<uint32_t, T>(P, nvec, Kp, x, y, e0, e1);
  else
    chunk_sigma_any<unsigned long long, T>(P, nvec, Kp, x, y, e0, e1);
}

// Ritz vectors V c, in FP64, into the FP64 correction block (T, then U): the
// kk wanted ones (seed 0: the solver's output), or the lowest kc (seed 1: the
// start of the FP64 phase of the mixed form).  Every problem, stopped or not.
template <typename T>
__global__ void __launch_bounds__(kT) k_b_ritz(BCommon g, int seed) {
  __shared__ double cs[kNB * 2 * kK];
  Chunk ch;
  uint32_t e0, e1;
  if (!sub_range(g, ch, e0, e1)) return;
  const BState &S = g.S[ch.prob];
  const BProb &P = g.P[ch.prob];
  const T *V = buf<T>(P).V;
  const uint32_t N = P.N;
  const int nv = S.nv, nc = seed ? min(S.kc, kK) : S.kk;
  for (int t = threadIdx.x; t < nv * nc; t += kT) cs[t] = S.c[t];
  __syncthreads();
  for (uint32_t e = e0 + threadIdx.x; e < e1; e += kT) {
    double xv[kK];
#pragma unroll
    for (int q = 0; q < kK; ++q) xv[q] = 0.0;
    for (int j = 0; j < nv; ++j) {
      const double vj = (double)V[(size_t)j * N + e];
#pragma unroll
      for (int q = 0; q < kK; ++q)
        if (q < nc) xv[q] = fma(vj, cs[j + nv * q], xv[q]);
    }
#pragma unroll
    for (int q = 0; q < kK; ++q)
      if (q < nc) P.T[(size_t)q * N + e] = xv[q];
  }
}

// Number of problems still iterating (one block of 1024 threads).
__global__ void k_b_count(const BState *S, int count, int *out) {
  __shared__ int w[32];
  int n = 0;
  for (int i = threadIdx.x; i < count; i += blockDim.x) n += S[i].active;
  for (int o = 16; o > 0; o >>= 1) n += __shfl_xor_sync(0xffffffffu, n, o);
  if ((threadIdx.x & 31) == 0) w[threadIdx.x >> 5] = n;
  __syncthreads();
  if (threadIdx.x == 0) {
    int t = 0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += w[i];
    *out = t;
  }
}

// Results: k energies, k residuals, iterations, sigma calls, converged,
// restarts, FP64 sigma calls.
__global__ void k_b_results(const BState *S, int count, int k, double *out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const BState &s = S[i];
  double *o = out + (size_t)i * (2 * k + 5);
  for (int q = 0; q < k; ++q) {
    o[q] = q < s.kk ? s.th[q] : NAN;
    o[k + q] = q < s.kk ? s.res[q] : NAN;
  }
  o[2 * k + 0] = s.iter + s.iter32;
  o[2 * k + 1] = s.sigma_calls + s.sigma32;
  o[2 * k + 2] = s.converged;
  o[2 * k + 3] = s.restarts;
  o[2 * k + 4] = s.sigma_calls;
}

}  // namespace

// Solves every problem of the batch with the same options, all problems in
// lock step (precision FP64, or MIXED: an FP32 phase then the FP64 phase).
// Problems must belong to one context; tables and diagonals are built here if
// missing.  E: count x nroots energies; reps: count reports (may be null); X:
// count pointers to host buffers of nroots x N (entries may be null).
void batch_davidson(Ctx &c, Problem **ps, int count, const sbdgb_davidson_opts &o, double *E, sbdgb_report *reps,
                    double **X) {
  using clock = std::chrono::steady_clock;
  const auto t0 = clock::now();
  SBDGB_REQUIRE(count >= 0, SBDGB_E_INPUT, "negative batch size");
  if (count == 0) return;
  SBDGB_REQUIRE(o.nroots >= 1 && o.nroots <= kK, SBDGB_E_UNSUPPORTED, "the batched solver takes 1..8 roots");
  SBDGB_REQUIRE(o.precision == SBDGB_FP64 || o.precision == SBDGB_MIXED, SBDGB_E_INPUT, "unknown precision");
  SBDGB_REQUIRE(o.init == 1, SBDGB_E_UNSUPPORTED, "the batched solver starts on the lowest diagonal (init 1)");
  const bool mixed = o.precision == SBDGB_MIXED;
  cudaStream_t s = c.stream;
  const int k = o.nroots, nb = std::min(std::max(o.max_nb, 2 * k), kNB);
  size_t total = 0;
  for (int i = 0; i < count; ++i) {
    Problem &p = *ps[i];
    SBDGB_REQUIRE(p.ctx == &c, SBDGB_E_INPUT, "batch problems must belong to the context");
    SBDGB_REQUIRE(p.N >= (uint64_t)k, SBDGB_E_INPUT, "more roots than determinants");
    total += p.N;
  }
  // per problem: V, HV (nb columns each), T, U (k each) in FP64; the FP32
  // phase uses the same shapes in the first half of the region
  const size_t per_elem = (size_t)2 * nb + 2 * k;
  const size_t bytes = sizeof(double) * total * per_elem;
  SBDGB_REQUIRE(!c.budget || c.in_use + bytes <= c.budget, SBDGB_E_NOMEM,
                "HBM budget exceeded by the batched solver's vectors");
  for (int i = 0; i < count; ++i) {
    Problem &p = *ps[i];
    if (!p.tables) build_tables(p, s);
    if (!p.diag) build_diag(p, s);
    if (mixed) prepare_mixed(p, s);
  }
  std::vector<BProb> hp(count);
  std::vector<Chunk> chunks;
  double *arena = (double *)tmp_alloc(&c, bytes);
  size_t off = 0;
  for (int i = 0; i < count; ++i) {
    Problem &p = *ps[i];
    const size_t N = p.N;
    BProb &q = hp[i];
    q = BProb{};
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
    if (mixed) {
      q.af.astr = p.astr;
      q.af.bstr = p.bstr;
      q.af.na = p.na;
      q.af.nb = p.nb;
      q.af.hii = p.hii;
      q.af.A = p.A;
      q.af.B = p.B;
      q.af.val_sa = p.val_sf[0];
      q.af.val_da = p.val_df[0];
      q.af.val_sb = p.val_sf[1];
      q.af.val_db = p.val_df[1];
      q.af.Jb = p.Jbf;
      q.af.Ja = p.Jaf;
      q.af.Kp = p.Kpf;
      q.af.npair = p.npair;
    }
    q.N = (uint32_t)N;
    q.norb = p.norb;
    q.max_nb = (int)std::min<size_t>((size_t)nb, N);
    q.max_steps = std::max(1, o.max_it) * q.max_nb;
    q.V = arena + off;
    q.HV = q.V + N * nb;
    q.T = q.HV + N * nb;
    q.U = q.T + N * k;
    q.Vf = (float *)q.V;
    q.HVf = q.Vf + N * nb;
    q.Tf = q.HVf + N * nb;
    q.Uf = q.Tf + N * k;
    off += N * per_elem;
    q.c0 = (uint32_t)chunks.size();
    for (size_t e0 = 0; e0 < N; e0 += kCH)
      chunks.push_back(Chunk{(uint32_t)i, (uint32_t)e0, (uint32_t)std::min(N, e0 + kCH)});
    q.c1 = (uint32_t)chunks.size();
  }
  const int nch = (int)chunks.size(), nsub = nch * kSubPer;
  // (P|Q) in shared memory for sigma when the largest table of the batch fits
  // in kKpSmem bytes (norb <= 12 in FP64, <= 14 in FP32)
  size_t npp_max = 0;
  for (int i = 0; i < count; ++i) npp_max = std::max(npp_max, (size_t)ps[i]->npair * ps[i]->npair);
  const bool kp64 = sizeof(double) * npp_max <= kKpSmem, kp32 = sizeof(float) * npp_max <= kKpSmem;
  const int nseed = std::min(2 * k, kK);
  const int pstride = std::max({nb * k + k * k, nseed * nseed, 3 * kK});
  const int rstride = 2 * k + 5;
  const size_t nres = (size_t)count * rstride;
  const size_t meta = sizeof(BProb) * count + sizeof(BState) * count + sizeof(double) * ((size_t)nch * pstride + nres) +
                      sizeof(Chunk) * nch + 64;
  char *mb = nullptr;
  try {
    mb = (char *)tmp_alloc(&c, meta);
  } catch (...) {
    tmp_free(&c, arena);
    throw;
  }
  BProb *dP = (BProb *)mb;
  BState *dS = (BState *)(dP + count);
  double *dpart = (double *)(dS + count);
  double *dres = dpart + (size_t)nch * pstride;
  Chunk *dch = (Chunk *)(dres + nres);
  int *dcount = (int *)(((uintptr_t)(dch + nch) + 7) & ~(uintptr_t)7);
  cudaGraphExec_t exec = nullptr;
  try {
    SBDGB_CUDA(cudaMemcpyAsync(dP, hp.data(), sizeof(BProb) * count, cudaMemcpyHostToDevice, s));
    SBDGB_CUDA(cudaMemcpyAsync(dch, chunks.data(), sizeof(Chunk) * nch, cudaMemcpyHostToDevice, s));
    int *pin = (int *)pinned_buffer(&c);
    int max_steps = 0;
    for (const BProb &q : hp) max_steps = std::max(max_steps, q.max_steps);
    // One phase: orthonormalise the start block and take its sigma, then
    // iterate (one captured graph per Davidson iteration of every problem)
    // until no problem is active.
    auto run_phase = [&](auto tag, const BCommon &g, int steps) {
      using T = decltype(tag);
      auto ortho_sigma = [&] {
        k_b_dots<T><<<nch, kT, 0, s>>>(g, 1);
        k_b_gs1<<<count, 32, 0, s>>>(g);
        k_b_project<T><<<nsub, kT, 0, s>>>(g);
        k_b_dots<T><<<nch, kT, 0, s>>>(g, 1);
        k_b_gs2<<<count, 32, 0, s>>>(g);
        k_b_newcols<T><<<nsub, kT, 0, s>>>(g);
        k_b_sigma<T><<<nsub, kT, g.kp_smem ? sizeof(T) * npp_max : 0, s>>>(g);
      };
      auto iteration = [&] {
        k_b_dots<T><<<nch, kT, 0, s>>>(g, 0);
        k_b_rr<<<count, 32, 0, s>>>(g);
        k_b_combine<T><<<nch, kT, 0, s>>>(g);
        k_b_ctl<<<count, 32, 0, s>>>(g);
        k_b_apply<T><<<nsub, kT, 0, s>>>(g);
        ortho_sigma();
      };
      ortho_sigma();
      count_launch(&c, 7);
      SBDGB_CUDA(cudaGetLastError());
      // the legacy default stream cannot be captured: launch directly there
      if (s != nullptr && s != cudaStreamLegacy && s != cudaStreamPerThread) {
        cudaGraph_t graph = nullptr;
        SBDGB_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        iteration();
        SBDGB_CUDA(cudaStreamEndCapture(s, &graph));
        const cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        SBDGB_CUDA(ie);
      }
      for (int it = 0; it <= steps;) {
        const int per_check = it < 8 ? 4 : 2;
        for (int r = 0; r < per_check; ++r, ++it) {
          if (exec)
            SBDGB_CUDA(cudaGraphLaunch(exec, s));
          else
            iteration();
          count_launch(&c, kStepLaunches);
        }
        SBDGB_CUDA(cudaGetLastError());
        k_b_count<<<1, 1024, 0, s>>>(dS, count, dcount);
        count_launch(&c);
        SBDGB_CUDA(cudaMemcpyAsync(pin, dcount, sizeof(int), cudaMemcpyDeviceToHost, s));
        SBDGB_CUDA(cudaStreamSynchronize(s));
        if (pin[0] == 0) break;
      }
      if (exec) {
        cudaGraphExecDestroy(exec);
        exec = nullptr;
      }
    };
    const BCommon g64{dP, dS, dch, dpart, pstride, k, o.eps, 0.0, 0, kp64 ? 1 : 0};
    if (mixed) {
      // FP32 phase to a relative residual of kMixedRel (at most 4 max_nb
      // iterations), then the FP64 phase from its lowest Ritz vectors
      const BCommon g32{dP, dS, dch, dpart, pstride, k, o.eps, kMixedRel, 4 * nb, kp32 ? 1 : 0};
      k_b_init<float><<<count, kT, 0, s>>>(g32);
      count_launch(&c);
      run_phase(float{}, g32, 4 * nb);
      k_b_ritz<float><<<nsub, kT, 0, s>>>(g32, 1);
      k_b_seed_state<<<(count + 127) / 128, 128, 0, s>>>(g64, count);
      count_launch(&c, 2);
    } else {
      k_b_init<double><<<count, kT, 0, s>>>(g64);
      count_launch(&c);
    }
    run_phase(double{}, g64, max_steps);
    k_b_results<<<(count + 127) / 128, 128, 0, s>>>(dS, count, k, dres);
    count_launch(&c);
    if (X) {
      k_b_ritz<double><<<nsub, kT, 0, s>>>(g64, 0);
      count_launch(&c);
    }
    SBDGB_CUDA(cudaGetLastError());
    std::vector<double> out(nres);
    SBDGB_CUDA(cudaMemcpyAsync(out.data(), dres, sizeof(double) * nres, cudaMemcpyDeviceToHost, s));
    if (X)
      for (int i = 0; i < count; ++i)
        if (X[i]) SBDGB_CUDA(cudaMemcpyAsync(X[i], hp[i].T, sizeof(double) * hp[i].N * k, cudaMemcpyDeviceToHost, s));
    SBDGB_CUDA(cudaStreamSynchronize(s));
    const double secs = std::chrono::duration<double>(clock::now() - t0).count();
    for (int i = 0; i < count; ++i) {
      const double *r = out.data() + (size_t)i * rstride;
      for (int q = 0; q < k; ++q) E[(size_t)i * k + q] = r[q];
      if (reps) {
        sbdgb_report &rp = reps[i];
        rp = sbdgb_report{};
        for (int q = 0; q < k && q < 16; ++q) rp.resid[q] = r[k + q];
        rp.iterations = (int)r[2 * k];
        rp.sigma_calls = (int)r[2 * k + 1];
        rp.converged = (int)r[2 * k + 2];
        rp.restarts = (int)r[2 * k + 3];
        rp.sigma_fp64 = (int)r[2 * k + 4];
        rp.seconds = secs;
      }
    }
  } catch (...) {
    if (exec) cudaGraphExecDestroy(exec);
    tmp_free(&c, mb);
    tmp_free(&c, arena);
    throw;
  }
  tmp_free(&c, mb);
  tmp_free(&c, arena);
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
