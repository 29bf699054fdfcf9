// sigma = H*C for the tensor-product basis (replaces sbd::mult, TRADMODE CPU
// loop chemistry/tpb/mult.h:440-558, and the Thrust MultTPBThrust::run,
// chemistry/tpb/mult_thrust.h:1170-1580).
//
// Gather formulation without atomics, one FP64 FMA per nonzero, phases applied
// by flipping the sign bit (integer work only):
//
//   kernel A  rows = alpha strings, columns = beta strings, reads C[ja][ib]
//             sigma[ia][ib] = hii*C + sum_alpha-pairs +/- V * C[ja][ib]
//                                    + sum_alpha-singles sum_beta-singles +/- K * C[ja][jb]
//   kernel B  rows = beta strings, columns = alpha strings, reads C^T[jb][ia]
//             sigma[ia][ib] += sum_beta-pairs +/- V * C^T[jb][ia]
//
// A CTA owns TA rows x (32*CPT*WARPS) columns.  Every thread keeps its columns'
// opposite-spin strings and TA*CPT accumulators in registers; the pair list
// of a row is the same for all threads of the CTA, so its metadata are
// broadcast loads and the ket-row reads are coalesced along the contiguous
// index.  Grid order puts consecutive CTAs on the same column chunk so that
// the ket rows' column slab stays resident in L2.
#include <algorithm>

#include "common.cuh"

namespace sbdgb {

namespace {

constexpr int kThreads = 128;

__device__ __forceinline__ double flip(double x, uint32_t ph) {
  return __longlong_as_double(__double_as_longlong(x) ^ ((unsigned long long)ph << 63));
}
__device__ __forceinline__ float flipf(float x, uint32_t ph) {
  return __int_as_float(__float_as_int(x) ^ (int)(ph << 31));
}

// Same-spin excitations of rows r0 .. r0+TA-1 applied to this thread's CPT
// columns.  In: ket-major input rows (ld = ldin), Jo: opposite-spin Coulomb
// table [npair][ldj] for the single excitations.
template <int TA, int CPT>
__device__ __forceinline__ void same_spin_sweep(const SpinTables &T, const double *__restrict__ Jo, size_t ldj,
                                                const double *__restrict__ In, size_t ldin, uint32_t r0,
                                                uint32_t nrow, const uint32_t (&col)[CPT], const bool (&ok)[CPT],
                                                const uint64_t (&opp)[CPT], double (&acc)[TA][CPT]) {
#pragma unroll
  for (int r = 0; r < TA; ++r) {
    const uint32_t row = r0 + r;
    if (row < nrow) {
      const uint32_t p0 = __ldg(T.off_s + row), p1 = __ldg(T.off_s + row + 1);
      for (uint32_t p = p0; p < p1; ++p) {
        const uint32_t ket = __ldg(T.ket_s + p), code = __ldg(T.code_s + p);
        const double v = __ldg(T.val_s + p);
        const uint64_t m = __ldg(T.mask_s + p);
        const double *in = In + (size_t)ket * ldin;
        const double *jo = Jo + (size_t)((code >> 16) & 0x7fffu) * ldj;
        const uint32_t sg = code >> 31;
#pragma unroll
        for (int c = 0; c < CPT; ++c)
          if (ok[c]) {
            const uint32_t ph = (__popcll(opp[c] & m) ^ sg) & 1u;
            acc[r][c] = fma(flip(v + __ldg(jo + col[c]), ph), __ldg(in + col[c]), acc[r][c]);
          }
      }
      const uint32_t d0 = __ldg(T.off_d + row), d1 = __ldg(T.off_d + row + 1);
      for (uint32_t p = d0; p < d1; ++p) {
        const uint32_t ket = __ldg(T.ket_d + p);
        const double v = __ldg(T.val_d + p);
        const uint64_t m = __ldg(T.mask_d + p);
        const double *in = In + (size_t)ket * ldin;
#pragma unroll
        for (int c = 0; c < CPT; ++c)
          if (ok[c]) {
            const uint32_t ph = __popcll(opp[c] & m) & 1u;
            acc[r][c] = fma(flip(v, ph), __ldg(in + col[c]), acc[r][c]);
          }
      }
    }
  }
}

// Phase of an alpha-single x beta-single element: TwoExcite
// (determinants.h:500-518) with i = 2 cr_a, j = 2 cr_b + 1, a = 2 an_a,
// b = 2 an_b + 1 on the bra determinant; the integral is (an_a cr_a|an_b cr_b)
// with a minus sign when A and I have different spins.
__device__ __forceinline__ uint32_t ab_phase(uint64_t alpha, uint64_t beta, int cra, int ana, int crb, int anb) {
  const int i = 2 * cra, j = 2 * crb + 1, a = 2 * ana, b = 2 * anb + 1;
  const int I = min(i, j), J = max(i, j), A = min(a, b), B = max(a, b);
  uint64_t ma1, mb1, ma2, mb2;
  interval_masks(min(I, A), max(I, A), ma1, mb1);
  interval_masks(min(J, B), max(J, B), ma2, mb2);
  uint32_t ph = __popcll(alpha & (ma1 ^ ma2)) + __popcll(beta & (mb1 ^ mb2));
  ph += (A > J || B < I) ? 1u : 0u;
  ph += ((A ^ I) & 1) ? 1u : 0u;
  return ph & 1u;
}

template <int TA, int CPT>
__global__ void __launch_bounds__(kThreads) k_sigma_alpha(SigmaArgs a) {
  constexpr int TB = kThreads * CPT;
  const uint32_t ia0 = blockIdx.x * TA;
  const uint32_t ib0 = blockIdx.y * TB;
  uint32_t col[CPT];
  bool ok[CPT];
  uint64_t beta[CPT];
#pragma unroll
  for (int c = 0; c < CPT; ++c) {
    col[c] = ib0 + threadIdx.x + kThreads * c;
    ok[c] = col[c] < a.nb;
    beta[c] = ok[c] ? __ldg(a.bstr + col[c]) : 0ull;
  }
  double acc[TA][CPT];
  // diagonal term (mult.h:169-174)
#pragma unroll
  for (int r = 0; r < TA; ++r)
#pragma unroll
    for (int c = 0; c < CPT; ++c) {
      const uint32_t ia = ia0 + r;
      acc[r][c] = 0.0;
      if (ok[c] && ia < a.na) {
        const size_t k = (size_t)ia * a.nb + col[c];
        acc[r][c] = __ldg(a.hii + k) * __ldg(a.C + k);
      }
    }
  // alpha singles and doubles (task type 2, mult.h:450-488)
  same_spin_sweep<TA, CPT>(a.A, a.Jb, a.nb, a.C, a.nb, ia0, a.na, col, ok, beta, acc);
  // alpha single x beta single (task type 0, mult.h:527-557)
#pragma unroll
  for (int r = 0; r < TA; ++r) {
    const uint32_t ia = ia0 + r;
    if (ia < a.na) {
      const uint64_t alpha = __ldg(a.astr + ia);
      const uint32_t p0 = __ldg(a.A.off_s + ia), p1 = __ldg(a.A.off_s + ia + 1);
      for (uint32_t p = p0; p < p1; ++p) {
        const uint32_t ja = __ldg(a.A.ket_s + p), ca = __ldg(a.A.code_s + p);
        const int cra = ca & 0xff, ana = (ca >> 8) & 0xff;
        const double *krow = a.Kp + (size_t)((ca >> 16) & 0x7fffu) * a.npair;
        const double *crow = a.C + (size_t)ja * a.nb;
#pragma unroll
        for (int c = 0; c < CPT; ++c)
          if (ok[c]) {
            const uint32_t q0 = __ldg(a.B.off_s + col[c]), q1 = __ldg(a.B.off_s + col[c] + 1);
            for (uint32_t q = q0; q < q1; ++q) {
              const uint32_t jb = __ldg(a.B.ket_s + q), cb = __ldg(a.B.code_s + q);
              const uint32_t ph = ab_phase(alpha, beta[c], cra, ana, cb & 0xff, (cb >> 8) & 0xff);
              acc[r][c] = fma(flip(__ldg(krow + ((cb >> 16) & 0x7fffu)), ph), __ldg(crow + jb), acc[r][c]);
            }
          }
      }
    }
  }
#pragma unroll
  for (int r = 0; r < TA; ++r)
#pragma unroll
    for (int c = 0; c < CPT; ++c) {
      const uint32_t ia = ia0 + r;
      if (ok[c] && ia < a.na) {
        const size_t k = (size_t)ia * a.nb + col[c];
        a.S[k] = a.accumulate ? a.S[k] + acc[r][c] : acc[r][c];
      }
    }
}

// beta singles and doubles (task type 1, mult.h:489-525) on the transposed
// vector; adds its TA consecutive beta entries of each alpha row into sigma.
template <int TA, int CPT>
__global__ void __launch_bounds__(kThreads) k_sigma_beta(SigmaArgs a) {
  constexpr int TB = kThreads * CPT;
  const uint32_t ib0 = blockIdx.x * TA;
  const uint32_t ia0 = blockIdx.y * TB;
  uint32_t col[CPT];
  bool ok[CPT];
  uint64_t alpha[CPT];
#pragma unroll
  for (int c = 0; c < CPT; ++c) {
    col[c] = ia0 + threadIdx.x + kThreads * c;
    ok[c] = col[c] < a.na;
    alpha[c] = ok[c] ? __ldg(a.astr + col[c]) : 0ull;
  }
  double acc[TA][CPT];
#pragma unroll
  for (int r = 0; r < TA; ++r)
#pragma unroll
    for (int c = 0; c < CPT; ++c) acc[r][c] = 0.0;
  same_spin_sweep<TA, CPT>(a.B, a.Ja, a.na, a.CT, a.na, ib0, a.nb, col, ok, alpha, acc);
#pragma unroll
  for (int c = 0; c < CPT; ++c)
    if (ok[c]) {
      double *srow = a.S + (size_t)col[c] * a.nb;
#pragma unroll
      for (int r = 0; r < TA; ++r) {
        const uint32_t ib = ib0 + r;
        if (ib < a.nb) srow[ib] += acc[r][c];
      }
    }
}

// out[c][r] = in[r][c] for an R x Cn row-major matrix.
template <typename T>
__global__ void k_transpose(const T *__restrict__ in, T *__restrict__ out, uint32_t R, uint32_t Cn) {
  __shared__ T tile[32][33];
  const uint32_t bx = blockIdx.x * 32, by = blockIdx.y * 32;
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const uint32_t r = by + k, c = bx + threadIdx.x;
    if (r < R && c < Cn) tile[k][threadIdx.x] = in[(size_t)r * Cn + c];
  }
  __syncthreads();
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const uint32_t c = bx + k, r = by + threadIdx.x;
    if (r < R && c < Cn) out[(size_t)c * R + r] = tile[threadIdx.x][k];
  }
}

constexpr int kTA = 8;
constexpr int kCPT = 2;

SigmaArgs make_args(Problem &p, const double *C, double *S, int accumulate) {
  SigmaArgs a;
  a.astr = p.astr;
  a.bstr = p.bstr;
  a.na = p.na;
  a.nb = p.nb;
  a.hii = p.hii;
  a.C = C;
  a.CT = p.CT;
  a.S = S;
  a.accumulate = accumulate;
  a.A = p.A;
  a.B = p.B;
  a.Jb = p.Jb;
  a.Ja = p.Ja;
  a.Kp = p.Kp;
  a.npair = p.npair;
  a.norb = p.norb;
  return a;
}

}  // namespace

void transpose_fp64(Problem &p, const double *in, double *out, uint32_t R, uint32_t Cn, cudaStream_t s) {
  dim3 grid((Cn + 31) / 32, (R + 31) / 32), block(32, 8);
  k_transpose<double><<<grid, block, 0, s>>>(in, out, R, Cn);
  count_launch(p.ctx);
}

void sigma_fp64(Problem &p, const double *C, double *S, int accumulate, cudaStream_t s) {
  if (!p.tables || !p.diag) throw Error(SBDGB_E_STATE, "sigma needs tables and diagonal");
  if (!p.CT) {
    p.CT = (double *)dev_alloc(p, sizeof(double) * p.N);
  }
  if (p.N == 0) return;
  transpose_fp64(p, C, p.CT, p.na, p.nb, s);
  SigmaArgs a = make_args(p, C, S, accumulate);
  constexpr int TB = kThreads * kCPT;
  dim3 ga((p.na + kTA - 1) / kTA, (p.nb + TB - 1) / TB);
  k_sigma_alpha<kTA, kCPT><<<ga, kThreads, 0, s>>>(a);
  dim3 gb((p.nb + kTA - 1) / kTA, (p.na + TB - 1) / TB);
  k_sigma_beta<kTA, kCPT><<<gb, kThreads, 0, s>>>(a);
  count_launch(p.ctx, 2);
  SBDGB_CUDA(cudaGetLastError());
}

}  // namespace sbdgb
