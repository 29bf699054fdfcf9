// One- and two-particle reduced density matrices of a vector (Correlation,
// chemistry/tpb/correlation.h:379-640, element rules chemistry/basic/
// correlation.h:17-299), in the reference's layout:
//
//   one[s][i + L*j]                      s = spin of the pair (0 alpha, 1 beta)
//   two[s1 + 2*s2][a + L*b + L^2*c + L^3*d]
//
// The reference visits every (bra, ket) pair of the excitation lists and adds
// each element's contributions with atomics.  Here the sums over the
// spectator string are taken first:
//   - same-spin single (bra -> ket, orbitals i -> a): the weighted overlap
//     s = sum_spectator W[bra] W[ket] (+-1) and, per opposite-spin orbital q,
//     u[q] = the same sum restricted to spectators with q occupied; the
//     contributions of the occupied same-spin orbitals of the bra depend on
//     s alone, those of the opposite-spin orbitals on u[q];
//   - same-spin double: s alone (four entries);
//   - alpha single x beta single: the sum over all pairs with the same four
//     orbitals, accumulated per alpha pair in shared memory and then per
//     orbital quadruple in a global L^4 array, scattered once at the end;
//   - the diagonal (ZeroDiffCorrelation): string weights for the same-spin
//     pairs and Y = (W o W) O_beta, M = O_alpha^T Y for the alpha-beta pairs.
// Phases are the ones of the sigma kernels (same tables, same masks); the
// same-spin doubles recompute theirs from the four orbitals.
#include <algorithm>

#include "common.cuh"

namespace sbdgb {

void transpose_fp64(Problem &p, const double *in, double *out, uint32_t R, uint32_t Cn, cudaStream_t s);
void string_norms(Problem &p, const double *W, double *r, double *c, cudaStream_t s);
const double *device_vector(Problem &p, const double *W, cudaStream_t s);

namespace {

constexpr int kT = 256;
constexpr int kMaxL = 64;

__device__ __forceinline__ size_t q4(int L, int a, int b, int c, int d) {
  return (size_t)a + (size_t)L * ((size_t)b + (size_t)L * ((size_t)c + (size_t)L * (size_t)d));
}

struct RdmArgs {
  const uint64_t *astr, *bstr;
  uint32_t na, nb;
  int L;
  const double *W;   // [ia][ib]
  const double *WT;  // [ib][ia]
  double *one;       // 2 L^2
  double *two;       // 4 L^4 (null: one-particle part only)
  double *R;         // L^4 alpha-beta sums [oi_a, oa_a, oj_b, ob_b]
  SpinTables A, B;
};

// Same-spin singles of spin S, one CTA per bra string: for each pair, s and
// u[q] over the spectators; for S = 0 also the alpha-beta sums of the pair.
template <int S>
__global__ void __launch_bounds__(kT) k_rdm_singles(RdmArgs a) {
  const SpinTables &T = S == 0 ? a.A : a.B;
  const SpinTables &O = S == 0 ? a.B : a.A;  // opposite-spin tables (alpha-beta part)
  const uint64_t *same = S == 0 ? a.astr : a.bstr;
  const uint64_t *opp = S == 0 ? a.bstr : a.astr;
  const double *Wr = S == 0 ? a.W : a.WT;  // rows indexed by this spin's strings
  const uint32_t nopp = S == 0 ? a.nb : a.na;
  const int L = a.L;
  const uint32_t bra = blockIdx.x;
  __shared__ double su[kMaxL];
  __shared__ double sR[S == 0 ? kMaxL * kMaxL : 1];
  __shared__ double red[kT / 32];
  const bool two = a.two != nullptr;
  const uint32_t p0 = T.off_s[bra], p1 = T.off_s[bra + 1];
  const uint64_t bs = same[bra];
  for (uint32_t p = p0; p < p1; ++p) {
    const uint32_t ket = T.ket_s[p], code = T.code_s[p];
    const uint64_t mask = T.mask_s[p];
    const int oi = code & 0xff, oa = (code >> 8) & 0xff;
    for (int t = threadIdx.x; t < L; t += kT) su[t] = 0.0;
    if (S == 0 && two)
      for (int t = threadIdx.x; t < L * L; t += kT) sR[t] = 0.0;
    __syncthreads();
    const double *rb = Wr + (size_t)bra * nopp, *rk = Wr + (size_t)ket * nopp;
    const uint64_t kstr = same[ket];
    double sacc = 0.0;
    for (uint32_t o = threadIdx.x; o < nopp; o += kT) {
      const uint64_t os = __ldg(opp + o);
      const double wb = __ldg(rb + o);
      const uint32_t ph = (__popcll(os & mask) ^ (code >> 31)) & 1u;
      const double v = (ph ? -wb : wb) * __ldg(rk + o);
      sacc += v;
      if (two && v != 0.0) {
        uint64_t bits = os;
        while (bits) {
          const int q = __ffsll((long long)bits) - 1;
          bits &= bits - 1;
          atomicAdd(&su[q], v);
        }
      }
      if (S == 0 && two && wb != 0.0) {
        // alpha single (bra -> ket) x beta singles of spectator o: element
        // W[bra][o] W[ket][jb] with the sigma kernels' alpha-beta phase
        const uint32_t q0 = O.off_s[o], q1 = O.off_s[o + 1];
        const uint32_t pa = (__popcll(os & mask) ^ (code >> 31)) & 1u;
        for (uint32_t q = q0; q < q1; ++q) {
          const uint32_t jb = __ldg(O.ket_s + q), cb = __ldg(O.code_s + q);
          const uint64_t mb = __ldg(O.mask_s + q);
          const uint32_t f = (pa ^ __popcll(kstr & mb) ^ (cb >> 31)) & 1u;
          const double x = wb * __ldg(rk + jb);
          atomicAdd(&sR[(cb & 0xff) * L + ((cb >> 8) & 0xff)], f ? -x : x);
        }
      }
    }
    for (int off = 16; off > 0; off >>= 1) sacc += __shfl_xor_sync(0xffffffffu, sacc, off);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = sacc;
    __syncthreads();
    if (threadIdx.x == 0) {
      double s = 0.0;
      for (int w = 0; w < kT / 32; ++w) s += red[w];
      atomicAdd(&a.one[(size_t)S * L * L + oi + (size_t)L * oa], s);
      if (two && s != 0.0) {
        double *blk = a.two + (size_t)(3 * S) * L * L * L * L;  // s1 = s2 = S
        uint64_t bits = bs;
        while (bits) {
          const int oj = __ffsll((long long)bits) - 1;
          bits &= bits - 1;
          if (oj == oi) continue;  // its four terms cancel
          atomicAdd(&blk[q4(L, oa, oj, oi, oj)], s);
          atomicAdd(&blk[q4(L, oj, oa, oj, oi)], s);
          atomicAdd(&blk[q4(L, oa, oj, oj, oi)], -s);
          atomicAdd(&blk[q4(L, oj, oa, oi, oj)], -s);
        }
      }
    }
    if (two) {
      // opposite-spin spectator orbitals: blocks S + 2(1-S) and (1-S) + 2S
      double *b1 = a.two + (size_t)(S + 2 * (1 - S)) * L * L * L * L;
      double *b2 = a.two + (size_t)((1 - S) + 2 * S) * L * L * L * L;
      for (int q = threadIdx.x; q < L; q += kT) {
        const double u = su[q];
        if (u != 0.0) {
          atomicAdd(&b1[q4(L, oa, q, oi, q)], u);
          atomicAdd(&b2[q4(L, q, oa, q, oi)], u);
        }
      }
      if (S == 0) {
        double *ab = a.R + (size_t)(oi * L + oa) * L * L;
        for (int t = threadIdx.x; t < L * L; t += kT)
          if (sR[t] != 0.0) atomicAdd(&ab[t], sR[t]);
      }
    }
    __syncthreads();
  }
}

// Same-spin doubles of spin S: one warp per pair (pairs of a bra string taken
// by the warps of its CTA); TwoDiffCorrelation's phase on the bra determinant.
template <int S>
__global__ void __launch_bounds__(kT) k_rdm_doubles(RdmArgs a) {
  const SpinTables &T = S == 0 ? a.A : a.B;
  const uint64_t *same = S == 0 ? a.astr : a.bstr;
  const uint64_t *opp = S == 0 ? a.bstr : a.astr;
  const double *Wr = S == 0 ? a.W : a.WT;
  const uint32_t nopp = S == 0 ? a.nb : a.na;
  const int L = a.L;
  const uint32_t bra = blockIdx.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t p0 = T.off_d[bra], p1 = T.off_d[bra + 1];
  const uint64_t bs = same[bra];
  double *blk = a.two + (size_t)(3 * S) * L * L * L * L;
  for (uint32_t p = p0 + warp; p < p1; p += kT / 32) {
    const uint32_t ket = T.ket_d[p], code = T.code_d[p];
    const int c0 = code & 63, c1 = (code >> 6) & 63, n0 = (code >> 12) & 63, n1 = (code >> 18) & 63;
    const int I = 2 * min(c0, c1) + S, J = 2 * max(c0, c1) + S, A = 2 * min(n0, n1) + S, B = 2 * max(n0, n1) + S;
    uint64_t ma1, mb1, ma2, mb2;
    interval_masks(min(I, A), max(I, A), ma1, mb1);
    interval_masks(min(J, B), max(J, B), ma2, mb2);
    const uint64_t ms1 = S == 0 ? ma1 : mb1, ms2 = S == 0 ? ma2 : mb2;  // same-spin parts
    const uint64_t mo = S == 0 ? (mb1 ^ mb2) : (ma1 ^ ma2);              // opposite-spin part
    uint32_t base = (__popcll(bs & ms1) + __popcll(bs & ms2)) & 1u;
    if (A > J || B < I) base ^= 1u;
    const double *rb = Wr + (size_t)bra * nopp, *rk = Wr + (size_t)ket * nopp;
    double s = 0.0;
    for (uint32_t o = lane; o < nopp; o += 32) {
      const uint32_t ph = (base ^ __popcll(__ldg(opp + o) & mo)) & 1u;
      const double v = __ldg(rb + o) * __ldg(rk + o);
      s += ph ? -v : v;
    }
    for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    if (lane == 0 && s != 0.0) {
      const int oi = I / 2, oj = J / 2, oa = A / 2, ob = B / 2;
      atomicAdd(&blk[q4(L, oa, ob, oi, oj)], s);
      atomicAdd(&blk[q4(L, ob, oa, oj, oi)], s);
      atomicAdd(&blk[q4(L, oa, ob, oj, oi)], -s);
      atomicAdd(&blk[q4(L, ob, oa, oi, oj)], -s);
    }
  }
}

// Diagonal, same-spin pairs and one-particle diagonal: thread per string with
// weight w[x] (row or column norm of W).
template <int S>
__global__ void k_rdm_diag_same(RdmArgs a, const double *__restrict__ w) {
  const uint64_t *str = S == 0 ? a.astr : a.bstr;
  const uint32_t n = S == 0 ? a.na : a.nb;
  const int L = a.L;
  const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= n) return;
  const double r = w[x];
  if (r == 0.0) return;
  const uint64_t bits0 = str[x];
  double *blk = a.two ? a.two + (size_t)(3 * S) * L * L * L * L : nullptr;
  uint64_t bi = bits0;
  while (bi) {
    const int p = __ffsll((long long)bi) - 1;
    bi &= bi - 1;
    atomicAdd(&a.one[(size_t)S * L * L + p + (size_t)L * p], r);
    if (!blk) continue;
    uint64_t bj = bi;  // q > p
    while (bj) {
      const int q = __ffsll((long long)bj) - 1;
      bj &= bj - 1;
      atomicAdd(&blk[q4(L, p, q, p, q)], r);
      atomicAdd(&blk[q4(L, q, p, q, p)], r);
      atomicAdd(&blk[q4(L, p, q, q, p)], -r);
      atomicAdd(&blk[q4(L, q, p, p, q)], -r);
    }
  }
}

// Y[ia][q] = sum_ib W[ia][ib]^2 [beta orbital q in ib]; one warp per row.
__global__ void __launch_bounds__(kT) k_rdm_occ_rows(RdmArgs a, double *__restrict__ Y) {
  const int lane = threadIdx.x & 31, L = a.L;
  const uint32_t warps = gridDim.x * (kT / 32);
  for (uint32_t ia = blockIdx.x * (kT / 32) + (threadIdx.x >> 5); ia < a.na; ia += warps) {
    double y[kMaxL];
#pragma unroll
    for (int q = 0; q < kMaxL; ++q) y[q] = 0.0;
    const double *row = a.W + (size_t)ia * a.nb;
    for (uint32_t ib = lane; ib < a.nb; ib += 32) {
      const double w = __ldg(row + ib), w2 = w * w;
      const uint64_t bs = __ldg(a.bstr + ib);
#pragma unroll
      for (int q = 0; q < kMaxL; ++q)
        if ((bs >> q) & 1ull) y[q] += w2;
    }
#pragma unroll
    for (int q = 0; q < kMaxL; ++q) {
      double v = y[q];
      for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
      if (lane == 0 && q < L) Y[(size_t)ia * L + q] = v;
    }
  }
}

// Alpha-beta diagonal pairs: M[p][q] = sum_ia [p in ia] Y[ia][q], added to
// two[2][p, q, p, q] and two[1][q, p, q, p]; thread per (p, q).
__global__ void k_rdm_diag_ab(RdmArgs a, const double *__restrict__ Y) {
  const int L = a.L;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= L * L) return;
  const int p = t / L, q = t % L;
  double m = 0.0;
  for (uint32_t ia = 0; ia < a.na; ++ia)
    if ((a.astr[ia] >> p) & 1ull) m += Y[(size_t)ia * L + q];
  if (m == 0.0) return;
  const size_t L4 = (size_t)L * L * L * L;
  atomicAdd(&a.two[2 * L4 + q4(L, p, q, p, q)], m);
  atomicAdd(&a.two[1 * L4 + q4(L, q, p, q, p)], m);
}

// Alpha-beta sums R[oi, oa, oj, ob] (alpha i -> a, beta j -> b) into the
// reference's entries (TwoDiffCorrelation with i = 2oi, j = 2oj+1, a = 2oa,
// b = 2ob+1; the element's phase is already in R).
__global__ void k_rdm_scatter_ab(RdmArgs a) {
  const int L = a.L;
  const size_t L4 = (size_t)L * L * L * L;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < L4; t += (size_t)gridDim.x * blockDim.x) {
    const double x = a.R[t];
    if (x == 0.0) continue;
    const int ob = t % L, oj = (t / L) % L, oa = (t / ((size_t)L * L)) % L, oi = (int)(t / ((size_t)L * L * L));
    const int i = 2 * oi, j = 2 * oj + 1, aa = 2 * oa, b = 2 * ob + 1;
    const int I = min(i, j), J = max(i, j), A = min(aa, b), B = max(aa, b);
    const int si = I & 1, sj = J & 1, sa = A & 1;
    const int Oi = I / 2, Oj = J / 2, Oa = A / 2, Ob = B / 2;
    if (si == sa) {
      atomicAdd(&a.two[(si + 2 * sj) * L4 + q4(L, Oa, Ob, Oi, Oj)], x);
      atomicAdd(&a.two[(sj + 2 * si) * L4 + q4(L, Ob, Oa, Oj, Oi)], x);
    } else {
      atomicAdd(&a.two[(si + 2 * sj) * L4 + q4(L, Oa, Ob, Oj, Oi)], x);
      atomicAdd(&a.two[(sj + 2 * si) * L4 + q4(L, Ob, Oa, Oi, Oj)], x);
    }
  }
}

}  // namespace

void rdm(Problem &p, const double *W, double *one_host, double *two_host, cudaStream_t s) {
  SBDGB_REQUIRE(p.tables, SBDGB_E_STATE, "RDMs need the excitation tables");
  SBDGB_REQUIRE(p.norb <= kMaxL, SBDGB_E_UNSUPPORTED, "norb > 64");
  W = device_vector(p, W, s);
  const int L = p.norb;
  const size_t L2 = (size_t)L * L, L4 = L2 * L2;
  RdmArgs a{};
  a.astr = p.astr;
  a.bstr = p.bstr;
  a.na = p.na;
  a.nb = p.nb;
  a.L = L;
  a.W = W;
  a.A = p.A;
  a.B = p.B;
  double *WT = (double *)workspace(p, WS_C64, sizeof(double) * p.N);
  transpose_fp64(p, W, WT, p.na, p.nb, s);
  a.WT = WT;
  a.one = (double *)workspace(p, WS_RDM1, sizeof(double) * 2 * L2);
  SBDGB_CUDA(cudaMemsetAsync(a.one, 0, sizeof(double) * 2 * L2, s));
  if (two_host) {
    a.two = (double *)workspace(p, WS_RDM2, sizeof(double) * 4 * L4);
    a.R = (double *)workspace(p, WS_RDMAB, sizeof(double) * L4);
    SBDGB_CUDA(cudaMemsetAsync(a.two, 0, sizeof(double) * 4 * L4, s));
    SBDGB_CUDA(cudaMemsetAsync(a.R, 0, sizeof(double) * L4, s));
  }
  double *r = (double *)workspace(p, WS_NORM_A, sizeof(double) * p.na);
  double *c = (double *)workspace(p, WS_NORM_B, sizeof(double) * p.nb);
  string_norms(p, W, r, c, s);
  k_rdm_diag_same<0><<<(p.na + 127) / 128, 128, 0, s>>>(a, r);
  k_rdm_diag_same<1><<<(p.nb + 127) / 128, 128, 0, s>>>(a, c);
  k_rdm_singles<0><<<p.na, kT, 0, s>>>(a);
  k_rdm_singles<1><<<p.nb, kT, 0, s>>>(a);
  count_launch(p.ctx, 5);
  if (two_host) {
    double *Y = (double *)workspace(p, WS_RED2, sizeof(double) * (size_t)p.na * L);
    int sms = 0;
    SBDGB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, p.ctx->device));
    const uint32_t rb = (uint32_t)std::min<size_t>(((size_t)p.na + 7) / 8, (size_t)sms * 8);
    k_rdm_occ_rows<<<rb, kT, 0, s>>>(a, Y);
    k_rdm_diag_ab<<<(int)((L2 + 127) / 128), 128, 0, s>>>(a, Y);
    k_rdm_doubles<0><<<p.na, kT, 0, s>>>(a);
    k_rdm_doubles<1><<<p.nb, kT, 0, s>>>(a);
    k_rdm_scatter_ab<<<(unsigned)std::min<size_t>((L4 + 255) / 256, (size_t)sms * 8), 256, 0, s>>>(a);
    count_launch(p.ctx, 5);
  }
  SBDGB_CUDA(cudaGetLastError());
  SBDGB_CUDA(cudaMemcpyAsync(one_host, a.one, sizeof(double) * 2 * L2, cudaMemcpyDeviceToHost, s));
  if (two_host) SBDGB_CUDA(cudaMemcpyAsync(two_host, a.two, sizeof(double) * 4 * L4, cudaMemcpyDeviceToHost, s));
  SBDGB_CUDA(cudaStreamSynchronize(s));
}

}  // namespace sbdgb

extern "C" int sbdgb_rdm(sbdgb_problem *pr, const double *W, double *one, double *two, void *stream) {
  if (!pr || !W || !one) return SBDGB_E_INPUT;
  sbdgb::Ctx *c = pr->p.ctx;
  try {
    SBDGB_CUDA(cudaSetDevice(c->device));
    sbdgb::rdm(pr->p, W, one, two, stream ? (cudaStream_t)stream : c->stream);
    c->last_error.clear();
    return SBDGB_OK;
  } catch (const sbdgb::Error &e) {
    c->last_error = e.what();
    return e.status;
  } catch (const std::exception &e) {
    c->last_error = e.what();
    return SBDGB_E_INPUT;
  }
}
