// sigma = H*C for the tensor-product basis (replaces sbd::mult, TRADMODE CPU
// loop chemistry/tpb/mult.h:440-558, and the Thrust MultTPBThrust::run,
// chemistry/tpb/mult_thrust.h:1170-1580).
//
// Gather formulation without atomics; phases are applied by flipping the sign
// bit (integer work only), so the plain FP64 form issues one FP64 FMA per
// nonzero:
//
//   kernel A  rows = alpha strings, columns = beta strings, reads C[ja][ib]
//             sigma[ia][ib] = hii*C + sum_alpha-pairs +/- V * C[ja][ib]
//                                    + sum_alpha-singles sum_beta-singles +/- K * C[ja][jb]
//   kernel B  rows = beta strings, columns = alpha strings, reads C^T[jb][ia]
//             sigma[ia][ib] += sum_beta-pairs +/- V * C^T[jb][ia]
//
// A CTA owns TA rows x (128*CPT) columns and walks its rows one at a time;
// every thread keeps its columns' opposite-spin strings and CPT accumulators
// in registers.  The pair list of a row is the same for all threads of the
// CTA, so its metadata are broadcast loads and the ket-row reads are
// coalesced along the contiguous index; pairs are taken four (doubles) or two
// (singles) at a time so that each thread has several independent ket-row
// loads in flight.  Grid order puts consecutive CTAs on the same column chunk
// so that the ket rows' column slab stays in L2.  The tile shape (TA, CPT) is
// picked per problem by timing the candidates on the first product.
//
// Alpha-beta phase.  The reference evaluates TwoExcite (determinants.h:
// 500-518) on the bra determinant with i = 2 cr_a, j = 2 cr_b + 1,
// a = 2 an_a, b = 2 an_b + 1, and the value (an_a cr_a|an_b cr_b) with a
// minus sign when A and I have different spins.  That sign equals the
// product of the alpha single's phase on the bra and the beta single's phase
// on the determinant after the alpha move (alpha string ja, beta string ib);
// tests/test_sign_factorisation.py checks the identity exhaustively on small
// orbital sets.  Both phases are stored in the single-excitation tables, so
// an alpha-beta element costs two popcounts.
//
// The mixed form (T = float) stores C, sigma and the table values in FP32,
// forms each pair-list sum in FP32 and adds it to an FP64 accumulator per
// element; the FP64 form (T = double) accumulates every product in FP64.
#include <algorithm>
#include <type_traits>

#include "common.cuh"
#include "sigma_dev.cuh"

namespace sbdgb {

namespace {

using namespace sdev;
constexpr int kThreads = 128;

// kFused: the beta singles and doubles (task type 1) of each column are
// added here too, reading row ia of C directly (per-thread pair lists, no
// transposed copy); for sparse beta lists this replaces the transpose and the
// beta sweep.
// The diagonal operands of one element: hii (FP64; FP32 in .hi with .lo = 0
// for the unshifted FP32 product, hi + lo otherwise) and C.
template <typename T>
using DiagOp = typename std::conditional<std::is_same<T, double>::value, double, dfloat>::type;
template <typename T>
__device__ __forceinline__ void load_diag(const Args<T> &a, size_t k, bool ok, DiagOp<T> &h, T &x) {
  if (!ok) {
    h = DiagOp<T>(0.0);
    x = T(0);
    return;
  }
  x = ldg(a.C + k);
  if constexpr (std::is_same<T, double>::value)
    h = ldg(a.hii + k);
  else if constexpr (std::is_same<T, float>::value)
    h = a.hii_f ? dfloat(ldg(a.hii_f + k), 0.f) : ldg(a.hii_df + k);
  else
    h = ldg(a.hii_df + k);
}

template <int TA, int CPT, typename T, typename Wd, bool kFused, bool kB>
__global__ void __launch_bounds__(kThreads) k_sigma_alpha(Args<T> a) {
  constexpr int TB = kThreads * CPT;
  // Grid order.  Two sweeps: row tiles fastest (2-D grid), so that a column
  // chunk's slab of C stays in L2 while the tiles gather from it.  Fused: one
  // dimension with column chunks fastest, so that the CTAs of a row tile run
  // together and the beta pairs' gathers along its C rows hit L2.
  uint32_t bt, bc;
  if constexpr (kFused) {
    const uint32_t nch = (a.nb + TB - 1) / TB;
    bt = blockIdx.x / nch;
    bc = blockIdx.x - bt * nch;
  } else {
    bt = blockIdx.x;
    bc = blockIdx.y;
  }
  const uint32_t tile = ldg(a.tile_order + bt);
  const uint32_t ia0 = ldg(a.tile_start + tile);
  const uint32_t rend = ldg(a.tile_start + tile + 1) - ia0;  // <= TA
  const uint32_t ib0 = bc * TB;
  uint32_t col[CPT], q0[CPT], q1[CPT];
  bool ok[CPT];
  Wd beta[CPT];
#pragma unroll
  for (int c = 0; c < CPT; ++c) {
    col[c] = ib0 + threadIdx.x + kThreads * c;
    ok[c] = col[c] < a.nb;
    beta[c] = ok[c] ? word<Wd>(a.bstr, col[c]) : Wd(0);
    q0[c] = ok[c] ? ldg(a.B.off_s + col[c]) : 0u;
    q1[c] = ok[c] ? ldg(a.B.off_s + col[c] + 1) : 0u;
  }
  // Fused: the beta doubles of this thread's columns are the same for every
  // row; the first kPre of each column are held in registers (ket, value,
  // mask), so that on each row their C gathers issue with the diagonal's
  // loads instead of after a chain of table loads.
  constexpr int kPre = 2;
  constexpr int CF = kFused ? CPT : 1;
  uint32_t d0[CF], d1[CF], pjb[CF][kPre];
  T pval[CF][kPre];
  Wd pmask[CF][kPre];
  if constexpr (kFused) {
#pragma unroll
    for (int c = 0; c < CPT; ++c) {
      d0[c] = ok[c] ? ldg(a.B.off_d + col[c]) : 0u;
      d1[c] = ok[c] ? ldg(a.B.off_d + col[c] + 1) : 0u;
#pragma unroll
      for (int u = 0; u < kPre; ++u) {
        const bool has = d0[c] + u < d1[c];
        pjb[c][u] = has ? ldg(a.B.ket_d + d0[c] + u) : 0u;
        pval[c][u] = has ? ldg(a.val_db + d0[c] + u) : T(0);
        pmask[c][u] = has ? mask_of<kB, Wd>(a.B.mask_d, d0[c] + u) : Wd(0);
      }
    }
  }
  DiagOp<T> hnext[CPT];
  T cnext[CPT];
#pragma unroll
  for (int c = 0; c < CPT; ++c) load_diag(a, (size_t)ia0 * a.nb + col[c], ok[c], hnext[c], cnext[c]);
#pragma unroll 1
  for (uint32_t r = 0; r < rend; ++r) {
    const uint32_t ia = ia0 + r;
    AccT<T> acc[CPT];
    // the prefetched beta doubles' gathers along row ia, issued first
    T xpre[CF][kPre];
    if constexpr (kFused) {
#pragma unroll
      for (int c = 0; c < CPT; ++c)
#pragma unroll
        for (int u = 0; u < kPre; ++u)
          xpre[c][u] = d0[c] + u < d1[c] ? ldg(a.C + (size_t)ia * a.nb + pjb[c][u]) : T(0);
    }
    // diagonal term (mult.h:169-174): FP64, or hi/lo FP32 parts of the FP64
    // diagonal in the mixed form.  Its operands were loaded one row ahead
    // (hcur, ccur), and the next row's are requested now, so that each thread
    // has two rows' streaming loads in flight.
    DiagOp<T> hcur[CPT];
    T ccur[CPT];
#pragma unroll
    for (int c = 0; c < CPT; ++c) {
      hcur[c] = hnext[c];
      ccur[c] = cnext[c];
      if (r + 1 < rend) load_diag(a, (size_t)(ia + 1) * a.nb + col[c], ok[c], hnext[c], cnext[c]);
      acc_zero(acc[c]);
      if (ok[c]) {
        if constexpr (std::is_same<T, double>::value) {
          acc[c] = hcur[c] * ccur[c];  // the FP64 form has no shift: one FP64 op
        } else if constexpr (std::is_same<T, float>::value) {
          if (a.hii_f)
            acc[c] = ff_prod(hcur[c].hi, ccur[c]);
          else
            acc[c] = ff_diag(hcur[c].hi, hcur[c].lo, a.shift_df.hi, a.shift_df.lo, ccur[c]);
        } else {
          acc[c] = (hcur[c] - a.shift_df) * ccur[c];
        }
      }
    }
    // alpha singles and doubles (task type 2, mult.h:450-488)
    same_spin_row<CPT, T, Wd, kB>(a.A, a.val_sa, a.val_da, a.Jb, a.nb, a.C, a.nb, ia, col, ok, beta, acc);
    // alpha single x beta single (task type 0, mult.h:527-557)
    T part[CPT];
#pragma unroll
    for (int c = 0; c < CPT; ++c) part[c] = T(0);
    const uint32_t p0 = ldg(a.A.off_s + ia), p1 = ldg(a.A.off_s + ia + 1);
    // the beta singles of each column outside (their table entries are read
    // once per thread), the alpha singles of the row inside (the same entries
    // for every thread: broadcast loads): a term costs two scattered loads
    // (the (P|Q) value and C) instead of five, and one more popcount
#pragma unroll
    for (int c = 0; c < CPT; ++c) {
      if (a.skip_ab) break;  // left to k_sigma_ab
      for (uint32_t q = q0[c]; q < q1[c]; ++q) {
        const uint32_t jb = ldg(a.B.ket_s + q), cb = ldg(a.B.code_s + q);
        const Wd mb = mask_of<kB, Wd>(a.B.mask_s, q);
        const uint32_t kb = (cb >> 16) & 0x7fffu, sb = cb >> 31;
        for (uint32_t p = p0; p < p1; ++p) {
          const uint32_t ja = ldg(a.A.ket_s + p), ca = ldg(a.A.code_s + p);
          const uint32_t ph =
              (par<kB>(beta[c] & mask_of<kB, Wd>(a.A.mask_s, p)) ^ par<kB>(word<Wd>(a.astr, ja) & mb) ^ (ca >> 31) ^ sb) &
              1u;
          madd(acc[c], part[c], flip(ldg(a.Kp + ((ca >> 16) & 0x7fffu) * a.npair + kb), ph),
               ldg(a.C + (size_t)ja * a.nb + jb));
        }
      }
    }
    if constexpr (kFused) {
      // beta singles and doubles (task type 1, mult.h:489-525) on row ia
      const Wd arow = word<Wd>(a.astr, ia);
      const T *crow_a = a.C + (size_t)ia * a.nb;
#pragma unroll
      for (int c = 0; c < CPT; ++c) {
        for (uint32_t q = q0[c]; q < q1[c]; ++q) {
          const uint32_t jb = ldg(a.B.ket_s + q), cb = ldg(a.B.code_s + q);
          const uint32_t ph = par<kB>(arow & mask_of<kB, Wd>(a.B.mask_s, q)) ^ (cb >> 31);
          const T j = ldg(a.Ja + (size_t)((cb >> 16) & 0x7fffu) * a.na + ia);
          madd(acc[c], part[c], flip(ldg(a.val_sb + q) + j, ph), ldg(crow_a + jb));
        }
#pragma unroll
        for (int u = 0; u < kPre; ++u)
          if (d0[c] + u < d1[c]) madd(acc[c], part[c], flip(pval[c][u], par<kB>(arow & pmask[c][u])), xpre[c][u]);
        for (uint32_t q = d0[c] + kPre; q < d1[c]; ++q) {
          const uint32_t jb = ldg(a.B.ket_d + q);
          madd(acc[c], part[c], flip(ldg(a.val_db + q), par<kB>(arow & mask_of<kB, Wd>(a.B.mask_d, q))),
               ldg(crow_a + jb));
        }
      }
    }
#pragma unroll
    for (int c = 0; c < CPT; ++c) {
      acc_add_part(acc[c], part[c]);
      if (ok[c]) {
        const size_t k = (size_t)ia * a.nb + col[c];
        if constexpr (std::is_same<T, float>::value) {
          if (a.accumulate) ff_add(acc[c], a.S[k]);
          a.S[k] = ff_value(acc[c]);
        } else {
          a.S[k] = a.accumulate ? a.S[k] + acc[c] : acc[c];
        }
      }
    }
  }
}

// beta singles and doubles (task type 1, mult.h:489-525) on the transposed
// vector.  Row results are staged in shared memory; each thread then adds the
// TA consecutive beta entries of its alpha rows into sigma.
template <int TA, int CPT, typename T, typename Wd, bool kB>
__global__ void __launch_bounds__(kThreads) k_sigma_beta(Args<T> a) {
  constexpr int TB = kThreads * CPT;
  __shared__ AccT<T> tile[TA][TB];
  const uint32_t t = ldg(a.tile_order + blockIdx.x);
  const uint32_t ib0 = ldg(a.tile_start + t);
  const uint32_t rend = ldg(a.tile_start + t + 1) - ib0;  // <= TA
  const uint32_t ia0 = blockIdx.y * TB;
  uint32_t col[CPT];
  bool ok[CPT];
  Wd alpha[CPT];
#pragma unroll
  for (int c = 0; c < CPT; ++c) {
    col[c] = ia0 + threadIdx.x + kThreads * c;
    ok[c] = col[c] < a.na;
    alpha[c] = ok[c] ? word<Wd>(a.astr, col[c]) : Wd(0);
  }
#pragma unroll 1
  for (uint32_t r = 0; r < rend; ++r) {
    AccT<T> acc[CPT];
#pragma unroll
    for (int c = 0; c < CPT; ++c) acc_zero(acc[c]);
    same_spin_row<CPT, T, Wd, kB>(a.B, a.val_sb, a.val_db, a.Ja, a.na, a.CT, a.na, ib0 + r, col, ok, alpha, acc);
#pragma unroll
    for (int c = 0; c < CPT; ++c) tile[r][threadIdx.x + kThreads * c] = acc[c];
  }
  // each thread owns its columns: no barrier needed between its own writes and reads
#pragma unroll
  for (int c = 0; c < CPT; ++c)
    if (ok[c]) {
      T *srow = a.S + (size_t)col[c] * a.nb + ib0;
      for (uint32_t r = 0; r < rend; ++r) {
        AccT<T> t = tile[r][threadIdx.x + kThreads * c];
        if constexpr (std::is_same<T, float>::value) {
          ff_add(t, srow[r]);
          srow[r] = ff_value(t);
        } else {
          srow[r] = srow[r] + t;
        }
      }
    }
}

// ---- sparse rows: every task type in one streaming pass ---------------------------
//
// For problems with few nonzeros per row (norb 58, 12000 x 12000 strings:
// 0.48 per row) sigma is a stream over hii, C and sigma.  k_sigma_sparse does
// every task type in one pass, with no transposed copy:
//  * a CTA owns one work-balanced tile of at most TA alpha rows and 128*VW
//    beta columns; a thread owns VW consecutive columns, so hii, C and sigma
//    move in 16-byte accesses (VW = 2 doubles, or 4 floats) when the row
//    length allows it (VW = 1 otherwise);
//  * the diagonal terms of all rows of the tile are loaded first (TA
//    independent vector loads per thread in flight);
//  * beta pairs (task type 1, mult.h:489-525) belong to a column: for each
//    pair of a thread's columns the tile's rows are gathered together;
//  * alpha pairs (type 2, mult.h:450-488) and alpha x beta pairs (type 0,
//    :527-557) belong to a row and are read once per CTA (broadcast loads).
// Rows are unrolled (TA accumulators per column live in registers).  FP32
// (mixed form): FP32 products and partial sums, float-float accumulation per
// element, no FP64 instruction.
template <int RG, int VW, typename T, typename Wd, bool kB>
__device__ __forceinline__ void sparse_rows(const Args<T> &a, uint32_t ia0, uint32_t nr, uint32_t c0,
                                            const Wd (&beta)[VW], const uint32_t (&q0)[VW],
                                            const uint32_t (&q1)[VW], const uint32_t (&d0)[VW],
                                            const uint32_t (&d1)[VW]) {
  constexpr bool kF64 = std::is_same<T, double>::value;
  Wd arow[RG];
#pragma unroll
  for (int r = 0; r < RG; ++r) arow[r] = (uint32_t)r < nr ? word<Wd>(a.astr, ia0 + r) : Wd(0);
  AccT<T> acc[RG][VW];
  T part[RG][VW];
  // diagonal terms of every row of the group (mult.h:169-174)
#pragma unroll
  for (int r = 0; r < RG; ++r) {
#pragma unroll
    for (int v = 0; v < VW; ++v) {
      acc_zero(acc[r][v]);
      part[r][v] = T(0);
    }
    if ((uint32_t)r < nr) {
      const size_t k = (size_t)(ia0 + r) * a.nb + c0;
      T x[VW];
      load_v<VW>(a.C + k, x);
      if constexpr (kF64) {
        double h[VW];
        load_v<VW>(a.hii + k, h);
#pragma unroll
        for (int v = 0; v < VW; ++v) acc[r][v] = h[v] * x[v];  // the FP64 form has no shift
      } else if (std::is_same<T, float>::value && a.hii_f) {
        float h[VW];
        load_v<VW>(reinterpret_cast<const float *>(a.hii_f) + k, h);
#pragma unroll
        for (int v = 0; v < VW; ++v) acc_diag_f(acc[r][v], h[v], x[v]);
      } else {
        dfloat h[VW];
        load_v<VW>(a.hii_df + k, h);
#pragma unroll
        for (int v = 0; v < VW; ++v) {
          if constexpr (std::is_same<T, float>::value)
            acc[r][v] = ff_diag(h[v].hi, h[v].lo, a.shift_df.hi, a.shift_df.lo, x[v]);
          else
            acc[r][v] = (h[v] - a.shift_df) * x[v];
        }
      }
    }
  }
  // beta singles and doubles of this thread's columns (task type 1)
#pragma unroll
  for (int v = 0; v < VW; ++v) {
    for (uint32_t q = d0[v]; q < d1[v]; ++q) {
      const uint32_t jb = ldg(a.B.ket_d + q);
      const T val = ldg(a.val_db + q);
      const Wd m = mask_of<kB, Wd>(a.B.mask_d, q);
      T x[RG];
#pragma unroll
      for (int r = 0; r < RG; ++r) x[r] = (uint32_t)r < nr ? ldg(a.C + (size_t)(ia0 + r) * a.nb + jb) : T(0);
#pragma unroll
      for (int r = 0; r < RG; ++r) madd(acc[r][v], part[r][v], flip(val, par<kB>(arow[r] & m)), x[r]);
    }
    for (uint32_t q = q0[v]; q < q1[v]; ++q) {
      const uint32_t jb = ldg(a.B.ket_s + q), code = ldg(a.B.code_s + q);
      const T val = ldg(a.val_sb + q);
      const Wd m = mask_of<kB, Wd>(a.B.mask_s, q);
      const T *jrow = a.Ja + (size_t)((code >> 16) & 0x7fffu) * a.na + ia0;
      T x[RG], j[RG];
#pragma unroll
      for (int r = 0; r < RG; ++r) {
        x[r] = (uint32_t)r < nr ? ldg(a.C + (size_t)(ia0 + r) * a.nb + jb) : T(0);
        j[r] = (uint32_t)r < nr ? ldg(jrow + r) : T(0);
      }
#pragma unroll
      for (int r = 0; r < RG; ++r)
        madd(acc[r][v], part[r][v], flip(val + j[r], par<kB>(arow[r] & m) ^ (code >> 31)), x[r]);
    }
  }
  // alpha pairs of each row (task type 2) and alpha x beta pairs (type 0)
#pragma unroll
  for (int r = 0; r < RG; ++r) {
    if ((uint32_t)r >= nr) break;
    const uint32_t ia = ia0 + r;
    const uint32_t p0 = ldg(a.A.off_s + ia), p1 = ldg(a.A.off_s + ia + 1);
    for (uint32_t p = p0; p < p1; ++p) {
      const uint32_t ja = ldg(a.A.ket_s + p), code = ldg(a.A.code_s + p);
      const T val = ldg(a.val_sa + p);
      const Wd m = mask_of<kB, Wd>(a.A.mask_s, p);
      const uint32_t P = (code >> 16) & 0x7fffu;
      T x[VW], j[VW];
      load_v<VW>(a.C + (size_t)ja * a.nb + c0, x);
      load_v<VW>(a.Jb + (size_t)P * a.nb + c0, j);
#pragma unroll
      for (int v = 0; v < VW; ++v)
        madd(acc[r][v], part[r][v], flip(val + j[v], par<kB>(beta[v] & m) ^ (code >> 31)), x[v]);
      // alpha x beta: this alpha single with every beta single of the column
      if (a.skip_ab) continue;  // left to k_sigma_ab
      const Wd aket = word<Wd>(a.astr, ja);
      const T *krow = a.Kp + (size_t)P * a.npair;
#pragma unroll
      for (int v = 0; v < VW; ++v)
        for (uint32_t q = q0[v]; q < q1[v]; ++q) {
          const uint32_t jb = ldg(a.B.ket_s + q), cb = ldg(a.B.code_s + q);
          const uint32_t ph =
              (par<kB>(beta[v] & m) ^ par<kB>(aket & mask_of<kB, Wd>(a.B.mask_s, q)) ^ (code >> 31) ^ (cb >> 31)) & 1u;
          madd(acc[r][v], part[r][v], flip(ldg(krow + ((cb >> 16) & 0x7fffu)), ph),
               ldg(a.C + (size_t)ja * a.nb + jb));
        }
    }
    const uint32_t e0 = ldg(a.A.off_d + ia), e1 = ldg(a.A.off_d + ia + 1);
    for (uint32_t p = e0; p < e1; ++p) {
      const uint32_t ja = ldg(a.A.ket_d + p);
      const T val = ldg(a.val_da + p);
      const Wd m = mask_of<kB, Wd>(a.A.mask_d, p);
      T x[VW];
      load_v<VW>(a.C + (size_t)ja * a.nb + c0, x);
#pragma unroll
      for (int v = 0; v < VW; ++v) madd(acc[r][v], part[r][v], flip(val, par<kB>(beta[v] & m)), x[v]);
    }
  }
  // write back
#pragma unroll
  for (int r = 0; r < RG; ++r) {
    if ((uint32_t)r >= nr) break;
    const size_t k = (size_t)(ia0 + r) * a.nb + c0;
    T out[VW];
    if (a.accumulate) {
      T old[VW];
      load_v<VW>(a.S + k, old);
#pragma unroll
      for (int v = 0; v < VW; ++v) {
        acc_add_part(acc[r][v], part[r][v]);
        if constexpr (std::is_same<T, float>::value) {
          ff_add(acc[r][v], old[v]);
          out[v] = ff_value(acc[r][v]);
        } else {
          out[v] = old[v] + acc[r][v];
        }
      }
    } else {
#pragma unroll
      for (int v = 0; v < VW; ++v) {
        acc_add_part(acc[r][v], part[r][v]);
        out[v] = (T)acc_value(acc[r][v]);
      }
    }
    store_v<VW>(a.S + k, out);
  }
}

// One CTA: a row tile of at most TA rows, swept RG = 4 rows at a time (RG
// accumulators per column in registers; few registers keep enough warps
// resident to cover the latency of the gathers).
template <int TA, int VW, typename T, typename Wd, bool kB>
__global__ void __launch_bounds__(kThreads) k_sigma_sparse(Args<T> a) {
  constexpr int RG = 4;
  // one-dimensional grid, column chunks fastest: the CTAs of one row tile run
  // together, so the rows of C that a tile's beta pairs gather across the
  // whole row are in L2 while its other chunks stream them
  const uint32_t nchunk = (a.nb + kThreads * VW - 1) / (kThreads * VW);
  const uint32_t tix = blockIdx.x / nchunk, chunk = blockIdx.x - tix * nchunk;
  const uint32_t tile = ldg(a.tile_order + tix);
  const uint32_t ia0 = ldg(a.tile_start + tile);
  const uint32_t rend = ldg(a.tile_start + tile + 1) - ia0;  // 1..TA
  const uint32_t c0 = chunk * (kThreads * VW) + threadIdx.x * VW;
  if (c0 >= a.nb) return;  // nb is a multiple of VW: a vector is wholly in or out
  Wd beta[VW];
  uint32_t q0[VW], q1[VW], d0[VW], d1[VW];
#pragma unroll
  for (int v = 0; v < VW; ++v) {
    beta[v] = word<Wd>(a.bstr, c0 + v);
    q0[v] = ldg(a.B.off_s + c0 + v);
    q1[v] = ldg(a.B.off_s + c0 + v + 1);
    d0[v] = ldg(a.B.off_d + c0 + v);
    d1[v] = ldg(a.B.off_d + c0 + v + 1);
  }
#pragma unroll 1
  for (uint32_t g = 0; g < rend; g += RG)
    sparse_rows<RG, VW, T, Wd, kB>(a, ia0 + g, min((uint32_t)RG, rend - g), c0, beta, q0, q1, d0, d1);
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

__global__ void k_to_float(const double *__restrict__ x, float *__restrict__ y, size_t n) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x)
    y[e] = (float)x[e];
}

// y = double-float(x): hi = fp32(x), lo = fp32(x - hi) (hi + lo carries 48
// bits of x), for the diagonal and tables of the FP32 and double-float kernels.
__global__ void k_split(const double *__restrict__ x, dfloat *__restrict__ y, size_t n) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x)
    y[e] = dfloat(x[e]);
}

// x_v *= eta(ia, ib) for nvec vectors at stride N (the sign between the
// interleaved and the block determinant of element ia * nb + ib).
template <typename T>
__global__ void k_eta(T *__restrict__ x, const uint64_t *__restrict__ astr, const uint64_t *__restrict__ bstr,
                      uint32_t nb, uint32_t N, int nvec) {
  for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < N; e += gridDim.x * blockDim.x) {
    const uint32_t ia = e / nb, ib = e - ia * nb;
    if (eta_parity(ldg(astr + ia), ldg(bstr + ib)))
      for (int v = 0; v < nvec; ++v) x[(size_t)v * N + e] = -x[(size_t)v * N + e];
  }
}

// ---- tile shapes and the autotuner ---------------------------------------------

constexpr int kNumShapes = 4;
constexpr int kFusedShape = 4;   // tune_b value meaning "beta sweep fused into kernel A"
constexpr int kSparseShape = 5;  // tune_b value meaning "k_sigma_sparse"; tune_a 0/1 = 8/16 rows per tile
constexpr int kNumSparse = 2;
constexpr int kStreamShape = 6;  // tune_b value meaning "the row kernel" (sigma_stream.cu); tune_a 0/1 = its two forms
inline bool needs_transpose(int shape_b) {
  return shape_b != kFusedShape && shape_b != kSparseShape && shape_b != kStreamShape;
}
constexpr int kShapeTA[kNumShapes] = {8, 8, 8, 16};
constexpr int kShapeCPT[kNumShapes] = {1, 2, 4, 2};

// Launchers: kB selects the block-ordering kernels (no opposite-spin
// parities; no string words are read for phases, so one word width serves).
template <typename T, int TA, int CPT, bool F, bool kB>
void launch_a_shape(const Problem &p, Args<T> a, cudaStream_t s) {
  constexpr int TB = kThreads * CPT;
  constexpr int v = TA == 8 ? 0 : 1;
  a.tile_start = p.tile_start[0][v];
  a.tile_order = p.tile_order[0][v];
  const dim3 g = F ? dim3(p.n_tiles[0][v] * ((p.nb + TB - 1) / TB)) : dim3(p.n_tiles[0][v], (p.nb + TB - 1) / TB);
  if (kB || p.norb <= 32)
    k_sigma_alpha<TA, CPT, T, uint32_t, F, kB><<<g, kThreads, 0, s>>>(a);
  else
    k_sigma_alpha<TA, CPT, T, unsigned long long, F, kB><<<g, kThreads, 0, s>>>(a);
}
template <typename T, int TA, int CPT, bool kB>
void launch_b_shape(const Problem &p, Args<T> a, cudaStream_t s) {
  constexpr int TB = kThreads * CPT;
  constexpr int v = TA == 8 ? 0 : 1;
  a.tile_start = p.tile_start[1][v];
  a.tile_order = p.tile_order[1][v];
  dim3 g(p.n_tiles[1][v], (p.na + TB - 1) / TB);
  if (kB || p.norb <= 32)
    k_sigma_beta<TA, CPT, T, uint32_t, kB><<<g, kThreads, 0, s>>>(a);
  else
    k_sigma_beta<TA, CPT, T, unsigned long long, kB><<<g, kThreads, 0, s>>>(a);
}

template <typename T, bool kB, bool F = false>
void launch_a(const Problem &p, const Args<T> &a, int shape, cudaStream_t s) {
  switch (shape) {
    case 0: launch_a_shape<T, 8, 1, F, kB>(p, a, s); break;
    case 1: launch_a_shape<T, 8, 2, F, kB>(p, a, s); break;
    case 2: launch_a_shape<T, 8, 4, F, kB>(p, a, s); break;
    default: launch_a_shape<T, 16, 2, F, kB>(p, a, s); break;
  }
}
inline bool aligned16(const void *x) { return ((uintptr_t)x & 15u) == 0; }

// The single streaming kernel for sparse rows: TA = 8 (variant 0) or 16 rows
// per tile; 16-byte vectors when the row length and the pointers allow.
template <typename T, int TA, typename Wd, bool kB>
void launch_sparse_ta(const Problem &p, Args<T> a, cudaStream_t s) {
  constexpr int v = TA == 8 ? 0 : 1;
  constexpr int VW = 16 / (int)sizeof(T);
  a.tile_start = p.tile_start[0][v];
  a.tile_order = p.tile_order[0][v];
  const bool vec = p.nb % VW == 0 && aligned16(a.C) && aligned16(a.S) && aligned16(a.Jb) &&
                   (std::is_same<T, double>::value ? aligned16(a.hii) : aligned16(a.hii_df)) &&
                   (a.hii_f == nullptr || aligned16(a.hii_f));
  if (vec) {
    const unsigned g = p.n_tiles[0][v] * ((p.nb + kThreads * VW - 1) / (kThreads * VW));
    k_sigma_sparse<TA, VW, T, Wd, kB><<<g, kThreads, 0, s>>>(a);
  } else {
    const unsigned g = p.n_tiles[0][v] * ((p.nb + kThreads - 1) / kThreads);
    k_sigma_sparse<TA, 1, T, Wd, kB><<<g, kThreads, 0, s>>>(a);
  }
}
template <typename T, bool kB>
void launch_sparse(const Problem &p, const Args<T> &a, int variant, cudaStream_t s) {
  if (kB || p.norb <= 32) {
    if (variant == 0) launch_sparse_ta<T, 8, uint32_t, kB>(p, a, s);
    else launch_sparse_ta<T, 16, uint32_t, kB>(p, a, s);
  } else {
    if (variant == 0) launch_sparse_ta<T, 8, unsigned long long, kB>(p, a, s);
    else launch_sparse_ta<T, 16, unsigned long long, kB>(p, a, s);
  }
}

// The fused single-kernel product (no transposed copy), in shape `shape`.
template <typename T, bool kB>
void launch_fused(const Problem &p, const Args<T> &a, int shape, cudaStream_t s) {
  launch_a<T, kB, true>(p, a, shape, s);
}
template <typename T, bool kB>
void launch_b(const Problem &p, const Args<T> &a, int shape, cudaStream_t s) {
  switch (shape) {
    case 0: launch_b_shape<T, 8, 1, kB>(p, a, s); break;
    case 1: launch_b_shape<T, 8, 2, kB>(p, a, s); break;
    case 2: launch_b_shape<T, 8, 4, kB>(p, a, s); break;
    default: launch_b_shape<T, 16, 2, kB>(p, a, s); break;
  }
}

// The row kernel when its pair list fits the problem, the sparse-row kernel
// otherwise (same results up to the order of floating-point sums).
template <typename T, bool kB>
void launch_stream_or_sparse(const Problem &p, const Args<T> &a, int variant, cudaStream_t s) {
  if (rows_fit<T>(p))
    launch_stream<T, kB>(p, a, variant, s);
  else
    launch_sparse<T, kB>(p, a, variant, s);
}

// One product in shapes (sa, sb) on a transposed copy already made when the
// shapes need one; with split > 0 those kernels skip the alpha x beta single
// pairs and k_sigma_ab adds them afterwards.
template <typename T, bool kB>
void launch_shapes(Problem &p, const Args<T> &a, int sa, int sb, int split, cudaStream_t s) {
  Args<T> b = a;
  b.skip_ab = split > 0 ? 1 : 0;
  if (sb == kSparseShape) {
    launch_sparse<T, kB>(p, b, sa, s);
    count_launch(p.ctx, 1);
  } else if (sb == kStreamShape) {
    launch_stream_or_sparse<T, kB>(p, b, sa, s);
    count_launch(p.ctx, 1);
  } else if (sb == kFusedShape) {
    launch_fused<T, kB>(p, b, sa, s);
    count_launch(p.ctx, 1);
  } else {
    launch_a<T, kB>(p, b, sa, s);
    launch_b<T, kB>(p, b, sb, s);
    count_launch(p.ctx, 2);
  }
  SBDGB_CUDA(cudaGetLastError());
  if (split > 0) launch_ab<T>(p, a, kB, s);
}

// Tuning slot of a kernel family: precision (0 FP64, 1 FP32, 2 double-float)
// in the interleaved (0..2) or block (3..5) ordering.
template <typename T, bool kB>
constexpr int slot_of() {
  return prec_of<T>() + (kB ? 3 : 0);
}

template <typename T>
void transpose(Problem &p, const T *in, T *out, uint32_t R, uint32_t Cn, cudaStream_t s);

// Times every tile shape of both kernels once (after one untimed run) on the
// problem's own vectors, writing into scratch, and keeps the fastest.
template <typename T, bool kB>
void autotune(Problem &p, Args<T> a, cudaStream_t s) {
  const int prec = slot_of<T, kB>();
  if (p.tune_a[prec] >= 0 && p.tune_b[prec] >= 0) return;
  const std::array<uint64_t, 6> key{(uint64_t)prec, (uint64_t)p.norb, p.na, p.nb, p.A.ns + p.A.nd, p.B.ns + p.B.nd};
  const auto hit = p.ctx->tuned.find(key);
  if (hit != p.ctx->tuned.end()) {
    p.tune_a[prec] = hit->second.a;
    p.tune_b[prec] = hit->second.b;
    p.split_ab[prec] = hit->second.split_ab;
    std::copy(&hit->second.ms[0][0], &hit->second.ms[0][0] + 3 * 8, &p.tune_ms[prec][0][0]);
    std::copy(hit->second.ab_ms, hit->second.ab_ms + 2, p.tune_ab_ms[prec]);
    return;
  }
  a.S = (T *)workspace(p, WS_TUNE, sizeof(T) * p.N);
  a.accumulate = 0;
  cudaEvent_t e0, e1;
  SBDGB_CUDA(cudaEventCreate(&e0));
  SBDGB_CUDA(cudaEventCreate(&e1));
  for (int kern = 0; kern < 2; ++kern) {
    float best = 1e30f;
    int best_shape = 1;
    for (int sh = 0; sh < kNumShapes; ++sh) {
      for (int rep = 0; rep < 2; ++rep) {
        SBDGB_CUDA(cudaEventRecord(e0, s));
        if (kern == 0)
          launch_a<T, kB>(p, a, sh, s);
        else
          launch_b<T, kB>(p, a, sh, s);
        SBDGB_CUDA(cudaEventRecord(e1, s));
        count_launch(p.ctx);
      }
      SBDGB_CUDA(cudaGetLastError());
      SBDGB_CUDA(cudaEventSynchronize(e1));
      float ms = 0.f;
      SBDGB_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      p.tune_ms[prec][kern][sh] = ms;
      if (ms < best) {
        best = ms;
        best_shape = sh;
      }
    }
    (kern == 0 ? p.tune_a : p.tune_b)[prec] = best_shape;
  }
  // the fused single kernel against transpose + both sweeps
  float t_tr = 0.f;
  SBDGB_CUDA(cudaEventRecord(e0, s));
  transpose<T>(p, a.C, const_cast<T *>(a.CT), p.na, p.nb, s);
  SBDGB_CUDA(cudaEventRecord(e1, s));
  SBDGB_CUDA(cudaEventSynchronize(e1));
  SBDGB_CUDA(cudaEventElapsedTime(&t_tr, e0, e1));
  const float two_kernels = t_tr + p.tune_ms[prec][0][p.tune_a[prec]] + p.tune_ms[prec][1][p.tune_b[prec]];
  float best_f = 1e30f;
  int best_fs = 0;
  for (int sh = 0; sh < kNumShapes; ++sh) {
    for (int rep = 0; rep < 2; ++rep) {
      SBDGB_CUDA(cudaEventRecord(e0, s));
      launch_fused<T, kB>(p, a, sh, s);
      SBDGB_CUDA(cudaEventRecord(e1, s));
      count_launch(p.ctx);
    }
    SBDGB_CUDA(cudaGetLastError());
    SBDGB_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    SBDGB_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    p.tune_ms[prec][2][sh] = ms;
    if (ms < best_f) {
      best_f = ms;
      best_fs = sh;
    }
  }
  // the single streaming kernel for sparse rows
  float best_s = 1e30f;
  int best_ss = 0;
  for (int sh = 0; sh < kNumSparse; ++sh) {
    for (int rep = 0; rep < 2; ++rep) {
      SBDGB_CUDA(cudaEventRecord(e0, s));
      launch_sparse<T, kB>(p, a, sh, s);
      SBDGB_CUDA(cudaEventRecord(e1, s));
      count_launch(p.ctx);
    }
    SBDGB_CUDA(cudaGetLastError());
    SBDGB_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    SBDGB_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    p.tune_ms[prec][2][kNumShapes + sh] = ms;
    if (ms < best_s) {
      best_s = ms;
      best_ss = sh;
    }
  }
  // the streaming kernel for sparse rows (per-warp beta pairs)
  float best_t = 1e30f;
  int best_ts = 0;
  for (int sh = 0; sh < kNumSparse && rows_fit<T>(p); ++sh) {
    for (int rep = 0; rep < 2; ++rep) {
      SBDGB_CUDA(cudaEventRecord(e0, s));
      launch_stream<T, kB>(p, a, sh, s);
      SBDGB_CUDA(cudaEventRecord(e1, s));
      count_launch(p.ctx);
    }
    SBDGB_CUDA(cudaGetLastError());
    SBDGB_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    SBDGB_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    p.tune_ms[prec][2][kNumShapes + kNumSparse + sh] = ms;
    if (ms < best_t) {
      best_t = ms;
      best_ts = sh;
    }
  }
  if (best_t < two_kernels && best_t <= best_f && best_t <= best_s) {
    p.tune_a[prec] = best_ts;
    p.tune_b[prec] = kStreamShape;
  } else if (best_s < two_kernels && best_s <= best_f) {
    p.tune_a[prec] = best_ss;
    p.tune_b[prec] = kSparseShape;
  } else if (best_f < two_kernels) {
    p.tune_a[prec] = best_fs;
    p.tune_b[prec] = kFusedShape;
  }
  // the alpha x beta single pairs in their own kernel, against inside the
  // chosen shapes (each timed over two products, transposed copy included)
  p.split_ab[prec] = 0;
  if (ab_fits<T>(p)) {
    for (int sp = 0; sp < 2; ++sp) {
      SBDGB_CUDA(cudaEventRecord(e0, s));
      for (int rep = 0; rep < 2; ++rep) {
        if (needs_transpose(p.tune_b[prec])) transpose<T>(p, a.C, const_cast<T *>(a.CT), p.na, p.nb, s);
        launch_shapes<T, kB>(p, a, p.tune_a[prec], p.tune_b[prec], sp, s);
      }
      SBDGB_CUDA(cudaEventRecord(e1, s));
      SBDGB_CUDA(cudaEventSynchronize(e1));
      float ms = 0.f;
      SBDGB_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      p.tune_ab_ms[prec][sp] = 0.5f * ms;
    }
    p.split_ab[prec] = p.tune_ab_ms[prec][1] < p.tune_ab_ms[prec][0] ? 1 : 0;
  }
  Ctx::Tuned t{p.tune_a[prec], p.tune_b[prec], p.split_ab[prec], {}, {}};
  std::copy(&p.tune_ms[prec][0][0], &p.tune_ms[prec][0][0] + 3 * 8, &t.ms[0][0]);
  std::copy(p.tune_ab_ms[prec], p.tune_ab_ms[prec] + 2, t.ab_ms);
  p.ctx->tuned[key] = t;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  release_workspace(p, WS_TUNE);
}

// Shape taken without timing (serving contexts): 128-column tiles when the
// swept dimension is short, so that small problems still spread over the SMs.
// The fused single kernel is taken when the beta lists are short (at most 8
// pairs per string on average), where its per-thread lists diverge little.
inline int size_shape(uint32_t columns) { return columns <= 1024 ? 0 : 1; }

// Nonzeros per row of H off the diagonal (same-spin pairs of both spins and
// the alpha x beta products, from the table sizes).
inline double nnz_per_row(const Problem &p) {
  const double sa = p.na ? (double)p.A.ns / p.na : 0.0, sb = p.nb ? (double)p.B.ns / p.nb : 0.0;
  return (p.na ? (double)(p.A.ns + p.A.nd) / p.na : 0.0) + (p.nb ? (double)(p.B.ns + p.B.nd) / p.nb : 0.0) + sa * sb;
}

// Alpha x beta single pairs per determinant above which the untimed choice
// gives them their own kernel (k_sigma_ab stages rows per alpha single; with
// a few singles per string on both sides that staging is cheap per term).
constexpr double kAbSplitPerElement = 4.0;

template <typename T, bool kB>
bool needs_tuning(Problem &p) {
  const int prec = slot_of<T, kB>();
  if (p.tune_a[prec] >= 0 && p.tune_b[prec] >= 0) return false;
  if (p.ctx->autotune) return true;
  p.split_ab[prec] =
      (ab_fits<T>(p) && (double)p.A.ns * (double)p.B.ns >= kAbSplitPerElement * (double)p.N) ? 1 : 0;
  if (nnz_per_row(p) <= 8.0) {
    p.tune_a[prec] = 0;
    p.tune_b[prec] = rows_fit<T>(p) ? kStreamShape : kSparseShape;
    return false;
  }
  p.tune_a[prec] = size_shape(p.nb);
  p.tune_b[prec] = (p.B.ns + p.B.nd) <= 8ull * p.nb ? kFusedShape : size_shape(p.na);
  return false;
}

template <typename T, bool kB>
void launch(Problem &p, const Args<T> &a, cudaStream_t s) {
  const int prec = slot_of<T, kB>();
  if (p.tune_a[prec] < 0 || p.tune_b[prec] < 0) autotune<T, kB>(p, a, s);
  launch_shapes<T, kB>(p, a, p.tune_a[prec], p.tune_b[prec], p.split_ab[prec], s);
}

// ---- multi-vector FP32 products (mixed form) --------------------------------------
//
// The FP32 kernels are bound by integer work per element (phase popcount,
// sign flip, gather address), not by FP32 arithmetic.  These variants apply
// one element to NV vectors at once: the phase, the signed value and the
// offset are formed once, then NV loads and NV FMAs follow.  Same sums in the
// same order per vector as the single-vector kernels.

constexpr int kMaxNV = 4;

struct ArgsMV {
  Args<float> a;  // tables, strings and integrals as in the single-vector form
  const float *Cv[kMaxNV];
  const float *CTv[kMaxNV];
  float *Sv[kMaxNV];
};

template <int CPT, int NV, typename Wd, bool kB>
__device__ __forceinline__ void same_spin_row_mv(const SpinTables &Tb, const float *__restrict__ vs,
                                                 const float *__restrict__ vd, const float *__restrict__ Jo,
                                                 uint32_t ldj, const float *const (&In)[kMaxNV], uint32_t ldin,
                                                 uint32_t row, const uint32_t (&col)[CPT], const bool (&ok)[CPT],
                                                 const Wd (&opp)[CPT], FF (&acc)[NV][CPT]) {
  float part[NV][CPT];
#pragma unroll
  for (int n = 0; n < NV; ++n)
#pragma unroll
    for (int c = 0; c < CPT; ++c) part[n][c] = 0.f;
  const uint32_t p0 = ldg(Tb.off_s + row), p1 = ldg(Tb.off_s + row + 1);
  for (uint32_t p = p0; p < p1; ++p) {
    const uint32_t ket = ldg(Tb.ket_s + p), code = ldg(Tb.code_s + p);
    const float v = ldg(vs + p);
    const Wd m = mask_of<kB, Wd>(Tb.mask_s, p);
#pragma unroll
    for (int c = 0; c < CPT; ++c)
      if (ok[c]) {
        const uint32_t off = ket * ldin + col[c];
        const float sv = flip(v + ldg(Jo + (((code >> 16) & 0x7fffu) * ldj + col[c])),
                              par<kB>(opp[c] & m) ^ (code >> 31));
#pragma unroll
        for (int n = 0; n < NV; ++n) part[n][c] = fmaf(sv, ldg(In[n] + off), part[n][c]);
      }
  }
  const uint32_t d0 = ldg(Tb.off_d + row), d1 = ldg(Tb.off_d + row + 1);
  uint32_t p = d0;
  for (; p + 2 <= d1; p += 2) {
    uint32_t ket[2];
    float v[2];
    Wd m[2];
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      ket[u] = ldg(Tb.ket_d + p + u);
      v[u] = ldg(vd + p + u);
      m[u] = mask_of<kB, Wd>(Tb.mask_d, p + u);
    }
#pragma unroll
    for (int c = 0; c < CPT; ++c)
      if (ok[c]) {
        float x[2][NV];
#pragma unroll
        for (int u = 0; u < 2; ++u)
#pragma unroll
          for (int n = 0; n < NV; ++n) x[u][n] = ldg(In[n] + (ket[u] * ldin + col[c]));
#pragma unroll
        for (int u = 0; u < 2; ++u) {
          const float sv = flip(v[u], par<kB>(opp[c] & m[u]));
#pragma unroll
          for (int n = 0; n < NV; ++n) part[n][c] = fmaf(sv, x[u][n], part[n][c]);
        }
      }
  }
  if (p < d1) {
    const uint32_t ket = ldg(Tb.ket_d + p);
    const float v = ldg(vd + p);
    const Wd m = mask_of<kB, Wd>(Tb.mask_d, p);
#pragma unroll
    for (int c = 0; c < CPT; ++c)
      if (ok[c]) {
        const float sv = flip(v, par<kB>(opp[c] & m));
#pragma unroll
        for (int n = 0; n < NV; ++n) part[n][c] = fmaf(sv, ldg(In[n] + (ket * ldin + col[c])), part[n][c]);
      }
  }
#pragma unroll
  for (int n = 0; n < NV; ++n)
#pragma unroll
    for (int c = 0; c < CPT; ++c) ff_add(acc[n][c], part[n][c]);
}

template <int TA, int CPT, int NV, typename Wd, bool kFused, bool kB>
__global__ void __launch_bounds__(kThreads) k_sigma_alpha_mv(ArgsMV m) {
  const Args<float> &a = m.a;
  constexpr int TB = kThreads * CPT;
  uint32_t bt, bc;  // grid order as in k_sigma_alpha
  if constexpr (kFused) {
    const uint32_t nch = (a.nb + TB - 1) / TB;
    bt = blockIdx.x / nch;
    bc = blockIdx.x - bt * nch;
  } else {
    bt = blockIdx.x;
    bc = blockIdx.y;
  }
  const uint32_t tile = ldg(a.tile_order + bt);
  const uint32_t ia0 = ldg(a.tile_start + tile);
  const uint32_t rend = ldg(a.tile_start + tile + 1) - ia0;
  const uint32_t ib0 = bc * TB;
  uint32_t col[CPT], q0[CPT], q1[CPT], d0[CPT], d1[CPT];
  bool ok[CPT];
  Wd beta[CPT];
#pragma unroll
  for (int c = 0; c < CPT; ++c) {
    col[c] = ib0 + threadIdx.x + kThreads * c;
    ok[c] = col[c] < a.nb;
    beta[c] = ok[c] ? word<Wd>(a.bstr, col[c]) : Wd(0);
    q0[c] = ok[c] ? ldg(a.B.off_s + col[c]) : 0u;
    q1[c] = ok[c] ? ldg(a.B.off_s + col[c] + 1) : 0u;
    d0[c] = (kFused && ok[c]) ? ldg(a.B.off_d + col[c]) : 0u;
    d1[c] = (kFused && ok[c]) ? ldg(a.B.off_d + col[c] + 1) : 0u;
  }
#pragma unroll 1
  for (uint32_t r = 0; r < rend; ++r) {
    const uint32_t ia = ia0 + r;
    FF acc[NV][CPT];
#pragma unroll
    for (int c = 0; c < CPT; ++c) {
      const uint32_t k = ia * a.nb + col[c];
      if (a.hii_f) {
        const float h = ok[c] ? ldg(a.hii_f + k) : 0.f;
#pragma unroll
        for (int n = 0; n < NV; ++n) acc[n][c] = ok[c] ? ff_prod(h, ldg(m.Cv[n] + k)) : FF{0.f, 0.f};
      } else {
        const dfloat h = ok[c] ? ldg(a.hii_df + k) : dfloat(0.f, 0.f);
        const float hh = h.hi, hl = h.lo;
#pragma unroll
        for (int n = 0; n < NV; ++n)
          acc[n][c] = ok[c] ? ff_diag(hh, hl, a.shift_df.hi, a.shift_df.lo, ldg(m.Cv[n] + k)) : FF{0.f, 0.f};
      }
    }
    same_spin_row_mv<CPT, NV, Wd, kB>(a.A, a.val_sa, a.val_da, a.Jb, a.nb, m.Cv, a.nb, ia, col, ok, beta, acc);
    float part[NV][CPT];
#pragma unroll
    for (int n = 0; n < NV; ++n)
#pragma unroll
      for (int c = 0; c < CPT; ++c) part[n][c] = 0.f;
    const uint32_t p0 = ldg(a.A.off_s + ia), p1 = a.skip_ab ? p0 : ldg(a.A.off_s + ia + 1);  // skip: k_sigma_ab
    if constexpr (sizeof(Wd) == 8) {
      // 64-bit words: beta singles outside, alpha singles inside (as in
      // k_sigma_alpha); with 32-bit words the extra popcount per term costs
      // more than the loads it saves once NV vectors share them
#pragma unroll
      for (int c = 0; c < CPT; ++c) {
        for (uint32_t q = q0[c]; q < q1[c]; ++q) {
          const uint32_t jb = ldg(a.B.ket_s + q), cb = ldg(a.B.code_s + q);
          const Wd mb = mask_of<kB, Wd>(a.B.mask_s, q);
          const uint32_t kb = (cb >> 16) & 0x7fffu, sb = cb >> 31;
          for (uint32_t p = p0; p < p1; ++p) {
            const uint32_t ja = ldg(a.A.ket_s + p), ca = ldg(a.A.code_s + p);
            const uint32_t ph =
                (par<kB>(beta[c] & mask_of<kB, Wd>(a.A.mask_s, p)) ^ par<kB>(word<Wd>(a.astr, ja) & mb) ^ (ca >> 31) ^ sb) &
                1u;
            const float kv = flip(ldg(a.Kp + ((ca >> 16) & 0x7fffu) * a.npair + kb), ph);
            const uint32_t off = ja * a.nb + jb;
#pragma unroll
            for (int n = 0; n < NV; ++n) part[n][c] = fmaf(kv, ldg(m.Cv[n] + off), part[n][c]);
          }
        }
      }
    } else {
      for (uint32_t p = p0; p < p1; ++p) {
        const uint32_t ja = ldg(a.A.ket_s + p), ca = ldg(a.A.code_s + p);
        const Wd ma = mask_of<kB, Wd>(a.A.mask_s, p);
        const Wd alpha_ket = word<Wd>(a.astr, ja);
        const float *krow = a.Kp + (size_t)((ca >> 16) & 0x7fffu) * a.npair;
        const uint32_t rowoff = ja * a.nb;
#pragma unroll
        for (int c = 0; c < CPT; ++c) {
          const uint32_t pa = par<kB>(beta[c] & ma) ^ (ca >> 31);
          for (uint32_t q = q0[c]; q < q1[c]; ++q) {
            const uint32_t jb = ldg(a.B.ket_s + q), cb = ldg(a.B.code_s + q);
            const uint32_t ph = (pa ^ par<kB>(alpha_ket & mask_of<kB, Wd>(a.B.mask_s, q)) ^ (cb >> 31)) & 1u;
            const float kv = flip(ldg(krow + ((cb >> 16) & 0x7fffu)), ph);
#pragma unroll
            for (int n = 0; n < NV; ++n) part[n][c] = fmaf(kv, ldg(m.Cv[n] + (rowoff + jb)), part[n][c]);
          }
        }
      }
    }
    if constexpr (kFused) {
      const Wd arow = word<Wd>(a.astr, ia);
      const uint32_t rowoff = ia * a.nb;
#pragma unroll
      for (int c = 0; c < CPT; ++c) {
        for (uint32_t q = q0[c]; q < q1[c]; ++q) {
          const uint32_t jb = ldg(a.B.ket_s + q), cb = ldg(a.B.code_s + q);
          const uint32_t ph = par<kB>(arow & mask_of<kB, Wd>(a.B.mask_s, q)) ^ (cb >> 31);
          const float sv = flip(ldg(a.val_sb + q) + ldg(a.Ja + (size_t)((cb >> 16) & 0x7fffu) * a.na + ia), ph);
#pragma unroll
          for (int n = 0; n < NV; ++n) part[n][c] = fmaf(sv, ldg(m.Cv[n] + (rowoff + jb)), part[n][c]);
        }
        for (uint32_t q = d0[c]; q < d1[c]; ++q) {
          const uint32_t jb = ldg(a.B.ket_d + q);
          const float sv = flip(ldg(a.val_db + q), par<kB>(arow & mask_of<kB, Wd>(a.B.mask_d, q)));
#pragma unroll
          for (int n = 0; n < NV; ++n) part[n][c] = fmaf(sv, ldg(m.Cv[n] + (rowoff + jb)), part[n][c]);
        }
      }
    }
#pragma unroll
    for (int c = 0; c < CPT; ++c)
      if (ok[c]) {
        const uint32_t k = ia * a.nb + col[c];
#pragma unroll
        for (int n = 0; n < NV; ++n) {
          ff_add(acc[n][c], part[n][c]);
          m.Sv[n][k] = ff_value(acc[n][c]);
        }
      }
  }
}

template <int TA, int CPT, int NV, typename Wd, bool kB>
__global__ void __launch_bounds__(kThreads) k_sigma_beta_mv(ArgsMV m) {
  const Args<float> &a = m.a;
  constexpr int TB = kThreads * CPT;
  extern __shared__ FF tile_mv[];  // [NV][TA][TB]
  const uint32_t t = ldg(a.tile_order + blockIdx.x);
  const uint32_t ib0 = ldg(a.tile_start + t);
  const uint32_t rend = ldg(a.tile_start + t + 1) - ib0;
  const uint32_t ia0 = blockIdx.y * TB;
  uint32_t col[CPT];
  bool ok[CPT];
  Wd alpha[CPT];
#pragma unroll
  for (int c = 0; c < CPT; ++c) {
    col[c] = ia0 + threadIdx.x + kThreads * c;
    ok[c] = col[c] < a.na;
    alpha[c] = ok[c] ? word<Wd>(a.astr, col[c]) : Wd(0);
  }
#pragma unroll 1
  for (uint32_t r = 0; r < rend; ++r) {
    FF acc[NV][CPT];
#pragma unroll
    for (int n = 0; n < NV; ++n)
#pragma unroll
      for (int c = 0; c < CPT; ++c) acc[n][c] = FF{0.f, 0.f};
    same_spin_row_mv<CPT, NV, Wd, kB>(a.B, a.val_sb, a.val_db, a.Ja, a.na, m.CTv, a.na, ib0 + r, col, ok, alpha, acc);
#pragma unroll
    for (int n = 0; n < NV; ++n)
#pragma unroll
      for (int c = 0; c < CPT; ++c) tile_mv[((size_t)n * TA + r) * TB + threadIdx.x + kThreads * c] = acc[n][c];
  }
#pragma unroll
  for (int c = 0; c < CPT; ++c)
    if (ok[c])
#pragma unroll
      for (int n = 0; n < NV; ++n) {
        float *srow = m.Sv[n] + (size_t)col[c] * a.nb + ib0;
        for (uint32_t r = 0; r < rend; ++r) {
          FF t = tile_mv[((size_t)n * TA + r) * TB + threadIdx.x + kThreads * c];
          ff_add(t, srow[r]);
          srow[r] = ff_value(t);
        }
      }
}

template <int TA, int CPT, int NV, bool F, bool kB>
void launch_a_mv_shape(const Problem &p, const ArgsMV &mv, cudaStream_t s) {
  ArgsMV m = mv;
  constexpr int TB = kThreads * CPT;
  constexpr int v = TA == 8 ? 0 : 1;
  m.a.tile_start = p.tile_start[0][v];
  m.a.tile_order = p.tile_order[0][v];
  const dim3 g = F ? dim3(p.n_tiles[0][v] * ((p.nb + TB - 1) / TB)) : dim3(p.n_tiles[0][v], (p.nb + TB - 1) / TB);
  if (kB || p.norb <= 32)
    k_sigma_alpha_mv<TA, CPT, NV, uint32_t, F, kB><<<g, kThreads, 0, s>>>(m);
  else
    k_sigma_alpha_mv<TA, CPT, NV, unsigned long long, F, kB><<<g, kThreads, 0, s>>>(m);
}
template <int TA, int CPT, int NV, bool kB>
void launch_b_mv_shape(const Problem &p, const ArgsMV &mv, cudaStream_t s) {
  ArgsMV m = mv;
  constexpr int TB = kThreads * CPT;
  constexpr int v = TA == 8 ? 0 : 1;
  m.a.tile_start = p.tile_start[1][v];
  m.a.tile_order = p.tile_order[1][v];
  dim3 g(p.n_tiles[1][v], (p.na + TB - 1) / TB);
  const size_t smem = sizeof(FF) * NV * TA * TB;
  if (kB || p.norb <= 32) {
    auto k = k_sigma_beta_mv<TA, CPT, NV, uint32_t, kB>;
    ensure_dynamic_smem((const void *)k, smem);
    k<<<g, kThreads, smem, s>>>(m);
  } else {
    auto k = k_sigma_beta_mv<TA, CPT, NV, unsigned long long, kB>;
    ensure_dynamic_smem((const void *)k, smem);
    k<<<g, kThreads, smem, s>>>(m);
  }
}
template <int NV, bool F, bool kB>
void launch_a_mv(const Problem &p, const ArgsMV &m, int shape, cudaStream_t s) {
  switch (shape) {
    case 0: launch_a_mv_shape<8, 1, NV, F, kB>(p, m, s); break;
    case 1: launch_a_mv_shape<8, 2, NV, F, kB>(p, m, s); break;
    case 2: launch_a_mv_shape<8, 4, NV, F, kB>(p, m, s); break;
    default: launch_a_mv_shape<16, 2, NV, F, kB>(p, m, s); break;
  }
}
template <int NV, bool kB>
void launch_b_mv(const Problem &p, const ArgsMV &m, int shape, cudaStream_t s) {
  switch (shape) {
    case 0: launch_b_mv_shape<8, 1, NV, kB>(p, m, s); break;
    case 1: launch_b_mv_shape<8, 2, NV, kB>(p, m, s); break;
    case 2: launch_b_mv_shape<8, 4, NV, kB>(p, m, s); break;
    default: launch_b_mv_shape<16, 2, NV, kB>(p, m, s); break;
  }
}
// Kernel B stages NV x TA x TB doubles; shapes whose staging would exceed
// 48 KB (and cut the CTAs per SM) fall back to narrower tiles.
template <int NV>
int shape_b_mv(int tuned) {
  auto fits = [](int sh) { return (size_t)NV * kShapeTA[sh] * kThreads * kShapeCPT[sh] * 8 <= 49152; };
  if (fits(tuned)) return tuned;
  return fits(1) ? 1 : 0;
}

template <int NV, bool kB>
void launch_mv(const Problem &p, const ArgsMV &mv, cudaStream_t s) {
  constexpr int ts = slot_of<float, kB>();
  const bool split = p.split_ab[ts] > 0;
  ArgsMV m = mv;
  m.a.skip_ab = split ? 1 : 0;
  if (p.tune_b[ts] == kSparseShape || p.tune_b[ts] == kStreamShape) {  // one stream per vector
    for (int n = 0; n < NV; ++n) {
      Args<float> a = m.a;
      a.C = m.Cv[n];
      a.S = m.Sv[n];
      if (p.tune_b[ts] == kSparseShape)
        launch_sparse<float, kB>(p, a, p.tune_a[ts], s);
      else
        launch_stream_or_sparse<float, kB>(p, a, p.tune_a[ts], s);
    }
  } else if (p.tune_b[ts] == kFusedShape) {
    launch_a_mv<NV, true, kB>(p, m, p.tune_a[ts], s);
  } else {
    launch_a_mv<NV, false, kB>(p, m, p.tune_a[ts], s);
    launch_b_mv<NV, kB>(p, m, shape_b_mv<NV>(p.tune_b[ts]), s);
  }
  if (split)  // the alpha x beta pairs of each vector in k_sigma_ab
    for (int n = 0; n < NV; ++n) {
      Args<float> a = mv.a;
      a.C = mv.Cv[n];
      a.S = mv.Sv[n];
      launch_ab<float>(p, a, kB, s);
    }
}

template <typename T>
void transpose(Problem &p, const T *in, T *out, uint32_t R, uint32_t Cn, cudaStream_t s) {
  dim3 grid((Cn + 31) / 32, (R + 31) / 32), block(32, 8);
  k_transpose<T><<<grid, block, 0, s>>>(in, out, R, Cn);
  count_launch(p.ctx);
}

void to_float(Problem &p, const double *x, float *y, size_t n, cudaStream_t s) {
  if (n == 0) return;
  unsigned blocks = (unsigned)std::min<size_t>((n + 255) / 256, 4096);
  k_to_float<<<blocks, 256, 0, s>>>(x, y, n);
  count_launch(p.ctx);
}

void to_df(Problem &p, const double *x, dfloat *y, size_t n, cudaStream_t s) {
  if (n == 0) return;
  unsigned blocks = (unsigned)std::min<size_t>((n + 255) / 256, 4096);
  k_split<<<blocks, 256, 0, s>>>(x, y, n);
  count_launch(p.ctx);
}

void begin_timing(Problem &p, cudaStream_t s, cudaEvent_t &ev0, cudaEvent_t &ev1) {
  if (!p.ctx->timing) return;
  ev0 = timing_event(p.ctx);
  ev1 = timing_event(p.ctx);
  SBDGB_CUDA(cudaEventRecord(ev0, s));
}

void end_timing(Problem &p, cudaStream_t s, cudaEvent_t ev0, cudaEvent_t ev1) {
  if (!ev1) return;
  SBDGB_CUDA(cudaEventRecord(ev1, s));
  p.ctx->sigma_events.emplace_back(ev0, ev1);
}

template <typename T>
Args<T> base_args(Problem &p, const T *C, T *S, int accumulate) {
  Args<T> a;
  a.astr = p.astr;
  a.bstr = p.bstr;
  a.na = p.na;
  a.nb = p.nb;
  a.hii = p.hii;
  a.hii_df = p.hii_df;
  a.hii_f = nullptr;
  a.shift_df = dfloat(0.f, 0.f);
  a.C = C;
  a.S = S;
  a.accumulate = accumulate;
  a.shift = 0.0;
  a.A = p.A;
  a.B = p.B;
  a.npair = p.npair;
  return a;
}

// The shift of a mixed-form product as FP32 hi + lo (FP64 kept for the FP64 kernels).
void set_shift(Args<float> &a, double shift) {
  a.shift = shift;
  a.shift_df = dfloat(shift);
}

// Rows [start[t], start[t+1]) of at most cap rows each, closed once their
// work reaches cap times the mean row work, so that a heavy row forms a tile
// of its own; order lists the tiles by decreasing work.
void make_tiles(const std::vector<double> &work, int cap, std::vector<uint32_t> &start,
                std::vector<uint32_t> &order) {
  const size_t n = work.size();
  double total = 0.0;
  for (double w : work) total += w;
  const double target = cap * (n ? total / (double)n : 1.0);
  start.assign(1, 0u);
  std::vector<double> tw;
  double acc = 0.0;
  int rows = 0;
  for (size_t r = 0; r < n; ++r) {
    acc += work[r];
    if (++rows == cap || acc >= target || r + 1 == n) {
      start.push_back((uint32_t)(r + 1));
      tw.push_back(acc);
      acc = 0.0;
      rows = 0;
    }
  }
  order.resize(tw.size());
  for (size_t t = 0; t < tw.size(); ++t) order[t] = (uint32_t)t;
  std::stable_sort(order.begin(), order.end(), [&](uint32_t x, uint32_t y) { return tw[x] > tw[y]; });
}

}  // namespace

template <typename T>
void apply_eta(Problem &p, T *x, int nvec, cudaStream_t s) {
  if (p.N == 0 || nvec <= 0) return;
  const unsigned blocks = (unsigned)std::min<uint64_t>((p.N + 255) / 256, 8192);
  k_eta<T><<<blocks, 256, 0, s>>>(x, p.astr, p.bstr, p.nb, (uint32_t)p.N, nvec);
  count_launch(p.ctx);
  SBDGB_CUDA(cudaGetLastError());
}
template void apply_eta<double>(Problem &, double *, int, cudaStream_t);
template void apply_eta<float>(Problem &, float *, int, cudaStream_t);
template void apply_eta<dfloat>(Problem &, dfloat *, int, cudaStream_t);

// hii as double-float, made once per problem (the FP32 kernels read its hi and
// lo parts, the double-float kernels the pair).
void split_hii(Problem &p, cudaStream_t s) {
  if (p.hii_df) return;
  p.hii_df = (dfloat *)dev_alloc(p, sizeof(dfloat) * (p.N ? p.N : 1));
  to_df(p, p.hii, p.hii_df, p.N, s);
}

// Row tiles of both sigma kernels (alpha rows for kernel A, beta rows for
// kernel B) for the row caps 8 and 16.  A row's work is its same-spin pair
// count, plus for kernel A its alpha singles times the mean number of beta
// singles per string (the alpha-beta term), plus one.
void build_row_tiles(Problem &p, cudaStream_t s) {
  std::vector<uint32_t> os[2], od[2];
  for (int sp = 0; sp < 2; ++sp) {
    const SpinTables &T = sp == 0 ? p.A : p.B;
    os[sp].resize(T.n + 1);
    od[sp].resize(T.n + 1);
    SBDGB_CUDA(cudaMemcpyAsync(os[sp].data(), T.off_s, sizeof(uint32_t) * (T.n + 1), cudaMemcpyDeviceToHost, s));
    SBDGB_CUDA(cudaMemcpyAsync(od[sp].data(), T.off_d, sizeof(uint32_t) * (T.n + 1), cudaMemcpyDeviceToHost, s));
  }
  SBDGB_CUDA(cudaStreamSynchronize(s));
  const double mean_sb = p.nb ? (double)p.B.ns / p.nb : 0.0;
  for (int sp = 0; sp < 2; ++sp) {
    const uint32_t n = sp == 0 ? p.na : p.nb;
    std::vector<double> work(n);
    for (uint32_t r = 0; r < n; ++r) {
      const double singles = os[sp][r + 1] - os[sp][r], doubles = od[sp][r + 1] - od[sp][r];
      work[r] = 1.0 + singles + doubles + (sp == 0 ? singles * mean_sb : 0.0);
    }
    for (int v = 0; v < 2; ++v) {
      std::vector<uint32_t> start, order;
      make_tiles(work, v == 0 ? 8 : 16, start, order);
      p.tile_start[sp][v] = (uint32_t *)dev_alloc(p, sizeof(uint32_t) * start.size());
      p.tile_order[sp][v] = (uint32_t *)dev_alloc(p, sizeof(uint32_t) * order.size());
      p.n_tiles[sp][v] = (uint32_t)order.size();
      SBDGB_CUDA(cudaMemcpyAsync(p.tile_start[sp][v], start.data(), sizeof(uint32_t) * start.size(),
                                 cudaMemcpyHostToDevice, s));
      SBDGB_CUDA(cudaMemcpyAsync(p.tile_order[sp][v], order.data(), sizeof(uint32_t) * order.size(),
                                 cudaMemcpyHostToDevice, s));
    }
  }
  build_ab_order(p, os[0], os[1], s);
  {  // the row kernel: rows with the most alpha pairs first
    std::vector<uint32_t> rows(p.na);
    for (uint32_t r = 0; r < p.na; ++r) rows[r] = r;
    auto w = [&](uint32_t r) { return os[0][r + 1] - os[0][r] + od[0][r + 1] - od[0][r]; };
    std::stable_sort(rows.begin(), rows.end(), [&](uint32_t x, uint32_t y) { return w(x) > w(y); });
    build_row_pairs(p, os[1], od[1], rows, s);
  }
  SBDGB_CUDA(cudaStreamSynchronize(s));  // the host vectors go out of scope
}

void transpose_fp64(Problem &p, const double *in, double *out, uint32_t R, uint32_t Cn, cudaStream_t s) {
  transpose<double>(p, in, out, R, Cn, s);
}

// FP64 sigma with a caller-provided transpose scratch of at least N doubles.
// Makes no allocation: it neither autotunes (it uses the tuned shapes when the
// problem has them, the 8x256 default otherwise) nor records timing events.
void sigma_fp64_scratch(Problem &p, const double *C, double *S, int accumulate, double *CT, cudaStream_t s) {
  if (!p.tables || !p.diag) throw Error(SBDGB_E_STATE, "sigma needs tables and diagonal");
  if (p.N == 0) return;
  Args<double> a = base_args<double>(p, C, S, accumulate);
  a.CT = CT;
  a.val_sa = p.A.val_s;
  a.val_da = p.A.val_d;
  a.val_sb = p.B.val_s;
  a.val_db = p.B.val_d;
  a.Jb = p.Jb;
  a.Ja = p.Ja;
  a.Kp = p.Kp;
  const int sa = p.tune_a[0] >= 0 ? p.tune_a[0] : 1, sb = p.tune_b[0] >= 0 ? p.tune_b[0] : 1;
  if (needs_transpose(sb)) transpose<double>(p, C, CT, p.na, p.nb, s);
  launch_shapes<double, false>(p, a, sa, sb, p.tune_a[0] >= 0 ? p.split_ab[0] : 0, s);
}

namespace {
// One product with the problem's tuned shapes (tuning first if needed), timed
// when the context records sigma timing; CT is the transpose scratch.
template <typename T, bool kB>
void run_sigma(Problem &p, const Args<T> &a, T *CT, cudaStream_t s) {
  constexpr int ts = slot_of<T, kB>();
  if (needs_tuning<T, kB>(p)) {
    transpose<T>(p, a.C, CT, p.na, p.nb, s);
    autotune<T, kB>(p, a, s);
  }
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  begin_timing(p, s, ev0, ev1);
  if (needs_transpose(p.tune_b[ts])) transpose<T>(p, a.C, CT, p.na, p.nb, s);
  launch<T, kB>(p, a, s);
  end_timing(p, s, ev0, ev1);
}
}  // namespace

void sigma_fp64(Problem &p, const double *C, double *S, int accumulate, cudaStream_t s, bool block) {
  if (!p.tables || !p.diag) throw Error(SBDGB_E_STATE, "sigma needs tables and diagonal");
  if (!p.CT) p.CT = (double *)dev_alloc(p, sizeof(double) * p.N);
  if (p.N == 0) return;
  Args<double> a = base_args<double>(p, C, S, accumulate);
  a.CT = p.CT;
  a.val_sa = p.A.val_s;
  a.val_da = p.A.val_d;
  a.val_sb = p.B.val_s;
  a.val_db = p.B.val_d;
  a.Jb = p.Jb;
  a.Ja = p.Ja;
  a.Kp = p.Kp;
  if (block)
    run_sigma<double, true>(p, a, p.CT, s);
  else
    run_sigma<double, false>(p, a, p.CT, s);
}

// Double-float copies of the table values and integral tables, for the
// double-float phase of the mixed form.
void prepare_df(Problem &p, cudaStream_t s) {
  if (p.df_ready) return;
  if (!p.tables || !p.diag) throw Error(SBDGB_E_STATE, "double-float sigma needs tables and diagonal");
  split_hii(p, s);
  const size_t npp = (size_t)p.npair * p.npair;
  p.Kpd = (dfloat *)dev_alloc(p, sizeof(dfloat) * npp);
  p.Jbd = (dfloat *)dev_alloc(p, sizeof(dfloat) * (size_t)p.npair * p.nb);
  p.Jad = (dfloat *)dev_alloc(p, sizeof(dfloat) * (size_t)p.npair * p.na);
  to_df(p, p.Kp, p.Kpd, npp, s);
  to_df(p, p.Jb, p.Jbd, (size_t)p.npair * p.nb, s);
  to_df(p, p.Ja, p.Jad, (size_t)p.npair * p.na, s);
  for (int sp = 0; sp < 2; ++sp) {
    SpinTables &T = sp == 0 ? p.A : p.B;
    p.val_sd[sp] = (dfloat *)dev_alloc(p, sizeof(dfloat) * (T.ns ? T.ns : 1));
    p.val_dd[sp] = (dfloat *)dev_alloc(p, sizeof(dfloat) * (T.nd ? T.nd : 1));
    to_df(p, T.val_s, p.val_sd[sp], T.ns, s);
    to_df(p, T.val_d, p.val_dd[sp], T.nd, s);
  }
  SBDGB_CUDA(cudaGetLastError());
  SBDGB_CUDA(cudaStreamSynchronize(s));
  p.df_ready = true;
}

// (H - shift) C in double-float (or accumulated into S): the same kernels as
// the FP64 form with double-float values, products and sums.
void sigma_df(Problem &p, const dfloat *C, dfloat *S, int accumulate, cudaStream_t s, double shift, bool block) {
  prepare_df(p, s);
  if (!p.CT) p.CT = (double *)dev_alloc(p, sizeof(double) * p.N);  // the FP64 transpose scratch, same size
  if (p.N == 0) return;
  Args<dfloat> a = base_args<dfloat>(p, C, S, accumulate);
  a.shift_df = dfloat(shift);
  dfloat *CT = reinterpret_cast<dfloat *>(p.CT);
  a.CT = CT;
  a.val_sa = p.val_sd[0];
  a.val_da = p.val_dd[0];
  a.val_sb = p.val_sd[1];
  a.val_db = p.val_dd[1];
  a.Jb = p.Jbd;
  a.Ja = p.Jad;
  a.Kp = p.Kpd;
  if (block)
    run_sigma<dfloat, true>(p, a, CT, s);
  else
    run_sigma<dfloat, false>(p, a, CT, s);
}

// FP32 copies of the table values and integral tables used by the mixed form.
void prepare_mixed(Problem &p, cudaStream_t s) {
  if (p.mixed_ready) return;
  if (!p.tables || !p.diag) throw Error(SBDGB_E_STATE, "mixed sigma needs tables and diagonal");
  const size_t npp = (size_t)p.npair * p.npair;
  p.Kpf = (float *)dev_alloc(p, sizeof(float) * npp);
  p.Jbf = (float *)dev_alloc(p, sizeof(float) * (size_t)p.npair * p.nb);
  p.Jaf = (float *)dev_alloc(p, sizeof(float) * (size_t)p.npair * p.na);
  to_float(p, p.Kp, p.Kpf, npp, s);
  to_float(p, p.Jb, p.Jbf, (size_t)p.npair * p.nb, s);
  to_float(p, p.Ja, p.Jaf, (size_t)p.npair * p.na, s);
  split_hii(p, s);
  p.hii_f = (float *)dev_alloc(p, sizeof(float) * (p.N ? p.N : 1));
  to_float(p, p.hii, p.hii_f, p.N, s);
  for (int sp = 0; sp < 2; ++sp) {
    SpinTables &T = sp == 0 ? p.A : p.B;
    p.val_sf[sp] = (float *)dev_alloc(p, sizeof(float) * (T.ns ? T.ns : 1));
    p.val_df[sp] = (float *)dev_alloc(p, sizeof(float) * (T.nd ? T.nd : 1));
    to_float(p, T.val_s, p.val_sf[sp], T.ns, s);
    to_float(p, T.val_d, p.val_df[sp], T.nd, s);
  }
  SBDGB_CUDA(cudaGetLastError());
  SBDGB_CUDA(cudaStreamSynchronize(s));
  p.mixed_ready = true;
}

namespace {
Args<float> mixed_args(Problem &p, const float *C, float *S, double shift) {
  Args<float> a = base_args<float>(p, C, S, 0);
  set_shift(a, shift);
  a.hii_f = shift == 0.0 ? p.hii_f : nullptr;
  a.CT = p.CTf;
  a.val_sa = p.val_sf[0];
  a.val_da = p.val_df[0];
  a.val_sb = p.val_sf[1];
  a.val_db = p.val_df[1];
  a.Jb = p.Jbf;
  a.Ja = p.Jaf;
  a.Kp = p.Kpf;
  return a;
}
}  // namespace

void sigma_mixed(Problem &p, const float *C, float *S, cudaStream_t s, double shift, bool block) {
  prepare_mixed(p, s);
  if (!p.CTf) p.CTf = (float *)dev_alloc(p, sizeof(float) * p.N);
  if (p.N == 0) return;
  const Args<float> a = mixed_args(p, C, S, shift);
  if (block)
    run_sigma<float, true>(p, a, p.CTf, s);
  else
    run_sigma<float, false>(p, a, p.CTf, s);
}

namespace {
template <bool kB>
void sigma_mixed_multi_impl(Problem &p, const float *C, float *S, int nvec, cudaStream_t s, double shift) {
  constexpr int ts = slot_of<float, kB>();
  if (needs_tuning<float, kB>(p)) sigma_mixed(p, C, S, s, shift, kB);  // tunes the FP32 shapes on the first vector
  ArgsMV m{};
  m.a = mixed_args(p, C, S, shift);
  const bool fused = !needs_transpose(p.tune_b[ts]);
  float *CT = fused ? nullptr : (float *)workspace(p, WS_CTMV, sizeof(float) * p.N * (size_t)nvec);
  for (int n = 0; n < nvec; ++n) {
    m.Cv[n] = C + (size_t)n * p.N;
    m.Sv[n] = S + (size_t)n * p.N;
    m.CTv[n] = fused ? nullptr : CT + (size_t)n * p.N;
    if (!fused) transpose<float>(p, m.Cv[n], CT + (size_t)n * p.N, p.na, p.nb, s);
  }
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  begin_timing(p, s, ev0, ev1);
  switch (nvec) {
    case 2: launch_mv<2, kB>(p, m, s); break;
    case 3: launch_mv<3, kB>(p, m, s); break;
    default: launch_mv<4, kB>(p, m, s); break;
  }
  end_timing(p, s, ev0, ev1);
  count_launch(p.ctx, (p.tune_b[ts] == kSparseShape || p.tune_b[ts] == kStreamShape) ? nvec : fused ? 1 : 2);
  // (k_sigma_ab counts its own launches)
  SBDGB_CUDA(cudaGetLastError());
}
}  // namespace

// (H - shift) C_j for nvec FP32 vectors at once (nvec <= 4; vectors and
// results at stride N), through the multi-vector kernels.
void sigma_mixed_multi(Problem &p, const float *C, float *S, int nvec, cudaStream_t s, double shift, bool block) {
  if (nvec <= 0) return;
  if (nvec == 1) {
    sigma_mixed(p, C, S, s, shift, block);
    return;
  }
  SBDGB_REQUIRE(nvec <= kMaxNV, SBDGB_E_UNSUPPORTED, "at most 4 vectors per multi-vector sigma");
  prepare_mixed(p, s);
  if (!p.CTf) p.CTf = (float *)dev_alloc(p, sizeof(float) * p.N);
  if (p.N == 0) return;
  if (block)
    sigma_mixed_multi_impl<true>(p, C, S, nvec, s, shift);
  else
    sigma_mixed_multi_impl<false>(p, C, S, nvec, s, shift);
}

}  // namespace sbdgb
