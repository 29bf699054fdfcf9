// sigma for problems with few nonzeros per row (norb 58, 12000 x 12000
// strings: 0.48 per row), where the product is a stream over hii, C and
// sigma (chemistry/tpb/mult.h:440-558, every task type in one pass).
//
// One CTA owns one whole alpha row.  The row's beta pairs (task type 1,
// mult.h:489-525: sigma[ia][ib] += +/- v * C[ia][jb]) read C along the same
// row at other columns, so the CTA first stages the row of C in shared memory
// (16-byte loads), and every beta pair of the problem is then one lane's
// product with a shared-memory operand.
//
// Beta pairs are a flat list of all columns' singles and doubles in column
// order (built once per problem, build_row_pairs), padded so that no column's
// run of pairs crosses a 32-entry boundary.  On every row lane e takes pair e:
// the products are dense (every lane busy), a segmented warp sum over each
// column's run (log2 of the longest run in steps) leaves the column's total
// in the run's last lane, and that lane adds it to the column's partial sum in
// shared memory.  The owner of a column never loops over a per-column list.
// That matters for the FP64 product: on this GPU a warp's FP64 instruction
// holds the FP64 pipe 16 cycles whatever its active lanes, about the time the
// SM's share of HBM takes to stream two elements, so per-lane loops whose
// lanes are mostly idle (most columns have no pair) cost as much FP64 time as
// full ones.  Here the FP64 instructions per row are the diagonal's (one per
// element), one per pair product, the short scan and one add per run.
//
// Steps per row: (1) the row of C to shared memory; (2) the beta pairs'
// products and run sums (kept in registers); (3) each thread's columns: the
// diagonal, alpha pairs (type 2, :450-488; warp-uniform table loads, C rows
// read as 16-byte vectors) and alpha x beta pairs (type 0, :527-557), into a
// second shared row (so (2) and (3) need no barrier between them and their
// loads overlap); (4) the runs' totals added; (5) the row written out.
// Deterministic: fixed summation order, no atomics.
#include <algorithm>

#include "common.cuh"
#include "sigma_dev.cuh"

namespace sbdgb {

namespace {

using namespace sdev;
constexpr int kRowEntries = 4096;  // beta pair entries (padding included) the row kernels hold

__device__ __forceinline__ double shfl_up(double v, int d) { return __shfl_up_sync(0xffffffffu, v, d); }
__device__ __forceinline__ float shfl_up(float v, int d) { return __shfl_up_sync(0xffffffffu, v, d); }
__device__ __forceinline__ dfloat shfl_up(dfloat v, int d) {
  return dfloat(__shfl_up_sync(0xffffffffu, v.hi, d), __shfl_up_sync(0xffffffffu, v.lo, d));
}

// VW elements from shared memory in one access (16 bytes when VW > 1).
template <int VW, typename T>
__device__ __forceinline__ void lds_v(const T *p, T (&x)[VW]) {
  static_assert(VW == 1 || sizeof(T) * VW == 16, "shared vectors of 16 bytes");
  if constexpr (VW == 1) {
    x[0] = *p;
  } else {
    const uint4 u = *reinterpret_cast<const uint4 *>(p);
    memcpy(x, &u, 16);
  }
}

struct RowPairs {
  const uint4 *ent;  // {column, ket column, info = single | P << 1 | phase << 31, table index}
  uint32_t n;        // entries, padding included
  uint32_t maxrun;   // longest run of one column's entries (<= 32)
};

// The alpha singles (with their alpha x beta pairs, task types 2 and 0) and
// alpha doubles of row ia for columns c .. c + VW - 1 of one thread, added
// into acc / part in table order.  beta: the columns' beta words
// (interleaved ordering only).
template <int VW, typename T, typename Wd, bool kB>
__device__ __forceinline__ void alpha_pairs(const Args<T> &a, uint32_t c, const Wd (&beta)[VW], AccT<T> (&acc)[VW],
                                            T (&part)[VW], uint32_t p0, uint32_t p1, uint32_t e0, uint32_t e1) {
  for (uint32_t p = p0; p < p1; ++p) {
    const uint32_t ja = ldg(a.A.ket_s + p), code = ldg(a.A.code_s + p);
    const T val = ldg(a.val_sa + p);
    const Wd m = mask_of<kB, Wd>(a.A.mask_s, p);
    const uint32_t P = (code >> 16) & 0x7fffu;
    T y[VW], j[VW];
    load_v<VW>(a.C + (size_t)ja * a.nb + c, y);
    load_v<VW>(a.Jb + (size_t)P * a.nb + c, j);
#pragma unroll
    for (int v = 0; v < VW; ++v) madd(acc[v], part[v], flip(val + j[v], par<kB>(beta[v] & m) ^ (code >> 31)), y[v]);
    if (!a.skip_ab) {
      const Wd aket = word<Wd>(a.astr, ja);
      const T *krow = a.Kp + (size_t)P * a.npair;
#pragma unroll
      for (int v = 0; v < VW; ++v) {
        const uint32_t q0 = ldg(a.B.off_s + c + v), q1 = ldg(a.B.off_s + c + v + 1);
        for (uint32_t q = q0; q < q1; ++q) {
          const uint32_t jb = ldg(a.B.ket_s + q), cb = ldg(a.B.code_s + q);
          const uint32_t ph =
              (par<kB>(beta[v] & m) ^ par<kB>(aket & mask_of<kB, Wd>(a.B.mask_s, q)) ^ (code >> 31) ^ (cb >> 31)) & 1u;
          madd(acc[v], part[v], flip(ldg(krow + ((cb >> 16) & 0x7fffu)), ph), ldg(a.C + (size_t)ja * a.nb + jb));
        }
      }
    }
  }
  for (uint32_t p = e0; p < e1; ++p) {
    const uint32_t ja = ldg(a.A.ket_d + p);
    const T val = ldg(a.val_da + p);
    const Wd m = mask_of<kB, Wd>(a.A.mask_d, p);
    T y[VW];
    load_v<VW>(a.C + (size_t)ja * a.nb + c, y);
#pragma unroll
    for (int v = 0; v < VW; ++v) madd(acc[v], part[v], flip(val, par<kB>(beta[v] & m)), y[v]);
  }
}

// Steps (2)-(5) of one row, with the row of C staged in Cs.  Ss receives the
// row of sigma; Hs, when not null, is the row of hii staged in FP32 (the
// unshifted FP32 product) and may be Ss itself (each thread reads its own
// columns' hii before writing their sigma).  kInPlace: Ss is Cs, so a barrier
// separates the pair products (any column of C) from step (3) (each thread
// reads its own columns of C, then overwrites them).  kStagedH: Hs is never
// null (the pipelined FP32 kernel), which enables the one-multiply branch for
// rows without alpha pairs.  Ends with the row stored.
template <int NT, int VW, typename T, typename Wd, bool kB, bool kInPlace = false, bool kStagedH = false>
__device__ __forceinline__ void row_steps(const Args<T> &a, const RowPairs &rp, uint32_t ia, const T *Cs, T *Ss,
                                          const float *Hs) {
  const size_t rk = (size_t)ia * a.nb;
  const uint32_t tid = threadIdx.x, lane = tid & 31u;
  const Wd arow = kB ? Wd(0) : word<Wd>(a.astr, ia);
  // (2) the beta pairs: products and run sums
  constexpr int RC = kRowEntries / NT;  // pair chunks per thread, held in registers
  T tot[RC];
  uint32_t key[RC];
#pragma unroll
  for (int k = 0; k < RC; ++k) {
    tot[k] = T(0);
    key[k] = ~0u;
  }
#pragma unroll
  for (int k = 0; k < RC; ++k) {
    if ((uint32_t)k * NT + (tid & ~31u) >= rp.n) break;  // warp-uniform
    const uint32_t e = tid + (uint32_t)k * NT;
    T t = T(0);
    uint32_t kk = ~0u;
    if (e < rp.n) {
      const uint4 en = ldg(rp.ent + e);
      kk = en.x;
      if (kk != ~0u) {
        if (en.z & 1u) {
          const T j = ldg(a.Ja + (size_t)((en.z >> 1) & 0x7fffu) * a.na + ia);
          t = flip(ldg(a.val_sb + en.w) + j, par<kB>(arow & mask_of<kB, Wd>(a.B.mask_s, en.w)) ^ (en.z >> 31)) *
              Cs[en.y];
        } else {
          t = flip(ldg(a.val_db + en.w), par<kB>(arow & mask_of<kB, Wd>(a.B.mask_d, en.w))) * Cs[en.y];
        }
      }
    }
    for (uint32_t d = 1; d < rp.maxrun; d <<= 1) {
      const T u = shfl_up(t, (int)d);
      const uint32_t ku = __shfl_up_sync(0xffffffffu, kk, (int)d);
      if (lane >= d && ku == kk) t = t + u;
    }
    const uint32_t kn = __shfl_down_sync(0xffffffffu, kk, 1);
    tot[k] = t;
    key[k] = (kk != ~0u && (lane == 31u || kn != kk)) ? kk : ~0u;  // run tails only
  }
  if constexpr (kInPlace) __syncthreads();
  // (3) each thread's columns into the sigma row (no barrier before: the
  // pairs above only read the C row, so their loads and these overlap)
  const uint32_t p0 = ldg(a.A.off_s + ia), p1 = ldg(a.A.off_s + ia + 1);
  const uint32_t e0 = ldg(a.A.off_d + ia), e1 = ldg(a.A.off_d + ia + 1);
  if constexpr (sizeof(T) == 8) {
    // FP64 and double-float: hii comes from global memory, so the diagonal
    // goes first with several chunks' loads in flight, and the alpha pairs
    // (few rows of a sparse problem have any) are added to it afterwards:
    // the same order of operations as one pass.
    constexpr int U = 2;
    for (uint32_t c0 = tid * VW; c0 < a.nb; c0 += U * NT * VW) {
      T h[U][VW];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const uint32_t c = c0 + (uint32_t)u * NT * VW;
        if (c < a.nb) {
          if constexpr (std::is_same<T, double>::value) load_v<VW>(a.hii + rk + c, h[u]);
          else load_v<VW>(a.hii_df + rk + c, h[u]);
        }
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const uint32_t c = c0 + (uint32_t)u * NT * VW;
        if (c < a.nb) {
          T x[VW], out[VW];
          lds_v<VW>(Cs + c, x);
#pragma unroll
          for (int v = 0; v < VW; ++v) {
            if constexpr (std::is_same<T, double>::value) out[v] = h[u][v] * x[v];
            else out[v] = (h[u][v] - a.shift_df) * x[v];
          }
          store_v<VW>(Ss + c, out);
        }
      }
    }
    if (p1 > p0 || e1 > e0) {
      for (uint32_t c = tid * VW; c < a.nb; c += NT * VW) {
        T acc[VW], part[VW];
        Wd beta[VW];
        lds_v<VW>(Ss + c, acc);
#pragma unroll
        for (int v = 0; v < VW; ++v) {
          part[v] = T(0);
          beta[v] = kB ? Wd(0) : word<Wd>(a.bstr, c + v);
        }
        alpha_pairs<VW, T, Wd, kB>(a, c, beta, acc, part, p0, p1, e0, e1);
        store_v<VW>(Ss + c, acc);
      }
    }
  } else if (kStagedH && p1 == p0 && e1 == e0) {
    // FP32, unshifted, a row without alpha pairs: the float-float
    // accumulator of the general branch would hold h x exactly as hi + lo and
    // round it back to fl(h x), so one multiply gives the same bits
    for (uint32_t c = tid * VW; c < a.nb; c += NT * VW) {
      float h[VW], x[VW], out[VW];
      lds_v<VW>(Cs + c, x);
      lds_v<VW>(Hs + c, h);
#pragma unroll
      for (int v = 0; v < VW; ++v) out[v] = h[v] * x[v];
      store_v<VW>(Ss + c, out);
    }
  } else {
    // FP32: each column's diagonal (hii staged in shared memory or read as
    // FP32 or as the shifted hi/lo pair) and its alpha pairs in one pass,
    // into float-float accumulators
    for (uint32_t c = tid * VW; c < a.nb; c += NT * VW) {
      const size_t k = rk + c;
      AccT<T> acc[VW];
      T part[VW];
      T x[VW];
      Wd beta[VW];
      lds_v<VW>(Cs + c, x);
#pragma unroll
      for (int v = 0; v < VW; ++v) {
        part[v] = T(0);
        beta[v] = kB ? Wd(0) : word<Wd>(a.bstr, c + v);  // only the alpha pairs' phases use it
      }
      if (Hs) {
        float h[VW];
        lds_v<VW>(Hs + c, h);
#pragma unroll
        for (int v = 0; v < VW; ++v) acc[v] = ff_prod(h[v], x[v]);
      } else if (a.hii_f) {
        float h[VW];
        load_v<VW>(a.hii_f + k, h);
#pragma unroll
        for (int v = 0; v < VW; ++v) acc[v] = ff_prod(h[v], x[v]);
      } else {
        dfloat h[VW];
        load_v<VW>(a.hii_df + k, h);
#pragma unroll
        for (int v = 0; v < VW; ++v) acc[v] = ff_diag(h[v].hi, h[v].lo, a.shift_df.hi, a.shift_df.lo, x[v]);
      }
      alpha_pairs<VW, T, Wd, kB>(a, c, beta, acc, part, p0, p1, e0, e1);
      T out[VW];
#pragma unroll
      for (int v = 0; v < VW; ++v) {
        acc_add_part(acc[v], part[v]);
        out[v] = (T)acc_value(acc[v]);
      }
      store_v<VW>(Ss + c, out);
    }
  }
  __syncthreads();
  // (4) the beta pairs' run totals
#pragma unroll
  for (int k = 0; k < RC; ++k)
    if (key[k] != ~0u) Ss[key[k]] = Ss[key[k]] + tot[k];
  __syncthreads();
  // (5) the row out
  for (uint32_t c = tid * VW; c < a.nb; c += NT * VW) {
    T out[VW];
    lds_v<VW>(Ss + c, out);
    if (a.accumulate) {
      T old[VW];
      load_v<VW>(a.S + rk + c, old);
#pragma unroll
      for (int v = 0; v < VW; ++v) out[v] = old[v] + out[v];
    }
    store_v<VW>(a.S + rk + c, out);
  }
}


// One row per CTA: the row of C loaded into shared memory, then its steps.
template <int NT, int VW, typename T, typename Wd, bool kB>
__global__ void __launch_bounds__(NT) k_sigma_rows(Args<T> a, RowPairs rp) {
  extern __shared__ __align__(16) unsigned char rows_smem[];
  T *Cs = reinterpret_cast<T *>(rows_smem);  // the row of C
  T *Ss = Cs + a.nb;                          // the row of sigma being formed
  const uint32_t ia = ldg(a.tile_order + blockIdx.x);  // rows, most alpha pairs first
  const size_t rk = (size_t)ia * a.nb;
  // (1) the row of C
  for (uint32_t c = threadIdx.x * VW; c < a.nb; c += NT * VW) {
    T x[VW];
    load_v<VW>(a.C + rk + c, x);
#pragma unroll
    for (int v = 0; v < VW; ++v) Cs[c + v] = x[v];
  }
  __syncthreads();
  row_steps<NT, VW, T, Wd, kB>(a, rp, ia, Cs, Ss, nullptr);
}

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
  const uint32_t sa = (uint32_t)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// The unshifted FP32 product, persistent: each CTA takes rows blockIdx.x,
// + gridDim.x, ...  The next row's C and hii are copied into the other half of
// a double buffer (cp.async, 16 bytes per thread and copy) while the current
// row is computed, so the row's streaming loads are off the critical path;
// the staged hii row is overwritten by the sigma row.  Needs 16 nb bytes of
// shared memory, nb a multiple of 4 and 16-byte aligned rows.
template <int NT, typename Wd, bool kB>
__global__ void __launch_bounds__(NT) k_sigma_rows_pipe(Args<float> a, RowPairs rp) {
  constexpr int VW = 4;
  extern __shared__ __align__(16) unsigned char rows_smem[];
  float *Cb[2], *Hb[2];
  Cb[0] = reinterpret_cast<float *>(rows_smem);
  Cb[1] = Cb[0] + a.nb;
  Hb[0] = Cb[1] + a.nb;
  Hb[1] = Hb[0] + a.nb;
  auto stage = [&](int slot, uint32_t ia) {
    const size_t rk = (size_t)ia * a.nb;
    for (uint32_t c = threadIdx.x * VW; c < a.nb; c += NT * VW) {
      cp_async16(Cb[slot] + c, a.C + rk + c);
      cp_async16(Hb[slot] + c, a.hii_f + rk + c);
    }
    cp_async_commit();
  };
  uint32_t i = blockIdx.x;
  if (i < a.na) stage(0, ldg(a.tile_order + i));
  for (int slot = 0; i < a.na; i += gridDim.x, slot ^= 1) {
    cp_async_wait_all();  // this row's copies (the only ones in flight)
    __syncthreads();      // ... visible to all, and every thread is done with the other half
    if (i + gridDim.x < a.na) stage(slot ^ 1, ldg(a.tile_order + i + gridDim.x));
    row_steps<NT, VW, float, Wd, kB, false, true>(a, rp, ldg(a.tile_order + i), Cb[slot], Hb[slot], Hb[slot]);
  }
}

// The same for the 8-byte products (FP64, double-float): two C rows fill
// 16 nb bytes, so the sigma row is formed in place of the current C row and
// hii is read from global memory.  nb a multiple of 2 and 16-byte aligned rows.
template <int NT, typename T, typename Wd, bool kB>
__global__ void __launch_bounds__(NT) k_sigma_rows_pipe8(Args<T> a, RowPairs rp) {
  static_assert(sizeof(T) == 8, "8-byte products");
  constexpr int VW = 2;
  extern __shared__ __align__(16) unsigned char rows_smem[];
  T *Cb[2];
  Cb[0] = reinterpret_cast<T *>(rows_smem);
  Cb[1] = Cb[0] + a.nb;
  auto stage = [&](int slot, uint32_t ia) {
    const size_t rk = (size_t)ia * a.nb;
    for (uint32_t c = threadIdx.x * VW; c < a.nb; c += NT * VW) cp_async16(Cb[slot] + c, a.C + rk + c);
    cp_async_commit();
  };
  uint32_t i = blockIdx.x;
  if (i < a.na) stage(0, ldg(a.tile_order + i));
  for (int slot = 0; i < a.na; i += gridDim.x, slot ^= 1) {
    cp_async_wait_all();
    __syncthreads();
    if (i + gridDim.x < a.na) stage(slot ^ 1, ldg(a.tile_order + i + gridDim.x));
    row_steps<NT, VW, T, Wd, kB, true>(a, rp, ldg(a.tile_order + i), Cb[slot], Cb[slot], nullptr);
  }
}

template <typename T>
size_t rows_smem(const Problem &p) {
  return 2 * sizeof(T) * (size_t)p.nb;  // the row of C and the row of sigma
}

template <typename T, int NT, typename Wd, bool kB>
void launch_rows_nt(const Problem &p, Args<T> a, cudaStream_t s) {
  constexpr int VW = 16 / (int)sizeof(T);
  a.tile_order = p.rp_rows;
  const RowPairs rp{p.rp_ent, p.rp_n, p.rp_maxrun};
  const size_t smem = rows_smem<T>(p);
  auto al = [](const void *x) { return ((uintptr_t)x & 15u) == 0; };
  const bool vec = p.nb % VW == 0 && al(a.C) && al(a.S) && al(a.Jb) &&
                   (std::is_same<T, double>::value ? al(a.hii) : al(a.hii_df)) && (a.hii_f == nullptr || al(a.hii_f));
  if (vec) {
    auto k = k_sigma_rows<NT, VW, T, Wd, kB>;
    ensure_dynamic_smem((const void *)k, smem);
    prefer_shared_carveout((const void *)k);
    k<<<p.na, NT, smem, s>>>(a, rp);
  } else {
    auto k = k_sigma_rows<NT, 1, T, Wd, kB>;
    ensure_dynamic_smem((const void *)k, smem);
    prefer_shared_carveout((const void *)k);
    k<<<p.na, NT, smem, s>>>(a, rp);
  }
}

}  // namespace

// The flat beta pair list of the row kernel: each column's singles, then its
// doubles, columns in order, runs padded not to cross 32-entry boundaries.
// Built when no column has more than 32 beta pairs; otherwise the kernel is
// not used.  rows: the alpha rows in the order the CTAs take them.
void build_row_pairs(Problem &p, const std::vector<uint32_t> &off_s, const std::vector<uint32_t> &off_d,
                     const std::vector<uint32_t> &rows, cudaStream_t s) {
  p.rp_n = 0;
  p.rp_ready = false;
  uint32_t maxrun = 1;
  for (uint32_t c = 0; c < p.nb; ++c) maxrun = std::max(maxrun, off_s[c + 1] - off_s[c] + off_d[c + 1] - off_d[c]);
  if (maxrun > 32u || p.npair >= 32768) return;
  std::vector<uint32_t> ks(p.B.ns), cs(p.B.ns), kd(p.B.nd);
  if (p.B.ns) {
    SBDGB_CUDA(cudaMemcpyAsync(ks.data(), p.B.ket_s, sizeof(uint32_t) * p.B.ns, cudaMemcpyDeviceToHost, s));
    SBDGB_CUDA(cudaMemcpyAsync(cs.data(), p.B.code_s, sizeof(uint32_t) * p.B.ns, cudaMemcpyDeviceToHost, s));
  }
  if (p.B.nd) SBDGB_CUDA(cudaMemcpyAsync(kd.data(), p.B.ket_d, sizeof(uint32_t) * p.B.nd, cudaMemcpyDeviceToHost, s));
  SBDGB_CUDA(cudaStreamSynchronize(s));
  std::vector<uint4> ent;
  ent.reserve(p.B.ns + p.B.nd + 64);
  const uint4 pad = make_uint4(~0u, 0u, 0u, 0u);
  for (uint32_t c = 0; c < p.nb; ++c) {
    const uint32_t n = off_s[c + 1] - off_s[c] + off_d[c + 1] - off_d[c];
    if (n == 0) continue;
    if (ent.size() % 32 + n > 32) ent.resize((ent.size() + 31) / 32 * 32, pad);
    for (uint32_t q = off_s[c]; q < off_s[c + 1]; ++q)
      ent.push_back(make_uint4(c, ks[q], 1u | ((cs[q] >> 16) & 0x7fffu) << 1 | (cs[q] & 0x80000000u), q));
    for (uint32_t q = off_d[c]; q < off_d[c + 1]; ++q) ent.push_back(make_uint4(c, kd[q], 0u, q));
  }
  p.rp_ent = (uint4 *)dev_alloc(p, sizeof(uint4) * std::max<size_t>(ent.size(), 1));
  p.rp_rows = (uint32_t *)dev_alloc(p, sizeof(uint32_t) * std::max<size_t>(rows.size(), 1));
  if (!ent.empty())
    SBDGB_CUDA(cudaMemcpyAsync(p.rp_ent, ent.data(), sizeof(uint4) * ent.size(), cudaMemcpyHostToDevice, s));
  if (!rows.empty())
    SBDGB_CUDA(cudaMemcpyAsync(p.rp_rows, rows.data(), sizeof(uint32_t) * rows.size(), cudaMemcpyHostToDevice, s));
  SBDGB_CUDA(cudaStreamSynchronize(s));  // the host vectors go out of scope
  p.rp_n = (uint32_t)ent.size();
  p.rp_maxrun = maxrun;
  p.rp_ready = true;
}

template <typename T>
bool rows_fit(const Problem &p) {
  if (!p.rp_ready) return false;
  if ((size_t)p.rp_n > (size_t)kRowEntries) return false;  // more pair entries than the kernels hold
  int dev = 0, optin = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return false;
  if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return false;
  return rows_smem<T>(p) <= (size_t)optin;
}

// The pipelined form when it applies (16-byte rows, 16 nb bytes of shared
// memory; for FP32 the unshifted product); false otherwise.
template <typename T, typename Wd, bool kB>
bool launch_rows_pipe(const Problem &p, Args<T> a, cudaStream_t s) {
  auto al = [](const void *x) { return ((uintptr_t)x & 15u) == 0; };
  int dev = 0, optin = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return false;
  const size_t smem = 16 * (size_t)p.nb;
  const unsigned grid = (unsigned)std::min<uint32_t>(p.na, (uint32_t)sms);
  if (smem > (size_t)optin || !al(a.C) || !al(a.S) || !al(a.Jb)) return false;
  a.tile_order = p.rp_rows;
  const RowPairs rp{p.rp_ent, p.rp_n, p.rp_maxrun};
  if constexpr (std::is_same<T, float>::value) {
    if (!a.hii_f || p.nb % 4 != 0 || !al(a.hii_f)) return false;
    auto k = k_sigma_rows_pipe<1024, Wd, kB>;
    ensure_dynamic_smem((const void *)k, smem);
    prefer_shared_carveout((const void *)k);
    k<<<grid, 1024, smem, s>>>(a, rp);
  } else {
    if (p.nb % 2 != 0 || !al(std::is_same<T, double>::value ? (const void *)a.hii : (const void *)a.hii_df))
      return false;
    auto k = k_sigma_rows_pipe8<1024, T, Wd, kB>;
    ensure_dynamic_smem((const void *)k, smem);
    prefer_shared_carveout((const void *)k);
    k<<<grid, 1024, smem, s>>>(a, rp);
  }
  return true;
}

template <typename T, bool kB>
void launch_stream(const Problem &p, const sdev::Args<T> &a, int variant, cudaStream_t s) {
  SBDGB_REQUIRE(rows_fit<T>(p), SBDGB_E_UNSUPPORTED, "the row kernel does not fit this problem");
  if (kB || p.norb <= 32) {
    if (variant == 0 && launch_rows_pipe<T, uint32_t, kB>(p, a, s)) return;
    if (variant == 0) launch_rows_nt<T, 512, uint32_t, kB>(p, a, s);
    else launch_rows_nt<T, 1024, uint32_t, kB>(p, a, s);
  } else {
    if (variant == 0 && launch_rows_pipe<T, unsigned long long, kB>(p, a, s)) return;
    if (variant == 0) launch_rows_nt<T, 512, unsigned long long, kB>(p, a, s);
    else launch_rows_nt<T, 1024, unsigned long long, kB>(p, a, s);
  }
}

template bool rows_fit<double>(const Problem &);
template bool rows_fit<float>(const Problem &);
template bool rows_fit<dfloat>(const Problem &);
template void launch_stream<double, false>(const Problem &, const sdev::Args<double> &, int, cudaStream_t);
template void launch_stream<double, true>(const Problem &, const sdev::Args<double> &, int, cudaStream_t);
template void launch_stream<float, false>(const Problem &, const sdev::Args<float> &, int, cudaStream_t);
template void launch_stream<float, true>(const Problem &, const sdev::Args<float> &, int, cudaStream_t);
template void launch_stream<dfloat, false>(const Problem &, const sdev::Args<dfloat> &, int, cudaStream_t);
template void launch_stream<dfloat, true>(const Problem &, const sdev::Args<dfloat> &, int, cudaStream_t);

}  // namespace sbdgb
