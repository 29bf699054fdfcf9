// Alpha x beta single pairs of sigma (task type 0, chemistry/tpb/mult.h:
// 527-557; the alpha-beta TwoExcite of chemistry/basic/determinants.h:
// 500-518) in a kernel of their own, for problems where they dominate:
//
//   sigma[ia][ib] += sum_{p in alpha singles of ia} sum_{q in beta singles of ib}
//                    phase(p, q) * (P_p|Q_q) * C[ja_p][jb_q]
//
// Done inside the alpha sweep (k_sigma_alpha), each such term costs two
// scattered global loads: the (P|Q) value and C[ja][jb] with jb different in
// every lane.  With a few tens of singles per string (norb 24, thousands of
// strings) these terms are most of the nonzeros and most of sigma's time.
//
// Here one CTA owns one alpha row ia.  It stages kG of the row's alpha singles
// at a time in shared memory: the C rows ja_p (every column) and the (P|Q) rows
// P_p, each (P|Q) value signed by its alpha single's phase, interleaved so that
// the kG values of one column (of one pair Q) form one 16-byte vector.  Every
// warp then walks the beta singles of 32 columns: per beta single one 16-byte
// shared load of C values, one of (P|Q) values and kG multiply-adds (one
// instruction per term: the phase is applied to the (P|Q) value's sign bit,
// which matters where the FP64 pipe is the bound).
//
// Beta singles layout (built once per problem, build_ab_order): the columns
// sorted by decreasing single count, cut into slices of 32; in a slice, entry
// j of the column in lane l sits at slice_start + 32 j + l, and the shorter
// columns are padded to the slice's longest with entries that point at a zero
// (P|Q) value.  So the 32 lanes of a warp read 32 consecutive words per step
// (one coalesced 128-byte load) and walk lists of the same length (sorted
// counts keep the padding small) -- the sliced ELLPACK format.  An entry packs
// jb << 13 | Q << 1 | phase into one 32-bit word (nb < 2^19, npair < 4095).
//
// The row's results stay in shared memory (one owner lane per column) and are
// added to sigma once.
//
// Phases.  In the block ordering (the solvers' convention: vectors multiplied
// by eta, see sigma_dev.cuh) the phase is the product of the two singles'
// same-spin phases, stored in their table entries.  In the reference's
// interleaved ordering it also has the opposite-spin parities: beta string ib
// under the alpha single's mask, and the alpha ket string ja under the beta
// single's mask (as in k_sigma_alpha); the masks follow the entries' layout.
#include <algorithm>

#include "common.cuh"
#include "sigma_dev.cuh"

namespace sbdgb {

namespace {

using namespace sdev;
constexpr int kAbThreads = 512;
constexpr int kAbWarps = kAbThreads / 32;
constexpr uint32_t kAbMaxNb = 1u << 19;    // column index bits of a packed entry
constexpr uint32_t kAbMaxPair = 4095;      // pair index bits (the pad entry uses index npair)

template <typename T>
struct __align__(16) Vec16 {
  static constexpr int G = 16 / (int)sizeof(T);
  T v[G];
};

struct AbOrder {
  const uint32_t *rows, *cols, *slice, *ent;
  const uint64_t *mask;
  uint32_t nslices;
};

template <typename T, typename Wd, bool kB>
__global__ void __launch_bounds__(kAbThreads) k_sigma_ab(Args<T> a, AbOrder o) {
  using V = Vec16<T>;
  constexpr int G = V::G;
  extern __shared__ __align__(16) unsigned char ab_smem[];
  V *Cs = reinterpret_cast<V *>(ab_smem);          // [nb]: C[ja_g][jb] for the staged singles g
  V *Ks = Cs + a.nb;                                // [npair + 1]: phase_g * (P_g|Q); [npair] = 0 (pad)
  T *Ss = reinterpret_cast<T *>(Ks + a.npair + 1);  // [nb]: this row's results
  const uint32_t ia = ldg(o.rows + blockIdx.x);
  const uint32_t p0 = ldg(a.A.off_s + ia), p1 = ldg(a.A.off_s + ia + 1);
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  for (uint32_t c = threadIdx.x; c < a.nb; c += kAbThreads) Ss[c] = T(0);
  if (threadIdx.x == 0) {
    V z;
#pragma unroll
    for (int g = 0; g < G; ++g) z.v[g] = T(0);
    Ks[a.npair] = z;
  }
  for (uint32_t pb = p0; pb < p1; pb += G) {
    uint32_t ja[G], P[G], sg[G];
    Wd aw[G], am[G];
    bool ok[G];
#pragma unroll
    for (int g = 0; g < G; ++g) {
      ok[g] = pb + g < p1;
      ja[g] = ok[g] ? ldg(a.A.ket_s + pb + g) : 0u;
      const uint32_t code = ok[g] ? ldg(a.A.code_s + pb + g) : 0u;
      P[g] = (code >> 16) & 0x7fffu;
      sg[g] = code >> 31;
      aw[g] = (!kB && ok[g]) ? word<Wd>(a.astr, ja[g]) : Wd(0);
      am[g] = ok[g] ? mask_of<kB, Wd>(a.A.mask_s, pb + g) : Wd(0);
    }
    __syncthreads();  // the previous batch is applied (and Ss is zero before the first)
    for (uint32_t c = threadIdx.x; c < a.nb; c += kAbThreads) {
      V x;
#pragma unroll
      for (int g = 0; g < G; ++g) x.v[g] = ok[g] ? ldg(a.C + (size_t)ja[g] * a.nb + c) : T(0);
      Cs[c] = x;
    }
    for (uint32_t Q = threadIdx.x; Q < (uint32_t)a.npair; Q += kAbThreads) {
      V k;
#pragma unroll
      for (int g = 0; g < G; ++g) k.v[g] = ok[g] ? flip(ldg(a.Kp + (size_t)P[g] * a.npair + Q), sg[g]) : T(0);
      Ks[Q] = k;
    }
    __syncthreads();
    // slices (longest first) dealt to the warps in snake order, so that every
    // warp gets a similar share of entries before the next barrier
    for (uint32_t base = 0; base < o.nslices; base += kAbWarps) {
      const uint32_t round = base / kAbWarps;
      const uint32_t sl = base + ((round & 1u) ? kAbWarps - 1u - warp : warp);
      if (sl >= o.nslices) continue;
      const uint32_t e0 = ldg(o.slice + sl), e1 = ldg(o.slice + sl + 1);
      const uint32_t k = sl * 32u + lane;
      const uint32_t ib = k < a.nb ? ldg(o.cols + k) : 0u;
      T acc = T(0);
      if constexpr (kB) {
        // one multiply-add per term with the sign on the (P|Q) value; two
        // entries per step so that two loads are in flight
        uint32_t e = e0 + lane;
        for (; e + 32u < e1; e += 64u) {
          const uint32_t w0 = ldg(o.ent + e), w1 = ldg(o.ent + e + 32u);
          const V k0 = Ks[(w0 >> 1) & 0xfffu], k1 = Ks[(w1 >> 1) & 0xfffu];
          const V c0 = Cs[w0 >> 13], c1 = Cs[w1 >> 13];
#pragma unroll
          for (int g = 0; g < G; ++g) acc = fma(flip(k0.v[g], w0 & 1u), c0.v[g], acc);
#pragma unroll
          for (int g = 0; g < G; ++g) acc = fma(flip(k1.v[g], w1 & 1u), c1.v[g], acc);
        }
        if (e < e1) {
          const uint32_t w = ldg(o.ent + e);
          const V kv = Ks[(w >> 1) & 0xfffu];
          const V cv = Cs[w >> 13];
#pragma unroll
          for (int g = 0; g < G; ++g) acc = fma(flip(kv.v[g], w & 1u), cv.v[g], acc);
        }
      } else {
        const Wd bw = word<Wd>(a.bstr, ib);
        uint32_t pa = 0;
#pragma unroll
        for (int g = 0; g < G; ++g) pa |= parity(bw & am[g]) << g;
        for (uint32_t e = e0 + lane; e < e1; e += 32u) {
          const uint32_t w = ldg(o.ent + e);
          const Wd mb = word<Wd>(o.mask, e);
          const V kv = Ks[(w >> 1) & 0xfffu];
          const V cv = Cs[w >> 13];
#pragma unroll
          for (int g = 0; g < G; ++g) {
            const uint32_t ph = (pa >> g) ^ parity(aw[g] & mb) ^ w;
            acc = fma(flip(kv.v[g], ph & 1u), cv.v[g], acc);
          }
        }
      }
      if (k < a.nb) Ss[ib] += acc;
    }
  }
  __syncthreads();
  T *srow = a.S + (size_t)ia * a.nb;
  for (uint32_t c = threadIdx.x; c < a.nb; c += kAbThreads) srow[c] = srow[c] + Ss[c];
}

template <typename T>
size_t ab_smem(const Problem &p) {
  return sizeof(Vec16<T>) * ((size_t)p.nb + (size_t)p.npair + 1) + sizeof(T) * (size_t)p.nb;
}

template <typename T, typename Wd, bool kB>
void launch_ab_kernel(const Problem &p, const Args<T> &a, cudaStream_t s) {
  const size_t smem = ab_smem<T>(p);
  auto k = k_sigma_ab<T, Wd, kB>;
  ensure_dynamic_smem((const void *)k, smem);
  prefer_shared_carveout((const void *)k);
  const AbOrder o{p.ab_rows, p.ab_cols, p.ab_slice, p.ab_ent, p.ab_mask, p.n_ab_slices};
  k<<<p.n_ab_rows, kAbThreads, smem, s>>>(a, o);
}

}  // namespace

void build_ab_order(Problem &p, const std::vector<uint32_t> &off_a, const std::vector<uint32_t> &off_b,
                    cudaStream_t s) {
  p.n_ab_rows = p.n_ab_slices = 0;
  if (p.A.ns == 0 || p.B.ns == 0 || p.nb >= kAbMaxNb || (uint32_t)p.npair >= kAbMaxPair) return;
  // alpha rows with singles, most first
  std::vector<uint32_t> rows;
  for (uint32_t r = 0; r < p.na; ++r)
    if (off_a[r + 1] > off_a[r]) rows.push_back(r);
  std::stable_sort(rows.begin(), rows.end(),
                   [&](uint32_t x, uint32_t y) { return off_a[x + 1] - off_a[x] > off_a[y + 1] - off_a[y]; });
  // beta columns by decreasing single count, in slices of 32
  auto cnt = [&](uint32_t c) { return off_b[c + 1] - off_b[c]; };
  std::vector<uint32_t> cols(p.nb);
  for (uint32_t c = 0; c < p.nb; ++c) cols[c] = c;
  std::stable_sort(cols.begin(), cols.end(), [&](uint32_t x, uint32_t y) { return cnt(x) > cnt(y); });
  const uint32_t nslices = (p.nb + 31) / 32;
  std::vector<uint32_t> slice(nslices + 1, 0);
  for (uint32_t sl = 0; sl < nslices; ++sl) slice[sl + 1] = slice[sl] + 32u * cnt(cols[32u * sl]);
  // the beta singles in that layout
  std::vector<uint32_t> ket(p.B.ns), code(p.B.ns);
  std::vector<uint64_t> mask(p.B.ns);
  SBDGB_CUDA(cudaMemcpyAsync(ket.data(), p.B.ket_s, sizeof(uint32_t) * p.B.ns, cudaMemcpyDeviceToHost, s));
  SBDGB_CUDA(cudaMemcpyAsync(code.data(), p.B.code_s, sizeof(uint32_t) * p.B.ns, cudaMemcpyDeviceToHost, s));
  SBDGB_CUDA(cudaMemcpyAsync(mask.data(), p.B.mask_s, sizeof(uint64_t) * p.B.ns, cudaMemcpyDeviceToHost, s));
  SBDGB_CUDA(cudaStreamSynchronize(s));
  const size_t total = slice[nslices];
  std::vector<uint32_t> ent(total, (uint32_t)p.npair << 1);  // pad: column 0, the zero (P|Q) entry
  std::vector<uint64_t> emask(total, 0ull);
  for (uint32_t sl = 0; sl < nslices; ++sl)
    for (uint32_t l = 0; l < 32u && 32u * sl + l < p.nb; ++l) {
      const uint32_t c = cols[32u * sl + l];
      for (uint32_t j = 0, q = off_b[c]; q < off_b[c + 1]; ++j, ++q) {
        const size_t e = slice[sl] + 32u * j + l;
        ent[e] = ket[q] << 13 | ((code[q] >> 16) & 0x7fffu) << 1 | code[q] >> 31;
        emask[e] = mask[q];
      }
    }
  p.ab_rows = (uint32_t *)dev_alloc(p, sizeof(uint32_t) * std::max<size_t>(rows.size(), 1));
  p.ab_cols = (uint32_t *)dev_alloc(p, sizeof(uint32_t) * cols.size());
  p.ab_slice = (uint32_t *)dev_alloc(p, sizeof(uint32_t) * slice.size());
  p.ab_ent = (uint32_t *)dev_alloc(p, sizeof(uint32_t) * std::max<size_t>(total, 1));
  p.ab_mask = (uint64_t *)dev_alloc(p, sizeof(uint64_t) * std::max<size_t>(total, 1));
  SBDGB_CUDA(cudaMemcpyAsync(p.ab_rows, rows.data(), sizeof(uint32_t) * rows.size(), cudaMemcpyHostToDevice, s));
  SBDGB_CUDA(cudaMemcpyAsync(p.ab_cols, cols.data(), sizeof(uint32_t) * cols.size(), cudaMemcpyHostToDevice, s));
  SBDGB_CUDA(cudaMemcpyAsync(p.ab_slice, slice.data(), sizeof(uint32_t) * slice.size(), cudaMemcpyHostToDevice, s));
  SBDGB_CUDA(cudaMemcpyAsync(p.ab_ent, ent.data(), sizeof(uint32_t) * total, cudaMemcpyHostToDevice, s));
  SBDGB_CUDA(cudaMemcpyAsync(p.ab_mask, emask.data(), sizeof(uint64_t) * total, cudaMemcpyHostToDevice, s));
  SBDGB_CUDA(cudaStreamSynchronize(s));  // the host vectors go out of scope
  p.n_ab_rows = (uint32_t)rows.size();
  p.n_ab_slices = nslices;
}

template <typename T>
bool ab_fits(const Problem &p) {
  int dev = 0, optin = 0;
  if (p.n_ab_rows == 0 || p.ab_ent == nullptr) return false;
  if (cudaGetDevice(&dev) != cudaSuccess) return false;
  if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return false;
  return ab_smem<T>(p) <= (size_t)optin;
}

template <typename T>
void launch_ab(const Problem &p, const sdev::Args<T> &a, bool block, cudaStream_t s) {
  if (p.n_ab_rows == 0) return;
  if (block)
    launch_ab_kernel<T, uint32_t, true>(p, a, s);
  else if (p.norb <= 32)
    launch_ab_kernel<T, uint32_t, false>(p, a, s);
  else
    launch_ab_kernel<T, unsigned long long, false>(p, a, s);
  count_launch(p.ctx);
  SBDGB_CUDA(cudaGetLastError());
}

template bool ab_fits<double>(const Problem &);
template bool ab_fits<float>(const Problem &);
template bool ab_fits<dfloat>(const Problem &);
template void launch_ab<double>(const Problem &, const sdev::Args<double> &, bool, cudaStream_t);
template void launch_ab<float>(const Problem &, const sdev::Args<float> &, bool, cudaStream_t);
template void launch_ab<dfloat>(const Problem &, const sdev::Args<dfloat> &, bool, cudaStream_t);

}  // namespace sbdgb
