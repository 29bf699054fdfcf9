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
// thread then walks the beta singles of its columns: per beta single one
// 16-byte shared load of C values, one of (P|Q) values and kG multiply-adds.
// Columns are visited in the order of decreasing beta-single count, so the 32
// lanes of a warp walk lists of similar length.  The row's results stay in
// shared memory (one owner thread per column) and are added to sigma once.
//
// Phases.  In the block ordering (the solvers' convention: vectors multiplied
// by eta, see sigma_dev.cuh) the phase is the product of the two singles'
// same-spin phases, stored in their table entries.  In the reference's
// interleaved ordering it also has the opposite-spin parities: beta string ib
// under the alpha single's mask, and the alpha ket string ja under the beta
// single's mask (as in k_sigma_alpha).
#include "common.cuh"
#include "sigma_dev.cuh"

namespace sbdgb {

namespace {

using namespace sdev;
constexpr int kAbThreads = 512;

template <typename T>
struct __align__(16) Vec16 {
  static constexpr int G = 16 / (int)sizeof(T);
  T v[G];
};

template <typename T, typename Wd, bool kB>
__global__ void __launch_bounds__(kAbThreads) k_sigma_ab(Args<T> a, const uint32_t *__restrict__ rows,
                                                         const uint32_t *__restrict__ cols) {
  using V = Vec16<T>;
  constexpr int G = V::G;
  extern __shared__ __align__(16) unsigned char ab_smem[];
  V *Cs = reinterpret_cast<V *>(ab_smem);      // [nb]: C[ja_g][jb] for the staged singles g
  V *Ks = Cs + a.nb;                            // [npair]: phase_g * (P_g|Q)
  T *Ss = reinterpret_cast<T *>(Ks + a.npair);  // [nb]: this row's results
  const uint32_t ia = ldg(rows + blockIdx.x);
  const uint32_t p0 = ldg(a.A.off_s + ia), p1 = ldg(a.A.off_s + ia + 1);
  for (uint32_t c = threadIdx.x; c < a.nb; c += kAbThreads) Ss[c] = T(0);
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
    for (uint32_t k = threadIdx.x; k < a.nb; k += kAbThreads) {
      const uint32_t ib = ldg(cols + k);
      const uint32_t q0 = ldg(a.B.off_s + ib), q1 = ldg(a.B.off_s + ib + 1);
      if (q0 == q1) break;  // columns come by decreasing count: this thread's others have none
      T acc = T(0);
      if constexpr (kB) {
        for (uint32_t q = q0; q < q1; ++q) {
          const uint32_t jb = ldg(a.B.ket_s + q), cb = ldg(a.B.code_s + q);
          const V kv = Ks[(cb >> 16) & 0x7fffu];
          const V cv = Cs[jb];
          T t = kv.v[0] * cv.v[0];
#pragma unroll
          for (int g = 1; g < G; ++g) t = fma(kv.v[g], cv.v[g], t);
          acc += flip(t, cb >> 31);
        }
      } else {
        const Wd bw = word<Wd>(a.bstr, ib);
        uint32_t pa = 0;
#pragma unroll
        for (int g = 0; g < G; ++g) pa |= parity(bw & am[g]) << g;
        for (uint32_t q = q0; q < q1; ++q) {
          const uint32_t jb = ldg(a.B.ket_s + q), cb = ldg(a.B.code_s + q);
          const Wd mb = word<Wd>(a.B.mask_s, q);
          const V kv = Ks[(cb >> 16) & 0x7fffu];
          const V cv = Cs[jb];
#pragma unroll
          for (int g = 0; g < G; ++g) {
            const uint32_t ph = (pa >> g) ^ parity(aw[g] & mb) ^ (cb >> 31);
            acc = fma(flip(kv.v[g], ph & 1u), cv.v[g], acc);
          }
        }
      }
      Ss[ib] += acc;
    }
  }
  __syncthreads();
  T *srow = a.S + (size_t)ia * a.nb;
  for (uint32_t c = threadIdx.x; c < a.nb; c += kAbThreads) srow[c] = srow[c] + Ss[c];
}

template <typename T>
size_t ab_smem(const Problem &p) {
  return sizeof(Vec16<T>) * ((size_t)p.nb + (size_t)p.npair) + sizeof(T) * (size_t)p.nb;
}

template <typename T, typename Wd, bool kB>
void launch_ab_kernel(const Problem &p, const Args<T> &a, cudaStream_t s) {
  const size_t smem = ab_smem<T>(p);
  auto k = k_sigma_ab<T, Wd, kB>;
  SBDGB_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  k<<<p.n_ab_rows, kAbThreads, smem, s>>>(a, p.ab_rows, p.ab_cols);
}

}  // namespace

template <typename T>
bool ab_fits(const Problem &p) {
  int dev = 0, optin = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return false;
  if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return false;
  return p.ab_rows != nullptr && p.A.ns > 0 && p.B.ns > 0 && ab_smem<T>(p) <= (size_t)optin;
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
