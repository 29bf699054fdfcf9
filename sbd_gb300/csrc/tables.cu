// Excitation tables (replaces the reference's MakeHelpers/RemakeHelpers at MPI
// size 1, chemistry/tpb/helper.h:729-873 and :935-1245, whose per-task work is
// GenerateExcitation, helper.h:185-342).
//
// The reference compares every bra string with every ket string of the same
// spin (Hamming distance 2 = single, 4 = double) and keeps the matches in
// ascending ket order.  Here one warp owns one bra string: lanes test 32 kets
// at a time, __ballot_sync collects the matches and __popc of the lower lanes
// gives each match its slot, so the CSR rows come out in the same ascending
// order without sorting.  Each matching lane then evaluates everything about
// the pair that does not depend on the opposite-spin string: the same-spin
// phase, the opposite-spin phase mask and the integral part of the matrix
// element (see SpinTables in common.cuh).
#include <algorithm>

#include "common.cuh"

namespace sbdgb {

namespace {

constexpr int kTile = 2048;  // ket strings staged in shared memory per pass

// Full (P|Q) over unordered orbital pairs from the 8-fold packed array
// (integrals.h:94-102 index rule).
__global__ void k_unpack_eri(const double *__restrict__ eri, double *__restrict__ Kp, int npair) {
  size_t total = (size_t)npair * npair;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
    size_t P = t / npair, Q = t % npair;
    size_t a = P > Q ? P : Q, b = P > Q ? Q : P;
    Kp[t] = eri[a * (a + 1) / 2 + b];
  }
}

// (pp|qq) and (pq|qp) in spatial orbitals.
__global__ void k_diag_ints(const double *__restrict__ Kp, int norb, int npair, double *__restrict__ J,
                            double *__restrict__ X) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= norb * norb) return;
  int p = t / norb, q = t % norb;
  J[t] = Kp[(size_t)pair_index(p, p) * npair + pair_index(q, q)];
  X[t] = Kp[(size_t)pair_index(p, q) * npair + pair_index(q, p)];
}

// Pass 1: number of singles and doubles of every bra string.
__global__ void k_count(const uint64_t *__restrict__ strs, uint32_t n, uint32_t *__restrict__ cs,
                        uint32_t *__restrict__ cd) {
  __shared__ uint64_t tile[kTile];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  const uint32_t bra = blockIdx.x * nwarp + warp;
  const uint64_t b = bra < n ? strs[bra] : 0ull;
  uint32_t ns = 0, nd = 0;
  for (uint32_t base = 0; base < n; base += kTile) {
    uint32_t cnt = min((uint32_t)kTile, n - base);
    __syncthreads();
    for (uint32_t t = threadIdx.x; t < cnt; t += blockDim.x) tile[t] = strs[base + t];
    __syncthreads();
    if (bra < n) {
      for (uint32_t k = lane; k < cnt; k += 32) {
        int d = __popcll(b ^ tile[k]);
        ns += (d == 2);
        nd += (d == 4);
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    ns += __shfl_xor_sync(0xffffffffu, ns, o);
    nd += __shfl_xor_sync(0xffffffffu, nd, o);
  }
  if (bra < n && lane == 0) {
    cs[bra] = ns;
    cd[bra] = nd;
  }
}

// Exclusive scan of n counts into n+1 offsets, one CTA; also reports totals.
__global__ void k_scan(const uint32_t *__restrict__ c, uint32_t n, uint32_t *__restrict__ off,
                       unsigned long long *__restrict__ total) {
  __shared__ unsigned long long part[1024];
  const uint32_t per = (n + blockDim.x - 1) / blockDim.x;
  const uint32_t lo = min(n, threadIdx.x * per), hi = min(n, lo + per);
  unsigned long long s = 0;
  for (uint32_t i = lo; i < hi; ++i) s += c[i];
  part[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long run = 0;
    for (uint32_t t = 0; t < blockDim.x; ++t) {
      unsigned long long v = part[t];
      part[t] = run;
      run += v;
    }
    *total = run;
  }
  __syncthreads();
  unsigned long long run = part[threadIdx.x];
  for (uint32_t i = lo; i < hi; ++i) {
    off[i] = (uint32_t)run;  // totals are checked on the host to fit 32 bits
    run += c[i];
  }
  if (threadIdx.x == blockDim.x - 1 || (hi == n && lo < hi)) off[n] = (uint32_t)run;
  if (n == 0 && threadIdx.x == 0) off[0] = 0;
}

struct FillArgs {
  const uint64_t *strs;
  uint32_t n;
  int spin;
  int norb;
  int npair;
  const double *Kp;
  const double *h1;
  const uint32_t *off_s, *off_d;
  uint32_t *ket_s, *ket_d, *code_s, *code_d;
  double *val_s, *val_d;
  uint64_t *mask_s, *mask_d;
};

__device__ inline double kp(const FillArgs &a, int p, int q, int r, int s) {
  return a.Kp[(size_t)pair_index(p, q) * a.npair + pair_index(r, s)];
}

// Same-spin part of the single-excitation element (OneExcite,
// determinants.h:476-498, restricted to the bra's same-spin electrons; the
// opposite-spin electrons only add (an cr|qq), applied in the sigma kernel).
__device__ double single_val(const FillArgs &a, uint64_t bra, int cr, int an) {
  double e = a.h1[an * a.norb + cr];
  uint64_t occ = bra;
  while (occ) {
    int j = __ffsll((long long)occ) - 1;
    occ &= occ - 1;
    e += kp(a, an, cr, j, j) - kp(a, an, j, j, cr);
  }
  return e;
}

// Pass 2: fill the rows in ascending ket order and evaluate each pair.
__global__ void k_fill(FillArgs a) {
  __shared__ uint64_t tile[kTile];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  const uint32_t bra = blockIdx.x * nwarp + warp;
  const uint64_t b = bra < a.n ? a.strs[bra] : 0ull;
  uint32_t ps = bra < a.n ? a.off_s[bra] : 0, pd = bra < a.n ? a.off_d[bra] : 0;
  const uint32_t lanemask_lt = (1u << lane) - 1u;
  const int s = a.spin;
  for (uint32_t base = 0; base < a.n; base += kTile) {
    uint32_t cnt = min((uint32_t)kTile, a.n - base);
    __syncthreads();
    for (uint32_t t = threadIdx.x; t < cnt; t += blockDim.x) tile[t] = a.strs[base + t];
    __syncthreads();
    if (bra >= a.n) continue;
    for (uint32_t k0 = 0; k0 < cnt; k0 += 32) {
      uint32_t k = k0 + lane;
      uint64_t ket = k < cnt ? tile[k] : b;
      int d = __popcll(b ^ ket);
      unsigned ms = __ballot_sync(0xffffffffu, d == 2);
      unsigned md = __ballot_sync(0xffffffffu, d == 4);
      if (d == 2) {
        uint32_t slot = ps + __popc(ms & lanemask_lt);
        int cr = __ffsll((long long)(b & ~ket)) - 1;
        int an = __ffsll((long long)(ket & ~b)) - 1;
        int i = 2 * cr + s, ai = 2 * an + s;
        uint64_t ma, mb;
        interval_masks(min(i, ai), max(i, ai), ma, mb);
        uint64_t same = s == 0 ? ma : mb, opp = s == 0 ? mb : ma;
        uint32_t sg = __popcll(b & same) & 1u;
        a.ket_s[slot] = base + k;
        a.code_s[slot] = (uint32_t)cr | ((uint32_t)an << 8) | ((uint32_t)pair_index(cr, an) << 16) | (sg << 31);
        a.val_s[slot] = single_val(a, b, cr, an);
        a.mask_s[slot] = opp;
      }
      if (d == 4) {
        uint32_t slot = pd + __popc(md & lanemask_lt);
        uint64_t c = b & ~ket, n2 = ket & ~b;
        int cr0 = __ffsll((long long)c) - 1;
        c &= c - 1;
        int cr1 = __ffsll((long long)c) - 1;
        int an0 = __ffsll((long long)n2) - 1;
        n2 &= n2 - 1;
        int an1 = __ffsll((long long)n2) - 1;
        // TwoExcite (determinants.h:500-518) with I<J, A<B from the ascending lists
        int I = 2 * cr0 + s, J = 2 * cr1 + s, A = 2 * an0 + s, B = 2 * an1 + s;
        uint64_t ma1, mb1, ma2, mb2;
        interval_masks(min(I, A), max(I, A), ma1, mb1);
        interval_masks(min(J, B), max(J, B), ma2, mb2);
        uint64_t same1 = s == 0 ? ma1 : mb1, same2 = s == 0 ? ma2 : mb2;
        uint64_t opp = s == 0 ? (mb1 ^ mb2) : (ma1 ^ ma2);
        uint32_t ph = (__popcll(b & same1) + __popcll(b & same2) + ((A > J || B < I) ? 1 : 0)) & 1u;
        double v = kp(a, an0, cr0, an1, cr1) - kp(a, an0, cr1, an1, cr0);
        a.ket_d[slot] = base + k;
        a.code_d[slot] = (uint32_t)cr0 | ((uint32_t)cr1 << 6) | ((uint32_t)an0 << 12) | ((uint32_t)an1 << 18);
        a.val_d[slot] = ph ? -v : v;
        a.mask_d[slot] = opp;
      }
      ps += __popc(ms);
      pd += __popc(md);
    }
  }
}

// Jo[P][i] = sum_{q occupied in strs[i]} (P|qq): the opposite-spin Coulomb
// part of the single-excitation elements (OneExcite terms with j of the other
// spin, whose exchange integral vanishes by spin).
// bra[e] = i for the entries e of CSR row i (the row of every entry, for
// kernels that walk entries rather than rows).
__global__ void k_bra_index(const uint32_t *__restrict__ off, uint32_t n, uint32_t *__restrict__ bra) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    for (uint32_t e = off[i]; e < off[i + 1]; ++e) bra[e] = i;
}

__global__ void k_opp_coulomb(const uint64_t *__restrict__ strs, uint32_t n, const double *__restrict__ Kp,
                              int npair, double *__restrict__ Jo) {
  const int P = blockIdx.y;
  const double *row = Kp + (size_t)P * npair;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    uint64_t occ = strs[i];
    double e = 0.0;
    while (occ) {
      int q = __ffsll((long long)occ) - 1;
      occ &= occ - 1;
      e += row[pair_index(q, q)];
    }
    Jo[(size_t)P * n + i] = e;
  }
}

void build_spin(Problem &p, int spin, cudaStream_t s) {
  SpinTables &T = spin == 0 ? p.A : p.B;
  const uint64_t *strs = spin == 0 ? p.astr : p.bstr;
  const uint32_t n = spin == 0 ? p.na : p.nb;
  T.n = n;
  uint32_t *cs = (uint32_t *)dev_alloc(p, sizeof(uint32_t) * (n + 1));
  uint32_t *cd = (uint32_t *)dev_alloc(p, sizeof(uint32_t) * (n + 1));
  T.off_s = (uint32_t *)dev_alloc(p, sizeof(uint32_t) * (n + 1));
  T.off_d = (uint32_t *)dev_alloc(p, sizeof(uint32_t) * (n + 1));
  unsigned long long *tot = (unsigned long long *)dev_alloc(p, 2 * sizeof(unsigned long long));
  const int threads = 256, bras_per_block = threads / 32;
  const unsigned blocks = (n + bras_per_block - 1) / bras_per_block;
  k_count<<<blocks, threads, 0, s>>>(strs, n, cs, cd);
  k_scan<<<1, 1024, 0, s>>>(cs, n, T.off_s, tot);
  k_scan<<<1, 1024, 0, s>>>(cd, n, T.off_d, tot + 1);
  count_launch(p.ctx, 3);
  SBDGB_CUDA(cudaGetLastError());
  unsigned long long h_tot[2];
  SBDGB_CUDA(cudaMemcpyAsync(h_tot, tot, sizeof(h_tot), cudaMemcpyDeviceToHost, s));
  SBDGB_CUDA(cudaStreamSynchronize(s));
  SBDGB_REQUIRE(h_tot[0] < (1ull << 32) && h_tot[1] < (1ull << 32), SBDGB_E_UNSUPPORTED,
                "more than 2^32 excitation pairs of one spin");
  T.ns = h_tot[0];
  T.nd = h_tot[1];
  const size_t ns1 = T.ns ? T.ns : 1, nd1 = T.nd ? T.nd : 1;
  T.ket_s = (uint32_t *)dev_alloc(p, sizeof(uint32_t) * ns1);
  T.code_s = (uint32_t *)dev_alloc(p, sizeof(uint32_t) * ns1);
  T.val_s = (double *)dev_alloc(p, sizeof(double) * ns1);
  T.mask_s = (uint64_t *)dev_alloc(p, sizeof(uint64_t) * ns1);
  T.ket_d = (uint32_t *)dev_alloc(p, sizeof(uint32_t) * nd1);
  T.code_d = (uint32_t *)dev_alloc(p, sizeof(uint32_t) * nd1);
  T.val_d = (double *)dev_alloc(p, sizeof(double) * nd1);
  T.mask_d = (uint64_t *)dev_alloc(p, sizeof(uint64_t) * nd1);
  FillArgs fa{strs, n, spin, p.norb, p.npair, p.Kp, p.h1, T.off_s, T.off_d, T.ket_s, T.ket_d,
              T.code_s, T.code_d, T.val_s, T.val_d, T.mask_s, T.mask_d};
  k_fill<<<blocks, threads, 0, s>>>(fa);
  T.bra_s = (uint32_t *)dev_alloc(p, sizeof(uint32_t) * ns1);
  T.bra_d = (uint32_t *)dev_alloc(p, sizeof(uint32_t) * nd1);
  const unsigned bb = (unsigned)std::min<uint32_t>((n + 255) / 256 + 1, 4096);
  k_bra_index<<<bb, 256, 0, s>>>(T.off_s, n, T.bra_s);
  k_bra_index<<<bb, 256, 0, s>>>(T.off_d, n, T.bra_d);
  count_launch(p.ctx, 3);
  SBDGB_CUDA(cudaGetLastError());
}

}  // namespace

void build_tables(Problem &p, cudaStream_t s) {
  const int L = p.norb, npair = p.npair;
  size_t nI2 = (size_t)npair * (npair + 1) / 2;
  (void)nI2;
  if (!p.Kp) throw Error(SBDGB_E_STATE, "integrals not uploaded");
  build_spin(p, 0, s);
  build_spin(p, 1, s);
  p.Jdiag = (double *)dev_alloc(p, sizeof(double) * L * L);
  p.Xdiag = (double *)dev_alloc(p, sizeof(double) * L * L);
  k_diag_ints<<<(L * L + 255) / 256, 256, 0, s>>>(p.Kp, L, npair, p.Jdiag, p.Xdiag);
  p.Jb = (double *)dev_alloc(p, sizeof(double) * (size_t)npair * p.nb);
  p.Ja = (double *)dev_alloc(p, sizeof(double) * (size_t)npair * p.na);
  {
    dim3 gb((p.nb + 255) / 256, npair), ga((p.na + 255) / 256, npair);
    k_opp_coulomb<<<gb, 256, 0, s>>>(p.bstr, p.nb, p.Kp, npair, p.Jb);
    k_opp_coulomb<<<ga, 256, 0, s>>>(p.astr, p.na, p.Kp, npair, p.Ja);
  }
  count_launch(p.ctx, 3);
  SBDGB_CUDA(cudaGetLastError());
  build_row_tiles(p, s);
  SBDGB_CUDA(cudaStreamSynchronize(s));
  p.tables = true;
}

void unpack_integrals(Problem &p, const double *eri_dev, cudaStream_t s) {
  size_t total = (size_t)p.npair * p.npair;
  unsigned blocks = (unsigned)std::min<size_t>((total + 255) / 256, 65535);
  k_unpack_eri<<<blocks, 256, 0, s>>>(eri_dev, p.Kp, p.npair);
  count_launch(p.ctx);
  SBDGB_CUDA(cudaGetLastError());
}

void export_tables(const Problem &p, int spin, uint64_t *off_s, uint64_t *ket_s, int32_t *cran_s,
                   uint64_t *off_d, uint64_t *ket_d, int32_t *cran_d) {
  const SpinTables &T = spin == 0 ? p.A : p.B;
  std::vector<uint32_t> os(T.n + 1), od(T.n + 1), ks(T.ns), kd(T.nd), cs(T.ns), cd(T.nd);
  SBDGB_CUDA(cudaMemcpy(os.data(), T.off_s, sizeof(uint32_t) * (T.n + 1), cudaMemcpyDeviceToHost));
  SBDGB_CUDA(cudaMemcpy(od.data(), T.off_d, sizeof(uint32_t) * (T.n + 1), cudaMemcpyDeviceToHost));
  if (T.ns) {
    SBDGB_CUDA(cudaMemcpy(ks.data(), T.ket_s, sizeof(uint32_t) * T.ns, cudaMemcpyDeviceToHost));
    SBDGB_CUDA(cudaMemcpy(cs.data(), T.code_s, sizeof(uint32_t) * T.ns, cudaMemcpyDeviceToHost));
  }
  if (T.nd) {
    SBDGB_CUDA(cudaMemcpy(kd.data(), T.ket_d, sizeof(uint32_t) * T.nd, cudaMemcpyDeviceToHost));
    SBDGB_CUDA(cudaMemcpy(cd.data(), T.code_d, sizeof(uint32_t) * T.nd, cudaMemcpyDeviceToHost));
  }
  for (uint32_t i = 0; i <= T.n; ++i) {
    if (off_s) off_s[i] = os[i];
    if (off_d) off_d[i] = od[i];
  }
  for (uint64_t k = 0; k < T.ns; ++k) {
    if (ket_s) ket_s[k] = ks[k];
    if (cran_s) {
      cran_s[2 * k + 0] = 2 * (int32_t)(cs[k] & 0xffu) + spin;
      cran_s[2 * k + 1] = 2 * (int32_t)((cs[k] >> 8) & 0xffu) + spin;
    }
  }
  for (uint64_t k = 0; k < T.nd; ++k) {
    if (ket_d) ket_d[k] = kd[k];
    if (cran_d) {
      for (int q = 0; q < 4; ++q) cran_d[4 * k + q] = 2 * (int32_t)((cd[k] >> (6 * q)) & 63u) + spin;
    }
  }
}

}  // namespace sbdgb
