// Diagonal terms hii (replaces makeQChamDiagTerms, chemistry/tpb/qcham.h:
// 289-340, which evaluates ZeroExcite, chemistry/basic/determinants.h:451-474,
// on every interleaved determinant, and the Thrust MakeQChamDiagTermKernel,
// chemistry/tpb/mult_thrust.h:1583-1618).
//
// ZeroExcite sums h_ii over occupied spin orbitals plus (ii|jj) - [same spin]
// (ij|ji) over occupied pairs.  That splits into a part of the alpha string,
// a part of the beta string and the alpha-beta Coulomb cross term
// sum_{p in alpha} sum_{q in beta} (pp|qq).  The two string parts and the
// row table Jx[ia][q] = sum_{p in alpha(ia)} (pp|qq) are built once, so each
// determinant costs popcount(beta) loads.
#include <algorithm>

#include "common.cuh"

namespace sbdgb {

namespace {

__global__ void k_string_energy(const uint64_t *__restrict__ strs, uint32_t n, const double *__restrict__ h1,
                                const double *__restrict__ J, const double *__restrict__ X, int L,
                                double *__restrict__ E) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint64_t occ = strs[i];
  double e = 0.0;
  uint64_t o1 = occ;
  while (o1) {
    int p = __ffsll((long long)o1) - 1;
    o1 &= o1 - 1;
    e += h1[p * L + p];
    uint64_t o2 = o1;
    while (o2) {
      int q = __ffsll((long long)o2) - 1;
      o2 &= o2 - 1;
      e += J[p * L + q] - X[p * L + q];
    }
  }
  E[i] = e;
}

__global__ void k_cross_rows(const uint64_t *__restrict__ astr, uint32_t na, const double *__restrict__ J, int L,
                             double *__restrict__ Jx) {
  size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (t >= (size_t)na * L) return;
  uint32_t ia = t / L;
  int q = t % L;
  uint64_t occ = astr[ia];
  double e = 0.0;
  while (occ) {
    int p = __ffsll((long long)occ) - 1;
    occ &= occ - 1;
    e += J[p * L + q];
  }
  Jx[t] = e;
}

__global__ void k_hii(const uint64_t *__restrict__ bstr, uint32_t na, uint32_t nb, const double *__restrict__ Ea,
                      const double *__restrict__ Eb, const double *__restrict__ Jx, int L, double ecore,
                      double *__restrict__ hii) {
  extern __shared__ double jrow[];
  for (uint32_t ia = blockIdx.y; ia < na; ia += gridDim.y) {
    __syncthreads();
    for (int q = threadIdx.x; q < L; q += blockDim.x) jrow[q] = Jx[(size_t)ia * L + q];
    __syncthreads();
    const double ea = Ea[ia] + ecore;
    for (uint32_t ib = blockIdx.x * blockDim.x + threadIdx.x; ib < nb; ib += gridDim.x * blockDim.x) {
      uint64_t occ = bstr[ib];
      double e = ea + Eb[ib];
      while (occ) {
        int q = __ffsll((long long)occ) - 1;
        occ &= occ - 1;
        e += jrow[q];
      }
      hii[(size_t)ia * nb + ib] = e;
    }
  }
}

}  // namespace

void build_diag(Problem &p, cudaStream_t s) {
  if (!p.tables) throw Error(SBDGB_E_STATE, "diagonal needs the integral tables");
  const int L = p.norb;
  if (!p.hii) p.hii = (double *)dev_alloc(p, sizeof(double) * (p.N ? p.N : 1));
  double *Ea = (double *)workspace(p, WS_DIAG0, sizeof(double) * (p.na + 1));
  double *Eb = (double *)workspace(p, WS_DIAG1, sizeof(double) * (p.nb + 1));
  double *Jx = (double *)workspace(p, WS_DIAG2, sizeof(double) * ((size_t)p.na * L + 1));
  k_string_energy<<<(p.na + 127) / 128, 128, 0, s>>>(p.astr, p.na, p.h1, p.Jdiag, p.Xdiag, L, Ea);
  k_string_energy<<<(p.nb + 127) / 128, 128, 0, s>>>(p.bstr, p.nb, p.h1, p.Jdiag, p.Xdiag, L, Eb);
  size_t nx = (size_t)p.na * L;
  k_cross_rows<<<(unsigned)((nx + 255) / 256), 256, 0, s>>>(p.astr, p.na, p.Jdiag, L, Jx);
  if (p.N) {
    unsigned gx = (unsigned)std::min<uint32_t>((p.nb + 255) / 256, 64);
    dim3 grid(gx, std::min<uint32_t>(p.na, 65535u));
    k_hii<<<grid, 256, sizeof(double) * L, s>>>(p.bstr, p.na, p.nb, Ea, Eb, Jx, L, p.ecore, p.hii);
  }
  count_launch(p.ctx, 4);
  SBDGB_CUDA(cudaGetLastError());
  SBDGB_CUDA(cudaStreamSynchronize(s));
  p.diag = true;
}

}  // namespace sbdgb
