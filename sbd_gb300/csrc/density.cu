// Occupation density of a vector (OccupationDensity, chemistry/tpb/
// occupation.h:11-95, as sbd::tpb::diag evaluates it with do_rdm == 0,
// chemistry/tpb/sbdiag.h:666-699):
//
//   density[2p]   = sum_{ia,ib} |W[ia][ib]|^2 [alpha orbital p in string ia]
//   density[2p+1] = sum_{ia,ib} |W[ia][ib]|^2 [beta orbital p in string ib]
//
// The sum factorises through the row and column norms of W (as an na x nb
// matrix): density_alpha = O_alpha^T r, density_beta = O_beta^T c with
// r[ia] = sum_ib W^2, c[ib] = sum_ia W^2 and O the string occupation
// matrices.  Two passes over W (8N bytes each, HBM bound), then an L-by-n
// reduction per spin.  Every sum runs in a fixed order, so the result does
// not depend on the launch.
#include <algorithm>

#include "common.cuh"

namespace sbdgb {

namespace {

constexpr int kThreads = 256;

// r[ia] = sum_ib W[ia][ib]^2, one warp per row.
__global__ void __launch_bounds__(kThreads) k_row_norms(const double *__restrict__ W, uint32_t na, uint32_t nb,
                                                         double *__restrict__ r) {
  const int lane = threadIdx.x & 31;
  const uint32_t warps = gridDim.x * (kThreads / 32);
  for (uint32_t ia = blockIdx.x * (kThreads / 32) + (threadIdx.x >> 5); ia < na; ia += warps) {
    const double *row = W + (size_t)ia * nb;
    double s = 0.0;
    for (uint32_t ib = lane; ib < nb; ib += 32) {
      const double w = __ldg(row + ib);
      s = fma(w, w, s);
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) r[ia] = s;
  }
}

// part[split][ib] = sum over the split's rows of W[ia][ib]^2 (coalesced along ib).
__global__ void __launch_bounds__(kThreads) k_col_norms(const double *__restrict__ W, uint32_t na, uint32_t nb,
                                                         uint32_t rows_per_split, double *__restrict__ part) {
  const uint32_t ib = blockIdx.x * kThreads + threadIdx.x;
  if (ib >= nb) return;
  const uint32_t r0 = blockIdx.y * rows_per_split, r1 = min(na, r0 + rows_per_split);
  double s = 0.0;
  for (uint32_t ia = r0; ia < r1; ++ia) {
    const double w = __ldg(W + (size_t)ia * nb + ib);
    s = fma(w, w, s);
  }
  part[(size_t)blockIdx.y * nb + ib] = s;
}

__global__ void k_sum_splits(const double *__restrict__ part, uint32_t nsplit, uint32_t n, double *__restrict__ c) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = 0.0;
  for (uint32_t k = 0; k < nsplit; ++k) s += part[(size_t)k * n + i];
  c[i] = s;
}

// out[2p + spin] = sum_s norm[s] [bit p of str[s]]; block (p, spin).
__global__ void __launch_bounds__(kThreads) k_occupation(const uint64_t *__restrict__ astr, const double *__restrict__ r,
                                                          uint32_t na, const uint64_t *__restrict__ bstr,
                                                          const double *__restrict__ c, uint32_t nb,
                                                          double *__restrict__ out) {
  const int p = blockIdx.x, spin = blockIdx.y;
  const uint64_t *str = spin == 0 ? astr : bstr;
  const double *nrm = spin == 0 ? r : c;
  const uint32_t n = spin == 0 ? na : nb;
  double s = 0.0;
  for (uint32_t i = threadIdx.x; i < n; i += kThreads)
    if ((__ldg(str + i) >> p) & 1ull) s += __ldg(nrm + i);
  __shared__ double red[kThreads / 32];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < kThreads / 32; ++w) t += red[w];
    out[2 * p + spin] = t;
  }
}

// Per row: how many |W|^2 exceed cut and their sum; one warp per row.
__global__ void __launch_bounds__(kThreads) k_row_cut(const double *__restrict__ W, uint32_t na, uint32_t nb,
                                                       double cut, unsigned long long *__restrict__ cnt,
                                                       double *__restrict__ wsum) {
  const int lane = threadIdx.x & 31;
  const uint32_t warps = gridDim.x * (kThreads / 32);
  for (uint32_t ia = blockIdx.x * (kThreads / 32) + (threadIdx.x >> 5); ia < na; ia += warps) {
    const double *row = W + (size_t)ia * nb;
    double s = 0.0;
    unsigned n = 0;
    for (uint32_t ib = lane; ib < nb; ib += 32) {
      const double w = __ldg(row + ib), w2 = w * w;
      if (w2 > cut) {
        s += w2;
        ++n;
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      s += __shfl_xor_sync(0xffffffffu, s, o);
      n += __shfl_xor_sync(0xffffffffu, n, o);
    }
    if (lane == 0) {
      cnt[ia] = n;
      wsum[ia] = s;
    }
  }
}

// part[split][ib] = number of rows of the split with |W[ia][ib]|^2 > cut.
__global__ void __launch_bounds__(kThreads) k_col_cut(const double *__restrict__ W, uint32_t na, uint32_t nb,
                                                       uint32_t rows_per_split, double cut,
                                                       unsigned long long *__restrict__ part) {
  const uint32_t ib = blockIdx.x * kThreads + threadIdx.x;
  if (ib >= nb) return;
  const uint32_t r0 = blockIdx.y * rows_per_split, r1 = min(na, r0 + rows_per_split);
  unsigned long long n = 0;
  for (uint32_t ia = r0; ia < r1; ++ia) {
    const double w = __ldg(W + (size_t)ia * nb + ib);
    n += (w * w > cut) ? 1ull : 0ull;
  }
  part[(size_t)blockIdx.y * nb + ib] = n;
}

__global__ void k_sum_splits_u64(const unsigned long long *__restrict__ part, uint32_t nsplit, uint32_t n,
                                 unsigned long long *__restrict__ c) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  unsigned long long s = 0;
  for (uint32_t k = 0; k < nsplit; ++k) s += part[(size_t)k * n + i];
  c[i] = s;
}

}  // namespace

// Row and column norms of W into r (na) and c (nb); device pointers.
void string_norms(Problem &p, const double *W, double *r, double *c, cudaStream_t s) {
  int sms = 0;
  SBDGB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, p.ctx->device));
  const uint32_t rb = (uint32_t)std::min<size_t>(((size_t)p.na + 7) / 8, (size_t)sms * 8);
  k_row_norms<<<rb, kThreads, 0, s>>>(W, p.na, p.nb, r);
  const uint32_t cx = (p.nb + kThreads - 1) / kThreads;
  const uint32_t want = std::max<uint32_t>(1, (uint32_t)(4 * sms) / cx);
  const uint32_t nsplit = std::min<uint32_t>(want, p.na);
  const uint32_t rows = (p.na + nsplit - 1) / nsplit;
  const uint32_t used = (p.na + rows - 1) / rows;
  double *part = (double *)workspace(p, WS_RED2, sizeof(double) * (size_t)used * p.nb);
  k_col_norms<<<dim3(cx, used), kThreads, 0, s>>>(W, p.na, p.nb, rows, part);
  k_sum_splits<<<(p.nb + 255) / 256, 256, 0, s>>>(part, used, p.nb, c);
  count_launch(p.ctx, 3);
  SBDGB_CUDA(cudaGetLastError());
}

// A device copy of W when it is host memory.
const double *device_vector(Problem &p, const double *W, cudaStream_t s) {
  cudaPointerAttributes at{};
  SBDGB_CUDA(cudaPointerGetAttributes(&at, W));
  if (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged) return W;
  double *Wd = (double *)workspace(p, WS_RES64, sizeof(double) * p.N);
  SBDGB_CUDA(cudaMemcpyAsync(Wd, W, sizeof(double) * p.N, cudaMemcpyHostToDevice, s));
  return Wd;
}

// Weights of the alpha and beta strings in W (DiagonalAdetReducedDensityMatrix
// and DiagonalBdetReducedDensityMatrix, chemistry/tpb/rdmat.h:13-60, 137-187).
void string_weights(Problem &p, const double *W, double *wa_host, double *wb_host, cudaStream_t s) {
  W = device_vector(p, W, s);
  double *r = (double *)workspace(p, WS_NORM_A, sizeof(double) * p.na);
  double *c = (double *)workspace(p, WS_NORM_B, sizeof(double) * p.nb);
  string_norms(p, W, r, c, s);
  SBDGB_CUDA(cudaMemcpyAsync(wa_host, r, sizeof(double) * p.na, cudaMemcpyDeviceToHost, s));
  SBDGB_CUDA(cudaMemcpyAsync(wb_host, c, sizeof(double) * p.nb, cudaMemcpyDeviceToHost, s));
  SBDGB_CUDA(cudaStreamSynchronize(s));
}

// Per string, how many determinants of W have |w|^2 > cut, and the total
// weight of those determinants (the selection step of the amplitude-based
// SinglesExtendHalfdets, chemistry/tpb/extend.h:13-60).
void string_cut_counts(Problem &p, const double *W, double cut, uint64_t *ca_host, uint64_t *cb_host,
                       double *total, cudaStream_t s) {
  W = device_vector(p, W, s);
  int sms = 0;
  SBDGB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, p.ctx->device));
  auto *ca = (unsigned long long *)workspace(p, WS_NORM_A, sizeof(unsigned long long) * p.na);
  auto *cb = (unsigned long long *)workspace(p, WS_NORM_B, sizeof(unsigned long long) * p.nb);
  double *ws = (double *)workspace(p, WS_OCC, sizeof(double) * p.na);
  const uint32_t rb = (uint32_t)std::min<size_t>(((size_t)p.na + 7) / 8, (size_t)sms * 8);
  k_row_cut<<<rb, kThreads, 0, s>>>(W, p.na, p.nb, cut, ca, ws);
  const uint32_t cx = (p.nb + kThreads - 1) / kThreads;
  const uint32_t want = std::max<uint32_t>(1, (uint32_t)(4 * sms) / cx);
  const uint32_t nsplit = std::min<uint32_t>(want, p.na);
  const uint32_t rows = (p.na + nsplit - 1) / nsplit;
  const uint32_t used = (p.na + rows - 1) / rows;
  auto *part = (unsigned long long *)workspace(p, WS_RED2, sizeof(unsigned long long) * (size_t)used * p.nb);
  k_col_cut<<<dim3(cx, used), kThreads, 0, s>>>(W, p.na, p.nb, rows, cut, part);
  k_sum_splits_u64<<<(p.nb + 255) / 256, 256, 0, s>>>(part, used, p.nb, cb);
  count_launch(p.ctx, 3);
  SBDGB_CUDA(cudaGetLastError());
  std::vector<double> wsum(p.na);
  SBDGB_CUDA(cudaMemcpyAsync(ca_host, ca, sizeof(uint64_t) * p.na, cudaMemcpyDeviceToHost, s));
  SBDGB_CUDA(cudaMemcpyAsync(cb_host, cb, sizeof(uint64_t) * p.nb, cudaMemcpyDeviceToHost, s));
  SBDGB_CUDA(cudaMemcpyAsync(wsum.data(), ws, sizeof(double) * p.na, cudaMemcpyDeviceToHost, s));
  SBDGB_CUDA(cudaStreamSynchronize(s));
  double t = 0.0;
  for (double x : wsum) t += x;
  if (total) *total = t;
}

void occupation_density(Problem &p, const double *W, double *density_host, cudaStream_t s) {
  W = device_vector(p, W, s);
  double *r = (double *)workspace(p, WS_NORM_A, sizeof(double) * p.na);
  double *c = (double *)workspace(p, WS_NORM_B, sizeof(double) * p.nb);
  double *out = (double *)workspace(p, WS_OCC, sizeof(double) * 2 * (size_t)p.norb);
  string_norms(p, W, r, c, s);
  k_occupation<<<dim3(p.norb, 2), kThreads, 0, s>>>(p.astr, r, p.na, p.bstr, c, p.nb, out);
  count_launch(p.ctx);
  SBDGB_CUDA(cudaGetLastError());
  SBDGB_CUDA(cudaMemcpyAsync(density_host, out, sizeof(double) * 2 * (size_t)p.norb, cudaMemcpyDeviceToHost, s));
  SBDGB_CUDA(cudaStreamSynchronize(s));
}

}  // namespace sbdgb

namespace {

template <typename F>
int guarded_call(sbdgb_problem *pr, void *stream, F &&f) {
  sbdgb::Ctx *c = pr->p.ctx;
  try {
    SBDGB_CUDA(cudaSetDevice(c->device));
    f(stream ? (cudaStream_t)stream : c->stream);
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

}  // namespace

extern "C" int sbdgb_string_weights(sbdgb_problem *pr, const double *W, double *wa, double *wb, void *stream) {
  if (!pr || !W || !wa || !wb) return SBDGB_E_INPUT;
  return guarded_call(pr, stream, [&](cudaStream_t s) { sbdgb::string_weights(pr->p, W, wa, wb, s); });
}

extern "C" int sbdgb_string_cut_counts(sbdgb_problem *pr, const double *W, double cutoff, uint64_t *ca, uint64_t *cb,
                                       double *total_weight, void *stream) {
  if (!pr || !W || !ca || !cb) return SBDGB_E_INPUT;
  return guarded_call(pr, stream,
                      [&](cudaStream_t s) { sbdgb::string_cut_counts(pr->p, W, cutoff, ca, cb, total_weight, s); });
}

extern "C" int sbdgb_occupation_density(sbdgb_problem *pr, const double *W_dev, double *density, void *stream) {
  if (!pr || !W_dev || !density) return SBDGB_E_INPUT;
  sbdgb::Ctx *c = pr->p.ctx;
  try {
    SBDGB_CUDA(cudaSetDevice(c->device));
    cudaStream_t s = stream ? (cudaStream_t)stream : c->stream;
    sbdgb::occupation_density(pr->p, W_dev, density, s);
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
