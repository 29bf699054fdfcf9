// sigma without any allocation, for callers that cannot call cudaMalloc.
//
// Some callers of this library are not allowed to allocate device memory once
// they are running: code inside a memory-pool-managed host application whose
// allocator owns the whole device, steps replayed in a fixed memory plan, or
// serving processes that must not grow their footprint after admission.  The
// regular sigma (sbdgb_sigma) allocates its transposed-vector scratch on first
// use and tunes its tile shapes on scratch memory.  This entry point computes
// the same product with the scratch in a file-scope device array instead.
//
// The array holds kNoAllocMaxDet doubles (16 MiB) on every device that loads
// the library, until the process exits.  Problems with more determinants are
// rejected with SBDGB_E_UNSUPPORTED.  Every call fully overwrites the part of
// the array it uses before reading it, so nothing has to start at zero; the
// array is shared by all calls, so calls that overlap on the GPU (different
// streams, or concurrent host threads) race on it and must be serialised by
// the caller.
#include <mutex>

#include "common.cuh"

namespace {

constexpr size_t kNoAllocMaxDet = size_t(1) << 21;  // 2,097,152 determinants

// Host code may not use this name as a device address: its address on a
// device is obtained with cudaGetSymbolAddress below.
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocMaxDet];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
double *g_scratch_on[kMaxDevices] = {};

// Device address of the scratch on the current device, looked up once per
// device (with that device current) and cached.  The cache belongs to the
// device's primary context as it was at that first call: a caller that
// resets the device (cudaDeviceReset) must not call this entry point again in
// the same process.
double *scratch_address() {
  int dev = 0;
  SBDGB_CUDA(cudaGetDevice(&dev));
  SBDGB_REQUIRE(dev >= 0 && dev < kMaxDevices, SBDGB_E_UNSUPPORTED, "device index out of range");
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_scratch_on[dev]) {
    void *ptr = nullptr;
    SBDGB_CUDA(cudaGetSymbolAddress(&ptr, g_noalloc_scratch));
    g_scratch_on[dev] = (double *)ptr;
  }
  return g_scratch_on[dev];
}

}  // namespace

extern "C" int sbdgb_sigma_noalloc(sbdgb_problem *pr, const double *Wk_dev, double *Wb_dev, int accumulate,
                                   void *stream) {
  if (!pr || !Wk_dev || !Wb_dev) return SBDGB_E_INPUT;
  sbdgb::Problem &p = pr->p;
  sbdgb::Ctx *c = p.ctx;
  try {
    SBDGB_CUDA(cudaSetDevice(c->device));
    SBDGB_REQUIRE(p.tables && p.diag, SBDGB_E_STATE, "build tables and diagonal first");
    SBDGB_REQUIRE(p.N <= kNoAllocMaxDet, SBDGB_E_UNSUPPORTED,
                  "problem has " + std::to_string(p.N) + " determinants; the allocation-free sigma holds at most " +
                      std::to_string(kNoAllocMaxDet));
    double *CT = scratch_address();
    cudaStream_t s = stream ? (cudaStream_t)stream : c->stream;
    sbdgb::sigma_fp64_scratch(p, Wk_dev, Wb_dev, accumulate, CT, s);
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
