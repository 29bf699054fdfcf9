// Mixed-precision sigma (FP32 vectors and products, FP64 accumulation).
#include "common.cuh"

namespace sbdgb {

void prepare_mixed(Problem &p, cudaStream_t s) {
  (void)p;
  (void)s;
  throw Error(SBDGB_E_UNSUPPORTED, "mixed precision sigma not built yet");
}

void sigma_mixed(Problem &p, const float *C, float *S, cudaStream_t s) {
  (void)C;
  (void)S;
  prepare_mixed(p, s);
}

}  // namespace sbdgb
