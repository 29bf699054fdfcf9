// Shared definitions of the GB300 TPB engine (device data layout, launch
// bookkeeping, error handling).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <array>
#include <cstdio>
#include <map>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "df.cuh"
#include "sbdgb.h"

namespace sbdgb {

// ---- errors ----------------------------------------------------------------

struct Error : std::runtime_error {
  int status;
  Error(int s, const std::string &m) : std::runtime_error(m), status(s) {}
};

#define SBDGB_CUDA(call)                                                                         \
  do {                                                                                            \
    cudaError_t _e = (call);                                                                      \
    if (_e != cudaSuccess)                                                                        \
      throw ::sbdgb::Error(SBDGB_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(_e));     \
  } while (0)

#define SBDGB_REQUIRE(cond, status, msg)                      \
  do {                                                        \
    if (!(cond)) throw ::sbdgb::Error((status), (msg));       \
  } while (0)

// ---- bit helpers ------------------------------------------------------------

// Orbitals [lo, hi) as a mask (0 <= lo <= hi <= 64).
__host__ __device__ inline uint64_t range_mask(int lo, int hi) {
  uint64_t h = (hi >= 64) ? ~0ull : ((1ull << hi) - 1ull);
  uint64_t l = (lo >= 64) ? ~0ull : ((1ull << lo) - 1ull);
  return (hi <= lo) ? 0ull : (h & ~l);
}

// The reference counts fermionic phases on the alpha/beta interleaved
// determinant (alpha p -> spin orbital 2p, beta p -> 2p+1;
// chemistry/basic/determinants.h:105-150): parity(start, end) is the parity of
// the occupied spin orbitals strictly between start and end
// (determinants.h:242-294; the start bit is excluded by its second flip).
// For spin orbitals s < e that set splits into an alpha-orbital range and a
// beta-orbital range, so the phase is popc(alpha & ma) + popc(beta & mb).
__host__ __device__ inline void interval_masks(int s, int e, uint64_t &ma, uint64_t &mb) {
  // alpha p with s < 2p < e ; beta p with s < 2p+1 < e
  int a_lo = s / 2 + 1, a_hi = (e - 1) / 2 + 1;
  int b_lo = (s + 1) / 2, b_hi = (e >= 2) ? (e - 2) / 2 + 1 : 0;
  ma = range_mask(a_lo, a_hi);
  mb = range_mask(b_lo, b_hi);
}

__host__ __device__ inline int pair_index(int i, int j) {
  int a = i > j ? i : j, b = i > j ? j : i;
  return a * (a + 1) / 2 + b;
}

// ---- device-side tables -------------------------------------------------------

// Excitation lists of one spin, CSR over bra strings, structure of arrays.
//  singles: code = cr | an << 8 | P << 16 (P = pair_index(cr, an)) | sgn << 31
//           val  = same-spin part of the element without phase:
//                  h(an,cr) + sum_{j in bra, same spin} [(an cr|j j) - (an j|j cr)]
//           mask = opposite-spin orbitals that enter the phase
//           sgn  = phase from the same-spin orbitals
//  doubles: code = cr0 | cr1 << 6 | an0 << 12 | an1 << 18 (spatial)
//           val  = same-spin phase * flip * [(a0 c0|a1 c1) - (a0 c1|a1 c0)]
//           mask = opposite-spin orbitals that enter the phase
struct SpinTables {
  uint32_t n = 0;
  uint64_t ns = 0, nd = 0;
  uint32_t *off_s = nullptr, *off_d = nullptr;  // n+1
  uint32_t *ket_s = nullptr, *ket_d = nullptr;
  uint32_t *code_s = nullptr, *code_d = nullptr;
  double *val_s = nullptr, *val_d = nullptr;
  uint64_t *mask_s = nullptr, *mask_d = nullptr;
  uint32_t *bra_s = nullptr, *bra_d = nullptr;  // bra string of each entry (the CSR row, flattened)
};

struct SigmaArgs {
  const uint64_t *astr, *bstr;
  uint32_t na, nb;
  const double *hii;
  const double *C;   // N, row-major [ia][ib]
  const double *CT;  // N, transposed [ib][ia]
  double *S;
  int accumulate;
  SpinTables A, B;
  const double *Jb;  // [npair][nb]: sum_{q in beta(ib)} (P|qq)
  const double *Ja;  // [npair][na]: sum_{q in alpha(ia)} (P|qq)
  const double *Kp;  // [npair][npair] full (P|Q)
  int npair;
  int norb;
};

// ---- context / problem ----------------------------------------------------------

struct Ctx;

// Reusable device buffers of a problem (grown on demand, freed with it).
enum WsSlot {
  WS_V, WS_HV, WS_X, WS_HX, WS_T, WS_PARTIAL, WS_RED, WS_COEF,
  WS_DIAG0, WS_DIAG1, WS_DIAG2,
  WS_VF, WS_HVF, WS_CF, WS_SF, WS_RES64, WS_C64, WS_TUNE,
  WS_U, WS_UF, WS_RED2, WS_NORM_A, WS_NORM_B, WS_OCC, WS_RDM1, WS_RDM2, WS_RDMAB, WS_CTMV,
  WS_VD, WS_HVD, WS_XD, WS_HXD, WS_TD, WS_UD,
  WS_COUNT
};

struct Problem {
  Ctx *ctx = nullptr;
  int norb = 0, npair = 0;
  uint32_t na = 0, nb = 0;
  uint64_t N = 0;
  int nocc_a = 0, nocc_b = 0;
  double ecore = 0.0;
  // device
  uint64_t *astr = nullptr, *bstr = nullptr;
  double *h1 = nullptr;   // L*L
  double *Kp = nullptr;   // npair*npair
  double *Jdiag = nullptr;  // L*L (pp|qq)
  double *Xdiag = nullptr;  // L*L (pq|qp)
  SpinTables A, B;
  double *Jb = nullptr, *Ja = nullptr;
  double *hii = nullptr;
  double *CT = nullptr;   // transpose scratch
  float *CTf = nullptr;   // mixed transpose scratch
  float *Kpf = nullptr, *Jbf = nullptr, *Jaf = nullptr;
  dfloat *hii_df = nullptr;  // hii as double-float (FP32 and double-float kernels)
  float *hii_f = nullptr;    // hii in FP32 (the FP32 kernels' unshifted products)
  // double-float copies of the tables and integral tables (double-float phase of the mixed form)
  dfloat *Kpd = nullptr, *Jbd = nullptr, *Jad = nullptr;
  dfloat *val_sd[2] = {nullptr, nullptr}, *val_dd[2] = {nullptr, nullptr};
  bool df_ready = false;
  float *val_sf[2] = {nullptr, nullptr}, *val_df[2] = {nullptr, nullptr};
  void *ws[WS_COUNT] = {};
  size_t ws_bytes[WS_COUNT] = {};
  bool tables = false, diag = false, mixed_ready = false;
  // Work-balanced row tiles of the sigma kernels, per spin and per row cap
  // (8 or 16): tile t covers rows [start[t], start[t+1]), and CTAs take the
  // tiles in order[] (heaviest first).
  uint32_t *tile_start[2][2] = {}, *tile_order[2][2] = {};
  uint32_t n_tiles[2][2] = {};
  // autotuned sigma tile shapes: FP64, FP32, double-float, in the interleaved
  // (0..2) and block (3..5) orderings
  int tune_a[6] = {-1, -1, -1, -1, -1, -1}, tune_b[6] = {-1, -1, -1, -1, -1, -1};
  float tune_ms[6][3][8] = {};  // timings the autotuner saw (A, B, fused + sparse)
  // 1: the alpha x beta single pairs run in their own kernel (sigma_ab.cu)
  // after the tuned shapes, which then skip them; -1 = not decided yet
  int split_ab[6] = {-1, -1, -1, -1, -1, -1};
  float tune_ab_ms[6][2] = {};  // the autotuner's time of the tuned shapes without and with the split
  // work order of the alpha x beta kernel (sigma_ab.cu): alpha rows with at
  // least one single (most singles first); beta columns by decreasing single
  // count in slices of 32, each slice's beta singles interleaved by lane
  uint32_t *ab_rows = nullptr, *ab_cols = nullptr, *ab_slice = nullptr, *ab_ent = nullptr;
  uint64_t *ab_mask = nullptr;
  uint32_t n_ab_rows = 0, n_ab_slices = 0;
  // the row kernel for sparse rows (sigma_stream.cu): every beta pair in
  // column order, runs padded not to cross 32 entries, and its row order
  uint4 *rp_ent = nullptr;
  uint32_t *rp_rows = nullptr;
  uint32_t rp_n = 0, rp_maxrun = 0;
  bool rp_ready = false;
  size_t bytes = 0;
  std::vector<void *> allocs;
  // host copies of strings
  std::vector<uint64_t> h_astr, h_bstr;
};

struct Ctx {
  int device = 0;
  size_t budget = 0;
  size_t in_use = 0;
  uint64_t launches = 0;
  std::string last_error;
  std::mutex mu;
  cudaStream_t stream = nullptr;      // stream in use
  cudaStream_t own_stream = nullptr;  // stream created with the context
  bool timing = false;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> sigma_events;
  std::vector<cudaEvent_t> event_pool;
  // Serving contexts: device memory comes from a shared stream-ordered pool
  // (allocation and release never synchronise the device), and sigma takes
  // its tile shapes from the problem size instead of timing candidates.
  cudaMemPool_t pool = nullptr;
  bool autotune = true;
  double *pinned = nullptr;  // page-locked read-back buffer (kPinnedDoubles), made on first use
  // Autotuned sigma shapes by problem shape (precision, norb, na, nb, alpha and
  // beta table entries): a problem of a shape seen before on this context takes
  // the shapes the autotuner chose then instead of timing the candidates again.
  struct Tuned {
    int a, b, split_ab;
    float ms[3][8];
    float ab_ms[2];
  };
  std::map<std::array<uint64_t, 6>, Tuned> tuned;
};

constexpr size_t kPinnedDoubles = 16384;
double *pinned_buffer(Ctx *c);

// sigma timing hooks (api.cu)
cudaEvent_t timing_event(Ctx *c);

void *dev_alloc(Problem &p, size_t bytes);
// Raises a kernel's dynamic shared-memory limit on the current device to at
// least `bytes`, never lowering it.  The limit belongs to the function, not to
// a context or a stream: serving workers run problems of different sizes on
// concurrent threads, and one that set a smaller limit between another's
// setting and launch made that launch fail.
void ensure_dynamic_smem(const void *kernel, size_t bytes);
// Asks for the largest shared-memory carveout for a kernel (once per kernel and
// device): kernels that stage tens of KB per CTA otherwise fit one CTA per SM.
void prefer_shared_carveout(const void *kernel);
// Temporary device buffer outside the problem's accounting (pool-aware).
void *tmp_alloc(Ctx *c, size_t bytes);
void tmp_free(Ctx *c, void *d);
// Upper bound of the device bytes a problem holds through a solve with
// options o, given its excitation-table entries (singles + doubles) per spin.
size_t solve_footprint(int norb, size_t na, size_t nb, const sbdgb_davidson_opts &o, uint64_t entries_a,
                       uint64_t entries_b);
void *workspace(Problem &p, int slot, size_t bytes);
void release_workspace(Problem &p, int slot);
void dev_free_all(Problem &p);

// counted kernel launch helper
inline void count_launch(Ctx *c, uint64_t n = 1) { c->launches += n; }

// tables.cu
void build_tables(Problem &p, cudaStream_t s);
void export_tables(const Problem &p, int spin, uint64_t *off_s, uint64_t *ket_s, int32_t *cran_s,
                   uint64_t *off_d, uint64_t *ket_d, int32_t *cran_d);
// diag.cu
void build_diag(Problem &p, cudaStream_t s);
// sigma.cu
void build_row_tiles(Problem &p, cudaStream_t s);
// sigma_ab.cu: whether the alpha x beta kernel's shared-memory staging (C
// rows and (P|Q) rows of its element type T) fits this problem; its work
// order from the host copies of the single-excitation offsets of both spins.
template <typename T>
bool ab_fits(const Problem &p);
void build_ab_order(Problem &p, const std::vector<uint32_t> &off_a, const std::vector<uint32_t> &off_b,
                    cudaStream_t s);
// sigma_stream.cu: the row kernel's beta pair list (off_s, off_d: host copies
// of the beta tables' offsets; rows: the order the CTAs take the alpha rows),
// and whether the kernel fits this problem in element type T.
void build_row_pairs(Problem &p, const std::vector<uint32_t> &off_s, const std::vector<uint32_t> &off_d,
                     const std::vector<uint32_t> &rows, cudaStream_t s);
template <typename T>
bool rows_fit(const Problem &p);
// block: the block-ordering product (H_block = eta H eta, no opposite-spin
// parities) that the solvers use on eta-signed vectors; false: the
// reference's interleaved convention.
void sigma_fp64(Problem &p, const double *C, double *S, int accumulate, cudaStream_t s, bool block = false);
void sigma_fp64_scratch(Problem &p, const double *C, double *S, int accumulate, double *CT, cudaStream_t s);
// (H - shift) C in the mixed form: the diagonal term is formed in FP64 before
// the result is rounded, so a shift near the spectrum keeps FP32 outputs small.
void sigma_mixed(Problem &p, const float *C, float *S, cudaStream_t s, double shift = 0.0, bool block = false);
// The same for nvec <= 4 vectors at once (inputs and outputs at stride N).
void sigma_mixed_multi(Problem &p, const float *C, float *S, int nvec, cudaStream_t s, double shift = 0.0,
                       bool block = false);
void prepare_mixed(Problem &p, cudaStream_t s);
// Double-float form: (H - shift) C, or accumulated into S (the second phase of the mixed solver).
void sigma_df(Problem &p, const dfloat *C, dfloat *S, int accumulate, cudaStream_t s, double shift = 0.0,
              bool block = false);
// x_j *= eta for nvec vectors of N (T = double, float or dfloat): converts
// between the interleaved convention and the block one (an involution).
template <typename T>
void apply_eta(Problem &p, T *x, int nvec, cudaStream_t s);
void prepare_df(Problem &p, cudaStream_t s);
void split_hii(Problem &p, cudaStream_t s);
// davidson.cu
void davidson(Problem &p, const sbdgb_davidson_opts &o, double *E, double *X, sbdgb_report *rep);
void lanczos(Problem &p, const sbdgb_davidson_opts &o, double *E, double *X, sbdgb_report *rep);
// batch.cu
void batch_davidson(Ctx &c, Problem **ps, int count, const sbdgb_davidson_opts &o, double *E, sbdgb_report *reps,
                    double **X);

}  // namespace sbdgb

// Opaque handles of the C ABI.
struct sbdgb_ctx {
  sbdgb::Ctx c;
};
struct sbdgb_problem {
  sbdgb::Problem p;
};
