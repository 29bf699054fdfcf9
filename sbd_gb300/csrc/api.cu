// C ABI of the engine (include/sbdgb.h): context and problem lifetime, input
// validation, HBM accounting, and the status/exception boundary.
#include <algorithm>
#include <cstring>
#include <set>

#include "common.cuh"

namespace sbdgb {

void unpack_integrals(Problem &p, const double *eri_dev, cudaStream_t s);

void *tmp_alloc(Ctx *c, size_t bytes) {
  if (bytes == 0) bytes = 8;
  void *d = nullptr;
  cudaError_t e = c->pool ? cudaMallocFromPoolAsync(&d, bytes, c->pool, c->stream) : cudaMalloc(&d, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    throw Error(SBDGB_E_NOMEM, std::string("device allocation failed: ") + cudaGetErrorString(e));
  }
  return d;
}

// Pool memory is released in stream order; plain memory after the stream
// has drained (cudaFree would otherwise wait for the whole device).
void tmp_free(Ctx *c, void *d) {
  if (!d) return;
  if (c->pool) {
    cudaFreeAsync(d, c->stream);
  } else {
    cudaStreamSynchronize(c->stream);
    cudaFree(d);
  }
}

void *dev_alloc(Problem &p, size_t bytes) {
  if (bytes == 0) bytes = 8;
  Ctx *c = p.ctx;
  if (c->budget && c->in_use + bytes > c->budget)
    throw Error(SBDGB_E_NOMEM, "HBM budget exceeded (" + std::to_string(c->in_use + bytes) + " > " +
                                   std::to_string(c->budget) + " bytes)");
  void *d = tmp_alloc(c, bytes);
  p.allocs.push_back(d);
  p.bytes += bytes;
  c->in_use += bytes;
  return d;
}

void ensure_dynamic_smem(const void *kernel, size_t bytes) {
  static std::mutex mu;
  static std::map<std::pair<int, const void *>, size_t> set;
  int dev = 0;
  SBDGB_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(mu);
  size_t &have = set[{dev, kernel}];
  if (bytes <= have) return;
  SBDGB_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  have = bytes;
}

void prefer_shared_carveout(const void *kernel) {
  static std::mutex mu;
  static std::set<std::pair<int, const void *>> done;
  int dev = 0;
  SBDGB_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(mu);
  if (!done.insert({dev, kernel}).second) return;
  SBDGB_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                                  (int)cudaSharedmemCarveoutMaxShared));
}

void *workspace(Problem &p, int slot, size_t bytes) {
  if (bytes == 0) bytes = 8;
  if (p.ws[slot] && p.ws_bytes[slot] >= bytes) return p.ws[slot];
  if (p.ws[slot]) release_workspace(p, slot);
  Ctx *c = p.ctx;
  if (c->budget && c->in_use + bytes > c->budget)
    throw Error(SBDGB_E_NOMEM, "HBM budget exceeded by a solver workspace");
  void *d = tmp_alloc(c, bytes);
  p.ws[slot] = d;
  p.ws_bytes[slot] = bytes;
  p.bytes += bytes;
  c->in_use += bytes;
  return d;
}

void release_workspace(Problem &p, int slot) {
  if (!p.ws[slot]) return;
  tmp_free(p.ctx, p.ws[slot]);
  p.bytes -= p.ws_bytes[slot];
  p.ctx->in_use -= p.ws_bytes[slot];
  p.ws[slot] = nullptr;
  p.ws_bytes[slot] = 0;
}

void dev_free_all(Problem &p) {
  Ctx *c = p.ctx;
  if (!c) return;
  if (!c->pool && c->stream) cudaStreamSynchronize(c->stream);
  for (void *d : p.allocs) {
    if (c->pool)
      cudaFreeAsync(d, c->stream);
    else
      cudaFree(d);
  }
  for (int i = 0; i < WS_COUNT; ++i) {
    if (!p.ws[i]) continue;
    if (c->pool)
      cudaFreeAsync(p.ws[i], c->stream);
    else
      cudaFree(p.ws[i]);
    p.ws[i] = nullptr;
    p.ws_bytes[i] = 0;
  }
  c->in_use -= std::min(c->in_use, p.bytes);
  p.allocs.clear();
  p.bytes = 0;
}

size_t solve_footprint(int norb, size_t na, size_t nb, const sbdgb_davidson_opts &o, uint64_t entries_a,
                       uint64_t entries_b) {
  const size_t N = na * nb, L = (size_t)norb, npair = L * (L + 1) / 2;
  const bool mixed = o.precision == SBDGB_MIXED;
  const size_t k = (size_t)std::max(1, o.nroots);
  size_t b = 0;
  // strings, h1, (P|Q)
  b += 8 * (na + nb) + 8 * L * L + 8 * npair * npair;
  // tables: per spin four offset arrays, 24 bytes per entry; (pp|qq), (pq|qp), Coulomb rows
  b += 16 * (na + nb + 2) + 16 + 28 * (entries_a + entries_b) + 16 * L * L + 8 * npair * (na + nb);
  b += 16 * (na + nb + 4);  // sigma row tiles (two row caps, start + order per spin)
  // diagonal and its workspaces
  b += 8 * N + 8 * (na + nb + 2) + 8 * (na * L + 1);
  // work order of the alpha x beta kernel: rows, columns, slice starts, and
  // 12 bytes per beta single in slices of 32 (padding at most 31 x the
  // longest list, itself at most L^2 / 4 singles)
  b += 4 * (na + nb) + 4 * (nb / 32 + 2) + 12 * (entries_b + 32 * (L * L / 4 + 1));
  b += 16 * (entries_b + 32 * (nb + 1)) + 4 * na;  // the row kernel's beta pair list (padded) and row order
  // FP64 sigma transpose scratch (also used by the mixed refinement)
  b += 8 * N;
  // solver reductions (partial sums of at most 4 blocks per SM of 64 values, staging)
  b += 8 * (size_t)(1024 * 32 * 16 + 64) + 8 * 4096 + 8 * 8192;
  const size_t max_nb = std::min<size_t>((size_t)std::max(o.max_nb, 2 * (int)k), std::max<size_t>(N, 1));
  if (!mixed) {
    b += 16 * N * max_nb + 64 * N * k;  // basis and sigma; 3k restart vectors and their sigma; T; U
  } else if (o.refine_every == 0) {
    // three-phase form: the FP32 solver's buffers and the double-float
    // solver's (its start block holds up to 2k seeds), 2k FP64 seed vectors,
    // the final FP64 check's buffers (subspace at most 4k), FP32 and
    // double-float tables, the FP32 transpose and multi-vector scratch
    b += 8 * N * max_nb + 32 * N * k;
    b += 16 * N * max_nb + 72 * N * k;
    b += 16 * N * k;
    b += 16 * N * std::min<size_t>(max_nb, 4 * k) + 64 * N * k;
    b += 4 * npair * npair + 4 * npair * (na + nb) + 4 * (entries_a + entries_b) + 16;
    b += 8 * npair * npair + 8 * npair * (na + nb) + 8 * (entries_a + entries_b) + 32;
    b += 4 * N + 4 * N * std::min<size_t>(4, k);
    b += 8 * N + 4 * N;  // the diagonal as double-float and as FP32
  } else {
    const size_t mmax = (size_t)std::max(std::min(o.max_nb, 64) - (int)k, 2 * (int)k);
    b += 4 * npair * npair + 4 * npair * (na + nb) + 4 * (entries_a + entries_b) + 16;  // FP32 tables
    b += 4 * N;                                                                          // FP32 transpose
    b += 4 * N * std::min<size_t>(4, k);  // transposed copies of the vectors of one multi-vector product
    b += 32 * N * k + 4 * N * (k + mmax) + 4 * N * mmax + 12 * N * k + 4 * (8 * 3 * 64 + 64);
    b += 8 * N + 4 * N;  // the diagonal as double-float (hi and lo FP32 parts) and as FP32
  }
  return b;
}

double *pinned_buffer(Ctx *c) {
  if (!c->pinned) SBDGB_CUDA(cudaMallocHost(&c->pinned, sizeof(double) * kPinnedDoubles));
  return c->pinned;
}

cudaEvent_t timing_event(Ctx *c) {
  if (!c->event_pool.empty()) {
    cudaEvent_t e = c->event_pool.back();
    c->event_pool.pop_back();
    return e;
  }
  cudaEvent_t e;
  SBDGB_CUDA(cudaEventCreate(&e));
  return e;
}

}  // namespace sbdgb


using sbdgb::Error;

namespace {

template <typename F>
int guarded(sbdgb::Ctx *c, F &&f) {
  try {
    if (c) SBDGB_CUDA(cudaSetDevice(c->device));
    f();
    if (c) c->last_error.clear();
    return SBDGB_OK;
  } catch (const Error &e) {
    if (c) c->last_error = e.what();
    return e.status;
  } catch (const std::exception &e) {
    if (c) c->last_error = e.what();
    return SBDGB_E_INPUT;
  }
}

}  // namespace

extern "C" {

int sbdgb_abi_version(void) { return SBDGB_ABI_VERSION; }

int sbdgb_ctx_create(sbdgb_ctx **out, int device, size_t hbm_budget_bytes) {
  if (!out) return SBDGB_E_INPUT;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
    cudaGetLastError();
    return SBDGB_E_CUDA;
  }
  if (device < 0 || device >= n) return SBDGB_E_INPUT;
  sbdgb_ctx *ctx = new sbdgb_ctx();
  ctx->c.device = device;
  ctx->c.budget = hbm_budget_bytes;
  int rc = guarded(&ctx->c, [&] {
    SBDGB_CUDA(cudaStreamCreateWithFlags(&ctx->c.own_stream, cudaStreamNonBlocking));
    ctx->c.stream = ctx->c.own_stream;
  });
  if (rc != SBDGB_OK) {
    delete ctx;
    return rc;
  }
  *out = ctx;
  return SBDGB_OK;
}

void sbdgb_ctx_destroy(sbdgb_ctx *ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->c.device);
  for (auto &pr : ctx->c.sigma_events) {
    cudaEventDestroy(pr.first);
    cudaEventDestroy(pr.second);
  }
  for (auto e : ctx->c.event_pool) cudaEventDestroy(e);
  if (ctx->c.pinned) cudaFreeHost(ctx->c.pinned);
  if (ctx->c.own_stream) cudaStreamDestroy(ctx->c.own_stream);
  delete ctx;
}

const char *sbdgb_last_error(const sbdgb_ctx *ctx) { return ctx ? ctx->c.last_error.c_str() : "null context"; }

size_t sbdgb_ctx_bytes_in_use(const sbdgb_ctx *ctx) { return ctx ? ctx->c.in_use : 0; }

uint64_t sbdgb_ctx_launch_count(const sbdgb_ctx *ctx) { return ctx ? ctx->c.launches : 0; }

int sbdgb_ctx_set_stream(sbdgb_ctx *ctx, void *stream) {
  if (!ctx) return SBDGB_E_INPUT;
  return guarded(&ctx->c, [&] {
    SBDGB_CUDA(cudaStreamSynchronize(ctx->c.stream));
    ctx->c.stream = stream ? (cudaStream_t)stream : ctx->c.own_stream;
  });
}

int sbdgb_ctx_enable_timing(sbdgb_ctx *ctx, int on) {
  if (!ctx) return SBDGB_E_INPUT;
  ctx->c.timing = on != 0;
  return SBDGB_OK;
}

int sbdgb_ctx_sigma_timing(sbdgb_ctx *ctx, uint64_t *calls, double *total_ms) {
  if (!ctx) return SBDGB_E_INPUT;
  return guarded(&ctx->c, [&] {
    double ms = 0.0;
    for (auto &pr : ctx->c.sigma_events) {
      SBDGB_CUDA(cudaEventSynchronize(pr.second));
      float t = 0.f;
      SBDGB_CUDA(cudaEventElapsedTime(&t, pr.first, pr.second));
      ms += t;
      ctx->c.event_pool.push_back(pr.first);
      ctx->c.event_pool.push_back(pr.second);
    }
    if (calls) *calls = ctx->c.sigma_events.size();
    if (total_ms) *total_ms = ms;
    ctx->c.sigma_events.clear();
  });
}

int sbdgb_check_comm_sizes(sbdgb_ctx *ctx, int h_size, int b_size, int t_size) {
  return guarded(ctx ? &ctx->c : nullptr, [&] {
    SBDGB_REQUIRE(h_size == 1 && b_size == 1 && t_size == 1, SBDGB_E_UNSUPPORTED,
                  "communicators of size > 1 are not supported: one GPU per problem");
  });
}

int sbdgb_problem_footprint(int norb, size_t na, size_t nb, int max_nb, int nroots, int precision,
                            size_t *bytes) {
  if (!bytes || norb < 1 || norb > 64 || nroots < 1) return SBDGB_E_INPUT;
  sbdgb_davidson_opts o;
  sbdgb_davidson_default_opts(&o);
  o.max_nb = max_nb;
  o.nroots = nroots;
  o.precision = precision;
  *bytes = sbdgb::solve_footprint(norb, na, nb, o, 0, 0);
  return SBDGB_OK;
}

int sbdgb_problem_create(sbdgb_ctx *ctx, int norb, const uint64_t *astr, size_t na, const uint64_t *bstr,
                         size_t nb, const double *h1, const double *eri_packed, double ecore,
                         sbdgb_problem **out) {
  if (!ctx || !out) return SBDGB_E_INPUT;
  *out = nullptr;
  sbdgb_problem *pr = new sbdgb_problem();
  sbdgb::Problem &p = pr->p;
  p.ctx = &ctx->c;
  int rc = guarded(&ctx->c, [&] {
    std::lock_guard<std::mutex> lk(ctx->c.mu);
    SBDGB_REQUIRE(norb >= 1 && norb <= 64, SBDGB_E_UNSUPPORTED, "norb must be in [1, 64]");
    SBDGB_REQUIRE(na >= 1 && nb >= 1, SBDGB_E_INPUT, "empty string list");
    SBDGB_REQUIRE(na < (1ull << 31) && nb < (1ull << 31), SBDGB_E_UNSUPPORTED, "too many strings");
    SBDGB_REQUIRE((uint64_t)na * nb < (1ull << 32), SBDGB_E_UNSUPPORTED,
                  "more than 2^32 determinants (one vector alone would exceed 34 GB)");
    SBDGB_REQUIRE((uint64_t)(norb * (norb + 1) / 2) * std::max(na, nb) < (1ull << 32), SBDGB_E_UNSUPPORTED,
                  "orbital pairs x strings >= 2^32 (the Coulomb tables would exceed 34 GB)");
    SBDGB_REQUIRE(astr && bstr && h1 && eri_packed, SBDGB_E_INPUT, "null input pointer");
    const uint64_t lim = norb == 64 ? ~0ull : ((1ull << norb) - 1ull);
    auto check = [&](const uint64_t *s, size_t n, const char *name, int &nocc) {
      nocc = __builtin_popcountll(s[0]);
      for (size_t i = 0; i < n; ++i) {
        SBDGB_REQUIRE((s[i] & ~lim) == 0, SBDGB_E_INPUT, std::string(name) + " string has bits beyond norb");
        SBDGB_REQUIRE(__builtin_popcountll(s[i]) == nocc, SBDGB_E_INPUT,
                      std::string(name) + " strings have different popcounts");
        if (i) SBDGB_REQUIRE(s[i] > s[i - 1], SBDGB_E_INPUT, std::string(name) + " strings not sorted/unique");
      }
    };
    check(astr, na, "alpha", p.nocc_a);
    check(bstr, nb, "beta", p.nocc_b);
    p.norb = norb;
    p.npair = norb * (norb + 1) / 2;
    p.na = (uint32_t)na;
    p.nb = (uint32_t)nb;
    p.N = (uint64_t)na * nb;
    p.ecore = ecore;
    p.h_astr.assign(astr, astr + na);
    p.h_bstr.assign(bstr, bstr + nb);
    cudaStream_t s = ctx->c.stream;
    p.astr = (uint64_t *)sbdgb::dev_alloc(p, 8 * na);
    p.bstr = (uint64_t *)sbdgb::dev_alloc(p, 8 * nb);
    p.h1 = (double *)sbdgb::dev_alloc(p, 8 * (size_t)norb * norb);
    p.Kp = (double *)sbdgb::dev_alloc(p, 8 * (size_t)p.npair * p.npair);
    const size_t neri = (size_t)p.npair * (p.npair + 1) / 2;
    double *eri = (double *)sbdgb::tmp_alloc(&ctx->c, 8 * neri);
    SBDGB_CUDA(cudaMemcpyAsync(p.astr, astr, 8 * na, cudaMemcpyHostToDevice, s));
    SBDGB_CUDA(cudaMemcpyAsync(p.bstr, bstr, 8 * nb, cudaMemcpyHostToDevice, s));
    SBDGB_CUDA(cudaMemcpyAsync(p.h1, h1, 8 * (size_t)norb * norb, cudaMemcpyHostToDevice, s));
    SBDGB_CUDA(cudaMemcpyAsync(eri, eri_packed, 8 * neri, cudaMemcpyHostToDevice, s));
    sbdgb::unpack_integrals(p, eri, s);
    sbdgb::tmp_free(&ctx->c, eri);
    SBDGB_CUDA(cudaStreamSynchronize(s));
  });
  if (rc != SBDGB_OK) {
    sbdgb::dev_free_all(p);
    delete pr;
    return rc;
  }
  *out = pr;
  return SBDGB_OK;
}

void sbdgb_problem_destroy(sbdgb_problem *pr) {
  if (!pr) return;
  cudaSetDevice(pr->p.ctx->device);
  sbdgb::dev_free_all(pr->p);
  delete pr;
}

int sbdgb_build_tables(sbdgb_problem *pr) {
  if (!pr) return SBDGB_E_INPUT;
  return guarded(pr->p.ctx, [&] {
    SBDGB_REQUIRE(!pr->p.tables, SBDGB_E_STATE, "tables already built");
    sbdgb::build_tables(pr->p, pr->p.ctx->stream);
  });
}

int sbdgb_table_counts(const sbdgb_problem *pr, int spin, uint64_t *ns, uint64_t *nd) {
  if (!pr || (spin != 0 && spin != 1)) return SBDGB_E_INPUT;
  if (!pr->p.tables) return SBDGB_E_STATE;
  const sbdgb::SpinTables &T = spin == 0 ? pr->p.A : pr->p.B;
  if (ns) *ns = T.ns;
  if (nd) *nd = T.nd;
  return SBDGB_OK;
}

int sbdgb_export_tables(const sbdgb_problem *pr, int spin, uint64_t *off_s, uint64_t *ket_s, int32_t *cran_s,
                        uint64_t *off_d, uint64_t *ket_d, int32_t *cran_d) {
  if (!pr || (spin != 0 && spin != 1)) return SBDGB_E_INPUT;
  return guarded(pr->p.ctx, [&] {
    SBDGB_REQUIRE(pr->p.tables, SBDGB_E_STATE, "tables not built");
    sbdgb::export_tables(pr->p, spin, off_s, ket_s, cran_s, off_d, ket_d, cran_d);
  });
}

int sbdgb_diag_terms(sbdgb_problem *pr, double *hii_out) {
  if (!pr) return SBDGB_E_INPUT;
  return guarded(pr->p.ctx, [&] {
    sbdgb::Problem &p = pr->p;
    if (!p.tables) sbdgb::build_tables(p, p.ctx->stream);
    if (!p.diag) sbdgb::build_diag(p, p.ctx->stream);
    if (hii_out) {
      SBDGB_CUDA(cudaMemcpyAsync(hii_out, p.hii, 8 * p.N, cudaMemcpyDefault, p.ctx->stream));
      SBDGB_CUDA(cudaStreamSynchronize(p.ctx->stream));
    }
  });
}

int sbdgb_sigma(sbdgb_problem *pr, const double *Wk_dev, double *Wb_dev, int accumulate, void *stream) {
  if (!pr || !Wk_dev || !Wb_dev) return SBDGB_E_INPUT;
  return guarded(pr->p.ctx, [&] {
    sbdgb::Problem &p = pr->p;
    SBDGB_REQUIRE(p.tables && p.diag, SBDGB_E_STATE, "build tables and diagonal first");
    cudaStream_t s = stream ? (cudaStream_t)stream : p.ctx->stream;
    sbdgb::sigma_fp64(p, Wk_dev, Wb_dev, accumulate, s);
  });
}

int sbdgb_sigma_mixed(sbdgb_problem *pr, const float *Wk_dev, float *Wb_dev, void *stream) {
  if (!pr || !Wk_dev || !Wb_dev) return SBDGB_E_INPUT;
  return guarded(pr->p.ctx, [&] {
    sbdgb::Problem &p = pr->p;
    SBDGB_REQUIRE(p.tables && p.diag, SBDGB_E_STATE, "build tables and diagonal first");
    cudaStream_t s = stream ? (cudaStream_t)stream : p.ctx->stream;
    sbdgb::sigma_mixed(p, Wk_dev, Wb_dev, s);
  });
}

int sbdgb_sigma_df(sbdgb_problem *pr, const float *Wk_dev, float *Wb_dev, int accumulate, void *stream) {
  if (!pr || !Wk_dev || !Wb_dev) return SBDGB_E_INPUT;
  return guarded(pr->p.ctx, [&] {
    sbdgb::Problem &p = pr->p;
    SBDGB_REQUIRE(p.tables && p.diag, SBDGB_E_STATE, "build tables and diagonal first");
    SBDGB_REQUIRE(((uintptr_t)Wk_dev | (uintptr_t)Wb_dev) % 8 == 0, SBDGB_E_INPUT,
                  "double-float vectors must be 8-byte aligned");
    cudaStream_t s = stream ? (cudaStream_t)stream : p.ctx->stream;
    sbdgb::sigma_df(p, reinterpret_cast<const sbdgb::dfloat *>(Wk_dev), reinterpret_cast<sbdgb::dfloat *>(Wb_dev),
                    accumulate, s, 0.0, false);
  });
}

int sbdgb_sigma_mixed_block(sbdgb_problem *pr, const float *Wk_dev, float *Wb_dev, int nvec, void *stream) {
  if (!pr || !Wk_dev || !Wb_dev || nvec < 1) return SBDGB_E_INPUT;
  return guarded(pr->p.ctx, [&] {
    sbdgb::Problem &p = pr->p;
    SBDGB_REQUIRE(p.tables && p.diag, SBDGB_E_STATE, "build tables and diagonal first");
    cudaStream_t s = stream ? (cudaStream_t)stream : p.ctx->stream;
    for (int j = 0; j < nvec; j += 4)
      sbdgb::sigma_mixed_multi(p, Wk_dev + (size_t)j * p.N, Wb_dev + (size_t)j * p.N, std::min(4, nvec - j), s);
  });
}

int sbdgb_problem_tuning(const sbdgb_problem *pr, int precision, int *shape_a, int *shape_b, float *ms_a,
                         float *ms_b, int n_shapes) {
  if (!pr || precision < 0 || precision > 5) return SBDGB_E_INPUT;
  const sbdgb::Problem &p = pr->p;
  if (shape_a) *shape_a = p.tune_a[precision];
  if (shape_b) *shape_b = p.tune_b[precision];
  for (int i = 0; i < n_shapes && i < 8; ++i) {
    if (ms_a) ms_a[i] = p.tune_ms[precision][0][i];
    if (ms_b) ms_b[i] = p.tune_ms[precision][1][i];
  }
  return SBDGB_OK;
}

int sbdgb_problem_tuning_times(const sbdgb_problem *pr, int precision, float *ms_fused, float *ms_sparse,
                               float *ms_stream) {
  if (!pr || precision < 0 || precision > 5) return SBDGB_E_INPUT;
  const sbdgb::Problem &p = pr->p;
  for (int i = 0; i < 4; ++i)
    if (ms_fused) ms_fused[i] = p.tune_ms[precision][2][i];
  for (int i = 0; i < 2; ++i) {
    if (ms_sparse) ms_sparse[i] = p.tune_ms[precision][2][4 + i];
    if (ms_stream) ms_stream[i] = p.tune_ms[precision][2][6 + i];
  }
  return SBDGB_OK;
}

int sbdgb_problem_set_tuning(sbdgb_problem *pr, int precision, int shape_a, int shape_b) {
  if (!pr || precision < 0 || precision > 5) return SBDGB_E_INPUT;
  if (shape_a < 0 || shape_a > 3 || shape_b < 0 || shape_b > 6 || (shape_b >= 5 && shape_a > 1)) return SBDGB_E_INPUT;
  pr->p.tune_a[precision] = shape_a;
  pr->p.tune_b[precision] = shape_b;
  return SBDGB_OK;
}

int sbdgb_problem_split(const sbdgb_problem *pr, int precision, int *split, float *ms) {
  if (!pr || precision < 0 || precision > 5) return SBDGB_E_INPUT;
  if (split) *split = pr->p.split_ab[precision];
  if (ms) {
    ms[0] = pr->p.tune_ab_ms[precision][0];
    ms[1] = pr->p.tune_ab_ms[precision][1];
  }
  return SBDGB_OK;
}

int sbdgb_problem_set_split(sbdgb_problem *pr, int precision, int split) {
  if (!pr || precision < 0 || precision > 5 || split < 0 || split > 1) return SBDGB_E_INPUT;
  return guarded(pr->p.ctx, [&] {
    sbdgb::Problem &p = pr->p;
    SBDGB_REQUIRE(p.tables, SBDGB_E_STATE, "build tables first");
    const int prec = precision % 3;
    const bool fits = prec == 0   ? sbdgb::ab_fits<double>(p)
                      : prec == 1 ? sbdgb::ab_fits<float>(p)
                                  : sbdgb::ab_fits<sbdgb::dfloat>(p);
    SBDGB_REQUIRE(split == 0 || fits, SBDGB_E_UNSUPPORTED, "alpha x beta staging does not fit in shared memory");
    p.split_ab[precision] = split;
  });
}

int sbdgb_mult_host(sbdgb_problem *pr, const double *hii, const double *Wk, double *Wb) {
  if (!pr || !Wk || !Wb) return SBDGB_E_INPUT;
  return guarded(pr->p.ctx, [&] {
    sbdgb::Problem &p = pr->p;
    cudaStream_t s = p.ctx->stream;
    if (!p.tables) sbdgb::build_tables(p, s);
    if (!p.diag) sbdgb::build_diag(p, s);
    double *C = (double *)sbdgb::workspace(p, sbdgb::WS_C64, 8 * p.N);
    double *S = (double *)sbdgb::workspace(p, sbdgb::WS_RES64, 8 * p.N);
    double *saved = nullptr;
    if (hii) {  // caller-supplied diagonal (the reference takes hii as an argument)
      saved = p.hii;
      p.hii = (double *)sbdgb::workspace(p, sbdgb::WS_DIAG2, 8 * p.N);
      SBDGB_CUDA(cudaMemcpyAsync(p.hii, hii, 8 * p.N, cudaMemcpyHostToDevice, s));
    }
    SBDGB_CUDA(cudaMemcpyAsync(C, Wk, 8 * p.N, cudaMemcpyHostToDevice, s));
    SBDGB_CUDA(cudaMemcpyAsync(S, Wb, 8 * p.N, cudaMemcpyHostToDevice, s));
    try {
      sbdgb::sigma_fp64(p, C, S, 1, s);
    } catch (...) {
      if (saved) p.hii = saved;
      throw;
    }
    if (saved) p.hii = saved;
    SBDGB_CUDA(cudaMemcpyAsync(Wb, S, 8 * p.N, cudaMemcpyDeviceToHost, s));
    SBDGB_CUDA(cudaStreamSynchronize(s));
  });
}

void sbdgb_davidson_default_opts(sbdgb_davidson_opts *o) {
  if (!o) return;
  o->max_it = 100;
  o->max_nb = 20;
  o->eps = 1e-8;
  o->max_time = 0.0;
  o->nroots = 1;
  o->init = 0;
  o->precision = SBDGB_FP64;
  o->refine_every = 0;
  o->verbose = 0;
}

int sbdgb_davidson(sbdgb_problem *pr, const sbdgb_davidson_opts *o, double *E, double *X, sbdgb_report *rep) {
  if (!pr || !o || !E) return SBDGB_E_INPUT;
  return guarded(pr->p.ctx, [&] {
    sbdgb::Problem &p = pr->p;
    if (!p.tables) sbdgb::build_tables(p, p.ctx->stream);
    if (!p.diag) sbdgb::build_diag(p, p.ctx->stream);
    sbdgb::davidson(p, *o, E, X, rep);
  });
}

int sbdgb_lanczos(sbdgb_problem *pr, const sbdgb_davidson_opts *o, double *E, double *X, sbdgb_report *rep) {
  if (!pr || !o || !E) return SBDGB_E_INPUT;
  return guarded(pr->p.ctx, [&] {
    sbdgb::Problem &p = pr->p;
    if (!p.tables) sbdgb::build_tables(p, p.ctx->stream);
    if (!p.diag) sbdgb::build_diag(p, p.ctx->stream);
    sbdgb::lanczos(p, *o, E, X, rep);
  });
}

}  // extern "C"
