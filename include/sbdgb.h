/*
 * sbdgb.h -- C ABI of the GB300 tensor-product-basis (TPB) engine.
 *
 * The engine computes the selected-CI Hamiltonian-vector product
 * sigma = H*C on one GPU, its helper tables and diagonal, and the Davidson
 * eigensolver around it, for the problems the reference's TPB path solves
 * (alpha/beta string lists + FCIDUMP integrals, MPI communicators of size 1).
 *
 * Every entry point returns an int status (SBDGB_OK on success); nothing
 * throws across the ABI.  sbdgb_last_error() gives the message of the last
 * failing call on a context.  All pointers are plain host or device pointers;
 * "_dev" names device memory, everything else is host memory.
 *
 * Data conventions (identical to the reference's):
 *   - a spin string is one uint64, bit p = orbital p (norb <= 64); lists are
 *     sorted ascending without duplicates, and the position in the list is the
 *     string index (framework/bit_manipulation.h:386-439);
 *   - determinant index = ia * nb + ib (beta contiguous,
 *     chemistry/tpb/mult.h:455-465);
 *   - h1 is the L x L spatial one-body matrix, eri the 8-fold packed two-body
 *     array of B(B+1)/2 doubles with B = L(L+1)/2 (chemistry/basic/
 *     integrals.h:94-102, makeintegrals.h:123-174);
 *   - spin-orbital index in exported tables: alpha p -> 2p, beta p -> 2p+1.
 */
#ifndef SBDGB_H
#define SBDGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SBDGB_ABI_VERSION 1

enum sbdgb_status {
  SBDGB_OK = 0,
  SBDGB_E_INPUT = 1,       /* malformed input (reference: std::invalid_argument) */
  SBDGB_E_UNSUPPORTED = 2, /* outside the supported envelope (norb > 64, comm size > 1, ...) */
  SBDGB_E_CUDA = 3,        /* CUDA runtime failure */
  SBDGB_E_NOMEM = 4,       /* device allocation failed or HBM budget exceeded */
  SBDGB_E_STATE = 5,       /* call made in the wrong order */
  SBDGB_E_TIMEOUT = 6      /* a bounded wait ran out */
};

enum sbdgb_precision {
  SBDGB_FP64 = 0,  /* plain: FP64 storage and arithmetic */
  SBDGB_MIXED = 1  /* FP32 phase, double-float phase, FP64 check of the result (refine_every 0),
                      or FP32 subspace with FP64 refinement (refine_every > 0) */
};

typedef struct sbdgb_ctx sbdgb_ctx;
typedef struct sbdgb_problem sbdgb_problem;

/* ---- context ------------------------------------------------------------ */

int sbdgb_abi_version(void);

/* One context per GPU.  hbm_budget_bytes = 0 means "all free memory".
 * Replaces the device set-up of the reference app (apps/
 * chemistry_tpb_selected_basis_diagonalization/main.cc:36-47). */
int sbdgb_ctx_create(sbdgb_ctx **ctx, int device, size_t hbm_budget_bytes);
void sbdgb_ctx_destroy(sbdgb_ctx *ctx);
const char *sbdgb_last_error(const sbdgb_ctx *ctx);
/* Bytes of device memory currently held by the context's problems. */
size_t sbdgb_ctx_bytes_in_use(const sbdgb_ctx *ctx);
/* Number of kernels this context has launched since creation. */
uint64_t sbdgb_ctx_launch_count(const sbdgb_ctx *ctx);

/* Runs every later call of this context on `stream` (a cudaStream_t the
 * caller keeps alive); NULL returns to the context's own stream. */
int sbdgb_ctx_set_stream(sbdgb_ctx *ctx, void *stream);

/* Sigma timing: when enabled, every sigma product records a pair of CUDA
 * events on the stream it is launched on; sbdgb_ctx_sigma_timing waits for
 * them and returns the number of products and their summed device time, then
 * clears the record.  Off by default. */
int sbdgb_ctx_enable_timing(sbdgb_ctx *ctx, int on);
int sbdgb_ctx_sigma_timing(sbdgb_ctx *ctx, uint64_t *calls, double *total_ms);

/* Checks the size of the communicators the reference would pass
 * (h_comm, b_comm, t_comm sizes; chemistry/tpb/helper.h:344-386).  Any size
 * other than 1 returns SBDGB_E_UNSUPPORTED: this engine is one GPU per
 * problem. */
int sbdgb_check_comm_sizes(sbdgb_ctx *ctx, int h_size, int b_size, int t_size);

/* ---- problem ------------------------------------------------------------ */

/* Uploads strings and integrals into context-owned device memory (the
 * reference copies them in MultTPBThrust::Init, chemistry/tpb/
 * mult_thrust.h:100-275).  astr/bstr must be sorted, duplicate-free, with
 * one popcount per list; norb <= 64. */
int sbdgb_problem_create(sbdgb_ctx *ctx, int norb, const uint64_t *astr, size_t na, const uint64_t *bstr,
                         size_t nb, const double *h1, const double *eri_packed, double ecore,
                         sbdgb_problem **out);
void sbdgb_problem_destroy(sbdgb_problem *p);
/* Upper bound of the device memory a problem holds through a Davidson solve
 * with these options, excluding its excitation tables (24 bytes per single or
 * double, 28 in the mixed form), whose size is known once they are built. */
int sbdgb_problem_footprint(int norb, size_t na, size_t nb, int max_nb, int nroots, int precision,
                            size_t *bytes);

/* Excitation tables: replaces MakeHelpers + RemakeHelpers at size 1
 * (chemistry/tpb/helper.h:729-873, 935-1245; GenerateExcitation :185-342). */
int sbdgb_build_tables(sbdgb_problem *p);
/* spin 0 = alpha, 1 = beta. */
int sbdgb_table_counts(const sbdgb_problem *p, int spin, uint64_t *n_singles, uint64_t *n_doubles);
/* Copies one spin's tables out in the reference helper layout
 * (TaskHelpers::*_flat, *Offset, *CrAn_flat; helper.h:48-65): offsets have
 * n+1 entries, kets ascending per bra, CrAn = (cr, an) for singles and
 * (cr0, cr1, an0, an1) for doubles as spin-orbital indices. */
int sbdgb_export_tables(const sbdgb_problem *p, int spin, uint64_t *off_s, uint64_t *ket_s, int32_t *cran_s,
                        uint64_t *off_d, uint64_t *ket_d, int32_t *cran_d);

/* Diagonal hii (makeQChamDiagTerms, chemistry/tpb/qcham.h:289-340).  The
 * problem keeps its own copy; hii_out may be a host pointer (copied) or NULL. */
int sbdgb_diag_terms(sbdgb_problem *p, double *hii_out);

/* sigma (sbd::mult, chemistry/tpb/mult.h:114-130; MultBase::run,
 * chemistry/basic/mult.h:19-103).  Wk_dev, Wb_dev: N = na*nb doubles of
 * device memory.  accumulate != 0 gives the reference's Wb += H*Wk,
 * accumulate == 0 writes Wb = H*Wk.  stream: a cudaStream_t, or NULL for the
 * context's stream (pass cudaStreamLegacy for the legacy default stream). */
int sbdgb_sigma(sbdgb_problem *p, const double *Wk_dev, double *Wb_dev, int accumulate, void *stream);
/* Mixed-precision sigma: FP32 vectors, FP32 products and pair-list sums, a
 * float-float accumulator per element (an FP32 sum and the rounding errors of
 * the additions into it, about 48 bits; FP32 instructions only) and the FP64
 * diagonal as FP32 hi + lo parts; FP32 result. */
int sbdgb_sigma_mixed(sbdgb_problem *p, const float *Wk_dev, float *Wb_dev, void *stream);
/* Double-float sigma: each element of Wk_dev and Wb_dev is a pair of FP32
 * numbers (hi, lo) whose sum is the value (2N floats, hi first; 48 significand
 * bits), and every product and sum is a double-float operation on the FP32
 * pipe.  This is the sigma of the second phase of the mixed solver: about
 * 2^-47 relative rounding per operation, several times the FP64 FMA rate of
 * this GPU.  accumulate as for sbdgb_sigma. */
int sbdgb_sigma_df(sbdgb_problem *p, const float *Wk_dev, float *Wb_dev, int accumulate, void *stream);
/* sbdgb_sigma_mixed for nvec vectors stored one after another (nvec*N floats
 * in and out).  Up to four vectors share each element's phase and address,
 * which is most of the FP32 kernels' work; results equal nvec single calls. */
int sbdgb_sigma_mixed_block(sbdgb_problem *p, const float *Wk_dev, float *Wb_dev, int nvec, void *stream);
/* The sigma tile shapes the autotuner picked on this problem's first product
 * (precision 0 = FP64, 1 = mixed FP32, 2 = double-float; -1 = not tuned yet) and the time it measured
 * for each of the n_shapes candidates of kernel A (alpha sweep) and B (beta
 * sweep).  Shapes: 0 = 8x128, 1 = 8x256, 2 = 8x512, 3 = 16x256 rows x columns;
 * shape_b = 4 means the beta sweep is fused into kernel A (one kernel, no
 * transposed copy; chosen when that is faster, typically for short beta lists);
 * shape_b = 5 means the single streaming kernel for sparse rows (16-byte
 * accesses along beta, every task type in one pass), with shape_a 0 or 1 for
 * row tiles of 8 or 16 rows (chosen for problems with a few nonzeros per row);
 * shape_b = 6 is the row kernel (sigma_stream.cu: one alpha row per CTA at a
 * time, every beta pair of the problem a lane's product with the row of C in
 * shared memory), with shape_a 0 = its persistent double-buffered form where
 * the row length and alignment allow it (one row per CTA of 512 threads
 * otherwise) or 1 = one row per CTA of 1024 threads.
 * The first product of each precision tunes (and synchronises), so make it
 * before any stream capture. */
int sbdgb_problem_tuning(const sbdgb_problem *p, int precision, int *shape_a, int *shape_b, float *ms_a,
                         float *ms_b, int n_shapes);
/* The autotuner's times (ms, 0 where not measured) of the fused kernel in
 * shapes 0..3 (ms_fused[4]), of the sparse-row kernel with 8 and 16 rows per
 * tile (ms_sparse[2]) and of the row kernel's two forms (ms_stream[2], in
 * shape_a order); any pointer may be NULL. */
int sbdgb_problem_tuning_times(const sbdgb_problem *p, int precision, float *ms_fused, float *ms_sparse,
                               float *ms_stream);
/* Sets the sigma tile shapes of one precision instead of the autotuner's
 * choice (shape_a 0..3 with shape_b 0..4, or shape_a 0..1 with shape_b 5 or 6,
 * as above); results do not depend on it beyond the order of floating-point sums. */
int sbdgb_problem_set_tuning(sbdgb_problem *p, int precision, int shape_a, int shape_b);
/* Whether the alpha x beta single pairs of sigma (task type 0) run in a kernel
 * of their own (split = 1: the tuned shapes skip them and a kernel that stages
 * the rows of C and (P|Q) of each alpha row's singles in shared memory adds
 * them; 0: inside the alpha sweep; -1: not decided yet), and the autotuner's
 * time of one product without and with the split (ms[2], 0 where not
 * measured; ms may be NULL).  The autotuner decides by timing; untimed
 * contexts split when there are at least 4 such pairs per determinant and
 * the staging fits in shared memory.  precision as above, + 3 for the
 * solvers' block ordering (vectors multiplied by the sign between the
 * interleaved and the block determinant).  No counterpart in the reference. */
int sbdgb_problem_split(const sbdgb_problem *p, int precision, int *split, float *ms);
/* Sets that choice (0 or 1) for one precision; 1 is refused with
 * SBDGB_E_UNSUPPORTED when the staging does not fit in shared memory. */
int sbdgb_problem_set_split(sbdgb_problem *p, int precision, int split);

/* sigma that makes no device allocation.  No counterpart in the reference:
 * it is for callers that cannot call cudaMalloc once they run (a host
 * application whose pool allocator owns the device, a replay in a fixed
 * memory plan).  Same result and arguments as sbdgb_sigma (FP64); the problem
 * must already have its tables and diagonal.  The transposed-vector scratch
 * is a file-scope device array of 2,097,152 doubles (16 MiB, held on every
 * device that loads the library until exit); larger problems return
 * SBDGB_E_UNSUPPORTED.  The first call on a device looks up the array's
 * address (make it before any stream capture; no other entry point, table
 * building and diagonal included, makes that lookup), and that address is
 * kept for the process: do not call it again after resetting the device.  All calls share the array:
 * calls that overlap on the GPU race and must be serialised by the caller.
 * It uses the autotuned tile shapes when the problem has them, the default
 * shape otherwise, and records no timing events. */
int sbdgb_sigma_noalloc(sbdgb_problem *p, const double *Wk_dev, double *Wb_dev, int accumulate, void *stream);

/* Occupation density of a vector (OccupationDensity, chemistry/tpb/
 * occupation.h:11-95, as sbd::tpb::diag reports it with do_rdm == 0,
 * sbdiag.h:666-699): density[2p] = sum over determinants of |W|^2 with alpha
 * orbital p occupied, density[2p+1] the same for beta.  W: N doubles of device
 * or host memory (a host vector is copied in); density: 2*norb doubles of host
 * memory (the call waits for it). */
int sbdgb_occupation_density(sbdgb_problem *p, const double *W, double *density, void *stream);

/* String weights of a vector, the diagonal of the half-determinant reduced
 * density matrices (DiagonalAdetReducedDensityMatrix / ...Bdet..., chemistry/
 * tpb/rdmat.h:13-60, 137-187) that carry-over selection ranks strings by:
 * wa[ia] = sum_ib |W[ia][ib]|^2 (na doubles), wb[ib] = sum_ia |W[ia][ib]|^2
 * (nb doubles), host outputs.  W: N doubles, device or host memory. */
int sbdgb_string_weights(sbdgb_problem *p, const double *W, double *wa, double *wb, void *stream);
/* For the amplitude-based basis extension (SinglesExtendHalfdets,
 * chemistry/tpb/extend.h:13-60): ca[ia] / cb[ib] = number of determinants of
 * that string with |W|^2 > cutoff, *total_weight = their summed weight. */
int sbdgb_string_cut_counts(sbdgb_problem *p, const double *W, double cutoff, uint64_t *ca, uint64_t *cb,
                            double *total_weight, void *stream);

/* One- and two-particle reduced density matrices of W (Correlation,
 * chemistry/tpb/correlation.h:379-640, as sbd::tpb::diag computes them with
 * do_rdm != 0), in the reference's layout: one = 2 blocks of norb^2 doubles
 * (spin s at s*norb^2, element i + norb*j), two = 4 blocks of norb^4 doubles
 * (spin pair s1 + 2*s2, element a + norb*b + norb^2*c + norb^3*d).  Host
 * outputs; two may be NULL (one-particle part only).  W: device or host. */
int sbdgb_rdm(sbdgb_problem *p, const double *W, double *one, double *two, void *stream);

/* Host-buffer form of sbd::mult: Wb += H*Wk with host vectors (copies
 * inside).  hii is ignored when NULL (the problem's own diagonal is used). */
int sbdgb_mult_host(sbdgb_problem *p, const double *hii, const double *Wk, double *Wb);

/* ---- Davidson ----------------------------------------------------------- */

typedef struct {
  int max_it;        /* restart cycles (reference --iteration) */
  int max_nb;        /* max subspace size (reference --block) */
  double eps;        /* residual-norm tolerance (reference --tolerance) */
  double max_time;   /* wall-clock cap in seconds (reference --max_time); <= 0: none */
  int nroots;        /* lowest roots wanted, 1..8 (the reference solves 1) */
  int init;          /* 0: unit vector on determinant 0 (reference init 0),
                        1: unit vectors on the lowest diagonal entries,
                        2: caller-supplied vectors in X */
  int precision;     /* sbdgb_precision */
  int refine_every;  /* MIXED: 0 (default) = FP32 Davidson, then double-float Davidson from its
                        lowest Ritz vectors to the tolerance, then FP64 sigma, Rayleigh-Ritz and
                        residual of the result (continuing in FP64 only if they miss it);
                        k > 0 = FP64 anchors, FP32 subspace, FP64 sigma and residual every k steps */
  int verbose;       /* print one line per iteration like the reference */
} sbdgb_davidson_opts;

typedef struct {
  int iterations;    /* Davidson steps taken */
  int sigma_calls;   /* sigma products (FP64 + mixed) */
  int sigma_fp64;    /* of which FP64 (the others FP32 or double-float) */
  int restarts;
  int converged;     /* 1 if every root reached eps */
  double seconds;    /* wall time of the solve */
  double resid[16];  /* final residual norms per root */
} sbdgb_report;

void sbdgb_davidson_default_opts(sbdgb_davidson_opts *o);
/* Davidson (chemistry/tpb/davidson.h:707-970, GPU form chemistry/basic/
 * davidson_thrust.h:97-385).  E receives nroots energies (ascending).
 * X (host, nroots*N, may be NULL) receives the normalized Ritz vectors and,
 * with init == 2, supplies the starting vectors. */
int sbdgb_davidson(sbdgb_problem *p, const sbdgb_davidson_opts *o, double *E, double *X, sbdgb_report *rep);

/* Lanczos (chemistry/tpb/lanczos.h:169-320, the solver of sbd::tpb::diag
 * --method 2): restarted Lanczos without reorthogonalisation, max_nb Krylov
 * vectors per cycle, max_it cycles, stop when the lowest Ritz value moves by
 * less than eps.  One root, FP64; init as for Davidson.  E[0] receives the
 * lowest Ritz value, X (may be NULL) the Ritz vector; rep->resid[0] is the
 * last change of the Ritz value and rep->restarts the cycles run. */
int sbdgb_lanczos(sbdgb_problem *p, const sbdgb_davidson_opts *o, double *E, double *X, sbdgb_report *rep);

/* Many small problems of one context solved together: every problem runs
 * the Davidson of sbdgb_davidson (init 1), all of them in lock step, each step
 * one kernel launch over all problems and each iteration one replay of a
 * captured CUDA graph, so a batch of thousands of small problems costs a few
 * launches per iteration instead of tens of launches and synchronisations per
 * iteration each.  No counterpart in the reference.  Options as for
 * sbdgb_davidson with nroots 1..8 and init 1; the subspace is capped at 32.
 * precision MIXED runs the iteration on FP32 vectors and an FP32 sigma until
 * every residual is below 5e-7 |E|, then in FP64 from the lowest Ritz vectors
 * of that phase to the full tolerance (rep->sigma_fp64 counts the FP64
 * products).  E: count*nroots energies; reps (may be NULL): count reports; X
 * (may be NULL, entries may be NULL): count host buffers of nroots*N for the
 * Ritz vectors.  Meant for problems of up to a few hundred thousand
 * determinants each. */
int sbdgb_batch_davidson(sbdgb_ctx *ctx, sbdgb_problem **problems, int count, const sbdgb_davidson_opts *o,
                         double *E, sbdgb_report *reps, double **X);

/* ---- serving: many solves at once, admitted by HBM footprint -------------
 * No single counterpart in the reference, whose app solves one problem per
 * run (apps/chemistry_tpb_selected_basis_diagonalization/main.cc:190-191);
 * each request is that run's diag on its own inputs. */

/* A request: the inputs of sbdgb_problem_create plus the Davidson options.
 * The server copies every input at submission except vectors_out. */
typedef struct {
  int norb;
  const uint64_t *astr;
  size_t na;
  const uint64_t *bstr;
  size_t nb;
  const double *h1;
  const double *eri_packed;
  double ecore;
  sbdgb_davidson_opts opts;
  double *vectors_out;   /* host, nroots*na*nb doubles, or NULL; must stay valid
                            until the ticket's sbdgb_server_wait returns */
} sbdgb_request;

typedef struct {
  int status;            /* SBDGB_OK or the failing step's status */
  int nroots;
  double energies[8];
  double resid[8];
  double queue_seconds;  /* submission to start */
  double run_seconds;    /* start to finish: upload, tables, diagonal, solve */
  double total_seconds;  /* submission to finish */
  int iterations;
  int sigma_calls;
  int converged;
  int worker;
  size_t reserved_bytes; /* HBM reserved for the request once its tables were built */
  uint64_t ndet;
  char message[200];     /* error message when status != SBDGB_OK */
} sbdgb_result;

typedef struct {
  uint64_t submitted, completed, failed, launches;
  size_t budget_bytes, reserved_bytes, peak_reserved_bytes;
  int workers, running, peak_running, queued;
  uint64_t batched;  /* requests solved in batched groups of two or more */
} sbdgb_serve_stats;

typedef struct sbdgb_server sbdgb_server;

/* `workers` solver threads (1..64), each with its own context and CUDA stream
 * on `device`, so that their kernels overlap on the GPU.  A queued request
 * starts when a worker is free and its reservation fits the HBM budget
 * (0 = 90% of the memory free at creation); the first queued request that
 * fits goes first, but none passes a request already passed 2*workers times.
 * A request reserves an upper bound of its device memory at submission and
 * shrinks it to its real size once its tables are built; it cannot use more
 * than it reserved.  Requests of at most 300,000 determinants that start
 * together with equal options (init 1, subspace <= 32, FP64 or the two-phase
 * mixed form) are solved as one sbdgb_batch_davidson batch of up to 64.
 * Results are those of sbdgb_davidson on the lone problem (to rounding). */
int sbdgb_server_create(int device, int workers, size_t hbm_budget_bytes, sbdgb_server **out);
/* Queues a request and returns its ticket.  SBDGB_E_NOMEM if its reservation
 * alone exceeds the budget. */
int sbdgb_server_submit(sbdgb_server *s, const sbdgb_request *req, uint64_t *ticket);
/* *done = 1 once the ticket's result is ready. */
int sbdgb_server_poll(sbdgb_server *s, uint64_t ticket, int *done);
/* Waits at most timeout_seconds (< 0: no limit) for the result; returns
 * SBDGB_E_TIMEOUT if it is not ready.  The ticket is released once read. */
int sbdgb_server_wait(sbdgb_server *s, uint64_t ticket, double timeout_seconds, sbdgb_result *out);
int sbdgb_server_stats(sbdgb_server *s, sbdgb_serve_stats *out);
const char *sbdgb_server_last_error(const sbdgb_server *s);
/* Finishes the running requests, fails the queued ones (SBDGB_E_STATE), joins
 * the workers and frees the pool.  Call it after every wait has returned. */
void sbdgb_server_destroy(sbdgb_server *s);

#ifdef __cplusplus
}
#endif
#endif
