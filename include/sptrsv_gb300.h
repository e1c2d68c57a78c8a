/*
 * sptrsv_gb300 — sync-free sparse triangular solve for GB300 (sm_103a).
 *
 * C ABI of the library (libsptrsv_gb300.so). Plain pointers and sizes only.
 * Matrices use the reference's storage: square CSC, 0-based int32 column
 * pointers [n+1] and row indices [nnz], rows strictly ascending inside each
 * column, the diagonal first in every column of a lower triangle (forward
 * substitution) and last in every column of an upper triangle (backward
 * substitution). Right-hand sides and solutions are n x rhs blocks, row-major
 * by default (x[i*rhs+k], as the reference stores them) or column-major.
 *
 * Conventions
 *  - Every function returns an sptrsv_status (0 on success); none prints,
 *    aborts or exits.
 *  - Handle functions take DEVICE pointers and a CUDA stream (cudaStream_t
 *    passed as void*, NULL = legacy default stream). Work is stream-ordered.
 *  - A handle is not thread-safe; separate handles are independent.
 *  - Device waits are bounded. A wait that runs out makes the affected call
 *    report SPTRSV_ERR_TIMEOUT instead of hanging (default limit 1000 ms per
 *    wait, see SPTRSV_OPTION_TIMEOUT_MS).
 *
 * Reference interfaces this header replaces (harunsasmaz/Benchmark-SpTRSV,
 * directory SpTRSV_cuda/) are cited next to each entry point.
 */
#ifndef SPTRSV_GB300_H
#define SPTRSV_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SPTRSV_GB300_VERSION 101

/* Substitution and multi-RHS lane modes: same values as common.h:25-30. */
#define SPTRSV_SUBSTITUTION_FORWARD 0
#define SPTRSV_SUBSTITUTION_BACKWARD 1
#define SPTRSV_OPT_WARP_NNZ 1
#define SPTRSV_OPT_WARP_RHS 2
#define SPTRSV_OPT_WARP_AUTO 3

typedef enum sptrsv_status {
  SPTRSV_OK = 0,
  SPTRSV_ERR_NOT_SQUARE = -1,     /* m != n; same value the reference returns (sptrsv_syncfree_cuda.h:423-427) */
  SPTRSV_ERR_BAD_STRUCTURE = -2,  /* unsorted rows, missing/zero diagonal, wrong triangle, bad pointers */
  SPTRSV_ERR_INVALID = -3,        /* bad argument (NULL pointer, negative size, unknown enum) */
  SPTRSV_ERR_CUDA = -4,           /* a CUDA runtime call failed */
  SPTRSV_ERR_TIMEOUT = -5,        /* a bounded device wait ran out */
  SPTRSV_ERR_OOM = -6,            /* device allocation failed */
  SPTRSV_ERR_STATE = -7,          /* call out of order (e.g. solve before analyse) */
  SPTRSV_ERR_NOT_CONVERGED = -8,  /* iterative refinement missed its tolerance */
  SPTRSV_ERR_UNSUPPORTED = -9     /* valid request the library does not serve */
} sptrsv_status;

typedef enum sptrsv_layout {
  SPTRSV_LAYOUT_ROW_MAJOR = 0,    /* x[i*rhs + k] (reference layout, main.cu:332) */
  SPTRSV_LAYOUT_COL_MAJOR = 1     /* x[k*n + i] */
} sptrsv_layout;

typedef enum sptrsv_dtype {
  SPTRSV_DTYPE_F64 = 0,
  SPTRSV_DTYPE_F32 = 1
} sptrsv_dtype;

typedef enum sptrsv_schedule {
  SPTRSV_SCHED_AUTO = 0,      /* pull executor with a plan chosen from the analysis (one rhs: warp-
                                 synchronous lanes; level order, or level order inside blocks of ~32
                                 level widths when >= 96 % of the dependencies stay inside them);
                                 options the caller sets explicitly override the plan */
  SPTRSV_SCHED_PUSH = 1,      /* in-degree counters + atomic partial sums (the reference scheme) */
  SPTRSV_SCHED_PULL = 2,      /* dependency gather with value-as-flag words (deterministic) */
  SPTRSV_SCHED_LEVELSET = 3   /* level sets with one grid barrier per level */
} sptrsv_schedule;

/* Tunable options (sptrsv_gb300_set_option / get_option). */
typedef enum sptrsv_option {
  SPTRSV_OPTION_SCHEDULE = 0,     /* sptrsv_schedule */
  SPTRSV_OPTION_LANES = 1,        /* lanes per unknown: 1, 2, 4, 8, 16, 32 */
  SPTRSV_OPTION_CHUNK = 2,        /* unknowns per CTA work unit (>= 1) */
  SPTRSV_OPTION_SMEM_TIER = 3,    /* 1: in-chunk dependencies through shared memory */
  SPTRSV_OPTION_EXACT = 4,        /* 1: pull executor in the serial executor's operation order */
  SPTRSV_OPTION_ORDER_BLOCK = 5,  /* schedule: level order inside blocks of this many unknowns
                                     (1 = natural order, >= n = global level order); re-layout on change */
  SPTRSV_OPTION_TIMEOUT_MS = 6,   /* bound of every device wait, milliseconds */
  SPTRSV_OPTION_SYNC_CHECK = 7,   /* 1 (default): solve calls synchronise and report device errors;
                                     0: fully asynchronous, errors surface in sptrsv_gb300_check */
  SPTRSV_OPTION_PROFILE = 8,      /* 1: record CUDA events around each executor launch
                                     (read with sptrsv_gb300_exec_ms) */
  SPTRSV_OPTION_BLOCK = 9,        /* threads per CTA of the sync-free executors: 64, 128, 256 (0 = auto) */
  SPTRSV_OPTION_BACKOFF_NS = 10,  /* cap of the sleep between two polls of a global flag (0 = spin) */
  SPTRSV_OPTION_CTAS_PER_SM = 11, /* resident CTAs per SM of the executors (0 = as many as fit) */
  SPTRSV_OPTION_STAGED = 12,      /* 1 (default): one-rhs pull solves stream each chunk's layout slices
                                     into shared memory with bulk copies (TMA), double-buffered */
  SPTRSV_OPTION_STAGE_ENTRIES = 13, /* staged executor: dependency entries per chunk buffer (0 = auto) */
  SPTRSV_OPTION_STAGES = 14,      /* staged executor: chunk buffers in the producer/consumer ring (2-4) */
  SPTRSV_OPTION_FUSED_GRAD = 15,  /* sptrsv_gb300_solve_adjoint with d_dval: 1 = the transposed-solve
                                     kernel writes the gradient as each lambda is known; 0 (default) =
                                     transposed solve, then one gradient pass over the stored pattern */
  SPTRSV_OPTION_WARP_SYNC = 16,   /* one-rhs pull without staging: 1 = the 32 lanes of a warp advance in
                                     lockstep (fast in-warp dependency chains; blocked orders) */
  SPTRSV_OPTION_SPLIT = 17,       /* warp-synchronous one-rhs pull (not exact): dependency lists longer
                                     than this many entries are split over up to 32 lanes (default 32;
                                     0 = one lane per unknown) */
  SPTRSV_OPTION_WSYNC_BATCH = 18, /* warp-synchronous one-rhs pull (not exact): dependencies a lane loads
                                     per lockstep iteration, 1, 2 or 4 (0 = automatic: 1 for lists
                                     averaging more than 3 entries; for shorter ones 2 when at least half
                                     of the unknowns have two or more dependencies on the level just
                                     before their own, else 1; 2 for split lists and the transposed walk;
                                     sptrsv_info.wsync_batch reports the forward walk's value) */
  SPTRSV_OPTION_IMPORT = 19,      /* 1 (default): warp-synchronous one-rhs forward pull on a blocked
                                     layout (chunk = order block) gives each CTA an importer warp that
                                     copies the chunk's external dependencies into shared memory */
  SPTRSV_OPTION_UNIT_PIPELINE = 20, /* warp-synchronous one-rhs forward pull on a blocked layout (chunk =
                                     order block): 1 = one consumer warp per unit reading every operand
                                     from shared memory, fed by a bulk-copy loader warp (stages of
                                     SPTRSV_OPTION_STAGE_ENTRIES entries, default 2048, in
                                     SPTRSV_OPTION_STAGES buffers, default 3) and an importer warp, with
                                     a ring of up to 8192 value slots per unit; a power of two from 128
                                     to 8192 = that ring size cap; 0 (default) = off */
  SPTRSV_OPTION_FUSED_REFINE = 21, /* sptrsv_gb300_solve_refine: the FP32 solve, the residual and the FP32
                                     correction of the first refinement step run as one pass over the
                                     dependency DAG (pull schedules, rhs <= 64, and for one rhs only
                                     where no dependency list is split over lanes). 2 (default) = the
                                     residual of that pass in double-float on the FP32 pipe (each FP64
                                     weight as two floats, exact products and sums, ~2^-44 relative to
                                     x; FP64 only once per unknown); 1 = the residual in FP64
                                     arithmetic; 0 = separate passes (FP64 residual) */
  SPTRSV_OPTION_OPT = 22,         /* the reference's opt argument (sptrsv_syncfree_cuda.h:234-286) for
                                     solves with several right-hand sides on the push schedule (the
                                     reference's scheme): SPTRSV_OPT_WARP_NNZ = the lanes of a column's
                                     group take its entries, each looping over the right-hand sides;
                                     SPTRSV_OPT_WARP_RHS = the lanes take right-hand sides, looping over
                                     the entries; SPTRSV_OPT_WARP_AUTO (default) = the reference's rule
                                     per column: right-hand-side lanes when (entries <= rhs or rhs > 16)
                                     and entries < 2048. The pull executors always put lanes over
                                     right-hand sides (tile: SPTRSV_OPTION_RHS_TILE) */
  SPTRSV_OPTION_RHS_TILE = 23,    /* pull executors with several right-hand sides: right-hand sides each
                                     lane covers, 1, 2 or 4 (so 4-32 lanes per unknown); 0 (default) =
                                     one per lane up to 32 right-hand sides, two beyond */
  SPTRSV_OPTION_STRETCH = 24      /* batches in level order (not the level-set schedule): 1 (default) =
                                     the schedule key of an unknown is its level stretched to T =
                                     65 % of the batch's depth (or to its system's depth, if deeper),
                                     floor(level * max(T, depth(system)) / depth(system)), so every
                                     system's chain spreads over most of the launch instead of a deep
                                     system waiting behind the shallow systems' wide levels; 0 = global
                                     level order */
} sptrsv_option;

typedef struct sptrsv_info {
  int n;
  int nnz;
  int substitution;
  int nlevels;          /* level sets (findlevel.h:6-69) */
  int parallelism_min;  /* findlevel_csc statistics (findlevel.h:123-136) */
  int parallelism_avg;
  int parallelism_max;
  int max_in_degree;
  int schedule;         /* executor used by the last solve */
  int lanes;
  int chunk;
  int order_block;
  double analysis_ms;   /* device time of the last analyse */
  size_t device_bytes;  /* device memory held by the handle */
  /* one-rhs executor settings in effect (explicit options or the automatic plan) */
  int block;            /* threads per CTA */
  int warp_sync;        /* 1: warp-synchronous lanes */
  int staged;           /* 1: TMA-staged chunks */
  int split;            /* split length of the forward walk (0: one lane per unknown) */
  int locality_permille; /* automatic plan: dependencies inside order blocks, per mille */
  int unit_pipeline;    /* 1: the last one-rhs solve ran the unit pipeline (SPTRSV_OPTION_UNIT_PIPELINE) */
  int wsync_batch;      /* dependencies per lane per lockstep iteration of the forward one-rhs walk */
  int coarrive_permille; /* lists of <= 3 entries on average: unknowns with two or more dependencies
                            on the level just before their own, per mille (0 otherwise) */
} sptrsv_info;

typedef struct sptrsv_gb300_handle_s *sptrsv_handle_t;

const char *sptrsv_gb300_status_string(int status);
int sptrsv_gb300_version(void);

/* ---------------------------------------------------------------------------
 * Reference-compatible host entry point.
 * Replaces int sptrsv_syncfree_cuda(...) of sptrsv_syncfree_cuda.h:409-421
 * (VALUE_TYPE = double): host arrays in, x out (row-major n x rhs); runs the
 * analysis and the solve `repeat` times (default 100, the reference's
 * BENCH_REPEAT, see sptrsv_gb300_set_bench_repeat), writes the GFLOPS of the
 * average solve (2*rhs*nnz / t, :546-550) into *gflops, and validates x
 * against x_ref with the L1-relative test of :554-570 (x_ref may be NULL to
 * skip it). Returns 0, -1 when m != n, or another sptrsv_status. Prints the
 * reference's report lines only after sptrsv_gb300_set_verbose(1).
 * ------------------------------------------------------------------------- */
int sptrsv_syncfree_cuda(const int *cscColPtrTR, const int *cscRowIdxTR, const double *cscValTR, int m, int n,
                         int nnzTR, int substitution, int rhs, int opt, double *x, const double *b,
                         const double *x_ref, double *gflops);
void sptrsv_gb300_set_verbose(int verbose);
void sptrsv_gb300_set_bench_repeat(int repeat);
/* Same call with explicit outputs: average solve and analysis times (ms) and
 * the L1-relative error against x_ref (NaN when x_ref is NULL). */
int sptrsv_gb300_syncfree_host(const int *cscColPtrTR, const int *cscRowIdxTR, const double *cscValTR, int m, int n,
                               int nnzTR, int substitution, int rhs, int opt, double *x, const double *b,
                               const double *x_ref, double *gflops, double *solve_ms, double *analysis_ms,
                               double *l1_err);

/* ---------------------------------------------------------------------------
 * Kernel-level surface (device pointers, stream-ordered).
 * sptrsv_gb300_analyser   replaces the kernel sptrsv_syncfree_cuda_analyser
 *                         (sptrsv_syncfree_cuda.h:8-19): d_graphInDegree[r] =
 *                         number of stored entries in row r, diagonal included
 *                         (the array is zeroed first).
 * sptrsv_gb300_executor   replaces sptrsv_syncfree_cuda_executor (:21-107) and
 *                         sptrsm_syncfree_cuda_executor_update (:290-407): one
 *                         warp per column in natural order, started in ticket
 *                         order; consumes d_graphInDegree as countdown counters
 *                         (a column is ready at 1) and accumulates into
 *                         d_left_sum (n*rhs, zero on entry). Like the reference,
 *                         the caller restores d_graphInDegree and zeroes
 *                         d_left_sum before the next call. Synchronises and
 *                         reports SPTRSV_ERR_TIMEOUT if a wait ran out, and
 *                         SPTRSV_ERR_BAD_STRUCTURE (nothing written past the
 *                         caller's arrays) if a row index lies outside [0, m).
 *                         The ticket and error words live in a small device
 *                         block the library keeps per (device, stream): calls
 *                         on one stream are ordered by it, calls on different
 *                         streams (from any host threads) are independent.
 * sptrsv_gb300_analyser   skips (never writes) row indices outside [0, m).
 * ------------------------------------------------------------------------- */
int sptrsv_gb300_analyser(const int *d_cscRowIdx, int m, int nnz, int *d_graphInDegree, void *stream);
int sptrsv_gb300_executor(const int *d_cscColPtr, const int *d_cscRowIdx, const double *d_cscVal,
                          int *d_graphInDegree, double *d_left_sum, int m, int substitution, int rhs, int opt,
                          const double *d_b, double *d_x, void *stream);

/* ---------------------------------------------------------------------------
 * Handle API: analyse once, solve many.
 * ------------------------------------------------------------------------- */
int sptrsv_gb300_create(sptrsv_handle_t *handle);
int sptrsv_gb300_destroy(sptrsv_handle_t handle);
int sptrsv_gb300_set_option(sptrsv_handle_t handle, int option, long long value);
int sptrsv_gb300_get_option(sptrsv_handle_t handle, int option, long long *value);

/* Validates the CSC structure, runs the in-degree analyser, builds the CSR
 * transpose (tranpose.h:6-43), the level sets (findlevel.h:6-69) and the
 * execution schedule. d_colPtr/d_rowIdx are read during this call only.
 * Synchronises `stream`. Returns SPTRSV_ERR_NOT_SQUARE when m != n and
 * SPTRSV_ERR_BAD_STRUCTURE for malformed input. */
int sptrsv_gb300_analyse(sptrsv_handle_t handle, int m, int n, int nnz, const int *d_colPtr, const int *d_rowIdx,
                         int substitution, void *stream);
int sptrsv_gb300_get_info(sptrsv_handle_t handle, sptrsv_info *info);

/* Batch analysis: `count` independent square triangles, each lower (forward)
 * or upper (backward) per h_substitution[s], analysed into ONE handle that
 * solves all of them in one persistent launch. h_n, h_nnz, h_substitution are
 * host arrays; d_colPtr concatenates the per-system column pointer arrays
 * (n_s+1 entries each, local 0-based), d_rowIdx the per-system row indices
 * (local). Afterwards the handle behaves as one system of sum(n_s) unknowns:
 * values are the per-system value arrays concatenated, and b / x are
 * sum(n_s) x rhs blocks (system s occupies rows off_s .. off_s+n_s-1).
 * The schedule interleaves the systems block by block (or by level with
 * SPTRSV_OPTION_ORDER_BLOCK >= sum(n_s)). */
int sptrsv_gb300_analyse_batch(sptrsv_handle_t handle, int count, const int *h_n, const int *h_nnz,
                               const int *h_substitution, const int *d_colPtr, const int *d_rowIdx, void *stream);
int sptrsv_gb300_batch_count(sptrsv_handle_t handle, int *count);

/* Copies level sets out (device pointers; level_ptr[nlevels+1] with the
 * row counts of findlevel, level_item[n] the rows of each level in ascending
 * natural order). */
int sptrsv_gb300_levels(sptrsv_handle_t handle, int *d_levelPtr, int *d_levelItem, void *stream);
/* CSR of the analysed triangle (tranpose.h:6-43 applied to the CSC input):
 * d_rowPtr[n+1], d_colIdx[nnz]; d_srcIdx[nnz] (optional) gets the CSC entry of
 * each CSR entry. */
int sptrsv_gb300_csr(sptrsv_handle_t handle, int *d_rowPtr, int *d_colIdx, int *d_srcIdx, void *stream);

/* Stages matrix values (CSC order, dtype F64 or F32) for later solves that
 * pass d_val = NULL. Returns SPTRSV_ERR_BAD_STRUCTURE on a zero diagonal. */
int sptrsv_gb300_set_values(sptrsv_handle_t handle, const void *d_val, int dtype, void *stream);

/* Solves op(L) X = B for rhs right-hand sides with the analysed pattern.
 * dtype selects the arithmetic: F64 (values, b, x double) or F32 (values, b,
 * x float; F64 values are accepted and rounded). d_val = NULL uses the staged
 * values. b and x must not overlap. */
int sptrsv_gb300_solve(sptrsv_handle_t handle, const void *d_val, int dtype, int rhs, int layout, const void *d_b,
                       void *d_x, void *stream);

/* Mixed-precision solve: values and x stored and solved in FP32 with FP32
 * accumulation, accuracy recovered by iterative refinement in which only the
 * residual R = B - L X (from the FP64 values) and the update X += D run in
 * FP64. b and x are FP64 (layout as in sptrsv_gb300_solve); d_val is FP64 (or
 * NULL for the staged FP64 values). With SPTRSV_OPTION_FUSED_REFINE (default)
 * the first solve and the first correction share one sync-free pass: each
 * unknown publishes its FP32 value and its FP32 correction together, so the
 * step costs one walk of the dependency chain instead of two, and by default
 * that pass forms the residual in double-float on the FP32 pipe (this GPU's
 * FP64 FMA issues at 1/64 of the FP32 rate with 64 cycles of latency);
 * further steps run as separate residual (FP64), solve and update passes. Stops when the estimated relative forward
 * error ||D_k||^2 / (||D_{k-1}|| ||X||) (max norms; D_0 = X_0) is at most
 * `tol`, after at least one refinement step and at most `max_iter`; tol <= 0
 * runs exactly max_iter steps without reading anything back (asynchronous,
 * capturable). Returns SPTRSV_ERR_NOT_CONVERGED when tol > 0 is not met; the
 * steps taken and the final estimate go to *iters and *est (may be NULL). */
int sptrsv_gb300_solve_refine(sptrsv_handle_t handle, const double *d_val, int rhs, int layout, const double *d_b,
                              double *d_x, double tol, int max_iter, int *iters, double *est, void *stream);

/* Transposed (adjoint) solve op(L)^T Lambda = G on the same analysis, walked
 * in reverse dependency order (pull executor). With d_x (the forward solution
 * X, same layout) and d_dval both non-NULL, the call also writes (in the solve
 * kernel or in one pass after it, SPTRSV_OPTION_FUSED_GRAD) the
 * gradient of a loss with dLoss/dX = G with respect to every stored value:
 * d_dval[e] = -sum_k Lambda[row(e),k] * X[col(e),k] (CSC entry order); the
 * gradient with respect to B is Lambda itself. d_val as in sptrsv_gb300_solve. */
int sptrsv_gb300_solve_adjoint(sptrsv_handle_t handle, const void *d_val, int dtype, int rhs, int layout,
                               const void *d_g, void *d_lambda, const void *d_x, void *d_dval, void *stream);

/* Standalone gradient kernel: d_dval[e] = -sum_k Lambda[row(e),k] * X[col(e),k]
 * over the stored pattern (CSC entry order). */
int sptrsv_gb300_grad_values(sptrsv_handle_t handle, int dtype, int rhs, int layout, const void *d_lambda,
                             const void *d_x, void *d_dval, void *stream);

/* CUDA graphs of the solve path (analyse once, replay many). kind 0 captures
 * `count` consecutive solves of the staged values (dtype/rhs/layout/b/x as in
 * sptrsv_gb300_solve, d_val = NULL); kind 1 captures one mixed-precision
 * refinement with exactly `count` refinement steps (tol <= 0 semantics; F64
 * b/x). One eager run before the capture sizes every workspace. Replays are
 * asynchronous: use sptrsv_gb300_check to read device errors. The graph keeps
 * pointers to b, x and the handle's buffers; changing the schedule or
 * re-staging values invalidates it. */
int sptrsv_gb300_graph_create(sptrsv_handle_t handle, int kind, int dtype, int rhs, int layout, const void *d_b,
                              void *d_x, int count, void **graph, void *stream);
int sptrsv_gb300_graph_launch(void *graph, void *stream);
int sptrsv_gb300_graph_destroy(void *graph);

/* Autotuner: times candidate executor configurations on this request,
 * `reps` timed solves each, skips candidates that fail, and leaves the
 * fastest configuration set on the handle (values re-staged from d_val).
 * Axes: executor family (pull warp-synchronous / staged / thread per unknown,
 * level sets, push), order block (candidates derived from the analysed level
 * widths: blocks of 16, 32 and 64 average level widths, besides global level
 * order), chunk size, threads per CTA, residency, poll back-off, lockstep
 * batch, split lists, shared- vs global-memory tier for in-chunk dependencies
 * (SPTRSV_OPTION_SMEM_TIER) and, with several right-hand sides, the
 * right-hand-side tile (SPTRSV_OPTION_RHS_TILE) and the reference's lane
 * modes (SPTRSV_OPTION_OPT) on the push schedule.
 * *best_ms (may be NULL) receives its median solve time. Read the chosen
 * options back with sptrsv_gb300_get_option. */
int sptrsv_gb300_tune(sptrsv_handle_t handle, const void *d_val, int dtype, int rhs, int layout, const void *d_b,
                      void *d_x, int reps, double *best_ms, void *stream);

/* ---------------------------------------------------------------------------
 * Allocation-free solve. No counterpart in the reference: it exists for
 * callers that may not allocate device memory themselves — code running
 * under a host framework that owns the whole device-memory budget (every
 * byte must come from its allocator or pool) and latency-critical loops that
 * cannot accept the device-wide synchronisation a cudaMalloc/cudaFree can
 * imply. One forward or backward FP64 solve with one right-hand side on a
 * CSC triangle (device pointers, reference conventions), using the
 * kernel-level analyser and executor with all scratch (counters, partial
 * sums, control words) in a fixed device array inside the library, sized for
 * at most SPTRSV_NOALLOC_MAX_N unknowns (about 3 MB, held by every GPU that
 * loads the library until the process exits). Larger n returns
 * SPTRSV_ERR_UNSUPPORTED. The structure is validated on the device before the
 * solve, in the same stream; malformed input (column pointers, a row index
 * outside [0, n), unsorted rows, a misplaced or missing diagonal, the wrong
 * triangle) returns SPTRSV_ERR_BAD_STRUCTURE and writes nothing past the array. The first call on a device looks up the array's
 * address (once per device); make it before any stream capture. All calls
 * share the array and each clears it before use, so calls whose GPU work
 * overlaps race: serialise them. Synchronises `stream`; returns
 * SPTRSV_ERR_TIMEOUT if a bounded device wait ran out. Allocates nothing.
 * ------------------------------------------------------------------------- */
#define SPTRSV_NOALLOC_MAX_N 262144
int sptrsv_gb300_solve_noalloc(const int *d_colPtr, const int *d_rowIdx, const double *d_val, int n, int nnz,
                               int substitution, const double *d_b, double *d_x, void *stream);

/* Synchronises `stream` and reports (then clears) a device error raised by
 * asynchronous solves since the last check. */
int sptrsv_gb300_check(sptrsv_handle_t handle, void *stream);

/* Device time (ms) of the executor kernel of the last solve, measured with
 * CUDA events on the solve's stream when SPTRSV_OPTION_PROFILE is 1 (waits
 * for that kernel to finish). Workspace preparation is excluded. */
int sptrsv_gb300_exec_ms(sptrsv_handle_t handle, double *ms);

#ifdef __cplusplus
}
#endif

#endif /* SPTRSV_GB300_H */
