/*
 * rschol_gpu.h -- C ABI of the GB300 rank-structured Cholesky preconditioner
 * and its PCG solve.
 *
 * Plain pointers and sizes only.  Matrices are CSC with full symmetric
 * storage (colptr[n] = nnz, 0-based int32 indices), as the reference's
 * SparseColumnMatrix (src/rschol/linearalgebra/SPARSE_MATRIX.h:187-300).
 * Host buffers unless a name ends in _device.  Every entry point returns a
 * status code and never aborts the process; rschol_last_error() gives the
 * message of the last failure on a context.
 */
#ifndef RSCHOL_GPU_H
#define RSCHOL_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

enum rschol_status {
  RSCHOL_OK = 0,
  RSCHOL_E_BAD_INPUT = 1,
  RSCHOL_E_NOT_PD_AFTER_RETRY = 2, /* IndefiniteDiagonalError of a compressed supernode after all retries */
  RSCHOL_E_OOM = 3,
  RSCHOL_E_CUDA = 4,
  RSCHOL_E_BREAKDOWN = 5,          /* PCG breakdown: d' A d == 0 */
  RSCHOL_E_TIMEOUT = 6,            /* a bounded wait between thread blocks of the factor or solve gave up */
  RSCHOL_E_NO_DEVICE = 7,
  RSCHOL_E_UNSUPPORTED = 8,
  RSCHOL_E_NOT_PD = 9              /* non-positive pivot in an uncompressed supernode (the reference aborts) */
};

enum rschol_precision {
  RSCHOL_FP64 = 0,   /* plain FP64 factor and solve */
  RSCHOL_MIXED = 1   /* FP32 factor storage and Schur/sketch products, FP64 PCG */
};

/* Factorisation parameters.  Defaults (rschol_default_params) are the
 * values the reference's pcg_solver driver passes
 * (src/pcg_solver.cpp:100-113, src/rschol/solver/FactorManager.cpp:58-71,
 * src/rschol/solver/SparseSolver.cpp:76-77). */
typedef struct rschol_params {
  int max_dense_block;       /* maxDenseBlock: larger separators are compressed (200) */
  int max_diag_block;        /* maxDiagonalBlock: HODLR leaf size bound (400) */
  int explicit_threshold;    /* diagonal blocks up to this size are built explicitly (4000) */
  int nd_leaf;               /* nested-dissection leaf size (64) */
  int oversampling;          /* OVER_SAMPLING (5) */
  int rank_cap;              /* 0 = reference rank heuristic; > 0 caps every rank */
  int power_iters;           /* POWER_ITERATIONS (1) */
  int reorder_separators;    /* sub-order separators by coordinates when given (1) */
  double rank_constant;      /* RANK_CONSTANT (0.4) */
  double diag_rank_constant; /* DIAGONAL_RANK_CONSTANT (0.5) */
  int max_factor_attempts;   /* retries on an indefinite diagonal (10) */
  double rank_alpha;         /* diagonal rank constant growth per retry (1.25) */
  unsigned seed;             /* generator reseed at every numeric factorisation (152) */
  int precision;             /* enum rschol_precision */
  int device;                /* CUDA device ordinal (0) */
  int root_fp64;             /* RSCHOL_MIXED only: the dense Cholesky of the root separator's
                                blocks in FP64, the rest of the factor FP32 (0) */
  int schur_bf16;            /* RSCHOL_MIXED only: the split-precision tensor-core products (the
                                Schur-complement updates, projections, U^T U, X doubling) as
                                BF16 hi/lo splits, three BF16 MMAs with FP32 accumulation, instead
                                of split TF32 (0) */
} rschol_params;

typedef struct rschol_ctx rschol_ctx;
typedef struct rschol_factor rschol_factor;

typedef struct rschol_pcg_info {
  int iterations;          /* PCG_SOLVER::_totalIterations for this solve */
  double residual;         /* final recurrence ||r|| / ||b|| */
  double true_residual;    /* ||b - A x|| / ||b|| recomputed at the end */
  double seconds;          /* wall time of the solve */
} rschol_pcg_info;

void rschol_default_params(rschol_params* p);

/* Context: owns the CUDA device selection, streams and error state. */
rschol_ctx* rschol_create(const rschol_params* p);
void rschol_destroy(rschol_ctx* ctx);
const char* rschol_last_error(const rschol_ctx* ctx);

/* Symbolic + numeric factorisation.
 * Replaces FactorPreconditioner::initialize
 * (src/rschol/solver/FactorPreconditioner.h:92-103, .cpp:70-131), which runs
 * SparseSolver::factorSymbolic (SparseSolver.cpp:95-154) and
 * SparseSolver::factorNumeric with its retry loop (SparseSolver.cpp:174-214).
 * xyz (3 doubles per unknown) may be NULL, as the reference's zero positions. */
int rschol_factor_create(rschol_ctx* ctx, int n, const int* colptr, const int* rowind,
                         const double* vals, const double* xyz, rschol_factor** out);

/* Whether rschol_factor_create can take this structure with these parameters
 * (NULL: the defaults): the host ordering and symbolic analysis alone, no
 * device and no values needed.  RSCHOL_OK; RSCHOL_E_BAD_INPUT for an invalid
 * pattern; RSCHOL_E_UNSUPPORTED when an uncompressed supernode would need a
 * hierarchical diagonal (one wider than max_diag_block), which the device
 * factorisation does not build.  The reason is written to msg (at most
 * msg_len bytes, NUL-terminated; msg may be NULL).  No reference counterpart:
 * the reference builds such a diagonal. */
int rschol_check_structure(int n, const int* colptr, const int* rowind, const double* xyz,
                           const rschol_params* params, char* msg, int msg_len);

/* New values, same pattern: FactorPreconditioner::initialize with only the
 * numeric factor needed (FactorPreconditioner.cpp:115-129). */
int rschol_refactor(rschol_factor* f, const double* vals);

/* Same, with the new values (full CSC order) already resident on the device. */
int rschol_refactor_device(rschol_factor* f, const double* d_vals);

void rschol_factor_free(rschol_factor* f);

/* The context's CUDA stream (cudaStream_t): every call of the context runs
 * on it and synchronises it before returning. */
void* rschol_stream(rschol_ctx* ctx);

/* CUDA-event timings on the context stream, for benchmarks: out[0] numeric
 * factorisation ms, [1] one preconditioner apply ms, [2] one SpMV ms, [3] one
 * PCG solve of d_b (device, original order) ms, [4] algorithmic bytes of an
 * apply, [5] of an SpMV, [6] factorisation launches, [7] launches of the PCG
 * solve, [10] its iterations, [11] its true residual. */
int rschol_profile(rschol_factor* f, const double* d_b, double* out);

/* x = M^{-1} b for nrhs column-major right-hand sides.
 * Replaces FactorPreconditioner::solve (FactorPreconditioner.cpp:135-162),
 * PRECONDITIONER::solve (src/rschol/linearalgebra/PRECONDITIONER.h:56). */
int rschol_precond_apply(rschol_factor* f, const double* b, double* x, int nrhs);
int rschol_precond_apply_device(rschol_factor* f, const double* d_b, double* d_x, int nrhs);

/* The same preconditioner application as rschol_precond_apply_device called
 * once per right-hand side (nrhs = 1 each time), but the call allocates no
 * device memory: for callers that apply the preconditioner inside their own
 * solver loop and cannot let a call allocate (cudaMalloc synchronises the
 * device and stalls their other streams, or their memory budget is fixed).
 * No counterpart in the reference (its solve allocates host work vectors).
 *   - n (the matrix order) must be <= RSCHOL_NOALLOC_MAX_N, otherwise
 *     RSCHOL_E_BAD_INPUT with a message naming the limit;
 *   - the permuted work vector is one static device array of
 *     RSCHOL_NOALLOC_MAX_N doubles (16 MiB) per device, shared by every
 *     factor: calls that overlap in time (other host threads, other factors'
 *     streams) race on it, so serialise them;
 *   - nothing in it has to start at zero: each right-hand side is written
 *     completely before it is read;
 *   - rschol_create looks up the array's device address (once per device,
 *     with that device current), so the call itself only reads a pointer;
 *   - like the other entry points it synchronises the context stream before
 *     returning. */
#define RSCHOL_NOALLOC_MAX_N 2097152
int rschol_precond_apply_device_noalloc(rschol_factor* f, const double* d_b, double* d_x, int nrhs);

/* Autotuner of the batched apply (no reference counterpart): times the
 * candidate tile shapes (interior (row, column) pair tiles, column groups of
 * the compressed-level products) of every width class (number of
 * right-hand sides rounded up to a power of two) up to max_columns and keeps
 * the fastest for this factor; run it while the GPU is otherwise quiet.  No
 * candidate changes any result: every shape forms each column's sums in the
 * same order.  Untuned classes use fixed shapes.  The choices are listed in
 * rschol_factor_describe ("batch_tuning": class, RA, RC, cwR, cwC, ms). */
int rschol_factor_autotune(rschol_factor* f, int max_columns);

/* Autotuner of the factor's schedule (no reference counterpart): times
 * `repeats` numeric factorisations of the factor's current values under each
 * candidate -- FP32 GEMM steps on the tensor cores (128 x 64 or 128 x 128
 * tiles) from K >= 32, 64, 96, 128 or 256, or none (64 x 64 SIMT tiles);
 * the blocked Cholesky
 * and TRSM chains of a level as one fused launch of 64 x 64 tile items or as
 * one launch per 64-column panel -- keeps the fastest and leaves the factor
 * refactored with it.  The candidates differ only in rounding.  Run it while
 * the GPU is otherwise quiet, before creating sessions on the factor.  The
 * choice is listed in rschol_factor_describe ("schedule": tc_min_k (-1: none),
 * fused, tuned_ms). */
int rschol_factor_tune_schedule(rschol_factor* f, int repeats);

/* ---- continuous batching on one factor (no reference counterpart) --------
 * A session keeps the Krylov state of up to max_columns right-hand sides of
 * one factor on the device (clamped to the factor's batch capacity, at most
 * 64; rschol_session_columns gives the value used).  rschol_session_add
 * queues a request of nrhs right-hand sides (b, x: host, stacked column after
 * column, in the original order; both must stay valid until the request is
 * done); its columns join the block at the next step as room allows.  Every
 * rschol_session_step advances each active column by one iteration of
 * PCG_SOLVER::solvePCG (src/rschol/linearalgebra/PCG_SOLVER.cpp:226-363,
 * the recurrences of rschol_pcg), retires the columns that meet their
 * stopping test (x written) and lists in done_tags (room for
 * rschol_session_columns entries) the requests whose every column is done;
 * rschol_session_result then gives their rschol_pcg_info and forgets them.
 * A column's iterates do not depend on the other columns in the block.
 * One thread at a time drives a session and its factor; the factor must
 * outlive the session. */
typedef struct rschol_session rschol_session;
rschol_session* rschol_session_create(rschol_factor* f, int max_columns);
int rschol_session_columns(const rschol_session* s);
int rschol_session_add(rschol_session* s, long long tag, int nrhs, const double* b, double* x, double eps, int maxit);
int rschol_session_step(rschol_session* s, long long* done_tags, int* ndone);
int rschol_session_result(rschol_session* s, long long tag, rschol_pcg_info* info);
int rschol_session_counts(const rschol_session* s, int* active, int* queued);
void rschol_session_destroy(rschol_session* s);

/* ---- serving loop (no reference counterpart: the reference's pcg_solver
 * driver solves one system per process) --------------------------------------
 * Continuous batching over many systems: requests (matrix id, CSC matrix as
 * for rschol_factor_create, 1..64 right-hand sides stacked column after
 * column) join the PCG session of their matrix's cached factor at the next
 * iteration boundary; `workers` threads step the sessions of different
 * matrices concurrently, each on its factor's own stream.  Factors are
 * cached on the device by matrix id within hbm_budget_bytes of live device
 * bytes (idle factors are evicted least recently used first; a factor that
 * does not fit next to busy ones waits, one larger than the budget fails its
 * requests with RSCHOL_E_OOM).  A request's result is the same alone and in
 * a mix.  submit copies its arguments and returns a request id (> 0) or
 * -status (only the request that builds a factor reads colptr/rowind/vals/
 * xyz); wait blocks until the request is done and returns its status, x
 * (stacked), info per right-hand side and times[5] = queued s (including
 * the factorisation it waited for), factorisation s (0 on a cache hit), PCG
 * s, latency s, cache hit (0/1).  stats[8] = completed, cache hits, misses,
 * evictions, cached bytes, peak cached bytes, cached factors, waiting
 * requests.  destroy finishes every submitted request first. */
typedef struct rschol_server rschol_server;
rschol_server* rschol_server_create(const rschol_params* p, int workers, double hbm_budget_bytes);
int rschol_server_submit(rschol_server* s, int matrix_id, int n, const int* colptr, const int* rowind,
                         const double* vals, const double* xyz, int nrhs, const double* b, double eps, int maxit);
int rschol_server_wait(rschol_server* s, int request_id, double* x, rschol_pcg_info* info, double* times);
int rschol_server_stats(rschol_server* s, double* stats);
void rschol_server_destroy(rschol_server* s);

/* Diagnostics (no reference counterpart): CUDA-event timing of every step of
 * the numeric factorisation while enabled.  out (may be null, else 24
 * doubles) receives, for step kinds 0..7 (GEMM, POTRF, TRSM, extend-add, QR,
 * identity basis, -, fused blocked Cholesky / TRSM), 3 values each: device
 * milliseconds, launches and algorithmic flops (GEMM and fused steps)
 * accumulated since timing was last switched on; enable = 1 also resets them
 * when timing was off. */
int rschol_step_timing(rschol_factor* f, int enable, double* out);

/* Diagnostics (no reference counterpart): one tensor-core GEMM
 * C = -1.25 op(A) op(B) + 0.5 C on random M x N x K operands (tA / tB:
 * transposed storage, split: 0 plain TF32, 1 split TF32, 2 split BF16 (the
 * schur_bf16 products); lower: lower-triangle tiles only) against a host
 * FP64 product.  out[0]: largest error relative to
 * sum_k |a_ik b_kj| (+ |beta c_ij|), out[1]: largest absolute error, out[2]:
 * 1 when the operands were staged by TMA (A M x K and B N x K row-major,
 * aligned, TF32), 0 when through registers.  out holds 3 values. */
int rschol_selftest_gemm(int M, int N, int K, int tA, int tB, int split, int lower, double* out);

/* Diagnostics (no reference counterpart): *ms = average device time of one
 * tensor-core launch C (M x N) -= A (M x K) B^T (A, B row-major, the
 * factor's update shape; split as in rschol_selftest_gemm; no K slices;
 * TF32 operands staged by TMA when K is a multiple of 4), over reps launches
 * after one warm-up, on zero operands. */
int rschol_bench_gemm(int M, int N, int K, int split, int reps, double* ms);

/* Preconditioned CG from x0 = 0 with the factor as M, stopping at
 * ||r|| / ||b|| <= eps or maxit iterations; nrhs right-hand sides are solved
 * together, sharing the factor.
 * Replaces PCG_SOLVER(A, eps, iters) + solvePCG(x, b, M)
 * (src/rschol/linearalgebra/PCG_SOLVER.h:52-65, PCG_SOLVER.cpp:226-363).
 * info may be NULL; otherwise it receives nrhs entries. */
int rschol_pcg(rschol_factor* f, const double* b, double* x, int nrhs, double eps, int maxit,
               rschol_pcg_info* info);
int rschol_pcg_device(rschol_factor* f, const double* d_b, double* d_x, int nrhs, double eps, int maxit,
                      rschol_pcg_info* info);

/* Drop-in for the reference's Python entry point
 * void pcg_pysolve(int nrow, const int* jc, const int* ir, const double* pr,
 *                  const double* rhs, double* solution)
 * (src/python/pcg_pysolver.h:35-36, .cpp:83-101): maxDenseBlock 200,
 * maxDiagonalBlock 400, eps 1e-6, 10000 iterations, zero positions. */
void rschol_pcg_pysolve(int nrow, const int* jc, const int* ir, const double* pr, const double* rhs,
                        double* solution);

/* ---- introspection (parity tests, benchmarks) ---------------------------- */
int rschol_factor_n(const rschol_factor* f);
/* live device bytes of the factor: factor arrays, solve and PCG work vectors
 * (the work vectors grow with the number of right-hand sides per call) */
double rschol_factor_device_bytes(const rschol_factor* f);
int rschol_factor_num_nodes(const rschol_factor* f);
/* info[0..7] = c0, c1, compressed, m (all rows), n_stored, rank, hodlr nodes, interior block */
int rschol_factor_node_info(const rschol_factor* f, int node, int* info);
/* dense expanded L11 (n x n row-major, lower) of a supernode */
int rschol_factor_node_l11(rschol_factor* f, int node, double* out);
/* interior node: stored rows (n_stored x n); compressed: V U^T (m x n) */
int rschol_factor_node_l21(rschol_factor* f, int node, double* out);
int rschol_factor_perm(const rschol_factor* f, int* perm);
/* JSON summary of the symbolic structure and the last factorisation */
const char* rschol_factor_describe(rschol_factor* f);
/* stats[0..7]: symbolic s, numeric s, attempts, diag rank constant,
 * kernel launches of the last factorisation, device bytes, gaussian draws, flops */
int rschol_factor_stats(const rschol_factor* f, double* stats);

/* ---- synthetic problems --------------------------------------------------- */
void* rschol_problem_diffusion(int dim, int nx, int ny, int nz, double sigma, unsigned seed, int nrhs);
void* rschol_problem_elasticity(int ne, double E, double nu, unsigned seed, int nrhs);
int rschol_problem_n(const void* p);
long long rschol_problem_nnz(const void* p);
int rschol_problem_nrhs(const void* p);
void rschol_problem_get(const void* p, int* colptr, int* rowind, double* vals, double* xyz, double* rhs);
void rschol_problem_free(void* p);
void rschol_mt_draws(unsigned seed, long long count, unsigned* out);
void rschol_mt_gaussians(unsigned seed, long long count, double* out);

/* ---- symbolic known-answer helpers ------------------------------------------
 * FactorManager::blockRank / diagonalBlockRank (FactorManager.cpp:7283-7338) */
int rschol_block_rank(int nRows, int nCols, double c, int oversampling, int cap);
/* SeparatorTree order / leafRanges (src/rschol/datastructure/SeparatorTree.cpp);
 * returns the number of leaves; leafFirst has nLeaves + 1 entries */
int rschol_separator_tree(int npts, const double* xyz, int maxLeaf, int* order, int* leafFirst);
/* cs_etree + cs_counts on an upper pattern with the identity postorder
 * (NestedDissection.cpp:409-429) */
void rschol_etree_counts(int n, const int* colptr, const int* rowind, int* parent, int* counts);
/* BuildRelaxedSupernodes (NestedDissection.cpp:1266-1735); returns nsuper,
 * superFirst has nsuper + 1 entries */
int rschol_relaxed_supernodes(int n, const int* parent, const int* counts, int ncomp, const int* compSize,
                              const int* compChildren, const int* compFirst, const int* compParent, int maxBlock,
                              int* superFirst, int* compressed);

#ifdef __cplusplus
}
#endif
#endif /* RSCHOL_GPU_H */
