/*
 * updes_gb300.h — C ABI of the GB300 global RBF collocation solver.
 *
 * This is the drop-in boundary for the hot path of Updes' `pde_solver` /
 * `pde_solver_jit` with support_size="max" (updes/operators.py:559-683).
 * Every pointer named "device" is a CUDA device pointer owned by the caller;
 * matrices are row-major with an explicit leading dimension.  `stream` is a
 * cudaStream_t passed as void* so that this header needs no CUDA include.
 * No entry point aborts, traps or allocates device memory: device-side
 * failures are reported through an integer status (and, where stated, an
 * `info` word), and scratch memory is a caller-provided workspace whose size
 * the matching *_workspace query returns.
 *
 * Python callers bind these symbols with ctypes (updes_gb300/_lib.py).
 */
#ifndef UPDES_GB300_H
#define UPDES_GB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define UPDES_API __attribute__((visibility("default")))
#else
#define UPDES_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
enum {
  UPDES_OK = 0,
  UPDES_ERR_INVALID = 1,        /* bad argument (size, pointer, enum)            */
  UPDES_ERR_CUDA = 2,           /* a CUDA runtime call failed                    */
  UPDES_ERR_SINGULAR = 3,       /* LU met an exactly zero or non-finite pivot    */
  UPDES_ERR_NOT_CONVERGED = 4,  /* refinement stalled or hit its iteration cap   */
  UPDES_ERR_TIMEOUT = 5,        /* a bounded device-side wait gave up            */
  UPDES_ERR_UNSUPPORTED = 6,    /* valid request this build does not implement   */
  UPDES_ERR_WORKSPACE = 7,      /* workspace too small                           */
  UPDES_ERR_TOO_LARGE = 8       /* beyond the fixed scratch of updes_lu_solve_noalloc */
};

/* ---- radial basis functions (updes/utils.py:30-69) --------------------- */
enum {
  UPDES_RBF_POLYHARMONIC = 0,          /* r^(2a+1),            param = a   */
  UPDES_RBF_GAUSSIAN = 1,              /* exp(-(eps r)^2),     param = eps */
  UPDES_RBF_MULTIQUADRIC = 2,          /* sqrt(1+(eps r)^2),   param = eps */
  UPDES_RBF_INVERSE_MULTIQUADRIC = 3,  /* 1/sqrt(1+(eps r)^2), param = eps */
  UPDES_RBF_THIN_PLATE = 4             /* log(r) r^(2a),       param = a   */
};

/* ---- boundary row kinds (updes/assembly.py:141-362) -------------------- */
enum {
  UPDES_ROW_DIRICHLET = 0,       /* phi(x_i, x_j)                                  */
  UPDES_ROW_NEUMANN = 1,         /* grad phi(x_i, x_j) . n1                        */
  UPDES_ROW_ROBIN = 2,           /* beta phi + grad phi . n1                       */
  UPDES_ROW_PERIODIC_VALUE = 3,  /* phi(x_i, x_j) - phi(x_p, x_j), every column    */
  UPDES_ROW_PERIODIC_FLUX = 4    /* grad phi(x_i).n1 + grad phi(x_p).n2, every col */
};

/* ---- precisions of the factorisation ----------------------------------- */
enum {
  UPDES_PREC_FP64 = 0,   /* FP64 LU (the plain path)                               */
  UPDES_PREC_FP32 = 1    /* FP32 LU + FP64 GMRES iterative refinement               */
};

/*
 * One collocation problem on one cloud.  Row order is the reference's sorted
 * node order (internal, Dirichlet, Neumann, Robin, periodic;
 * updes/cloud.py:124-150), so row r < Ni is an interior operator row and row
 * Ni <= r < N is boundary row r - Ni.  n = N + M.
 */
typedef struct {
  int32_t N;                  /* nodes                                              */
  int32_t Ni;                 /* interior nodes (rows carrying the PDE operator)     */
  int32_t M;                  /* monomials: 1, 3, 6, 10 or 15 (max_degree 0..4)       */
  int32_t rbf;                /* UPDES_RBF_*                                          */
  double rbf_param;           /* a (polyharmonic, thin plate) or eps                  */
  int32_t self_term;          /* 0 = the reference's zero diagonal in Phi blocks      */
  int32_t support_width;      /* 0: every node's support is all other nodes ("max");
                                 S > 0: local supports, S = support_size - 1 nodes each */
  const double* nodes;        /* device, N x 2, (x, y) per node                       */
  const double* op_weights;   /* device, Ni x 5: value, d/dx, d/dy, d2/dx2, d2/dy2    */
  const int32_t* bd_kind;     /* device, N - Ni: UPDES_ROW_*                          */
  const int32_t* bd_node;     /* device, (N - Ni) x 2: evaluation node, partner node  */
  const double* bd_geom;      /* device, (N - Ni) x 8: n1x n1y n2x n2y nPx nPy beta 0 */
  const int32_t* supports;    /* device, N x support_width node ids (NULL when 0): the
                                 support of node i (updes/cloud.py:83-112).  A row of
                                 a Phi block keeps only its node's support columns (both
                                 nodes' on a periodic row; updes/assembly.py:20-32,
                                 125-128, 169-258); the P and P^T blocks stay dense.
                                 Not supported by the batched and double-float entry
                                 points (they return UPDES_ERR_UNSUPPORTED).          */
} updes_problem;

/* Library version (major*10000 + minor*100 + patch). */
UPDES_API int updes_version(void);

/* Human-readable text of a status code. */
UPDES_API const char* updes_status_string(int status);

/* Text of the last CUDA runtime failure seen by the library (thread-safe copy). */
UPDES_API const char* updes_last_error(void);

/* Padded leading dimension used for an n x n matrix of `elem_bytes` elements
 * (a multiple of 32 elements, so rows start on 128-byte boundaries). */
UPDES_API int64_t updes_matrix_ld(int64_t n, int32_t elem_bytes);

/*
 * Assemble the augmented Kansa matrix
 *     K = [[op(Phi), op(P)], [bd(Phi), bd(P)], [P^T, 0]]     (n x n)
 * in FP64 (K64) and/or FP32 (K32, the rounding of the FP64 entries); either
 * output may be NULL.  Entries are computed in FP64 with closed-form kernel
 * derivatives.  Columns n..ld-1 are written as zero.
 * Replaces assemble_op_Phi_P (updes/assembly.py:93-137), assemble_bd_Phi_P
 * (assembly.py:141-362) and the P^T block of assemble_A (assembly.py:62-85);
 * the reference multiplies [op; bd] by inv(A) instead (assembly.py:366-401).
 */
UPDES_API int updes_assemble(const updes_problem* p, double* K64, int64_t ld64, float* K32, int64_t ld32,
                   void* stream);

/*
 * The same K for a polyharmonic kernel (UPDES_ERR_UNSUPPORTED otherwise), evaluated in
 * double-float arithmetic on the FP32 pipes and written unscaled as two FP32
 * planes: Khi = FP32 rounding of the entry, Klo = FP32 rounding of the rest
 * (hi + lo within a few units of 2^-48 of the entry).  Columns n..ld-1 are
 * written as zero; ld a multiple of 4, planes 16-byte aligned.  rowmax (device,
 * n, may be NULL, must start at zero) receives each row's max |hi| as float
 * bits; range_flag (device, may be NULL) is set to 1 if an entry is not finite
 * or nonzero below 2^-100 in magnitude (then use updes_assemble).  scratch:
 * device, updes_assemble_df_scratch() bytes, 16-byte aligned.  The mixed-precision
 * solve assembles polyharmonic systems this way.  Same matrix as assemble_A's
 * blocks (updes/assembly.py:62-362), different arithmetic.
 */
UPDES_API int updes_assemble_df_scratch(const updes_problem* p, size_t* bytes);
UPDES_API int updes_assemble_df(const updes_problem* p, float* Khi, float* Klo, int64_t ld, uint32_t* rowmax,
                   int32_t* range_flag, void* scratch, size_t scratch_bytes, void* stream);

/*
 * vals = [Phi P] c at the nodes (Phi_ii = 0 unless self_term), FP64,
 * regenerating Phi on the fly.  coeffs: device, n; vals: device, N.
 * Replaces the `vals` of the reference, which come out of its QR solve
 * (updes/operators.py:612-613) and satisfy A c = [vals; 0] (assembly.py:404-410).
 */
UPDES_API int updes_eval_values(const updes_problem* p, const double* coeffs, double* vals, void* stream);

/*
 * Field value (what = 0, out: m), gradient (what = 1, out: m x 2) or Laplacian
 * (what = 2, out: m) at m arbitrary points from coefficients c (N + M) on the
 * N centers, summing over every center (phi(0) included, derivatives 0 there).
 * Replaces value / gradient / laplacian (updes/operators.py:118-184, 319-348).
 */
UPDES_API int updes_eval_field(int32_t m, const double* points, int32_t N, const double* centers, int32_t M,
                               int32_t rbf, double rbf_param, const double* coeffs, int32_t what, double* out,
                               void* stream);

/*
 * Workspace bytes for updes_lu_factor / updes_lu_solve on an n x n matrix.
 */
UPDES_API int updes_lu_workspace(int32_t n, int32_t precision, size_t* bytes);

/*
 * LU with partial pivoting, P A = L U (L unit lower), row-major.
 * A: device FP64 n x lda, the matrix; it is used as the working storage and
 * destroyed.  Factors go to F (device, n x ldf): with UPDES_PREC_FP64, F is
 * FP64 and may be A itself (in-place); with UPDES_PREC_FP32, F is FP32 and
 * receives L and U rounded to FP32 while every Schur-complement update is
 * accumulated in FP64 in A (FP32 factors of an FP64-accurate elimination).
 * piv: device, 2n ints: [0, n) the interchanges (row k swapped with piv[k] at
 * step k, LAPACK getrf convention, 0-based), [n, 2n) the resulting row
 * permutation (row i of P A is row piv[n + i] of A).
 * info: host; 0, or 1 + the first step whose pivot was exactly zero or
 * non-finite (the factorisation still runs to the end, like LAPACK).
 * Replaces the LAPACK getrf behind jnp.linalg.inv (updes/assembly.py:87-90)
 * and the lineax QR factorisation (updes/operators.py:612-613).
 */
UPDES_API int updes_lu_factor(int32_t n, double* A, int64_t lda, int32_t precision, void* F, int64_t ldf, int32_t* piv,
                    void* workspace, size_t workspace_bytes, int32_t* info, void* stream);

/*
 * Solve with the factors of updes_lu_factor: x = A^-1 b (trans = 0) or
 * x = A^-T b (trans = 1) for `nrhs` right-hand sides stored as the columns of
 * the row-major n x nrhs block b (leading dimension ldb), overwritten by x.
 * Arithmetic is FP64 for both factor precisions.  The transpose solve is the
 * adjoint's (the reference differentiates through lineax instead).
 */
UPDES_API int updes_lu_solve(int32_t n, const void* F, int64_t ldf, int32_t precision, const int32_t* piv, double* b,
                   int32_t nrhs, int64_t ldb, int32_t trans, void* workspace, size_t workspace_bytes,
                   void* stream);

/*
 * updes_lu_solve without any device allocation or caller workspace.
 *
 * No counterpart in the reference.  It exists for callers that are not
 * allowed to allocate device memory at the point where they solve: a handler
 * run by another framework's executor (an XLA custom call, for instance,
 * receives only the buffers the framework planned and must not allocate
 * behind its back), or a time-stepping loop that has to stay off the
 * allocator.  They pass the factors, pivots and right-hand sides as for
 * updes_lu_solve; the scratch (a status word, the triangular solves' block
 * flags and two n-vectors) is a fixed array inside the library, about 387 KB
 * on every GPU that loads it, kept until the process exits.
 *
 * Limit: n <= UPDES_NOALLOC_MAX_N; larger n returns UPDES_ERR_TOO_LARGE before
 * any GPU work.  The first call on each device looks up the array's device
 * address (cudaGetSymbolAddress) with that device current, so make that
 * first call before any stream capture (a failed lookup during capture
 * returns UPDES_ERR_CUDA, and updes_last_error says why).  Device ordinals
 * 64 and above return UPDES_ERR_UNSUPPORTED.  Every call on a device shares the
 * same array: calls that overlap on the GPU (different streams, or different
 * host threads) race, so order them, e.g. on one stream.  Each call clears
 * the parts that must start at zero itself.
 */
#define UPDES_NOALLOC_MAX_N 24576
UPDES_API int updes_lu_solve_noalloc(int32_t n, const void* F, int64_t ldf, int32_t precision, const int32_t* piv,
                                     double* b, int32_t nrhs, int64_t ldb, int32_t trans, void* stream);

/* r = b - K x (trans = 0) or r = b - K^T x (trans = 1) with FP64 K, x, b, r (device, n). */
UPDES_API int updes_residual(int32_t n, const double* K, int64_t ldk, const double* x, const double* b,
                   double* r, int32_t trans, void* stream);

/* ---- the full solve ------------------------------------------------------ */

typedef struct {
  int32_t precision;      /* UPDES_PREC_FP64 or UPDES_PREC_FP32                          */
  int32_t max_iters;      /* refinement cap (GMRES iterations in total)                  */
  int32_t restart;        /* GMRES restart length                                        */
  int32_t fallback_fp64;  /* 1: if refinement stalls, refactor in FP64 and solve again    */
  double tol;             /* stop when ||b - K c|| <= tol ||b||, or when the componentwise
                             backward error reaches 256 FP64 unit roundoffs (what the
                             double-float planes of K can certify)                          */
} updes_solve_opts;

typedef struct {
  int32_t iters;          /* GMRES iterations of the FP32-LU attempt (0 for the FP64 path)      */
  int32_t fell_back;      /* 1 if the FP64 fallback ran                                        */
  int32_t lu_info;        /* info of the last factorisation                                    */
  int32_t converged;      /* 1 if the stopping test was met                                    */
  double rel_residual;    /* final ||b - K c|| / ||b|| (equilibrated system)                   */
  double backward_error;  /* final max_i |b - K c|_i / (|K| |c| + |b|)_i (equilibrated system) */
  double t_assemble_ms, t_factor_ms, t_refine_ms, t_eval_ms;
} updes_solve_info;

/* Workspace bytes for updes_solve (matrices, factors and Krylov basis). */
UPDES_API int updes_solve_workspace(const updes_problem* p, const updes_solve_opts* opts, size_t* bytes);

/*
 * Assemble, factor and solve K c = [q; 0], then vals = [Phi P] c.
 * q: device, N (interior rhs then boundary values in sorted order);
 * coeffs: device, n; vals: device, N (may be NULL).
 * Replaces pde_solver's assemble_B → lineax QR → core_compute_coefficients
 * sequence (updes/operators.py:602-618).
 */
UPDES_API int updes_solve(const updes_problem* p, const double* q, double* coeffs, double* vals,
                const updes_solve_opts* opts, updes_solve_info* info, void* workspace,
                size_t workspace_bytes, void* stream);

/*
 * Factor once, solve many.  updes_factor assembles, equilibrates and factors K
 * into `workspace` (layout of updes_solve_workspace); updes_solve_factored then
 * solves nrhs right-hand sides (the columns of the row-major N x nrhs block Q,
 * leading dimension ldq) against those factors, writing coeffs (n x nrhs, ldc)
 * and vals (N x nrhs, ldv, may be NULL), each refined in FP64 like updes_solve
 * (an FP64 refactorisation replaces the factors if refinement stalls).
 * updes_solve is updes_factor followed by one updes_solve_factored column.
 * The reference rebuilds and refactors on every call (time stepping in
 * demos/Advection/00_advection_with_rbf.py:83-93, two solves per epoch in
 * demos/Laplace/03_laplace_with_adjoint.py:88-143).
 */
UPDES_API int updes_factor(const updes_problem* p, const updes_solve_opts* opts, updes_solve_info* info,
                           void* workspace, size_t workspace_bytes, void* stream);
UPDES_API int updes_solve_factored(const updes_problem* p, int32_t nrhs, const double* Q, int64_t ldq,
                                   double* coeffs, int64_t ldc, double* vals, int64_t ldv,
                                   const updes_solve_opts* opts, updes_solve_info* info, void* workspace,
                                   size_t workspace_bytes, void* stream);

/*
 * Batched right-hand sides with a fixed number of refinement sweeps.  R <= 64
 * columns of the row-major N x R block Q (ldq) are solved together against the
 * factors that updes_factor left in `workspace`: X = M^-1 Q, then `sweeps`
 * times X += M^-1 (Q - K X), with the residual and the triangular solves in
 * double-float arithmetic; coeffs (n x R, ldc) receives X.  FP64 factors
 * (precision UPDES_PREC_FP64) give M^-1 the accuracy of an FP64 solve, so one
 * sweep reaches FP64 quality; FP32 factors converge only as fast as classical
 * refinement on them allows.
 * updes_batch_prepare (once per factorisation; synchronises) derives the
 * batch's copy of the factors.  updes_solve_batch then only launches kernels on
 * `stream`: no synchronisation and no host reads, so a time step built from it
 * can be captured in a CUDA graph.  A stale or missing preparation, and any
 * timed-out wait, land in the workspace's status word, which
 * updes_workspace_status reads and clears.
 * batch_ws: scratch of updes_batch_workspace(n) bytes.
 * The reference solves each right-hand side with a full rebuild
 * (demos/Advection/00_advection_with_rbf.py:83-93).
 */
UPDES_API int updes_batch_workspace(int32_t n, size_t* bytes);
UPDES_API int updes_batch_prepare(const updes_problem* p, void* workspace, size_t workspace_bytes, void* batch_ws,
                                  size_t batch_ws_bytes, void* stream);
UPDES_API int updes_solve_batch(const updes_problem* p, int32_t R, const double* Q, int64_t ldq, double* coeffs,
                                int64_t ldc, int32_t sweeps, void* workspace, size_t workspace_bytes,
                                void* batch_ws, size_t batch_ws_bytes, void* stream);
UPDES_API int updes_workspace_status(const updes_problem* p, void* workspace, size_t workspace_bytes,
                                     int32_t* error, void* stream);

/* vals (N x R, ldv) = [Phi P] C for coefficient columns C (n x R, ldc), R <= 64: the batched
 * counterpart of updes_eval_values (kernel values regenerated once per pair, shared by the columns). */
UPDES_API int updes_eval_values_batch(const updes_problem* p, int32_t R, const double* C, int64_t ldc, double* vals,
                                      int64_t ldv, void* stream);

/*
 * Many independent systems in one call: problems[i] (its own cloud, kernel and
 * boundary rows) with rhs q[i] (N_i) gives coeffs[i] (n_i) and, when vals is
 * non-null and vals[i] non-null, vals[i] (N_i); infos (may be null) receives
 * each solve's report.  `streams` (1..64) host threads each drive one CUDA
 * stream with its own workspace slice and take the next unsolved system,
 * largest first; every solve is updes_solve.  The call returns when all are
 * done, with the first nonzero status it met (the others still ran).
 * workspace: updes_solve_many_workspace bytes (the largest system's solve
 * workspace per stream).  The reference runs one pde_solver call per system
 * (updes/operators.py:559-618).
 */
UPDES_API int updes_solve_many_workspace(const updes_problem* problems, int32_t count, const updes_solve_opts* opts,
                                         int32_t streams, size_t* bytes);
UPDES_API int updes_solve_many(const updes_problem* problems, int32_t count, const double* const* q,
                               double* const* coeffs, double* const* vals, const updes_solve_opts* opts,
                               updes_solve_info* infos, void* workspace, size_t workspace_bytes, int32_t streams);

/*
 * Many independent systems in ONE persistent launch.  `ctas` CTAs (0 = one
 * per SM) take systems from a device work queue, largest first, and each CTA
 * runs a system's whole solve by itself: assembly of K (FP64, equilibrated by
 * powers of two) and of the value rows [Phi P]; LU with partial pivoting in
 * panels of panel_width[i] columns (1..64, NULL = 16; chosen per system size
 * by the caller's autotuner) in double-float arithmetic on the FP32 pipes
 * (precision[i] = UPDES_PREC_FP32, about 48-bit factors) or in FP64
 * (UPDES_PREC_FP64) (precision NULL = all FP32); then classical refinement
 * sweeps with an FP64 residual, at most max_sweeps, while the componentwise
 * backward error still halves (down to 2 FP64 unit roundoffs; converged = at
 * most 32); coeffs[i]
 * (n_i) and vals[i] (N_i; vals or vals[i] may be NULL).  infos (may be NULL):
 * iters = refinement sweeps, lu_info, converged, backward_error.  Systems
 * must have N + M <= 4096 and no local supports (UPDES_ERR_UNSUPPORTED
 * otherwise).  No CTA waits for another.  The call synchronises `stream`; a
 * singular system gives UPDES_ERR_SINGULAR (the others are still solved).
 * workspace: updes_solve_batched_workspace bytes (per CTA, K, the working
 * matrix and the value rows of the largest system: about 24 n_max^2 bytes).
 * The reference runs one pde_solver call per system
 * (updes/operators.py:559-618).
 */
UPDES_API int updes_solve_batched_workspace(const updes_problem* problems, int32_t count, int32_t ctas,
                                            size_t* bytes);
UPDES_API int updes_solve_batched(const updes_problem* problems, int32_t count, const double* const* q,
                                  double* const* coeffs, double* const* vals, const int32_t* precision,
                                  const int32_t* panel_width, int32_t max_sweeps, int32_t ctas,
                                  updes_solve_info* infos, void* workspace, size_t workspace_bytes, void* stream);

/* ---- adjoint (reverse mode through the solve) ------------------------------
 * The reference differentiates pde_solver with jax.grad through inv, the GEMM
 * and the lineax QR (demos/Laplace/10_laplace_with_diff_phys.py:89-104) or runs
 * a second full solve for a hand-written adjoint
 * (demos/Laplace/03_laplace_with_adjoint.py:98-108).  Here the adjoint reuses
 * the forward factors:  with K c = [q; 0] and vals = [Phi P] c,
 *   g       = dJ/dc + [Phi P]^T dJ/dvals               (updes_eval_values_t)
 *   lambda  = K^-T g                                   (updes_solve_transpose)
 *   dJ/dq   = lambda[0:N]
 *   dJ/dW_i = -lambda_i (D c)_i per interior row        (updes_coeff_grad)
 * where W_i are the operator weights of row i and D the five primitives.
 */

/* out (n) = [Phi P]^T g for g (N): Phi g (Phi symmetric) then P^T g. */
UPDES_API int updes_eval_values_t(const updes_problem* p, const double* g, double* out, void* stream);

/*
 * lambda (n) = K^-T g (n) with the factors that the last updes_solve on this
 * workspace left there (FP64 GMRES refinement on K^T, same stopping test).
 * Returns UPDES_ERR_INVALID if the workspace holds no factorisation of an
 * n x n system.
 */
UPDES_API int updes_solve_transpose(const updes_problem* p, const double* g, double* lambda,
                                    const updes_solve_opts* opts, updes_solve_info* info, void* workspace,
                                    size_t workspace_bytes, void* stream);

/* dW (Ni x 5) = -lambda_i * sum_j D_k(x_i, x_j) c_j (monomial columns included), entries regenerated
 * on the fly (no matrix is stored). */
UPDES_API int updes_coeff_grad(const updes_problem* p, const double* coeffs, const double* lambda, double* dW,
                               void* stream);

/* ---- bounded waits ---------------------------------------------------------
 * Every spin-wait between CTAs (grid barriers, the panels' record exchange, the
 * triangular solves' block flags) gives up after a number of polls and then
 * reports UPDES_ERR_TIMEOUT instead of hanging; by default that is 2^26 polls
 * (seconds).  updes_set_spin_limit sets the number of polls on the current
 * device for every later launch of the library (0 restores the default); a
 * caller with a watchdog of its own may shorten it.  The tensor-core update's
 * waits on its own copies keep the default.  Not part of the reference, which
 * has no device-side waits (its errors are Python exceptions and
 * asserts, updes/assembly.py:474, updes/operators.py:729).
 */
UPDES_API int updes_set_spin_limit(int64_t iterations);

/* ---- instrumentation ------------------------------------------------------ */

/* Kernel classes of updes_stats: 0 trailing update, 1 panel, 2 TRSM, 3 triangular
 * solves, 4 FP64 GEMV/residual, 5 assembly, 6 other. */
#define UPDES_STAT_CATEGORIES 7

typedef struct {
  int64_t launches;                       /* kernels launched since the last reset        */
  int64_t count[UPDES_STAT_CATEGORIES];   /* timed launches per class                      */
  double ms[UPDES_STAT_CATEGORIES];       /* summed CUDA-event time per class              */
  double flops[UPDES_STAT_CATEGORIES];    /* algorithmic flops of the timed launches       */
  double bytes[UPDES_STAT_CATEGORIES];    /* algorithmic bytes of the timed launches       */
} updes_stats;

/* Zero the counters; enable_timing = 1 brackets every launch with CUDA events on
 * its stream (adds a little host overhead).  Not part of the reference. */
UPDES_API void updes_stats_reset(int32_t enable_timing);
UPDES_API void updes_stats_read(updes_stats* out);

#ifdef __cplusplus
}
#endif

#endif /* UPDES_GB300_H */
