/*
 * boxqp.h -- C-ABI of the GB300 box-constrained convex QP engine.
 *
 *   minimise 1/2 x'Qx + c'x  subject to  l <= x <= u,   Q sparse symmetric PSD.
 *
 * The engine keeps the reference's FISTA iteration (02-software/solver/src/accelerated_qp.cpp:13-61)
 * and its original-model verification (02-software/solver/src/qp_admm.cpp:63-117), and runs both
 * on the GPU: the fused CSR SpMV + gradient step + clamp + momentum kernel, the FP64 KKT /
 * objective block reductions, the FP32 iterations with FP64 checks and an FP64 free-set polish
 * (mixed precision), and many instances per launch (batching / continuous serving).
 *
 * Every entry point is plain C: pointers and sizes, no C++ types, no exceptions.  Functions
 * return BQP_OK (0) or a BQP_ERR_* code; the message of the last error on a context is
 * available from bqp_last_error().  Host arrays passed in are copied before the call returns
 * (the caller keeps ownership); output arrays are owned and sized by the caller.
 *
 * Threading: bqp_submit / bqp_poll / bqp_fetch / bqp_release / bqp_last_error are safe to call
 * from several host threads on one context (an internal lock guards them); the context's own
 * engine thread owns its CUDA stream and graphs.  One context drives one GPU.
 */
#ifndef BOXQP_H
#define BOXQP_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- return codes ---------------------------------------------------------------------- */
#define BQP_OK               0
#define BQP_ERR_INVALID      1  /* bad argument; the reference throws std::invalid_argument      */
#define BQP_ERR_CUDA         2  /* CUDA runtime error; the reference throws runtime_error("CUDA: ")*/
#define BQP_ERR_NO_DEVICE    3  /* "No CUDA device available" (src/cuda_box.cu:35)              */
#define BQP_ERR_ADMISSION    4  /* the context's device-memory cap would be exceeded             */
#define BQP_ERR_NOT_FOUND    5  /* unknown solve id                                              */
#define BQP_ERR_NOT_READY    6  /* the solve is still queued or running                          */
#define BQP_ERR_UNSUPPORTED  7  /* zero Hessian: the reference sends these to its CPU LP path    */
#define BQP_ERR_NO_MEMORY    8  /* host or device allocation failed                              */

/* ---- solve status, one-to-one with the reference's status strings (QpResult::status) --- */
#define BQP_STATUS_OPTIMAL                0  /* "optimal"                */
#define BQP_STATUS_ITERATION_LIMIT        1  /* "iteration_limit"        */
#define BQP_STATUS_TIME_LIMIT             2  /* "time_limit"             */
#define BQP_STATUS_NUMERICAL_ERROR        3  /* "numerical_error"        */
#define BQP_STATUS_UNSUPPORTED_CURVATURE  4  /* "unsupported_curvature"  */
#define BQP_STATUS_INFEASIBLE_BOUNDS      5  /* "infeasible_bounds"      */
#define BQP_STATUS_QUEUED               100  /* submitted, waiting for admission              */
#define BQP_STATUS_RUNNING              101  /* resident on the device, iterating             */

/* ---- precision of the iterations ------------------------------------------------------- */
#define BQP_PRECISION_FP64        0  /* plain engine: FP64 values and iterates (reference numerics)   */
#define BQP_PRECISION_MIXED       1  /* FP32 values/iterates, FP64 checks + FP64 free-set polish      */
#define BQP_PRECISION_FP64_EXACT  2  /* FP64, one thread per row, no FMA contraction, division by L:
                                        reproduces the CPU oracle's iterates bit for bit              */

/* ---- step size ------------------------------------------------------------------------- */
#define BQP_LIPSCHITZ_GERSHGORIN  0  /* L = max_i sum_k |Q_ik|, as src/accelerated_qp.cpp:25-26      */
#define BQP_LIPSCHITZ_POWER       1  /* FP64 estimate of lambda_max on the device at admission: Lanczos
                                        on the power iteration's Krylov space (32 steps from a fixed
                                        start), L = min(Gershgorin, max(theta + residual, 1.001 theta)),
                                        theta the largest Ritz value.  An estimate, not a bound; of
                                        V Q V for the preconditioned mixed steps.  stats.lipschitz
                                        reports it.                                                    */

typedef struct bqp_ctx bqp_ctx;

/* Options of one solve.  Defaults mirror QpOptions (02-software/solver/include/qp.hpp:24-29). */
typedef struct bqp_options {
    double  tolerance;        /* KKT tolerance of the verification, default 1e-7                 */
    double  time_limit;       /* seconds from submission, default 30                             */
    int64_t iteration_limit;  /* FISTA iterations, default 200000                                */
    int32_t precision;        /* BQP_PRECISION_*, default BQP_PRECISION_FP64                      */
    int32_t lipschitz;        /* BQP_LIPSCHITZ_*, default BQP_LIPSCHITZ_GERSHGORIN                */
    int32_t check_interval;   /* iterations between checks, 1..32; default 0 = auto: 25 for the FP64
                                 engines (the reference's cadence, src/accelerated_qp.cpp:40);
                                 mixed: 10 when nnz >= 8 n, else 25                              */
    int32_t diagonal_gate;    /* -1 auto from the CSR; 0/1 force the reference's positive-diagonal
                                 dual-gap gate (src/qp_admm.cpp:72-78,106-116)                  */
    double  offset;           /* constant term of the objective (LinearProblem::offset)          */
    int32_t kernel_variant;   /* SpMV structure of the FISTA step: -1 auto (tuning default), 0 block-
                                 staged tile, 64 warp-staged rows, 1/2/4/8/16/32 lanes per row     */
    int32_t scaling;          /* mixed engine: 0 auto (= 1), 1 diagonally preconditioned FISTA steps
                                 (per-row step 1 / (L' Q_ii), L' the Gershgorin bound of
                                 D^-1/2 Q D^-1/2: FISTA in Jacobi-scaled variables, with iterates,
                                 checks and results in the original ones), 2 scalar step 1/L.
                                 The FP64 engines always take the reference's scalar step.      */
    double  polish_switch;    /* mixed: stationarity at or below which, with the active set
                                 unchanged since the previous check, the FP64 free-set polish is
                                 attempted (x0.1 after each failed attempt); default 0 = auto:
                                 0.1 with a check interval <= 10, else 3e-2                      */
} bqp_options;

/* Result of one solve (the numeric fields of QpResult plus engine accounting). */
typedef struct bqp_stats {
    int32_t status;                 /* BQP_STATUS_*                                              */
    int32_t verified;               /* optimality_verified by the device FP64 check              */
    int64_t iterations;             /* FISTA iterations at the final check (QpResult::iterations)*/
    int64_t polish_iterations;      /* CG iterations of the FP64 free-set polish (mixed)          */
    int64_t polish_rounds;          /* polish attempts (mixed)                                    */
    double  objective;              /* 1/2 x'Qx + c'x + offset, FP64 (double-double sum)          */
    double  primal_residual;        /* scaled bound violation (src/mps.cpp:279-303)               */
    double  stationarity_residual;  /* max_j |x_j - clip(x_j - g_j)| / (1 + |x_j|)                */
    double  complementarity_residual; /* 0 for box QPs                                            */
    double  dual_bound;             /* tangent (or separable) dual bound                          */
    double  relative_gap;           /* |objective - dual_bound| / (1 + |objective|)               */
    double  lipschitz;              /* step-size constant actually used                          */
    double  device_seconds;         /* device time from admission to completion                  */
    double  bytes;                  /* algorithmic HBM bytes of all iterations, checks, polish    */
    int64_t device_start_ns;        /* device clock (%globaltimer) at admission                  */
    int64_t device_end_ns;          /* device clock at completion                                */
    int64_t checks;                 /* device verifications run                                  */
} bqp_stats;

void bqp_options_default(bqp_options* options);

/* ---- context ----------------------------------------------------------------------------
 * bqp_create: one context on one device.  mem_cap_bytes bounds the device memory of resident
 * solves (0 = 90% of the free memory at creation).  Returns NULL on failure; the reason is
 * then available from bqp_last_error(NULL).                                                  */
bqp_ctx*    bqp_create(int device, size_t mem_cap_bytes);
void        bqp_destroy(bqp_ctx* ctx);
const char* bqp_last_error(const bqp_ctx* ctx);
/* Name of the CUDA device, as sovereign::cuda_device_name() (src/cuda_box.cu:38).            */
int         bqp_device_name(int device, char* out, size_t cap);
/* Page-locks a host range the caller submits from repeatedly (cudaHostRegister, portable):
 * uploads from it become asynchronous DMA with no staging copy on the host.  The range must
 * stay allocated until bqp_host_unregister(ptr).                                             */
int         bqp_host_register(void* ptr, size_t bytes);
int         bqp_host_unregister(void* ptr);

/* ---- asynchronous solves (continuous batching) -------------------------------------------
 * bqp_submit copies one problem (full symmetric CSR, int32 indices, columns ascending in each
 * row) and queues it.  The engine admits queued solves into the running batch as memory and
 * slots free up, iterates every resident solve in the same launches, and retires each one when
 * its own verification passes.  Returns BQP_ERR_ADMISSION only when the problem can never fit
 * under the context's memory cap.
 * Checks, in the reference's order (src/accelerated_qp.cpp:14-28): the call itself validates the
 * row pointers, costs and bounds (BQP_ERR_INVALID at once).  The Hessian's entries are checked by
 * the device's admission pass, which reads them anyway: a column out of range or a value that is
 * not finite ends the solve with BQP_ERR_INVALID ("Invalid Hessian"), a non-convex Hessian with
 * BQP_STATUS_UNSUPPORTED_CURVATURE, a zero Hessian with BQP_ERR_UNSUPPORTED, reported by bqp_wait
 * and bqp_fetch (nnz = 0 is refused at once).  A problem with infeasible bounds finishes at the
 * call, with its entries checked on the host.                                                */
int bqp_submit(bqp_ctx* ctx, int64_t n, int64_t nnz, const int32_t* rowptr, const int32_t* col,
               const double* val, const double* c, const double* lower, const double* upper,
               const bqp_options* options, uint64_t* id);
/* bqp_submit without the host copy: the engine uploads straight from the caller's arrays, which
 * must stay valid and unchanged until the solve has finished (bqp_wait / bqp_poll / bqp_wait_any
 * report it) or until bqp_release of the still-queued solve returns.  Validation, the convexity
 * gate and the errors are bqp_submit's.                                                      */
int bqp_submit_borrowed(bqp_ctx* ctx, int64_t n, int64_t nnz, const int32_t* rowptr, const int32_t* col,
                        const double* val, const double* c, const double* lower, const double* upper,
                        const bqp_options* options, uint64_t* id);
int bqp_poll(bqp_ctx* ctx, uint64_t id, int32_t* status);
/* Blocks until the solve is finished (timeout_seconds < 0: no timeout).                      */
int bqp_wait(bqp_ctx* ctx, uint64_t id, double timeout_seconds);
/* Blocks until some solve submitted with bqp_submit (or re-armed with bqp_resolve) finishes and
 * returns its id; each finished solve is reported once, in completion order.  BQP_ERR_NOT_READY
 * on timeout (timeout_seconds < 0: no timeout).                                              */
int bqp_wait_any(bqp_ctx* ctx, double timeout_seconds, uint64_t* id);
/* Copies the primal (n doubles, caller-owned) and the statistics of a finished solve.  The
 * primal comes straight from the solve's device memory; a bqp_release or bqp_resolve of the same
 * solve on another thread waits for the copy.                                                */
int bqp_fetch(bqp_ctx* ctx, uint64_t id, double* x, bqp_stats* stats);
/* Frees the solve's device memory; the id becomes unknown.                                   */
int bqp_release(bqp_ctx* ctx, uint64_t id);
/* Re-runs finished, still-resident solves from x0 = clip(0) without any upload; all `count`
 * solves are admitted into the same running batch.                                          */
int bqp_resolve(bqp_ctx* ctx, const uint64_t* ids, int64_t count);
/* Latency mode for serving: bound each device launch to about `ms` milliseconds so arriving
 * solves are admitted promptly (0 = throughput mode: one launch runs until the batch drains). */
int bqp_set_latency_target(bqp_ctx* ctx, double ms);
/* Number of queued and running solves, and the peak number resident at once so far.          */
int bqp_load(bqp_ctx* ctx, int64_t* queued, int64_t* running, int64_t* peak_resident,
             int64_t* resident_bytes);

/* Host-side fault injection for tests: the next `count` admissions on this context fail as if
 * the device allocation of their memory had failed (no device call is made for them).  Such a
 * solve finishes with BQP_ERR_NO_MEMORY from bqp_wait / bqp_fetch and its message in
 * bqp_last_error; the context keeps serving the solves after it.  A real allocation failure at
 * admission is reported the same way.  No counterpart in the reference (its CUDA plugin has no
 * admission).                                                                                */
int bqp_inject_admission_oom(bqp_ctx* ctx, int32_t count);

/* ---- measurement -------------------------------------------------------------------------
 * bqp_timer: device time of the engine stream's graph launches and re-arm kernels since the
 * last reset, measured with CUDA events on that stream; `kernels` counts the engine kernels
 * those launches executed (counted on the device), `graph_launches` the graph launches.
 * bqp_profile_step: times `launches` back-to-back launches of the FISTA step kernel of one
 * finished resident solve (same kernel and grid as the graph) with CUDA events; returns the
 * mean time per launch and the algorithmic bytes of one iteration.  The engine must be idle;
 * the solve's iterate is scrambled afterwards (re-run it with bqp_resolve).                */
int bqp_timer(bqp_ctx* ctx, int32_t reset, double* device_ms, int64_t* kernels, int64_t* graph_launches);
int bqp_profile_step(bqp_ctx* ctx, uint64_t id, int32_t launches, double* ms_per_launch,
                     double* bytes_per_launch);
/* bqp_profile_cg: on a finished, still-resident mixed-precision solve that ended in its FP64
 * polish, re-runs the polish from the solve's FP32 iterate (untimed) and times `iterations` CG
 * iterations with CUDA events, the product kernel (w = Q_FF u with the fused reduction) and the
 * vector kernel separately; returns their mean times and algorithmic bytes per launch on the
 * packed Q_FF (product 12 nnz_FF + 48 n_F, vector 104 n_F).  Same conditions and side effect as
 * bqp_profile_step.                                                                         */
int bqp_profile_cg(bqp_ctx* ctx, uint64_t id, int32_t iterations, double* ms_matvec, double* ms_vector,
                   double* bytes_matvec, double* bytes_vector);

/* ---- synchronous single solve (the CLI path) --------------------------------------------- */
int bqp_solve_sync(bqp_ctx* ctx, int64_t n, int64_t nnz, const int32_t* rowptr, const int32_t* col,
                   const double* val, const double* c, const double* lower, const double* upper,
                   const bqp_options* options, double* x, bqp_stats* stats);

/* ---- constrained-QP ADMM inner solve -----------------------------------------------------
 * The linear system of the reference's ADMM x-update (02-software/solver/src/qp_admm.cpp:157-161)
 *     K x = rhs,  K = H + sigma I + A' diag(rho) A,
 * H (n x n, full symmetric CSR) and A (m x n, CSR) resident on the device.  bqp_admm_set_rho
 * stores rho (m entries, > 0) and sigma (>= 0) and forms the Jacobi preconditioner
 * diag(H) + sigma + sum_i rho_i a_ij^2 (qp_admm.cpp:153-156); bqp_admm_solve runs the reference's
 * preconditioned CG (qp_admm.cpp:262-273) from the caller's x until max|r| <= accuracy, after
 * max_inner iterations, or when d'K d is not positive and finite; x is overwritten, and the
 * iterations and the final max|r| are returned.  bqp_admm_apply: out = K v.  Host arrays of n
 * doubles; one call at a time per system.  NULL / BQP_ERR_* on failure (bqp_admm_last_error). */
typedef struct bqp_admm bqp_admm;
bqp_admm*   bqp_admm_create(int device, int64_t n, int64_t m, const int32_t* h_rowptr, const int32_t* h_col,
                            const double* h_val, const int32_t* a_rowptr, const int32_t* a_col,
                            const double* a_val);
int         bqp_admm_set_rho(bqp_admm* s, const double* rho, double sigma);
int         bqp_admm_apply(bqp_admm* s, const double* v, double* out);
int         bqp_admm_solve(bqp_admm* s, const double* rhs, double* x, double accuracy, int64_t max_inner,
                           int64_t* inner_out, double* residual_out);
/* Runs `iterations` iterations of the reference's ADMM loop (qp_admm.cpp:255-279) on the device
 * for the scaled problem the caller formed (qp_admm.cpp:136-161): A holds every constraint row,
 * bound rows included; c (n) is the scaled cost, lo/up (one per row of A) the constraint bounds;
 * x (n), z and y (one per row of A) are the state, read and written back.  Each iteration builds
 * rhs = A'(rho z - y) + sigma x - c, solves K next = rhs from x as bqp_admm_solve does, with the
 * accuracy min(1e-7, .05 / (it + 1)^1.6) (1 + max|rhs|) and at most min(4000, 2n + 20) inner
 * iterations (it = first_iteration + the step), then z, y and x = 1.6 next - .6 x.  The ADMM
 * checks, rho adaptation and polish stay with the caller.                                    */
int         bqp_admm_iterate(bqp_admm* s, const double* c, const double* lo, const double* up, double* x,
                             double* z, double* y, int64_t first_iteration, int64_t iterations,
                             int64_t* inner_total);
const char* bqp_admm_last_error(void);
void        bqp_admm_destroy(bqp_admm* s);

/* ---- plugin level: the reference's BoxIteration contract ----------------------------------
 * Mirrors sovereign::make_cuda_box / BoxIteration::step / BoxIteration::primal
 * (02-software/solver/include/accelerated_qp.hpp:9-16, src/cuda_box.cu:22-37): the problem is
 * resident on the device, each step is one FISTA iteration with the caller's momentum, and
 * primal() copies x back.  Uses FP64 and divides by L like the reference's CPU loop.         */
typedef struct bqp_box bqp_box;
bqp_box* bqp_box_create(int device, int64_t n, int64_t nnz, const int32_t* rowptr, const int32_t* col,
                        const double* val, const double* c, const double* lower, const double* upper,
                        double lipschitz);
int      bqp_box_step(bqp_box* box, double momentum);
int      bqp_box_primal(bqp_box* box, double* x);
void     bqp_box_destroy(bqp_box* box);
const char* bqp_box_last_error(const bqp_box* box);

/* ---- verification on device data ----------------------------------------------------------
 * The FP64 KKT / objective reduction of the engine as a standalone call on caller-owned
 * DEVICE pointers (full CSR, x, c, l, u), replacing check_qp_solution's host pass
 * (src/qp_admm.cpp:63-117) for a box QP.  Uses device scratch allocated per call.  It runs on a
 * stream of its own (non-blocking), which does not wait for work the caller queued on its own
 * streams: synchronize the stream that wrote the arrays before calling.  BQP_ERR_INVALID comes
 * with a message from bqp_box_last_error(NULL).                                             */
int bqp_check_device(int64_t n, const int32_t* d_rowptr, const int32_t* d_col, const double* d_val,
                     const double* d_x, const double* d_c, const double* d_lower, const double* d_upper,
                     double tolerance, double offset, int32_t diagonal_gate, bqp_stats* stats);

/* ---- convexity gate on device data ---------------------------------------------------------
 * The engine's admission pass as a standalone call on caller-owned DEVICE pointers (full
 * symmetric CSR, columns ascending per row), replacing the fast path of check_convex_hessian
 * (src/qp_admm.cpp:30-39) and the Gershgorin bound (src/accelerated_qp.cpp:25-26):
 * *lipschitz = max_i sum_k |Q_ik| summed in column order (bit for bit the reference's L);
 * *indefinite = 1 when some row has Q_ii < 0, or Q_ii = 0 beside off-diagonal entries (not
 * convex); *nondominant = 1 when some row has Q_ii < sum_{j != i} |Q_ij| (the FP64 column-order
 * sum), where check_convex_hessian goes on to its sparse LDL' (bqp_check_convex on the host).
 * Q_ii sums a row's diagonal entries; d_diag (n doubles on the device, or NULL) receives it.
 * Device scratch allocated per call, a non-blocking stream of its own: synchronize the stream
 * that wrote the arrays before calling.  BQP_ERR_INVALID comes with a message from
 * bqp_box_last_error(NULL).                                                                   */
int bqp_gate_device(int64_t n, const int32_t* d_rowptr, const int32_t* d_col, const double* d_val,
                    double* d_diag, double* lipschitz, int32_t* indefinite, int32_t* nondominant);

/* ---- verification without any device allocation -------------------------------------------
 * No counterpart in the reference.  Same computation and arguments as bqp_check_device, for
 * callers that cannot allocate device memory: a serving loop in which cudaMalloc/cudaFree would
 * synchronize the device and stall the solves in flight, or a process whose device memory is
 * already reserved by another allocator (a framework's caching pool), where cudaMalloc fails.
 * It allocates nothing: its scratch is a 96 KiB static device array in libboxqp.so, held by
 * every context that loads the library until the context ends, which limits n to 4,194,304 rows
 * (larger n returns BQP_ERR_INVALID with a message from bqp_box_last_error(NULL)).
 * The first call in a context (per device, and again after that context is destroyed and
 * recreated) sets up: it looks up the array's device address with cudaGetSymbolAddress and
 * loads the check kernel.  Under lazy module loading (the CUDA default) that set-up is when the
 * library's device code and the array take their device memory, so make the first call before
 * another allocator reserves the device's memory, and before any stream capture.
 * All calls share the one array and run on the legacy default stream: calls that overlap on the
 * GPU (from several host threads) race.  The legacy stream does not wait for non-blocking
 * streams (a framework's side streams): synchronize the stream that wrote the arrays before
 * calling.                                                                                   */
int bqp_check_device_noalloc(int64_t n, const int32_t* d_rowptr, const int32_t* d_col, const double* d_val,
                             const double* d_x, const double* d_c, const double* d_lower,
                             const double* d_upper, double tolerance, double offset,
                             int32_t diagonal_gate, bqp_stats* stats);

/* ---- host helpers ---------------------------------------------------------------------------
 * Full symmetric CSR from lower-triangle triplets, as CsrMatrix(n, rows) builds it after the
 * mirroring in src/accelerated_qp.cpp:20-24 (columns ascending, duplicates summed in input
 * order, exact zeros dropped), times sign.  Capacity: rowptr n+1, col/val 2*nh.  Returns nnz
 * through *nnz.                                                                              */
int bqp_csr_from_lower(int64_t n, int64_t nh, const int64_t* hrow, const int64_t* hcol,
                       const double* hval, double sign, int32_t* rowptr, int32_t* col, double* val,
                       int64_t* nnz);
/* check_convex_hessian (src/qp_admm.cpp:30-62): 1 convex, 0 not, BQP_ERR_INVALID-style -1. */
int bqp_check_convex(int64_t n, int64_t nh, const int64_t* hrow, const int64_t* hcol,
                     const double* hval, int32_t maximize);
/* Gershgorin bound max_i sum_k |Q_ik| of a full CSR.                                         */
double bqp_gershgorin(int64_t n, const int32_t* rowptr, const double* val);
/* sum_j a_j b_j accumulated in long double, in order (the reference's dot, src/qp_admm.cpp:23
 * and src/qp_dual_newton.cpp:35): the host side of the constrained-QP loop's CG steps.       */
double bqp_dot_ld(int64_t n, const double* a, const double* b);

/* ---- planted instance generator (synthetic workloads) ------------------------------------
 * Families: 0 random-graph weighted Laplacian + diagonal, 1 five-point grid Laplacian + shift,
 * 2 the reference's tridiagonal scale family (src/scale_benchmark.cpp:13-18).
 * The planted optimum x* and duals z make x* the unique solution: c = -Q x* + z.           */
typedef struct bqp_planted_spec {
    int32_t  family;
    int32_t  edges_per_vertex; /* family 0                                               */
    int64_t  n;                /* family 0 and 2; family 1 uses grid_side^2                 */
    int32_t  grid_side;        /* family 1                                               */
    int32_t  bounds_mode;      /* 0: scalar [lower, upper]; 1: l ~ U[-1,-.5], u ~ U[.5,1]    */
    uint64_t seed;
    double   lower, upper;     /* scalar bounds (bounds_mode 0)                          */
    double   frac_lower, frac_upper;     /* planted pattern: share at lower / upper bound */
    double   interior_lo, interior_hi;   /* interior x* = l + (u-l) * U(lo, hi)          */
    double   diag_lo, diag_hi;           /* family 0: D ~ U[diag_lo, diag_hi]            */
    double   weight_lo, weight_hi;       /* family 0: edge weights U[weight_lo, weight_hi] */
    double   shift;                      /* family 1: + shift * I                        */
    double   dual_lo, dual_hi;           /* |z| ~ U[dual_lo, dual_hi] at active bounds   */
} bqp_planted_spec;
typedef struct bqp_planted bqp_planted;

/* Presets of the synthetic workloads: 0 n=10k graph (5 edges/vertex, [0,1], 30/30/40);
 * 1 n=1M graph (7 edges/vertex, [-1,1], 25/25/50); 2 1024x1024 grid (+1e-3 I, random bounds,
 * 20/20/60); 3 instance `index` of the 4096-instance uneven batch; 4 request `index` of the
 * serving stream (n log-uniform in [1000, 200000]); 5 reference tridiagonal family.
 * `n_override` > 0 replaces n (families 0 and 2).                                            */
int bqp_planted_preset(int32_t preset, uint64_t seed, int64_t index, int64_t n_override,
                       bqp_planted_spec* spec);
bqp_planted* bqp_planted_create(const bqp_planted_spec* spec);
int  bqp_planted_info(const bqp_planted* p, int64_t* n, int64_t* nnz, int64_t* nnz_lower, double* fstar);
/* Any output pointer may be NULL.  Sizes: rowptr n+1, col/val nnz, vectors n.               */
int  bqp_planted_copy(const bqp_planted* p, int32_t* rowptr, int32_t* col, double* val, double* c,
                      double* lower, double* upper, double* xstar, double* z);
/* Lower-triangle triplets (row >= col), row-major: the reference's QuadraticProblem form.    */
int  bqp_planted_copy_lower(const bqp_planted* p, int64_t* hrow, int64_t* hcol, double* hval);
void bqp_planted_free(bqp_planted* p);

/* splitmix64 step used by every generator draw (exposed so hosts derive identical seeds).   */
uint64_t bqp_splitmix64(uint64_t* state);

#ifdef __cplusplus
}
#endif
#endif /* BOXQP_H */
