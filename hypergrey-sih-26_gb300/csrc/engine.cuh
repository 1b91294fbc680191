// Device-side data layout of the box-QP engine (shared by the kernels and the host engine).
//
// One resident solve ("instance") owns a device slab holding its CSR and vectors; a
// batch is an array of instance records plus a table of row tiles.  Every kernel is a
// grid-stride loop over the tile table, reads the tile's instance record, and skips
// instances that are not in the phase the kernel serves, so one captured graph serves
// any mix of instances that are admitted, iterating, polishing or retired.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace bqp {

constexpr int kBlock = 256;          // threads per CTA of every tile kernel
constexpr int kMaxInterval = 32;     // maximum check interval (iterations per chunk)
constexpr int kTileNnz = 4096;       // target nonzeros per tile
constexpr int kTileRows = 512;       // maximum rows per tile
constexpr int kCgUnitMin = 4;        // tiles per work unit of the polish CG product kernel: about
constexpr int kCgUnitMax = 8;        //   this many at least, and up to this many for large instances (cg_units)
constexpr int kCgRowsum = kCgUnitMin * kTileRows;  // rows per CG work unit at most (its row sums, 16 KB)
constexpr int kCgGroups = 2;         // row groups per warp whose loads the CG product keeps in flight
constexpr int kCgUnroll = 2;         // entries per row group and lane (and epilogue rows per thread) per pass of the CG product
constexpr int kRearmRows = 1024;     // rows per block when re-arming resident solves (8192: 32 us on 1M rows, latency-bound)
constexpr int64_t kHostPrimal = 131072;  // primals up to this size come back at completion, larger at fetch

enum Phase : int32_t {
    PH_FISTA = 0,        // FISTA iterations (FP64 or FP32 per precision)
    PH_POLISH_INIT = 1,  // FP64 free-set polish: snap the active set, start CG
    PH_POLISH_CG = 2,    // FP64 conjugate gradient on Q_FF
    PH_POLISH_FINISH = 3,  // CG done, xp clipped: the next check verifies the polished point
    PH_DONE = 4
};

enum Status : int32_t {
    ST_OPTIMAL = 0,
    ST_ITERATION_LIMIT = 1,
    ST_TIME_LIMIT = 2,
    ST_NUMERICAL_ERROR = 3,
    ST_RUNNING = 101
};

enum Precision : int32_t { PREC_FP64 = 0, PREC_MIXED = 1, PREC_FP64_EXACT = 2 };

// SpMV structure of a tile's step kernel (chosen per instance by the autotuning table).
enum Variant : int32_t {
    VAR_TILE = 0,    // block-staged: products of the whole tile, then one thread per row
    VAR_WARP = 64,   // warp-staged: 32 rows per warp, products then one lane per row
    // 1, 2, 4, 8, 16, 32: sub-warp rows, that many lanes per row
};

// Step-kernel groups: one kernel per (precision, variant) for the FP64 and mixed engines, each
// over its own list of tiles, so a kernel carries one SpMV structure and the registers of that
// structure alone (the FP64_EXACT engine has one structure and no groups).
constexpr int kVariants = 8;
constexpr int kStepGroups = 2 * kVariants;
__host__ __device__ constexpr int variant_index(int variant) {
    return variant == VAR_WARP ? 7 : variant == 32 ? 6 : variant == 16 ? 5 : variant == 8 ? 4 : variant == 4 ? 3
         : variant == 2 ? 2 : variant == 1 ? 1 : 0;
}
__host__ __device__ constexpr int step_group(int precision, int variant) {
    return precision == PREC_FP64_EXACT ? -1 : (precision == PREC_MIXED ? kVariants : 0) + variant_index(variant);
}

struct Tile {
    int32_t inst;
    int32_t row_begin;
    int32_t row_end;
    int32_t variant;  // Variant, or lanes per row (1..32)
};

// Per-tile partial results of one check (or of one CG reduction).  Sums are plain FP64 reduced in
// a fixed tree; maxima of non-negative doubles travel as their IEEE bit patterns, whose unsigned
// integer order is the numeric order, so they reduce on the integer pipes.
struct __align__(16) Partial {
    double obj;           // objective terms
    double bnd;           // tangent dual-bound terms
    double sep;           // separable dual-bound terms
    double a;             // CG: dot product
    uint64_t stat;        // max stationarity (bits)
    uint64_t prim;        // max scaled bound violation (bits, >= +0)
    uint64_t b;           // CG: max scaled residual (bits)
    uint64_t hash;        // active-set signature
    int64_t n_active;     // variables at a bound
    int32_t flags;        // bit0: non-finite x, bit1: infinite bound target
    int32_t pad;
};

// The convexity gate of an instance, computed on the device at admission from the uploaded full
// CSR (convexity_gate_kernel): the fast path of check_convex_hessian (src/qp_admm.cpp:30-39) and the
// Gershgorin bound of src/accelerated_qp.cpp:25-26.  Flags are 0/1, OR-reduced over the rows.
struct __align__(16) GateResult {
    unsigned long long lip_bits;  // max_i sum_k |Q_ik|, row sums in column order, as double bits
    int32_t indefinite;           // a row with Q_ii < 0, or Q_ii = 0 beside an off-diagonal entry
    int32_t nondominant;          // a row with Q_ii < sum_{j != i} |Q_ij| (diagonal dominance fails)
    unsigned long long floor_bits;  // during the pass: the largest lower bound of a row sum seen yet
    int32_t flags;                  // kGate* bits below
    int32_t pad;
};
constexpr int32_t kGateInvalid = 1;      // an entry whose column is out of range or whose value is not finite
constexpr int32_t kGateNonzero = 2;      // some value is not zero
constexpr int32_t kGateOffDiagonal = 4;  // some nonzero value lies off the diagonal
constexpr int32_t kGateNonPositive = 8;  // some row has Q_ii <= 0 (or no diagonal entry)

struct __align__(16) InstDev {
    // problem
    const int32_t* rowptr;
    const int32_t* col;
    const double* val64;   // FP64 values (PREC_FP64, PREC_FP64_EXACT)
    const float* vhi;      // FP32 high part (PREC_MIXED)
    const float* vlo;      // FP32 low part, val ~= hi + lo (PREC_MIXED)
    const double* c;
    const double* l;
    const double* u;
    const float* c32;
    const float* l32;      // smallest float >= l
    const float* u32;      // largest float <= u
    const double* diag;    // FP64 diagonal of Q
    const double* dinv;    // 1 / diagonal (mixed: Jacobi preconditioner of the polish)
    // iterates
    union {
        double* x64;       // FP64 engines: the iterate
        double* xf;        // mixed engine: the polish's x on the free-list positions (below)
    };
    double* w64[2];
    float* x32;
    float* w32[2];
    double* xp;            // polished point (FP64)
    float2* xp2;           // xp as an FP32 pair (hi, lo) for FP32-only gathers
    // The polish's CG vectors live on free-list positions: free row j of a tile is position
    // row_begin + j (each tile's free rows packed at the front of its row range), so the CG
    // kernels stream them without the row indices, and Q_FF's packed columns are positions.
    float2* p2;            // CG: u as an FP32 pair (gathered by the product)
    double* r;
    double* p;
    double* q;             // CG: w = Q_FF u
    double* s;             // polish: s = Q p (Chronopoulos-Gear CG)
    double* z;             // CG: u = M^-1 r
    int4* xq;              // polish: per row the snapped point's FP32 pair (x, y as bits) and the row's
                           // free-list position (z; -1 held at a bound): one 16-byte gather per entry
                           // of the residual pass's products
    int32_t* pos_of;       // polish: the free-list positions alone (-1 held at a bound), for its count
    int32_t* free_rows;    // polish: free rows of each tile, listed from the tile's first row
    int32_t* free_cnt;     // polish: free rows per tile (index within the instance's tiles)
    int32_t* col_ff;       // polish: the free-column entries of a tile's free rows, packed row
    float* hi_ff;          //   after row (list order) from the start of the tile's own extent
    float* lo_ff;          //   [rowptr[row_begin], ...): row r at [start_ff[r], + cnt_ff[r])
    int32_t* cnt_ff;
    int32_t* start_ff;
    double* pc_inv;        // polish preconditioner, per free-list position: 1 / pivot of the chain factorization (1 / Q_rr on a Jacobi row)
    double* pc_e;          //   and the kept coupling to the next position (0 ends a chain)
    int32_t* pc_tile;      //   per tile (index within the instance): 1 when the tile has a chain
    unsigned long long stat_floor;  // within a running check: the largest stationarity ratio (FP64
                                    // bits) published so far; rows that cannot exceed it skip the division
    // geometry (the instance's tile range lives in View::ranges)
    int32_t n;
    int32_t diag_gate;
    // control
    int32_t status;
    int32_t phase;
    int32_t interval;
    int32_t polish_rounds;
    int32_t precision;
    int32_t polish;        // mixed: free-set polish enabled
    int32_t arm_chunk;     // 1: admission arms the first chunk without a check of x0 (mixed)
    int32_t lip_device;    // 1: L is the device power estimate in *lprec (BQP_LIPSCHITZ_POWER)
    int32_t moved[2];      // mixed: a variable entered or left a bound in the chunk's last two steps
    float* sstep;          // mixed, preconditioned: per-row step 1 / (L' Q_ii) (null: scalar 1/L)
    double* lprec;         // L' of the preconditioned mixed engine, or the power estimate of L (device-computed at admission)
    GateResult* gate;      // the admission's convexity gate and Gershgorin bound (convexity_gate_kernel)
    int32_t lanes_res;     // polish: lanes per row of the residual pass (full rows)
    int32_t lanes_cg;      // polish: lanes per row of the CG products (free-free rows) and of the mixed checks
    int64_t it0;          // first iteration of the current chunk (beta[k] is iteration it0 + k)
    int64_t it_cur;        // iteration of the body's first step launch; a chunk may span bodies
    int64_t it_next;       // iteration of the next check
    int64_t max_iter;
    int64_t deadline_ns;   // %globaltimer deadline
    int64_t start_ns;
    int64_t end_ns;
    double L;
    double invL;
    float invLf;
    int32_t result_src;    // where the answer lives: 0 x64, 1 x32, 2 xp
    double tol;
    double offset;
    double t;              // FISTA t_k
    double beta[kMaxInterval];
    float beta32[kMaxInterval];  // the same rounded to FP32, for the mixed steps (no per-tile conversion)
    // last check
    double objective;
    double primal_res;
    double stationarity;
    double dual_bound;
    double rel_gap;
    int32_t verified;
    int32_t stable_checks;
    int64_t iterations;
    uint64_t active_hash;
    int64_t n_active;
    double best_stat;
    // polish (CG on the free set)
    double rz;
    double alpha;
    double beta_cg;
    double cg_res;
    double cg_tol;
    double polish_switch;  // stationarity that triggers the first polish attempt
    double step_switch;    // the same after a step-stable chunk (see after_check)
    int64_t cg_it;
    int64_t cg_total;
    int64_t cg_max;
    // accounting
    int64_t fista_iters;
    int64_t checks;
    int64_t ff_nnz;        // polish: entries of the packed Q_FF of the current polish round
    int64_t ff_rows;       // polish: free rows of the current polish round
    double polish_bytes;   // polish: algorithmic bytes of the residual passes and CG iterations
};
static_assert(sizeof(InstDev) % 16 == 0, "rearm_kernel copies records as 16-byte words");

struct Ctrl {
    int32_t n_inst;        // instance records in use
    int32_t n_tiles;       // tiles in use
    int32_t n_units;       // CG work units in use (View::units)
    int32_t bodies;        // loop bodies run in the current launch
    int32_t body_cap;      // stop the device loop after this many bodies
    int32_t running;       // instances still running (written by the control kernel)
    int32_t n_fista[3];    // instances in the FISTA phase, per precision
    int32_t n_polish;
    int32_t error;         // non-zero: a kernel detected an inconsistency
    int32_t n_cg;          // instances that may still run CG iterations in this body
    int32_t cg_iters;      // CG iterations run in this body
    long long kernels;     // engine kernels executed by this launch (counted by gate/control)
    int32_t group_begin[kStepGroups + 1];  // step groups: [begin, end) in View::group_tiles
    int32_t check_due[3];  // instances due for each check family in the next body (0: its kernel returns at once)
    int32_t step_due[3];   // per precision: step launches of this body with work (later ones return at once)
};

// Everything a tile kernel needs, passed by value.
struct View {
    InstDev* inst;
    const Tile* tiles;
    Partial* partial;
    int32_t* tile_done;    // per-instance count of finished tiles (check / CG reductions)
    Ctrl* ctrl;
    int32_t* status_mirror;  // per-instance status, rewritten by the control kernel every body
    const int2* ranges;      // per-instance tile range [x, y) in the tile table
    const int32_t* group_tiles;  // tile indices ordered by step group (Ctrl::group_begin)
    const int4* units;           // CG work units: x the first tile of a run of y consecutive tiles of one
                                 // instance, z the unit's index within the instance, w its unit count
};

}  // namespace bqp
