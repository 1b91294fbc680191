// Host side of the box-QP engine: resident solves, admission under a device-memory cap,
// the tile table, the captured conditional CUDA graph and the engine thread.
//
// The graph is one WHILE loop whose body is
//     check -> gate -> IF(fp64) K x (step per fp64 group) -> IF(mixed) K x (step per mixed group)
//           -> IF(exact) K x step -> IF(polish) [polish_init, polish_residual,
//              WHILE(an instance iterates, <= 25 per body) (cg_matvec, cg_vector)] -> control
// (K: the shortest check interval among the running solves; a group: one SpMV structure).
// The check kernel's per-instance finalizers decide each instance's next phase, the gate kernel
// arms the IF nodes for the phases present, and the control kernel ends the loop when no
// instance is running or after `body_cap` bodies (so the engine thread can admit new solves
// between launches).  All state the kernels read lives in device tables, so the graph is
// captured once and replayed for any mix of resident solves.
#include "boxqp.h"
#include "engine.cuh"
#include "kernels.cuh"
#include "workers.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <limits>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

namespace bqp {
namespace {

thread_local std::string g_thread_error;

double host_seconds() {
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

// BOXQP_PROFILE=1 also prints host-side times of each submission and admission to stderr.
bool host_profile() {
    static const bool on = [] {
        const char* m = std::getenv("BOXQP_PROFILE");
        return m && std::string(m) == "1";
    }();
    return on;
}


size_t align_up(size_t x, size_t a = 256) { return (x + a - 1) / a * a; }
constexpr int kCgPerBody = 25;  // CG iterations per polish body
constexpr size_t kNone = std::numeric_limits<size_t>::max();

struct Layout {
    size_t rowptr = kNone, col = kNone, val64 = kNone, vhi = kNone, vlo = kNone;
    size_t c = kNone, l = kNone, u = kNone, diag = kNone;
    size_t c32 = kNone, l32 = kNone, u32 = kNone, x32 = kNone, w32a = kNone, w32b = kNone;
    size_t x64 = kNone, w64a = kNone, w64b = kNone;
    size_t xp = kNone, r = kNone, p = kNone, q = kNone, z = kNone, xq = kNone, pos_of = kNone, xf = kNone;
    size_t xp2 = kNone, p2 = kNone, dinv = kNone, free_rows = kNone, free_cnt = kNone;
    size_t col_ff = kNone, hi_ff = kNone, lo_ff = kNone, cnt_ff = kNone, start_ff = kNone;
    size_t sstep = kNone, lprec = kNone, s = kNone, gate = kNone;
    size_t pc_inv = kNone, pc_e = kNone, pc_tile = kNone;
    size_t total = 0;
};

Layout make_layout(int64_t n, int64_t nnz, int64_t tiles, int precision) {
    Layout L;
    size_t o = 0;
    // 64 bytes of slack behind every array keep 16-byte vector loads of a tail in bounds.
    auto take = [&](size_t bytes) {
        size_t at = o;
        o = align_up(o + bytes + 64);
        return at;
    };
    const size_t N = static_cast<size_t>(n), Z = static_cast<size_t>(nnz);
    L.rowptr = take((N + 1) * 4);
    L.col = take(Z * 4);
    if (precision == PREC_MIXED) {
        L.vhi = take(Z * 4);
        L.vlo = take(Z * 4);
    } else {
        L.val64 = take(Z * 8);
    }
    L.c = take(N * 8);
    L.l = take(N * 8);
    L.u = take(N * 8);
    L.diag = take(N * 8);
    if (precision == PREC_MIXED) {
        L.c32 = take(N * 4);
        L.l32 = take(N * 4);
        L.u32 = take(N * 4);
        L.x32 = take(N * 4);
        L.w32a = take(N * 4);
        L.w32b = take(N * 4);
        L.xp = take(N * 8);
        L.r = take(N * 8);
        L.p = take(N * 8);
        L.q = take(N * 8);
        L.z = take(N * 8);
        L.xp2 = take(N * 8);
        L.p2 = take(N * 8);
        L.dinv = take(N * 8);
        L.xq = take(N * 16);
        L.pos_of = take(N * 4);
        L.xf = take(N * 8);
        L.free_rows = take(N * 4);
        L.free_cnt = take(static_cast<size_t>(tiles) * 4);
        L.col_ff = take(Z * 4);
        L.hi_ff = take(Z * 4);
        L.lo_ff = take(Z * 4);
        L.cnt_ff = take(N * 4);
        L.start_ff = take(N * 4);
        L.sstep = take(N * 4);
        L.s = take(N * 8);
        L.pc_inv = take(N * 8);
        L.pc_e = take(N * 8);
        L.pc_tile = take(static_cast<size_t>(tiles) * 4);
    } else {
        L.x64 = take(N * 8);
        L.w64a = take(N * 8);
        L.w64b = take(N * 8);
    }
    L.lprec = take(8);
    L.gate = take(sizeof(GateResult));
    L.total = o;
    return L;
}

template <class T>
T* at(void* base, size_t off) {
    return off == kNone ? nullptr : reinterpret_cast<T*>(static_cast<char*>(base) + off);
}

enum JobState { JOB_QUEUED = 0, JOB_ADMITTING = 1, JOB_RUNNING = 2, JOB_DONE = 3 };

// Host copies of submitted inputs (asynchronous submit) live in buffers kept for reuse: a fresh
// allocation of a few hundred MB costs more in first-touch page faults than the copy itself.
class HostBufferCache {
public:
    static HostBufferCache& get() {
        static HostBufferCache* cache = new HostBufferCache;  // never destroyed: usable at exit
        return *cache;
    }
    char* acquire(size_t bytes, size_t* got) {
        {
            std::lock_guard<std::mutex> g(mu_);
            size_t best = free_.size();
            for (size_t k = 0; k < free_.size(); ++k)
                if (free_[k].second >= bytes && free_[k].second <= 2 * bytes + (1 << 20) &&
                    (best == free_.size() || free_[k].second < free_[best].second))
                    best = k;
            if (best != free_.size()) {
                char* p = free_[best].first;
                *got = free_[best].second;
                cached_ -= *got;
                free_.erase(free_.begin() + static_cast<std::ptrdiff_t>(best));
                return p;
            }
        }
        *got = bytes;
        return static_cast<char*>(std::malloc(bytes ? bytes : 1));
    }
    void release(char* p, size_t bytes) {
        if (!p) return;
        std::lock_guard<std::mutex> g(mu_);
        if (cached_ + bytes > kLimit) {
            std::free(p);
            return;
        }
        free_.emplace_back(p, bytes);
        cached_ += bytes;
    }

private:
    static constexpr size_t kLimit = size_t(4) << 30;
    std::mutex mu_;
    std::vector<std::pair<char*, size_t>> free_;
    size_t cached_ = 0;
};

struct Job {
    uint64_t id = 0;
    int64_t n = 0, nnz = 0;
    bqp_options opt{};
    // owned copy in one cached host buffer (asynchronous submit) or borrowed pointers (synchronous solve)
    char* own = nullptr;
    size_t own_bytes = 0;
    const int32_t* rowptr = nullptr;
    const int32_t* col = nullptr;
    const double* val = nullptr;
    const double* c = nullptr;
    const double* l = nullptr;
    const double* u = nullptr;
    double lipschitz = 0;
    int diag_gate = 0;  // -1: decided by the admission gate (a diagonal Hessian with a positive diagonal)
    int variant = 0;
    std::vector<Tile> tiles;  // local tiles (inst field filled at admission)
    int state = JOB_QUEUED;
    bool resolve = false;     // re-run of a resident solve
    bool notify = false;      // report completion through the completion queue (bqp_wait_any)
    bool resident = false;
    int slot = -1;
    void* slab = nullptr;
    Layout layout;
    InstDev rec{};            // host image of the device record
    int error = BQP_OK;
    GateResult* gate_host = nullptr;  // page-locked copy of the admission's convexity gate result
    bool out_of_memory = false;  // the admission's device allocation failed (or was made to fail)
    std::string error_text;
    bqp_stats stats{};
    // upload in progress (engine thread): host -> device copies still to issue, then the
    // admission kernels; tmp holds the FP64 values of a mixed solve, power the Lanczos scratch
    struct Piece {
        void* dst;
        const void* src;
        size_t bytes;
    };
    std::vector<Piece> pieces;
    size_t piece = 0, piece_off = 0;
    void* tmp = nullptr;
    void* power = nullptr;
    double t_upload = 0;
    std::vector<double> x;    // primal of a solve that holds no device memory (finished at submission)
    const void* x_dev = nullptr;  // primal of a finished resident solve, in its slab
    bool x_f32 = false;           // ... as FP32 (the mixed engine's unpolished iterate)
    int fetching = 0;             // bqp_fetch calls copying x_dev (under the engine lock)
    double t_submit = 0, t_done = 0;
    ~Job() { HostBufferCache::get().release(own, own_bytes); }
};

void free_inputs(Job& j) {
    HostBufferCache::get().release(j.own, j.own_bytes);
    j.own = nullptr;
    j.own_bytes = 0;
    j.rowptr = nullptr; j.col = nullptr; j.val = nullptr; j.c = nullptr; j.l = nullptr; j.u = nullptr;
}

// check_convex_hessian (src/qp_admm.cpp:30-62) on the host, from a full CSR: diagonal dominance
// per row, else the sparse LDL^T of bqp_check_convex on the lower triangle.  Used where the
// device gate cannot decide (a solve finishing before admission, or a Hessian that is not
// diagonally dominant).
bool host_gate_convex(int64_t n, const int32_t* rowptr, const int32_t* col, const double* val) {
    bool dominant = true;
    for (int64_t i = 0; i < n; ++i) {
        double d = 0, radius = 0;
        for (int64_t k = rowptr[i]; k < rowptr[i + 1]; ++k) {
            if (col[k] == i) d += val[k];
            else radius += std::abs(val[k]);
        }
        if (d < 0 || (d == 0 && radius > 0)) return false;
        if (d < radius) dominant = false;
    }
    if (dominant) return true;
    std::vector<int64_t> tr, tc;
    std::vector<double> tv;
    for (int64_t i = 0; i < n; ++i)
        for (int64_t k = rowptr[i]; k < rowptr[i + 1]; ++k)
            if (col[k] <= i) {
                tr.push_back(i);
                tc.push_back(col[k]);
                tv.push_back(val[k]);
            }
    return bqp_check_convex(n, static_cast<int64_t>(tr.size()), tr.data(), tc.data(), tv.data(), 0) == 1;
}

// The result record of a solve refused as unsupported_curvature (the reference's QpResult defaults).
void set_unsupported(bqp_stats& st) {
    st.status = BQP_STATUS_UNSUPPORTED_CURVATURE;
    st.verified = 0;
    st.iterations = 0;
    st.objective = std::numeric_limits<double>::quiet_NaN();
    st.primal_residual = st.stationarity_residual = HUGE_VAL;
    st.complementarity_residual = st.relative_gap = HUGE_VAL;
    st.dual_bound = -HUGE_VAL;
}

// Default SpMV structure of the step kernel when the caller's options do not name one
// (kernel_variant < 0): rows longer than a warp use sub-warps, the rest the block-staged tile.
int default_variant(int64_t n, int64_t nnz, int precision) {
    if (precision == PREC_FP64_EXACT) return 1;
    const double avg = n > 0 ? static_cast<double>(nnz) / static_cast<double>(n) : 1.0;
    if (avg >= 48) return 32;
    return VAR_TILE;
}

// CG work units of one instance (its `count` tiles at t), appended to `out` as {first tile, tiles,
// index, units}: as many units as the product kernel has resident blocks (`slots`), so that one
// round runs them on the whole GPU, but units of about kCgUnitMin tiles at least; the tiles are
// spread evenly (sizes differ by one at most), and no unit goes above kCgRowsum rows (the row
// sums' shared buffer; units of kCgUnitMin tiles always fit).  Depends on the instance alone, so
// the product's partial sums, and the CG iterates, are the same in a batch as solo.
void cg_units(const Tile* t, int count, int first, int slots, std::vector<int4>& out) {
    const int fewest = (count + kCgUnitMax - 1) / kCgUnitMax;
    const int most = std::max(1, (count + kCgUnitMin - 1) / kCgUnitMin);
    int u = std::max(fewest, std::min(std::max(slots, 1), most));
    for (;; ++u) {
        bool fits = true;
        for (int k = 0, b = 0; k < u && fits; ++k) {
            const int e = b + count / u + (k < count % u ? 1 : 0);
            fits = t[e - 1].row_end - t[b].row_begin <= kCgRowsum;
            b = e;
        }
        if (fits || u >= count) break;
    }
    for (int k = 0, b = 0; k < u; ++k) {
        const int len = count / u + (k < count % u ? 1 : 0);
        out.push_back(make_int4(first + b, len, k, u));
        b += len;
    }
}

// Row tiles of one instance: contiguous rows with about kTileNnz nonzeros and at most
// kTileRows rows, the row count rounded down to a multiple of 256 (one 32-row group per warp of
// a block) or else of 32 where that many fit, so that the warps of a block finish a tile together.
// Depends on the instance alone, so its reductions are the same whether it runs alone or inside
// any batch.
std::vector<Tile> make_tiles(int64_t n, const int32_t* rowptr, int variant) {
    std::vector<Tile> t;
    int64_t r = 0;
    while (r < n) {
        // the first e in (r, min(n, r + kTileRows)) whose rows [r, e] pass kTileNnz nonzeros, else
        // that end: a binary search over the nondecreasing row pointers
        const int64_t hi = std::min<int64_t>(n, r + kTileRows);
        const int64_t limit = static_cast<int64_t>(rowptr[r]) + kTileNnz;
        const int32_t* p = std::upper_bound(rowptr + r + 2, rowptr + hi + 1, limit,
                                            [](int64_t v, int32_t x) { return v < static_cast<int64_t>(x); });
        int64_t e = (p - rowptr) - 1;
        if (e < n) {
            const int64_t rows = e - r;
            if (rows >= kBlock) e = r + rows / kBlock * kBlock;
            else if (rows >= 32) e = r + rows / 32 * 32;
        }
        t.push_back(Tile{0, static_cast<int32_t>(r), static_cast<int32_t>(e), variant});
        r = e;
    }
    return t;
}

// Algorithmic bytes, fixed accounting: per FISTA iteration nnz (s_v + 4) + 4 (n + 1) + 7 n s_x;
// per check nnz 12 + 4 (n + 1) + 32 n.  The polish's bytes are counted on the device on the
// packed Q_FF of each round (polish_bytes: residual pass and CG iterations, kernels.cu).
double algorithmic_bytes(int64_t n, int64_t nnz, int precision, int64_t iters, int64_t checks, double polish_bytes) {
    const double N = static_cast<double>(n), Z = static_cast<double>(nnz);
    const double sv = precision == PREC_MIXED ? 4.0 : 8.0;
    const double b_iter = Z * (sv + 4) + 4 * (N + 1) + 7 * N * sv;
    const double b_check = Z * 12 + 4 * (N + 1) + 32 * N;
    return static_cast<double>(iters) * b_iter + static_cast<double>(checks) * b_check + polish_bytes;
}

int status_code(int32_t st) {
    switch (st) {
    case ST_OPTIMAL: return BQP_STATUS_OPTIMAL;
    case ST_ITERATION_LIMIT: return BQP_STATUS_ITERATION_LIMIT;
    case ST_TIME_LIMIT: return BQP_STATUS_TIME_LIMIT;
    case ST_NUMERICAL_ERROR: return BQP_STATUS_NUMERICAL_ERROR;
    default: return BQP_STATUS_RUNNING;
    }
}

}  // namespace

class Engine {
public:
    Engine(int device, size_t cap) : device_(device), cap_(cap) {}
    ~Engine() { shutdown(); }

    bool init(std::string& why);
    void shutdown();

    int submit(Job* job, uint64_t* id);
    int poll(uint64_t id, int32_t* status);
    int wait(uint64_t id, double timeout);
    int fetch(uint64_t id, double* x, bqp_stats* stats);
    int release(uint64_t id);
    int resolve(const uint64_t* ids, int64_t count);
    int wait_any(double timeout, uint64_t* id);
    int load(int64_t* queued, int64_t* running, int64_t* peak, int64_t* resident_bytes);
    int timer(int reset, double* ms, int64_t* kernels, int64_t* launches) {
        std::lock_guard<std::mutex> g(mu_);
        if (ms) *ms = timer_ms_;
        if (kernels) *kernels = timer_kernels_;
        if (launches) *launches = timer_launches_;
        if (reset) {
            timer_ms_ = 0;
            timer_kernels_ = 0;
            timer_launches_ = 0;
        }
        return BQP_OK;
    }
    int profile_step(uint64_t id, int launches, double* ms, double* bytes);
    int profile_cg(uint64_t id, int iterations, double* ms_matvec, double* ms_vector, double* bytes_matvec,
                   double* bytes_vector);
    void set_latency_target(double ms) {
        std::lock_guard<std::mutex> g(mu_);
        latency_ms_ = ms;
    }
    void inject_admission_oom(int count) { inject_oom_.store(count); }
    // page-locked slots for the gate results of solves between upload and installation (engine
    // thread); chunks of kGateChunk slots, kept until the engine closes
    GateResult* acquire_gate_slot() {
        if (gate_free_.empty()) {
            GateResult* chunk = nullptr;
            if (cudaMallocHost(&chunk, sizeof(GateResult) * kGateChunk) != cudaSuccess) return nullptr;
            gate_chunks_.push_back(chunk);
            for (int k = 0; k < kGateChunk; ++k) gate_free_.push_back(chunk + k);
        }
        GateResult* g = gate_free_.back();
        gate_free_.pop_back();
        return g;
    }
    void release_gate_slot(Job& j) {
        if (j.gate_host) gate_free_.push_back(j.gate_host);
        j.gate_host = nullptr;
    }
    bool gate_uploaded(std::vector<Job*>& batch, std::vector<Job*>& refused, std::string& why);
    void finish_refused(Job* j);  // caller holds mu_
    void set_error(const std::string& e) {
        std::lock_guard<std::mutex> g(err_mu_);
        error_ = e;
    }
    const char* error() const {
        std::lock_guard<std::mutex> g(err_mu_);
        err_copy_ = error_;
        return err_copy_.c_str();
    }

private:
    void loop();
    bool upload(Job& j, std::string& why);
    bool upload_begin(Job& j, std::string& why);
    bool upload_copy(Job& j, size_t budget);
    bool upload_finish(Job& j, std::string& why);
    void fail_admission(Job* j, size_t reserved, const std::string& why);  // caller holds mu_
    void finish_paused_upload(std::unique_lock<std::mutex>& lk);
    static void CUDART_CB on_launch_done(void* self) {
        Engine* e = static_cast<Engine*>(self);
        {
            std::lock_guard<std::mutex> g(e->mu_);
            e->launch_done_ = true;
            e->t_launch_done_ = host_seconds();
        }
        e->cv_work_.notify_all();
    }
    // a new solve at the head of the queue that fits under the cap (caller holds mu_)
    bool uploadable_head() const {
        if (uploading_) return true;
        if (queue_.empty() || queue_.front()->resolve) return false;
        const Job* j = queue_.front();
        return resident_bytes_ + make_layout(j->n, j->nnz, static_cast<int64_t>(j->tiles.size()), j->opt.precision).total <= cap_;
    }
    bool install(std::vector<Job*>& jobs, std::string& why);
    void upload_waiting();
    bool rearm(const std::vector<Job*>& batch, std::string& why);
    void reset_record(Job& j);
    void update_steps();
    bool run_once(std::string& why);
    bool run_stream(int cap, std::string& why);
    void update_grid();
    void collect(std::unique_lock<std::mutex>& lk);
    void process_frees();
    void upload_tables();
    // step groups of precision `prec` that a body launches (bits of graph_groups_)
    std::vector<int> body_groups(int prec) const {
        std::vector<int> g;
        for (int k = 0; k < kStepGroups; ++k)
            if (((graph_groups_ >> k) & 1u) && (k >= kVariants) == (prec == PREC_MIXED)) g.push_back(k);
        return g;
    }
    void launch_body_steps(const View& v, int prec, int K, int grid, cudaStream_t s) const {
        if (prec == PREC_FP64_EXACT) {
            for (int j = 0; j < K; ++j) launch_step_exact(v, j, grid, s);
            return;
        }
        std::vector<int> groups = body_groups(prec);
        if (groups.empty()) groups.push_back(step_group(prec, VAR_TILE));  // no tiles: exits at once
        for (int j = 0; j < K; ++j)
            for (int g : groups) launch_step_group(v, g, j, grid, s);
    }
    StepLaunches body_launches(int K) const {
        StepLaunches L;
        L.n[PREC_FP64] = K * std::max<int>(1, static_cast<int>(body_groups(PREC_FP64).size()));
        L.n[PREC_MIXED] = K * std::max<int>(1, static_cast<int>(body_groups(PREC_MIXED).size()));
        L.n[PREC_FP64_EXACT] = K;
        return L;
    }
    bool ensure_tables(int need_inst, int need_tiles, std::string& why);
    bool build_graph(std::string& why);
    View view() const {
        View v;
        v.inst = d_inst_;
        v.tiles = d_tiles_;
        v.partial = d_partial_;
        v.tile_done = d_tile_done_;
        v.ctrl = d_ctrl_;
        v.status_mirror = d_status_;
        v.ranges = d_ranges_;
        v.group_tiles = d_group_tiles_;
        v.units = d_units_;
        return v;
    }
    bool cuda_ok(cudaError_t e, std::string& why, const char* what) {
        if (e == cudaSuccess) return true;
        why = std::string("CUDA: ") + what + ": " + cudaGetErrorString(e);
        return false;
    }

    int device_;
    size_t cap_;
    int sms_ = 152;
    int grid_max_ = 152 * 8;
    int cg_slots_ = 152 * 4;  // resident blocks of the CG product kernel
    cudaStream_t stream_ = nullptr;
    cudaStream_t capture_ = nullptr;
    cudaStream_t ustream_ = nullptr;   // uploads of new solves, overlapping the running graph
    cudaStream_t fstream_ = nullptr;   // bqp_fetch copies of finished primals (caller threads, fmu_)
    std::mutex fmu_;
    cudaEvent_t uev_ = nullptr;        // end of the latest upload on ustream_
    std::vector<Job*> uploaded_;       // uploaded, not yet installed (engine thread only)
    Job* uploading_ = nullptr;         // upload paused when a launch ended (engine thread, mu_)
    // bytes issued between launch tests: a pageable chunk holds the engine thread while the host
    // stages it (about 0.05 ms for 8 MB at this host's ~200 GB/s), so the end of a launch is seen
    // at most that late (32 MB chunks delayed the next launch by up to 0.45 ms)
    static constexpr size_t kUploadChunk = size_t(4) << 20;
    // Between launches the engine thread uploads queued solves itself only up to this many input
    // bytes (always at least one solve when the device would otherwise idle); the rest upload
    // during the next launch, so a stream of large solves overlaps each upload with the
    // previous solve instead of idling the device for the whole queue's copies.
    static constexpr size_t kSyncUploadBudget = size_t(64) << 20;
    bool launch_done_ = true;          // the host callback behind the current launch has run (mu_)
    double t_launch_done_ = 0;         // host time of that callback (BOXQP_PROFILE: gap to the next launch)
    // BOXQP_PROFILE: host times of the steps between two launches (engine thread)
    double t_synced_ = 0, t_collected_ = 0, t_freed_ = 0, t_gated_ = 0, t_installed_ = 0;
    cudaMemPool_t pool_ = nullptr;

    // device tables
    InstDev* d_inst_ = nullptr;
    int2* d_ranges_ = nullptr;
    int32_t* d_tile_done_ = nullptr;
    int32_t* d_status_ = nullptr;
    Tile* d_tiles_ = nullptr;
    Partial* d_partial_ = nullptr;
    Ctrl* d_ctrl_ = nullptr;
    Ctrl* h_ctrl_ = nullptr;       // pinned
    int32_t* h_status_ = nullptr;  // pinned
    int inst_cap_ = 0, tile_cap_ = 0;
    // re-arm staging (pinned host / device): records, slots, row spans
    InstDev* h_stage_ = nullptr;
    InstDev* d_stage_ = nullptr;
    int32_t* h_stage_slots_ = nullptr;
    int32_t* d_stage_slots_ = nullptr;
    int2* h_spans_ = nullptr;
    int2* d_spans_ = nullptr;
    int stage_cap_ = 0, span_cap_ = 0;

    // host mirrors
    std::vector<Tile> h_tiles_;
    std::vector<int2> h_ranges_;
    std::vector<Job*> slot_job_;
    std::vector<int32_t> slot_prec_;      // precision of the solve in each slot
    std::vector<int32_t> h_group_tiles_;  // tile indices ordered by step group
    // page-locked staging of the tables above: their copies to the device run as DMA behind the
    // engine stream instead of a pageable copy each (rewritten only after that stream drained)
    unsigned char* h_table_stage_ = nullptr;
    size_t table_stage_bytes_ = 0;
    std::vector<int4> h_units_;           // CG work units: first tile, tiles, index, units of the instance
    int32_t group_begin_[kStepGroups + 1] = {};
    uint32_t groups_present_ = 0;         // step groups with tiles
    uint32_t graph_groups_ = 0;           // step groups the graph launches
    int32_t* d_group_tiles_ = nullptr;
    int4* d_units_ = nullptr;
    std::vector<int> free_slots_;
    int n_inst_ = 0;
    bool tables_dirty_ = false;

    // graph
    cudaGraph_t graph_ = nullptr;
    cudaGraphExec_t exec_ = nullptr;
    int graph_grid_ = 0;
    int graph_interval_ = 25;
    bool graph_valid_ = false;

    // jobs
    mutable std::mutex mu_;
    std::condition_variable cv_work_, cv_done_;
    std::map<uint64_t, std::unique_ptr<Job>> jobs_;
    std::deque<Job*> queue_;
    std::deque<uint64_t> completed_;  // finished notify-jobs, in completion order
    std::vector<std::pair<int, void*>> pending_free_;
    uint64_t next_id_ = 1;
    int64_t n_running_ = 0, peak_resident_ = 0;
    size_t resident_bytes_ = 0;
    double latency_ms_ = 0;
    std::atomic<int> inject_oom_{0};
    static constexpr int kGateChunk = 1024;
    std::vector<GateResult*> gate_chunks_;
    std::vector<GateResult*> gate_free_;  // admissions left to fail as out of memory (host-side fault injection)
    double body_ms_ = 0.5;
    double timer_ms_ = 0;
    int64_t timer_kernels_ = 0, timer_launches_ = 0;
    cudaEvent_t ev0_ = nullptr, ev1_ = nullptr;
    // the last re-arm, not waited for: its staging buffers are reused and its device time counted
    // once it has completed (settle_rearm)
    cudaEvent_t rev0_ = nullptr, rev1_ = nullptr;
    bool rearm_pending_ = false;
    bool settle_rearm(std::string& why);
    // launch mode: conditional graph (default) or host-driven stream launches (BOXQP_LAUNCH=stream;
    // per-kernel profilers cannot see kernels inside conditional graphs)
    bool stream_mode_ = false;
    bool profile_phases_ = false;  // BOXQP_PROFILE=1: per-phase CUDA-event times, printed at exit
    cudaEvent_t pev_[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    double phase_ms_[4] = {0, 0, 0, 0};  // check+gate, steps, polish, control
    int64_t phase_bodies_ = 0;
    bool stop_ = false;
    std::thread thread_;

    mutable std::mutex err_mu_;
    std::string error_;
    mutable std::string err_copy_;
};

bool Engine::init(std::string& why) {
    int prev = 0;
    cudaGetDevice(&prev);
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        why = "No CUDA device available";
        return false;
    }
    if (device_ < 0 || device_ >= count) {
        why = "Invalid CUDA device index";
        return false;
    }
    if (!cuda_ok(cudaSetDevice(device_), why, "set device")) return false;
    cudaDeviceGetAttribute(&sms_, cudaDevAttrMultiProcessorCount, device_);
    grid_max_ = tile_grid(sms_);
    cg_slots_ = cg_matvec_slots();
    // the running launch's stream at the highest priority, the uploads and admission kernels of
    // new solves at the lowest: their blocks take the SMs the launch leaves free (its kernels'
    // tails and the gaps between them) instead of slowing it down
    int prio_least = 0, prio_greatest = 0;
    cudaDeviceGetStreamPriorityRange(&prio_least, &prio_greatest);
    if (!cuda_ok(cudaStreamCreateWithPriority(&stream_, cudaStreamNonBlocking, prio_greatest), why, "stream")) return false;
    if (!cuda_ok(cudaStreamCreateWithFlags(&capture_, cudaStreamNonBlocking), why, "stream")) return false;
    if (!cuda_ok(cudaStreamCreateWithPriority(&ustream_, cudaStreamNonBlocking, prio_least), why, "stream")) return false;
    if (!cuda_ok(cudaStreamCreateWithFlags(&fstream_, cudaStreamNonBlocking), why, "stream")) return false;
    if (!cuda_ok(cudaEventCreateWithFlags(&uev_, cudaEventDisableTiming), why, "event")) return false;
    cudaMemPoolProps props;
    std::memset(&props, 0, sizeof(props));
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = device_;
    if (!cuda_ok(cudaMemPoolCreate(&pool_, &props), why, "memory pool")) return false;
    uint64_t threshold = std::numeric_limits<uint64_t>::max();
    cudaMemPoolSetAttribute(pool_, cudaMemPoolAttrReleaseThreshold, &threshold);
    if (cap_ == 0) {
        size_t free_b = 0, total_b = 0;
        cudaMemGetInfo(&free_b, &total_b);
        cap_ = static_cast<size_t>(0.9 * static_cast<double>(free_b));
    }
    if (const char* m = std::getenv("BOXQP_LAUNCH")) stream_mode_ = std::string(m) == "stream";
    if (const char* m = std::getenv("BOXQP_PROFILE")) profile_phases_ = std::string(m) == "1";
    if (profile_phases_)
        for (auto& e : pev_) cudaEventCreate(&e);
    if (!cuda_ok(cudaEventCreate(&ev0_), why, "event")) return false;
    if (!cuda_ok(cudaEventCreate(&ev1_), why, "event")) return false;
    if (!cuda_ok(cudaEventCreate(&rev0_), why, "event")) return false;
    if (!cuda_ok(cudaEventCreate(&rev1_), why, "event")) return false;
    if (!cuda_ok(cudaMalloc(&d_ctrl_, sizeof(Ctrl)), why, "control block")) return false;
    if (!cuda_ok(cudaMemset(d_ctrl_, 0, sizeof(Ctrl)), why, "control block")) return false;
    if (!cuda_ok(cudaMallocHost(&h_ctrl_, sizeof(Ctrl)), why, "pinned control")) return false;
    std::memset(h_ctrl_, 0, sizeof(Ctrl));
    if (!ensure_tables(256, 1024, why)) return false;
    cudaSetDevice(prev);
    thread_ = std::thread([this] { loop(); });
    return true;
}

void Engine::shutdown() {
    {
        std::lock_guard<std::mutex> g(mu_);
        if (stop_ && !thread_.joinable()) return;
        stop_ = true;
    }
    cv_work_.notify_all();
    if (thread_.joinable()) thread_.join();
    if (stream_) {
        cudaSetDevice(device_);
        if (ustream_) cudaStreamSynchronize(ustream_);
        cudaStreamSynchronize(stream_);
        for (auto& kv : jobs_) if (kv.second->slab) cudaFreeAsync(kv.second->slab, stream_);
        for (auto& pf : pending_free_) if (pf.second) cudaFreeAsync(pf.second, stream_);
        cudaStreamSynchronize(stream_);
    }
    jobs_.clear();
    if (exec_) cudaGraphExecDestroy(exec_);
    if (graph_) cudaGraphDestroy(graph_);
    exec_ = nullptr;
    graph_ = nullptr;
    cudaFree(d_inst_); cudaFree(d_ranges_); cudaFree(d_tile_done_); cudaFree(d_status_);
    cudaFree(d_tiles_); cudaFree(d_partial_); cudaFree(d_ctrl_); cudaFree(d_group_tiles_); cudaFree(d_units_);
    d_inst_ = nullptr; d_ranges_ = nullptr; d_tile_done_ = nullptr; d_status_ = nullptr;
    d_tiles_ = nullptr; d_partial_ = nullptr; d_ctrl_ = nullptr; d_group_tiles_ = nullptr; d_units_ = nullptr;
    if (h_ctrl_) cudaFreeHost(h_ctrl_);
    if (h_stage_) cudaFreeHost(h_stage_);
    if (h_stage_slots_) cudaFreeHost(h_stage_slots_);
    if (h_spans_) cudaFreeHost(h_spans_);
    if (h_table_stage_) cudaFreeHost(h_table_stage_);
    h_table_stage_ = nullptr;
    table_stage_bytes_ = 0;
    for (GateResult* c : gate_chunks_) cudaFreeHost(c);
    gate_chunks_.clear();
    gate_free_.clear();
    cudaFree(d_stage_);
    cudaFree(d_stage_slots_);
    cudaFree(d_spans_);
    h_stage_ = nullptr; h_stage_slots_ = nullptr; h_spans_ = nullptr;
    d_stage_ = nullptr; d_stage_slots_ = nullptr; d_spans_ = nullptr;
    if (h_status_) cudaFreeHost(h_status_);
    h_ctrl_ = nullptr;
    h_status_ = nullptr;
    if (pool_) cudaMemPoolDestroy(pool_);
    pool_ = nullptr;
    if (profile_phases_) {
        std::fprintf(stderr, "[boxqp] phase ms over %lld bodies: check+gate %.3f steps %.3f polish %.3f control %.3f\n",
                     static_cast<long long>(phase_bodies_), phase_ms_[0], phase_ms_[1], phase_ms_[2], phase_ms_[3]);
        for (auto& e : pev_) if (e) cudaEventDestroy(e);
    }
    if (ev0_) cudaEventDestroy(ev0_);
    if (ev1_) cudaEventDestroy(ev1_);
    if (rev0_) cudaEventDestroy(rev0_);
    if (rev1_) cudaEventDestroy(rev1_);
    ev0_ = nullptr;
    ev1_ = nullptr;
    rev0_ = nullptr;
    rev1_ = nullptr;
    if (stream_) cudaStreamDestroy(stream_);
    if (capture_) cudaStreamDestroy(capture_);
    if (ustream_) cudaStreamDestroy(ustream_);
    if (fstream_) cudaStreamDestroy(fstream_);
    if (uev_) cudaEventDestroy(uev_);
    stream_ = nullptr;
    capture_ = nullptr;
    ustream_ = nullptr;
    fstream_ = nullptr;
    uev_ = nullptr;
}

// Grows the device tables (instance records, tile table, partials); invalidates the graph.
bool Engine::ensure_tables(int need_inst, int need_tiles, std::string& why) {
    if (need_inst > inst_cap_) {
        int cap = std::max(need_inst, std::max(256, inst_cap_ * 2));
        InstDev* inst = nullptr;
        int2* ranges = nullptr;
        int32_t *done = nullptr, *status = nullptr, *h_status = nullptr;
        if (!cuda_ok(cudaMalloc(&inst, sizeof(InstDev) * cap), why, "instance table")) return false;
        if (!cuda_ok(cudaMalloc(&ranges, sizeof(int2) * cap), why, "range table")) return false;
        if (!cuda_ok(cudaMalloc(&done, sizeof(int32_t) * cap), why, "tile counters")) return false;
        if (!cuda_ok(cudaMalloc(&status, sizeof(int32_t) * cap), why, "status mirror")) return false;
        if (!cuda_ok(cudaMallocHost(&h_status, sizeof(int32_t) * cap), why, "pinned status")) return false;
        cudaMemsetAsync(inst, 0, sizeof(InstDev) * cap, stream_);
        cudaMemsetAsync(ranges, 0, sizeof(int2) * cap, stream_);
        cudaMemsetAsync(done, 0, sizeof(int32_t) * cap, stream_);
        cudaMemsetAsync(status, 0xff, sizeof(int32_t) * cap, stream_);
        if (d_inst_) {
            cudaMemcpyAsync(inst, d_inst_, sizeof(InstDev) * inst_cap_, cudaMemcpyDeviceToDevice, stream_);
            cudaMemcpyAsync(done, d_tile_done_, sizeof(int32_t) * inst_cap_, cudaMemcpyDeviceToDevice, stream_);
        }
        cudaStreamSynchronize(stream_);
        cudaFree(d_inst_); cudaFree(d_ranges_); cudaFree(d_tile_done_); cudaFree(d_status_);
        if (h_status_) cudaFreeHost(h_status_);
        d_inst_ = inst; d_ranges_ = ranges; d_tile_done_ = done; d_status_ = status; h_status_ = h_status;
        inst_cap_ = cap;
        h_ranges_.resize(cap, int2{0, 0});
        slot_job_.resize(cap, nullptr);
        slot_prec_.resize(cap, 0);
        tables_dirty_ = true;
        graph_valid_ = false;
    }
    if (need_tiles > tile_cap_) {
        int cap = std::max(need_tiles, std::max(1024, tile_cap_ * 2));
        Tile* tiles = nullptr;
        Partial* partial = nullptr;
        int32_t* group_tiles = nullptr;
        int4* units = nullptr;
        if (!cuda_ok(cudaMalloc(&tiles, sizeof(Tile) * cap), why, "tile table")) return false;
        if (!cuda_ok(cudaMalloc(&partial, sizeof(Partial) * cap), why, "partials")) return false;
        if (!cuda_ok(cudaMalloc(&group_tiles, sizeof(int32_t) * cap), why, "step groups")) return false;
        if (!cuda_ok(cudaMalloc(&units, sizeof(int4) * cap), why, "CG work units")) return false;
        cudaFree(d_tiles_);
        cudaFree(d_partial_);
        cudaFree(d_group_tiles_);
        cudaFree(d_units_);
        d_tiles_ = tiles;
        d_partial_ = partial;
        d_group_tiles_ = group_tiles;
        d_units_ = units;
        tile_cap_ = cap;
        tables_dirty_ = true;
        graph_valid_ = false;
    }
    return true;
}

void Engine::update_grid() {
    const int grid_max = grid_max_;
    int want = static_cast<int>(std::min<size_t>(static_cast<size_t>(grid_max), align_up(std::max<size_t>(h_tiles_.size(), 1), 32)));
    graph_grid_ = std::max(want, graph_grid_);
    if (graph_grid_ > grid_max) graph_grid_ = grid_max;
}

// Host-driven launches of the same loop body: the host reads the gate's phase counts after
// each check and launches only the kernels those phases need.
bool Engine::run_stream(int cap, std::string& why) {
    update_grid();
    graph_groups_ = groups_present_;
    const int grid = graph_grid_;
    const int K = graph_interval_;
    const View v = view();
    const int precisions[3] = {PREC_FP64, PREC_MIXED, PREC_FP64_EXACT};
    long long kernels = 0;
    int bodies = 0;
    for (; bodies < cap; ++bodies) {
        if (profile_phases_) cudaEventRecord(pev_[0], stream_);
        launch_check(v, grid, stream_);
        launch_gate_plain(v, K, stream_);
        kernels += 4;
        cudaMemcpyAsync(h_ctrl_, d_ctrl_, sizeof(Ctrl), cudaMemcpyDeviceToHost, stream_);
        if (!cuda_ok(cudaStreamSynchronize(stream_), why, "engine check")) return false;
        if (profile_phases_) cudaEventRecord(pev_[1], stream_);
        const StepLaunches L = body_launches(K);
        for (int k = 0; k < 3; ++k) {
            if (h_ctrl_->n_fista[k] <= 0) continue;
            launch_body_steps(v, precisions[k], K, grid, stream_);
            kernels += L.n[k];
        }
        if (profile_phases_) cudaEventRecord(pev_[2], stream_);
        if (h_ctrl_->n_polish > 0) {
            launch_polish_init(v, grid, stream_);
            launch_polish_residual(v, grid, stream_);
            kernels += 2;
            // the CG loop as the graph runs it: stop once no instance iterates (read back after
            // every iteration; this mode serves per-kernel profiling, not speed)
            for (int j = 0; j < kCgPerBody; ++j) {
                launch_cg_matvec(v, grid, stream_);
                launch_cg_vector(v, grid, stream_);
                kernels += 2;
                cudaMemcpyAsync(h_ctrl_, d_ctrl_, sizeof(Ctrl), cudaMemcpyDeviceToHost, stream_);
                if (!cuda_ok(cudaStreamSynchronize(stream_), why, "engine polish")) return false;
                if (h_ctrl_->n_cg <= 0) break;
            }
        }
        if (profile_phases_) cudaEventRecord(pev_[3], stream_);
        launch_control_plain(v, K, stream_);
        kernels += 1;
        if (profile_phases_) cudaEventRecord(pev_[4], stream_);
        cudaMemcpyAsync(h_ctrl_, d_ctrl_, sizeof(Ctrl), cudaMemcpyDeviceToHost, stream_);
        if (!cuda_ok(cudaStreamSynchronize(stream_), why, "engine body")) return false;
        if (profile_phases_) {
            float a = 0;
            for (int k = 0; k < 4; ++k) {
                cudaEventElapsedTime(&a, pev_[k], pev_[k + 1]);
                phase_ms_[k] += a;
            }
            phase_bodies_++;
        }
        if (h_ctrl_->running == 0) {
            ++bodies;
            break;
        }
    }
    h_ctrl_->kernels = kernels;
    h_ctrl_->bodies = bodies;
    return cuda_ok(cudaGetLastError(), why, "stream launches");
}

bool Engine::build_graph(std::string& why) {
    if (exec_) cudaGraphExecDestroy(exec_);
    if (graph_) cudaGraphDestroy(graph_);
    exec_ = nullptr;
    graph_ = nullptr;
    update_grid();
    graph_groups_ = groups_present_;
    const int grid = graph_grid_;
    const int K = graph_interval_;
    const View v = view();

    if (!cuda_ok(cudaGraphCreate(&graph_, 0), why, "graph create")) return false;
    cudaGraphConditionalHandle h_loop, h_f[3], h_pol, h_cg;
    if (!cuda_ok(cudaGraphConditionalHandleCreate(&h_loop, graph_, 1, cudaGraphCondAssignDefault), why, "conditional handle")) return false;
    for (int k = 0; k < 3; ++k)
        if (!cuda_ok(cudaGraphConditionalHandleCreate(&h_f[k], graph_, 0, cudaGraphCondAssignDefault), why, "conditional handle")) return false;
    if (!cuda_ok(cudaGraphConditionalHandleCreate(&h_pol, graph_, 0, cudaGraphCondAssignDefault), why, "conditional handle")) return false;
    if (!cuda_ok(cudaGraphConditionalHandleCreate(&h_cg, graph_, 0, cudaGraphCondAssignDefault), why, "conditional handle")) return false;

    cudaGraphNodeParams wp = {cudaGraphNodeTypeConditional};
    wp.conditional.handle = h_loop;
    wp.conditional.type = cudaGraphCondTypeWhile;
    wp.conditional.size = 1;
    cudaGraphNode_t wnode;
    if (!cuda_ok(cudaGraphAddNode(&wnode, graph_, nullptr, nullptr, 0, &wp), why, "while node")) return false;
    cudaGraph_t body = wp.conditional.phGraph_out[0];

    auto capture = [&](cudaGraph_t g, const cudaGraphNode_t* deps, size_t ndeps, auto&& launches,
                       cudaGraphNode_t* last) -> bool {
        if (!cuda_ok(cudaStreamBeginCaptureToGraph(capture_, g, deps, nullptr, ndeps, cudaStreamCaptureModeThreadLocal), why, "begin capture")) return false;
        launches();
        if (last) {
            cudaStreamCaptureStatus st;
            const cudaGraphNode_t* tail = nullptr;
            size_t ntail = 0;
            if (!cuda_ok(cudaStreamGetCaptureInfo(capture_, &st, nullptr, nullptr, &tail, nullptr, &ntail), why, "capture info")) return false;
            *last = ntail ? tail[0] : nullptr;
        }
        cudaGraph_t out = nullptr;
        if (!cuda_ok(cudaStreamEndCapture(capture_, &out), why, "end capture")) return false;
        return cuda_ok(cudaGetLastError(), why, "captured launch");
    };
    auto add_cond = [&](cudaGraph_t g, cudaGraphNode_t dep, cudaGraphConditionalHandle h, cudaGraphConditionalNodeType type,
                        cudaGraphNode_t* node, cudaGraph_t* inner) -> bool {
        cudaGraphNodeParams p = {cudaGraphNodeTypeConditional};
        p.conditional.handle = h;
        p.conditional.type = type;
        p.conditional.size = 1;
        if (!cuda_ok(cudaGraphAddNode(node, g, &dep, nullptr, dep ? 1 : 0, &p), why, "conditional node")) return false;
        *inner = p.conditional.phGraph_out[0];
        return true;
    };
    auto add_if = [&](cudaGraphNode_t dep, cudaGraphConditionalHandle h, cudaGraphNode_t* node, cudaGraph_t* inner) {
        return add_cond(body, dep, h, cudaGraphCondTypeIf, node, inner);
    };

    cudaGraphNode_t last = nullptr;
    if (!capture(body, nullptr, 0, [&] {
            launch_check(v, grid, capture_);
            launch_gate(v, h_f, h_pol, h_cg, body_launches(K), K, capture_);
        }, &last)) return false;
    const int precisions[3] = {PREC_FP64, PREC_MIXED, PREC_FP64_EXACT};
    for (int k = 0; k < 3; ++k) {
        cudaGraphNode_t node;
        cudaGraph_t inner;
        if (!add_if(last, h_f[k], &node, &inner)) return false;
        if (!capture(inner, nullptr, 0, [&] { launch_body_steps(v, precisions[k], K, grid, capture_); }, nullptr))
            return false;
        last = node;
    }
    {
        cudaGraphNode_t node;
        cudaGraph_t inner;
        if (!add_if(last, h_pol, &node, &inner)) return false;
        // polish: init + residual, then WHILE (an instance is iterating, < kCgPerBody iterations)
        // { matvec, update, direction }; the direction kernel sets the loop's condition.
        cudaGraphNode_t head = nullptr, loop_node;
        cudaGraph_t loop_body;
        if (!capture(inner, nullptr, 0, [&] {
                launch_polish_init(v, grid, capture_);
                launch_polish_residual(v, grid, capture_);
            }, &head)) return false;
        if (!add_cond(inner, head, h_cg, cudaGraphCondTypeWhile, &loop_node, &loop_body)) return false;
        if (!capture(loop_body, nullptr, 0, [&] {
                launch_cg_matvec(v, grid, capture_);
                launch_cg_vector(v, grid, capture_, h_cg, kCgPerBody);
            }, nullptr)) return false;
        last = node;
    }
    if (!capture(body, &last, 1, [&] { launch_control(v, h_loop, K, capture_); }, nullptr)) return false;
    if (!cuda_ok(cudaGraphInstantiate(&exec_, graph_, 0), why, "graph instantiate")) return false;
    graph_valid_ = true;
    return true;
}

int Engine::submit(Job* raw, uint64_t* id) {
    std::unique_ptr<Job> job(raw);
    std::lock_guard<std::mutex> g(mu_);
    if (stop_) return BQP_ERR_INVALID;
    job->id = next_id_++;
    job->t_submit = host_seconds();
    Job* j = job.get();
    if (id) *id = j->id;
    const bool done = j->state == JOB_DONE;
    jobs_[j->id] = std::move(job);
    if (done && j->notify) {
        completed_.push_back(j->id);
        cv_done_.notify_all();
    }
    if (!done) {
        queue_.push_back(j);
        cv_work_.notify_all();
    }
    return BQP_OK;
}

int Engine::wait_any(double timeout, uint64_t* id) {
    std::unique_lock<std::mutex> lk(mu_);
    auto pred = [&] { return !completed_.empty() || stop_; };
    if (timeout < 0) cv_done_.wait(lk, pred);
    else if (!cv_done_.wait_for(lk, std::chrono::duration<double>(timeout), pred)) return BQP_ERR_NOT_READY;
    if (completed_.empty()) return BQP_ERR_NOT_READY;
    *id = completed_.front();
    completed_.pop_front();
    return BQP_OK;
}

int Engine::poll(uint64_t id, int32_t* status) {
    std::lock_guard<std::mutex> g(mu_);
    auto it = jobs_.find(id);
    if (it == jobs_.end()) return BQP_ERR_NOT_FOUND;
    const Job& j = *it->second;
    if (status) {
        if (j.state == JOB_DONE) *status = j.stats.status;
        else if (j.state == JOB_RUNNING) *status = BQP_STATUS_RUNNING;
        else *status = BQP_STATUS_QUEUED;
    }
    return BQP_OK;
}

int Engine::wait(uint64_t id, double timeout) {
    std::unique_lock<std::mutex> lk(mu_);
    auto pred = [&] {
        auto it = jobs_.find(id);
        return it == jobs_.end() || it->second->state == JOB_DONE;
    };
    if (timeout < 0) cv_done_.wait(lk, pred);
    else if (!cv_done_.wait_for(lk, std::chrono::duration<double>(timeout), pred)) return BQP_ERR_NOT_READY;
    auto it = jobs_.find(id);
    if (it == jobs_.end()) return BQP_ERR_NOT_FOUND;
    return it->second->error;
}

int Engine::fetch(uint64_t id, double* x, bqp_stats* stats) {
    const void* src = nullptr;
    bool f32 = false;
    int64_t n = 0;
    int rc;
    Job* jp = nullptr;
    {
        std::lock_guard<std::mutex> g(mu_);
        auto it = jobs_.find(id);
        if (it == jobs_.end()) return BQP_ERR_NOT_FOUND;
        Job& j = *it->second;
        if (j.state != JOB_DONE) return BQP_ERR_NOT_READY;
        if (stats) *stats = j.stats;
        if (j.error != BQP_OK) set_error(j.error_text);
        rc = j.error;
        if (x && j.x.empty() && j.resident && j.x_dev) {
            src = j.x_dev;
            f32 = j.x_f32;
            n = j.n;
            ++j.fetching;  // release() waits for the copy
            jp = &j;
        } else if (x && !j.x.empty()) {
            std::memcpy(x, j.x.data(), sizeof(double) * j.x.size());
        }
    }
    if (!src) return rc;
    // device -> caller memory outside the engine lock, on this engine's fetch stream
    cudaError_t e;
    {
        std::lock_guard<std::mutex> fg(fmu_);
        int prev = -1;
        cudaGetDevice(&prev);
        if (prev != device_) cudaSetDevice(device_);
        const size_t N = static_cast<size_t>(n);
        if (f32) {
            std::vector<float> tmp(N);
            e = cudaMemcpyAsync(tmp.data(), src, sizeof(float) * N, cudaMemcpyDeviceToHost, fstream_);
            if (e == cudaSuccess) e = cudaStreamSynchronize(fstream_);
            if (e == cudaSuccess)
                for (size_t i = 0; i < N; ++i) x[i] = static_cast<double>(tmp[i]);
        } else {
            e = cudaMemcpyAsync(x, src, sizeof(double) * N, cudaMemcpyDeviceToHost, fstream_);
            if (e == cudaSuccess) e = cudaStreamSynchronize(fstream_);
        }
        if (prev >= 0 && prev != device_) cudaSetDevice(prev);
    }
    std::lock_guard<std::mutex> g(mu_);
    --jp->fetching;
    if (jp->fetching == 0) cv_done_.notify_all();
    if (e != cudaSuccess) {
        set_error(std::string("CUDA: fetch primal: ") + cudaGetErrorString(e));
        return BQP_ERR_CUDA;
    }
    return rc;
}

int Engine::release(uint64_t id) {
    std::unique_lock<std::mutex> lk(mu_);
    // a bqp_fetch of this solve on another thread finishes its copy first
    cv_done_.wait(lk, [&] {
        auto f = jobs_.find(id);
        return f == jobs_.end() || f->second->fetching == 0;
    });
    auto it = jobs_.find(id);
    if (it == jobs_.end()) return BQP_ERR_NOT_FOUND;
    Job& j = *it->second;
    if (j.state == JOB_QUEUED) {
        queue_.erase(std::remove(queue_.begin(), queue_.end(), &j), queue_.end());
    } else if (j.state != JOB_DONE) {
        return BQP_ERR_NOT_READY;
    }
    completed_.erase(std::remove(completed_.begin(), completed_.end(), id), completed_.end());
    if (j.resident) {
        // the job object dies below: the engine thread must not see it through its slot (its
        // slot, tiles and slab are reclaimed at the next loop iteration)
        if (j.slot >= 0 && j.slot < static_cast<int>(slot_job_.size()) && slot_job_[j.slot] == &j)
            slot_job_[j.slot] = nullptr;
        pending_free_.emplace_back(j.slot, j.slab);
        resident_bytes_ -= j.layout.total;
        j.slab = nullptr;
        cv_work_.notify_all();
    }
    jobs_.erase(it);
    return BQP_OK;
}

int Engine::resolve(const uint64_t* ids, int64_t count) {
    std::unique_lock<std::mutex> lk(mu_);
    // a re-run overwrites the primal: bqp_fetch copies in flight finish first
    cv_done_.wait(lk, [&] {
        for (int64_t k = 0; k < count; ++k) {
            auto f = jobs_.find(ids[k]);
            if (f != jobs_.end() && f->second->fetching != 0) return false;
        }
        return true;
    });
    for (int64_t k = 0; k < count; ++k) {
        auto it = jobs_.find(ids[k]);
        if (it == jobs_.end()) return BQP_ERR_NOT_FOUND;
        if (it->second->state != JOB_DONE || !it->second->resident) return BQP_ERR_NOT_READY;
    }
    for (int64_t k = 0; k < count; ++k) {
        Job& j = *jobs_[ids[k]];
        j.state = JOB_QUEUED;
        j.resolve = true;
        j.notify = true;
        j.error = BQP_OK;
        j.t_submit = host_seconds();
        queue_.push_back(&j);
    }
    cv_work_.notify_all();
    return BQP_OK;
}

int Engine::load(int64_t* queued, int64_t* running, int64_t* peak, int64_t* resident_bytes) {
    std::lock_guard<std::mutex> g(mu_);
    if (queued) *queued = static_cast<int64_t>(queue_.size());
    if (running) *running = n_running_;
    if (peak) *peak = peak_resident_;
    if (resident_bytes) *resident_bytes = static_cast<int64_t>(resident_bytes_);
    return BQP_OK;
}

// Control state of a solve at its start (a new upload or a re-arm of a resident solve).
void Engine::reset_record(Job& j) {
    InstDev& R = j.rec;
    R.status = ST_RUNNING;
    R.phase = PH_FISTA;
    R.polish_rounds = 0;
    R.it0 = 0;
    R.it_cur = 0;
    R.it_next = 0;
    R.t = 1.0;
    R.deadline_ns = static_cast<int64_t>(std::min(j.opt.time_limit, 1e9) * 1e9);  // budget; made absolute on device
    R.verified = 0;
    R.stable_checks = 0;
    R.active_hash = 0;
    R.n_active = -1;
    R.result_src = 0;
    R.cg_it = 0;
    R.cg_total = 0;
    R.fista_iters = 0;
    R.checks = 0;
    R.ff_nnz = 0;
    R.ff_rows = 0;
    R.polish_bytes = 0.0;
    R.iterations = 0;
    R.arm_chunk = (j.opt.precision == PREC_MIXED && R.max_iter > 0) ? 1 : 0;
    R.moved[0] = 0;
    R.moved[1] = 0;
}

// Re-arms resident solves (bqp_resolve): one upload of the staged records and one kernel for the
// whole batch.  Engine thread only.
bool Engine::rearm(const std::vector<Job*>& batch, std::string& why) {
    // the staging buffers are reused (or reallocated): the previous re-arm must have completed
    // (in steady state it has, long before)
    if (!settle_rearm(why)) return false;
    const int count = static_cast<int>(batch.size());
    int spans = 0;
    for (const Job* j : batch) spans += static_cast<int>((j->n + kRearmRows - 1) / kRearmRows);
    if (count > stage_cap_) {
        const int cap = std::max(count, std::max(256, 2 * stage_cap_));
        if (h_stage_) cudaFreeHost(h_stage_);
        if (h_stage_slots_) cudaFreeHost(h_stage_slots_);
        cudaFree(d_stage_);
        cudaFree(d_stage_slots_);
        h_stage_ = nullptr; h_stage_slots_ = nullptr; d_stage_ = nullptr; d_stage_slots_ = nullptr;
        stage_cap_ = 0;
        if (!cuda_ok(cudaMallocHost(&h_stage_, sizeof(InstDev) * cap), why, "re-arm staging")) return false;
        if (!cuda_ok(cudaMallocHost(&h_stage_slots_, sizeof(int32_t) * cap), why, "re-arm staging")) return false;
        if (!cuda_ok(cudaMalloc(&d_stage_, sizeof(InstDev) * cap), why, "re-arm staging")) return false;
        if (!cuda_ok(cudaMalloc(&d_stage_slots_, sizeof(int32_t) * cap), why, "re-arm staging")) return false;
        stage_cap_ = cap;
    }
    if (spans > span_cap_) {
        const int cap = std::max(spans, std::max(256, 2 * span_cap_));
        if (h_spans_) cudaFreeHost(h_spans_);
        cudaFree(d_spans_);
        h_spans_ = nullptr; d_spans_ = nullptr;
        span_cap_ = 0;
        if (!cuda_ok(cudaMallocHost(&h_spans_, sizeof(int2) * cap), why, "re-arm staging")) return false;
        if (!cuda_ok(cudaMalloc(&d_spans_, sizeof(int2) * cap), why, "re-arm staging")) return false;
        span_cap_ = cap;
    }
    int s = 0;
    for (int k = 0; k < count; ++k) {
        Job& j = *batch[k];
        reset_record(j);
        h_stage_[k] = j.rec;
        h_stage_slots_[k] = j.slot;
        for (int64_t r = 0; r < j.n; r += kRearmRows) h_spans_[s++] = int2{k, static_cast<int>(r)};
    }
    cudaEventRecord(rev0_, stream_);
    cudaMemcpyAsync(d_stage_, h_stage_, sizeof(InstDev) * count, cudaMemcpyHostToDevice, stream_);
    cudaMemcpyAsync(d_stage_slots_, h_stage_slots_, sizeof(int32_t) * count, cudaMemcpyHostToDevice, stream_);
    cudaMemcpyAsync(d_spans_, h_spans_, sizeof(int2) * spans, cudaMemcpyHostToDevice, stream_);
    launch_rearm(view(), d_stage_, d_stage_slots_, d_spans_, spans, stream_);
    cudaEventRecord(rev1_, stream_);
    if (!cuda_ok(cudaGetLastError(), why, "re-arm kernel")) return false;
    rearm_pending_ = true;  // the next launch on stream_ runs after it
    return true;
}

// Waits for the last re-arm (if any is outstanding) and counts its device time: re-arming
// resident solves is part of their device time.
bool Engine::settle_rearm(std::string& why) {
    if (!rearm_pending_) return true;
    if (!cuda_ok(cudaEventSynchronize(rev1_), why, "re-arm")) return false;
    rearm_pending_ = false;
    float ms = 0;
    cudaEventElapsedTime(&ms, rev0_, rev1_);
    std::lock_guard<std::mutex> g(mu_);
    timer_ms_ += ms;
    timer_kernels_ += 1;
    return true;
}

// Steps per body: the shortest check interval among the running solves (a longer chunk spans
// several bodies; each solve checks at its own iterations whatever the batch).
void Engine::update_steps() {
    int steps = kMaxInterval;
    bool any = false;
    for (const Job* r : slot_job_)
        if (r && r->state == JOB_RUNNING) {
            steps = std::min(steps, r->rec.interval);
            any = true;
        }
    if (!any) return;
    steps = std::max(1, steps);
    if (steps != graph_interval_) {
        graph_interval_ = steps;
        graph_valid_ = false;
    }
}

// Uploads one new solve on the upload stream (inputs, slab, device-side forms), without touching
// the tables the running graph reads; install() makes it part of the batch.  Engine thread only.
// Upload of one new solve on ustream_, in three steps so that the engine thread can pause it when
// the running launch ends: upload_begin (slab, record, the list of copies), upload_copy (issues
// copies up to a byte budget; pageable copies are staged by this thread), upload_finish
// (admission kernels, the upload event).
bool Engine::upload(Job& j, std::string& why) {
    if (!upload_begin(j, why)) return false;
    upload_copy(j, static_cast<size_t>(-1));
    return upload_finish(j, why);
}

bool Engine::upload_begin(Job& j, std::string& why) {
    j.t_upload = host_seconds();
    const int prec = j.opt.precision;
    j.layout = make_layout(j.n, j.nnz, static_cast<int64_t>(j.tiles.size()), prec);
    void* slab = nullptr;
    // host-side fault injection (bqp_inject_admission_oom): fail as an exhausted pool would,
    // without any device call
    for (int left = inject_oom_.load(); left > 0;) {
        if (inject_oom_.compare_exchange_weak(left, left - 1)) {
            j.out_of_memory = true;
            why = "CUDA: allocate solve: out of memory (injected on the host)";
            return false;
        }
    }
    const cudaError_t alloc = cudaMallocFromPoolAsync(&slab, j.layout.total, pool_, ustream_);
    if (alloc == cudaErrorMemoryAllocation) {
        cudaGetLastError();  // not sticky: clear it so later calls do not report it
        j.out_of_memory = true;
        why = std::string("CUDA: allocate solve: ") + cudaGetErrorString(alloc);
        return false;
    }
    if (!cuda_ok(alloc, why, "allocate solve")) return false;
    j.slab = slab;
    j.resident = true;
    const Layout& L = j.layout;
    const size_t N = static_cast<size_t>(j.n), Z = static_cast<size_t>(j.nnz);
    j.pieces.clear();
    j.piece = j.piece_off = 0;
    j.pieces.push_back({at<int32_t>(slab, L.rowptr), j.rowptr, (N + 1) * 4});
    if (Z) j.pieces.push_back({at<int32_t>(slab, L.col), j.col, Z * 4});
    j.pieces.push_back({at<double>(slab, L.c), j.c, N * 8});
    j.pieces.push_back({at<double>(slab, L.l), j.l, N * 8});
    j.pieces.push_back({at<double>(slab, L.u), j.u, N * 8});
    InstDev& R = j.rec;
    std::memset(&R, 0, sizeof(R));
    R.rowptr = at<int32_t>(slab, L.rowptr);
    R.col = at<int32_t>(slab, L.col);
    R.val64 = at<double>(slab, L.val64);
    R.vhi = at<float>(slab, L.vhi);
    R.vlo = at<float>(slab, L.vlo);
    R.c = at<double>(slab, L.c);
    R.l = at<double>(slab, L.l);
    R.u = at<double>(slab, L.u);
    R.c32 = at<float>(slab, L.c32);
    R.l32 = at<float>(slab, L.l32);
    R.u32 = at<float>(slab, L.u32);
    R.diag = at<double>(slab, L.diag);
    R.x64 = at<double>(slab, L.x64);
    if (L.xf != kNone) R.xf = at<double>(slab, L.xf);  // the same field (mixed engines have no x64)
    R.w64[0] = at<double>(slab, L.w64a);
    R.w64[1] = at<double>(slab, L.w64b);
    R.x32 = at<float>(slab, L.x32);
    R.w32[0] = at<float>(slab, L.w32a);
    R.w32[1] = at<float>(slab, L.w32b);
    R.xp = at<double>(slab, L.xp);
    R.r = at<double>(slab, L.r);
    R.p = at<double>(slab, L.p);
    R.q = at<double>(slab, L.q);
    R.z = at<double>(slab, L.z);
    R.xq = at<int4>(slab, L.xq);
    R.pos_of = at<int32_t>(slab, L.pos_of);
    R.xp2 = at<float2>(slab, L.xp2);
    R.p2 = at<float2>(slab, L.p2);
    R.dinv = at<double>(slab, L.dinv);
    R.free_rows = at<int32_t>(slab, L.free_rows);
    R.free_cnt = at<int32_t>(slab, L.free_cnt);
    R.pc_inv = at<double>(slab, L.pc_inv);
    R.pc_e = at<double>(slab, L.pc_e);
    R.pc_tile = at<int32_t>(slab, L.pc_tile);
    R.stat_floor = 0;
    R.col_ff = at<int32_t>(slab, L.col_ff);
    R.hi_ff = at<float>(slab, L.hi_ff);
    R.lo_ff = at<float>(slab, L.lo_ff);
    R.cnt_ff = at<int32_t>(slab, L.cnt_ff);
    R.start_ff = at<int32_t>(slab, L.start_ff);
    R.sstep = at<float>(slab, L.sstep);
    R.s = at<double>(slab, L.s);
    R.lprec = at<double>(slab, L.lprec);
    R.gate = at<GateResult>(slab, L.gate);
    // polish lanes per row: about a quarter of the average row length, a power of two
    auto lanes_for = [](double avg) {
        int lanes = 1;
        while (lanes < 32 && 4.0 * lanes * 1.5 <= avg) lanes *= 2;
        return lanes;
    };
    const double avg_row = static_cast<double>(j.nnz) / static_cast<double>(std::max<int64_t>(j.n, 1));
    R.lanes_res = lanes_for(avg_row);
    R.lanes_cg = lanes_for(0.5 * avg_row);
    R.n = static_cast<int32_t>(j.n);
    R.diag_gate = j.diag_gate > 0 ? 1 : 0;
    R.precision = prec;
    R.L = j.lipschitz;
    R.invL = 1.0 / j.lipschitz;
    R.invLf = static_cast<float>(1.0 / j.lipschitz);
    R.tol = j.opt.tolerance;
    R.offset = j.opt.offset;
    R.interval = j.opt.check_interval;
    R.max_iter = j.opt.iteration_limit;
    R.polish = prec == PREC_MIXED ? 1 : 0;
    R.cg_max = std::max<int64_t>(50, std::min<int64_t>(5000, j.n));
    // CG stops at half the tolerance on max |r|/(1+|x|), the free rows' stationarity ratio, a 2x
    // margin for the verification (which recomputes it from Q and x in FP64).  0.3 / 0.5 / 0.7:
    // the 1024^2 grid 24 / 22 / 22 CG iterations, graph10k 7 / 7 / 6; graph1m and the tridiagonal
    // family unchanged; every solve verified.
    R.cg_tol = 0.5 * j.opt.tolerance;
    R.polish_switch = j.opt.polish_switch;
    // a step-stable chunk (its last three iterates share their active set) starts the polish at
    // 3x the switch.  On chain-like rows (tridiagonal) the free runs are long; with the Jacobi
    // preconditioner alone an early polish there cost more CG iterations than the FISTA steps it
    // saved, but the polish's chain preconditioner solves such runs directly (tridiagonal family:
    // polish at 25 FISTA steps instead of 50, the same 8 CG iterations, 1.97 -> 1.48 ms)
    R.step_switch = 3.0 * j.opt.polish_switch;
    R.lip_device = j.opt.lipschitz == BQP_LIPSCHITZ_POWER ? 1 : 0;
    j.power = nullptr;
    j.tmp = nullptr;
    if (R.lip_device &&
        !cuda_ok(cudaMallocFromPoolAsync(&j.power, power_scratch_bytes(j.n), pool_, ustream_), why, "allocate power scratch"))
        return false;
    if (prec == PREC_MIXED) {
        // FP64 values only for the admission kernels (hi/lo split, diagonal, preconditioner)
        if (!cuda_ok(cudaMallocFromPoolAsync(&j.tmp, Z * 8 + 64, pool_, ustream_), why, "allocate upload buffer")) return false;
        if (Z) j.pieces.push_back({j.tmp, j.val, Z * 8});
    } else if (Z) {
        j.pieces.push_back({at<double>(slab, L.val64), j.val, Z * 8});
    }
    return true;
}

// Issues copies of up to `budget` bytes; true once every copy of the solve is issued.
bool Engine::upload_copy(Job& j, size_t budget) {
    while (j.piece < j.pieces.size() && budget > 0) {
        const Job::Piece& p = j.pieces[j.piece];
        const size_t take = std::min(budget, p.bytes - j.piece_off);
        cudaMemcpyAsync(static_cast<char*>(p.dst) + j.piece_off, static_cast<const char*>(p.src) + j.piece_off, take,
                        cudaMemcpyHostToDevice, ustream_);
        budget -= take;
        j.piece_off += take;
        if (j.piece_off == p.bytes) {
            ++j.piece;
            j.piece_off = 0;
        }
    }
    return j.piece == j.pieces.size();
}

bool Engine::upload_finish(Job& j, std::string& why) {
    InstDev& R = j.rec;
    const int prec = j.opt.precision;
    // the convexity gate and the Gershgorin bound first: the other admission kernels read L from
    // its result, and the engine thread reads the result back before it installs the solve
    j.gate_host = acquire_gate_slot();
    if (!j.gate_host) {
        why = "host memory for the convexity gate result";
        return false;
    }
    launch_gate(R, j.n, prec == PREC_MIXED ? static_cast<const double*>(j.tmp) : R.val64, ustream_);
    cudaMemcpyAsync(j.gate_host, R.gate, sizeof(GateResult), cudaMemcpyDeviceToHost, ustream_);
    if (prec == PREC_MIXED) {
        launch_prepare_instance(R, j.n, ustream_);
        launch_precondition(R, j.n, static_cast<const double*>(j.tmp), j.opt.scaling != 2, j.power, ustream_);
        cudaFreeAsync(j.tmp, ustream_);
    } else {
        const double* val = R.val64;
        launch_prepare_instance(R, j.n, ustream_);
        if (R.lip_device) {
            cudaMemcpyAsync(R.lprec, &R.gate->lip_bits, sizeof(double), cudaMemcpyDeviceToDevice, ustream_);
            launch_power_lipschitz(R, j.n, val, false, j.power, ustream_);
        }
    }
    if (j.power) cudaFreeAsync(j.power, ustream_);
    j.tmp = nullptr;
    j.power = nullptr;
    std::vector<Job::Piece>().swap(j.pieces);
    if (!cuda_ok(cudaGetLastError(), why, "admission kernels")) return false;
    cudaEventRecord(uev_, ustream_);
    if (host_profile()) {
        const double t1 = host_seconds();
        cudaStreamSynchronize(ustream_);
        std::fprintf(stderr, "[boxqp] upload n=%lld: enqueue %.3f ms, device done %.3f ms\n", static_cast<long long>(j.n),
                     1e3 * (t1 - j.t_upload), 1e3 * (host_seconds() - j.t_upload));
    }
    return true;
}

// Makes uploaded solves part of the batch: slots, tiles and records (one re-arm launch, after
// the uploads on ustream_).  Engine thread, between graph launches.
bool Engine::install(std::vector<Job*>& jobs, std::string& why) {
    for (Job* jp : jobs) {
        Job& j = *jp;
        int slot;
        if (!free_slots_.empty()) {
            slot = free_slots_.back();
            free_slots_.pop_back();
        } else {
            if (!ensure_tables(n_inst_ + 1, 0, why)) return false;
            slot = n_inst_++;
        }
        j.slot = slot;
        slot_prec_[slot] = j.opt.precision;
        for (Tile& t : j.tiles) t.inst = slot;
        const int begin = static_cast<int>(h_tiles_.size());
        if (!ensure_tables(0, begin + static_cast<int>(j.tiles.size()), why)) return false;
        h_tiles_.insert(h_tiles_.end(), j.tiles.begin(), j.tiles.end());
        h_ranges_[slot] = int2{begin, static_cast<int>(h_tiles_.size())};
        tables_dirty_ = true;
    }
    if (!cuda_ok(cudaStreamWaitEvent(stream_, uev_, 0), why, "upload order")) return false;
    if (!rearm(jobs, why)) return false;
    if (graph_grid_ < grid_max_ && static_cast<int>(h_tiles_.size()) > graph_grid_) graph_valid_ = false;
    return true;
}

// While a graph runs: uploads the new solves at the head of the queue that fit under the cap, in
// chunks of kUploadChunk bytes; when the launch ends, an upload in progress pauses (uploading_)
// so that the next launch is not held up by the host staging of a large solve.
void Engine::upload_waiting() {
    std::unique_lock<std::mutex> lk(mu_);
    while (!stop_ && !launch_done_) {
        Job* j = uploading_;
        if (!j) {
            if (queue_.empty()) break;
            j = queue_.front();
            if (j->resolve) break;
            const size_t need = make_layout(j->n, j->nnz, static_cast<int64_t>(j->tiles.size()), j->opt.precision).total;
            if (resident_bytes_ + need > cap_) break;
            queue_.pop_front();
            j->state = JOB_ADMITTING;
            resident_bytes_ += need;
            lk.unlock();
            std::string why;
            const bool ok = upload_begin(*j, why);
            lk.lock();
            if (!ok) {
                fail_admission(j, need, why);
                continue;
            }
            uploading_ = j;
        }
        lk.unlock();
        std::string why;
        const bool copied = upload_copy(*j, kUploadChunk);
        bool ok = true;
        if (copied) ok = upload_finish(*j, why);
        lk.lock();
        if (copied) {
            uploading_ = nullptr;
            if (ok) uploaded_.push_back(j);
            else fail_admission(j, j->layout.total, why);
        }
    }
}

// Completes a paused upload (no launch running); caller holds mu_ through lk.
void Engine::finish_paused_upload(std::unique_lock<std::mutex>& lk) {
    Job* j = uploading_;
    if (!j) return;
    lk.unlock();
    std::string why;
    upload_copy(*j, static_cast<size_t>(-1));
    const bool ok = upload_finish(*j, why);
    lk.lock();
    uploading_ = nullptr;
    if (ok) uploaded_.push_back(j);
    else fail_admission(j, j->layout.total, why);
}

// Decides the convexity gate of solves uploaded since the last installation, once their upload
// stream work is done: the device's Gershgorin bound becomes the solve's L (the FISTA step); an
// indefinite row, or a Hessian that is not diagonally dominant and fails the host LDL^T test on
// its CSR (kept for this until now), sends the solve to `refused` (unsupported_curvature).  The
// inputs are released here.  Engine thread, without mu_.
bool Engine::gate_uploaded(std::vector<Job*>& batch, std::vector<Job*>& refused, std::string& why) {
    if (!cuda_ok(cudaEventSynchronize(uev_), why, "admission gate")) return false;
    std::vector<Job*> keep;
    keep.reserve(batch.size());
    for (Job* j : batch) {
        const GateResult g = *j->gate_host;
        release_gate_slot(*j);
        // the order of solve_accelerated_box (src/accelerated_qp.cpp:19-28): check_convex_hessian
        // rejects invalid entries, then decides convexity; then a zero Hessian is refused
        if (g.flags & kGateInvalid) {
            free_inputs(*j);
            j->error = BQP_ERR_INVALID;
            j->error_text = "Invalid Hessian";
            refused.push_back(j);
            continue;
        }
        bool convex = g.indefinite == 0;
        if (convex && g.nondominant) convex = host_gate_convex(j->n, j->rowptr, j->col, j->val);
        free_inputs(*j);
        if (!convex) {
            refused.push_back(j);
            continue;
        }
        if (!(g.flags & kGateNonzero)) {  // the Gershgorin bound is zero
            j->error = BQP_ERR_UNSUPPORTED;
            j->error_text = "Zero-Hessian models use the CPU LP path";
            refused.push_back(j);
            continue;
        }
        if (j->diag_gate < 0) j->rec.diag_gate = (g.flags & (kGateOffDiagonal | kGateNonPositive)) ? 0 : 1;
        double L = 0;
        std::memcpy(&L, &g.lip_bits, sizeof(double));
        j->lipschitz = L;
        j->rec.L = L;
        j->rec.invL = 1.0 / L;
        j->rec.invLf = static_cast<float>(1.0 / L);
        keep.push_back(j);
    }
    batch.swap(keep);
    return true;
}

// A solve refused at the gate after its upload: its memory goes back and it finishes as
// unsupported_curvature, or with the error the gate found (invalid entries, zero Hessian).
// Caller holds mu_.
void Engine::finish_refused(Job* j) {
    resident_bytes_ -= j->layout.total;
    if (j->resident) {
        pending_free_.emplace_back(-1, j->slab);
        j->slab = nullptr;
        j->resident = false;
    }
    if (j->error != BQP_OK) set_error(j->error_text);
    else set_unsupported(j->stats);
    j->state = JOB_DONE;
    if (j->notify) completed_.push_back(j->id);
    cv_done_.notify_all();
}

// A solve whose admission failed: its reserved bytes and any slab go back, it finishes with the
// CUDA error.  Caller holds mu_.
void Engine::fail_admission(Job* j, size_t reserved, const std::string& why) {
    release_gate_slot(*j);
    resident_bytes_ -= reserved;
    if (j->resident) {
        pending_free_.emplace_back(-1, j->slab);
        j->slab = nullptr;
        j->resident = false;
    }
    j->error = j->out_of_memory ? BQP_ERR_NO_MEMORY : BQP_ERR_CUDA;
    j->error_text = why;
    j->state = JOB_DONE;
    if (j->notify) completed_.push_back(j->id);
    set_error(why);
    cv_done_.notify_all();
}

void Engine::process_frees() {
    if (pending_free_.empty()) return;
    std::vector<char> dead(static_cast<size_t>(std::max(n_inst_, 1)), 0);
    for (auto& pf : pending_free_) {
        if (pf.second) cudaFreeAsync(pf.second, stream_);
        if (pf.first >= 0) {
            dead[pf.first] = 1;
            slot_job_[pf.first] = nullptr;
            free_slots_.push_back(pf.first);
            h_ranges_[pf.first] = int2{0, 0};
        }
    }
    pending_free_.clear();
    std::vector<Tile> kept;
    kept.reserve(h_tiles_.size());
    for (const Tile& t : h_tiles_) if (!dead[t.inst]) kept.push_back(t);
    h_tiles_.swap(kept);
    for (int s = 0; s < n_inst_; ++s) h_ranges_[s] = int2{0, 0};
    for (int k = 0; k < static_cast<int>(h_tiles_.size()); ++k) {
        int2& r = h_ranges_[h_tiles_[k].inst];
        if (r.y == 0) r.x = k;
        r.y = k + 1;
    }
    tables_dirty_ = true;
}

// Uploads the tile and range tables and the step groups (tiles ordered by (precision, variant),
// a counting sort in table order) when they changed.  A group the graph does not launch yet
// invalidates it.
void Engine::upload_tables() {
    if (!tables_dirty_) return;
    int32_t count[kStepGroups + 1] = {};
    for (const Tile& t : h_tiles_) {
        const int g = step_group(slot_prec_[t.inst], t.variant);
        if (g >= 0) count[g + 1]++;
    }
    groups_present_ = 0;
    for (int g = 0; g < kStepGroups; ++g) {
        if (count[g + 1]) groups_present_ |= 1u << g;
        count[g + 1] += count[g];
    }
    std::memcpy(group_begin_, count, sizeof(group_begin_));
    h_group_tiles_.resize(static_cast<size_t>(count[kStepGroups]));
    for (int k = 0; k < static_cast<int>(h_tiles_.size()); ++k) {
        const int g = step_group(slot_prec_[h_tiles_[k].inst], h_tiles_[k].variant);
        if (g >= 0) h_group_tiles_[static_cast<size_t>(count[g]++)] = k;
    }
    // CG work units: runs of consecutive tiles of one instance (cg_units; a unit depends on the
    // instance alone, not on the batch)
    h_units_.clear();
    for (int i = 0; i < n_inst_; ++i) {
        const int2 R = h_ranges_[i];
        if (R.y > R.x) cg_units(h_tiles_.data() + R.x, R.y - R.x, R.x, cg_slots_, h_units_);
    }
    // the four tables through one page-locked staging buffer (16-byte aligned parts)
    const size_t b_tiles = sizeof(Tile) * h_tiles_.size();
    const size_t b_group = sizeof(int32_t) * h_group_tiles_.size();
    const size_t b_units = sizeof(int4) * h_units_.size();
    const size_t b_ranges = sizeof(int2) * static_cast<size_t>(std::max(n_inst_, 1));
    auto up16 = [](size_t b) { return (b + 15) & ~size_t(15); };
    const size_t need = up16(b_tiles) + up16(b_group) + up16(b_units) + up16(b_ranges);
    if (need > table_stage_bytes_) {
        const size_t cap = std::max(need, 2 * table_stage_bytes_);
        if (h_table_stage_) cudaFreeHost(h_table_stage_);
        h_table_stage_ = nullptr;
        table_stage_bytes_ = 0;
        if (cudaMallocHost(&h_table_stage_, cap) == cudaSuccess) table_stage_bytes_ = cap;
    }
    auto stage = [&](void* dst, const void* src, size_t bytes, size_t& at) {
        if (bytes == 0) return;
        if (h_table_stage_) {
            std::memcpy(h_table_stage_ + at, src, bytes);
            cudaMemcpyAsync(dst, h_table_stage_ + at, bytes, cudaMemcpyHostToDevice, stream_);
            at += up16(bytes);
        } else {
            cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, stream_);  // pageable fallback
        }
    };
    size_t at = 0;
    stage(d_tiles_, h_tiles_.data(), b_tiles, at);
    stage(d_group_tiles_, h_group_tiles_.data(), b_group, at);
    stage(d_units_, h_units_.data(), b_units, at);
    stage(d_ranges_, h_ranges_.data(), b_ranges, at);
    // the staging buffer is rewritten only by the next call, after the engine stream drained
    if (groups_present_ & ~graph_groups_) graph_valid_ = false;
    tables_dirty_ = false;
}

bool Engine::run_once(std::string& why) {
    const double t_enter = host_profile() ? host_seconds() : 0.0;
    upload_tables();
    const double t_tables = host_profile() ? host_seconds() : 0.0;
    if (!stream_mode_ && !graph_valid_ && !build_graph(why)) return false;
    int cap = std::numeric_limits<int>::max() / 2;
    double latency;
    {
        std::lock_guard<std::mutex> g(mu_);
        latency = latency_ms_;
    }
    if (latency > 0) cap = std::max(1, static_cast<int>(latency / std::max(body_ms_, 1e-3)));
    h_ctrl_->n_inst = n_inst_;
    h_ctrl_->n_tiles = static_cast<int32_t>(h_tiles_.size());
    h_ctrl_->n_units = static_cast<int32_t>(h_units_.size());
    std::memcpy(h_ctrl_->group_begin, group_begin_, sizeof(group_begin_));
    for (int k = 0; k < 3; ++k) {
        h_ctrl_->check_due[k] = 1;  // the first body checks whatever is due; later ones as counted
        h_ctrl_->step_due[k] = kMaxInterval;
    }
    h_ctrl_->bodies = 0;
    h_ctrl_->body_cap = cap;
    h_ctrl_->error = 0;
    h_ctrl_->kernels = 0;
    const double t0 = host_seconds();
    if (!cuda_ok(cudaMemcpyAsync(d_ctrl_, h_ctrl_, sizeof(Ctrl), cudaMemcpyHostToDevice, stream_), why, "control upload")) return false;
    cudaEventRecord(ev0_, stream_);
    if (stream_mode_) {
        if (!run_stream(cap, why)) return false;
        cudaMemcpyAsync(d_ctrl_, h_ctrl_, sizeof(Ctrl), cudaMemcpyHostToDevice, stream_);
    } else if (!cuda_ok(cudaGraphLaunch(exec_, stream_), why, "graph launch")) {
        return false;
    }
    if (host_profile()) {
        const double t_launched = host_seconds();
        std::fprintf(stderr, "[boxqp] launch preparation: tables %.3f ms, control %.3f ms, graph launch %.3f ms\n",
                     1e3 * (t_tables - t_enter), 1e3 * (t0 - t_tables), 1e3 * (t_launched - t0));
        std::lock_guard<std::mutex> g(mu_);
        // steps since the previous launch's callback: its stream synchronised, finished solves
        // collected, frees, the admission gate read back, installation (each -1 when not run)
        auto since = [&](double t) { return t >= t_launch_done_ ? 1e3 * (t - t_launch_done_) : -1.0; };
        std::fprintf(stderr,
                     "[boxqp] launch: %d solves running, %.3f ms since the previous launch ended (synced %.3f, "
                     "collected %.3f, freed %.3f, gated %.3f, installed %.3f)\n",
                     n_running_, 1e3 * (t0 - t_launch_done_), since(t_synced_), since(t_collected_), since(t_freed_),
                     since(t_gated_), since(t_installed_));
    }
    cudaEventRecord(ev1_, stream_);
    cudaMemcpyAsync(h_status_, d_status_, sizeof(int32_t) * std::max(n_inst_, 1), cudaMemcpyDeviceToHost, stream_);
    cudaMemcpyAsync(h_ctrl_, d_ctrl_, sizeof(Ctrl), cudaMemcpyDeviceToHost, stream_);
    // while the device runs the launch, upload the new solves that arrive (they are installed
    // before the next launch); a host callback behind the launch ends the wait
    {
        std::lock_guard<std::mutex> g(mu_);
        launch_done_ = false;
    }
    if (!cuda_ok(cudaLaunchHostFunc(stream_, &Engine::on_launch_done, this), why, "launch callback")) return false;
    for (;;) {
        upload_waiting();
        std::unique_lock<std::mutex> lk(mu_);
        cv_work_.wait(lk, [&] { return launch_done_ || stop_ || uploadable_head(); });
        if (launch_done_ || stop_) break;
    }
    if (!cuda_ok(cudaStreamSynchronize(stream_), why, "engine launch")) return false;
    if (host_profile()) t_synced_ = host_seconds();
    if (!settle_rearm(why)) return false;  // completed before the launch: no wait
    const double dt = host_seconds() - t0;
    float ms = 0;
    cudaEventElapsedTime(&ms, ev0_, ev1_);
    {
        std::lock_guard<std::mutex> g(mu_);
        timer_ms_ += ms;
        timer_kernels_ += h_ctrl_->kernels;
        timer_launches_ += 1;
    }
    if (h_ctrl_->bodies > 0) body_ms_ = 0.7 * body_ms_ + 0.3 * (1e3 * dt / h_ctrl_->bodies);
    return true;
}

// Moves finished solves to the done state: copies their records and primals back.
void Engine::collect(std::unique_lock<std::mutex>& lk) {
    std::vector<Job*> finished;
    for (int s = 0; s < n_inst_; ++s) {
        Job* j = slot_job_[s];
        if (j && j->state == JOB_RUNNING && h_status_[s] != ST_RUNNING) finished.push_back(j);
    }
    if (finished.empty()) return;
    lk.unlock();
    std::vector<InstDev> recs(finished.size());
    for (size_t k = 0; k < finished.size(); ++k)
        cudaMemcpyAsync(&recs[k], &d_inst_[finished[k]->slot], sizeof(InstDev), cudaMemcpyDeviceToHost, stream_);
    cudaStreamSynchronize(stream_);
    // Primals of up to kHostPrimal variables come back now, all behind one synchronisation; a
    // larger one stays in the slab (final, untouched until release or re-run) and bqp_fetch
    // copies it straight to the caller's array, off the engine thread.
    std::vector<std::vector<float>> x32(finished.size());
    bool small = false;
    for (size_t k = 0; k < finished.size(); ++k) {
        Job& j = *finished[k];
        const InstDev& R = recs[k];
        j.x_f32 = R.result_src == 1;
        j.x_dev = R.result_src == 1 ? static_cast<const void*>(R.x32)
                                    : static_cast<const void*>(R.result_src == 2 ? R.xp : R.x64);
        j.x.clear();
        if (j.n > kHostPrimal) continue;
        small = true;
        j.x.resize(static_cast<size_t>(j.n));
        void* dst = j.x.data();
        if (j.x_f32) {
            x32[k].resize(static_cast<size_t>(j.n));
            dst = x32[k].data();
        }
        cudaMemcpyAsync(dst, j.x_dev, (j.x_f32 ? 4 : 8) * static_cast<size_t>(j.n), cudaMemcpyDeviceToHost, stream_);
    }
    if (small) cudaStreamSynchronize(stream_);
    const double now = host_seconds();
    for (size_t k = 0; k < finished.size(); ++k) {
        Job& j = *finished[k];
        const InstDev& R = recs[k];
        if (!j.x.empty()) {
            if (j.x_f32)
                for (int64_t i = 0; i < j.n; ++i) j.x[i] = static_cast<double>(x32[k][i]);
            j.x_dev = nullptr;
        }
        bqp_stats& s = j.stats;
        s.status = status_code(R.status);
        s.verified = R.verified;
        s.iterations = R.iterations;
        s.polish_iterations = R.cg_total;
        s.polish_rounds = R.polish_rounds + (R.result_src == 2 ? 1 : 0);
        s.objective = R.objective;
        s.primal_residual = R.primal_res;
        s.stationarity_residual = R.stationarity;
        s.complementarity_residual = 0.0;
        s.dual_bound = R.dual_bound;
        s.relative_gap = R.rel_gap;
        s.lipschitz = R.L;
        s.device_start_ns = R.start_ns;
        s.device_end_ns = R.end_ns;
        s.device_seconds = 1e-9 * static_cast<double>(R.end_ns - R.start_ns);
        s.checks = R.checks;
        s.bytes = algorithmic_bytes(j.n, j.nnz, j.opt.precision, R.fista_iters, R.checks, R.polish_bytes);
        j.t_done = now;
    }
    lk.lock();
    for (Job* j : finished) {
        j->state = JOB_DONE;
        j->resolve = false;
        n_running_--;
        if (j->notify) completed_.push_back(j->id);
    }
    cv_done_.notify_all();
}

// Times the FISTA step kernel alone on one finished resident solve: `launches` back-to-back
// launches of the same kernel and grid the graph uses, bracketed by CUDA events on the engine
// stream.  Runs while the engine is idle (holds the engine lock); the solve's iterate is left
// scrambled, so it must be re-solved (bqp_resolve) before its result is used again.
int Engine::profile_step(uint64_t id, int launches, double* ms_out, double* bytes_out) {
    std::lock_guard<std::mutex> g(mu_);
    auto it = jobs_.find(id);
    if (it == jobs_.end()) return BQP_ERR_NOT_FOUND;
    Job& j = *it->second;
    if (j.state != JOB_DONE || !j.resident || n_running_ != 0 || !queue_.empty() || launches < 1) return BQP_ERR_NOT_READY;
    cudaSetDevice(device_);
    std::string why;
    update_grid();
    InstDev saved;
    cudaMemcpy(&saved, &d_inst_[j.slot], sizeof(InstDev), cudaMemcpyDeviceToHost);
    InstDev R = saved;
    R.status = ST_RUNNING;
    R.phase = PH_FISTA;
    R.it0 = 0;
    R.it_cur = 0;
    R.it_next = 1LL << 40;
    for (int k = 0; k < kMaxInterval; ++k) {
        R.beta[k] = 0.5;
        R.beta32[k] = 0.5f;
    }
    cudaMemcpyAsync(&d_inst_[j.slot], &R, sizeof(InstDev), cudaMemcpyHostToDevice, stream_);
    upload_tables();
    h_ctrl_->n_inst = n_inst_;
    h_ctrl_->n_tiles = static_cast<int32_t>(h_tiles_.size());
    h_ctrl_->n_units = static_cast<int32_t>(h_units_.size());
    std::memcpy(h_ctrl_->group_begin, group_begin_, sizeof(group_begin_));
    for (int k = 0; k < 3; ++k) h_ctrl_->step_due[k] = kMaxInterval;
    cudaMemcpyAsync(d_ctrl_, h_ctrl_, sizeof(Ctrl), cudaMemcpyHostToDevice, stream_);
    const View v = view();
    const int group = step_group(j.opt.precision, j.variant);
    auto step = [&] {
        if (group >= 0) launch_step_group(v, group, 0, graph_grid_, stream_);
        else launch_step_exact(v, 0, graph_grid_, stream_);
    };
    step();  // warm-up
    cudaEventRecord(ev0_, stream_);
    for (int k = 0; k < launches; ++k) step();
    cudaEventRecord(ev1_, stream_);
    cudaMemcpyAsync(&d_inst_[j.slot], &saved, sizeof(InstDev), cudaMemcpyHostToDevice, stream_);
    cudaError_t e = cudaStreamSynchronize(stream_);
    if (e != cudaSuccess) {
        set_error(std::string("CUDA: ") + cudaGetErrorString(e));
        return BQP_ERR_CUDA;
    }
    float ms = 0;
    cudaEventElapsedTime(&ms, ev0_, ev1_);
    if (ms_out) *ms_out = ms / launches;
    if (bytes_out) *bytes_out = algorithmic_bytes(j.n, j.nnz, j.opt.precision, 1, 0, 0.0);
    return BQP_OK;
}

// Re-runs the polish of a finished mixed-precision solve from its FP32 iterate (snap, residual and
// packing untimed), then times `iterations` CG iterations, the product kernel and the vector
// kernel separately, with CUDA events on the engine stream.  The CG tolerance is set below zero so
// every timed iteration does the whole work.  Bytes per launch: the device's per-iteration CG
// accounting split between the two kernels, on the round's packed Q_FF (ff_nnz entries, ff_rows
// free rows): product 12 ff_nnz + 52 ff_rows (Q_FF values and columns, row starts and counts,
// the free list, u gathered once, u, r, x read and w written per free row), vector 84 ff_rows.
int Engine::profile_cg(uint64_t id, int iterations, double* ms_matvec, double* ms_vector, double* bytes_matvec,
                       double* bytes_vector) {
    std::lock_guard<std::mutex> g(mu_);
    auto it = jobs_.find(id);
    if (it == jobs_.end()) return BQP_ERR_NOT_FOUND;
    Job& j = *it->second;
    if (j.state != JOB_DONE || !j.resident || n_running_ != 0 || !queue_.empty() || iterations < 1 ||
        j.opt.precision != PREC_MIXED)
        return BQP_ERR_NOT_READY;
    cudaSetDevice(device_);
    update_grid();
    InstDev saved;
    cudaMemcpy(&saved, &d_inst_[j.slot], sizeof(InstDev), cudaMemcpyDeviceToHost);
    if (!saved.polish || saved.result_src != 2) return BQP_ERR_NOT_READY;  // the solve did not end in a polish
    InstDev R = saved;
    R.status = ST_RUNNING;
    R.phase = PH_POLISH_INIT;
    R.cg_it = 0;
    R.cg_tol = -1.0;
    R.cg_max = 1LL << 40;
    R.ff_nnz = 0;
    R.ff_rows = 0;
    cudaMemcpyAsync(&d_inst_[j.slot], &R, sizeof(InstDev), cudaMemcpyHostToDevice, stream_);
    upload_tables();
    h_ctrl_->n_inst = n_inst_;
    h_ctrl_->n_tiles = static_cast<int32_t>(h_tiles_.size());
    h_ctrl_->n_units = static_cast<int32_t>(h_units_.size());
    h_ctrl_->n_cg = 1;
    cudaMemcpyAsync(d_ctrl_, h_ctrl_, sizeof(Ctrl), cudaMemcpyHostToDevice, stream_);
    const View v = view();
    const int grid = graph_grid_;
    launch_polish_init(v, grid, stream_);
    launch_polish_residual(v, grid, stream_);
    std::vector<cudaEvent_t> ev(static_cast<size_t>(2 * iterations + 1), nullptr);
    for (auto& e : ev) cudaEventCreate(&e);
    cudaEventRecord(ev[0], stream_);
    for (int k = 0; k < iterations; ++k) {
        launch_cg_matvec(v, grid, stream_);
        cudaEventRecord(ev[2 * k + 1], stream_);
        launch_cg_vector(v, grid, stream_);
        cudaEventRecord(ev[2 * k + 2], stream_);
    }
    InstDev after;
    cudaMemcpyAsync(&after, &d_inst_[j.slot], sizeof(InstDev), cudaMemcpyDeviceToHost, stream_);
    cudaMemcpyAsync(&d_inst_[j.slot], &saved, sizeof(InstDev), cudaMemcpyHostToDevice, stream_);
    cudaError_t e = cudaStreamSynchronize(stream_);
    double mv = 0, vec = 0;
    for (int k = 0; k < iterations && e == cudaSuccess; ++k) {
        float a = 0, b = 0;
        cudaEventElapsedTime(&a, ev[2 * k], ev[2 * k + 1]);
        cudaEventElapsedTime(&b, ev[2 * k + 1], ev[2 * k + 2]);
        mv += a;
        vec += b;
    }
    for (auto& x : ev) cudaEventDestroy(x);
    if (e != cudaSuccess) {
        set_error(std::string("CUDA: ") + cudaGetErrorString(e));
        return BQP_ERR_CUDA;
    }
    if (after.phase != PH_POLISH_CG || after.cg_it != iterations) {
        set_error("profile_cg: the CG iterations did not all run");
        return BQP_ERR_NOT_READY;
    }
    const double fz = static_cast<double>(after.ff_nnz), fr = static_cast<double>(after.ff_rows);
    if (ms_matvec) *ms_matvec = mv / iterations;
    if (ms_vector) *ms_vector = vec / iterations;
    // product: the packed entries (column, hi, lo); per free row its start and count, u, r and x
    // read, w written, and u's FP32 pair gathered once.  Vector step: p, u, s, w, r, x and the
    // preconditioner read, p, s, x, r, u and u's pair written.
    if (bytes_matvec) *bytes_matvec = 12.0 * fz + 48.0 * fr;
    if (bytes_vector) *bytes_vector = 104.0 * fr;
    return BQP_OK;
}

void Engine::loop() {
    cudaSetDevice(device_);
    std::unique_lock<std::mutex> lk(mu_);
    while (!stop_) {
        if (!pending_free_.empty()) process_frees();
        if (host_profile()) t_freed_ = host_seconds();
        // an upload paused when the last launch ended continues during the next launch; only
        // when there is nothing else to run is it completed here
        if (uploading_ && n_running_ == 0 && uploaded_.empty()) finish_paused_upload(lk);
        // admission: FIFO while the head fits under the cap; consecutive re-arms of resident
        // solves go together in one upload and one kernel
        bool admitted = false;
        size_t sync_bytes = 0;  // inputs uploaded by this thread since the last launch
        while (!queue_.empty()) {
            Job* j = queue_.front();
            if (j->resolve) {
                std::vector<Job*> batch;
                while (!queue_.empty() && queue_.front()->resolve) {
                    batch.push_back(queue_.front());
                    queue_.pop_front();
                }
                for (Job* b : batch) b->state = JOB_ADMITTING;
                lk.unlock();
                std::string why;
                const bool ok = rearm(batch, why);
                lk.lock();
                for (Job* b : batch) {
                    if (ok) {
                        b->state = JOB_RUNNING;
                        slot_job_[b->slot] = b;
                        n_running_++;
                    } else {
                        b->error = BQP_ERR_CUDA;
                        b->error_text = why;
                        b->state = JOB_DONE;
                        if (b->notify) completed_.push_back(b->id);
                    }
                }
                if (!ok) {
                    set_error(why);
                    cv_done_.notify_all();
                }
                admitted = true;
                continue;
            }
            if (uploading_) break;  // FIFO: the paused upload goes first
            const size_t need = make_layout(j->n, j->nnz, static_cast<int64_t>(j->tiles.size()), j->opt.precision).total;
            if (resident_bytes_ + need > cap_) {
                if (n_running_ == 0 && uploaded_.empty()) {
                    queue_.pop_front();
                    j->error = BQP_ERR_ADMISSION;
                    j->error_text = "solve does not fit under the device-memory cap";
                    j->state = JOB_DONE;
                    if (j->notify) completed_.push_back(j->id);
                    cv_done_.notify_all();
                    continue;
                }
                break;
            }
            const size_t input = static_cast<size_t>(j->nnz) * 12 + static_cast<size_t>(j->n) * 28 + 4;
            if ((sync_bytes > 0 || n_running_ > 0 || !uploaded_.empty()) && sync_bytes + input > kSyncUploadBudget)
                break;  // uploads during the next launch (upload_waiting)
            sync_bytes += input;
            queue_.pop_front();
            j->state = JOB_ADMITTING;
            resident_bytes_ += need;
            lk.unlock();
            std::string why;
            const bool ok = upload(*j, why);
            lk.lock();
            if (ok) uploaded_.push_back(j);
            else fail_admission(j, need, why);
        }
        // install what was uploaded here and during the previous launch
        if (!uploaded_.empty()) {
            std::vector<Job*> batch, refused;
            batch.swap(uploaded_);
            lk.unlock();
            std::string why;
            bool ok = gate_uploaded(batch, refused, why);
            if (host_profile()) t_gated_ = host_seconds();
            if (ok && !batch.empty()) ok = install(batch, why);
            if (host_profile()) t_installed_ = host_seconds();
            lk.lock();
            for (Job* j : refused) finish_refused(j);
            for (Job* j : batch) {
                if (ok) {
                    j->state = JOB_RUNNING;
                    slot_job_[j->slot] = j;
                    n_running_++;
                } else {
                    j->error = BQP_ERR_CUDA;
                    j->error_text = why;
                    j->state = JOB_DONE;
                    if (j->notify) completed_.push_back(j->id);
                }
            }
            if (!ok) {
                set_error(why);
                cv_done_.notify_all();
            }
            admitted = true;
        }
        if (admitted) {
            peak_resident_ = std::max(peak_resident_, n_running_);
            update_steps();
        }
        if (n_running_ == 0) {
            if (queue_.empty() && pending_free_.empty()) cv_work_.wait(lk);
            continue;
        }
        lk.unlock();
        std::string why;
        bool ok = run_once(why);
        lk.lock();
        if (!ok) {
            // A CUDA error on the engine stream: fail every running solve.
            set_error(why);
            for (Job* j : slot_job_) {
                if (j && j->state == JOB_RUNNING) {
                    j->state = JOB_DONE;
                    j->error = BQP_ERR_CUDA;
                    j->error_text = why;
                    n_running_--;
                    if (j->notify) completed_.push_back(j->id);
                }
            }
            cv_done_.notify_all();
            continue;
        }
        collect(lk);
        if (host_profile()) t_collected_ = host_seconds();
    }
}

}  // namespace bqp

// =============================================================================================
// C-ABI
// =============================================================================================
using bqp::Engine;
using bqp::Job;

struct bqp_ctx {
    Engine* engine;
};

namespace {
thread_local std::string g_error;

int validate_problem(int64_t n, int64_t nnz, const int32_t* rowptr, const int32_t* col, const double* val,
                     const double* c, const double* l, const double* u, const bqp_options* o, std::string& why) {
    if (n <= 0 || n > 2000000000LL || nnz < 0 || nnz > 2000000000LL || !rowptr || !c || !l || !u || (nnz && (!col || !val))) {
        why = "Invalid linear problem dimensions or offset";
        return BQP_ERR_INVALID;
    }
    if (!o || !(o->tolerance > 0) || !std::isfinite(o->tolerance) || o->time_limit < 0 || !std::isfinite(o->time_limit) ||
        o->iteration_limit < 0 || o->check_interval < 0 || o->check_interval > bqp::kMaxInterval ||
        (o->precision != BQP_PRECISION_FP64 && o->precision != BQP_PRECISION_MIXED && o->precision != BQP_PRECISION_FP64_EXACT) ||
        !std::isfinite(o->offset) || !(o->polish_switch >= 0) || !std::isfinite(o->polish_switch) ||
        (o->kernel_variant >= 0 && o->kernel_variant != 0 && o->kernel_variant != 64 && o->kernel_variant != 1 &&
         o->kernel_variant != 2 && o->kernel_variant != 4 && o->kernel_variant != 8 && o->kernel_variant != 16 &&
         o->kernel_variant != 32)) {
        why = "Invalid box QP options";
        return BQP_ERR_INVALID;
    }
    if (o->scaling < 0 || o->scaling > 2) {
        why = "Invalid box QP options";
        return BQP_ERR_INVALID;
    }
    if (o->lipschitz != BQP_LIPSCHITZ_GERSHGORIN && o->lipschitz != BQP_LIPSCHITZ_POWER) {
        why = "Invalid box QP options";
        return BQP_ERR_INVALID;
    }
    if (rowptr[0] != 0 || rowptr[n] != nnz) {
        why = "Invalid CSR row pointers";
        return BQP_ERR_INVALID;
    }
    return BQP_OK;
}

// One pass over the problem, split over host threads by row ranges: the reference's input checks
// (validate_linear_problem, src/mps.cpp:47-60, plus CSR sanity: every column index is checked
// before the upload, since the device uses it as a gather address), the positive-diagonal gate
// (src/qp_admm.cpp:72-78), infeasible bounds and whether any entry is non-zero (a zero Hessian
// goes to the reference's LP path).  Every row checks its own pointers before touching its
// entries.  The convexity gate and the Gershgorin bound are computed on the device at admission
// (convexity_gate_kernel).
// The submission's host scan reads the rows: row pointers, costs and bounds (validate_linear_problem,
// src/mps.cpp:47, comes first in solve_accelerated_box).  The Hessian's entries (column range,
// finite values, a zero Hessian, the diagonal pattern) are checked by the admission pass on the
// device, which reads them anyway; only a solve that finishes at submission (infeasible bounds)
// has them checked here (scan_hessian).
struct Scan {
    int error = 0;  // 1 row pointers, 2 coefficient/bound, 3 Hessian entry
    bool nonzero = false;
    bool infeasible = false;
};

// Destination of the host copy taken during the scan (asynchronous submit), or all null.
struct InputCopy {
    int32_t* rowptr = nullptr;
    int32_t* col = nullptr;
    double* val = nullptr;
    double* c = nullptr;
    double* l = nullptr;
    double* u = nullptr;
};

Scan scan_rows(int64_t r0, int64_t r1, int64_t n, int64_t nnz, const int32_t* rowptr, const int32_t* col, const double* val,
               const double* c, const double* l, const double* u, const InputCopy& dst) {
    Scan s;
    // the copy follows the scan in pieces of about 16K nonzeros, while they are still in cache:
    // the input is read from memory once
    int64_t copied = r0;
    auto copy_rows = [&](int64_t e) {
        const int64_t k0 = rowptr[copied], k1 = rowptr[e];
        std::memcpy(dst.rowptr + copied, rowptr + copied, sizeof(int32_t) * static_cast<size_t>(e - copied + (e == n ? 1 : 0)));
        std::memcpy(dst.col + k0, col + k0, sizeof(int32_t) * static_cast<size_t>(k1 - k0));
        std::memcpy(dst.val + k0, val + k0, sizeof(double) * static_cast<size_t>(k1 - k0));
        std::memcpy(dst.c + copied, c + copied, sizeof(double) * static_cast<size_t>(e - copied));
        std::memcpy(dst.l + copied, l + copied, sizeof(double) * static_cast<size_t>(e - copied));
        std::memcpy(dst.u + copied, u + copied, sizeof(double) * static_cast<size_t>(e - copied));
        copied = e;
    };
    for (int64_t i = r0; i < r1; ++i) {
        const int64_t a = rowptr[i], b = rowptr[i + 1];
        if (a < 0 || b < a || b > nnz) { s.error = 1; return s; }
        if (!std::isfinite(c[i]) || std::isnan(l[i]) || std::isnan(u[i]) || l[i] == HUGE_VAL || u[i] == -HUGE_VAL) {
            s.error = 2;
            return s;
        }
        if (l[i] > u[i]) s.infeasible = true;
        // rows [copied, i] validated: their nonzeros lie in [rowptr[copied], rowptr[i + 1]] within [0, nnz]
        if (dst.rowptr && (b - rowptr[copied] >= 16384 || i + 1 - copied >= 4096 || i + 1 == r1)) copy_rows(i + 1);
    }
    return s;
}

Scan scan_problem(int64_t n, int64_t nnz, const int32_t* rowptr, const int32_t* col, const double* val,
                  const double* c, const double* l, const double* u, const InputCopy& dst) {
    // pieces of about 128K nonzeros (by the average row), at least 2048 rows; below 256K
    // nonzeros the calling thread scans alone.  The result does not depend on the pieces: the
    // first error by row, and/or of the flags.
    const double avg = static_cast<double>(nnz) / static_cast<double>(n) + 1.0;
    const int64_t rows = std::max<int64_t>(2048, static_cast<int64_t>(131072.0 / avg));
    const int64_t pieces = nnz < 262144 ? 1 : (n + rows - 1) / rows;
    std::vector<Scan> part(static_cast<size_t>(pieces));
    bqp::WorkerPool::get().run(pieces, [&](int64_t p) {
        const int64_t r0 = n * p / pieces, r1 = n * (p + 1) / pieces;
        part[static_cast<size_t>(p)] = scan_rows(r0, r1, n, nnz, rowptr, col, val, c, l, u, dst);
    });
    Scan s;
    for (const Scan& p : part) {
        if (p.error && !s.error) s.error = p.error;
        s.infeasible = s.infeasible || p.infeasible;
    }
    return s;
}

// The Hessian entries' checks of the admission pass, on the host (rows already validated):
// error 3 for a column out of range or a value not finite, and whether some value is nonzero.
Scan scan_hessian(int64_t n, const int32_t* rowptr, const int32_t* col, const double* val) {
    const int64_t nnz = rowptr[n];
    const int64_t pieces = nnz < 262144 ? 1 : std::min<int64_t>(n, (nnz + 131071) / 131072);
    std::vector<Scan> part(static_cast<size_t>(pieces));
    bqp::WorkerPool::get().run(pieces, [&](int64_t p) {
        const int64_t r0 = n * p / pieces, r1 = n * (p + 1) / pieces;
        Scan& s = part[static_cast<size_t>(p)];
        for (int64_t k = rowptr[r0]; k < rowptr[r1]; ++k) {
            if (col[k] < 0 || col[k] >= n || !std::isfinite(val[k])) {
                s.error = 3;
                return;
            }
            if (val[k] != 0) s.nonzero = true;
        }
    });
    Scan s;
    for (const Scan& p : part) {
        if (p.error && !s.error) s.error = p.error;
        s.nonzero = s.nonzero || p.nonzero;
    }
    return s;
}

// Builds a job: validation, Gershgorin L, diagonal gate, tiles; infeasible bounds finish at once.
int make_job(int64_t n, int64_t nnz, const int32_t* rowptr, const int32_t* col, const double* val,
             const double* c, const double* l, const double* u, const bqp_options* options, bool copy,
             Job** out, std::string& why) {
    using bqp::host_seconds;
    using bqp::host_profile;
    using bqp::align_up;
    using bqp::HostBufferCache;
    const double t0 = host_seconds();
    bqp_options o;
    if (options) o = *options;
    else bqp_options_default(&o);
    int rc = validate_problem(n, nnz, rowptr, col, val, c, l, u, &o, why);
    if (rc != BQP_OK) return rc;
    std::unique_ptr<Job> j(new Job);
    InputCopy dst;
    if (copy) {
        // one cached host buffer: rowptr, col, val, c, l, u (64-byte aligned sections)
        const size_t N = static_cast<size_t>(n), Z = static_cast<size_t>(nnz);
        const size_t o_col = align_up((N + 1) * 4, 64), o_val = o_col + align_up(Z * 4, 64);
        const size_t o_c = o_val + align_up(Z * 8, 64), o_l = o_c + align_up(N * 8, 64), o_u = o_l + align_up(N * 8, 64);
        const size_t bytes = o_u + N * 8;
        j->own = HostBufferCache::get().acquire(bytes, &j->own_bytes);
        if (!j->own) {
            why = "host memory for the input copy";
            return BQP_ERR_NO_MEMORY;
        }
        dst.rowptr = reinterpret_cast<int32_t*>(j->own);
        dst.col = reinterpret_cast<int32_t*>(j->own + o_col);
        dst.val = reinterpret_cast<double*>(j->own + o_val);
        dst.c = reinterpret_cast<double*>(j->own + o_c);
        dst.l = reinterpret_cast<double*>(j->own + o_l);
        dst.u = reinterpret_cast<double*>(j->own + o_u);
    }
    const Scan scan = scan_problem(n, nnz, rowptr, col, val, c, l, u, dst);
    if (scan.error) {
        why = scan.error == 1 ? "Invalid CSR row pointers" : "Invalid variable coefficient or bound";
        return BQP_ERR_INVALID;
    }
    const double t_scan = host_seconds();
    if (nnz == 0) {  // the Gershgorin bound is zero (src/accelerated_qp.cpp:27-28)
        why = "Zero-Hessian models use the CPU LP path";
        return BQP_ERR_UNSUPPORTED;
    }
    // check_convex_hessian comes first, as in solve_accelerated_box (src/accelerated_qp.cpp:19).
    // The device decides it at admission (convexity_gate_kernel, with the host LDL^T only where
    // diagonal dominance fails), with the entries' validity and the zero-Hessian test.  A solve
    // with infeasible bounds finishes here without an admission, so it takes those on the host:
    // invalid entries, then a non-convex Hessian (unsupported_curvature), then a zero Hessian come
    // before infeasible_bounds, as in the reference.
    if (scan.infeasible) {
        const Scan hs = scan_hessian(n, rowptr, col, val);
        if (hs.error) {
            why = "Invalid Hessian";
            return BQP_ERR_INVALID;
        }
        if (!bqp::host_gate_convex(n, rowptr, col, val)) {
            j->n = n;
            j->nnz = nnz;
            j->opt = o;
            j->state = bqp::JOB_DONE;
            bqp::set_unsupported(j->stats);
            *out = j.release();
            return BQP_OK;
        }
        if (!hs.nonzero) {
            why = "Zero-Hessian models use the CPU LP path";
            return BQP_ERR_UNSUPPORTED;
        }
    }
    j->n = n;
    j->nnz = nnz;
    j->opt = o;
    // Engine defaults (0 = auto).  FP64 engines check every 25 iterations, the reference's
    // cadence.  The mixed engine checks only to find its polish point.  Where a FISTA step is
    // dear (rows of 8 or more nonzeros, bound by their random gathers, and 4M or more nonzeros)
    // it checks every 8 iterations (the first check after 12) with a polish switch at
    // stationarity 0.1; elsewhere a check costs several steps, and it checks every 25 with a
    // switch at 0.03.
    const bool dear_steps = o.precision == BQP_PRECISION_MIXED && nnz >= 8 * n && nnz >= 4000000;
    if (j->opt.check_interval == 0) j->opt.check_interval = dear_steps ? 8 : 25;
    if (j->opt.polish_switch == 0) j->opt.polish_switch = j->opt.check_interval <= 10 ? 0.1 : 3e-2;
    j->diag_gate = o.diagonal_gate >= 0 ? (o.diagonal_gate ? 1 : 0) : -1;
    if (scan.infeasible) {
        j->state = bqp::JOB_DONE;
        j->stats.status = BQP_STATUS_INFEASIBLE_BOUNDS;
        j->stats.objective = std::numeric_limits<double>::quiet_NaN();
        j->stats.primal_residual = j->stats.stationarity_residual = HUGE_VAL;
        j->stats.complementarity_residual = j->stats.relative_gap = HUGE_VAL;
        j->stats.dual_bound = -HUGE_VAL;
        *out = j.release();
        return BQP_OK;
    }
    if (o.precision == BQP_PRECISION_FP64_EXACT) j->variant = 1;
    else if (o.kernel_variant >= 0) j->variant = o.kernel_variant;
    else j->variant = bqp::default_variant(n, nnz, o.precision);
    j->tiles = bqp::make_tiles(n, rowptr, j->variant);
    const double t_tiles = host_seconds();
    if (copy) {
        j->rowptr = dst.rowptr; j->col = dst.col; j->val = dst.val; j->c = dst.c; j->l = dst.l; j->u = dst.u;
    } else {
        j->rowptr = rowptr; j->col = col; j->val = val; j->c = c; j->l = l; j->u = u;
    }
    if (host_profile())
        std::fprintf(stderr, "[boxqp] submit n=%lld: validate+scan %.3f ms, tiles %.3f ms, copy %.3f ms\n",
                     static_cast<long long>(n), 1e3 * (t_scan - t0), 1e3 * (t_tiles - t_scan),
                     1e3 * (host_seconds() - t_tiles));
    *out = j.release();
    return BQP_OK;
}

int fail(bqp_ctx* ctx, int rc, const std::string& why) {
    if (ctx) ctx->engine->set_error(why);
    g_error = why;
    return rc;
}
}  // namespace

extern "C" {

void bqp_options_default(bqp_options* o) {
    if (!o) return;
    o->tolerance = 1e-7;
    o->time_limit = 30;
    o->iteration_limit = 200000;
    o->precision = BQP_PRECISION_FP64;
    o->lipschitz = BQP_LIPSCHITZ_GERSHGORIN;
    o->check_interval = 0;
    o->diagonal_gate = -1;
    o->offset = 0;
    o->kernel_variant = -1;
    o->scaling = 0;
    o->polish_switch = 0;
}

bqp_ctx* bqp_create(int device, size_t mem_cap_bytes) {
    std::unique_ptr<Engine> e(new (std::nothrow) Engine(device, mem_cap_bytes));
    if (!e) {
        g_error = "out of host memory";
        return nullptr;
    }
    std::string why;
    if (!e->init(why)) {
        g_error = why;
        return nullptr;
    }
    bqp_ctx* ctx = new (std::nothrow) bqp_ctx;
    if (!ctx) {
        g_error = "out of host memory";
        return nullptr;
    }
    ctx->engine = e.release();
    return ctx;
}

void bqp_destroy(bqp_ctx* ctx) {
    if (!ctx) return;
    delete ctx->engine;
    delete ctx;
}

const char* bqp_last_error(const bqp_ctx* ctx) {
    if (!ctx) return g_error.c_str();
    return ctx->engine->error();
}

int bqp_host_register(void* ptr, size_t bytes) {
    if (!ptr || !bytes) return BQP_ERR_INVALID;
    const cudaError_t e = cudaHostRegister(ptr, bytes, cudaHostRegisterPortable);
    if (e != cudaSuccess) {
        cudaGetLastError();
        g_error = std::string("CUDA: host register: ") + cudaGetErrorString(e);
        return e == cudaErrorHostMemoryAlreadyRegistered ? BQP_ERR_INVALID : BQP_ERR_CUDA;
    }
    return BQP_OK;
}

int bqp_host_unregister(void* ptr) {
    if (!ptr) return BQP_ERR_INVALID;
    const cudaError_t e = cudaHostUnregister(ptr);
    if (e != cudaSuccess) {
        cudaGetLastError();
        g_error = std::string("CUDA: host unregister: ") + cudaGetErrorString(e);
        return BQP_ERR_INVALID;
    }
    return BQP_OK;
}

int bqp_device_name(int device, char* out, size_t cap) {
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        const char* msg = "No CUDA device available";
        if (out && cap) { std::strncpy(out, msg, cap - 1); out[cap - 1] = 0; }
        g_error = msg;
        return BQP_ERR_NO_DEVICE;
    }
    cudaDeviceProp p;
    if (device < 0 || device >= count || cudaGetDeviceProperties(&p, device) != cudaSuccess) {
        g_error = "Invalid CUDA device index";
        return BQP_ERR_INVALID;
    }
    if (out && cap) {
        std::strncpy(out, p.name, cap - 1);
        out[cap - 1] = 0;
    }
    return BQP_OK;
}

int bqp_submit(bqp_ctx* ctx, int64_t n, int64_t nnz, const int32_t* rowptr, const int32_t* col, const double* val,
               const double* c, const double* lower, const double* upper, const bqp_options* options, uint64_t* id) {
    if (!ctx) return fail(nullptr, BQP_ERR_INVALID, "null context");
    Job* j = nullptr;
    std::string why;
    int rc = make_job(n, nnz, rowptr, col, val, c, lower, upper, options, true, &j, why);
    if (rc != BQP_OK) return fail(ctx, rc, why);
    j->notify = true;
    return ctx->engine->submit(j, id);
}

int bqp_submit_borrowed(bqp_ctx* ctx, int64_t n, int64_t nnz, const int32_t* rowptr, const int32_t* col,
                        const double* val, const double* c, const double* lower, const double* upper,
                        const bqp_options* options, uint64_t* id) {
    if (!ctx) return fail(nullptr, BQP_ERR_INVALID, "null context");
    Job* j = nullptr;
    std::string why;
    int rc = make_job(n, nnz, rowptr, col, val, c, lower, upper, options, false, &j, why);
    if (rc != BQP_OK) return fail(ctx, rc, why);
    j->notify = true;
    return ctx->engine->submit(j, id);
}

int bqp_wait_any(bqp_ctx* ctx, double timeout_seconds, uint64_t* id) {
    if (!ctx || !id) return BQP_ERR_INVALID;
    return ctx->engine->wait_any(timeout_seconds, id);
}

int bqp_poll(bqp_ctx* ctx, uint64_t id, int32_t* status) {
    if (!ctx) return BQP_ERR_INVALID;
    return ctx->engine->poll(id, status);
}

int bqp_wait(bqp_ctx* ctx, uint64_t id, double timeout_seconds) {
    if (!ctx) return BQP_ERR_INVALID;
    return ctx->engine->wait(id, timeout_seconds);
}

int bqp_fetch(bqp_ctx* ctx, uint64_t id, double* x, bqp_stats* stats) {
    if (!ctx) return BQP_ERR_INVALID;
    return ctx->engine->fetch(id, x, stats);
}

int bqp_release(bqp_ctx* ctx, uint64_t id) {
    if (!ctx) return BQP_ERR_INVALID;
    return ctx->engine->release(id);
}

int bqp_resolve(bqp_ctx* ctx, const uint64_t* ids, int64_t count) {
    if (!ctx || (count > 0 && !ids) || count < 0) return BQP_ERR_INVALID;
    return ctx->engine->resolve(ids, count);
}

int bqp_set_latency_target(bqp_ctx* ctx, double ms) {
    if (!ctx || !(ms >= 0) || !std::isfinite(ms)) return BQP_ERR_INVALID;
    ctx->engine->set_latency_target(ms);
    return BQP_OK;
}

int bqp_inject_admission_oom(bqp_ctx* ctx, int32_t count) {
    if (!ctx || count < 0) return BQP_ERR_INVALID;
    ctx->engine->inject_admission_oom(count);
    return BQP_OK;
}

int bqp_timer(bqp_ctx* ctx, int32_t reset, double* device_ms, int64_t* kernels, int64_t* graph_launches) {
    if (!ctx) return BQP_ERR_INVALID;
    return ctx->engine->timer(reset, device_ms, kernels, graph_launches);
}

int bqp_profile_cg(bqp_ctx* ctx, uint64_t id, int32_t iterations, double* ms_matvec, double* ms_vector,
                   double* bytes_matvec, double* bytes_vector) {
    if (!ctx) return BQP_ERR_INVALID;
    return ctx->engine->profile_cg(id, iterations, ms_matvec, ms_vector, bytes_matvec, bytes_vector);
}

int bqp_profile_step(bqp_ctx* ctx, uint64_t id, int32_t launches, double* ms_per_launch, double* bytes_per_launch) {
    if (!ctx) return BQP_ERR_INVALID;
    return ctx->engine->profile_step(id, launches, ms_per_launch, bytes_per_launch);
}

int bqp_load(bqp_ctx* ctx, int64_t* queued, int64_t* running, int64_t* peak_resident, int64_t* resident_bytes) {
    if (!ctx) return BQP_ERR_INVALID;
    return ctx->engine->load(queued, running, peak_resident, resident_bytes);
}

int bqp_solve_sync(bqp_ctx* ctx, int64_t n, int64_t nnz, const int32_t* rowptr, const int32_t* col, const double* val,
                   const double* c, const double* lower, const double* upper, const bqp_options* options, double* x,
                   bqp_stats* stats) {
    if (!ctx) return fail(nullptr, BQP_ERR_INVALID, "null context");
    Job* j = nullptr;
    std::string why;
    int rc = make_job(n, nnz, rowptr, col, val, c, lower, upper, options, false, &j, why);
    if (rc != BQP_OK) return fail(ctx, rc, why);
    uint64_t id = 0;
    rc = ctx->engine->submit(j, &id);
    if (rc != BQP_OK) return rc;
    rc = ctx->engine->wait(id, -1);
    int frc = ctx->engine->fetch(id, x, stats);
    ctx->engine->release(id);
    return rc != BQP_OK ? rc : frc;
}

}  // extern "C"
