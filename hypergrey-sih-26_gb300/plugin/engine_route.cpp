// Engine route of the reference's C++ API: sovereign::solve_accelerated_box(q, opt, cuda = true)
// on the device-resident GB300 engine instead of the per-iteration BoxIteration plugin.
//
// The reference's CUDA backend (02-software/solver/src/accelerated_qp.cpp:36-48) launches two
// kernels per FISTA iteration through make_cuda_box and copies x back for a host check every 25
// iterations.  The one-line change that sends its cuda = true branch to the whole-solve engine is
//
//     if (cuda) return gb300::solve_box_on_device(q, opt);      // first line of the function
//
// This file implements that function over the C-ABI of libboxqp.so (bqp_solve_sync), and also
// provides it without editing the reference: linked with
//     -Wl,--wrap=_ZN9sovereign21solve_accelerated_boxERKNS_16QuadraticProblemERKNS_9QpOptionsEb
// every call of sovereign::solve_accelerated_box made from another object file (the JSON CLI,
// src/main.cpp:146, and the scale harness, src/scale_benchmark.cpp:20) lands in __wrap_ below,
// which routes cuda = true to the engine and everything else to the reference's own function
// (__real_).
//
// Behaviour kept from the reference (src/accelerated_qp.cpp:14-33): validate_linear_problem, the
// std::invalid_argument messages for rows, integer variables, bad options and a zero Hessian on
// CUDA, "unsupported_curvature" from the reference's own check_convex_hessian, and
// "infeasible_bounds".  The engine verifies with the reference's check_qp_solution measures on
// the device (FP64) and returns the same QpResult fields and status strings.  Precision of the
// iterations: BOXQP_PRECISION = fp64 | mixed | fp64_exact (default mixed: FP32 iterations, FP64
// verification and free-set polish; the result is still verified in FP64 at opt.tolerance).
#include "accelerated_qp.hpp"
#include "boxqp.h"

#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

namespace gb300 {

namespace {
std::mutex g_ctx_mu;
bqp_ctx* g_ctx = nullptr;

bqp_ctx* engine_context() {
    std::lock_guard<std::mutex> g(g_ctx_mu);
    if (!g_ctx) {
        g_ctx = bqp_create(0, 0);
        if (!g_ctx) {
            const std::string why = bqp_last_error(nullptr);
            if (why == "No CUDA device available") throw std::runtime_error(why);
            throw std::runtime_error("CUDA: " + why);
        }
    }
    return g_ctx;
}

int32_t precision_from_env() {
    const char* p = std::getenv("BOXQP_PRECISION");
    if (!p || !*p || std::strcmp(p, "mixed") == 0) return BQP_PRECISION_MIXED;
    if (std::strcmp(p, "fp64") == 0) return BQP_PRECISION_FP64;
    if (std::strcmp(p, "fp64_exact") == 0) return BQP_PRECISION_FP64_EXACT;
    throw std::invalid_argument("BOXQP_PRECISION must be fp64, mixed or fp64_exact");
}

const char* status_name(int32_t s) {
    switch (s) {
        case BQP_STATUS_OPTIMAL: return "optimal";
        case BQP_STATUS_ITERATION_LIMIT: return "iteration_limit";
        case BQP_STATUS_TIME_LIMIT: return "time_limit";
        case BQP_STATUS_NUMERICAL_ERROR: return "numerical_error";
        case BQP_STATUS_UNSUPPORTED_CURVATURE: return "unsupported_curvature";
        case BQP_STATUS_INFEASIBLE_BOUNDS: return "infeasible_bounds";
        default: return "numerical_error";
    }
}
}  // namespace

sovereign::QpResult solve_box_on_device(const sovereign::QuadraticProblem& q, const sovereign::QpOptions& opt) {
    const auto start = std::chrono::steady_clock::now();
    sovereign::validate_linear_problem(q.linear);
    if (!q.linear.rows.empty()) throw std::invalid_argument("Accelerated box QP requires box constraints only");
    for (bool v : q.linear.integer)
        if (v) throw std::invalid_argument("Accelerated box QP requires continuous variables");
    if (opt.tolerance <= 0 || !std::isfinite(opt.tolerance) || opt.time_limit < 0 || !std::isfinite(opt.time_limit) ||
        opt.threads < 1)
        throw std::invalid_argument("Invalid box QP options");
    sovereign::QpResult r;
    r.algorithm = "cuda_fista_box";
    if (!sovereign::check_convex_hessian(q)) {
        r.status = "unsupported_curvature";
        return r;
    }
    const auto& p = q.linear;
    const int64_t n = static_cast<int64_t>(p.cost.size());
    const double sign = p.maximize ? -1.0 : 1.0;
    const int64_t nh = static_cast<int64_t>(q.hessian.size());
    std::vector<int64_t> hrow(static_cast<size_t>(nh)), hcol(static_cast<size_t>(nh));
    std::vector<double> hval(static_cast<size_t>(nh));
    for (int64_t k = 0; k < nh; ++k) {
        hrow[k] = static_cast<int64_t>(q.hessian[k].row);
        hcol[k] = static_cast<int64_t>(q.hessian[k].col);
        hval[k] = q.hessian[k].value;
    }
    // Full symmetric CSR with the reference's merge (src/accelerated_qp.cpp:20-24).
    std::vector<int32_t> rowptr(static_cast<size_t>(n) + 1), col(static_cast<size_t>(2 * nh) + 1);
    std::vector<double> val(static_cast<size_t>(2 * nh) + 1);
    int64_t nnz = 0;
    if (bqp_csr_from_lower(n, nh, hrow.data(), hcol.data(), hval.data(), sign, rowptr.data(), col.data(), val.data(),
                           &nnz) != BQP_OK)
        throw std::invalid_argument("Invalid Hessian entry");
    if (bqp_gershgorin(n, rowptr.data(), val.data()) == 0)
        throw std::invalid_argument("Zero-Hessian models use the CPU LP path");
    for (int64_t j = 0; j < n; ++j)
        if (p.lower[j] > p.upper[j]) {
            r.status = "infeasible_bounds";
            return r;
        }
    std::vector<double> c(p.cost);
    for (double& v : c) v *= sign;
    bqp_options o;
    bqp_options_default(&o);
    o.tolerance = opt.tolerance;
    const double spent = std::chrono::duration<double>(std::chrono::steady_clock::now() - start).count();
    o.time_limit = opt.time_limit > spent ? opt.time_limit - spent : 0.0;
    o.iteration_limit = static_cast<int64_t>(opt.iteration_limit);
    o.precision = precision_from_env();
    o.offset = sign * p.offset;
    bqp_ctx* ctx = engine_context();
    std::vector<double> x(static_cast<size_t>(n));
    bqp_stats st;
    const int rc = bqp_solve_sync(ctx, n, nnz, rowptr.data(), col.data(), val.data(), c.data(), p.lower.data(),
                                  p.upper.data(), &o, x.data(), &st);
    if (rc == BQP_ERR_INVALID) throw std::invalid_argument(bqp_last_error(ctx));
    if (rc == BQP_ERR_NO_DEVICE) throw std::runtime_error("No CUDA device available");
    if (rc != BQP_OK) throw std::runtime_error(std::string("CUDA: ") + bqp_last_error(ctx));
    r.status = status_name(st.status);
    r.primal.swap(x);
    r.row_dual.clear();
    r.objective = sign * st.objective;
    r.primal_residual = st.primal_residual;
    r.stationarity_residual = st.stationarity_residual;
    r.complementarity_residual = st.complementarity_residual;
    r.iterations = static_cast<std::size_t>(st.iterations);
    r.dual_bound = st.dual_bound;
    r.relative_gap = st.relative_gap;
    r.optimality_verified = st.verified != 0;
    return r;
}

}  // namespace gb300

// The link-level form of the change (see the file comment): active only when the binary is
// linked with -Wl,--wrap for the mangled name of sovereign::solve_accelerated_box.
extern "C" {
sovereign::QpResult __real__ZN9sovereign21solve_accelerated_boxERKNS_16QuadraticProblemERKNS_9QpOptionsEb(
    const sovereign::QuadraticProblem& q, const sovereign::QpOptions& opt, bool cuda);

sovereign::QpResult __wrap__ZN9sovereign21solve_accelerated_boxERKNS_16QuadraticProblemERKNS_9QpOptionsEb(
    const sovereign::QuadraticProblem& q, const sovereign::QpOptions& opt, bool cuda) {
    if (cuda) return gb300::solve_box_on_device(q, opt);
    return __real__ZN9sovereign21solve_accelerated_boxERKNS_16QuadraticProblemERKNS_9QpOptionsEb(q, opt, cuda);
}
}
