// C shim over the reference's own C++ box-QP API (TEST INFRASTRUCTURE ONLY).
//
// Compiled by oracle/ref.mk together with the reference's unmodified solver sources
// into oracle/_ref/libsovereign_ref.so, so that Python tests and the golden-vector
// script can call the real reference engine through ctypes:
//   - sovereign::solve_accelerated_box(q, opt, false)   src/accelerated_qp.cpp:13-61
//   - sovereign::check_qp_solution(q, r, tol)           src/qp_admm.cpp:63-117
//   - sovereign::check_convex_hessian(q)                src/qp_admm.cpp:30-62
//   - sovereign::read_qplib(stream)                     src/qp.cpp:67-117
// No C++ exception crosses this boundary: errors come back as codes plus a message.
#include "accelerated_qp.hpp"
#include "qp.hpp"

#include <chrono>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <stdexcept>
#include <string>

namespace sovereign {
QpResult solve_diagonal_equalities(const QuadraticProblem&, const QpOptions&);
}

namespace {
void put_message(char* out, std::size_t cap, const std::string& text) {
    if (!out || !cap) return;
    std::size_t n = text.size() < cap - 1 ? text.size() : cap - 1;
    std::memcpy(out, text.data(), n);
    out[n] = 0;
}

sovereign::QuadraticProblem make_problem(int64_t n, int64_t nh, const int64_t* hrow, const int64_t* hcol,
                                         const double* hval, const double* cost, const double* lower,
                                         const double* upper, int maximize, double offset) {
    sovereign::QuadraticProblem q;
    auto& p = q.linear;
    p.name = "shim";
    p.names.resize(static_cast<std::size_t>(n));
    for (int64_t j = 0; j < n; ++j) p.names[j] = "x" + std::to_string(j);
    p.cost.assign(cost, cost + n);
    p.lower.assign(lower, lower + n);
    p.upper.assign(upper, upper + n);
    p.integer.assign(static_cast<std::size_t>(n), false);
    p.offset = offset;
    p.maximize = maximize != 0;
    q.hessian.reserve(static_cast<std::size_t>(nh));
    for (int64_t k = 0; k < nh; ++k)
        q.hessian.push_back({static_cast<std::size_t>(hrow[k]), static_cast<std::size_t>(hcol[k]), hval[k]});
    return q;
}

void fill_stats(const sovereign::QpResult& r, double* stats) {
    stats[0] = r.objective;
    stats[1] = r.primal_residual;
    stats[2] = r.stationarity_residual;
    stats[3] = r.complementarity_residual;
    stats[4] = r.dual_bound;
    stats[5] = r.relative_gap;
    stats[6] = r.optimality_verified ? 1.0 : 0.0;
    stats[7] = static_cast<double>(r.iterations);
}

struct QplibHandle {
    sovereign::QuadraticProblem q;
};

// Wall time of the last solve_accelerated_box call of ref_solve_box: the scope the reference's
// own scale harness times (src/scale_benchmark.cpp:20-21), without the shim's problem set-up.
thread_local double g_last_solve_seconds = 0;
}  // namespace

extern "C" {

double ref_last_solve_seconds() { return g_last_solve_seconds; }

// Runs the reference CPU engine.  status_out receives the reference's status string.
// Returns 0 on success, 1 if the reference threw std::invalid_argument, 2 for any
// other exception (message in status_out).
int ref_solve_box(int64_t n, int64_t nh, const int64_t* hrow, const int64_t* hcol, const double* hval,
                  const double* cost, const double* lower, const double* upper, int maximize, double offset,
                  double tol, int64_t iteration_limit, double time_limit, int threads,
                  double* x_out, double* stats, char* status_out, int status_cap) {
    try {
        auto q = make_problem(n, nh, hrow, hcol, hval, cost, lower, upper, maximize, offset);
        sovereign::QpOptions o;
        o.tolerance = tol;
        o.iteration_limit = static_cast<std::size_t>(iteration_limit);
        o.time_limit = time_limit;
        o.threads = threads;
        const auto start = std::chrono::steady_clock::now();
        auto r = sovereign::solve_accelerated_box(q, o, false);
        g_last_solve_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - start).count();
        fill_stats(r, stats);
        for (std::size_t j = 0; j < r.primal.size() && j < static_cast<std::size_t>(n); ++j) x_out[j] = r.primal[j];
        put_message(status_out, static_cast<std::size_t>(status_cap), r.status);
        return 0;
    } catch (const std::invalid_argument& e) {
        put_message(status_out, static_cast<std::size_t>(status_cap), e.what());
        return 1;
    } catch (const std::exception& e) {
        put_message(status_out, static_cast<std::size_t>(status_cap), e.what());
        return 2;
    }
}

// Runs the reference's ADMM (solve_qp_admm, src/qp_admm.cpp:118-280) on a QP with linear
// constraint rows row_lower <= A x <= row_upper (A in CSR, m rows) and bounds; x_out receives the
// primal.  Same returns as ref_solve_box.
int ref_solve_qp_admm(int64_t n, int64_t nh, const int64_t* hrow, const int64_t* hcol, const double* hval,
                      const double* cost, const double* lower, const double* upper, int64_t m,
                      const int32_t* a_rowptr, const int32_t* a_col, const double* a_val, const double* row_lower,
                      const double* row_upper, double tol, int64_t iteration_limit, double time_limit, int scaling,
                      int maximize, double offset, double* x_out, double* row_dual_out, double* stats,
                      char* status_out, int status_cap) {
    try {
        auto q = make_problem(n, nh, hrow, hcol, hval, cost, lower, upper, maximize, offset);
        auto& p = q.linear;
        p.rows.resize(static_cast<std::size_t>(m));
        for (int64_t i = 0; i < m; ++i)
            for (int32_t k = a_rowptr[i]; k < a_rowptr[i + 1]; ++k)
                p.rows[static_cast<std::size_t>(i)].push_back({static_cast<std::size_t>(a_col[k]), a_val[k]});
        p.row_lower.assign(row_lower, row_lower + m);
        p.row_upper.assign(row_upper, row_upper + m);
        sovereign::QpOptions o;
        o.tolerance = tol;
        o.iteration_limit = static_cast<std::size_t>(iteration_limit);
        o.time_limit = time_limit;
        o.threads = 1;
        o.scaling = scaling != 0;
        auto r = sovereign::solve_qp_admm(q, o);
        fill_stats(r, stats);
        for (std::size_t j = 0; j < r.primal.size() && j < static_cast<std::size_t>(n); ++j) x_out[j] = r.primal[j];
        if (row_dual_out)
            for (std::size_t i = 0; i < r.row_dual.size() && i < static_cast<std::size_t>(m); ++i)
                row_dual_out[i] = r.row_dual[i];
        put_message(status_out, static_cast<std::size_t>(status_cap), r.status);
        return 0;
    } catch (const std::invalid_argument& e) {
        put_message(status_out, static_cast<std::size_t>(status_cap), e.what());
        return 1;
    } catch (const std::exception& e) {
        put_message(status_out, static_cast<std::size_t>(status_cap), e.what());
        return 2;
    }
}

// Runs the reference's diagonal-Hessian equality solver (src/qp_dual_newton.cpp) alone, with the
// same options solve_qp_admm would pass it except the time limit.
int ref_solve_diagonal_equalities(int64_t n, int64_t nh, const int64_t* hrow, const int64_t* hcol, const double* hval,
                                  const double* cost, const double* lower, const double* upper, int64_t m,
                                  const int32_t* a_rowptr, const int32_t* a_col, const double* a_val,
                                  const double* row_lower, const double* row_upper, double tol, int64_t iteration_limit,
                                  int scaling, double* x_out, double* row_dual_out, double* stats, char* status_out,
                                  int status_cap) {
    try {
        auto q = make_problem(n, nh, hrow, hcol, hval, cost, lower, upper, 0, 0.0);
        auto& p = q.linear;
        p.rows.resize(static_cast<std::size_t>(m));
        for (int64_t i = 0; i < m; ++i)
            for (int32_t k = a_rowptr[i]; k < a_rowptr[i + 1]; ++k)
                p.rows[static_cast<std::size_t>(i)].push_back({static_cast<std::size_t>(a_col[k]), a_val[k]});
        p.row_lower.assign(row_lower, row_lower + m);
        p.row_upper.assign(row_upper, row_upper + m);
        sovereign::QpOptions o;
        o.tolerance = tol;
        o.iteration_limit = static_cast<std::size_t>(iteration_limit);
        o.time_limit = 600;
        o.threads = 1;
        o.scaling = scaling != 0;
        auto r = sovereign::solve_diagonal_equalities(q, o);
        fill_stats(r, stats);
        for (std::size_t j = 0; j < r.primal.size() && j < static_cast<std::size_t>(n); ++j) x_out[j] = r.primal[j];
        for (std::size_t i = 0; i < r.row_dual.size() && i < static_cast<std::size_t>(m); ++i)
            row_dual_out[i] = r.row_dual[i];
        put_message(status_out, static_cast<std::size_t>(status_cap), r.status);
        return 0;
    } catch (const std::exception& e) {
        put_message(status_out, static_cast<std::size_t>(status_cap), e.what());
        return 2;
    }
}

// Runs the reference checker on a caller-supplied primal and row duals of a problem with linear
// rows (A in CSR, row_lower <= A x <= row_upper).
int ref_check_rows(int64_t n, int64_t nh, const int64_t* hrow, const int64_t* hcol, const double* hval,
                   const double* cost, const double* lower, const double* upper, int maximize, double offset,
                   int64_t m, const int32_t* a_rowptr, const int32_t* a_col, const double* a_val,
                   const double* row_lower, const double* row_upper, const double* x, const double* row_dual,
                   double tol, double* stats) {
    try {
        auto q = make_problem(n, nh, hrow, hcol, hval, cost, lower, upper, maximize, offset);
        auto& p = q.linear;
        p.rows.resize(static_cast<std::size_t>(m));
        for (int64_t i = 0; i < m; ++i)
            for (int32_t k = a_rowptr[i]; k < a_rowptr[i + 1]; ++k)
                p.rows[static_cast<std::size_t>(i)].push_back({static_cast<std::size_t>(a_col[k]), a_val[k]});
        p.row_lower.assign(row_lower, row_lower + m);
        p.row_upper.assign(row_upper, row_upper + m);
        sovereign::QpResult r;
        r.primal.assign(x, x + n);
        r.row_dual.assign(row_dual, row_dual + m);
        sovereign::check_qp_solution(q, r, tol);
        fill_stats(r, stats);
        return 0;
    } catch (...) {
        return 2;
    }
}

// Runs the reference checker on a caller-supplied primal.
int ref_check(int64_t n, int64_t nh, const int64_t* hrow, const int64_t* hcol, const double* hval,
              const double* cost, const double* lower, const double* upper, int maximize, double offset,
              const double* x, double tol, double* stats) {
    try {
        auto q = make_problem(n, nh, hrow, hcol, hval, cost, lower, upper, maximize, offset);
        sovereign::QpResult r;
        r.primal.assign(x, x + n);
        sovereign::check_qp_solution(q, r, tol);
        fill_stats(r, stats);
        return 0;
    } catch (...) {
        return 2;
    }
}

// 1 convex, 0 not convex, -2 invalid Hessian (the reference throws invalid_argument).
int ref_check_convex(int64_t n, int64_t nh, const int64_t* hrow, const int64_t* hcol, const double* hval, int maximize) {
    try {
        std::vector<double> zero(static_cast<std::size_t>(n), 0.0);
        auto q = make_problem(n, nh, hrow, hcol, hval, zero.data(), zero.data(), zero.data(), maximize, 0.0);
        return sovereign::check_convex_hessian(q) ? 1 : 0;
    } catch (...) {
        return -2;
    }
}

// QPLIB reading through the reference parser: open, query sizes, copy, close.
void* ref_qplib_open(const char* path, char* message, int cap) {
    try {
        std::ifstream in(path);
        if (!in) throw std::runtime_error("Cannot open model");
        auto* h = new QplibHandle;
        h->q = sovereign::read_qplib(in);
        return h;
    } catch (const std::exception& e) {
        put_message(message, static_cast<std::size_t>(cap), e.what());
        return nullptr;
    }
}

void ref_qplib_sizes(void* handle, int64_t* n, int64_t* nh, int64_t* m, int* maximize, double* offset) {
    auto* h = static_cast<QplibHandle*>(handle);
    *n = static_cast<int64_t>(h->q.linear.cost.size());
    *nh = static_cast<int64_t>(h->q.hessian.size());
    *m = static_cast<int64_t>(h->q.linear.rows.size());
    *maximize = h->q.linear.maximize ? 1 : 0;
    *offset = h->q.linear.offset;
}

void ref_qplib_copy(void* handle, int64_t* hrow, int64_t* hcol, double* hval, double* cost, double* lower, double* upper) {
    auto* h = static_cast<QplibHandle*>(handle);
    for (std::size_t k = 0; k < h->q.hessian.size(); ++k) {
        hrow[k] = static_cast<int64_t>(h->q.hessian[k].row);
        hcol[k] = static_cast<int64_t>(h->q.hessian[k].col);
        hval[k] = h->q.hessian[k].value;
    }
    const auto& p = h->q.linear;
    for (std::size_t j = 0; j < p.cost.size(); ++j) {
        cost[j] = p.cost[j];
        lower[j] = p.lower[j];
        upper[j] = p.upper[j];
    }
}

// The rows of a model read by ref_qplib_open: CSR in the reader's order (row by row, each row's
// entries as the file listed them) and the row bounds.
void ref_qplib_rows(void* handle, int32_t* rowptr, int32_t* col, double* val, double* row_lower, double* row_upper) {
    auto* h = static_cast<QplibHandle*>(handle);
    const auto& p = h->q.linear;
    int32_t k = 0;
    rowptr[0] = 0;
    for (std::size_t i = 0; i < p.rows.size(); ++i) {
        for (const auto& e : p.rows[i]) {
            col[k] = static_cast<int32_t>(e.first);
            val[k] = e.second;
            ++k;
        }
        rowptr[i + 1] = k;
        row_lower[i] = p.row_lower[i];
        row_upper[i] = p.row_upper[i];
    }
}

int64_t ref_qplib_row_entries(void* handle) {
    int64_t k = 0;
    for (const auto& r : static_cast<QplibHandle*>(handle)->q.linear.rows) k += static_cast<int64_t>(r.size());
    return k;
}

void ref_qplib_close(void* handle) { delete static_cast<QplibHandle*>(handle); }

}  // extern "C"
