/*
 * CPU oracle for the box-constrained convex QP path (TEST INFRASTRUCTURE ONLY).
 *
 * This file is a plain-C restatement of the reference's FP64 box-QP engine and of
 * its original-model checker.  It exists to check the CUDA engine: only the tests,
 * the smoke check and the CPU-baseline leg of the benchmark load it.  The product
 * library never links or calls it, and nothing here runs on the GPU.
 *
 * Reference anchors (paths inside the reference project, 02-software/solver/):
 *   - solve_accelerated_box ........ src/accelerated_qp.cpp:13-61
 *   - CsrMatrix(n, rows) ........... include/sparse_matrix.hpp:10-17
 *   - CsrMatrix::multiply .......... include/sparse_matrix.hpp:26-33
 *   - check_convex_hessian ......... src/qp_admm.cpp:30-62
 *   - check_qp_solution ............ src/qp_admm.cpp:63-117
 *   - original_violation ........... src/mps.cpp:279-303
 *   - validate_linear_problem ...... src/mps.cpp:47-60
 *
 * Floating-point contract: compile with -ffp-contract=off so that every product and
 * sum is rounded separately, as the reference's x86-64 build does; the sums over a
 * CSR row run in ascending column order from 0.0, as CsrMatrix::multiply does.
 * Long-double accumulators follow the reference (80-bit on x86-64, binary128 on
 * aarch64; the last bits of the objective may therefore differ between the two).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_OK 0
#define ORC_INVALID_ARGUMENT 1
#define ORC_NO_MEMORY 2

/* Status codes shared with the engine's C-ABI (see include/boxqp.h). */
enum {
    ORC_STATUS_OPTIMAL = 0,
    ORC_STATUS_ITERATION_LIMIT = 1,
    ORC_STATUS_TIME_LIMIT = 2,
    ORC_STATUS_NUMERICAL_ERROR = 3,
    ORC_STATUS_UNSUPPORTED_CURVATURE = 4,
    ORC_STATUS_INFEASIBLE_BOUNDS = 5,
    ORC_STATUS_ZERO_HESSIAN = 6 /* the reference hands these to its LP engine */
};

/* Result record in the order of QpResult's residual fields (include/qp.hpp:11-22). */
typedef struct {
    double objective;
    double primal_residual;
    double stationarity_residual;
    double complementarity_residual;
    double dual_bound;
    double relative_gap;
    double verified;   /* 1.0 or 0.0 */
    double iterations;
} orc_stats;

static double orc_inf(void) { return HUGE_VAL; }

/* std::max / std::min semantics: max(a,b) = a<b ? b : a ; min(a,b) = b<a ? b : a. */
static inline double smax(double a, double b) { return (a < b) ? b : a; }
static inline double smin(double a, double b) { return (b < a) ? b : a; }
static inline double sclip(double x, double lo, double up) { return smax(lo, smin(up, x)); }

static double now_seconds(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

/* validate_linear_problem for a box-only, continuous problem (src/mps.cpp:47-60). */
int orc_validate_box(int64_t n, const double* cost, const double* lower, const double* upper, double offset) {
    if (n <= 0 || !isfinite(offset)) return ORC_INVALID_ARGUMENT;
    for (int64_t j = 0; j < n; ++j) {
        if (!isfinite(cost[j]) || isnan(lower[j]) || isnan(upper[j]) || lower[j] == HUGE_VAL || upper[j] == -HUGE_VAL)
            return ORC_INVALID_ARGUMENT;
    }
    return ORC_OK;
}

/* original_violation(p, x, scaled=true) for a problem with no rows (src/mps.cpp:279-303). */
double orc_original_violation(int64_t n, const double* lower, const double* upper, const double* x) {
    double result = 0;
    for (int64_t j = 0; j < n; ++j) {
        if (!isfinite(x[j])) return orc_inf();
        long double ax = fabsl((long double)x[j]);
        if (isfinite(lower[j])) {
            long double v = (long double)lower[j] - (long double)x[j];
            v /= 1 + fabsl((long double)lower[j]) + ax;
            result = smax(result, (double)v);
        }
        if (isfinite(upper[j])) {
            long double v = (long double)x[j] - (long double)upper[j];
            v /= 1 + fabsl((long double)upper[j]) + ax;
            result = smax(result, (double)v);
        }
    }
    return result;
}

/* ---------------------------------------------------------------------------------
 * CSR assembly: mirror the lower-triangle triplets into per-row lists in triplet
 * order (src/accelerated_qp.cpp:23), then merge each row by ascending column,
 * summing duplicates in insertion order and dropping exact zeros
 * (include/sparse_matrix.hpp:10-17).
 * Output capacity: rowptr[n+1], col/val[2*nh].  Returns nnz, or -1 on bad input.
 * ------------------------------------------------------------------------------- */
typedef struct { int64_t col; int64_t seq; double val; } orc_entry;

static int entry_cmp(const void* a, const void* b) {
    const orc_entry* x = (const orc_entry*)a;
    const orc_entry* y = (const orc_entry*)b;
    if (x->col != y->col) return x->col < y->col ? -1 : 1;
    if (x->seq != y->seq) return x->seq < y->seq ? -1 : 1;
    return 0;
}

int64_t orc_build_csr(int64_t n, int64_t nh, const int64_t* hrow, const int64_t* hcol, const double* hval,
                      double sign, int32_t* rowptr, int32_t* col, double* val) {
    int64_t* count = (int64_t*)calloc((size_t)n + 1, sizeof(int64_t));
    if (!count) return -1;
    for (int64_t k = 0; k < nh; ++k) {
        if (hrow[k] < 0 || hrow[k] >= n || hcol[k] < 0 || hcol[k] >= n) { free(count); return -1; }
        count[hrow[k] + 1]++;
        if (hrow[k] != hcol[k]) count[hcol[k] + 1]++;
    }
    for (int64_t i = 0; i < n; ++i) count[i + 1] += count[i];
    int64_t total = count[n];
    orc_entry* e = (orc_entry*)malloc(sizeof(orc_entry) * (size_t)(total ? total : 1));
    int64_t* fill = (int64_t*)malloc(sizeof(int64_t) * (size_t)n);
    if (!e || !fill) { free(count); free(e); free(fill); return -1; }
    memcpy(fill, count, sizeof(int64_t) * (size_t)n);
    int64_t seq = 0;
    for (int64_t k = 0; k < nh; ++k) {
        double v = sign * hval[k];
        orc_entry a = {hcol[k], seq++, v};
        e[fill[hrow[k]]++] = a;
        if (hrow[k] != hcol[k]) {
            orc_entry b = {hrow[k], seq++, v};
            e[fill[hcol[k]]++] = b;
        }
    }
    int64_t nnz = 0;
    rowptr[0] = 0;
    for (int64_t i = 0; i < n; ++i) {
        int64_t b = count[i], t = count[i + 1];
        if (t - b > 1) qsort(e + b, (size_t)(t - b), sizeof(orc_entry), entry_cmp);
        int64_t k = b;
        while (k < t) {
            int64_t c = e[k].col;
            double s = 0.0;
            while (k < t && e[k].col == c) { s += e[k].val; ++k; }
            if (s != 0) { col[nnz] = (int32_t)c; val[nnz] = s; ++nnz; }
        }
        if (nnz > 2000000000LL) { free(count); free(e); free(fill); return -1; }
        rowptr[i + 1] = (int32_t)nnz;
    }
    free(count); free(e); free(fill);
    return nnz;
}

/* CsrMatrix::multiply: y_i = sum_k value_k * x[index_k], row order, from 0.0. */
void orc_csr_multiply(int64_t n, const int32_t* rowptr, const int32_t* col, const double* val,
                      const double* x, double* y, int threads) {
#ifdef _OPENMP
#pragma omp parallel for num_threads(threads) if (threads > 1 && n > 2000) schedule(static)
#endif
    for (long long i = 0; i < (long long)n; ++i) {
        double sum = 0;
        for (int32_t k = rowptr[i]; k < rowptr[i + 1]; ++k) sum += val[k] * x[col[k]];
        y[i] = sum;
    }
    (void)threads;
}

/* Gershgorin bound used as the Lipschitz constant (src/accelerated_qp.cpp:25-26). */
double orc_max_abs_row_sum(int64_t n, const int32_t* rowptr, const double* val) {
    double lipschitz = 0;
    for (int64_t i = 0; i < n; ++i) {
        double sum = 0;
        for (int32_t k = rowptr[i]; k < rowptr[i + 1]; ++k) sum += fabs(val[k]);
        lipschitz = smax(lipschitz, sum);
    }
    return lipschitz;
}

/* ---------------------------------------------------------------------------------
 * check_convex_hessian (src/qp_admm.cpp:30-62): diagonal dominance with a
 * non-negative diagonal proves PSD; otherwise a congruence-scaled LDL^T with full
 * fill decides.  The oracle restates the LDL^T fallback densely and therefore
 * limits it to n <= 4096 (returns -1 above that); every planted family in the
 * tests is diagonally dominant and never reaches it.
 * Returns 1 (convex), 0 (not convex), -1 (oracle limit), -2 (invalid input).
 * ------------------------------------------------------------------------------- */
int orc_check_convex(int64_t n, int64_t nh, const int64_t* hrow, const int64_t* hcol, const double* hval, int maximize) {
    double sign = maximize ? -1.0 : 1.0;
    double* diagonal = (double*)calloc((size_t)n, sizeof(double));
    double* radius = (double*)calloc((size_t)n, sizeof(double));
    if (!diagonal || !radius) { free(diagonal); free(radius); return -2; }
    for (int64_t k = 0; k < nh; ++k) {
        if (hrow[k] < 0 || hrow[k] >= n || hcol[k] < 0 || hcol[k] >= n || !isfinite(hval[k])) {
            free(diagonal); free(radius); return -2;
        }
        if (hrow[k] == hcol[k]) diagonal[hrow[k]] += sign * hval[k];
        else { radius[hrow[k]] += fabs(hval[k]); radius[hcol[k]] += fabs(hval[k]); }
    }
    int dd = 1;
    for (int64_t j = 0; j < n; ++j) {
        if (diagonal[j] < 0 || (diagonal[j] == 0 && radius[j] > 0)) { free(diagonal); free(radius); return 0; }
        if (diagonal[j] < radius[j]) dd = 0;
    }
    if (dd) { free(diagonal); free(radius); return 1; }
    if (n > 4096) { free(diagonal); free(radius); return -1; }
    /* Dense lower-triangular store: a[i*n + j] holds entry (i, j) with i >= j
       (the reference keeps lower[j][i], i >= j). */
    double* a = (double*)calloc((size_t)(n * n), sizeof(double));
    unsigned char* present = (unsigned char*)calloc((size_t)(n * n), 1);
    if (!a || !present) { free(a); free(present); free(diagonal); free(radius); return -2; }
    for (int64_t k = 0; k < nh; ++k) {
        int64_t i = hrow[k] > hcol[k] ? hrow[k] : hcol[k];
        int64_t j = hrow[k] > hcol[k] ? hcol[k] : hrow[k];
        if (diagonal[i] > 0 && diagonal[j] > 0) {
            a[i * n + j] += sign * hval[k] / sqrt(diagonal[i] * diagonal[j]);
            present[i * n + j] = 1;
        }
    }
    int64_t fill = nh;
    int result = 1;
    for (int64_t k = 0; k < n && result; ++k) {
        double d = present[k * n + k] ? a[k * n + k] : 0;
        if (d < -1e-12) { result = 0; break; }
        if (d <= 1e-12) {
            for (int64_t i = k + 1; i < n; ++i)
                if (present[i * n + k] && fabs(a[i * n + k]) > 1e-10) { result = 0; break; }
            continue;
        }
        for (int64_t u = k + 1; u < n && result; ++u) {
            if (!present[u * n + k]) continue;
            for (int64_t v = u; v < n; ++v) {
                if (!present[v * n + k]) continue;
                /* The reference updates lower[i][j] with i = off[u], j = off[v], i <= j. */
                int64_t i = u, j = v;
                if (!present[j * n + i]) {
                    if (++fill > 4000000) { result = 0; break; }
                    present[j * n + i] = 1;
                }
                a[j * n + i] -= a[u * n + k] * a[v * n + k] / d;
            }
        }
        for (int64_t i = k; i < n; ++i) present[i * n + k] = 0;
    }
    free(a); free(present); free(diagonal); free(radius);
    return result;
}

/* ---------------------------------------------------------------------------------
 * check_qp_solution for a box-only problem (src/qp_admm.cpp:63-117).
 * ------------------------------------------------------------------------------- */
void orc_check(int64_t n, int64_t nh, const int64_t* hrow, const int64_t* hcol, const double* hval,
               const double* cost, const double* lower, const double* upper, int maximize, double offset,
               const double* x, double tol, orc_stats* r) {
    double sign = maximize ? -1.0 : 1.0;
    r->verified = 0;
    r->objective = NAN;
    r->dual_bound = -orc_inf();
    r->primal_residual = r->stationarity_residual = r->complementarity_residual = r->relative_gap = orc_inf();
    for (int64_t j = 0; j < n; ++j) if (!isfinite(x[j])) return;
    double* gradient = (double*)calloc((size_t)n, sizeof(double));
    if (!gradient) return;
    long double value = sign * offset;
    int positive_diagonal = 1;
    for (int64_t k = 0; k < nh; ++k) {
        int64_t i = hrow[k], j = hcol[k];
        gradient[i] += sign * hval[k] * x[j];
        if (i != j) {
            gradient[j] += sign * hval[k] * x[i];
            if (hval[k] != 0) positive_diagonal = 0;
        }
    }
    long double* diagonal = NULL;
    long double* linear = NULL;
    if (positive_diagonal) {
        diagonal = (long double*)calloc((size_t)n, sizeof(long double));
        for (int64_t k = 0; k < nh; ++k) if (hrow[k] == hcol[k]) diagonal[hrow[k]] += sign * hval[k];
        for (int64_t j = 0; j < n; ++j) if (!(diagonal[j] > 0)) positive_diagonal = 0;
        if (positive_diagonal) {
            linear = (long double*)malloc(sizeof(long double) * (size_t)n);
            for (int64_t j = 0; j < n; ++j) linear[j] = sign * cost[j];
        }
    }
    for (int64_t j = 0; j < n; ++j) {
        value += .5L * x[j] * gradient[j] + sign * cost[j] * x[j];
        gradient[j] += sign * cost[j];
    }
    r->objective = sign * (double)value;
    r->primal_residual = orc_original_violation(n, lower, upper, x);
    r->complementarity_residual = 0;
    long double bound = value, dual_constant = sign * offset;
    r->stationarity_residual = 0;
    for (int64_t j = 0; j < n; ++j) {
        const double g = gradient[j];
        double residual = fabs(x[j] - sclip(x[j] - g, lower[j], upper[j])) / (1 + fabs(x[j]));
        if (!isfinite(g) || !isfinite(residual)) residual = orc_inf();
        r->stationarity_residual = smax(r->stationarity_residual, residual);
        if (g != 0) {
            double target = g > 0 ? lower[j] : upper[j];
            if (isfinite(target)) bound += g * (target - x[j]);
            else bound = -HUGE_VALL;
        }
    }
    if (positive_diagonal) {
        bound = dual_constant;
        for (int64_t j = 0; j < n; ++j) {
            long double m = -linear[j] / diagonal[j];
            long double lo = (long double)lower[j], up = (long double)upper[j];
            long double inner = (m < up) ? m : up;          /* std::min(upper, m) */
            long double minimizer = (lo < inner) ? inner : lo; /* std::max(lower, .) */
            bound += .5L * diagonal[j] * minimizer * minimizer + linear[j] * minimizer;
        }
    }
    r->dual_bound = (double)bound;
    r->relative_gap = isfinite(bound) ? (double)(fabsl(value - bound) / (1 + fabsl(value))) : orc_inf();
    double worst = smax(r->primal_residual, smax(r->stationarity_residual, r->complementarity_residual));
    int ok = isfinite(r->objective) && worst <= tol;
    if (positive_diagonal) ok = ok && r->relative_gap <= tol;
    r->verified = ok ? 1.0 : 0.0;
    free(gradient); free(diagonal); free(linear);
}

/* ---------------------------------------------------------------------------------
 * FISTA steps on an assembled CSR (the CPU branch of src/accelerated_qp.cpp:50-57):
 *   next = max(l, min(u, w - (H w + c) / L)); w = next + beta (next - x); x = next
 * with beta_k = (t_k - 1)/t_{k+1}, t_{k+1} = (1 + sqrt(1 + 4 t_k^2))/2, t_0 = 1.
 * Runs steps for iterations [it_begin, it_end) starting from state (x, w, *t).
 * ------------------------------------------------------------------------------- */
void orc_fista_steps(int64_t n, const int32_t* rowptr, const int32_t* col, const double* val,
                     const double* c, const double* lower, const double* upper, double lipschitz,
                     double* x, double* w, double* t, int64_t steps, int threads) {
    double* gradient = (double*)malloc(sizeof(double) * (size_t)n);
    if (!gradient) return;
    for (int64_t s = 0; s < steps; ++s) {
        double next_t = (1 + sqrt(1 + 4 * (*t) * (*t))) / 2, beta = (*t - 1) / next_t;
        *t = next_t;
        orc_csr_multiply(n, rowptr, col, val, w, gradient, threads);
#ifdef _OPENMP
#pragma omp parallel for num_threads(threads) if (threads > 1 && n > 2000) schedule(static)
#endif
        for (long long j = 0; j < (long long)n; ++j) {
            double next = smax(lower[j], smin(upper[j], w[j] - (gradient[j] + c[j]) / lipschitz));
            w[j] = next + beta * (next - x[j]);
            x[j] = next;
        }
    }
    free(gradient);
}

/* ---------------------------------------------------------------------------------
 * solve_accelerated_box(q, opt, cuda=false) (src/accelerated_qp.cpp:13-61), for a
 * box-only continuous problem given by lower-triangle triplets.
 * On return: status code, x (n), stats (objective ... iterations).
 * Returns ORC_OK or ORC_INVALID_ARGUMENT (the reference throws invalid_argument).
 * ------------------------------------------------------------------------------- */
int orc_solve_box(int64_t n, int64_t nh, const int64_t* hrow, const int64_t* hcol, const double* hval,
                  const double* cost, const double* lower, const double* upper, int maximize, double offset,
                  double tol, int64_t iteration_limit, double time_limit, int threads,
                  double* x_out, orc_stats* r, int* status) {
    double start = now_seconds();
    if (orc_validate_box(n, cost, lower, upper, offset) != ORC_OK) return ORC_INVALID_ARGUMENT;
    if (tol <= 0 || !isfinite(tol) || time_limit < 0 || !isfinite(time_limit) || threads < 1 || iteration_limit < 0)
        return ORC_INVALID_ARGUMENT;
    memset(r, 0, sizeof(*r));
    r->objective = NAN;
    r->primal_residual = r->stationarity_residual = r->complementarity_residual = r->relative_gap = orc_inf();
    r->dual_bound = -orc_inf();
    int convex = orc_check_convex(n, nh, hrow, hcol, hval, maximize);
    if (convex == -2) return ORC_INVALID_ARGUMENT;
    if (convex != 1) { *status = ORC_STATUS_UNSUPPORTED_CURVATURE; return ORC_OK; }
    double sign = maximize ? -1.0 : 1.0;
    int32_t* rowptr = (int32_t*)malloc(sizeof(int32_t) * (size_t)(n + 1));
    int32_t* col = (int32_t*)malloc(sizeof(int32_t) * (size_t)(2 * nh + 1));
    double* val = (double*)malloc(sizeof(double) * (size_t)(2 * nh + 1));
    double* c = (double*)malloc(sizeof(double) * (size_t)n);
    double* x = (double*)malloc(sizeof(double) * (size_t)n);
    double* w = (double*)malloc(sizeof(double) * (size_t)n);
    if (!rowptr || !col || !val || !c || !x || !w) {
        free(rowptr); free(col); free(val); free(c); free(x); free(w);
        return ORC_NO_MEMORY;
    }
    for (int64_t j = 0; j < n; ++j) c[j] = cost[j] * sign;
    int64_t nnz = orc_build_csr(n, nh, hrow, hcol, hval, sign, rowptr, col, val);
    (void)nnz;
    double lipschitz = orc_max_abs_row_sum(n, rowptr, val);
    if (lipschitz == 0) {
        *status = ORC_STATUS_ZERO_HESSIAN;
        free(rowptr); free(col); free(val); free(c); free(x); free(w);
        return ORC_OK;
    }
    for (int64_t j = 0; j < n; ++j) {
        if (lower[j] > upper[j]) {
            *status = ORC_STATUS_INFEASIBLE_BOUNDS;
            free(rowptr); free(col); free(val); free(c); free(x); free(w);
            return ORC_OK;
        }
        x[j] = smax(lower[j], smin(upper[j], 0.0));
    }
    memcpy(w, x, sizeof(double) * (size_t)n);
    double t = 1;
    *status = ORC_STATUS_ITERATION_LIMIT;
    for (int64_t iteration = 0; iteration <= iteration_limit; ++iteration) {
        r->iterations = (double)iteration;
        if (iteration % 25 == 0 || iteration == iteration_limit) {
            orc_check(n, nh, hrow, hcol, hval, cost, lower, upper, maximize, offset, x, tol, r);
            r->iterations = (double)iteration;
            if (r->verified != 0) { *status = ORC_STATUS_OPTIMAL; break; }
            if (!isfinite(r->objective) || !isfinite(r->stationarity_residual)) { *status = ORC_STATUS_NUMERICAL_ERROR; break; }
            if (now_seconds() - start >= time_limit) { *status = ORC_STATUS_TIME_LIMIT; break; }
        }
        if (iteration == iteration_limit) break;
        orc_fista_steps(n, rowptr, col, val, c, lower, upper, lipschitz, x, w, &t, 1, threads);
    }
    memcpy(x_out, x, sizeof(double) * (size_t)n);
    free(rowptr); free(col); free(val); free(c); free(x); free(w);
    return ORC_OK;
}

/* Same loop on an already assembled full CSR (used when the caller holds the CSR and
   the lower triplets together, e.g. the planted generator's output).  The check still
   runs on the lower triplets exactly as check_qp_solution does. */
int orc_solve_box_csr(int64_t n, const int32_t* rowptr, const int32_t* col, const double* val,
                      int64_t nh, const int64_t* hrow, const int64_t* hcol, const double* hval,
                      const double* cost, const double* lower, const double* upper,
                      double tol, int64_t iteration_limit, double time_limit, int threads,
                      double* x_out, orc_stats* r, int* status) {
    double start = now_seconds();
    memset(r, 0, sizeof(*r));
    double lipschitz = orc_max_abs_row_sum(n, rowptr, val);
    if (lipschitz == 0) { *status = ORC_STATUS_ZERO_HESSIAN; return ORC_OK; }
    double* x = (double*)malloc(sizeof(double) * (size_t)n);
    double* w = (double*)malloc(sizeof(double) * (size_t)n);
    if (!x || !w) { free(x); free(w); return ORC_NO_MEMORY; }
    for (int64_t j = 0; j < n; ++j) {
        if (lower[j] > upper[j]) { *status = ORC_STATUS_INFEASIBLE_BOUNDS; free(x); free(w); return ORC_OK; }
        x[j] = smax(lower[j], smin(upper[j], 0.0));
    }
    memcpy(w, x, sizeof(double) * (size_t)n);
    double t = 1;
    *status = ORC_STATUS_ITERATION_LIMIT;
    for (int64_t iteration = 0; iteration <= iteration_limit; ++iteration) {
        r->iterations = (double)iteration;
        if (iteration % 25 == 0 || iteration == iteration_limit) {
            orc_check(n, nh, hrow, hcol, hval, cost, lower, upper, 0, 0.0, x, tol, r);
            r->iterations = (double)iteration;
            if (r->verified != 0) { *status = ORC_STATUS_OPTIMAL; break; }
            if (!isfinite(r->objective) || !isfinite(r->stationarity_residual)) { *status = ORC_STATUS_NUMERICAL_ERROR; break; }
            if (now_seconds() - start >= time_limit) { *status = ORC_STATUS_TIME_LIMIT; break; }
        }
        if (iteration == iteration_limit) break;
        orc_fista_steps(n, rowptr, col, val, cost, lower, upper, lipschitz, x, w, &t, 1, threads);
    }
    memcpy(x_out, x, sizeof(double) * (size_t)n);
    free(x); free(w);
    return ORC_OK;
}

int orc_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
