/* TEST INFRASTRUCTURE ONLY: the reference's own CUDA plugin on this GPU.
 *
 * The reference's CUDA backend (02-software/solver/src/cuda_box.cu) is two kernels,
 * csr_product (:16-18, one thread per row) and fista_step (:19-21, clamp + momentum with
 * step = 1/L), driven by solve_accelerated_box (src/accelerated_qp.cpp:36-57): two launches
 * per iteration on the default stream, and every 25 iterations a synchronous copy of x to the
 * host and the host check (src/qp_admm.cpp:63-117, restated as orc_check in boxqp_oracle.c).
 * oracle/ref.mk compiles cuda_box.cu unmodified, where it lies in the reference checkout, into
 * oracle/_ref/cuda_box_sm103a.cubin; this harness loads that module through the CUDA driver API
 * and runs the same loop, so the reference's GPU path can be timed beside the engine on the
 * same instance.  It is only run by the benchmark's reference arm.
 */
#include <cuda.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

typedef struct {
    double objective;
    double primal_residual;
    double stationarity_residual;
    double complementarity_residual;
    double dual_bound;
    double relative_gap;
    double verified;
    double iterations;
} orc_stats;

void orc_check(int64_t n, int64_t nh, const int64_t* hrow, const int64_t* hcol, const double* hval,
               const double* cost, const double* lower, const double* upper, int maximize, double offset,
               const double* x, double tol, orc_stats* r);
double orc_max_abs_row_sum(int64_t n, const int32_t* rowptr, const double* val);

static double wall_seconds(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

#define HCHECK(call)                                                                   \
    do {                                                                               \
        CUresult rc_ = (call);                                                         \
        if (rc_ != CUDA_SUCCESS) {                                                     \
            const char* s_ = NULL;                                                     \
            cuGetErrorString(rc_, &s_);                                                \
            snprintf(err, (size_t)errlen, "%s: %s", #call, s_ ? s_ : "CUDA error");  \
            goto done;                                                                 \
        }                                                                              \
    } while (0)

/* status: 0 optimal, 1 iteration_limit, 2 time_limit, 3 numerical_error (as the reference);
 * seconds[0] = whole solve (uploads, loop, checks), seconds[1] = the iteration loop alone. */
int ref_cuda_solve(const char* cubin_path, int64_t n, const int32_t* rowptr, const int32_t* col, const double* val,
                   int64_t nh, const int64_t* hrow, const int64_t* hcol, const double* hval, const double* cost,
                   const double* lower, const double* upper, double tol, int64_t iteration_limit,
                   double time_limit, double* x_out, orc_stats* r, int* status, double* seconds, char* err,
                   int errlen) {
    int ok = -1;
    CUdevice dev;
    CUcontext ctx = NULL;
    CUmodule mod = NULL;
    CUfunction product = NULL, step_fn = NULL;
    CUdeviceptr d_start = 0, d_col = 0, d_val = 0, d_c = 0, d_lo = 0, d_up = 0, d_x = 0, d_w = 0, d_g = 0;
    const int64_t nnz = rowptr[n];
    double* x = (double*)malloc(sizeof(double) * (size_t)n);
    err[0] = 0;
    if (!x) {
        snprintf(err, (size_t)errlen, "host memory");
        return -1;
    }
    const double t_start = wall_seconds();
    HCHECK(cuInit(0));
    HCHECK(cuDeviceGet(&dev, 0));
    HCHECK(cuDevicePrimaryCtxRetain(&ctx, dev));
    HCHECK(cuCtxSetCurrent(ctx));
    HCHECK(cuModuleLoad(&mod, cubin_path));
    {
        unsigned int count = 0;
        HCHECK(cuModuleGetFunctionCount(&count, mod));
        CUfunction fns[16];
        if (count > 16) count = 16;
        HCHECK(cuModuleEnumerateFunctions(fns, count, mod));
        for (unsigned int k = 0; k < count; ++k) {
            const char* name = NULL;
            HCHECK(cuFuncGetName(&name, fns[k]));
            if (name && strstr(name, "csr_product")) product = fns[k];
            if (name && strstr(name, "fista_step")) step_fn = fns[k];
        }
        if (!product || !step_fn) {
            snprintf(err, (size_t)errlen, "kernels not found in %s", cubin_path);
            goto done;
        }
    }
    /* CudaBox's DeviceArray uploads (synchronous cudaMemcpy) */
    HCHECK(cuMemAlloc(&d_start, sizeof(int32_t) * (size_t)(n + 1)));
    HCHECK(cuMemAlloc(&d_col, sizeof(int32_t) * (size_t)(nnz > 0 ? nnz : 1)));
    HCHECK(cuMemAlloc(&d_val, sizeof(double) * (size_t)(nnz > 0 ? nnz : 1)));
    HCHECK(cuMemAlloc(&d_c, sizeof(double) * (size_t)n));
    HCHECK(cuMemAlloc(&d_lo, sizeof(double) * (size_t)n));
    HCHECK(cuMemAlloc(&d_up, sizeof(double) * (size_t)n));
    HCHECK(cuMemAlloc(&d_x, sizeof(double) * (size_t)n));
    HCHECK(cuMemAlloc(&d_w, sizeof(double) * (size_t)n));
    HCHECK(cuMemAlloc(&d_g, sizeof(double) * (size_t)n));
    const double lipschitz = orc_max_abs_row_sum(n, rowptr, val);
    if (lipschitz == 0) {
        snprintf(err, (size_t)errlen, "zero Hessian");
        goto done;
    }
    for (int64_t j = 0; j < n; ++j) {
        const double lo = lower[j], up = upper[j];
        x[j] = (lo < ((0.0 < up) ? 0.0 : up)) ? ((0.0 < up) ? 0.0 : up) : lo; /* max(lo, min(up, 0)) */
    }
    HCHECK(cuMemcpyHtoD(d_start, rowptr, sizeof(int32_t) * (size_t)(n + 1)));
    if (nnz) HCHECK(cuMemcpyHtoD(d_col, col, sizeof(int32_t) * (size_t)nnz));
    if (nnz) HCHECK(cuMemcpyHtoD(d_val, val, sizeof(double) * (size_t)nnz));
    HCHECK(cuMemcpyHtoD(d_c, cost, sizeof(double) * (size_t)n));
    HCHECK(cuMemcpyHtoD(d_lo, lower, sizeof(double) * (size_t)n));
    HCHECK(cuMemcpyHtoD(d_up, upper, sizeof(double) * (size_t)n));
    HCHECK(cuMemcpyHtoD(d_x, x, sizeof(double) * (size_t)n));
    HCHECK(cuMemcpyHtoD(d_w, x, sizeof(double) * (size_t)n));
    {
        const double t_loop = wall_seconds();
        const int ni = (int)n;
        const unsigned grid = (unsigned)((n + 255) / 256);
        const double stepsize = 1 / lipschitz;
        double t = 1;
        *status = 1;
        memset(r, 0, sizeof(*r));
        for (int64_t iteration = 0; iteration <= iteration_limit; ++iteration) {
            if (iteration % 25 == 0 || iteration == iteration_limit) {
                HCHECK(cuMemcpyDtoH(x, d_x, sizeof(double) * (size_t)n)); /* primal(): synchronous copy */
                orc_check(n, nh, hrow, hcol, hval, cost, lower, upper, 0, 0.0, x, tol, r);
                r->iterations = (double)iteration;
                if (r->verified != 0) { *status = 0; break; }
                if (!isfinite(r->objective) || !isfinite(r->stationarity_residual)) { *status = 3; break; }
                if (wall_seconds() - t_start >= time_limit) { *status = 2; break; }
            }
            if (iteration == iteration_limit) break;
            const double next_t = (1 + sqrt(1 + 4 * t * t)) / 2, beta = (t - 1) / next_t;
            t = next_t;
            void* pa[] = {(void*)&ni, &d_start, &d_col, &d_val, &d_w, &d_g};
            HCHECK(cuLaunchKernel(product, grid, 1, 1, 256, 1, 1, 0, NULL, pa, NULL));
            void* pb[] = {(void*)&ni, &d_x, &d_w, &d_g, &d_c, &d_lo, &d_up, (void*)&stepsize, &beta};
            HCHECK(cuLaunchKernel(step_fn, grid, 1, 1, 256, 1, 1, 0, NULL, pb, NULL));
        }
        seconds[1] = wall_seconds() - t_loop;
    }
    memcpy(x_out, x, sizeof(double) * (size_t)n);
    seconds[0] = wall_seconds() - t_start;
    ok = 0;
done:
    if (d_start) cuMemFree(d_start);
    if (d_col) cuMemFree(d_col);
    if (d_val) cuMemFree(d_val);
    if (d_c) cuMemFree(d_c);
    if (d_lo) cuMemFree(d_lo);
    if (d_up) cuMemFree(d_up);
    if (d_x) cuMemFree(d_x);
    if (d_w) cuMemFree(d_w);
    if (d_g) cuMemFree(d_g);
    if (mod) cuModuleUnload(mod);
    if (ctx) cuDevicePrimaryCtxRelease(dev);
    free(x);
    return ok;
}
