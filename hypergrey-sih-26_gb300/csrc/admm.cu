// Constrained-QP ADMM inner solve on the GPU: the linear system of the reference's ADMM x-update
// (02-software/solver/src/qp_admm.cpp:157-161)
//     K x = rhs,   K = H + sigma I + A' diag(rho) A
// with H (n x n) and A (m x n) resident in CSR (A' built once, by a stable transpose), solved by
// the reference's Jacobi-preconditioned CG (qp_admm.cpp:262-273): r = rhs - K x, pre = r / M,
// d = pre, then while inner < max_inner and max|r| > accuracy: alpha = r'pre / d'K d (stop when
// that denominator is not positive and finite), x += alpha d, r -= alpha K d, beta = new r'pre /
// old, d = pre + beta d.  M = diag(H) + sigma + sum_i rho_i a_ij^2 as qp_admm.cpp:153-156 forms it
// (same order of additions, no FMA contraction: the same bits).
//
// One CUDA graph per system: the set-up kernels, then a WHILE node over one CG iteration (A d,
// then H d + sigma d + A'(rho A d) with the partial sums of d'K d, then the vector updates with
// the partial sums of r'pre and the maximum of |r|, then the new direction); the last block of
// each reduction finalizes it in a fixed order and sets the loop condition, so a solve is one
// graph launch with no host round trip per iteration.  FP64 throughout (the reference's inner
// products; its long double dot accumulation is not reproduced, so iterates agree to rounding).
#include "boxqp.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <new>
#include <string>
#include <vector>

namespace {

constexpr int kB = 256;
constexpr int kLanes = 4;         // lanes per CSR row
constexpr int kRows = kB / kLanes;
constexpr int kMaxBlocks = 152 * 4;

struct AdmmState {
    double rz, alpha, beta;
    double accuracy;
    unsigned long long rmax;  // max |r| as the bit pattern of a non-negative double
    long long max_inner;
    long long inner;
    long long inner_sum;      // inner iterations over the ADMM iterations of one bqp_admm_iterate call
    unsigned ticket;
    int stop;                 // a non-positive or non-finite d'K d ended the loop
};

__device__ __forceinline__ unsigned long long umax64(unsigned long long a, unsigned long long b) { return a < b ? b : a; }
__device__ __forceinline__ unsigned long long dbits(double v) {
    return static_cast<unsigned long long>(__double_as_longlong(v));
}

// y = M v for rows [0, rows) of a CSR matrix, kLanes lanes per row in a fixed order; returns the
// row sum in the group's lane 0 (valid for r < rows).
__device__ __forceinline__ double csr_row(const int32_t* __restrict__ rp, const int32_t* __restrict__ ci,
                                          const double* __restrict__ va, const double* __restrict__ v, int r, int rows,
                                          int sl) {
    double s = 0;
    if (r < rows) {
        const int ks = __ldg(rp + r), ke = __ldg(rp + r + 1);
        for (int k = ks + sl; k < ke; k += kLanes) s = fma(__ldg(va + k), v[__ldg(ci + k)], s);
    }
#pragma unroll
    for (int o = kLanes / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    return s;
}

// Fixed-order block sums of two doubles and a maximum; the last block (ticket) adds the block
// partials, all its threads strided over them and then the same fixed tree, and returns true in
// its thread 0 with the grid totals.
__device__ __forceinline__ void block_tree(double& a, double& b, unsigned long long& mx, double* ra, double* rb,
                                           unsigned long long* rm) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
        mx = umax64(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
        ra[warp] = a;
        rb[warp] = b;
        rm[warp] = mx;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        a = 0;
        b = 0;
        mx = 0;
        for (int w = 0; w < kB / 32; ++w) {
            a += ra[w];
            b += rb[w];
            mx = umax64(mx, rm[w]);
        }
    }
}

__device__ bool reduce_last(double a, double b, unsigned long long mx, double* partial, AdmmState* st, double* ta,
                            double* tb, unsigned long long* tm) {
    __shared__ double ra[kB / 32], rb[kB / 32];
    __shared__ unsigned long long rm[kB / 32];
    __shared__ int last;
    block_tree(a, b, mx, ra, rb, rm);
    if (threadIdx.x == 0) {
        partial[3 * blockIdx.x] = a;
        partial[3 * blockIdx.x + 1] = b;
        partial[3 * blockIdx.x + 2] = __longlong_as_double(static_cast<long long>(mx));
        __threadfence();
        last = atomicAdd(&st->ticket, 1u) == gridDim.x - 1 ? 1 : 0;
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    double sa = 0, sb = 0;
    unsigned long long sm = 0;
    for (unsigned k = threadIdx.x; k < gridDim.x; k += kB) {
        sa += __ldcg(partial + 3 * k);
        sb += __ldcg(partial + 3 * k + 1);
        sm = umax64(sm, dbits(__ldcg(partial + 3 * k + 2)));
    }
    block_tree(sa, sb, sm, ra, rb, rm);  // thread 0 read the first tree's ra/rb/rm before the barrier above
    if (threadIdx.x != 0) return false;
    st->ticket = 0;
    *ta = sa;
    *tb = sb;
    *tm = sm;
    return true;
}

struct Sys {
    int n, m;
    const int32_t *hrp, *hci, *arp, *aci, *trp, *tci;
    const double *hva, *ava, *tva;
    const double* rho;
    double sigma;
    const double* precond;
    double* t;      // rho .* (A v), m
};

// t = rho .* (A v)
__global__ void __launch_bounds__(kB) admm_a_kernel(Sys s, const double* __restrict__ v, const AdmmState* st) {
    if (st->stop) return;
    const int sl = threadIdx.x % kLanes;
    for (int base = blockIdx.x * kRows; base < s.m; base += gridDim.x * kRows) {
        const int r = base + static_cast<int>(threadIdx.x) / kLanes;
        const double y = csr_row(s.arp, s.aci, s.ava, v, r, s.m, sl);
        if (r < s.m && sl == 0) s.t[r] = s.rho[r] * y;
    }
}

// out = H v + sigma v + A' t, then by mode:
//   0 (apply): nothing more;
//   1 (set-up, v = x): r = rhs - out, pre = r / M, d = pre; rz = r'pre, max|r|; the loop runs while
//     max_inner > 0 and max|r| > accuracy;
//   2 (iteration, v = d): d'out -> alpha = rz / d'out, or stop.
__global__ void __launch_bounds__(kB) admm_k_kernel(Sys s, const double* __restrict__ v, double* __restrict__ out,
                                                    int mode, const double* __restrict__ rhs, double* __restrict__ r,
                                                    double* __restrict__ pre, double* __restrict__ d, double* partial,
                                                    AdmmState* st, cudaGraphConditionalHandle loop) {
    if (mode == 2 && st->stop) return;
    const int sl = threadIdx.x % kLanes;
    double acc_a = 0, acc_b = 0;
    unsigned long long acc_m = 0;
    for (int base = blockIdx.x * kRows; base < s.n; base += gridDim.x * kRows) {
        const int j = base + static_cast<int>(threadIdx.x) / kLanes;
        const double hv = csr_row(s.hrp, s.hci, s.hva, v, j, s.n, sl);
        const double at = csr_row(s.trp, s.tci, s.tva, s.t, j, s.n, sl);
        if (j < s.n && sl == 0) {
            // the reference's expression, output[j] += sigma v[j] + product[j], unfused
            const double o = __dadd_rn(hv, __dadd_rn(__dmul_rn(s.sigma, v[j]), at));
            out[j] = o;
            if (mode == 1) {
                const double rr = __dsub_rn(rhs[j], o);
                const double pp = __ddiv_rn(rr, s.precond[j]);
                r[j] = rr;
                pre[j] = pp;
                d[j] = pp;
                acc_a = fma(rr, pp, acc_a);
                acc_m = umax64(acc_m, dbits(fabs(rr)));
            } else if (mode == 2) {
                acc_a = fma(v[j], o, acc_a);
            }
        }
    }
    if (mode == 0) return;
    double ta, tb;
    unsigned long long tm;
    if (!reduce_last(acc_a, acc_b, acc_m, partial, st, &ta, &tb, &tm)) return;
    if (mode == 1) {
        st->rz = ta;
        st->rmax = tm;
        st->inner = 0;
        st->stop = 0;
        cudaGraphSetConditional(loop, (st->max_inner > 0 && __longlong_as_double(static_cast<long long>(tm)) > st->accuracy) ? 1u : 0u);
    } else {
        if (!(ta > 0) || !isfinite(ta)) st->stop = 1;
        else st->alpha = st->rz / ta;
    }
}

// x += alpha d, r -= alpha K d, pre = r / M; then rz, beta and the loop condition
__global__ void __launch_bounds__(kB) admm_update_kernel(Sys s, double* __restrict__ x, double* __restrict__ r,
                                                         double* __restrict__ pre, const double* __restrict__ d,
                                                         const double* __restrict__ kd, double* partial, AdmmState* st,
                                                         cudaGraphConditionalHandle loop) {
    if (st->stop) {
        if (blockIdx.x == 0 && threadIdx.x == 0) cudaGraphSetConditional(loop, 0u);
        return;
    }
    const double alpha = st->alpha;
    double acc_a = 0;
    unsigned long long acc_m = 0;
    for (int j = blockIdx.x * kB + threadIdx.x; j < s.n; j += gridDim.x * kB) {
        x[j] = __dadd_rn(x[j], __dmul_rn(alpha, d[j]));
        const double rr = __dsub_rn(r[j], __dmul_rn(alpha, kd[j]));
        const double pp = __ddiv_rn(rr, s.precond[j]);
        r[j] = rr;
        pre[j] = pp;
        acc_a = fma(rr, pp, acc_a);
        acc_m = umax64(acc_m, dbits(fabs(rr)));
    }
    double ta, tb;
    unsigned long long tm;
    if (!reduce_last(acc_a, 0.0, acc_m, partial, st, &ta, &tb, &tm)) return;
    st->beta = ta / st->rz;
    st->rz = ta;
    st->rmax = tm;
    st->inner += 1;
    cudaGraphSetConditional(loop, (st->inner < st->max_inner && __longlong_as_double(static_cast<long long>(tm)) > st->accuracy) ? 1u : 0u);
}

// d = pre + beta d
__global__ void __launch_bounds__(kB) admm_direction_kernel(int n, double* __restrict__ d, const double* __restrict__ pre,
                                                            const AdmmState* st) {
    if (st->stop) return;
    const double beta = st->beta;
    for (int j = blockIdx.x * kB + threadIdx.x; j < n; j += gridDim.x * kB) d[j] = __dadd_rn(pre[j], __dmul_rn(beta, d[j]));
}

// M = diag(H) + sigma + sum_i rho_i a_ij^2, row j of A' in increasing i (the reference's order)
__global__ void __launch_bounds__(kB) admm_precond_kernel(Sys s, double* __restrict__ precond) {
    for (int j = blockIdx.x * kB + threadIdx.x; j < s.n; j += gridDim.x * kB) {
        double dg = 0;
        for (int k = s.hrp[j]; k < s.hrp[j + 1]; ++k)
            if (s.hci[k] == j) dg = s.hva[k];
        double p = __dadd_rn(dg, s.sigma);
        for (int k = s.trp[j]; k < s.trp[j + 1]; ++k) {
            const double a = s.tva[k];
            p = __dadd_rn(p, __dmul_rn(__dmul_rn(s.rho[s.tci[k]], a), a));
        }
        precond[j] = p;
    }
}

// ---- the ADMM iteration around the inner solve (qp_admm.cpp:255-279) --------------------------
// rhs = A'(rho z - y) + (sigma x - c); the inner accuracy min(1e-7, .05 / (it+1)^1.6) (1 + max|rhs|)
// and the inner iteration cap go to the state the inner solve's set-up reads; x0 of the inner
// solve = x.
__global__ void __launch_bounds__(kB) admm_rhs_kernel(Sys s, const double* __restrict__ z, const double* __restrict__ y,
                                                      const double* __restrict__ xa, const double* __restrict__ c,
                                                      double* __restrict__ rhs, double* __restrict__ x0, double* partial,
                                                      AdmmState* st, double iteration_factor) {
    const int sl = threadIdx.x % kLanes;
    unsigned long long mx = 0;
    for (int base = blockIdx.x * kRows; base < s.n; base += gridDim.x * kRows) {
        const int j = base + static_cast<int>(threadIdx.x) / kLanes;
        double acc = 0;
        if (j < s.n) {
            const int ks = __ldg(s.trp + j), ke = __ldg(s.trp + j + 1);
            for (int k = ks + sl; k < ke; k += kLanes) {
                const int i = __ldg(s.tci + k);
                const double yz = __dsub_rn(__dmul_rn(s.rho[i], z[i]), y[i]);  // the reference's yz[i]
                acc = fma(__ldg(s.tva + k), yz, acc);
            }
        }
#pragma unroll
        for (int o = kLanes / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (j < s.n && sl == 0) {
            const double v = __dadd_rn(acc, __dsub_rn(__dmul_rn(s.sigma, xa[j]), c[j]));
            rhs[j] = v;
            x0[j] = xa[j];
            mx = umax64(mx, dbits(fabs(v)));
        }
    }
    double ta, tb;
    unsigned long long tm;
    if (!reduce_last(0.0, 0.0, mx, partial, st, &ta, &tb, &tm)) return;
    const double rmax = __longlong_as_double(static_cast<long long>(tm));
    st->accuracy = __dmul_rn(iteration_factor, __dadd_rn(1.0, rmax));
    st->max_inner = s.n * 2LL + 20 < 4000 ? s.n * 2LL + 20 : 4000;
    st->stop = 0;  // a breakdown of the previous inner solve does not carry over
}

// ax = A next; relaxed = 1.6 ax - .6 z; z+ = clip(relaxed + y / rho, lo, up); y += rho (relaxed - z+)
__global__ void __launch_bounds__(kB) admm_zy_kernel(Sys s, const double* __restrict__ next, double* __restrict__ z,
                                                     double* __restrict__ y, const double* __restrict__ lo,
                                                     const double* __restrict__ up, AdmmState* st) {
    if (blockIdx.x == 0 && threadIdx.x == 0) st->inner_sum += st->inner;
    const int sl = threadIdx.x % kLanes;
    for (int base = blockIdx.x * kRows; base < s.m; base += gridDim.x * kRows) {
        const int i = base + static_cast<int>(threadIdx.x) / kLanes;
        const double ax = csr_row(s.arp, s.aci, s.ava, next, i, s.m, sl);
        if (i < s.m && sl == 0) {
            const double zi = z[i], yi = y[i], ri = s.rho[i];
            const double relaxed = __dsub_rn(__dmul_rn(1.6, ax), __dmul_rn(.6, zi));
            const double w = __dadd_rn(relaxed, __ddiv_rn(yi, ri));
            const double t = w < up[i] ? w : up[i];  // std::max(lo, std::min(up, w))
            const double nz = lo[i] < t ? t : lo[i];
            y[i] = __dadd_rn(yi, __dmul_rn(ri, __dsub_rn(relaxed, nz)));
            z[i] = nz;
        }
    }
}

// x = 1.6 next - .6 x
__global__ void __launch_bounds__(kB) admm_x_kernel(int n, const double* __restrict__ next, double* __restrict__ xa) {
    for (int j = blockIdx.x * kB + threadIdx.x; j < n; j += gridDim.x * kB)
        xa[j] = __dsub_rn(__dmul_rn(1.6, next[j]), __dmul_rn(.6, xa[j]));
}

int grid_for(int rows, int per_block) {
    int g = (rows + per_block - 1) / per_block;
    return std::max(1, std::min(g, kMaxBlocks));
}

}  // namespace

struct bqp_admm {
    int device = 0;
    int64_t n = 0, m = 0;
    cudaStream_t stream = nullptr;
    // device arrays
    int32_t *hrp = nullptr, *hci = nullptr, *arp = nullptr, *aci = nullptr, *trp = nullptr, *tci = nullptr;
    double *hva = nullptr, *ava = nullptr, *tva = nullptr;
    double *rho = nullptr, *t = nullptr, *precond = nullptr;
    double *rhs = nullptr, *x = nullptr, *r = nullptr, *pre = nullptr, *d = nullptr, *kd = nullptr, *v = nullptr;
    double* partial = nullptr;
    AdmmState* st = nullptr;
    AdmmState* h_st = nullptr;
    // ADMM state of bqp_admm_iterate (allocated on first use): x, the cost, z, y and the
    // constraint bounds (one per row of A)
    double *xa = nullptr, *c = nullptr, *z = nullptr, *y = nullptr, *lo = nullptr, *up = nullptr;
    double sigma = 0;
    bool rho_set = false;
    cudaGraph_t graph = nullptr, apply_graph = nullptr;
    cudaGraphExec_t exec = nullptr, apply_exec = nullptr;
    std::string error;

    Sys sys() const {
        Sys s;
        s.n = static_cast<int>(n);
        s.m = static_cast<int>(m);
        s.hrp = hrp; s.hci = hci; s.hva = hva;
        s.arp = arp; s.aci = aci; s.ava = ava;
        s.trp = trp; s.tci = tci; s.tva = tva;
        s.rho = rho;
        s.sigma = sigma;
        s.precond = precond;
        s.t = t;
        return s;
    }
    bool ok(cudaError_t e, const char* what) {
        if (e == cudaSuccess) return true;
        error = std::string("CUDA: ") + what + ": " + cudaGetErrorString(e);
        return false;
    }
    // graphs are built once rho and sigma are known (sigma is a kernel argument)
    bool build() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        if (apply_exec) cudaGraphExecDestroy(apply_exec);
        if (apply_graph) cudaGraphDestroy(apply_graph);
        exec = nullptr; graph = nullptr; apply_exec = nullptr; apply_graph = nullptr;
        const Sys s = sys();
        const int gm = grid_for(static_cast<int>(m), kRows), gn = grid_for(static_cast<int>(n), kRows);
        const int gv = grid_for(static_cast<int>(n), kB);
        if (!ok(cudaGraphCreate(&graph, 0), "graph")) return false;
        cudaGraphConditionalHandle h;
        if (!ok(cudaGraphConditionalHandleCreate(&h, graph, 0, cudaGraphCondAssignDefault), "conditional handle")) return false;
        // set-up: sys = K x, r, pre, d, rz, max|r|, the loop condition
        cudaStream_t cap = nullptr;
        if (!ok(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking), "capture stream")) return false;
        bool good = ok(cudaStreamBeginCaptureToGraph(cap, graph, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal), "capture");
        cudaGraphNode_t tail = nullptr;
        if (good) {
            admm_a_kernel<<<gm, kB, 0, cap>>>(s, x, st);
            admm_k_kernel<<<gn, kB, 0, cap>>>(s, x, kd, 1, rhs, r, pre, d, partial, st, h);
            cudaStreamCaptureStatus cs;
            const cudaGraphNode_t* last = nullptr;
            size_t nlast = 0;
            good = ok(cudaStreamGetCaptureInfo(cap, &cs, nullptr, nullptr, &last, nullptr, &nlast), "capture info");
            if (good && nlast) tail = last[0];
            cudaGraph_t out = nullptr;
            good = ok(cudaStreamEndCapture(cap, &out), "end capture") && good && tail;
        }
        if (good) {
            cudaGraphNodeParams p = {cudaGraphNodeTypeConditional};
            p.conditional.handle = h;
            p.conditional.type = cudaGraphCondTypeWhile;
            p.conditional.size = 1;
            cudaGraphNode_t wnode;
            good = ok(cudaGraphAddNode(&wnode, graph, &tail, nullptr, 1, &p), "while node");
            if (good) {
                cudaGraph_t body = p.conditional.phGraph_out[0];
                good = ok(cudaStreamBeginCaptureToGraph(cap, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal), "capture");
                if (good) {
                    admm_a_kernel<<<gm, kB, 0, cap>>>(s, d, st);
                    admm_k_kernel<<<gn, kB, 0, cap>>>(s, d, kd, 2, rhs, r, pre, d, partial, st, h);
                    admm_update_kernel<<<gv, kB, 0, cap>>>(s, x, r, pre, d, kd, partial, st, h);
                    admm_direction_kernel<<<gv, kB, 0, cap>>>(s.n, d, pre, st);
                    cudaGraph_t out = nullptr;
                    good = ok(cudaStreamEndCapture(cap, &out), "end capture");
                }
            }
        }
        if (good) good = ok(cudaGraphInstantiate(&exec, graph, 0), "graph instantiate");
        // K v alone
        if (good) good = ok(cudaGraphCreate(&apply_graph, 0), "graph");
        if (good) good = ok(cudaStreamBeginCaptureToGraph(cap, apply_graph, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal), "capture");
        if (good) {
            admm_a_kernel<<<gm, kB, 0, cap>>>(s, v, st);
            admm_k_kernel<<<gn, kB, 0, cap>>>(s, v, kd, 0, rhs, r, pre, d, partial, st, 0);
            cudaGraph_t out = nullptr;
            good = ok(cudaStreamEndCapture(cap, &out), "end capture");
        }
        if (good) good = ok(cudaGraphInstantiate(&apply_exec, apply_graph, 0), "graph instantiate");
        cudaStreamDestroy(cap);
        return good && ok(cudaGetLastError(), "admm kernels");
    }
    ~bqp_admm() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        if (apply_exec) cudaGraphExecDestroy(apply_exec);
        if (apply_graph) cudaGraphDestroy(apply_graph);
        for (void* p : {static_cast<void*>(hrp), static_cast<void*>(hci), static_cast<void*>(arp), static_cast<void*>(aci),
                        static_cast<void*>(trp), static_cast<void*>(tci), static_cast<void*>(hva), static_cast<void*>(ava),
                        static_cast<void*>(tva), static_cast<void*>(rho), static_cast<void*>(t), static_cast<void*>(precond),
                        static_cast<void*>(rhs), static_cast<void*>(x), static_cast<void*>(r), static_cast<void*>(pre),
                        static_cast<void*>(d), static_cast<void*>(kd), static_cast<void*>(v), static_cast<void*>(partial),
                        static_cast<void*>(st), static_cast<void*>(xa), static_cast<void*>(c), static_cast<void*>(z),
                        static_cast<void*>(y), static_cast<void*>(lo), static_cast<void*>(up)})
            if (p) cudaFree(p);
        if (h_st) cudaFreeHost(h_st);
        if (stream) cudaStreamDestroy(stream);
    }
};

namespace {
std::string g_admm_error;

bool valid_csr(int64_t rows, int64_t cols, int64_t nnz, const int32_t* rp, const int32_t* ci, const double* va) {
    if (rows < 0 || nnz < 0 || !rp || (nnz && (!ci || !va)) || rp[0] != 0 || rp[rows] != nnz) return false;
    for (int64_t i = 0; i < rows; ++i)
        if (rp[i + 1] < rp[i]) return false;
    for (int64_t k = 0; k < nnz; ++k)
        if (ci[k] < 0 || ci[k] >= cols || !std::isfinite(va[k])) return false;
    return true;
}
}  // namespace

extern "C" {

bqp_admm* bqp_admm_create(int device, int64_t n, int64_t m, const int32_t* h_rowptr, const int32_t* h_col,
                          const double* h_val, const int32_t* a_rowptr, const int32_t* a_col, const double* a_val) {
    if (n <= 0 || m < 0 || n > 2000000000LL || m > 2000000000LL || !h_rowptr || !a_rowptr) {
        g_admm_error = "Invalid ADMM system dimensions";
        return nullptr;
    }
    const int64_t hz = h_rowptr[n], az = a_rowptr[m];
    if (!valid_csr(n, n, hz, h_rowptr, h_col, h_val) || !valid_csr(m, n, az, a_rowptr, a_col, a_val)) {
        g_admm_error = "Invalid CSR arrays of H or A";
        return nullptr;
    }
    // A' by a stable counting sort: row j of A' lists the rows i of A in increasing order
    std::vector<int32_t> trp(static_cast<size_t>(n) + 1, 0), tci(static_cast<size_t>(az));
    std::vector<double> tva(static_cast<size_t>(az));
    for (int64_t k = 0; k < az; ++k) trp[static_cast<size_t>(a_col[k]) + 1]++;
    for (int64_t j = 0; j < n; ++j) trp[j + 1] += trp[j];
    {
        std::vector<int32_t> next(trp.begin(), trp.end() - 1);
        for (int64_t i = 0; i < m; ++i)
            for (int64_t k = a_rowptr[i]; k < a_rowptr[i + 1]; ++k) {
                const int32_t pos = next[a_col[k]]++;
                tci[pos] = static_cast<int32_t>(i);
                tva[pos] = a_val[k];
            }
    }
    std::unique_ptr<bqp_admm> s(new (std::nothrow) bqp_admm);
    if (!s) {
        g_admm_error = "host memory";
        return nullptr;
    }
    s->device = device;
    s->n = n;
    s->m = m;
    int prev = -1;
    cudaGetDevice(&prev);
    auto fail = [&](const char* what, cudaError_t e) {
        g_admm_error = std::string("CUDA: ") + what + ": " + cudaGetErrorString(e);
        if (prev >= 0) cudaSetDevice(prev);
        return static_cast<bqp_admm*>(nullptr);
    };
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return fail("set device", e);
    const size_t N = static_cast<size_t>(n), M = static_cast<size_t>(std::max<int64_t>(m, 1));
    auto alloc = [&](auto** p, size_t count) {
        return cudaMalloc(reinterpret_cast<void**>(p), sizeof(**p) * std::max<size_t>(count, 1));
    };
    if ((e = alloc(&s->hrp, N + 1)) || (e = alloc(&s->hci, static_cast<size_t>(hz))) || (e = alloc(&s->hva, static_cast<size_t>(hz))) ||
        (e = alloc(&s->arp, M + 1)) || (e = alloc(&s->aci, static_cast<size_t>(az))) || (e = alloc(&s->ava, static_cast<size_t>(az))) ||
        (e = alloc(&s->trp, N + 1)) || (e = alloc(&s->tci, static_cast<size_t>(az))) || (e = alloc(&s->tva, static_cast<size_t>(az))) ||
        (e = alloc(&s->rho, M)) || (e = alloc(&s->t, M)) || (e = alloc(&s->precond, N)) || (e = alloc(&s->rhs, N)) ||
        (e = alloc(&s->x, N)) || (e = alloc(&s->r, N)) || (e = alloc(&s->pre, N)) || (e = alloc(&s->d, N)) ||
        (e = alloc(&s->kd, N)) || (e = alloc(&s->v, N)) || (e = alloc(&s->partial, 3 * static_cast<size_t>(kMaxBlocks))) ||
        (e = alloc(&s->st, 1)))
        return fail("allocate", e);
    if ((e = cudaMallocHost(reinterpret_cast<void**>(&s->h_st), sizeof(AdmmState)))) return fail("allocate", e);
    if ((e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking))) return fail("stream", e);
    cudaMemcpy(s->hrp, h_rowptr, sizeof(int32_t) * (N + 1), cudaMemcpyHostToDevice);
    if (hz) cudaMemcpy(s->hci, h_col, sizeof(int32_t) * static_cast<size_t>(hz), cudaMemcpyHostToDevice);
    if (hz) cudaMemcpy(s->hva, h_val, sizeof(double) * static_cast<size_t>(hz), cudaMemcpyHostToDevice);
    cudaMemcpy(s->arp, a_rowptr, sizeof(int32_t) * (static_cast<size_t>(m) + 1), cudaMemcpyHostToDevice);
    if (az) cudaMemcpy(s->aci, a_col, sizeof(int32_t) * static_cast<size_t>(az), cudaMemcpyHostToDevice);
    if (az) cudaMemcpy(s->ava, a_val, sizeof(double) * static_cast<size_t>(az), cudaMemcpyHostToDevice);
    cudaMemcpy(s->trp, trp.data(), sizeof(int32_t) * (N + 1), cudaMemcpyHostToDevice);
    if (az) cudaMemcpy(s->tci, tci.data(), sizeof(int32_t) * static_cast<size_t>(az), cudaMemcpyHostToDevice);
    if (az) cudaMemcpy(s->tva, tva.data(), sizeof(double) * static_cast<size_t>(az), cudaMemcpyHostToDevice);
    cudaMemset(s->st, 0, sizeof(AdmmState));
    if ((e = cudaDeviceSynchronize())) return fail("upload", e);
    if (prev >= 0) cudaSetDevice(prev);
    return s.release();
}

int bqp_admm_set_rho(bqp_admm* s, const double* rho, double sigma) {
    if (!s || (s->m && !rho) || !std::isfinite(sigma) || sigma < 0) return BQP_ERR_INVALID;
    for (int64_t i = 0; i < s->m; ++i)
        if (!(rho[i] > 0) || !std::isfinite(rho[i])) return BQP_ERR_INVALID;
    int prev = -1;
    cudaGetDevice(&prev);
    cudaSetDevice(s->device);
    if (s->m) cudaMemcpyAsync(s->rho, rho, sizeof(double) * static_cast<size_t>(s->m), cudaMemcpyHostToDevice, s->stream);
    s->sigma = sigma;
    admm_precond_kernel<<<grid_for(static_cast<int>(s->n), kB), kB, 0, s->stream>>>(s->sys(), s->precond);
    bool good = s->ok(cudaStreamSynchronize(s->stream), "preconditioner") && s->build();
    s->rho_set = good;
    if (prev >= 0) cudaSetDevice(prev);
    if (!good) {
        g_admm_error = s->error;
        return BQP_ERR_CUDA;
    }
    return BQP_OK;
}

int bqp_admm_apply(bqp_admm* s, const double* v, double* out) {
    if (!s || !v || !out) return BQP_ERR_INVALID;
    if (!s->rho_set) return BQP_ERR_NOT_READY;
    int prev = -1;
    cudaGetDevice(&prev);
    cudaSetDevice(s->device);
    const size_t N = static_cast<size_t>(s->n);
    cudaMemcpyAsync(s->v, v, sizeof(double) * N, cudaMemcpyHostToDevice, s->stream);
    cudaMemsetAsync(s->st, 0, sizeof(AdmmState), s->stream);
    cudaGraphLaunch(s->apply_exec, s->stream);
    cudaMemcpyAsync(out, s->kd, sizeof(double) * N, cudaMemcpyDeviceToHost, s->stream);
    const bool good = s->ok(cudaStreamSynchronize(s->stream), "apply");
    if (prev >= 0) cudaSetDevice(prev);
    if (!good) {
        g_admm_error = s->error;
        return BQP_ERR_CUDA;
    }
    return BQP_OK;
}

int bqp_admm_solve(bqp_admm* s, const double* rhs, double* x, double accuracy, int64_t max_inner, int64_t* inner_out,
                   double* residual_out) {
    if (!s || !rhs || !x || !(accuracy >= 0) || max_inner < 0) return BQP_ERR_INVALID;
    if (!s->rho_set) return BQP_ERR_NOT_READY;
    int prev = -1;
    cudaGetDevice(&prev);
    cudaSetDevice(s->device);
    const size_t N = static_cast<size_t>(s->n);
    std::memset(s->h_st, 0, sizeof(AdmmState));
    s->h_st->accuracy = accuracy;
    s->h_st->max_inner = max_inner;
    cudaMemcpyAsync(s->rhs, rhs, sizeof(double) * N, cudaMemcpyHostToDevice, s->stream);
    cudaMemcpyAsync(s->x, x, sizeof(double) * N, cudaMemcpyHostToDevice, s->stream);
    cudaMemcpyAsync(s->st, s->h_st, sizeof(AdmmState), cudaMemcpyHostToDevice, s->stream);
    cudaGraphLaunch(s->exec, s->stream);
    cudaMemcpyAsync(x, s->x, sizeof(double) * N, cudaMemcpyDeviceToHost, s->stream);
    cudaMemcpyAsync(s->h_st, s->st, sizeof(AdmmState), cudaMemcpyDeviceToHost, s->stream);
    const bool good = s->ok(cudaStreamSynchronize(s->stream), "solve");
    if (prev >= 0) cudaSetDevice(prev);
    if (!good) {
        g_admm_error = s->error;
        return BQP_ERR_CUDA;
    }
    if (inner_out) *inner_out = s->h_st->inner;
    if (residual_out) std::memcpy(residual_out, &s->h_st->rmax, sizeof(double));
    return BQP_OK;
}

int bqp_admm_iterate(bqp_admm* s, const double* c, const double* lo, const double* up, double* x, double* z, double* y,
                     int64_t first_iteration, int64_t iterations, int64_t* inner_total) {
    if (!s || !c || !x || (s->m && (!lo || !up || !z || !y)) || first_iteration < 0 || iterations < 0)
        return BQP_ERR_INVALID;
    if (!s->rho_set) return BQP_ERR_NOT_READY;
    int prev = -1;
    cudaGetDevice(&prev);
    cudaSetDevice(s->device);
    const size_t N = static_cast<size_t>(s->n), M = static_cast<size_t>(std::max<int64_t>(s->m, 1));
    cudaError_t e = cudaSuccess;
    if (!s->xa) {
        if ((e = cudaMalloc(&s->xa, sizeof(double) * N)) || (e = cudaMalloc(&s->c, sizeof(double) * N)) ||
            (e = cudaMalloc(&s->z, sizeof(double) * M)) || (e = cudaMalloc(&s->y, sizeof(double) * M)) ||
            (e = cudaMalloc(&s->lo, sizeof(double) * M)) || (e = cudaMalloc(&s->up, sizeof(double) * M))) {
            s->ok(e, "allocate ADMM state");
            if (prev >= 0) cudaSetDevice(prev);
            g_admm_error = s->error;
            return BQP_ERR_NO_MEMORY;
        }
    }
    const size_t mb = sizeof(double) * static_cast<size_t>(s->m);
    cudaMemcpyAsync(s->xa, x, sizeof(double) * N, cudaMemcpyHostToDevice, s->stream);
    cudaMemcpyAsync(s->c, c, sizeof(double) * N, cudaMemcpyHostToDevice, s->stream);
    if (mb) {
        cudaMemcpyAsync(s->z, z, mb, cudaMemcpyHostToDevice, s->stream);
        cudaMemcpyAsync(s->y, y, mb, cudaMemcpyHostToDevice, s->stream);
        cudaMemcpyAsync(s->lo, lo, mb, cudaMemcpyHostToDevice, s->stream);
        cudaMemcpyAsync(s->up, up, mb, cudaMemcpyHostToDevice, s->stream);
    }
    cudaMemsetAsync(s->st, 0, sizeof(AdmmState), s->stream);
    const Sys sy = s->sys();
    const int gn = grid_for(static_cast<int>(s->n), kRows), gm = grid_for(static_cast<int>(s->m), kRows);
    const int gv = grid_for(static_cast<int>(s->n), kB);
    for (int64_t k = 0; k < iterations; ++k) {
        const double it = static_cast<double>(first_iteration + k + 1);
        const double factor = std::min(1e-7, .05 / std::pow(it, 1.6));
        admm_rhs_kernel<<<gn, kB, 0, s->stream>>>(sy, s->z, s->y, s->xa, s->c, s->rhs, s->x, s->partial, s->st, factor);
        cudaGraphLaunch(s->exec, s->stream);
        admm_zy_kernel<<<gm, kB, 0, s->stream>>>(sy, s->x, s->z, s->y, s->lo, s->up, s->st);
        admm_x_kernel<<<gv, kB, 0, s->stream>>>(static_cast<int>(s->n), s->x, s->xa);
    }
    cudaMemcpyAsync(x, s->xa, sizeof(double) * N, cudaMemcpyDeviceToHost, s->stream);
    if (mb) {
        cudaMemcpyAsync(z, s->z, mb, cudaMemcpyDeviceToHost, s->stream);
        cudaMemcpyAsync(y, s->y, mb, cudaMemcpyDeviceToHost, s->stream);
    }
    cudaMemcpyAsync(s->h_st, s->st, sizeof(AdmmState), cudaMemcpyDeviceToHost, s->stream);
    const bool good = s->ok(cudaStreamSynchronize(s->stream), "iterate") && s->ok(cudaGetLastError(), "ADMM kernels");
    if (prev >= 0) cudaSetDevice(prev);
    if (!good) {
        g_admm_error = s->error;
        return BQP_ERR_CUDA;
    }
    if (inner_total) *inner_total = s->h_st->inner_sum;
    return BQP_OK;
}

const char* bqp_admm_last_error(void) { return g_admm_error.c_str(); }

void bqp_admm_destroy(bqp_admm* s) {
    if (!s) return;
    int prev = -1;
    cudaGetDevice(&prev);
    cudaSetDevice(s->device);
    delete s;
    if (prev >= 0) cudaSetDevice(prev);
}

}  // extern "C"
