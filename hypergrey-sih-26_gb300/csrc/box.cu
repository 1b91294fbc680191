// Plugin-level entry points: the reference's BoxIteration contract on the GPU, and the FP64
// verification reduction on caller-owned device arrays.
//
// bqp_box_* mirror sovereign::make_cuda_box / CudaBox (02-software/solver/src/cuda_box.cu:22-37):
// the CSR and vectors are uploaded once, step(beta) runs one FISTA iteration on the device and
// primal() copies x back.  One fused kernel replaces the reference's csr_product + fista_step
// pair; w is double-buffered instead of keeping a separate gradient array.  The arithmetic is
// the CPU loop's (division by L, separately rounded products and sums), so a host loop driving
// this plugin reproduces the CPU engine's iterates.
#include "boxqp.h"
#include "engine.cuh"
#include "kernels.cuh"

#include <cuda.h>

#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

struct bqp_box {
    int device = 0;
    int64_t n = 0, nnz = 0;
    double L = 0;
    int32_t* rowptr = nullptr;
    int32_t* col = nullptr;
    double* val = nullptr;
    double* c = nullptr;
    double* l = nullptr;
    double* u = nullptr;
    double* x = nullptr;
    double* w[2] = {nullptr, nullptr};
    int cur = 0;
    cudaStream_t stream = nullptr;
    std::string error;
};

namespace {
thread_local std::string g_box_error;

void box_free(bqp_box* b) {
    if (!b) return;
    cudaFree(b->rowptr); cudaFree(b->col); cudaFree(b->val); cudaFree(b->c); cudaFree(b->l); cudaFree(b->u);
    cudaFree(b->x); cudaFree(b->w[0]); cudaFree(b->w[1]);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

bool ok(cudaError_t e, std::string& why) {
    if (e == cudaSuccess) return true;
    why = std::string("CUDA: ") + cudaGetErrorString(e);
    return false;
}
// ---- scratch of bqp_check_device_noalloc ------------------------------------------------------
// The verification reduction needs global scratch for its per-block partials, its completion
// counter and its 8 result values.  bqp_check_device_noalloc takes that scratch from this
// file-scope device array instead of cudaMalloc: 96 KiB in every context that loads this
// module, held until the context ends.  At most 1024 blocks of partials fit, which bounds n to
// kNoAllocMaxRows.  In host code the name of the array is only a host-side stand-in, so its
// device address is looked up with cudaGetSymbolAddress, with the device current, once per
// context: the lookup is cached under the current context's unique id (cuCtxGetId), so a
// context that is destroyed and recreated (cudaDeviceReset) gets a fresh lookup instead of a
// stale address.  The same set-up loads the check kernel into the context, so that later
// calls do not load code (which takes device memory) under lazy module loading.
constexpr int64_t kNoAllocMaxRows = 4194304;
constexpr size_t kNoAllocBytes = 96 * 1024;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

constexpr int kMaxDevices = 64;
struct NoallocSlot {
    unsigned long long context_id = 0;  // 0: not set up
    void* address = nullptr;
};
std::mutex g_noalloc_mu;
NoallocSlot g_noalloc_slot[kMaxDevices];

// The driver's cuCtxGetCurrent / cuCtxGetId, reached through the runtime (no libcuda link).
typedef CUresult (*CtxGetCurrentFn)(CUcontext*);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long*);

cudaError_t current_context_id(unsigned long long* id) {
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<CtxGetCurrentFn>(f);
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<CtxGetIdFn>(f);
    });
    if (!get_current || !get_id) return cudaErrorNotSupported;
    CUcontext ctx = nullptr;
    if (get_current(&ctx) != CUDA_SUCCESS || !ctx) return cudaErrorDeviceUninitialized;
    return get_id(ctx, id) == CUDA_SUCCESS ? cudaSuccess : cudaErrorDeviceUninitialized;
}

// Device address of g_noalloc_scratch in the current context (set up on the first call there).
// No context current yet: the symbol lookup initializes the runtime's context on this device.
cudaError_t noalloc_scratch(void** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    unsigned long long id = 0;
    const bool have_id = current_context_id(&id) == cudaSuccess;
    std::lock_guard<std::mutex> g(g_noalloc_mu);
    NoallocSlot& slot = g_noalloc_slot[dev];
    if (!have_id || slot.context_id != id) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        e = bqp::load_check_standalone();
        if (e != cudaSuccess) return e;
        // a driver that cannot name the context (no cuCtxGetId) gets this set-up on every call
        // instead of a cached address
        if (current_context_id(&id) != cudaSuccess) {
            *out = p;
            return cudaSuccess;
        }
        slot.address = p;
        slot.context_id = id;
    }
    *out = slot.address;
    return cudaSuccess;
}
}  // namespace

extern "C" {

bqp_box* bqp_box_create(int device, int64_t n, int64_t nnz, const int32_t* rowptr, const int32_t* col,
                        const double* val, const double* c, const double* lower, const double* upper,
                        double lipschitz) {
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        g_box_error = "No CUDA device available";
        return nullptr;
    }
    if (device < 0 || device >= count || n <= 0 || nnz < 0 || !rowptr || !c || !lower || !upper || (nnz && (!col || !val)) ||
        !(lipschitz > 0) || !std::isfinite(lipschitz) || n > 2000000000LL) {
        g_box_error = "invalid argument";
        return nullptr;
    }
    bqp_box* b = new bqp_box;
    b->device = device;
    b->n = n;
    b->nnz = nnz;
    b->L = lipschitz;
    std::string why;
    const size_t N = static_cast<size_t>(n), Z = static_cast<size_t>(nnz);
    // x0 = w0 = clip(0, l, u) (CudaBox::initial, src/cuda_box.cu:25)
    std::vector<double> x0(N);
    for (size_t j = 0; j < N; ++j) {
        double v = (0.0 < upper[j]) ? 0.0 : upper[j];
        x0[j] = (lower[j] < v) ? v : lower[j];
    }
    bool good = ok(cudaSetDevice(device), why) && ok(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking), why) &&
                ok(cudaMalloc(&b->rowptr, (N + 1) * 4), why) && ok(cudaMalloc(&b->col, Z * 4 + 16), why) &&
                ok(cudaMalloc(&b->val, Z * 8 + 16), why) && ok(cudaMalloc(&b->c, N * 8), why) &&
                ok(cudaMalloc(&b->l, N * 8), why) && ok(cudaMalloc(&b->u, N * 8), why) &&
                ok(cudaMalloc(&b->x, N * 8), why) && ok(cudaMalloc(&b->w[0], N * 8), why) &&
                ok(cudaMalloc(&b->w[1], N * 8), why) &&
                ok(cudaMemcpy(b->rowptr, rowptr, (N + 1) * 4, cudaMemcpyHostToDevice), why) &&
                (Z == 0 || ok(cudaMemcpy(b->col, col, Z * 4, cudaMemcpyHostToDevice), why)) &&
                (Z == 0 || ok(cudaMemcpy(b->val, val, Z * 8, cudaMemcpyHostToDevice), why)) &&
                ok(cudaMemcpy(b->c, c, N * 8, cudaMemcpyHostToDevice), why) &&
                ok(cudaMemcpy(b->l, lower, N * 8, cudaMemcpyHostToDevice), why) &&
                ok(cudaMemcpy(b->u, upper, N * 8, cudaMemcpyHostToDevice), why) &&
                ok(cudaMemcpy(b->x, x0.data(), N * 8, cudaMemcpyHostToDevice), why) &&
                ok(cudaMemcpy(b->w[0], x0.data(), N * 8, cudaMemcpyHostToDevice), why);
    if (!good) {
        g_box_error = why;
        box_free(b);
        return nullptr;
    }
    return b;
}

int bqp_box_step(bqp_box* b, double momentum) {
    if (!b) return BQP_ERR_INVALID;
    cudaSetDevice(b->device);
    bqp::launch_box_step(b->n, b->rowptr, b->col, b->val, b->c, b->l, b->u, b->L, momentum, b->x, b->w[b->cur],
                         b->w[b->cur ^ 1], b->stream);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        b->error = std::string("CUDA: ") + cudaGetErrorString(e);
        return BQP_ERR_CUDA;
    }
    b->cur ^= 1;
    return BQP_OK;
}

int bqp_box_primal(bqp_box* b, double* x) {
    if (!b || !x) return BQP_ERR_INVALID;
    cudaSetDevice(b->device);
    cudaError_t e = cudaMemcpyAsync(x, b->x, static_cast<size_t>(b->n) * 8, cudaMemcpyDeviceToHost, b->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) {
        b->error = std::string("CUDA: ") + cudaGetErrorString(e);
        return BQP_ERR_CUDA;
    }
    return BQP_OK;
}

void bqp_box_destroy(bqp_box* b) {
    if (!b) return;
    cudaSetDevice(b->device);
    cudaStreamSynchronize(b->stream);
    box_free(b);
}

const char* bqp_box_last_error(const bqp_box* b) { return b ? b->error.c_str() : g_box_error.c_str(); }

int bqp_check_device(int64_t n, const int32_t* d_rowptr, const int32_t* d_col, const double* d_val, const double* d_x,
                     const double* d_c, const double* d_lower, const double* d_upper, double tolerance, double offset,
                     int32_t diagonal_gate, bqp_stats* stats) {
    if (n <= 0 || n > 2000000000LL || !d_rowptr || !d_x || !d_c || !d_lower || !d_upper || !stats ||
        !(tolerance > 0) || !std::isfinite(offset)) {
        g_box_error = "bqp_check_device: invalid argument (n must be in 1..2e9, the device pointers and stats "
                      "non-null, the tolerance positive and the offset finite)";
        return BQP_ERR_INVALID;
    }
    const size_t bytes = bqp::check_scratch_bytes(n) + 8 * sizeof(double);
    void* scratch = nullptr;
    cudaStream_t s = nullptr;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return BQP_ERR_CUDA;
    if (cudaMalloc(&scratch, bytes) != cudaSuccess) {
        cudaStreamDestroy(s);
        return BQP_ERR_NO_MEMORY;
    }
    double* result = reinterpret_cast<double*>(static_cast<char*>(scratch) + bqp::check_scratch_bytes(n));
    double host[8];
    cudaMemsetAsync(scratch, 0, bytes, s);
    bqp::launch_check_standalone(n, d_rowptr, d_col, d_val, d_x, d_c, d_lower, d_upper, tolerance, offset,
                                 diagonal_gate > 0 ? 1 : 0, scratch, result, s);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(host, result, sizeof(host), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(scratch);
    cudaStreamDestroy(s);
    if (e != cudaSuccess) return BQP_ERR_CUDA;
    std::memset(stats, 0, sizeof(*stats));
    stats->objective = host[0];
    stats->primal_residual = host[1];
    stats->stationarity_residual = host[2];
    stats->complementarity_residual = host[3];
    stats->dual_bound = host[4];
    stats->relative_gap = host[5];
    stats->verified = host[6] != 0 ? 1 : 0;
    stats->status = stats->verified ? BQP_STATUS_OPTIMAL : BQP_STATUS_RUNNING;
    return BQP_OK;
}

int bqp_gate_device(int64_t n, const int32_t* d_rowptr, const int32_t* d_col, const double* d_val, double* d_diag,
                    double* lipschitz, int32_t* indefinite, int32_t* nondominant) {
    if (n <= 0 || n > 2000000000LL || !d_rowptr || !d_col || !d_val || !lipschitz || !indefinite || !nondominant) {
        g_box_error = "bqp_gate_device: invalid argument (n must be in 1..2e9, the CSR device pointers and the "
                      "three results non-null)";
        return BQP_ERR_INVALID;
    }
    cudaStream_t s = nullptr;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return BQP_ERR_CUDA;
    bqp::GateResult* out = nullptr;
    if (cudaMalloc(&out, sizeof(bqp::GateResult)) != cudaSuccess) {
        cudaStreamDestroy(s);
        g_box_error = "bqp_gate_device: device memory for the result";
        return BQP_ERR_NO_MEMORY;
    }
    bqp::GateResult host{};
    bqp::launch_gate_raw(n, d_rowptr, d_col, d_val, out, d_diag, nullptr, nullptr, s);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(&host, out, sizeof(host), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(out);
    cudaStreamDestroy(s);
    if (e != cudaSuccess) {
        g_box_error = std::string("CUDA: ") + cudaGetErrorString(e);
        return BQP_ERR_CUDA;
    }
    std::memcpy(lipschitz, &host.lip_bits, sizeof(double));
    *indefinite = host.indefinite;
    *nondominant = host.nondominant;
    return BQP_OK;
}

int bqp_check_device_noalloc(int64_t n, const int32_t* d_rowptr, const int32_t* d_col, const double* d_val,
                             const double* d_x, const double* d_c, const double* d_lower, const double* d_upper,
                             double tolerance, double offset, int32_t diagonal_gate, bqp_stats* stats) {
    if (n <= 0 || !d_rowptr || !d_x || !d_c || !d_lower || !d_upper || !stats || !(tolerance > 0) ||
        !std::isfinite(offset)) {
        g_box_error = "bqp_check_device_noalloc: invalid argument (n must be positive, the device pointers and "
                      "stats non-null, the tolerance positive and the offset finite)";
        return BQP_ERR_INVALID;
    }
    if (n > kNoAllocMaxRows) {
        g_box_error = "bqp_check_device_noalloc: n = " + std::to_string(n) + " exceeds the limit of " +
                      std::to_string(kNoAllocMaxRows) + " rows of its static scratch; use bqp_check_device";
        return BQP_ERR_INVALID;
    }
    const size_t head = bqp::check_scratch_bytes(n);
    const size_t bytes = head + 8 * sizeof(double);
    if (bytes > kNoAllocBytes) {
        g_box_error = "bqp_check_device_noalloc: scratch size exceeds the static array";
        return BQP_ERR_INVALID;
    }
    void* scratch = nullptr;
    cudaError_t e = noalloc_scratch(&scratch);
    if (e != cudaSuccess) {
        g_box_error = std::string("CUDA: ") + cudaGetErrorString(e);
        return BQP_ERR_CUDA;
    }
    double* result = reinterpret_cast<double*>(static_cast<char*>(scratch) + head);
    double host[8];
    // The array keeps the previous call's contents: clear the completion counter, partials and
    // result before the launch.  All calls use the legacy default stream.
    e = cudaMemsetAsync(scratch, 0, bytes, 0);
    if (e == cudaSuccess) {
        bqp::launch_check_standalone(n, d_rowptr, d_col, d_val, d_x, d_c, d_lower, d_upper, tolerance, offset,
                                     diagonal_gate > 0 ? 1 : 0, scratch, result, 0);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(host, result, sizeof(host), cudaMemcpyDeviceToHost, 0);
    if (e == cudaSuccess) e = cudaStreamSynchronize(0);
    if (e != cudaSuccess) {
        g_box_error = std::string("CUDA: ") + cudaGetErrorString(e);
        return BQP_ERR_CUDA;
    }
    std::memset(stats, 0, sizeof(*stats));
    stats->objective = host[0];
    stats->primal_residual = host[1];
    stats->stationarity_residual = host[2];
    stats->complementarity_residual = host[3];
    stats->dual_bound = host[4];
    stats->relative_gap = host[5];
    stats->verified = host[6] != 0 ? 1 : 0;
    stats->status = stats->verified ? BQP_STATUS_OPTIMAL : BQP_STATUS_RUNNING;
    return BQP_OK;
}

}  // extern "C"
