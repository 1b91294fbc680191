// Standalone measurement (not part of libboxqp): the GB300's ceiling for the memory pattern of
// the FISTA step on the 1M-variable random graph (n = 1,000,000, nnz = 15,000,000).
//
//   nvcc -gencode arch=compute_103a,code=sm_103a -O3 -std=c++17 \
//        -o gather_ceiling hypergrey-sih-26_gb300/csrc/gather_ceiling.cu && ./gather_ceiling
//
// It times, with CUDA events after an L2 flush (a 512 MB memset):
//   stream   the coalesced column-index + value stream alone (8 bytes per nonzero, 120 MB)
//   gather   the same stream plus one 4-byte gather per nonzero at a uniformly random column of
//            a 4 MB vector (the vector stays in L2): the step kernel's SpMV without rows
//   dsmem    the random 4-byte reads served from the distributed shared memory of 8-CTA clusters
//            (160 KB per CTA) instead of L2
//   smem     the random reads served from each CTA's own shared memory (the upper bound)
// Every index is in bounds by construction (columns and offsets are taken modulo the sizes).
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <random>
#include <vector>

namespace cg = cooperative_groups;

namespace {

constexpr int kSlice = 40960;  // floats of shared memory per CTA in the dsmem/smem cases

__device__ __forceinline__ uint32_t hash32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352dU;
    x ^= x >> 15;
    x *= 0x846ca68bU;
    x ^= x >> 16;
    return x;
}

__global__ void stream_kernel(const int* __restrict__ col, const float* __restrict__ val, int64_t nnz, float* out) {
    float acc = 0;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nnz; k += (int64_t)gridDim.x * blockDim.x)
        acc += val[k] * (float)(col[k] & 7);
    if (acc == 12345.f) out[0] = acc;
}

__global__ void gather_kernel(const int* __restrict__ col, const float* __restrict__ val, const float* __restrict__ x,
                              int64_t nnz, float* out) {
    float acc = 0;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nnz; k += (int64_t)gridDim.x * blockDim.x)
        acc += val[k] * __ldg(x + col[k]);
    if (acc == 12345.f) out[0] = acc;
}

__global__ void __cluster_dims__(8, 1, 1) dsmem_kernel(int64_t per_thread, float* out) {
    extern __shared__ float sm[];
    cg::cluster_group cluster = cg::this_cluster();
    for (int i = threadIdx.x; i < kSlice; i += blockDim.x) sm[i] = (float)(i & 15);
    cluster.sync();
    float acc = 0;
    const uint32_t seed = (blockIdx.x * blockDim.x + threadIdx.x) * 2654435761u;
    for (int64_t k = 0; k < per_thread; ++k) {
        const uint32_t h = hash32(seed + (uint32_t)k);
        const float* p = cluster.map_shared_rank(sm, (int)(h & 7));
        acc += p[(h >> 3) % kSlice];
    }
    cluster.sync();  // no CTA leaves while others read its shared memory
    if (acc == 1234.5f) out[0] = acc;
}

__global__ void smem_kernel(int64_t per_thread, float* out) {
    extern __shared__ float sm[];
    for (int i = threadIdx.x; i < kSlice; i += blockDim.x) sm[i] = (float)(i & 15);
    __syncthreads();
    float acc = 0;
    const uint32_t seed = (blockIdx.x * blockDim.x + threadIdx.x) * 2654435761u;
    for (int64_t k = 0; k < per_thread; ++k) acc += sm[(hash32(seed + (uint32_t)k) >> 3) % kSlice];
    if (acc == 1234.5f) out[0] = acc;
}

}  // namespace

int main() {
    const int64_t n = 1000000, nnz = 15000000;
    std::mt19937 g(1);
    std::vector<int> col(nnz);
    for (int64_t k = 0; k < nnz; ++k) col[k] = (int)(g() % n);
    int* dcol = nullptr;
    float *dval = nullptr, *dx = nullptr, *dout = nullptr, *dflush = nullptr;
    const size_t flush_bytes = size_t(512) << 20;
    if (cudaMalloc(&dcol, nnz * 4) || cudaMalloc(&dval, nnz * 4) || cudaMalloc(&dx, n * 4) || cudaMalloc(&dout, 64) ||
        cudaMalloc(&dflush, flush_bytes)) {
        std::printf("allocation failed\n");
        return 1;
    }
    cudaMemcpy(dcol, col.data(), nnz * 4, cudaMemcpyHostToDevice);
    cudaMemset(dval, 0, nnz * 4);
    cudaMemset(dx, 0, n * 4);
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
    const int smem = kSlice * 4;
    cudaFuncSetAttribute(dsmem_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    cudaFuncSetAttribute(smem_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    int clusters = 0;
    {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(8 * 64);
        cfg.blockDim = dim3(512);
        cfg.dynamicSmemBytes = smem;
        cudaLaunchAttribute at;
        at.id = cudaLaunchAttributeClusterDimension;
        at.val.clusterDim.x = 8;
        at.val.clusterDim.y = 1;
        at.val.clusterDim.z = 1;
        cfg.attrs = &at;
        cfg.numAttrs = 1;
        cudaOccupancyMaxActiveClusters(&clusters, dsmem_kernel, &cfg);
    }
    if (clusters <= 0) clusters = 16;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    auto best_us = [&](auto launch) {
        float best = 1e30f;
        for (int r = 0; r < 23; ++r) {
            cudaMemsetAsync(dflush, r & 0xff, flush_bytes);
            cudaEventRecord(e0);
            launch();
            cudaEventRecord(e1);
            cudaEventSynchronize(e1);
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            if (r >= 3) best = std::min(best, ms);
        }
        return best * 1e3f;
    };
    std::printf("GB300 random-gather ceiling, n = %lld, nnz = %lld, %d SMs\n", (long long)n, (long long)nnz, sms);
    for (int bps : {4, 8, 16}) {
        const dim3 grid(sms * bps), block(256);
        const float ts = best_us([&] { stream_kernel<<<grid, block>>>(dcol, dval, nnz, dout); });
        const float tg = best_us([&] { gather_kernel<<<grid, block>>>(dcol, dval, dx, nnz, dout); });
        std::printf("%2d blocks/SM: stream %.1f us (%.0f GB/s), stream + 15M random gathers %.1f us (%.1f G gathers/s)\n",
                    bps, ts, nnz * 8.0 / (ts * 1e-6) * 1e-9, tg, nnz / (tg * 1e-6) * 1e-9);
    }
    {
        const int ctas = clusters * 8, threads = 512;
        const int64_t per = (nnz + (int64_t)ctas * threads - 1) / ((int64_t)ctas * threads);
        const double reads = (double)per * ctas * threads;
        const float td = best_us([&] { dsmem_kernel<<<ctas, threads, smem>>>(per, dout); });
        const float tl = best_us([&] { smem_kernel<<<ctas, threads, smem>>>(per, dout); });
        std::printf("%d clusters of 8: %.1fM random reads from distributed shared memory %.1f us (%.1f G/s), "
                    "from own shared memory %.1f us (%.1f G/s)\n",
                    clusters, reads * 1e-6, td, reads / (td * 1e-6) * 1e-9, tl, reads / (tl * 1e-6) * 1e-9);
    }
    const cudaError_t e = cudaDeviceSynchronize();
    std::printf("status %s\n", cudaGetErrorString(e));
    return e != cudaSuccess;
}
