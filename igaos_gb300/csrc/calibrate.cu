// Calibration of the gather-bound SpMV roofline: the rate at which the GPU
// serves random 4-byte reads of a resident vector (igaos_pdhg_gather_rate).
// Every thread keeps kCalUnroll independent gathers in flight; indices come
// from a hash of a per-thread linear congruential stream (no index traffic),
// so the figure is the memory system's random-sector rate for a vector of the
// given size (L1-, L2- or HBM-resident), the ceiling of a product whose
// gathers miss L1.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>

#include "engine.hpp"
#include "igaos_pdhg.h"

namespace {

constexpr int kCalThreads = 256;
constexpr int kCalUnroll = 8;

__device__ __forceinline__ unsigned cal_mix(unsigned h) {
    h ^= h >> 16;
    h *= 0x7feb352dU;
    h ^= h >> 15;
    h *= 0x846ca68bU;
    h ^= h >> 16;
    return h;
}

__global__ void __launch_bounds__(kCalThreads) k_gather_rate(const float* __restrict__ x,
                                                             unsigned mask, int iters,
                                                             float* __restrict__ sink) {
    unsigned s = cal_mix(blockIdx.x * kCalThreads + threadIdx.x + 1u);
    float acc = 0.f;
    for (int it = 0; it < iters; ++it) {
        float v[kCalUnroll];
#pragma unroll
        for (int u = 0; u < kCalUnroll; ++u) {
            s = s * 1664525u + 1013904223u;
            v[u] = __ldg(x + (cal_mix(s) & mask));
        }
#pragma unroll
        for (int u = 0; u < kCalUnroll; ++u) acc += v[u];
    }
    if (acc == 1234.5f) sink[0] = acc;  // keeps the loads; never true for a zero vector
}

}  // namespace

extern "C" int igaos_pdhg_gather_rate(int log2_words, int device, double* gathers_per_s) {
    if (!gathers_per_s || log2_words < 10 || log2_words > 28)
        return igx::igx_set_error(IGAOS_PDHG_ERR_INVALID, "log2_words must be in [10, 28]");
    try {
        if (device >= 0) CU(cudaSetDevice(device));
        int dev = 0, sms = 0;
        CU(cudaGetDevice(&dev));
        CU(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        const size_t words = (size_t)1 << log2_words;
        float *x = nullptr, *sink = nullptr;
        CU(cudaMalloc(&x, words * sizeof(float)));
        struct Free {
            float *a, *b;
            ~Free() {
                cudaFree(a);
                cudaFree(b);
            }
        } guard{x, nullptr};
        CU(cudaMalloc(&sink, sizeof(float)));
        guard.b = sink;
        CU(cudaMemset(x, 0, words * sizeof(float)));
        const int grid = std::max(1, sms) * 8, iters = 64;
        cudaEvent_t e0, e1;
        CU(cudaEventCreate(&e0));
        CU(cudaEventCreate(&e1));
        float best = 1e30f;
        for (int rep = 0; rep < 4; ++rep) {  // first launch warms the vector into the caches
            CU(cudaEventRecord(e0));
            k_gather_rate<<<grid, kCalThreads>>>(x, (unsigned)(words - 1), iters, sink);
            CU(cudaEventRecord(e1));
            CU(cudaEventSynchronize(e1));
            CU(cudaGetLastError());
            float ms = 0.f;
            CU(cudaEventElapsedTime(&ms, e0, e1));
            if (rep > 0) best = std::min(best, ms);
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        *gathers_per_s = (double)grid * kCalThreads * iters * kCalUnroll / (best * 1e-3);
        return igx::igx_set_error(IGAOS_PDHG_OK, "");
    } catch (const igx::CudaError& e) {
        return igx::igx_set_error(e.code, e.what());
    }
}
