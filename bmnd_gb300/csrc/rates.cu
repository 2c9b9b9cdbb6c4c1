// rates.cu -- measured issue rates of the units that bound this path's kernels.
//
// The deviance matching kernels are bound by the special-function unit (one
// log2 per voxel term) and the exact variance by FP32 fused multiply-adds; the
// copy bandwidth and the BF16 tensor rate are measured outside this library.
// Each kernel below runs independent dependency chains of one instruction kind
// on every SM, enough warps and chains to hide the latency, so the rate it
// reaches is the unit's throughput on this GPU at its current clock.
#include <cuda_runtime.h>
#include <stdint.h>

#include "bmnd_common.cuh"

namespace bmnd {
namespace {

constexpr int kChains = 8;

// the form the matching kernels use (lg2.approx.ftz.f32)
__device__ __forceinline__ float mufu_lg2(float x) {
    float y;
    asm volatile("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// x <- log2(x) + 1 keeps x in [1, 2): one MUFU lg2 and one FP32 add per step
__global__ void lg2_rate_kernel(float* sink, int iters) {
    float x[kChains];
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = 1.0f + 0.01f * static_cast<float>((threadIdx.x + c) & 63);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < kChains; ++c) x[c] = mufu_lg2(x[c]) + 1.0f;
    }
    float s = 0.0f;
#pragma unroll
    for (int c = 0; c < kChains; ++c) s += x[c];
    if (s == 12345.0f) sink[0] = s;  // keeps the chains live
}

// x <- x * a + b with |a| < 1: one FP32 fused multiply-add per step
__global__ void ffma_rate_kernel(float* sink, int iters) {
    float x[kChains];
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = 0.5f + 0.001f * static_cast<float>((threadIdx.x + c) & 63);
    const float a = 0.999f, b = 0.001f;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < kChains; ++c) x[c] = fmaf(x[c], a, b);
    }
    float s = 0.0f;
#pragma unroll
    for (int c = 0; c < kChains; ++c) s += x[c];
    if (s == 12345.0f) sink[0] = s;
}

template <typename K>
int32_t time_rate(K kernel, int blocks, int threads, int iters, float* sink, cudaStream_t stream, double* per_s) {
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    BMND_CUDA_TRY(cudaEventCreate(&e0));
    BMND_CUDA_TRY(cudaEventCreate(&e1));
    kernel<<<blocks, threads, 0, stream>>>(sink, iters / 8);  // warm-up
    BMND_LAUNCH_CHECK("rate kernel");
    BMND_CUDA_TRY(cudaEventRecord(e0, stream));
    kernel<<<blocks, threads, 0, stream>>>(sink, iters);
    BMND_LAUNCH_CHECK("rate kernel");
    BMND_CUDA_TRY(cudaEventRecord(e1, stream));
    BMND_CUDA_TRY(cudaEventSynchronize(e1));
    float ms = 0.0f;
    BMND_CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
    (void)cudaEventDestroy(e0);
    (void)cudaEventDestroy(e1);
    *per_s = static_cast<double>(blocks) * threads * kChains * static_cast<double>(iters) / (ms * 1e-3);
    return BMND_OK;
}

}  // namespace
}  // namespace bmnd

using namespace bmnd;

extern "C" int32_t bmnd_unit_rates(double* lg2_per_s, double* ffma_per_s, void* d_sink, uint64_t stream) {
    clear_error();
    if (!lg2_per_s || !ffma_per_s || !d_sink) return fail(BMND_ERR_INVALID_ARG, "null argument");
    int dev = 0, sms = 0;
    BMND_CUDA_TRY(cudaGetDevice(&dev));
    BMND_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    float* sink = static_cast<float*>(d_sink);
    const int blocks = sms * 8, threads = 256;  // 64 warps per SM, 8 chains each
    if (int32_t rc = time_rate(lg2_rate_kernel, blocks, threads, 4096, sink, s, lg2_per_s)) return rc;
    return time_rate(ffma_rate_kernel, blocks, threads, 16384, sink, s, ffma_per_s);
}
