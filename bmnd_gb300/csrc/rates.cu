// rates.cu -- measured issue rates of the units that bound this path's kernels.
//
// The deviance matching kernels are bound by the special-function unit (one
// log2 per voxel term) and the exact variance by FP32 fused multiply-adds; the
// copy bandwidth and the BF16 tensor rate are measured outside this library.
// Each kernel below runs independent dependency chains of one instruction kind
// on every SM, enough warps and chains to hide the latency, so the rate it
// reaches is the unit's throughput on this GPU at its current clock.
//
// The pilot net's tensor-core layers issue many small MMAs (M = 128, N = the
// channel count, K = 16); mma_rate_kernel measures the clocks one such MMA
// takes when one or more threads of a CTA issue them back to back.
#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "bmnd_common.cuh"
#include "tc_common.cuh"

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

// One CTA per SM.  `issuers` threads (lane 0 of warps 0 .. issuers - 1) each
// issue `n` tcgen05.mma kind::f16 (BF16 in, FP32 accumulate, M = 128, N = n_cols,
// K = 16, both operands no-swizzle K-major in zeroed shared memory: 4 KB of A
// and N x 32 bytes of B per MMA) into their own accumulator, then commit to
// one mbarrier; thread 0 waits for it (bounded) and records the CTA's clock64
// span.  Eight MMAs per loop trip with fixed descriptors keep the issuing
// thread's own instruction stream short.
constexpr uint32_t kMmaSmem = 40960;  // A at 0 (4 KB), B at 8 KB (up to 16 KB for N = 256)

__global__ void __launch_bounds__(128, 1) mma_rate_kernel(int n_cols, int issuers, int n, long long* clk, int* err) {
    extern __shared__ __align__(128) unsigned char mr_smem[];
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t slot;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    for (uint32_t i = tid; i < kMmaSmem / 16; i += blockDim.x)
        reinterpret_cast<uint4*>(mr_smem)[i] = make_uint4(0u, 0u, 0u, 0u);
    const uint32_t s0 = static_cast<uint32_t>(__cvta_generic_to_shared(mr_smem));
    const uint32_t b0 = static_cast<uint32_t>(__cvta_generic_to_shared(&bar));
    if (tid == 0) {
        mbar_init(b0, static_cast<uint32_t>(issuers));
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;\n" ::"r"(
                         static_cast<uint32_t>(__cvta_generic_to_shared(&slot)))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = slot;
    const long long t0 = clock64();
    if (warp < issuers && lane == 0) {
        const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | (static_cast<uint32_t>(n_cols >> 3) << 17) |
                               (static_cast<uint32_t>(128 >> 4) << 24);
        const uint64_t ad = umma_desc(s0, 128, 256);         // core matrices: K pairs 128 B apart, 8-row groups 256 B
        const uint64_t bd = umma_desc(s0 + 8192, 128, 256);
        const uint32_t d = tmem + static_cast<uint32_t>(warp * n_cols);
        for (int i = 0; i < n; i += 8) {
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const uint32_t acc = (i | u) != 0 ? 1u : 0u;
                asm volatile(
                    "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d),
                    "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
                    : "memory");
            }
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(b0)
                     : "memory");
    }
    if (tid == 0) {
        if (!mbar_wait(b0, 0, 2000000000ull)) atomicExch(err, 1);
        clk[blockIdx.x] = clock64() - t0;
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;\n" ::"r"(tmem) : "memory");
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

extern "C" int32_t bmnd_mma_rates(int32_t count, const int32_t* n_cols, const int32_t* issuers,
                                  double* clocks_per_mma, void* d_scratch, uint64_t stream) {
    clear_error();
    if (count < 0 || (count > 0 && (!n_cols || !issuers || !clocks_per_mma || !d_scratch)))
        return fail(BMND_ERR_INVALID_ARG, "null argument");
    for (int32_t i = 0; i < count; ++i) {
        const int32_t nc = n_cols[i], is = issuers[i];
        if (nc < 16 || nc > 256 || nc % 16 != 0 || is < 1 || is > 4 || nc * is > 512)
            return fail(BMND_ERR_INVALID_ARG,
                        "mma rate: N must be 16..256 in steps of 16, 1..4 issuers, N x issuers <= 512");
    }
    if (count == 0) return BMND_OK;
    int dev = 0, sms = 0;
    BMND_CUDA_TRY(cudaGetDevice(&dev));
    BMND_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    long long* clk = static_cast<long long*>(d_scratch);
    int* err = reinterpret_cast<int*>(clk + sms);
    std::vector<long long> host(static_cast<size_t>(sms));
    constexpr int kMmas = 4096;
    for (int32_t i = 0; i < count; ++i) {
        BMND_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), s));
        int per_sm = 0, nsm = 0;
        // one CTA per SM: the shared memory request leaves room for no second CTA
        const size_t smem = 120 * 1024;
        if (int32_t rc =
                kernel_residency(reinterpret_cast<const void*>(mma_rate_kernel), 128, smem, false, &per_sm, &nsm))
            return rc;
        mma_rate_kernel<<<sms, 128, smem, s>>>(n_cols[i], issuers[i], kMmas / issuers[i], clk, err);
        BMND_LAUNCH_CHECK("mma_rate_kernel");
        int herr = 0;
        BMND_CUDA_TRY(cudaMemcpyAsync(host.data(), clk, sizeof(long long) * sms, cudaMemcpyDeviceToHost, s));
        BMND_CUDA_TRY(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, s));
        BMND_CUDA_TRY(cudaStreamSynchronize(s));
        if (herr) return fail(BMND_ERR_TIMEOUT, "mma rate: the completion wait ran out");
        double sum = 0.0;
        for (int j = 0; j < sms; ++j) sum += static_cast<double>(host[j]);
        const int per_issuer = (kMmas / issuers[i] + 7) / 8 * 8;
        clocks_per_mma[i] = sum / sms / (static_cast<double>(per_issuer) * issuers[i]);
    }
    return BMND_OK;
}
