// ssdtc.cu -- SSD block matching on the fifth-generation tensor cores:
// the screening distances (blockmatching.py:332-336 restated as
// |a - b|^2 = |a|^2 + |b|^2 - 2 a.b, with the cross term as a dense product).
//
// References are sorted into spatial tiles (12^3 patch-grid positions in 3-D,
// 24^2 in 2-D) so that up to 128 nearby references share one union box of
// candidate positions.  Squared distances do not change when both patches are
// shifted by the same constant, so every tile works on values centred on mu_t,
// the mean of its references' patches: the error of the BF16 products scales
// with the centred norms, which for smooth data are far below the raw ones.
// One CTA takes a block of references of one tile:
//   A (M = 128 references x K = patch, zero padded to a multiple of 16) holds
//     their centred patches split as a = hi + lo, hi = bf16(a), lo = bf16(a - hi);
//   for every chunk of 128 candidates of the union box (x fastest), the CTA
//     gathers the candidates' patches into B (N = 128 x K, the same split)
//     and one thread issues 3 K/16 tcgen05.mma (kind::f16, BF16 in, FP32
//     accumulate in tensor memory): hi.hi + hi.lo + lo.hi, the cross term to
//     about 2^-16 relative;
//   the epilogue reads the accumulator (tcgen05.ld), and writes for every
//     (reference, candidate in its window) d~ = |a|^2 + |b|^2 - 2 a.b to the
//     reference's row of screening distances, in window order.
// Two B buffers and two accumulators let the gather of chunk i, the MMAs of
// chunk i and the epilogue of chunk i - 1 overlap.  Operands are no-swizzle
// K-major core matrices (8 rows x 16 bytes); the patches of the candidates are
// read from the volume in place (consecutive candidates are consecutive x, so
// the gathers are coalesced).  Every mbarrier wait is bounded; a timeout sets
// *err, which makes the selection kernel hand every reference to the exact
// kernel.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "bmnd_common.cuh"
#include "tc_common.cuh"

namespace bmnd {
namespace {

constexpr int kTcThreads = 256;  // eight warps: gathers and epilogue; thread 0 also issues the MMAs
constexpr int kTcM = 128;        // references per block (MMA M)
constexpr int kTcN = 128;        // candidates per chunk (MMA N)
constexpr uint64_t kTcWaitNs = 1000000000ull;

template <int KP>
struct ScreenSmem {
    static constexpr uint32_t lbo = kTcM * 16;      // next 8 K elements: 128 rows x 16 bytes
    static constexpr uint32_t mat = (KP / 8) * lbo;  // one 128 x KP BF16 operand
    static constexpr uint32_t a_hi = 0, a_lo = mat;
    static constexpr uint32_t b(int s, int lo) { return (2 + 2 * s + lo) * mat; }
    static constexpr uint32_t bytes = 6 * mat;  // A hi/lo, two B buffers hi/lo
};

__device__ __forceinline__ uint32_t pack_bf16(float x, float y) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(x, y);
    return *reinterpret_cast<const uint32_t*>(&v);
}

// eight values of one operand row -> 16 bytes of hi and 16 bytes of lo
__device__ __forceinline__ void split_store(const float (&v)[8], unsigned char* hi, unsigned char* lo) {
    float h[8], l[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) {
        h[e] = __bfloat162float(__float2bfloat16_rn(v[e]));
        l[e] = v[e] - h[e];  // exact: h holds the leading 8 bits of v
    }
    *reinterpret_cast<uint4*>(hi) = make_uint4(pack_bf16(h[0], h[1]), pack_bf16(h[2], h[3]), pack_bf16(h[4], h[5]),
                                               pack_bf16(h[6], h[7]));
    *reinterpret_cast<uint4*>(lo) = make_uint4(pack_bf16(l[0], l[1]), pack_bf16(l[2], l[3]), pack_bf16(l[4], l[5]),
                                               pack_bf16(l[6], l[7]));
}

// per patch origin: sum of squares of its patch (float32, patch order); the
// rows of origins off the patch grid stay unread
template <int ND, int B0, int B1, int B2>
__global__ void sqbox_kernel(const float* __restrict__ src, SsdScreenArgs a, int64_t nvox, float* __restrict__ out,
                             float* __restrict__ out_sum) {
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < nvox;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        int64_t rem = i;
        bool ok = true;
        int c[3] = {0, 0, 0};
        for (int d = ND - 1; d >= 0; --d) {
            const int n = a.counts[d] + a.block[d] - 1;
            c[d] = static_cast<int>(rem % n);
            rem /= n;
            ok = ok && c[d] < a.counts[d];
        }
        float s = 0.0f, s1 = 0.0f;
        if (ok) {
#pragma unroll 1
            for (int p0 = 0; p0 < B0; ++p0)
#pragma unroll
                for (int p1 = 0; p1 < (ND > 1 ? B1 : 1); ++p1) {
                    const float* row = src + i + p0 * a.vstride[0] + (ND > 1 ? p1 * a.vstride[1] : 0);
                    if (ND == 3) {
#pragma unroll
                        for (int p2 = 0; p2 < B2; ++p2) {
                            const float v = __ldg(row + p2);
                            s = fmaf(v, v, s);
                            s1 += v;
                        }
                    } else {
                        const float v = __ldg(row);
                        s = fmaf(v, v, s);
                        s1 += v;
                    }
                }
        }
        out[i] = s;
        out_sum[i] = s1;
    }
}

// tile of a reference: its patch-grid position divided by the tile edge per axis
__device__ __forceinline__ int ref_tile(const SsdScreenArgs& a, const int32_t* refs, int64_t r) {
    int t = 0;
    for (int d = 0; d < a.ndim; ++d) t = t * a.tiles[d] + refs[r * a.ndim + d] / a.tile_edge[d];
    return t;
}

__global__ void tile_count_kernel(SsdScreenArgs a, int64_t n_refs, int32_t* __restrict__ cnt) {
    for (int64_t r = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; r < n_refs;
         r += static_cast<int64_t>(gridDim.x) * blockDim.x)
        atomicAdd(cnt + ref_tile(a, a.refs, r), 1);
}

// order inside a tile does not matter: every reference's row is its own
__global__ void tile_fill_kernel(SsdScreenArgs a, int64_t n_refs, const int32_t* __restrict__ start,
                                 int32_t* __restrict__ cursor, int32_t* __restrict__ perm) {
    for (int64_t r = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; r < n_refs;
         r += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int t = ref_tile(a, a.refs, r);
        perm[start[t] + atomicAdd(cursor + t, 1)] = static_cast<int32_t>(r);
    }
}

// per tile: the mean value of its references' patches (one warp per tile,
// a fixed order), the centre of the tile's screening
__global__ void tile_mean_kernel(SsdScreenArgs a, int P, float* __restrict__ mu) {
    const int lane = threadIdx.x & 31;
    const int warps = static_cast<int>(gridDim.x * (blockDim.x >> 5));
    for (int t = static_cast<int>(blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)); t < a.n_tiles; t += warps) {
        const int t0 = a.tile_start[t], t1 = a.tile_start[t + 1];
        float s = 0.0f;
        for (int i = t0 + lane; i < t1; i += 32) {
            const int32_t r = a.perm[i];
            int64_t org = 0;
            for (int d = 0; d < a.ndim; ++d) org += static_cast<int64_t>(a.refs[static_cast<int64_t>(r) * a.ndim + d]) *
                                                  a.vstride[d];
            s += __ldg(a.sums + org);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        const float m = t1 > t0 ? s / (static_cast<float>(t1 - t0) * static_cast<float>(P)) : 0.0f;
        if (lane == 0) mu[t] = m;
        for (int i = t0 + lane; i < t1; i += 32) a.ref_mu[a.perm[i]] = m;
    }
}

template <int ND, int B0, int B1, int B2>
__global__ void __launch_bounds__(kTcThreads, 1) ssd_screen_tc_kernel(SsdScreenArgs a) {
    constexpr int P = B0 * B1 * B2;
    constexpr int KP = (P + 15) / 16 * 16;
    using S = ScreenSmem<KP>;
    extern __shared__ __align__(128) unsigned char tc_raw[];
    __shared__ __align__(8) uint64_t bars[2];
    __shared__ uint32_t tmem_slot;
    __shared__ int abort_flag;
    __shared__ int32_t poff[P];
    __shared__ int32_t r_glob[kTcM], r_lo[3][kTcM], r_ext[3][kTcM];
    __shared__ float r_na[kTcM];
    __shared__ int32_t c_crd[2][3][kTcN];
    __shared__ float c_nb[2][kTcN];
    __shared__ int ub_lo[3], ub_ext[3];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t sbase = static_cast<uint32_t>(__cvta_generic_to_shared(tc_raw));
    const uint32_t bar0 = static_cast<uint32_t>(__cvta_generic_to_shared(bars));
    volatile int* abort_v = &abort_flag;

    if (tid == 0) {
        mbar_init(bar0, 1);
        mbar_init(bar0 + 8, 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        abort_flag = (sbase & 127u) != 0u ? 1 : 0;
        if (abort_flag) atomicExch(a.err, 2);
    }
    for (int p = tid; p < P; p += blockDim.x) {
        int rem = p;
        int64_t off = 0;
        for (int d = ND - 1; d >= 0; --d) {
            off += static_cast<int64_t>(rem % a.block[d]) * a.vstride[d];
            rem /= a.block[d];
        }
        poff[p] = static_cast<int32_t>(off);
    }
    if (warp == 0) {
        const uint32_t slot = static_cast<uint32_t>(__cvta_generic_to_shared(&tmem_slot));
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(slot), "r"(256)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_slot;
    constexpr uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | (static_cast<uint32_t>(kTcN >> 3) << 17) |
                               (static_cast<uint32_t>(kTcM >> 4) << 24);
    int it = 0;  // chunks issued by this CTA (mbarrier phases)

    // epilogue of the chunk issued as number `j` (accumulator j & 1)
    auto epilogue = [&](int j, int64_t chunk, int nref) {
        const int s = j & 1;
        bool got = mbar_wait(bar0 + 8u * s, (j >> 1) & 1, kTcWaitNs);
        if (!got) {
            *abort_v = 1;
            atomicExch(a.err, 1);
        }
        tc_fence_after();
        const int q = warp & 3, half = warp >> 2;
        const int m = 32 * q + lane;
        uint32_t r[64];
#pragma unroll
        for (int c0 = 0; c0 < 64; c0 += 16) {
            const uint32_t taddr = tmem + (static_cast<uint32_t>(32 * q) << 16) + static_cast<uint32_t>(s) * kTcN +
                                   static_cast<uint32_t>(half * 64 + c0);
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, "
                "%12, %13, %14, %15}, [%16];\n"
                : "=r"(r[c0 + 0]), "=r"(r[c0 + 1]), "=r"(r[c0 + 2]), "=r"(r[c0 + 3]), "=r"(r[c0 + 4]),
                  "=r"(r[c0 + 5]), "=r"(r[c0 + 6]), "=r"(r[c0 + 7]), "=r"(r[c0 + 8]), "=r"(r[c0 + 9]),
                  "=r"(r[c0 + 10]), "=r"(r[c0 + 11]), "=r"(r[c0 + 12]), "=r"(r[c0 + 13]), "=r"(r[c0 + 14]),
                  "=r"(r[c0 + 15])
                : "r"(taddr));
        }
        asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
        if (!got || m >= nref) return;
        const int64_t rg = r_glob[m];
        float* row = a.out + rg * a.wmax;
        const float na = r_na[m];
        int lo[3], ex[3];
#pragma unroll
        for (int d = 0; d < ND; ++d) {
            lo[d] = r_lo[d][m];
            ex[d] = r_ext[d][m];
        }
        const int64_t ncand = static_cast<int64_t>(ub_ext[0]) * (ND > 1 ? ub_ext[1] : 1) * (ND > 2 ? ub_ext[2] : 1);
        const int64_t cbase = chunk * kTcN + half * 64;
#pragma unroll
        for (int jj = 0; jj < 64; ++jj) {
            const int n = half * 64 + jj;
            int64_t widx = 0;
            bool in = cbase + jj < ncand;
#pragma unroll
            for (int d = 0; d < ND; ++d) {
                const int o = c_crd[s][d][n] - lo[d];
                in = in && o >= 0 && o < ex[d];
                widx = widx * ex[d] + o;
            }
            if (in) row[widx] = na + c_nb[s][n] - 2.0f * __uint_as_float(r[jj]);
        }
    };

    for (int t = blockIdx.x; t < a.n_tiles && !*abort_v; t += gridDim.x) {
        const int t0 = a.tile_start[t], t1 = a.tile_start[t + 1];
        const float mu = __ldg(a.mu + t);
        for (int mb = t0; mb < t1 && !*abort_v; mb += kTcM) {
            const int nref = min(kTcM, t1 - mb);
            // references of the block: position, clipped window, norm
            if (tid < kTcM) {
                if (tid < nref) {
                    const int32_t rg = a.perm[mb + tid];
                    r_glob[tid] = rg;
                    int64_t org = 0;
                    for (int d = 0; d < ND; ++d) {
                        const int cd = a.refs[static_cast<int64_t>(rg) * ND + d];
                        const int l = max(cd - a.radius[d], 0);
                        r_lo[d][tid] = l;
                        r_ext[d][tid] = min(cd + a.radius[d], a.counts[d] - 1) - l + 1;
                        org += static_cast<int64_t>(cd) * a.vstride[d];
                    }
                    r_na[tid] = centred_norm(__ldg(a.norms + org), __ldg(a.sums + org), mu, P);
                } else {
                    r_glob[tid] = -1;
                }
            }
            __syncthreads();
            if (tid == 0) {
                for (int d = 0; d < ND; ++d) {
                    int l = r_lo[d][0], h = r_lo[d][0] + r_ext[d][0] - 1;
                    for (int i = 1; i < nref; ++i) {
                        l = min(l, r_lo[d][i]);
                        h = max(h, r_lo[d][i] + r_ext[d][i] - 1);
                    }
                    ub_lo[d] = l;
                    ub_ext[d] = h - l + 1;
                }
            }
            // A: the references' patches (rows >= nref zero)
            for (int item = tid; item < kTcM * (KP / 8); item += kTcThreads) {
                const int m = item % kTcM, kg = item / kTcM;
                float v[8];
                int64_t org = 0;
                if (m < nref) {
                    const int32_t rg = a.perm[mb + m];
                    for (int d = 0; d < ND; ++d) org += static_cast<int64_t>(a.refs[static_cast<int64_t>(rg) * ND + d]) *
                                                        a.vstride[d];
                }
#pragma unroll
                for (int e = 0; e < 8; ++e) {
                    const int p = 8 * kg + e;
                    v[e] = (m < nref && p < P) ? __ldg(a.src + org + poff[p]) - mu : 0.0f;
                }
                const uint32_t off = static_cast<uint32_t>(kg) * S::lbo + static_cast<uint32_t>(m >> 3) * 128u +
                                     static_cast<uint32_t>(m & 7) * 16u;
                split_store(v, tc_raw + S::a_hi + off, tc_raw + S::a_lo + off);
            }
            __syncthreads();
            const int64_t ncand = static_cast<int64_t>(ub_ext[0]) * (ND > 1 ? ub_ext[1] : 1) * (ND > 2 ? ub_ext[2] : 1);
            const int64_t nchunks = (ncand + kTcN - 1) / kTcN;
            for (int64_t ch = 0; ch <= nchunks; ++ch) {
                const int s = it & 1;
                if (ch < nchunks) {
                    // B: the chunk's candidates (columns >= ncand zero), their coordinates and norms
                    for (int item = tid; item < kTcN * (KP / 8); item += kTcThreads) {
                        const int n = item % kTcN, kg = item / kTcN;
                        const int64_t j = ch * kTcN + n;
                        const bool ok = j < ncand;
                        int64_t rem = ok ? j : 0, org = 0;
                        int crd[3] = {0, 0, 0};
#pragma unroll
                        for (int d = ND - 1; d >= 0; --d) {
                            crd[d] = ub_lo[d] + static_cast<int>(rem % ub_ext[d]);
                            rem /= ub_ext[d];
                            org += static_cast<int64_t>(crd[d]) * a.vstride[d];
                        }
                        if (kg == 0) {
#pragma unroll
                            for (int d = 0; d < ND; ++d) c_crd[s][d][n] = crd[d];
                            c_nb[s][n] = ok ? centred_norm(__ldg(a.norms + org), __ldg(a.sums + org), mu, P) : 0.0f;
                        }
                        float v[8];
#pragma unroll
                        for (int e = 0; e < 8; ++e) {
                            const int p = 8 * kg + e;
                            v[e] = (ok && p < P) ? __ldg(a.src + org + poff[p]) - mu : 0.0f;
                        }
                        const uint32_t off = static_cast<uint32_t>(kg) * S::lbo +
                                             static_cast<uint32_t>(n >> 3) * 128u + static_cast<uint32_t>(n & 7) * 16u;
                        split_store(v, tc_raw + S::b(s, 0) + off, tc_raw + S::b(s, 1) + off);
                    }
                    // generic-proxy writes made visible to the tensor core's async proxy
                    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
                }
                __syncthreads();
                if (ch < nchunks && tid == 0 && !*abort_v) {
                    tc_fence_after();
                    const uint32_t d_tmem = tmem + static_cast<uint32_t>(s) * kTcN;
#pragma unroll
                    for (int prod = 0; prod < 3; ++prod) {
                        const uint32_t aoff = prod == 2 ? S::a_lo : S::a_hi;
                        const uint32_t boff = S::b(s, prod == 1 ? 1 : 0);
                        const uint64_t ad0 = umma_desc(sbase + aoff, S::lbo, 128);
                        const uint64_t bd0 = umma_desc(sbase + boff, S::lbo, 128);
#pragma unroll
                        for (int ks = 0; ks < KP / 16; ++ks) {
                            // start-address field += 2 core matrices along K (stays below 2^14)
                            const uint64_t step = static_cast<uint64_t>(ks) * (2 * S::lbo / 16);
                            const uint32_t acc = (prod | ks) != 0 ? 1u : 0u;
                            asm volatile(
                                "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                                "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
                                "l"(ad0 + step), "l"(bd0 + step), "r"(idesc), "r"(acc)
                                : "memory");
                        }
                    }
                    asm volatile(
                        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                            bar0 + 8u * s)
                        : "memory");
                }
                if (ch > 0 && !*abort_v) epilogue(it - 1, ch - 1, nref);
                tc_fence_before();
                __syncthreads();
                if (ch < nchunks) ++it;
                if (*abort_v) break;
            }
        }
    }
    // MMAs still in flight after an abort: wait (bounded) for the last commit
    if (tid == 0 && *abort_v && it > 0) (void)mbar_wait(bar0 + 8u * ((it - 1) & 1), ((it - 1) >> 1) & 1, kTcWaitNs);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(256) : "memory");
}

int64_t grid_cap(int64_t n, int threads, int64_t cap) {
    int64_t b = (n + threads - 1) / threads;
    if (b < 1) b = 1;
    return b > cap ? cap : b;
}

template <int ND, int B0, int B1, int B2>
int32_t run_screen(SsdScreenArgs a, int64_t nvox, cudaStream_t stream) {
    sqbox_kernel<ND, B0, B1, B2><<<static_cast<unsigned>(grid_cap(nvox, 256, 152 * 32)), 256, 0, stream>>>(
        a.src, a, nvox, const_cast<float*>(a.norms), const_cast<float*>(a.sums));
    BMND_LAUNCH_CHECK("sqbox_kernel");
    tile_mean_kernel<<<static_cast<unsigned>(grid_cap(a.n_tiles, 8, 152 * 16)), 256, 0, stream>>>(
        a, B0 * B1 * B2, const_cast<float*>(a.mu));
    BMND_LAUNCH_CHECK("tile_mean_kernel");
    constexpr int KP = (B0 * B1 * B2 + 15) / 16 * 16;
    using S = ScreenSmem<KP>;
    auto kernel = ssd_screen_tc_kernel<ND, B0, B1, B2>;
    int per_sm = 0, sms = 0;
    if (int32_t rc = kernel_residency(reinterpret_cast<const void*>(kernel), kTcThreads, S::bytes, false, &per_sm,
                                      &sms))
        return rc;
    if (per_sm < 1) return fail(BMND_ERR_UNSUPPORTED, "SSD screening kernel does not fit on an SM");
    int64_t blocks = static_cast<int64_t>(sms) * per_sm;
    if (blocks > a.n_tiles) blocks = a.n_tiles;
    if (blocks < 1) return BMND_OK;
    kernel<<<static_cast<unsigned>(blocks), kTcThreads, S::bytes, stream>>>(a);
    BMND_LAUNCH_CHECK("ssd_screen_tc_kernel");
    return BMND_OK;
}

}  // namespace

bool ssd_screen_shape(int ndim, const int32_t* block) {
    return (ndim == 2 && block[0] == 8 && block[1] == 8) ||
           (ndim == 3 && block[0] == 5 && block[1] == 5 && block[2] == 5) ||
           (ndim == 3 && block[0] == 4 && block[1] == 4 && block[2] == 4);
}

SsdScratchLayout ssd_scratch_layout(int ndim, const int32_t* counts, const int32_t* block, const int32_t* radius,
                                    int64_t n_refs) {
    auto a256 = [](uint64_t v) { return (v + 255) & ~uint64_t(255); };
    SsdScratchLayout L{};
    int64_t nvox = 1, wmax = 1, n_tiles = 1;
    for (int d = 0; d < ndim; ++d) {
        nvox *= counts[d] + block[d] - 1;
        wmax *= std::min<int64_t>(2 * radius[d] + 1, counts[d]);
        const int edge = ndim == 3 ? 12 : 24;
        n_tiles *= (counts[d] + edge - 1) / edge;
    }
    L.wmax = wmax;
    L.n_tiles = n_tiles;
    uint64_t off = 0;
    auto take = [&](uint64_t bytes) {
        const uint64_t o = off;
        off += a256(bytes);
        return o;
    };
    L.o_norms = take(4ull * static_cast<uint64_t>(nvox));
    L.o_psum = take(4ull * static_cast<uint64_t>(nvox));
    L.o_mu = take(4ull * static_cast<uint64_t>(n_tiles));
    L.o_rmu = take(4ull * static_cast<uint64_t>(n_refs));
    L.o_rows = take(4ull * static_cast<uint64_t>(n_refs) * static_cast<uint64_t>(wmax));
    L.o_start = take(4ull * static_cast<uint64_t>(n_tiles + 1));
    L.o_cursor = take(4ull * static_cast<uint64_t>(n_tiles));
    L.o_sums = take(4ull * static_cast<uint64_t>(n_tiles / 1024 + 2));
    L.o_perm = take(4ull * static_cast<uint64_t>(n_refs));
    L.o_err = take(4);
    L.bytes = off;
    return L;
}

int32_t launch_ssd_screen(SsdScreenArgs a, int64_t nvox, int64_t n_refs, char* base, const SsdScratchLayout& L,
                          cudaStream_t stream) {
    a.norms = reinterpret_cast<float*>(base + L.o_norms);
    a.sums = reinterpret_cast<float*>(base + L.o_psum);
    a.mu = reinterpret_cast<float*>(base + L.o_mu);
    a.ref_mu = reinterpret_cast<float*>(base + L.o_rmu);
    a.out = reinterpret_cast<float*>(base + L.o_rows);
    a.wmax = L.wmax;
    a.err = reinterpret_cast<int*>(base + L.o_err);
    a.n_tiles = static_cast<int>(L.n_tiles);
    for (int d = 0; d < 3; ++d) {
        a.tile_edge[d] = a.ndim == 3 ? 12 : 24;
        a.tiles[d] = d < a.ndim ? (a.counts[d] + a.tile_edge[d] - 1) / a.tile_edge[d] : 1;
    }
    int32_t* start = reinterpret_cast<int32_t*>(base + L.o_start);
    int32_t* cursor = reinterpret_cast<int32_t*>(base + L.o_cursor);
    int32_t* sums = reinterpret_cast<int32_t*>(base + L.o_sums);
    int32_t* perm = reinterpret_cast<int32_t*>(base + L.o_perm);
    a.tile_start = start;
    a.perm = perm;
    BMND_CUDA_TRY(cudaMemsetAsync(a.err, 0, sizeof(int), stream));
    BMND_CUDA_TRY(cudaMemsetAsync(cursor, 0, 4ull * static_cast<uint64_t>(L.n_tiles), stream));
    const unsigned gb = static_cast<unsigned>(grid_cap(n_refs, 256, 152 * 16));
    tile_count_kernel<<<gb, 256, 0, stream>>>(a, n_refs, cursor);
    BMND_LAUNCH_CHECK("tile_count_kernel");
    if (int32_t rc = launch_exclusive_scan(cursor, L.n_tiles, start, sums, stream)) return rc;
    BMND_CUDA_TRY(cudaMemsetAsync(cursor, 0, 4ull * static_cast<uint64_t>(L.n_tiles), stream));
    tile_fill_kernel<<<gb, 256, 0, stream>>>(a, n_refs, start, cursor, perm);
    BMND_LAUNCH_CHECK("tile_fill_kernel");
    const int* b = a.block;
    if (a.ndim == 2 && b[0] == 8 && b[1] == 8) return run_screen<2, 8, 8, 1>(a, nvox, stream);
    if (a.ndim == 3 && b[0] == 5 && b[1] == 5 && b[2] == 5) return run_screen<3, 5, 5, 5>(a, nvox, stream);
    if (a.ndim == 3 && b[0] == 4 && b[1] == 4 && b[2] == 4) return run_screen<3, 4, 4, 4>(a, nvox, stream);
    return fail(BMND_ERR_UNSUPPORTED, "no tensor-core SSD screening for this patch shape");
}

}  // namespace bmnd
