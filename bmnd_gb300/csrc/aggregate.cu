// aggregate.cu -- deterministic weighted aggregation without global atomics on
// floating-point data (replaces the scatter-add of patchaggregation.py:170-199
// and the final division of bmndalgo.py:626-631, :1039-1044).
//
// The reference adds every filtered patch into float32 numerator and
// denominator volumes in schedule order.  Here each voxel's sums have a fixed
// order of their own, so two runs give the same bits:
//   1. entry index: every (group, member) entry is listed under its patch
//      origin (the member's patch-grid lin), sorted by (group, member); entry
//      counts use integer atomics (exact), the per-origin order is a sort;
//   2. the group filter writes each member's weighted filtered patch
//      fl(y * fl(w * window)) to the store row of its entry (coalesced rows)
//      and its weight w beside it, instead of adding them into the volumes;
//   3. origin sums: per origin and patch offset p, the sum over its entries,
//      stored as float32 planes PC[p][origin] (one CTA per 32 consecutive
//      origins, transposed through shared memory so that every plane row is
//      written with full 128-byte lines), and the sum of the entries' weights
//      W[origin];
//   4. gather and finalize: one thread per voxel x sums, in patch-offset
//      order, num = sum_p PC[p][x - p] and den = sum_p window[p] W[x - p], then
//      writes den > 0 ? num / (den + eps) : noisy in float32.
// Every plane read in step 4 is coalesced (consecutive voxels read consecutive
// origins of the same plane).  The sums are compensated: a float32 pair (s, c)
// updated by Knuth's error-free TwoSum carries about 48 significant bits, the
// accuracy of a float64 accumulator, on the FP32 pipe (the FP64 pipe of this
// GPU runs at a small fraction of the FP32 rate).  A fixed order makes the
// pair, and so the result, the same on every run.
#include <cuda_runtime.h>
#include <stdint.h>

#include "bmnd_common.cuh"

namespace bmnd {
namespace {

constexpr int kScanBlock = 1024;

// compensated sum: s + c holds the exact running sum to about 2^-48 relative
struct Sum2 {
    float s = 0.0f, c = 0.0f;
    __device__ __forceinline__ void add(float x) {
        // Knuth's TwoSum, every operation rounded on its own (no contraction)
        const float t = __fadd_rn(s, x);
        const float z = __fsub_rn(t, s);
        const float e = __fadd_rn(__fsub_rn(s, __fsub_rn(t, z)), __fsub_rn(x, z));
        c = __fadd_rn(c, e);
        s = t;
    }
    __device__ __forceinline__ float value() const { return __fadd_rn(s, c); }
};

// entries per origin (integer atomics: the counts do not depend on order)
__global__ void entry_count_kernel(const int32_t* __restrict__ sel, const int32_t* __restrict__ count,
                                   int64_t n_refs, int max_stack, int32_t* __restrict__ per_origin) {
    const int64_t total = n_refs * max_stack;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < total;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int64_t g = i / max_stack;
        const int m = static_cast<int>(i - g * max_stack);
        if (m < count[g]) atomicAdd(per_origin + sel[i], 1);
    }
}

// exclusive scan, phase 1: within blocks of kScanBlock values, plus each block's total
__global__ void scan_block_kernel(const int32_t* __restrict__ in, int64_t n, int32_t* __restrict__ out,
                                  int32_t* __restrict__ block_sums) {
    __shared__ int32_t warp_tot[kScanBlock / 32];
    const int64_t base = static_cast<int64_t>(blockIdx.x) * kScanBlock;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int64_t i = base + tid;
    const int32_t v = i < n ? in[i] : 0;
    int32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int32_t t = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += t;
    }
    if (lane == 31) warp_tot[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int32_t w = warp_tot[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int32_t t = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += t;
        }
        warp_tot[lane] = w;  // inclusive over warps
    }
    __syncthreads();
    const int32_t before = warp == 0 ? 0 : warp_tot[warp - 1];
    if (i < n) out[i] = before + x - v;
    if (tid == kScanBlock - 1) block_sums[blockIdx.x] = before + x;
}

// exclusive scan, phase 2: the block totals, one block looping over them
__global__ void scan_sums_kernel(int32_t* __restrict__ sums, int64_t nb, int32_t* __restrict__ grand_total) {
    __shared__ int32_t warp_tot[kScanBlock / 32];
    __shared__ int32_t carry;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) carry = 0;
    __syncthreads();
    for (int64_t base = 0; base < nb; base += kScanBlock) {
        const int64_t i = base + tid;
        const int32_t v = i < nb ? sums[i] : 0;
        int32_t x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int32_t t = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += t;
        }
        if (lane == 31) warp_tot[warp] = x;
        __syncthreads();
        if (warp == 0) {
            int32_t w = warp_tot[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int32_t t = __shfl_up_sync(0xffffffffu, w, o);
                if (lane >= o) w += t;
            }
            warp_tot[lane] = w;
        }
        __syncthreads();
        const int32_t before = warp == 0 ? 0 : warp_tot[warp - 1];
        const int32_t c = carry;
        if (i < nb) sums[i] = c + before + x - v;
        __syncthreads();
        if (tid == kScanBlock - 1) carry = c + before + x;
        __syncthreads();
    }
    if (tid == 0) *grand_total = carry;
}

// exclusive scan, phase 3: add each block's offset; start[n] = the total
__global__ void scan_add_kernel(int32_t* __restrict__ out, int64_t n, const int32_t* __restrict__ block_sums,
                                const int32_t* __restrict__ grand_total) {
    const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (i < n) out[i] += block_sums[i / kScanBlock];
    if (i == n) out[n] = *grand_total;
}

// slots: an entry takes the next free slot of its origin (order fixed below)
__global__ void entry_fill_kernel(const int32_t* __restrict__ sel, const int32_t* __restrict__ count,
                                  int64_t n_refs, int max_stack, const int32_t* __restrict__ start,
                                  int32_t* __restrict__ cursor, int32_t* __restrict__ entries) {
    const int64_t total = n_refs * max_stack;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < total;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int64_t g = i / max_stack;
        const int m = static_cast<int>(i - g * max_stack);
        if (m < count[g]) {
            const int32_t o = sel[i];
            entries[start[o] + atomicAdd(cursor + o, 1)] = static_cast<int32_t>(i);
        }
    }
}

// each origin's entries in ascending (group, member) order, and every entry's slot
__global__ void entry_sort_kernel(const int32_t* __restrict__ start, int64_t n_lins, int32_t* __restrict__ entries,
                                  int32_t* __restrict__ slot_of) {
    for (int64_t o = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; o < n_lins;
         o += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int32_t lo = start[o], hi = start[o + 1];
        for (int32_t i = lo + 1; i < hi; ++i) {
            const int32_t v = entries[i];
            int32_t j = i - 1;
            while (j >= lo && entries[j] > v) {
                entries[j + 1] = entries[j];
                --j;
            }
            entries[j + 1] = v;
        }
        for (int32_t i = lo; i < hi; ++i) slot_of[entries[i]] = i;
    }
}

// step 3: per origin, compensated sums of its entries' rows.  One CTA of eight
// warps per 32 consecutive origins: warp w sums origins w, w + 8, w + 16,
// w + 24 (lane l takes the patch offsets l, l + 32, ...; every row read is a
// coalesced 128-byte line), the sums go to a shared tile, and the warps then
// write the planes PC[p][origin] transposed, 32 consecutive origins per line.
constexpr int kSumThreads = 256;

template <int PJ>  // patch offsets per lane: ceil(P / 32)
__global__ void __launch_bounds__(kSumThreads) origin_sum_kernel(const float* __restrict__ store, int row,
                                                                 const float* __restrict__ wstore,
                                                                 const int32_t* __restrict__ start, int64_t n_lins,
                                                                 int P, float* __restrict__ planes,
                                                                 float* __restrict__ wsum) {
    constexpr int kPad = 32 * PJ + 1;  // conflict-free transposed reads
    __shared__ float tile[32 * kPad];
    __shared__ int32_t bounds[33];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int64_t o0 = static_cast<int64_t>(blockIdx.x) * 32; o0 < n_lins; o0 += static_cast<int64_t>(gridDim.x) * 32) {
        if (threadIdx.x < 33) {
            const int64_t o = o0 + threadIdx.x;
            bounds[threadIdx.x] = __ldg(start + (o < n_lins ? o : n_lins));
        }
        __syncthreads();
        for (int oi = w; oi < 32; oi += kSumThreads / 32) {
            Sum2 acc[PJ];
            Sum2 ws;
            const int32_t lo = bounds[oi], hi = bounds[oi + 1];
            for (int32_t s = lo; s < hi; ++s) {
                const float* r = store + static_cast<int64_t>(s) * row;
#pragma unroll
                for (int j = 0; j < PJ; ++j) {
                    const int p = lane + 32 * j;
                    if (p < P) acc[j].add(__ldg(r + p));
                }
                ws.add(__ldg(wstore + s));
            }
#pragma unroll
            for (int j = 0; j < PJ; ++j) tile[oi * kPad + lane + 32 * j] = acc[j].value();
            if (lane == 0 && o0 + oi < n_lins) wsum[o0 + oi] = ws.value();
        }
        __syncthreads();
        const int64_t o = o0 + lane;
        if (o < n_lins)
            for (int p = w; p < P; p += kSumThreads / 32)
                planes[static_cast<int64_t>(p) * n_lins + o] = tile[lane * kPad + p];
        __syncthreads();
    }
}

// volume geometry padded to three axes (leading axes of extent 1)
struct Vol3 {
    int shape[3], block[3], counts[3];
    int64_t nvox, n_lins;
    __device__ explicit Vol3(const BmndStageParams& sp) {
        for (int d = 0; d < 3; ++d) shape[d] = block[d] = counts[d] = 1;
        const int off = 3 - sp.ndim;
        for (int d = 0; d < sp.ndim; ++d) {
            shape[off + d] = sp.shape[d];
            block[off + d] = sp.block[d];
            counts[off + d] = sp.shape[d] - sp.block[d] + 1;
        }
        nvox = static_cast<int64_t>(shape[0]) * shape[1] * shape[2];
        n_lins = static_cast<int64_t>(counts[0]) * counts[1] * counts[2];
    }
};

// step 4: num and den of every voxel from the planes, then the estimate.
// BB0..BB2 > 0: compile-time patch extents (padded to three axes), every
// offset's loads unrolled and issued together; 0: runtime extents.
template <int BB0, int BB1, int BB2>
__global__ void __launch_bounds__(256) gather_finalize_kernel(const float* __restrict__ planes,
                                                              const float* __restrict__ wsum, BmndStageParams sp,
                                                              const float* __restrict__ noisy,
                                                              float* __restrict__ out) {
    const Vol3 g(sp);
    const float eps_f = static_cast<float>(sp.eps);
    const int no_eps = sp.mass_conserve ? 1 : 0;
    __shared__ float win[BMND_MAX_PATCH];
    const int P = g.block[0] * g.block[1] * g.block[2];
    for (int p = threadIdx.x; p < P; p += blockDim.x) win[p] = sp.window[p];
    __syncthreads();
    const int c0 = g.counts[0], c1 = g.counts[1], c2 = g.counts[2];
    for (int64_t v = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; v < g.nvox;
         v += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int x2 = static_cast<int>(v % g.shape[2]);
        const int x1 = static_cast<int>((v / g.shape[2]) % g.shape[1]);
        const int x0 = static_cast<int>(v / (static_cast<int64_t>(g.shape[2]) * g.shape[1]));
        Sum2 num, den;
        if constexpr (BB0 > 0) {
            // origin x - d for offset d; terms of offsets whose origin lies off
            // the patch grid add zero, which leaves the compensated pair unchanged
            const int64_t ox = (static_cast<int64_t>(x0) * c1 + x1) * c2 + x2;
#pragma unroll
            for (int d0 = 0; d0 < BB0; ++d0) {
                const bool v0 = d0 <= x0 && x0 - d0 < c0;
#pragma unroll
                for (int d1 = 0; d1 < BB1; ++d1) {
                    const bool v1 = v0 && d1 <= x1 && x1 - d1 < c1;
                    float pv[BB2], wv[BB2];
#pragma unroll
                    for (int d2 = 0; d2 < BB2; ++d2) {
                        const bool ok = v1 && d2 <= x2 && x2 - d2 < c2;
                        const int p = (d0 * BB1 + d1) * BB2 + d2;
                        const int64_t o = ox - ((static_cast<int64_t>(d0) * c1 + d1) * c2 + d2);
                        pv[d2] = ok ? __ldg(planes + static_cast<int64_t>(p) * g.n_lins + o) : 0.0f;
                        wv[d2] = ok ? mul_rn(win[p], __ldg(wsum + o)) : 0.0f;
                    }
#pragma unroll
                    for (int d2 = 0; d2 < BB2; ++d2) {
                        num.add(pv[d2]);
                        den.add(wv[d2]);
                    }
                }
            }
        } else {
            const int a0 = max(0, x0 - c0 + 1), b0 = min(g.block[0] - 1, x0);
            const int a1 = max(0, x1 - c1 + 1), b1 = min(g.block[1] - 1, x1);
            const int a2 = max(0, x2 - c2 + 1), b2 = min(g.block[2] - 1, x2);
            for (int d0 = a0; d0 <= b0; ++d0)
                for (int d1 = a1; d1 <= b1; ++d1) {
                    const int64_t orow = (static_cast<int64_t>(x0 - d0) * c1 + (x1 - d1)) * c2;
                    const int prow = (d0 * g.block[1] + d1) * g.block[2];
                    for (int d2 = a2; d2 <= b2; ++d2) {
                        const int64_t o = orow + (x2 - d2);
                        const int p = prow + d2;
                        num.add(__ldg(planes + static_cast<int64_t>(p) * g.n_lins + o));
                        // window x weight sum, rounded once as the reference rounds w * window
                        den.add(mul_rn(win[p], __ldg(wsum + o)));
                    }
                }
        }
        const float d = den.value();
        out[v] = d > 0.0f ? div_rn(num.value(), no_eps ? d : add_rn(d, eps_f)) : noisy[v];
    }
}

// step 4 for compile-time patch extents, tiled: a CTA of 256 threads takes 32 x 8
// voxels of one plane (one voxel per thread) and first copies the weight sums
// W of every origin its voxels read (the tile grown by the patch extent minus
// one on the low side of each axis) into shared memory, so the 125 reads of W
// per voxel come from there instead of L2.  Same terms, same order and the same
// compensated sums as gather_finalize_kernel: the results are bit-identical.
constexpr int kGatherTX = 32, kGatherTY = 8;

template <int BB0, int BB1, int BB2>
__global__ void __launch_bounds__(256, 4) gather_finalize_tiled_kernel(const float* __restrict__ planes,
                                                                    const float* __restrict__ wsum,
                                                                    BmndStageParams sp,
                                                                    const float* __restrict__ noisy,
                                                                    float* __restrict__ out) {
    constexpr int SX = kGatherTX + BB2 - 1, SY = kGatherTY + BB1 - 1, SZ = BB0;
    __shared__ float win[BB0 * BB1 * BB2];
    __shared__ float wt[SZ * SY * SX];
    const Vol3 g(sp);
    const float eps_f = static_cast<float>(sp.eps);
    const int no_eps = sp.mass_conserve ? 1 : 0;
    for (int p = threadIdx.x; p < BB0 * BB1 * BB2; p += blockDim.x) win[p] = sp.window[p];
    const int c0 = g.counts[0], c1 = g.counts[1], c2 = g.counts[2];
    const int tiles_x = (g.shape[2] + kGatherTX - 1) / kGatherTX;
    const int tiles_y = (g.shape[1] + kGatherTY - 1) / kGatherTY;
    const int64_t ntiles = static_cast<int64_t>(tiles_x) * tiles_y * g.shape[0];
    const int tx = static_cast<int>(threadIdx.x) % kGatherTX, ty = static_cast<int>(threadIdx.x) / kGatherTX;
    for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int bx = static_cast<int>(t % tiles_x);
        const int by = static_cast<int>((t / tiles_x) % tiles_y);
        const int x0 = static_cast<int>(t / (static_cast<int64_t>(tiles_x) * tiles_y));
        const int y1 = by * kGatherTY, y2 = bx * kGatherTX;
        __syncthreads();  // the previous tile's weight sums are no longer read
        for (int i = threadIdx.x; i < SZ * SY * SX; i += blockDim.x) {
            const int iz = i / (SY * SX), iy = (i / SX) % SY, ix = i % SX;
            const int o0 = x0 - (BB0 - 1) + iz, o1 = y1 - (BB1 - 1) + iy, o2 = y2 - (BB2 - 1) + ix;
            float w = 0.0f;
            if (o0 >= 0 && o0 < c0 && o1 >= 0 && o1 < c1 && o2 >= 0 && o2 < c2)
                w = __ldg(wsum + (static_cast<int64_t>(o0) * c1 + o1) * c2 + o2);
            wt[i] = w;
        }
        __syncthreads();
        const int x1 = y1 + ty, x2 = y2 + tx;
        if (x1 >= g.shape[1] || x2 >= g.shape[2]) continue;
        const int64_t v = (static_cast<int64_t>(x0) * g.shape[1] + x1) * g.shape[2] + x2;
        Sum2 num, den;
        // origin x - d for offset d; terms of offsets whose origin lies off
        // the patch grid add zero, which leaves the compensated pair unchanged
        const int64_t ox = (static_cast<int64_t>(x0) * c1 + x1) * c2 + x2;
#pragma unroll
        for (int d0 = 0; d0 < BB0; ++d0) {
            const bool v0 = d0 <= x0 && x0 - d0 < c0;
#pragma unroll
            for (int d1 = 0; d1 < BB1; ++d1) {
                const bool v1 = v0 && d1 <= x1 && x1 - d1 < c1;
                float pv[BB2], wv[BB2];
#pragma unroll
                for (int d2 = 0; d2 < BB2; ++d2) {
                    const bool ok = v1 && d2 <= x2 && x2 - d2 < c2;
                    const int p = (d0 * BB1 + d1) * BB2 + d2;
                    const int64_t o = ox - ((static_cast<int64_t>(d0) * c1 + d1) * c2 + d2);
                    const int si = ((BB0 - 1 - d0) * SY + (ty + BB1 - 1 - d1)) * SX + (tx + BB2 - 1 - d2);
                    pv[d2] = ok ? __ldg(planes + static_cast<int64_t>(p) * g.n_lins + o) : 0.0f;
                    wv[d2] = ok ? mul_rn(win[p], wt[si]) : 0.0f;
                }
#pragma unroll
                for (int d2 = 0; d2 < BB2; ++d2) {
                    num.add(pv[d2]);
                    den.add(wv[d2]);
                }
            }
        }
        const float d = den.value();
        out[v] = d > 0.0f ? div_rn(num.value(), no_eps ? d : add_rn(d, eps_f)) : noisy[v];
    }
}

int64_t grid_for(int64_t n, int threads, int64_t cap = 152 * 32) {
    int64_t b = (n + threads - 1) / threads;
    if (b < 1) b = 1;
    return b > cap ? cap : b;
}

}  // namespace

int64_t agg_row_floats(const BmndStageParams& sp) {
    const int P = patch_volume(sp);
    return (P + 31) / 32 * 32;
}

AggregationLayout aggregation_layout(const BmndStageParams& sp, int64_t n_refs) {
    auto a256 = [](uint64_t v) { return (v + 255) & ~uint64_t(255); };
    AggregationLayout L{};
    int64_t n_lins = 1;
    for (int d = 0; d < sp.ndim; ++d) n_lins *= sp.shape[d] - sp.block[d] + 1;
    const uint64_t entries = static_cast<uint64_t>(n_refs) * static_cast<uint64_t>(sp.max_stack);
    const uint64_t P = static_cast<uint64_t>(patch_volume(sp));
    uint64_t off = 0;
    auto take = [&](uint64_t bytes) {
        const uint64_t o = off;
        off += a256(bytes);
        return o;
    };
    L.n_lins = n_lins;
    L.o_start = take(4ull * (static_cast<uint64_t>(n_lins) + 1));
    L.o_cursor = take(4ull * static_cast<uint64_t>(n_lins));
    L.o_block_sums = take(4ull * ((static_cast<uint64_t>(n_lins) + kScanBlock - 1) / kScanBlock + 1));
    L.o_entries = take(4ull * entries);
    L.o_slot = take(4ull * entries);
    L.o_store = take(4ull * entries * static_cast<uint64_t>(agg_row_floats(sp)));
    L.o_wstore = take(4ull * entries);
    L.o_planes = take(4ull * P * static_cast<uint64_t>(n_lins));
    L.o_wsum = take(4ull * static_cast<uint64_t>(n_lins));
    L.bytes = off;
    return L;
}

int32_t launch_exclusive_scan(const int32_t* in, int64_t n, int32_t* out, int32_t* block_sums,
                              cudaStream_t stream) {
    const int64_t nb = (n + kScanBlock - 1) / kScanBlock;
    if (nb > 0) {
        scan_block_kernel<<<static_cast<unsigned>(nb), kScanBlock, 0, stream>>>(in, n, out, block_sums);
        BMND_LAUNCH_CHECK("scan_block_kernel");
    }
    scan_sums_kernel<<<1, kScanBlock, 0, stream>>>(block_sums, nb, block_sums + nb);
    BMND_LAUNCH_CHECK("scan_sums_kernel");
    scan_add_kernel<<<static_cast<unsigned>((n + 1 + 255) / 256), 256, 0, stream>>>(out, n, block_sums,
                                                                                  block_sums + nb);
    BMND_LAUNCH_CHECK("scan_add_kernel");
    return BMND_OK;
}

int32_t launch_entry_index(const BmndStageParams& sp, const int32_t* sel, const int32_t* count, int64_t n_refs,
                           char* base, const AggregationLayout& L, cudaStream_t stream) {
    int32_t* start = reinterpret_cast<int32_t*>(base + L.o_start);
    int32_t* cursor = reinterpret_cast<int32_t*>(base + L.o_cursor);
    int32_t* sums = reinterpret_cast<int32_t*>(base + L.o_block_sums);
    int32_t* entries = reinterpret_cast<int32_t*>(base + L.o_entries);
    int32_t* slot_of = reinterpret_cast<int32_t*>(base + L.o_slot);
    const int64_t n = L.n_lins;
    if (n + 1 > 0x7fffffffLL || n_refs * sp.max_stack > 0x7fffffffLL)
        return fail(BMND_ERR_UNSUPPORTED, "too many patch origins or entries for the entry index");
    BMND_CUDA_TRY(cudaMemsetAsync(cursor, 0, 4ull * static_cast<uint64_t>(n), stream));
    const int64_t total = n_refs * sp.max_stack;
    entry_count_kernel<<<static_cast<unsigned>(grid_for(total, 256)), 256, 0, stream>>>(sel, count, n_refs,
                                                                                       sp.max_stack, cursor);
    BMND_LAUNCH_CHECK("entry_count_kernel");
    if (int32_t rc = launch_exclusive_scan(cursor, n, start, sums, stream)) return rc;
    BMND_CUDA_TRY(cudaMemsetAsync(cursor, 0, 4ull * static_cast<uint64_t>(n), stream));
    entry_fill_kernel<<<static_cast<unsigned>(grid_for(total, 256)), 256, 0, stream>>>(sel, count, n_refs,
                                                                                      sp.max_stack, start, cursor,
                                                                                      entries);
    BMND_LAUNCH_CHECK("entry_fill_kernel");
    entry_sort_kernel<<<static_cast<unsigned>(grid_for(n, 256)), 256, 0, stream>>>(start, n, entries, slot_of);
    BMND_LAUNCH_CHECK("entry_sort_kernel");
    return BMND_OK;
}

int32_t launch_gather(const BmndStageParams& sp, const float* noisy, float* out, char* base,
                      const AggregationLayout& L, cudaStream_t stream) {
    const float* store = reinterpret_cast<const float*>(base + L.o_store);
    const float* wstore = reinterpret_cast<const float*>(base + L.o_wstore);
    const int32_t* start = reinterpret_cast<const int32_t*>(base + L.o_start);
    float* planes = reinterpret_cast<float*>(base + L.o_planes);
    float* wsum = reinterpret_cast<float*>(base + L.o_wsum);
    const int P = patch_volume(sp);
    const int row = static_cast<int>(agg_row_floats(sp));
    const int64_t n = L.n_lins;
    const unsigned blocks = static_cast<unsigned>(grid_for((n + 31) / 32, 1, 152 * 64));
    constexpr int T = kSumThreads;
    switch ((P + 31) / 32) {
        case 1: origin_sum_kernel<1><<<blocks, T, 0, stream>>>(store, row, wstore, start, n, P, planes, wsum); break;
        case 2: origin_sum_kernel<2><<<blocks, T, 0, stream>>>(store, row, wstore, start, n, P, planes, wsum); break;
        case 3: origin_sum_kernel<3><<<blocks, T, 0, stream>>>(store, row, wstore, start, n, P, planes, wsum); break;
        case 4: origin_sum_kernel<4><<<blocks, T, 0, stream>>>(store, row, wstore, start, n, P, planes, wsum); break;
        default: return fail(BMND_ERR_UNSUPPORTED, "deterministic aggregation supports patches up to 128 voxels");
    }
    BMND_LAUNCH_CHECK("origin_sum_kernel");
    const int64_t nvox = volume_voxels(sp);
    const unsigned gb = static_cast<unsigned>(grid_for(nvox, 256, 152 * 16));
    const int* b = sp.block;
    // tiles of 32 x 8 voxels of one plane (padded geometry: z, y, x)
    int64_t ntiles = 1;
    {
        int sh[3] = {1, 1, 1};
        for (int d = 0; d < sp.ndim; ++d) sh[3 - sp.ndim + d] = sp.shape[d];
        ntiles = static_cast<int64_t>((sh[2] + kGatherTX - 1) / kGatherTX) * ((sh[1] + kGatherTY - 1) / kGatherTY) *
                 sh[0];
    }
    const unsigned tb = static_cast<unsigned>(ntiles < 152 * 16 ? ntiles : 152 * 16);
    if (sp.ndim == 3 && b[0] == 5 && b[1] == 5 && b[2] == 5)
        gather_finalize_tiled_kernel<5, 5, 5><<<tb, 256, 0, stream>>>(planes, wsum, sp, noisy, out);
    else if (sp.ndim == 3 && b[0] == 4 && b[1] == 4 && b[2] == 4)
        gather_finalize_tiled_kernel<4, 4, 4><<<tb, 256, 0, stream>>>(planes, wsum, sp, noisy, out);
    else if (sp.ndim == 2 && b[0] == 8 && b[1] == 8)
        gather_finalize_tiled_kernel<1, 8, 8><<<tb, 256, 0, stream>>>(planes, wsum, sp, noisy, out);
    else
        gather_finalize_kernel<0, 0, 0><<<gb, 256, 0, stream>>>(planes, wsum, sp, noisy, out);
    BMND_LAUNCH_CHECK("gather_finalize_kernel");
    return BMND_OK;
}

}  // namespace bmnd
