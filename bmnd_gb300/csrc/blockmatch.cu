// blockmatch.cu -- exhaustive window block matching with sorted top-K selection.
//
// Semantics follow _fused_blockmatch_groups_batch_numba
// (src/bmnd/blockmatching.py:1045-1205) and its helpers:
//   * the window is the clipped box center +- radius on the patch grid
//     (:1085-1099);
//   * distances are _patch_distance_numba (:322-371) evaluated per term in
//     float32 with IEEE division and logf;
//   * with stabilize_ties the comparisons use canonical keys (:957-984,
//     :1032-1042); ordering is (key, lin) lexicographic, which is exactly what
//     the reference's insertion sort realises (:987-1029);
//   * the top max_matches accepted and the top min(min,max) rejected
//     candidates are kept, the accepted are filled from the rejected up to
//     min_matches (:1179-1189), then the reference is put first, duplicates
//     dropped and the stack truncated to the largest power of two >= min
//     (_finalize_selected_lin_indices_numba, :913-954).
//
// GPU mapping: one warp per reference.  Every lane scores a strided subset of
// the window and keeps its own ascending top-K list of 64-bit composite keys
// (order_bits(key) << 32 | lin) in shared memory (interleaved by lane, so the
// list walks are bank-conflict free); the 32 lists are then merged with warp
// shuffles.  The reference patch sits in shared memory and is broadcast.
#include <cuda_runtime.h>
#include <stdint.h>

#include "bmnd_common.cuh"

namespace bmnd {
namespace {

constexpr int kWarps = 4;  // references per CTA
constexpr int kMaxList = BMND_MAX_STACK;

struct MatchArgs {
    int32_t ndim;
    int32_t counts[BMND_MAX_DIMS];
    int32_t radius[BMND_MAX_DIMS];
    int64_t grid_stride[BMND_MAX_DIMS];  // source offset of one patch-grid step per axis
    int32_t max_m;
    int32_t min_m;
    int32_t required;  // min(min_m, max_m)
    int32_t pow2;
    int32_t stab;
    int32_t P;
    float inv_scale;
    float scalar_threshold;
    const float* src;       // volume or patch table
    int32_t table;          // 1: src is a patch table (element p at offset p)
    int32_t block[BMND_MAX_DIMS];   // patch extents (volume source)
    int64_t vstride[BMND_MAX_DIMS]; // voxel strides (volume source)
    const int32_t* refs;
    const float* thresholds;  // per reference, or null -> scalar_threshold
    int64_t n_refs;
    int32_t* sel;
    int32_t* count;
    int32_t* accepted;
};

template <int CODE>
__device__ __forceinline__ float patch_distance(const float* __restrict__ ref,
                                                const float* __restrict__ src, int64_t origin,
                                                const int32_t* __restrict__ poff, int P,
                                                float inv) {
    float d = 0.0f;
    if (CODE == BMND_DIST_SSD) {
        for (int p = 0; p < P; ++p) {
            float diff = sub_rn(__ldg(src + origin + poff[p]), ref[p]);
            d = add_rn(d, mul_rn(diff, diff));
        }
        return d;
    }
    for (int p = 0; p < P; ++p) {
        float r = mul_rn(ref[p], inv);
        if (r < 0.0f) r = 0.0f;
        float c = mul_rn(__ldg(src + origin + poff[p]), inv);
        if (c < 0.0f) c = 0.0f;
        if (CODE == BMND_DIST_POISSON_DEVIANCE) {
            float s = add_rn(r, c);
            if (s > 0.0f) {
                float contrib = 0.0f;
                if (r > 0.0f) contrib = add_rn(contrib, mul_rn(r, logf(div_rn(mul_rn(2.0f, r), s))));
                if (c > 0.0f) contrib = add_rn(contrib, mul_rn(c, logf(div_rn(mul_rn(2.0f, c), s))));
                d = add_rn(d, mul_rn(2.0f, contrib));
            }
        } else if (CODE == BMND_DIST_PEARSON) {
            float s = add_rn(r, c);
            if (s > 0.0f) {
                float diff = sub_rn(c, r);
                d = add_rn(d, div_rn(mul_rn(diff, diff), s));
            }
        } else {
            float rs = mul_rn(2.0f, sqrtf(add_rn(r, 0.375f)));
            float cs = mul_rn(2.0f, sqrtf(add_rn(c, 0.375f)));
            float diff = sub_rn(cs, rs);
            d = add_rn(d, mul_rn(mul_rn(0.5f, diff), diff));
        }
    }
    if (d < 0.0f) d = 0.0f;
    return div_rn(d, static_cast<float>(P));
}

// insert `key` into an ascending list of `size` entries (capacity `cap`),
// stored at list[i * 32] (one column per lane)
__device__ __forceinline__ int list_insert(uint64_t* list, int size, int cap, uint64_t key) {
    if (cap == 0) return size;
    int at;
    if (size < cap) {
        at = size;
        ++size;
    } else {
        if (key >= list[(cap - 1) * 32]) return size;
        at = cap - 1;
    }
    while (at > 0) {
        uint64_t prev = list[(at - 1) * 32];
        if (key >= prev) break;
        list[at * 32] = prev;
        --at;
    }
    list[at * 32] = key;
    return size;
}

__device__ __forceinline__ uint64_t warp_min_u64(uint64_t v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        uint64_t other = __shfl_xor_sync(0xffffffffu, v, o);
        v = other < v ? other : v;
    }
    return v;
}

// merge the per-lane ascending lists into out[0..cap) (warp-wide); returns merged size
__device__ int warp_merge(const uint64_t* list, int size, int cap, uint64_t* out, int lane) {
    int head = 0;
    int n = 0;
    for (int t = 0; t < cap; ++t) {
        uint64_t mine = head < size ? list[head * 32] : ~0ull;
        uint64_t best = warp_min_u64(mine);
        if (best == ~0ull) break;
        if (mine == best) ++head;
        if (lane == 0) out[t] = best;
        ++n;
    }
    return n;
}

template <int CODE>
__global__ void __launch_bounds__(kWarps * 32) blockmatch_kernel(MatchArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const int64_t r = static_cast<int64_t>(blockIdx.x) * kWarps + warp;
    const int P = a.P;
    const int K = a.max_m;
    const int R = a.required;

    // per-warp shared layout: lists [K+R][32] u64, merged [K+R] u64, ref patch [P] f32
    const int list_rows = K + R;
    uint64_t* lists = reinterpret_cast<uint64_t*>(smem_raw) +
                      static_cast<size_t>(warp) * (list_rows * 32 + list_rows);
    uint64_t* acc_list = lists;
    uint64_t* rej_list = lists + K * 32;
    uint64_t* merged = lists + list_rows * 32;
    int32_t* poff_s = reinterpret_cast<int32_t*>(reinterpret_cast<uint64_t*>(smem_raw) +
                                                 static_cast<size_t>(kWarps) * (list_rows * 32 + list_rows));
    float* ref_s = reinterpret_cast<float*>(poff_s + P) + static_cast<size_t>(warp) * P;

    // offsets of the patch elements relative to the patch origin (C order over the block)
    for (int i = threadIdx.x; i < P; i += blockDim.x) {
        if (a.table) {
            poff_s[i] = i;
        } else {
            int rem = i;
            int64_t off = 0;
            for (int d = a.ndim - 1; d >= 0; --d) {
                off += static_cast<int64_t>(rem % a.block[d]) * a.vstride[d];
                rem /= a.block[d];
            }
            poff_s[i] = static_cast<int32_t>(off);
        }
    }
    __syncthreads();
    if (r >= a.n_refs) return;

    int center[BMND_MAX_DIMS], lo[BMND_MAX_DIMS], ext[BMND_MAX_DIMS];
    int64_t center_lin = 0, center_origin = 0;
    int64_t window = 1;
    for (int d = 0; d < a.ndim; ++d) {
        center[d] = a.refs[r * a.ndim + d];
        center_lin = center_lin * a.counts[d] + center[d];
        center_origin += static_cast<int64_t>(center[d]) * a.grid_stride[d];
        int l = center[d] - a.radius[d];
        if (l < 0) l = 0;
        int h = center[d] + a.radius[d];
        if (h > a.counts[d] - 1) h = a.counts[d] - 1;
        lo[d] = l;
        ext[d] = h - l + 1;
        window *= ext[d];
    }
    for (int p = lane; p < P; p += 32) ref_s[p] = __ldg(a.src + center_origin + poff_s[p]);
    __syncwarp();

    const float thr = a.thresholds ? a.thresholds[r] : a.scalar_threshold;
    const bool stab = a.stab && CODE != BMND_DIST_SSD;
    const float tkey = stab ? canonical_key(thr) : thr;

    uint64_t* my_acc = acc_list + lane;
    uint64_t* my_rej = rej_list + lane;
    int acc_size = 0, rej_size = 0, acc_count = 0;
    for (int64_t c = lane; c < window; c += 32) {
        int64_t rem = c;
        int coord[BMND_MAX_DIMS];
        for (int d = a.ndim - 1; d >= 0; --d) {
            coord[d] = lo[d] + static_cast<int>(rem % ext[d]);
            rem /= ext[d];
        }
        int64_t lin = 0, origin = 0;
        for (int d = 0; d < a.ndim; ++d) {
            lin = lin * a.counts[d] + coord[d];
            origin += static_cast<int64_t>(coord[d]) * a.grid_stride[d];
        }
        float dist = patch_distance<CODE>(ref_s, a.src, origin, poff_s, P, a.inv_scale);
        float key = stab ? canonical_key(dist) : dist;
        uint64_t ck = composite_key(key, static_cast<int32_t>(lin));
        if (key < tkey) {
            ++acc_count;
            acc_size = list_insert(my_acc, acc_size, K, ck);
        } else {
            rej_size = list_insert(my_rej, rej_size, R, ck);
        }
    }
    __syncwarp();
    int total_accepted = acc_count;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) total_accepted += __shfl_xor_sync(0xffffffffu, total_accepted, o);

    int n_acc = warp_merge(my_acc, acc_size, K, merged, lane);
    int n_rej = warp_merge(my_rej, rej_size, R, merged + K, lane);
    __syncwarp();

    if (lane == 0) {
        int32_t out[kMaxList];
        int n = 0;
        int selected = n_acc;
        int take = 0;
        if (selected < R) {
            int need = R - selected;
            take = need < n_rej ? need : n_rej;
        }
        out[n++] = static_cast<int32_t>(center_lin);
        for (int t = 0; t < n_acc + take && n < K; ++t) {
            uint64_t ck = t < n_acc ? merged[t] : merged[K + (t - n_acc)];
            int32_t l = static_cast<int32_t>(ck & 0xffffffffu);
            if (l < 0 || l == center_lin) continue;
            out[n++] = l;
        }
        if (a.pow2 && n > 0) {
            int target = 1;
            while ((target << 1) <= n) target <<= 1;
            if (a.min_m > target) target = a.min_m;
            if (target < n) n = target;
        }
        int32_t* row = a.sel + r * K;
        for (int t = 0; t < K; ++t) row[t] = t < n ? out[t] : -1;
        a.count[r] = n;
        a.accepted[r] = total_accepted;
    }
}

size_t match_smem_bytes(int K, int R, int P) {
    size_t rows = static_cast<size_t>(K + R);
    return static_cast<size_t>(kWarps) * (rows * 32 + rows) * sizeof(uint64_t) +
           static_cast<size_t>(P) * sizeof(int32_t) + static_cast<size_t>(kWarps) * P * sizeof(float);
}

int32_t launch(MatchArgs& a, int code, cudaStream_t stream) {
    if (a.n_refs == 0) return BMND_OK;
    size_t smem = match_smem_bytes(a.max_m, a.required, a.P);
    int64_t blocks = (a.n_refs + kWarps - 1) / kWarps;
    if (blocks > 0x7fffffff) return fail(BMND_ERR_INVALID_ARG, "too many references");
    dim3 grid(static_cast<unsigned>(blocks));
    switch (code) {
        case BMND_DIST_SSD:
            BMND_CUDA_TRY(cudaFuncSetAttribute(blockmatch_kernel<BMND_DIST_SSD>,
                                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            blockmatch_kernel<BMND_DIST_SSD><<<grid, kWarps * 32, smem, stream>>>(a);
            break;
        case BMND_DIST_POISSON_DEVIANCE:
            BMND_CUDA_TRY(cudaFuncSetAttribute(blockmatch_kernel<BMND_DIST_POISSON_DEVIANCE>,
                                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            blockmatch_kernel<BMND_DIST_POISSON_DEVIANCE><<<grid, kWarps * 32, smem, stream>>>(a);
            break;
        case BMND_DIST_PEARSON:
            BMND_CUDA_TRY(cudaFuncSetAttribute(blockmatch_kernel<BMND_DIST_PEARSON>,
                                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            blockmatch_kernel<BMND_DIST_PEARSON><<<grid, kWarps * 32, smem, stream>>>(a);
            break;
        case BMND_DIST_ANSCOMBE_SSD:
            BMND_CUDA_TRY(cudaFuncSetAttribute(blockmatch_kernel<BMND_DIST_ANSCOMBE_SSD>,
                                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            blockmatch_kernel<BMND_DIST_ANSCOMBE_SSD><<<grid, kWarps * 32, smem, stream>>>(a);
            break;
        default:
            return fail(BMND_ERR_INVALID_ARG, "unknown distance code");
    }
    BMND_LAUNCH_CHECK("blockmatch_kernel");
    return BMND_OK;
}

int32_t validate_match(const BmndMatchParams& mp) {
    if (mp.ndim < 1 || mp.ndim > BMND_MAX_DIMS) return fail(BMND_ERR_INVALID_ARG, "ndim out of range");
    if (mp.max_matches < 1 || mp.max_matches > BMND_MAX_STACK)
        return fail(BMND_ERR_UNSUPPORTED, "max_matches must be in [1, 32]");
    if (mp.min_matches < 1) return fail(BMND_ERR_INVALID_ARG, "min_matches must be positive");
    if (mp.distance < 0 || mp.distance > 3) return fail(BMND_ERR_INVALID_ARG, "unknown distance code");
    int64_t grid = 1;
    for (int d = 0; d < mp.ndim; ++d) {
        if (mp.counts[d] < 1) return fail(BMND_ERR_INVALID_ARG, "patch-grid counts must be positive");
        if (mp.search_radius[d] < 0) return fail(BMND_ERR_INVALID_ARG, "search radius must be >= 0");
        grid *= mp.counts[d];
    }
    if (grid > 0x7fffffffLL) return fail(BMND_ERR_UNSUPPORTED, "patch grid exceeds int32 indexing");
    if (!(mp.count_scale > 0.0) && mp.distance != BMND_DIST_SSD)
        return fail(BMND_ERR_INVALID_ARG, "count_scale must be positive");
    return BMND_OK;
}

void fill_common(MatchArgs& a, const BmndMatchParams& mp) {
    a.ndim = mp.ndim;
    for (int d = 0; d < BMND_MAX_DIMS; ++d) {
        a.counts[d] = d < mp.ndim ? mp.counts[d] : 1;
        a.radius[d] = d < mp.ndim ? mp.search_radius[d] : 0;
    }
    a.max_m = mp.max_matches;
    a.min_m = mp.min_matches;
    a.required = mp.min_matches < mp.max_matches ? mp.min_matches : mp.max_matches;
    a.pow2 = mp.prefer_power_of_two;
    a.stab = mp.stabilize_ties;
    double scale = mp.distance == BMND_DIST_SSD ? 1.0 : mp.count_scale;
    a.inv_scale = static_cast<float>(1.0 / scale);
}

}  // namespace

int32_t launch_blockmatch_volume(const BmndMatchParams& mp, const float* volume,
                                 const int32_t* shape, const int32_t* block, const int32_t* refs,
                                 int64_t n_refs, const float* thresholds, float scalar_threshold,
                                 int32_t* sel, int32_t* count, int32_t* accepted,
                                 cudaStream_t stream) {
    int32_t rc = validate_match(mp);
    if (rc) return rc;
    MatchArgs a{};
    fill_common(a, mp);
    int P = 1;
    int64_t vstride[BMND_MAX_DIMS];
    int64_t s = 1;
    for (int d = mp.ndim - 1; d >= 0; --d) {
        vstride[d] = s;
        s *= shape[d];
    }
    for (int d = 0; d < mp.ndim; ++d) {
        if (shape[d] - block[d] + 1 != mp.counts[d])
            return fail(BMND_ERR_INVALID_ARG, "counts must equal shape - block + 1");
        P *= block[d];
        a.grid_stride[d] = vstride[d];
        a.vstride[d] = vstride[d];
        a.block[d] = block[d];
    }
    if (P > BMND_MAX_PATCH) return fail(BMND_ERR_UNSUPPORTED, "patch volume exceeds 512");
    if (s > 0x7fffffffLL) return fail(BMND_ERR_UNSUPPORTED, "volume exceeds int32 voxel offsets");
    a.P = P;
    a.src = volume;
    a.table = 0;
    a.refs = refs;
    a.thresholds = thresholds;
    a.scalar_threshold = scalar_threshold;
    a.n_refs = n_refs;
    a.sel = sel;
    a.count = count;
    a.accepted = accepted;
    return launch(a, mp.distance, stream);
}

int32_t launch_blockmatch_patches(const BmndMatchParams& mp, const float* patches,
                                  int32_t patch_vol, const int32_t* refs, int64_t n_refs,
                                  const float* thresholds, int32_t* sel, int32_t* count,
                                  int32_t* accepted, cudaStream_t stream) {
    int32_t rc = validate_match(mp);
    if (rc) return rc;
    if (patch_vol < 1 || patch_vol > BMND_MAX_PATCH)
        return fail(BMND_ERR_UNSUPPORTED, "patch volume must be in [1, 512]");
    MatchArgs a{};
    fill_common(a, mp);
    int64_t s = patch_vol;
    for (int d = mp.ndim - 1; d >= 0; --d) {
        a.grid_stride[d] = s;
        s *= mp.counts[d];
    }
    a.P = patch_vol;
    a.src = patches;
    a.table = 1;
    a.refs = refs;
    a.thresholds = thresholds;
    a.scalar_threshold = 0.0f;
    a.n_refs = n_refs;
    a.sel = sel;
    a.count = count;
    a.accepted = accepted;
    return launch(a, mp.distance, stream);
}

}  // namespace bmnd
