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

#include <algorithm>
#include <cmath>

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
    int32_t use_table;  // integer-count lookup of Poisson-deviance terms
    int32_t fixup;      // only redo references whose count is negative
    int32_t approx;     // screened kernel: zero bound, the screening distances decide
    // approx mode, volume source (or null): c = max(x * inv_scale, 0) per
    // voxel, and the sum of B(c) = c + c log2 c over the patch at each origin
    const float* cv;
    const float* boxb;
    // SSD noise-bias correction (blockmatching.py:1133-1139): distance -=
    // gamma * noise_ssd[offset of the candidate from the reference], or null
    const float* noise_ssd;
    float gamma;
    // Poisson SSD noise-bias correction (blockmatching.py:1140-1145,
    // :432-443): distance -= gamma * sum_p bias_scale * (r_p + c_p) over
    // r_p + c_p > 0, for every candidate but the reference itself
    int32_t poisson_bias;
    float bias_scale;
    // threshold computed on the device (one float), overrides the scalar one
    const float* thr_dev;
    int32_t no_alloc;  // 1: no stream-ordered scratch (approx mode then runs the bounded form)
    float* aux_ws;          // caller workspace for the approximate form's per-voxel arrays, or null
    int64_t aux_ws_floats;  // its size in floats
    char* ssd_ws;           // caller workspace for the tensor-core SSD matching, or null
    uint64_t ssd_ws_bytes;
    // subsampled mode: prescreen on the patch's even sub-lattice (box sums in
    // boxb_sub), then the screening form for the presel smallest
    int32_t sub;
    int32_t presel;
    const float* boxb_sub;
    // candidate standardisation (blockmatching.py:372-428): null means then
    // variances by pooled count 0..null_max, or null
    const double* null_moments;
    int32_t null_max;
};

constexpr int kTable = 64;  // counts 0..63 are tabulated

// 2 * [r ln(2r/s) + c ln(2c/s)] with the reference's float32 operation order
// (blockmatching.py:347-355); 0 when r + c == 0 (the term is skipped there)
__device__ __forceinline__ float deviance_term(float r, float c) {
    float s = add_rn(r, c);
    if (!(s > 0.0f)) return 0.0f;
    float contrib = 0.0f;
    if (r > 0.0f) contrib = add_rn(contrib, mul_rn(r, logf(div_rn(mul_rn(2.0f, r), s))));
    if (c > 0.0f) contrib = add_rn(contrib, mul_rn(c, logf(div_rn(mul_rn(2.0f, c), s))));
    return mul_rn(2.0f, contrib);
}

// Poisson deviance with integer counts looked up in table[r * kTable + c],
// which holds deviance_term(r, c) for r, c < kTable; other terms are
// evaluated directly.  Bit-identical to patch_distance<DEV> with inv == 1.
__device__ __forceinline__ float deviance_tabulated(const float* __restrict__ ref,
                                                    const int* __restrict__ ref_row,
                                                    const float* __restrict__ src, int64_t origin,
                                                    const int32_t* __restrict__ poff, int P,
                                                    const float* __restrict__ table) {
    float d = 0.0f;
    for (int p = 0; p < P; ++p) {
        float c = __ldg(src + origin + poff[p]);
        if (c < 0.0f) c = 0.0f;
        const int rb = ref_row[p];
        const int ci = __float2int_rz(c);
        float t;
        if (rb >= 0 && ci < kTable && __int2float_rn(ci) == c)
            t = table[rb + ci];
        else
            t = deviance_term(ref[p], c);
        d = add_rn(d, t);
    }
    if (d < 0.0f) d = 0.0f;
    return div_rn(d, static_cast<float>(P));
}

// SSD and the Poisson SSD noise bias of one candidate in one pass, float32
// in patch order as the reference evaluates them (blockmatching.py:323-336,
// :432-443): bias = sum over r + c > 0 of scale * (r + c)
__device__ __forceinline__ float ssd_pooled_bias(const float* __restrict__ ref, const float* __restrict__ src,
                                                 int64_t origin, const int32_t* __restrict__ poff, int P,
                                                 float scale, float& bias) {
    float d = 0.0f, b = 0.0f;
    for (int p = 0; p < P; ++p) {
        const float r = ref[p];
        const float c = __ldg(src + origin + poff[p]);
        const float diff = sub_rn(c, r);
        d = add_rn(d, mul_rn(diff, diff));
        const float pooled = add_rn(r, c);
        if (pooled > 0.0f) b = add_rn(b, mul_rn(scale, pooled));
    }
    bias = b;
    return d;
}

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
            if (add_rn(r, c) > 0.0f) d = add_rn(d, deviance_term(r, c));
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

// (sum of terms - sum of null means) / sqrt(sum of null variances), every sum
// in float32 in patch order, the null moments of the pooled count rint(r + c)
// (float32 copies of the float64 table; above the table: mean 1, variance 2)
template <int CODE>
__device__ __forceinline__ float standardized_distance(const float* __restrict__ ref,
                                                       const float* __restrict__ src, int64_t origin,
                                                       const int32_t* __restrict__ poff, int P, float inv,
                                                       const double* __restrict__ moments, int max_count) {
    float dsum = 0.0f, msum = 0.0f, vsum = 0.0f;
    for (int p = 0; p < P; ++p) {
        float r = mul_rn(ref[p], inv);
        if (r < 0.0f) r = 0.0f;
        float c = mul_rn(__ldg(src + origin + poff[p]), inv);
        if (c < 0.0f) c = 0.0f;
        const float s = add_rn(r, c);
        if (!(s > 0.0f)) continue;
        if (CODE == BMND_DIST_POISSON_DEVIANCE) {
            dsum = add_rn(dsum, deviance_term(r, c));
        } else if (CODE == BMND_DIST_PEARSON) {
            const float diff = sub_rn(c, r);
            dsum = add_rn(dsum, div_rn(mul_rn(diff, diff), s));
        } else {
            const float rs = mul_rn(2.0f, __fsqrt_rn(add_rn(r, 0.375f)));
            const float cs = mul_rn(2.0f, __fsqrt_rn(add_rn(c, 0.375f)));
            const float diff = sub_rn(cs, rs);
            dsum = add_rn(dsum, mul_rn(mul_rn(0.5f, diff), diff));
        }
        const float k = rintf(s);
        if (k <= static_cast<float>(max_count)) {
            const int ki = static_cast<int>(k);
            msum = add_rn(msum, static_cast<float>(__ldg(moments + ki)));
            vsum = add_rn(vsum, static_cast<float>(__ldg(moments + max_count + 1 + ki)));
        } else {
            msum = add_rn(msum, 1.0f);
            vsum = add_rn(vsum, 2.0f);
        }
    }
    if (vsum <= 0.0f) return 0.0f;
    return div_rn(sub_rn(dsum, msum), __fsqrt_rn(vsum));
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

// patch-grid linear index and source offset of window candidate c (C order
// over the clipped window lo + [0, ext)); windows below 2^21 candidates are
// decoded with float reciprocals (small_div), larger ones with 64-bit division
__device__ __forceinline__ int64_t window_origin(const MatchArgs& a, const int* lo, const int* ext,
                                                 const float* inv_ext, bool small_window, int64_t c,
                                                 int64_t* lin_out) {
    int coord[BMND_MAX_DIMS] = {0, 0, 0};
    if (small_window) {
        int rem = static_cast<int>(c);
#pragma unroll
        for (int d = BMND_MAX_DIMS - 1; d >= 0; --d) {
            if (d < a.ndim) {
                const int q = d > 0 ? small_div(rem, inv_ext[d]) : 0;
                coord[d] = lo[d] + rem - q * ext[d];
                rem = q;
            }
        }
    } else {
        int64_t rem = c;
#pragma unroll
        for (int d = BMND_MAX_DIMS - 1; d >= 0; --d) {
            if (d < a.ndim) {
                coord[d] = lo[d] + static_cast<int>(rem % ext[d]);
                rem /= ext[d];
            }
        }
    }
    int64_t lin = 0, origin = 0;
#pragma unroll
    for (int d = 0; d < BMND_MAX_DIMS; ++d) {
        if (d < a.ndim) {
            lin = lin * a.counts[d] + coord[d];
            origin += static_cast<int64_t>(coord[d]) * a.grid_stride[d];
        }
    }
    *lin_out = lin;
    return origin;
}

// window_origin, plus the index of the candidate's offset in a table over the
// search offsets (C order over 2 radius + 1 per axis), from the reference's
// patch-grid coordinates rc
__device__ __forceinline__ int64_t window_origin_offset(const MatchArgs& a, const int* lo, const int* ext,
                                                        const float* inv_ext, bool small_window, int64_t c,
                                                        const int* rc, int64_t* lin_out, int* gidx_out) {
    int coord[BMND_MAX_DIMS] = {0, 0, 0};
    if (small_window) {
        int rem = static_cast<int>(c);
#pragma unroll
        for (int d = BMND_MAX_DIMS - 1; d >= 0; --d) {
            if (d < a.ndim) {
                const int q = d > 0 ? small_div(rem, inv_ext[d]) : 0;
                coord[d] = lo[d] + rem - q * ext[d];
                rem = q;
            }
        }
    } else {
        int64_t rem = c;
#pragma unroll
        for (int d = BMND_MAX_DIMS - 1; d >= 0; --d) {
            if (d < a.ndim) {
                coord[d] = lo[d] + static_cast<int>(rem % ext[d]);
                rem /= ext[d];
            }
        }
    }
    int64_t lin = 0, origin = 0;
    int gidx = 0;
#pragma unroll
    for (int d = 0; d < BMND_MAX_DIMS; ++d) {
        if (d < a.ndim) {
            lin = lin * a.counts[d] + coord[d];
            origin += static_cast<int64_t>(coord[d]) * a.grid_stride[d];
            gidx = gidx * (2 * a.radius[d] + 1) + (coord[d] - rc[d] + a.radius[d]);
        }
    }
    *lin_out = lin;
    *gidx_out = gidx;
    return origin;
}

template <int CODE>
__global__ void __launch_bounds__(kWarps * 32) blockmatch_kernel(MatchArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const int P = a.P;
    const int K = a.max_m;
    const int R = a.required;

    // shared layout: per warp [K+R][32] u64 lists + [K+R] merged; then
    // poff[P] i32, ref[kWarps][P] f32, ref_row[kWarps][P] i32, table[64*64] f32
    const int list_rows = K + R;
    uint64_t* lists = reinterpret_cast<uint64_t*>(smem_raw) +
                      static_cast<size_t>(warp) * (list_rows * 32 + list_rows);
    uint64_t* acc_list = lists;
    uint64_t* rej_list = lists + K * 32;
    uint64_t* merged = lists + list_rows * 32;
    int32_t* poff_s = reinterpret_cast<int32_t*>(reinterpret_cast<uint64_t*>(smem_raw) +
                                                 static_cast<size_t>(kWarps) * (list_rows * 32 + list_rows));
    float* ref_s = reinterpret_cast<float*>(poff_s + P) + static_cast<size_t>(warp) * P;
    int* ref_row = reinterpret_cast<int*>(reinterpret_cast<float*>(poff_s + P) + kWarps * P) +
                   static_cast<size_t>(warp) * P;
    float* table = reinterpret_cast<float*>(reinterpret_cast<int*>(reinterpret_cast<float*>(poff_s + P) +
                                                                   kWarps * P) + kWarps * P);
    const bool use_table = CODE == BMND_DIST_POISSON_DEVIANCE && a.use_table;

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
    if (use_table)
        for (int i = threadIdx.x; i < kTable * kTable; i += blockDim.x)
            table[i] = deviance_term(static_cast<float>(i / kTable), static_cast<float>(i % kTable));
    __syncthreads();

    const bool stab = a.stab && CODE != BMND_DIST_SSD;
    uint64_t* my_acc = acc_list + lane;
    uint64_t* my_rej = rej_list + lane;
    const int64_t stride = static_cast<int64_t>(gridDim.x) * kWarps;
    for (int64_t r = static_cast<int64_t>(blockIdx.x) * kWarps + warp; r < a.n_refs; r += stride) {
        if (a.fixup && a.count[r] >= 0) continue;
        int lo[BMND_MAX_DIMS] = {0, 0, 0}, ext[BMND_MAX_DIMS] = {1, 1, 1};
        float inv_ext[BMND_MAX_DIMS] = {1.0f, 1.0f, 1.0f};
        int64_t center_lin = 0, center_origin = 0;
        int64_t window = 1;
#pragma unroll
        for (int d = 0; d < BMND_MAX_DIMS; ++d) {
            if (d < a.ndim) {
                const int cd = a.refs[r * a.ndim + d];
                center_lin = center_lin * a.counts[d] + cd;
                center_origin += static_cast<int64_t>(cd) * a.grid_stride[d];
                const int l = max(cd - a.radius[d], 0);
                const int h = min(cd + a.radius[d], a.counts[d] - 1);
                lo[d] = l;
                ext[d] = h - l + 1;
                inv_ext[d] = 1.0f / static_cast<float>(ext[d]);
                window *= ext[d];
            }
        }
        const bool small_window = window < (int64_t(1) << 21);
        __syncwarp();
        for (int p = lane; p < P; p += 32) {
            float v = __ldg(a.src + center_origin + poff_s[p]);
            if (use_table) {
                float rv = v < 0.0f ? 0.0f : v;
                int ri = __float2int_rz(rv);
                ref_s[p] = rv;
                ref_row[p] = (ri < kTable && __int2float_rn(ri) == rv) ? ri * kTable : -1;
            } else {
                ref_s[p] = v;
            }
        }
        __syncwarp();

        const float thr = a.thresholds ? a.thresholds[r] : (a.thr_dev ? *a.thr_dev : a.scalar_threshold);
        const float tkey = stab ? canonical_key(thr) : thr;
        int acc_size = 0, rej_size = 0, acc_count = 0;
        for (int64_t c = lane; c < window; c += 32) {
            int64_t lin;
            const int64_t origin = window_origin(a, lo, ext, inv_ext, small_window, c, &lin);
            float dist;
            if (CODE == BMND_DIST_SSD && a.poisson_bias) {
                float bias;
                dist = ssd_pooled_bias(ref_s, a.src, origin, poff_s, P, a.bias_scale, bias);
                if (lin != center_lin) dist = sub_rn(dist, mul_rn(a.gamma, bias));
            } else {
                dist = a.null_moments ? standardized_distance<CODE>(ref_s, a.src, origin, poff_s, P, a.inv_scale,
                                                                    a.null_moments, a.null_max)
                       : use_table    ? deviance_tabulated(ref_s, ref_row, a.src, origin, poff_s, P, table)
                                      : patch_distance<CODE>(ref_s, a.src, origin, poff_s, P, a.inv_scale);
            }
            if (CODE == BMND_DIST_SSD && a.noise_ssd) {
                // offset of the candidate from the reference, C order over 2 r + 1 per axis
                int64_t rem = c, gidx = 0, mul = 1;
#pragma unroll
                for (int d = BMND_MAX_DIMS - 1; d >= 0; --d) {
                    if (d < a.ndim) {
                        const int cd = lo[d] + static_cast<int>(rem % ext[d]);
                        rem /= ext[d];
                        gidx += (cd - a.refs[r * a.ndim + d] + a.radius[d]) * mul;
                        mul *= 2 * a.radius[d] + 1;
                    }
                }
                dist = sub_rn(dist, mul_rn(a.gamma, __ldg(a.noise_ssd + gidx)));
            }
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
            int32_t* row = a.sel + r * K;
            int n = 0;
            int take = 0;
            if (n_acc < R) {
                int need = R - n_acc;
                take = need < n_rej ? need : n_rej;
            }
            row[n++] = static_cast<int32_t>(center_lin);
            for (int t = 0; t < n_acc + take && n < K; ++t) {
                uint64_t ck = t < n_acc ? merged[t] : merged[K + (t - n_acc)];
                int32_t l = static_cast<int32_t>(ck & 0xffffffffu);
                if (l < 0 || l == center_lin) continue;
                row[n++] = l;
            }
            if (a.pow2 && n > 0) {
                int target = 1;
                while ((target << 1) <= n) target <<= 1;
                if (a.min_m > target) target = a.min_m;
                if (target < n) n = target;
            }
            for (int t = n; t < K; ++t) row[t] = -1;
            a.count[r] = n;
            a.accepted[r] = total_accepted;
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// SSD matching on the tensor cores: selection with exact rescoring
//
// ssd_screen_tc_kernel (ssdtc.cu) writes, for every reference, the screening
// distance d~ = |a'|^2 + |b'|^2 - 2 a'.b' of every window candidate, where
// a' = a - mu and b' = b - mu are the patches centred on their tile's mean mu
// and the cross term comes from three BF16 tcgen05 products (hi/lo splits of
// a' and b', FP32 accumulation).  Its error, with the reference's float32
// per-term SSD and the rounding of the bounds below, stays under
//   2^-10 (|a'|^2 + |b'|^2)              the products and their sums (a
//       worst-case analysis, every tensor-core addition rounding with up to
//       17 terms, gives 2^-12.5; the rest is margin), plus
//   2^-14 (|a|^2 + |b|^2 + 2 P mu^2)     the centred norms, formed in float32
//       from the sums of squares and the sums of the raw patches (each of
//       those sums is off by at most P 2^-24 of |a|^2 + P mu^2 for P <= 128,
//       the centring expression by 3 roundings of the same size),
// so the exact distance of candidate c lies in [lo_c, hi_c] = d~_c -+ that.
// This kernel, one warp per reference (the exact kernel's layout):
//   pass 1: counts the certainly accepted candidates (hi < threshold) and finds
//           V, the K-th smallest (hi, lin) among them;
//   pass 2: rescores exactly, in float32 per term in patch order (the exact
//           kernel's arithmetic), every candidate that may be accepted and
//           may reach the top K (lo < threshold and lo <= V) or whose accept
//           decision is open (lo < threshold <= hi), and keeps the top K by
//           (exact key, lin).
// No other candidate can change the match set or the accepted count, so both
// equal the exact kernel's bit for bit.  A reference with fewer than
// min(min, max) certain accepts may need the best rejected candidates: it is
// marked (count = -1) and redone by the exact kernel.
// ---------------------------------------------------------------------------
constexpr float kSsdBoundRel = 9.765625e-4f;  // 2^-10
constexpr float kSsdBoundCancel = 6.103515625e-5f;  // 2^-14
constexpr float kSsdBoundAbs = 1e-30f;         // products flushed to zero at the bottom of the range

__global__ void __launch_bounds__(kWarps * 32) ssd_select_kernel(MatchArgs a, const float* __restrict__ dtil,
                                                                 const float* __restrict__ norms,
                                                                 const float* __restrict__ sums,
                                                                 const float* __restrict__ ref_mu, int64_t wmax,
                                                                 const int* __restrict__ screen_err) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const int P = a.P;
    const int K = a.max_m;
    const int R = a.required;
    const int list_rows = K + R;
    uint64_t* lists = reinterpret_cast<uint64_t*>(smem_raw) +
                      static_cast<size_t>(warp) * (list_rows * 32 + list_rows);
    uint64_t* my_acc = lists + lane;
    uint64_t* merged = lists + list_rows * 32;
    int32_t* poff_s = reinterpret_cast<int32_t*>(reinterpret_cast<uint64_t*>(smem_raw) +
                                                 static_cast<size_t>(kWarps) * (list_rows * 32 + list_rows));
    float* ref_s = reinterpret_cast<float*>(poff_s + P) + static_cast<size_t>(warp) * P;
    for (int i = threadIdx.x; i < P; i += blockDim.x) {
        int rem = i;
        int64_t off = 0;
        for (int d = a.ndim - 1; d >= 0; --d) {
            off += static_cast<int64_t>(rem % a.block[d]) * a.vstride[d];
            rem /= a.block[d];
        }
        poff_s[i] = static_cast<int32_t>(off);
    }
    __syncthreads();
    const bool screened = *screen_err == 0;  // a screening that stopped early settles nothing
    const int64_t stride = static_cast<int64_t>(gridDim.x) * kWarps;
    for (int64_t r = static_cast<int64_t>(blockIdx.x) * kWarps + warp; r < a.n_refs; r += stride) {
        if (!screened) {
            if (lane == 0) a.count[r] = -1;
            continue;
        }
        int lo[BMND_MAX_DIMS] = {0, 0, 0}, ext[BMND_MAX_DIMS] = {1, 1, 1};
        float inv_ext[BMND_MAX_DIMS] = {1.0f, 1.0f, 1.0f};
        int64_t center_lin = 0, center_origin = 0, window = 1;
        int rc[BMND_MAX_DIMS] = {0, 0, 0};
#pragma unroll
        for (int d = 0; d < BMND_MAX_DIMS; ++d) {
            if (d < a.ndim) {
                const int cd = a.refs[r * a.ndim + d];
                rc[d] = cd;
                center_lin = center_lin * a.counts[d] + cd;
                center_origin += static_cast<int64_t>(cd) * a.grid_stride[d];
                const int l = max(cd - a.radius[d], 0);
                const int h = min(cd + a.radius[d], a.counts[d] - 1);
                lo[d] = l;
                ext[d] = h - l + 1;
                inv_ext[d] = 1.0f / static_cast<float>(ext[d]);
                window *= ext[d];
            }
        }
        const bool small_window = window < (int64_t(1) << 21);
        __syncwarp();
        for (int p = lane; p < P; p += 32) ref_s[p] = __ldg(a.src + center_origin + poff_s[p]);
        __syncwarp();
        const float thr = a.thresholds ? a.thresholds[r] : (a.thr_dev ? *a.thr_dev : a.scalar_threshold);
        const float mu = __ldg(ref_mu + r);
        const float na2 = __ldg(norms + center_origin);
        const float na = centred_norm(na2, __ldg(sums + center_origin), mu, P);
        const float pmu2 = 2.0f * static_cast<float>(P) * mu * mu;
        const float* row = dtil + r * wmax;
        // the bounds of candidate c, with the noise-bias correction of its offset:
        // the products' error scales with the centred norms, the cancellation in
        // the centred norms with the raw sums of squares
        auto bounds = [&](int64_t c, int64_t origin, int gidx, float& blo, float& bhi) {
            const float nb2 = __ldg(norms + origin);
            const float nb = centred_norm(nb2, __ldg(sums + origin), mu, P);
            const float del = fmaf(kSsdBoundRel, na + nb, fmaf(kSsdBoundCancel, na2 + nb2 + pmu2, kSsdBoundAbs));
            const float dv = __ldg(row + c);
            blo = dv - del;
            bhi = dv + del;
            if (a.noise_ssd) {
                const float g = mul_rn(a.gamma, __ldg(a.noise_ssd + gidx));
                blo = sub_rn(blo, g);  // rounding is monotone: the bounds stay bounds
                bhi = sub_rn(bhi, g);
            }
        };
        // pass 1: the certain accepts, and V at or above the K-th smallest upper
        // bound among them: every lane keeps its 4 smallest, and V is the K-th
        // smallest of the warp's 128 kept values (K <= 32).  At least K certain
        // accepts have upper bounds <= V, so no candidate whose lower bound
        // exceeds V can reach the top K.
        int n_cert = 0;
        float t0 = INFINITY, t1 = INFINITY, t2 = INFINITY, t3 = INFINITY;
        for (int64_t c = lane; c < window; c += 32) {
            int64_t lin;
            int gidx;
            const int64_t origin = window_origin_offset(a, lo, ext, inv_ext, small_window, c, rc, &lin, &gidx);
            float blo, bhi;
            bounds(c, origin, gidx, blo, bhi);
            if (bhi < thr) {
                ++n_cert;
                if (bhi < t3) {
                    if (bhi < t2) {
                        t3 = t2;
                        if (bhi < t1) {
                            t2 = t1;
                            if (bhi < t0) {
                                t1 = t0;
                                t0 = bhi;
                            } else {
                                t1 = bhi;
                            }
                        } else {
                            t2 = bhi;
                        }
                    } else {
                        t3 = bhi;
                    }
                }
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) n_cert += __shfl_xor_sync(0xffffffffu, n_cert, o);
        if (n_cert < R) {
            if (lane == 0) a.count[r] = -1;  // may need rejected candidates: the exact kernel redoes it
            __syncwarp();
            continue;
        }
        float vkey = thr;
        if (n_cert >= K) {
            // rank of each kept value among all 128, ties ordered by (lane, slot)
            const float mine[4] = {t0, t1, t2, t3};
            int rank[4] = {0, 0, 0, 0};
            for (int sl = 0; sl < 32; ++sl) {
                float other[4];
#pragma unroll
                for (int p = 0; p < 4; ++p) other[p] = __shfl_sync(0xffffffffu, mine[p], sl);
#pragma unroll
                for (int q = 0; q < 4; ++q)
#pragma unroll
                    for (int p = 0; p < 4; ++p)
                        rank[q] += (other[p] < mine[q] || (other[p] == mine[q] && (sl < lane || (sl == lane && p < q))))
                                       ? 1 : 0;
            }
            float pick = 0.0f;
            bool has = false;
#pragma unroll
            for (int q = 0; q < 4; ++q)
                if (rank[q] == K - 1) {
                    pick = mine[q];
                    has = true;
                }
            const unsigned who = __ballot_sync(0xffffffffu, has);
            vkey = __shfl_sync(0xffffffffu, pick, __ffs(who) - 1);
        }
        int acc_size = 0;
        __syncwarp();
        // pass 2: exact rescoring of every candidate that can matter
        acc_size = 0;
        int acc_open = 0;
        for (int64_t c = lane; c < window; c += 32) {
            int64_t lin;
            int gidx;
            const int64_t origin = window_origin_offset(a, lo, ext, inv_ext, small_window, c, rc, &lin, &gidx);
            float blo, bhi;
            bounds(c, origin, gidx, blo, bhi);
            const bool certain = bhi < thr;
            if (!(blo < thr) || (certain && blo > vkey)) continue;
            float dist = patch_distance<BMND_DIST_SSD>(ref_s, a.src, origin, poff_s, P, 1.0f);
            if (a.noise_ssd) dist = sub_rn(dist, mul_rn(a.gamma, __ldg(a.noise_ssd + gidx)));
            if (dist < thr) {
                if (!certain) ++acc_open;
                acc_size = list_insert(my_acc, acc_size, K, composite_key(dist, static_cast<int32_t>(lin)));
            }
        }
        __syncwarp();
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc_open += __shfl_xor_sync(0xffffffffu, acc_open, o);
        const int n_acc = warp_merge(my_acc, acc_size, K, merged, lane);
        __syncwarp();
        if (lane == 0) {
            int32_t* out_row = a.sel + r * K;
            int n = 0;
            out_row[n++] = static_cast<int32_t>(center_lin);
            for (int t = 0; t < n_acc && n < K; ++t) {
                const int32_t l = static_cast<int32_t>(merged[t] & 0xffffffffu);
                if (l < 0 || l == center_lin) continue;
                out_row[n++] = l;
            }
            if (a.pow2 && n > 0) {
                int target = 1;
                while ((target << 1) <= n) target <<= 1;
                if (a.min_m > target) target = a.min_m;
                if (target < n) n = target;
            }
            for (int t = n; t < K; ++t) out_row[t] = -1;
            a.count[r] = n;
            a.accepted[r] = n_cert + acc_open;
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// Screened Poisson-deviance matching for real-valued sources
//
// Exact per-term evaluation (two IEEE divisions and two logf) is needed only
// where it can change the result.  Pass A scores every candidate with a
// cancellation-free form of the same deviance term: with s = r + c and
// u = (r - c) / s,
//   t = 2 [r ln(2r/s) + c ln(2c/s)] = s u^2 sum_{k>=1} u^(2k-2) / (k (2k - 1)),
// summed to k = 6 for u^2 <= 0.16 (truncation < 2.2e-7 relative) and with the
// SFU log2 otherwise.  A rigorous bound D(d) = Dabs + Drel d on the distance to
// the exact float32 result covers the screening arithmetic, the exact path's
// own rounding (its division error enters each log absolutely, 2^-21 s per
// term), both float32 accumulations, times a safety factor 4.  A candidate is
//   * certainly accepted   if canonical(d + D) < canonical(threshold),
//   * certainly rejected   if canonical(d - D) >= canonical(threshold);
// among the certainly accepted a radix select finds V with at least K of them
// scoring <= V, so no candidate with canonical(d - D) > canonical(V + D(V))
// can reach the top K.  Everything else (uncertain accept decisions, possible
// top-K members) is rescored exactly, warp-parallel from a shared queue, and
// the top K is kept by (canonical key, lin) as in the exact kernel.
// References that end with fewer than min(min, max) accepted candidates need
// the best rejected ones too; they are marked (count = -1) and redone by the
// exact kernel.
// ---------------------------------------------------------------------------

// Screening of one candidate with the ratio form
//   t = 2 ln 2 [r log2(2r/s) + c log2(2c/s)],  s = r + c,
// using the SFU reciprocal and log2.  Near r = c both logs are near zero and
// carry only the SFU's absolute error, so the form has no cancellation.
// Per term the screening error is below s (e_lg + 1.45 e_rcp + 2^-22.5 +
// 1.27 2^-23) in log2 units (r |log2 q_r| + c |log2 q_c| <= 1.27 s), and the
// exact float32 path's own error below 2^-21 s; the bound uses the sum of s
// over the patch.  kScreenAbs is that per-unit-s constant in distance units,
// times a safety factor 2, with the SFU errors e_lg, e_rcp measured on GB300
// over the argument ranges used here.
// measured: lg2.approx abs error <= 2^-22.06 max(|log2 x|, 1) (so r e_lg + c e_lg
// <= 2^-22.06 2.27 s), rcp.approx relative error <= 2^-23.28
constexpr float kScreenAbs = 2.0f * (1.38629436f * (5.41e-07f + 1.45f * 9.83e-08f + 1.69e-07f + 1.52e-07f) +
                                     4.77e-07f);

// SFU reciprocal and log2 of normal arguments (callers clamp to FLT_MIN)
__device__ __forceinline__ float sfu_rcp(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float sfu_lg2(float x) {
    float y;
    asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// r2 = 2 r; returns r log2(2r/s) + c log2(2c/s)
__device__ __forceinline__ float ratio_term(float r, float r2, float c, float& ss) {
    const float kMin = 1.17549435e-38f;
    const float s = r + c;
    const float rs = sfu_rcp(fmaxf(s, kMin));
    const float lr = sfu_lg2(fmaxf(r2 * rs, kMin));
    const float lc = sfu_lg2(fmaxf((c + c) * rs, kMin));
    ss += s;
    return fmaf(r, lr, c * lc);
}

// generic (runtime patch) screening
__device__ __forceinline__ float2 screen_deviance(const float2* __restrict__ ref,
                                                  const float* __restrict__ src, int64_t origin,
                                                  const int32_t* __restrict__ poff, int P, float inv) {
    float sum_t = 0.0f, ss = 0.0f;
    for (int p = 0; p < P; ++p) {
        const float c = fmaxf(__ldg(src + origin + poff[p]) * inv, 0.0f);
        const float2 rr = ref[p];
        sum_t += ratio_term(rr.x, rr.y, c, ss);
    }
    const float fp = static_cast<float>(P);
    return make_float2(fmaxf(1.38629436f * sum_t, 0.0f) / fp, kScreenAbs * ss / fp + 1e-30f);
}

// compile-time patch (volume source, count scale 1): fully unrolled
template <int ND, int B0, int B1, int B2>
__device__ __forceinline__ float2 screen_deviance_fixed(const float2* __restrict__ ref,
                                                        const float* __restrict__ src, int64_t origin,
                                                        int64_t s0, int64_t s1,
                                                        const int32_t* __restrict__ poff) {
    float sum_t = 0.0f, ss = 0.0f;
    const float* base = src + origin;
#pragma unroll 1
    for (int a0 = 0; a0 < B0; ++a0) {
#pragma unroll
        for (int a1 = 0; a1 < B1; ++a1) {
            const float* row = ND == 3 ? base + a0 * s0 + a1 * s1 : base + a0 * s0;
#pragma unroll
            for (int a2 = 0; a2 < B2; ++a2) {
                const int p = (a0 * B1 + a1) * B2 + a2;
                const float c = fmaxf(__ldg(row + (ND == 3 ? a2 : a1)), 0.0f);
                const float2 rr = ref[p];
                sum_t += ratio_term(rr.x, rr.y, c, ss);
            }
        }
    }
    constexpr int P = B0 * B1 * B2;
    return make_float2(fmaxf(1.38629436f * sum_t, 0.0f) / static_cast<float>(P),
                       kScreenAbs * ss / static_cast<float>(P) + 1e-30f);
}

// Approximate mode (no error bound): with s = r + c the deviance term is
//   2 ln 2 [r log2(2r/s) + c log2(2c/s)] = 2 ln 2 [A_r + B_c - s log2 s],
// A_r = r + r log2 r, B_c = c + c log2 c.  Summed over a patch, the A part is
// one number per reference and the B part one number per candidate origin
// (a box sum over the patch, prepared once per volume), so only
// -sum_p s_p log2 s_p remains per candidate: one SFU log2 and two FP32
// operations per term.  A thread scores XR candidates that are neighbours
// along x, so one row of XR + BX - 1 voxels serves XR x BX terms.
__global__ void approx_voxel_kernel(const float* __restrict__ src, float inv, int64_t n, float* __restrict__ cv,
                                    float* __restrict__ bv) {
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const float c = fmaxf(src[i] * inv, 0.0f);
        cv[i] = c;
        bv[i] = c > 0.0f ? c + c * log2f(c) : 0.0f;
    }
}

// boxb[o] = sum over the patch at origin o of bv (0 where no patch starts);
// S = 2: over the patch's even sub-lattice only
template <int ND, int B0, int B1, int B2, int S>
__global__ void approx_box_kernel(const float* __restrict__ bv, int n0, int n1, int n2, float* __restrict__ boxb) {
    const int64_t n = static_cast<int64_t>(n0) * n1 * n2;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int x = static_cast<int>(i % n2);
        const int y = static_cast<int>((i / n2) % n1);
        const int z = static_cast<int>(i / (static_cast<int64_t>(n1) * n2));
        float sum = 0.0f;
        if (ND == 3 ? (z <= n0 - B0 && y <= n1 - B1 && x <= n2 - B2) : (y <= n1 - B0 && x <= n2 - B1)) {
#pragma unroll 1
            for (int a0 = 0; a0 < B0; a0 += S) {
#pragma unroll
                for (int a1 = 0; a1 < (ND == 3 ? B1 : 1); a1 += (ND == 3 ? S : 1)) {
                    const float* row = ND == 3 ? bv + i + (static_cast<int64_t>(a0) * n1 + a1) * n2
                                               : bv + i + static_cast<int64_t>(a0) * n2;
#pragma unroll
                    for (int a2 = 0; a2 < (ND == 3 ? B2 : B1); a2 += S) sum += __ldg(row + a2);
                }
            }
        }
        boxb[i] = sum;
    }
}

// -sum_p s_p log2 s_p for the XR candidates at origin + j (j < XR) along x;
// ref[p].y holds max(r, 2^-100), so s > 0; xroom voxels of the row exist
// whether patch element p (C order) lies on the even sub-lattice of the patch
template <int ND, int B0, int B1, int B2>
__device__ __forceinline__ bool sub_lattice(int p) {
    if (ND == 3) return ((p / (B1 * B2)) % 2 == 0) && (((p / B2) % B1) % 2 == 0) && ((p % B2) % 2 == 0);
    return ((p / B1) % 2 == 0) && ((p % B1) % 2 == 0);
}

// S = 1: every patch element; S = 2: the even sub-lattice only
template <int ND, int B0, int B1, int B2, int XR, int S>
__device__ __forceinline__ void approx_unit(const float2* __restrict__ ref, const float* __restrict__ cv,
                                            int64_t origin, int64_t s0, int64_t s1, int xroom, float (&acc)[XR]) {
    constexpr int BX = ND == 3 ? B2 : B1;  // patch extent along x
    constexpr int BR = ND == 3 ? B1 : 1;   // rows per step of axis 0
    constexpr int NL = XR + BX - 1;
#pragma unroll
    for (int j = 0; j < XR; ++j) acc[j] = 0.0f;
    const float* base = cv + origin;
#pragma unroll 1
    for (int a0 = 0; a0 < B0; a0 += S) {
#pragma unroll
        for (int a1 = 0; a1 < BR; a1 += (ND == 3 ? S : 1)) {
            const float* row = base + a0 * s0 + (ND == 3 ? a1 * s1 : 0);
            float xv[NL];
#pragma unroll
            for (int i = 0; i < NL; ++i) xv[i] = i < xroom ? __ldg(row + i) : 0.0f;
#pragma unroll
            for (int ax = 0; ax < BX; ax += S) {
                const float r = ref[(a0 * BR + a1) * BX + ax].y;
#pragma unroll
                for (int j = 0; j < XR; ++j) {
                    const float sv = r + xv[ax + j];
                    acc[j] = fmaf(-sv, sfu_lg2(sv), acc[j]);
                }
            }
        }
    }
}

// exact deviance with the reference patch already scaled and clamped (.x)
__device__ __forceinline__ float exact_deviance(const float2* __restrict__ ref, const float* __restrict__ src,
                                                int64_t origin, const int32_t* __restrict__ poff, int P,
                                                float inv) {
    float d = 0.0f;
    for (int p = 0; p < P; ++p) {
        const float r = ref[p].x;
        float c = mul_rn(__ldg(src + origin + poff[p]), inv);
        if (c < 0.0f) c = 0.0f;
        if (add_rn(r, c) > 0.0f) d = add_rn(d, deviance_term(r, c));
    }
    if (d < 0.0f) d = 0.0f;
    return div_rn(d, static_cast<float>(P));
}

constexpr int kSThreads = 128;   // one CTA per reference
constexpr int kSQueue = 512;     // rescoring queue (overflow -> exact redo)

// per-CTA shared layout of the screened kernel
struct ScreenSmem {
    __host__ __device__ static size_t cand(int64_t wmax) { return (static_cast<size_t>(wmax) * 4 + 15) & ~size_t(15); }
    __host__ __device__ static size_t bytes(int P, int64_t wmax) {
        return ((static_cast<size_t>(P) * 4 + 15) & ~size_t(15))   // poff
               + static_cast<size_t>(P) * 8                           // ref (r, 2r)
               + cand(wmax)                                           // screening distances
               + 256 * 4                                              // histogram
               + kSQueue * 4 + kSQueue * 8                            // queue index, exact keys
               + kSQueue * 4                                          // subsampled mode: compact -> window index
               + 64 * 8                                               // scratch (reductions, top list)
               + 64;
    }
};

// resident CTAs per SM the screened kernel is compiled for, and the x-run of
// candidates one thread scores in approximate mode (compile-time tunables)
#ifndef BMND_SCREEN_MIN_BLOCKS
#define BMND_SCREEN_MIN_BLOCKS 8
#endif
#ifndef BMND_APPROX_XR
#define BMND_APPROX_XR 2
#endif
// x-run of the subsampled prescreen.  3 divides the default 15-wide window
// rows, but its warps span more window rows per load; at 256^3 the matching
// took 31.0 ms with 3 against 28.1 ms with 2
#ifndef BMND_SUB_XR
#define BMND_SUB_XR 2
#endif

template <int ND, int B0, int B1, int B2>
__global__ void __launch_bounds__(kSThreads, BMND_SCREEN_MIN_BLOCKS) blockmatch_screened_kernel(MatchArgs a,
                                                                                              int32_t wmax) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int tid = threadIdx.x;
    const int warp = tid >> 5, lane = tid & 31;
    const int P = a.P;
    const int K = a.max_m;
    const int R = a.required;
    unsigned char* b = smem_raw;
    int32_t* poff_s = reinterpret_cast<int32_t*>(b);
    b += (static_cast<size_t>(P) * 4 + 15) & ~size_t(15);
    float2* ref = reinterpret_cast<float2*>(b);
    b += static_cast<size_t>(P) * 8;
    float* cand = reinterpret_cast<float*>(b);
    b += ScreenSmem::cand(wmax);
    uint32_t* hist = reinterpret_cast<uint32_t*>(b);
    b += 256 * 4;
    int32_t* qidx = reinterpret_cast<int32_t*>(b);
    b += kSQueue * 4;
    uint64_t* qkey = reinterpret_cast<uint64_t*>(b);
    b += kSQueue * 8;
    int32_t* cmap = reinterpret_cast<int32_t*>(b);
    b += kSQueue * 4;
    uint64_t* top = reinterpret_cast<uint64_t*>(b);  // [32]
    float* redf = reinterpret_cast<float*>(top + 32);  // [4 warps]
    int* redi = reinterpret_cast<int*>(redf + 8);      // [8]

    for (int i = tid; i < P; i += blockDim.x) {
        if (a.table) {
            poff_s[i] = i;
        } else {
            int rem = i;
            int64_t o = 0;
            for (int d = a.ndim - 1; d >= 0; --d) {
                o += static_cast<int64_t>(rem % a.block[d]) * a.vstride[d];
                rem /= a.block[d];
            }
            poff_s[i] = static_cast<int32_t>(o);
        }
    }
    const bool fixed = ND > 0 && !a.table && a.inv_scale == 1.0f;
    // relative part of the bound: float32 accumulation of both sums (P 2^-24 each)
    // and the final scalings, x2
    const float drel = a.approx ? 0.0f : 2.0f * (2.0f * 5.96046448e-08f * static_cast<float>(P) + 4.76837158e-07f);

    for (int64_t r = blockIdx.x; r < a.n_refs; r += gridDim.x) {
        int lo[BMND_MAX_DIMS] = {0, 0, 0}, ext[BMND_MAX_DIMS] = {1, 1, 1};
        float inv_ext[BMND_MAX_DIMS] = {1.0f, 1.0f, 1.0f};
        int64_t center_lin = 0, center_origin = 0, window = 1;
#pragma unroll
        for (int d = 0; d < BMND_MAX_DIMS; ++d) {
            if (d < a.ndim) {
                const int cd = a.refs[r * a.ndim + d];
                center_lin = center_lin * a.counts[d] + cd;
                center_origin += static_cast<int64_t>(cd) * a.grid_stride[d];
                const int l = max(cd - a.radius[d], 0);
                const int h = min(cd + a.radius[d], a.counts[d] - 1);
                lo[d] = l;
                ext[d] = h - l + 1;
                inv_ext[d] = 1.0f / static_cast<float>(ext[d]);
                window *= ext[d];
            }
        }
        const bool small_window = window < (int64_t(1) << 21);
        __syncthreads();  // previous reference's shared data is no longer read
        const bool cheap = fixed && a.approx && a.cv != nullptr;
        float sa = 0.0f, sa_sub = 0.0f;  // cheap mode: sum_p A_r over the patch and over its even sub-lattice
        for (int p = tid; p < P; p += blockDim.x) {
            float rv = mul_rn(__ldg(a.src + center_origin + poff_s[p]), a.inv_scale);
            if (rv < 0.0f) rv = 0.0f;
            if (cheap) {
                const float av = rv > 0.0f ? rv + rv * log2f(rv) : 0.0f;
                sa += av;
                if constexpr (ND > 0)
                    if (sub_lattice<ND, B0, B1, B2>(p)) sa_sub += av;
            }
            ref[p] = make_float2(rv, cheap ? fmaxf(rv, 7.88860905e-31f) : rv + rv);
        }
        if (cheap) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                sa += __shfl_xor_sync(0xffffffffu, sa, o);
                sa_sub += __shfl_xor_sync(0xffffffffu, sa_sub, o);
            }
            if (lane == 0) {
                redf[4 + warp] = sa;
                reinterpret_cast<float*>(redi + 16)[warp] = sa_sub;
            }
        }
        for (int i = tid; i < 256; i += blockDim.x) hist[i] = 0u;
        if (tid == 0) {
            redi[0] = 0;  // queue length
            redi[3] = 0;  // accepted keys in the queue
        }
        __syncthreads();
        const float thr = a.thresholds ? a.thresholds[r] : (a.thr_dev ? *a.thr_dev : a.scalar_threshold);
        const float tkey = canonical_key(thr);

        float Dabs = 0.0f;  // the reference-wide absolute bound, set after pass A
        const float drel_k = drel;
        // candidates still in the race: the whole window, or (subsampled mode)
        // the prescreened ones, compacted to cand[0, wlen) with cmap[] their
        // window indices
        int64_t wlen = window;
        bool compact = false;
        // radix select over the upper bounds d + D of the certainly accepted
        // (of every candidate with `all`): the smallest v with >= need of them
        // bounded by it, or infinity when there are fewer.  `passes` 8-bit
        // digits are resolved; with 2 the result is the top of its 16-bit bin,
        // so the candidates bounded by it are a superset of those bounded by
        // the 3-pass result (the approximate modes, whose selections are
        // heuristic anyway, take the pass and its barriers off)
        auto select_kth = [&](int need, bool all, int passes) -> float {
            uint32_t prefix = 0;
            bool found = true;
            for (int i = tid; i < 256; i += blockDim.x) hist[i] = 0u;
            __syncthreads();
            for (int pass = 0; pass < passes && found; ++pass) {
                const int shift = 24 - 8 * pass;
                if (pass > 0) {
                    for (int i = tid; i < 256; i += blockDim.x) hist[i] = 0u;
                    __syncthreads();
                }
                // warp-uniform sweep; lanes that share a bin add once (most
                // candidates share the leading bits, so plain atomics serialise)
                for (int64_t base = static_cast<int64_t>(warp) * 32; base < wlen; base += blockDim.x) {
                    const int64_t c = base + lane;
                    bool take = false;
                    uint32_t bin = 0;
                    if (c < wlen) {
                        const float dv = cand[c];
                        const float up = dv + (Dabs + drel_k * dv);
                        if (all || canonical_key(up) < tkey) {
                            const uint32_t bits = __float_as_uint(up);
                            if (pass == 0 || (bits >> (32 - 8 * pass)) == prefix) {
                                take = true;
                                bin = (bits >> shift) & 0xffu;
                            }
                        }
                    }
                    const unsigned tm = __ballot_sync(0xffffffffu, take);
                    if (take) {
                        const unsigned peers = __match_any_sync(tm, bin);
                        if (lane == __ffs(peers) - 1) atomicAdd(hist + bin, static_cast<uint32_t>(__popc(peers)));
                    }
                }
                __syncthreads();
                if (warp == 0) {
                    uint32_t local[8];
                    uint32_t lsum = 0;
#pragma unroll
                    for (int i = 0; i < 8; ++i) {
                        local[i] = hist[lane * 8 + i];
                        lsum += local[i];
                    }
                    uint32_t incl = lsum;
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
                        if (lane >= o) incl += t;
                    }
                    const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
                    int bin = -1;
                    uint32_t before = 0;
                    if (total >= static_cast<uint32_t>(need)) {
                        uint32_t run = incl - lsum;
#pragma unroll
                        for (int i = 0; i < 8; ++i) {
                            if (bin < 0 && run + local[i] >= static_cast<uint32_t>(need)) {
                                bin = lane * 8 + i;
                                before = run;
                            }
                            run += local[i];
                        }
                    }
                    const unsigned has = __ballot_sync(0xffffffffu, bin >= 0);
                    if (lane == 0 && !has) redi[1] = -1;
                    if (has) {
                        const int src_lane = __ffs(has) - 1;
                        const int bsel = __shfl_sync(0xffffffffu, bin, src_lane);
                        const uint32_t bef = __shfl_sync(0xffffffffu, before, src_lane);
                        if (lane == 0) {
                            redi[1] = bsel;
                            redi[2] = static_cast<int>(bef);
                        }
                    }
                }
                __syncthreads();
                const int bsel = redi[1];
                if (bsel < 0) {
                    found = false;
                } else {
                    need -= redi[2];
                    prefix = pass == 0 ? static_cast<uint32_t>(bsel) : ((prefix << 8) | static_cast<uint32_t>(bsel));
                }
                __syncthreads();
            }
            if (!found) return INFINITY;
            return passes == 3 ? __uint_as_float((prefix << 8) | 0xffu) : __uint_as_float((prefix << 16) | 0xffffu);
        };

        // pass A: screening distances and the reference-wide absolute bound
        float dmax = 0.0f;
        if (cheap && !a.sub) {
            if constexpr (ND > 0) {
                constexpr int XR = BMND_APPROX_XR;
                constexpr int BX = ND == 3 ? B2 : B1;
                const float sum_a = redf[4] + redf[5] + redf[6] + redf[7];
                const int ex = ext[ND - 1];
                const int nu = (ex + XR - 1) / XR;
                const float inv_nu = 1.0f / static_cast<float>(nu);
                const int nx = a.counts[ND - 1] + BX - 1;  // voxels along x
                const int64_t units = window / ex * nu;
                for (int64_t u = tid; u < units; u += blockDim.x) {
                    // unit -> (row of the window, x run); rows are C-ordered over the outer axes
                    const int ui = static_cast<int>(u);
                    const int rowi = small_div(ui, inv_nu);
                    const int k = ui - rowi * nu;
                    int64_t origin = 0;
                    if (ND == 3) {
                        const int i0 = small_div(rowi, inv_ext[1]);
                        const int i1 = rowi - i0 * ext[1];
                        origin = static_cast<int64_t>(lo[0] + i0) * a.grid_stride[0] +
                                 static_cast<int64_t>(lo[1] + i1) * a.grid_stride[1];
                    } else {
                        origin = static_cast<int64_t>(lo[0] + rowi) * a.grid_stride[0];
                    }
                    const int x0 = lo[ND - 1] + k * XR;
                    origin += x0;
                    float acc[XR];
                    approx_unit<ND, B0, B1, B2, XR, 1>(ref, a.cv, origin, a.vstride[0], a.vstride[ND > 1 ? 1 : 0],
                                                       nx - x0, acc);
                    const int64_t c0 = static_cast<int64_t>(rowi) * ex + k * XR;
                    const int nvalid = min(XR, ex - k * XR);
#pragma unroll
                    for (int j = 0; j < XR; ++j) {
                        if (j < nvalid) {
                            const float d = 1.38629436f * (sum_a + __ldg(a.boxb + origin + j) + acc[j]);
                            cand[c0 + j] = fmaxf(d, 0.0f) / static_cast<float>(P);
                        }
                    }
                }
            }
        } else if (cheap) {
            // subsampled mode, pass A': the same screening form on the even
            // sub-lattice of the patch for every candidate, then the full form
            // for the a.presel smallest; the rest are out of the race
            if constexpr (ND > 0) {
                constexpr int XR = BMND_SUB_XR;
                constexpr int BX = ND == 3 ? B2 : B1;
                constexpr int PS = ((B0 + 1) / 2) * ((B1 + 1) / 2) * (ND == 3 ? (B2 + 1) / 2 : 1);
                const float* fs = reinterpret_cast<const float*>(redi + 16);
                const float sum_s = fs[0] + fs[1] + fs[2] + fs[3];
                const int ex = ext[ND - 1];
                const int nu = (ex + XR - 1) / XR;
                const float inv_nu = 1.0f / static_cast<float>(nu);
                const int nx = a.counts[ND - 1] + BX - 1;
                const int64_t units = window / ex * nu;
                for (int64_t u = tid; u < units; u += blockDim.x) {
                    const int ui = static_cast<int>(u);
                    const int rowi = small_div(ui, inv_nu);
                    const int k = ui - rowi * nu;
                    int64_t origin = 0;
                    if (ND == 3) {
                        const int i0 = small_div(rowi, inv_ext[1]);
                        const int i1 = rowi - i0 * ext[1];
                        origin = static_cast<int64_t>(lo[0] + i0) * a.grid_stride[0] +
                                 static_cast<int64_t>(lo[1] + i1) * a.grid_stride[1];
                    } else {
                        origin = static_cast<int64_t>(lo[0] + rowi) * a.grid_stride[0];
                    }
                    const int x0 = lo[ND - 1] + k * XR;
                    origin += x0;
                    float acc[XR];
                    approx_unit<ND, B0, B1, B2, XR, 2>(ref, a.cv, origin, a.vstride[0], a.vstride[ND > 1 ? 1 : 0],
                                                       nx - x0, acc);
                    const int64_t c0 = static_cast<int64_t>(rowi) * ex + k * XR;
                    const int nvalid = min(XR, ex - k * XR);
#pragma unroll
                    for (int j = 0; j < XR; ++j) {
                        if (j < nvalid) {
                            const float d = 1.38629436f * (sum_s + __ldg(a.boxb_sub + origin + j) + acc[j]);
                            cand[c0 + j] = fmaxf(d, 0.0f) / static_cast<float>(PS);
                        }
                    }
                }
                __syncthreads();
                const float vs = select_kth(a.presel, true, 2);
                const float vskey = canonical_key(vs);
                // the prescreened candidates in window order (ballots and warp
                // counts, no atomics), so that when ties at the cut fill the
                // queue the same candidates are kept on every run
                // (warp w takes a contiguous 1/nwarps of the window: it counts
                // its candidates, the warps' counts are added in warp order, and
                // it writes them; two barriers in all)
                const int nwarps = static_cast<int>(blockDim.x >> 5);
                const int64_t span = ((window + nwarps - 1) / nwarps + 31) / 32 * 32;
                const int64_t w0 = min(window, static_cast<int64_t>(warp) * span);
                const int64_t w1 = min(window, w0 + span);
                int mine = 0;
                for (int64_t c0 = w0; c0 < w1; c0 += 32) {
                    const int64_t c = c0 + lane;
                    const bool take = c < w1 && canonical_key(cand[c]) <= vskey;
                    mine += __popc(__ballot_sync(0xffffffffu, take));
                }
                if (lane == 0) hist[warp] = static_cast<uint32_t>(mine);
                __syncthreads();
                int before = 0, nq = 0;
                for (int w = 0; w < nwarps; ++w) {
                    const int cw = static_cast<int>(hist[w]);
                    if (w < warp) before += cw;
                    nq += cw;
                }
                for (int64_t c0 = w0; c0 < w1; c0 += 32) {
                    const int64_t c = c0 + lane;
                    const bool take = c < w1 && canonical_key(cand[c]) <= vskey;
                    const unsigned m = __ballot_sync(0xffffffffu, take);
                    if (take) {
                        const int slot = before + __popc(m & ((1u << lane) - 1u));
                        if (slot < kSQueue) qidx[slot] = static_cast<int32_t>(c);
                    }
                    before += __popc(m);
                }
                __syncthreads();
                const int nsel = min(nq, kSQueue);
                const float sum_a = redf[4] + redf[5] + redf[6] + redf[7];
                for (int i = tid; i < nsel; i += blockDim.x) {
                    int64_t lin;
                    const int64_t origin = window_origin(a, lo, ext, inv_ext, small_window, qidx[i], &lin);
                    float acc[1];
                    approx_unit<ND, B0, B1, B2, 1, 1>(ref, a.cv, origin, a.vstride[0], a.vstride[ND > 1 ? 1 : 0],
                                                      BX, acc);
                    const float d = 1.38629436f * (sum_a + __ldg(a.boxb + origin) + acc[0]);
                    cand[i] = fmaxf(d, 0.0f) / static_cast<float>(P);  // compacted (nothing reads cand here)
                    cmap[i] = qidx[i];
                }
                __syncthreads();
                wlen = nsel;
                compact = true;
                if (tid == 0) redi[0] = 0;
            }
        } else {
            for (int64_t c = tid; c < window; c += blockDim.x) {
                int64_t lin;
                const int64_t origin = window_origin(a, lo, ext, inv_ext, small_window, c, &lin);
                const float2 sd = fixed ? screen_deviance_fixed<ND, B0, B1, B2>(ref, a.src, origin, a.vstride[0],
                                                                                a.vstride[ND > 1 ? 1 : 0], poff_s)
                                        : screen_deviance(ref, a.src, origin, poff_s, P, a.inv_scale);
                cand[c] = sd.x;
                dmax = fmaxf(dmax, sd.y);
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) dmax = fmaxf(dmax, __shfl_xor_sync(0xffffffffu, dmax, o));
        if (lane == 0) redf[warp] = dmax;
        __syncthreads();
        Dabs = redf[0];
        for (int w = 1; w < static_cast<int>(blockDim.x >> 5); ++w) Dabs = fmaxf(Dabs, redf[w]);
        if (a.approx) Dabs = 0.0f;

        const float vstar = select_kth(K, false, a.approx ? 2 : 3);
        // at least K certainly accepted candidates have exact distances <= vstar
        const float vkey = canonical_key(vstar);

        // pass C: classify; queue the uncertain and the possible top-K members
        int acc_t = 0;
        for (int64_t c = tid; c < wlen; c += blockDim.x) {
            const float dv = cand[c];
            const float D = Dabs + drel * dv;
            const float lo_key = canonical_key(fmaxf(dv - D, 0.0f));
            const bool cert = canonical_key(dv + D) < tkey;
            const bool poss = lo_key < tkey;
            if (cert) ++acc_t;
            if (poss && (!cert || lo_key <= vkey)) {
                const int slot = atomicAdd(redi, 1);
                if (slot < kSQueue)
                    qidx[slot] = (compact ? cmap[c] : static_cast<int32_t>(c)) |
                                 (cert ? static_cast<int32_t>(0x80000000u) : 0);
            }
        }
        __syncthreads();
        const int qn_all = redi[0];
        const bool overflow = qn_all > kSQueue;
        const int qn = overflow ? 0 : qn_all;
        // rescoring of the queue.  Fast mode: the exact float32 distance, one
        // thread per candidate, bit-identical to the exact kernel.  Approx mode:
        // the ratio form of the screened mode (one SFU reciprocal and two log2
        // per term, free of cancellation, within 4e-6 per unit of r + c of the
        // exact terms) over the full patch, one warp per candidate (lanes over
        // patch elements, tree-ordered sum), so the whole CTA works on the queue;
        // the IEEE division and two full logarithms of the exact term cost
        // about eight times as many instructions.
        if (a.approx) {
            const int nwarps = static_cast<int>(blockDim.x >> 5);
            for (int i = warp; i < qn; i += nwarps) {
                const int32_t q = qidx[i];
                int64_t lin;
                const int64_t origin = window_origin(a, lo, ext, inv_ext, small_window, q & 0x7fffffff, &lin);
                float d = 0.0f, ss = 0.0f;
                for (int p = lane; p < P; p += 32) {
                    float c = mul_rn(__ldg(a.src + origin + poff_s[p]), a.inv_scale);
                    if (c < 0.0f) c = 0.0f;
                    const float r = ref[p].x;
                    d += ratio_term(r, r + r, c, ss);
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
                if (lane == 0) {
                    const float key = canonical_key(fmaxf(1.38629436f * d, 0.0f) / static_cast<float>(P));
                    const bool accepted = key < tkey;
                    if (accepted && q >= 0) ++acc_t;
                    qkey[i] = accepted ? composite_key(key, static_cast<int32_t>(lin)) : ~0ull;
                }
            }
        } else {
            for (int i = tid; i < qn; i += blockDim.x) {
                const int32_t q = qidx[i];
                int64_t lin;
                const int64_t origin = window_origin(a, lo, ext, inv_ext, small_window, q & 0x7fffffff, &lin);
                const float dist = exact_deviance(ref, a.src, origin, poff_s, P, a.inv_scale);
                const float key = canonical_key(dist);
                const bool accepted = key < tkey;
                if (accepted && q >= 0) ++acc_t;
                qkey[i] = accepted ? composite_key(key, static_cast<int32_t>(lin)) : ~0ull;
            }
        }
        // accepted count (block sum)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc_t += __shfl_xor_sync(0xffffffffu, acc_t, o);
        if (lane == 0) redi[4 + warp] = acc_t;
        __syncthreads();
        int total_accepted = 0;
        for (int w = 0; w < static_cast<int>(blockDim.x >> 5); ++w) total_accepted += redi[4 + w];
        bool complete = !overflow && total_accepted >= R;
        int limit = K;  // entries of top[] the group takes
        // top K of the rescored accepted keys: each key's rank among the queue
        // (composite keys are unique), in parallel
        if (complete) {
            for (int i = tid; i < qn; i += blockDim.x) {
                const uint64_t k = qkey[i];
                if (k == ~0ull) continue;
                int rank = 0;
                for (int j = 0; j < qn; ++j) rank += qkey[j] < k ? 1 : 0;
                if (rank < K) top[rank] = k;
                atomicAdd(redi + 3, 1);
            }
        } else if (a.approx && !overflow) {
            // approximate mode, fewer than `required` accepted: the group is the
            // R smallest screening distances overall, the accepted (below the
            // threshold) first, then the best rejected, as the reference fills it
            __syncthreads();
            const float v2 = select_kth(R, true, 3);
            const float v2key = canonical_key(v2);
            if (tid == 0) {
                redi[0] = 0;
                redi[3] = 0;
            }
            __syncthreads();
            for (int64_t c = tid; c < wlen; c += blockDim.x) {
                if (canonical_key(cand[c]) <= v2key) {
                    const int slot = atomicAdd(redi, 1);
                    if (slot < kSQueue) qidx[slot] = static_cast<int32_t>(c);
                }
            }
            __syncthreads();
            const int qn2 = redi[0];
            if (qn2 <= kSQueue) {
                for (int i = tid; i < qn2; i += blockDim.x) {
                    int64_t lin;
                    (void)window_origin(a, lo, ext, inv_ext, small_window, compact ? cmap[qidx[i]] : qidx[i], &lin);
                    qkey[i] = composite_key(canonical_key(cand[qidx[i]]), static_cast<int32_t>(lin));
                }
                __syncthreads();
                for (int i = tid; i < qn2; i += blockDim.x) {
                    const uint64_t k = qkey[i];
                    int rank = 0;
                    for (int j = 0; j < qn2; ++j) rank += qkey[j] < k ? 1 : 0;
                    if (rank < R) top[rank] = k;
                    atomicAdd(redi + 3, 1);
                }
                complete = true;
                limit = R;
            }
        }
        __syncthreads();
        if (tid == 0) {
            if (!complete) {
                a.count[r] = -1;  // queue overflow, or the best rejected are needed: exact redo
            } else {
                const int ntop = min(redi[3], limit);
                int32_t* row = a.sel + r * K;
                int n = 0;
                row[n++] = static_cast<int32_t>(center_lin);
                for (int t = 0; t < ntop && n < K; ++t) {
                    const int32_t l = static_cast<int32_t>(top[t] & 0xffffffffu);
                    if (l < 0 || l == center_lin) continue;
                    row[n++] = l;
                }
                if (a.pow2 && n > 0) {
                    int target = 1;
                    while ((target << 1) <= n) target <<= 1;
                    if (a.min_m > target) target = a.min_m;
                    if (target < n) n = target;
                }
                for (int t = n; t < K; ++t) row[t] = -1;
                a.count[r] = n;
                a.accepted[r] = total_accepted;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Integer-count Poisson-deviance matching (volume source, count scale 1)
//
// One CTA per reference.  For Poisson counts almost every term of the deviance
// pairs two small integers, so the CTA tabulates, per reference,
//   trow[p][c] = deviance_term(r_p, c),  c = 0..62,
// (one row per patch element; rows of integer r_p < 63 are copied from a
// 64 x 64 table of the same function, others are evaluated directly) and
// stages the search box of the reference as byte codes 4 * c (c = the clamped
// count if it is an integer below 63, else 63, whose table entry is NaN).  A
// term is then one byte load, one table load and one float32 add, in the
// reference's patch order, so the sum is bit-identical to the per-term
// evaluation; a candidate whose sum came out NaN (it touched a code-63 voxel)
// is recomputed term by term from the float source.  Selection keeps one
// ascending top-K list per thread (accepted and rejected, as the warp kernel
// does), merged per warp and then across the CTA's warps.
// ---------------------------------------------------------------------------
constexpr int kCThreads = 128;
constexpr int kCWarps = kCThreads / 32;
constexpr int kCodes = 64;      // row length of trow; code 63 marks "not tabulated"
constexpr int kCodeMax = 63;    // counts 0..62 are tabulated

__device__ float g_count_table[kCodes * kCodes];  // deviance_term(r, c), r, c < 64

__global__ void count_table_kernel() {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kCodes * kCodes; i += gridDim.x * blockDim.x)
        g_count_table[i] = deviance_term(static_cast<float>(i / kCodes), static_cast<float>(i % kCodes));
}

// Shared layout of the count kernel; every section starts on a 16-byte
// boundary.  trow comes first: its byte offset is a compile-time 0, so a
// term's table load addresses [code + p * 256].
struct CountSmem {
    size_t trow, box, poff, ref, lists, wmerged, fin, total;
    __host__ __device__ CountSmem(int P, int64_t boxmax, int rows) {
        auto r16 = [](size_t v) { return (v + 15) & ~size_t(15); };
        size_t o = 0;
        trow = o;
        o += r16(static_cast<size_t>(P) * kCodes * 4);               // per-reference table
        box = o;
        o += r16(static_cast<size_t>(boxmax));                       // box codes
        poff = o;
        o += r16(static_cast<size_t>(P) * 4);                        // voxel offsets of the patch
        ref = o;
        o += r16(static_cast<size_t>(P) * 8);                        // reference values, row index
        lists = o;
        o += r16(static_cast<size_t>(rows) * kCThreads * 8);         // per-thread lists
        wmerged = o;
        o += r16(static_cast<size_t>(kCWarps) * rows * 8);           // per-warp merged lists
        fin = o;
        o += 64 * 8;                                                 // final lists (48), reductions (16 ints)
        total = o;
    }
};

// ascending list of `size` entries (capacity `cap`) at list[i * stride]
__device__ __forceinline__ int list_insert_s(uint64_t* list, int stride, int size, int cap, uint64_t key) {
    if (cap == 0) return size;
    int at;
    if (size < cap) {
        at = size;
        ++size;
    } else {
        if (key >= list[(cap - 1) * stride]) return size;
        at = cap - 1;
    }
    while (at > 0) {
        const uint64_t prev = list[(at - 1) * stride];
        if (key >= prev) break;
        list[at * stride] = prev;
        --at;
    }
    list[at * stride] = key;
    return size;
}

// warp-wide merge of one ascending list per lane (mine[i * stride], `size`
// entries) into out[0..cap); returns the merged size
__device__ int warp_merge_s(const uint64_t* mine_list, int stride, int size, int cap, uint64_t* out, int lane) {
    int head = 0, n = 0;
    for (int t = 0; t < cap; ++t) {
        const uint64_t mine = head < size ? mine_list[head * stride] : ~0ull;
        const uint64_t best = warp_min_u64(mine);
        if (best == ~0ull) break;
        if (mine == best) ++head;
        if (lane == 0) out[t] = best;
        ++n;
    }
    return n;
}

template <int ND, int B0, int B1, int B2>
__device__ __forceinline__ float counts_distance_fixed(const unsigned char* __restrict__ smem,
                                                       const unsigned char* __restrict__ cand, int S0, int S1) {
    float d = 0.0f;
#pragma unroll
    for (int a0 = 0; a0 < B0; ++a0) {
#pragma unroll
        for (int a1 = 0; a1 < B1; ++a1) {
            const unsigned char* row = cand + a0 * S0 + (ND == 3 ? a1 * S1 : a1);
#pragma unroll
            for (int a2 = 0; a2 < B2; ++a2) {
                constexpr int kRow = kCodes * 4;
                const int p = (a0 * B1 + a1) * B2 + a2;
                const unsigned code4 = row[ND == 3 ? a2 : 0];
                d = add_rn(d, *reinterpret_cast<const float*>(smem + code4 + p * kRow));
            }
        }
    }
    return d;
}

template <int ND, int B0, int B1, int B2>
__global__ void __launch_bounds__(kCThreads, 4) blockmatch_counts_kernel(MatchArgs a, int32_t rows) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int tid = threadIdx.x;
    const int warp = tid >> 5, lane = tid & 31;
    const int P = a.P;
    const int K = a.max_m;
    const int R = a.required;
    const int nd = ND > 0 ? ND : a.ndim;
    int64_t boxmax = 1;
    for (int d = 0; d < nd; ++d) boxmax *= min(2 * a.radius[d] + 1, a.counts[d]) + a.block[d] - 1;
    const CountSmem L(P, boxmax, rows);
    float* trow = reinterpret_cast<float*>(smem + L.trow);
    unsigned char* box = smem + L.box;
    int32_t* poff_s = reinterpret_cast<int32_t*>(smem + L.poff);
    float* refv = reinterpret_cast<float*>(smem + L.ref);
    int* refi = reinterpret_cast<int*>(refv + P);
    uint64_t* lists = reinterpret_cast<uint64_t*>(smem + L.lists);      // [rows][kCThreads]
    uint64_t* wmerged = reinterpret_cast<uint64_t*>(smem + L.wmerged);  // [kCWarps][rows]
    uint64_t* fin = reinterpret_cast<uint64_t*>(smem + L.fin);          // [K + R <= 48] final merged keys
    int* redi = reinterpret_cast<int*>(fin + 48);                        // [16]

    for (int i = tid; i < P; i += blockDim.x) {
        int rem = i;
        int64_t o = 0;
        for (int d = nd - 1; d >= 0; --d) {
            o += static_cast<int64_t>(rem % a.block[d]) * a.vstride[d];
            rem /= a.block[d];
        }
        poff_s[i] = static_cast<int32_t>(o);
    }
    uint64_t* acc_list = lists + tid;
    uint64_t* rej_list = lists + static_cast<size_t>(K) * kCThreads + tid;

    for (int64_t r = blockIdx.x; r < a.n_refs; r += gridDim.x) {
        int lo[BMND_MAX_DIMS] = {0, 0, 0}, ext[BMND_MAX_DIMS] = {1, 1, 1}, bx[BMND_MAX_DIMS] = {1, 1, 1};
        float inv_ext[BMND_MAX_DIMS] = {1.0f, 1.0f, 1.0f};
        int64_t center_lin = 0, center_origin = 0, window = 1, nbox = 1;
#pragma unroll
        for (int d = 0; d < BMND_MAX_DIMS; ++d) {
            if (d < nd) {
                const int cd = a.refs[r * nd + d];
                center_lin = center_lin * a.counts[d] + cd;
                center_origin += static_cast<int64_t>(cd) * a.vstride[d];
                const int l = max(cd - a.radius[d], 0);
                const int h = min(cd + a.radius[d], a.counts[d] - 1);
                lo[d] = l;
                ext[d] = h - l + 1;
                inv_ext[d] = 1.0f / static_cast<float>(ext[d]);
                bx[d] = ext[d] + a.block[d] - 1;
                window *= ext[d];
                nbox *= bx[d];
            }
        }
        const bool small_window = window < (int64_t(1) << 21);
        __syncthreads();  // the previous reference's shared data is no longer read
        // reference values and their table rows
        for (int p = tid; p < P; p += blockDim.x) {
            float v = __ldg(a.src + center_origin + poff_s[p]);
            if (v < 0.0f) v = 0.0f;
            const int vi = __float2int_rz(v);
            refv[p] = v;
            refi[p] = (vi < kCodeMax && __int2float_rn(vi) == v) ? vi * kCodes : -1;
        }
        // search box as byte codes, one box row (last axis) per warp pass
        {
            const int inner = bx[nd - 1];
            const int64_t nrows = nbox / inner;
            for (int64_t row = warp; row < nrows; row += kCWarps) {
                int64_t rem = row, vo = 0;
                for (int d = nd - 2; d >= 0; --d) {
                    vo += static_cast<int64_t>(lo[d] + static_cast<int>(rem % bx[d])) * a.vstride[d];
                    rem /= bx[d];
                }
                vo += lo[nd - 1];
                for (int x = lane; x < inner; x += 32) {
                    float v = __ldg(a.src + vo + x);
                    if (v < 0.0f) v = 0.0f;
                    const int vi = __float2int_rz(v);
                    const int code = (vi < kCodeMax && __int2float_rn(vi) == v) ? vi : kCodeMax;
                    box[row * inner + x] = static_cast<unsigned char>(code * 4);
                }
            }
        }
        __syncthreads();
        for (int e = tid; e < P * kCodes; e += blockDim.x) {
            const int p = e / kCodes, c = e % kCodes;
            const int ri = refi[p];
            float t;
            if (c == kCodeMax) t = __int_as_float(0x7fc00000);
            else if (ri >= 0) t = g_count_table[ri + c];
            else t = deviance_term(refv[p], static_cast<float>(c));
            trow[e] = t;
        }
        __syncthreads();

        const float thr = a.thresholds ? a.thresholds[r] : (a.thr_dev ? *a.thr_dev : a.scalar_threshold);
        const float tkey = canonical_key(thr);
        int acc_size = 0, rej_size = 0, acc_count = 0;
        const int S0 = nd == 3 ? bx[1] * bx[2] : bx[1];
        const int S1 = nd == 3 ? bx[2] : 1;
        for (int64_t c = tid; c < window; c += blockDim.x) {
            int w[BMND_MAX_DIMS] = {0, 0, 0};
            if (small_window) {
                int rem = static_cast<int>(c);
#pragma unroll
                for (int d = BMND_MAX_DIMS - 1; d >= 0; --d) {
                    if (d < nd) {
                        const int q = d > 0 ? small_div(rem, inv_ext[d]) : 0;
                        w[d] = rem - q * ext[d];
                        rem = q;
                    }
                }
            } else {
                int64_t rem = c;
#pragma unroll
                for (int d = BMND_MAX_DIMS - 1; d >= 0; --d) {
                    if (d < nd) {
                        w[d] = static_cast<int>(rem % ext[d]);
                        rem /= ext[d];
                    }
                }
            }
            int64_t lin = 0;
            int boff = 0;
#pragma unroll
            for (int d = 0; d < BMND_MAX_DIMS; ++d) {
                if (d < nd) {
                    lin = lin * a.counts[d] + lo[d] + w[d];
                    boff = boff * bx[d] + w[d];
                }
            }
            float dsum;
            if constexpr (ND > 0) {
                dsum = counts_distance_fixed<ND, B0, B1, B2>(smem, box + boff, S0, S1);
            } else {
                dsum = 0.0f;
                for (int p = 0; p < P; ++p) {
                    int rp = p, bo = 0, mul = 1;
                    for (int d = nd - 1; d >= 0; --d) {
                        bo += (rp % a.block[d]) * mul;
                        mul *= bx[d];
                        rp /= a.block[d];
                    }
                    const unsigned code4 = box[boff + bo];
                    dsum = add_rn(dsum, *reinterpret_cast<const float*>(smem + code4 + p * (kCodes * 4)));
                }
            }
            if (dsum != dsum) {
                // a voxel outside the table: term-by-term evaluation from the source
                int64_t origin = 0;
#pragma unroll
                for (int d = 0; d < BMND_MAX_DIMS; ++d)
                    if (d < nd) origin += static_cast<int64_t>(lo[d] + w[d]) * a.vstride[d];
                dsum = 0.0f;
                for (int p = 0; p < P; ++p) {
                    float cv = __ldg(a.src + origin + poff_s[p]);
                    if (cv < 0.0f) cv = 0.0f;
                    const float rv = refv[p];
                    if (add_rn(rv, cv) > 0.0f) dsum = add_rn(dsum, deviance_term(rv, cv));
                }
            }
            if (dsum < 0.0f) dsum = 0.0f;
            const float key = canonical_key(div_rn(dsum, static_cast<float>(P)));
            const uint64_t ck = composite_key(key, static_cast<int32_t>(lin));
            if (key < tkey) {
                ++acc_count;
                acc_size = list_insert_s(acc_list, kCThreads, acc_size, K, ck);
            } else {
                rej_size = list_insert_s(rej_list, kCThreads, rej_size, R, ck);
            }
        }
        // per-warp merge, then across warps
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc_count += __shfl_xor_sync(0xffffffffu, acc_count, o);
        uint64_t* wm = wmerged + static_cast<size_t>(warp) * rows;
        const int n_acc_w = warp_merge_s(acc_list, kCThreads, acc_size, K, wm, lane);
        const int n_rej_w = warp_merge_s(rej_list, kCThreads, rej_size, R, wm + K, lane);
        if (lane == 0) {
            redi[warp] = n_acc_w;
            redi[kCWarps + warp] = n_rej_w;
            redi[2 * kCWarps + warp] = acc_count;
        }
        __syncthreads();
        if (warp == 0) {
            const bool mine = lane < kCWarps;
            const uint64_t* ml = wmerged + static_cast<size_t>(mine ? lane : 0) * rows;
            const int n_acc = warp_merge_s(ml, 1, mine ? redi[lane] : 0, K, fin, lane);
            const int n_rej = warp_merge_s(ml + K, 1, mine ? redi[kCWarps + lane] : 0, R, fin + K, lane);
            __syncwarp();
            if (lane == 0) {
                int total_accepted = 0;
                for (int w2 = 0; w2 < kCWarps; ++w2) total_accepted += redi[2 * kCWarps + w2];
                int32_t* row = a.sel + r * K;
                int n = 0, take = 0;
                if (n_acc < R) {
                    const int need = R - n_acc;
                    take = need < n_rej ? need : n_rej;
                }
                row[n++] = static_cast<int32_t>(center_lin);
                for (int t = 0; t < n_acc + take && n < K; ++t) {
                    const uint64_t ck = t < n_acc ? fin[t] : fin[K + (t - n_acc)];
                    const int32_t l = static_cast<int32_t>(ck & 0xffffffffu);
                    if (l < 0 || l == center_lin) continue;
                    row[n++] = l;
                }
                if (a.pow2 && n > 0) {
                    int target = 1;
                    while ((target << 1) <= n) target <<= 1;
                    if (a.min_m > target) target = a.min_m;
                    if (target < n) n = target;
                }
                for (int t = n; t < K; ++t) row[t] = -1;
                a.count[r] = n;
                a.accepted[r] = total_accepted;
            }
        }
    }
}

size_t counts_smem_bytes(const MatchArgs& a) {
    int64_t boxmax = 1;
    for (int d = 0; d < a.ndim; ++d)
        boxmax *= std::min<int64_t>(2 * a.radius[d] + 1, a.counts[d]) + a.block[d] - 1;
    return CountSmem(a.P, boxmax, a.max_m + a.required).total;
}

int32_t launch_counts(MatchArgs& a, cudaStream_t stream) {
    count_table_kernel<<<(kCodes * kCodes + 255) / 256, 256, 0, stream>>>();
    BMND_LAUNCH_CHECK("count_table_kernel");
    const size_t smem = counts_smem_bytes(a);
    const int32_t rows = a.max_m + a.required;
    auto run = [&](auto kernel) -> int32_t {
        int per_sm = 0, sms = 0;
        if (int32_t rc = kernel_residency(reinterpret_cast<const void*>(kernel), kCThreads, smem, false, &per_sm,
                                          &sms))
            return rc;
        if (per_sm < 1) per_sm = 1;
        int64_t blocks = static_cast<int64_t>(sms) * per_sm;
        if (blocks > a.n_refs) blocks = a.n_refs;
        kernel<<<static_cast<unsigned>(blocks), kCThreads, smem, stream>>>(a, rows);
        BMND_LAUNCH_CHECK("blockmatch_counts_kernel");
        return BMND_OK;
    };
    const int* bl = a.block;
    if (a.ndim == 2 && bl[0] == 8 && bl[1] == 8) return run(blockmatch_counts_kernel<2, 8, 8, 1>);
    if (a.ndim == 3 && bl[0] == 4 && bl[1] == 4 && bl[2] == 4) return run(blockmatch_counts_kernel<3, 4, 4, 4>);
    if (a.ndim == 3 && bl[0] == 5 && bl[1] == 5 && bl[2] == 5) return run(blockmatch_counts_kernel<3, 5, 5, 5>);
    return run(blockmatch_counts_kernel<0, 1, 1, 1>);
}

size_t screened_smem_bytes(int K, int P, int64_t wmax) {
    (void)K;
    return ScreenSmem::bytes(P, wmax);
}

size_t match_smem_bytes(int K, int R, int P, bool table) {
    size_t rows = static_cast<size_t>(K + R);
    return static_cast<size_t>(kWarps) * (rows * 32 + rows) * sizeof(uint64_t) +
           static_cast<size_t>(P) * sizeof(int32_t) + static_cast<size_t>(kWarps) * P * sizeof(float) +
           static_cast<size_t>(kWarps) * P * sizeof(int) + (table ? kTable * kTable * sizeof(float) : 0);
}

// patch shapes with a box-sum kernel for the approximate screening form
bool approx_box_shape(int ndim, const int32_t* b) {
    return (ndim == 2 && b[0] == 8 && b[1] == 8) || (ndim == 3 && b[0] == 5 && b[1] == 5 && b[2] == 5) ||
           (ndim == 3 && b[0] == 4 && b[1] == 4 && b[2] == 4);
}

// raise a kernel's dynamic shared-memory limit (cached, see kernel_residency)
template <typename K>
int32_t set_smem_limit(K kernel, size_t smem) {
    int per_sm = 0, sms = 0;
    return kernel_residency(reinterpret_cast<const void*>(kernel), kWarps * 32, smem, false, &per_sm, &sms);
}

int32_t launch_exact(MatchArgs& a, int code, cudaStream_t stream);

// whether a volume's SSD matching can run on the tensor cores
bool ssd_tc_applies(const MatchArgs& a) {
    return !a.table && !a.fixup && !a.poisson_bias && !a.null_moments && a.max_m <= 32 &&
           ssd_screen_shape(a.ndim, a.block) && a.grid_stride[a.ndim - 1] == 1 && a.P <= 128;
}

// SSD matching with tensor-core screening (ssdtc.cu) and exact rescoring
// (ssd_select_kernel); the references it cannot settle go to the exact kernel
int32_t launch_ssd_tc(MatchArgs& a, cudaStream_t stream) {
    const SsdScratchLayout L = ssd_scratch_layout(a.ndim, a.counts, a.block, a.radius, a.n_refs);
    char* base = nullptr;
    bool owned = false;
    if (a.ssd_ws && a.ssd_ws_bytes >= L.bytes) {
        base = a.ssd_ws;
    } else if (!a.no_alloc) {
        if (cudaMallocAsync(reinterpret_cast<void**>(&base), L.bytes, stream) == cudaSuccess) {
            owned = true;
            note_device_alloc();
        } else {
            (void)cudaGetLastError();
            base = nullptr;
        }
    }
    if (!base) return launch_exact(a, BMND_DIST_SSD, stream);
    auto release = [&]() {
        if (owned) (void)cudaFreeAsync(base, stream);
    };
    SsdScreenArgs sa{};
    sa.src = a.src;
    sa.ndim = a.ndim;
    int64_t nvox = 1;
    for (int d = 0; d < 3; ++d) {
        sa.counts[d] = d < a.ndim ? a.counts[d] : 1;
        sa.radius[d] = d < a.ndim ? a.radius[d] : 0;
        sa.block[d] = d < a.ndim ? a.block[d] : 1;
        sa.vstride[d] = d < a.ndim ? a.grid_stride[d] : 0;
        if (d < a.ndim) nvox *= a.counts[d] + a.block[d] - 1;
    }
    sa.refs = a.refs;
    int32_t rc = launch_ssd_screen(sa, nvox, a.n_refs, base, L, stream);
    if (rc) {
        release();
        return rc;
    }
    const int list_rows = a.max_m + a.required;
    const size_t smem = static_cast<size_t>(kWarps) * (list_rows * 32 + list_rows) * 8 +
                        static_cast<size_t>(a.P) * 4 + static_cast<size_t>(kWarps) * a.P * 4;
    if ((rc = set_smem_limit(ssd_select_kernel, smem))) {
        release();
        return rc;
    }
    int64_t blocks = (a.n_refs + kWarps - 1) / kWarps;
    if (blocks > 152 * 16) blocks = 152 * 16;
    ssd_select_kernel<<<static_cast<unsigned>(blocks), kWarps * 32, smem, stream>>>(
        a, reinterpret_cast<const float*>(base + L.o_rows), reinterpret_cast<const float*>(base + L.o_norms),
        reinterpret_cast<const float*>(base + L.o_psum), reinterpret_cast<const float*>(base + L.o_rmu), L.wmax,
        reinterpret_cast<const int*>(base + L.o_err));
    note_launch();
    if (const cudaError_t e = cudaGetLastError(); e != cudaSuccess) {
        release();
        return cuda_fail(e, "ssd_select_kernel");
    }
    release();
    // references that may need rejected candidates: the exact kernel
    MatchArgs fix = a;
    fix.fixup = 1;
    fix.use_table = 0;
    fix.approx = 0;
    return launch_exact(fix, BMND_DIST_SSD, stream);
}

int32_t launch(MatchArgs& a, int code, int precision, cudaStream_t stream) {
    if (a.n_refs == 0) return BMND_OK;
    if (code == BMND_DIST_SSD && precision == BMND_MATCH_FAST && ssd_tc_applies(a)) return launch_ssd_tc(a, stream);
    int64_t wmax = 1;
    for (int d = 0; d < a.ndim; ++d) wmax *= std::min<int64_t>(2 * a.radius[d] + 1, a.counts[d]);
    a.approx = precision == BMND_MATCH_APPROX || precision == BMND_MATCH_SUBSAMPLED;
    a.sub = precision == BMND_MATCH_SUBSAMPLED;
    // subsampled prescreen: candidates kept for the full form, 3K in 3-D (the
    // sub-lattice holds 27 of 125 voxels; 256^3: 26.2 ms against 28.0 ms with
    // 4K, +0.072 against +0.080 dB over the plain path), 4K in 2-D (16 of 64
    // voxels, a noisier estimate)
    a.presel = std::min((a.ndim == 3 ? 3 : 4) * a.max_m, kSQueue);
    if (a.null_moments) {
        // candidate standardisation: exact warp kernel, per-term evaluation
        a.use_table = 0;
        return launch_exact(a, code, stream);
    }
    const bool screened = code == BMND_DIST_POISSON_DEVIANCE && a.stab &&
                          (precision == BMND_MATCH_FAST || precision == BMND_MATCH_APPROX ||
                           precision == BMND_MATCH_SUBSAMPLED ||
                           precision == BMND_MATCH_REAL_VALUED) &&
                          a.max_m <= 32 && screened_smem_bytes(a.max_m, a.P, wmax) <= 200 * 1024;
    if (!screened) {
        const bool counts = code == BMND_DIST_POISSON_DEVIANCE && a.use_table && !a.table && !a.fixup &&
                            a.P <= 128 && a.max_m + a.required <= 48 && counts_smem_bytes(a) <= 96 * 1024;
        return counts ? launch_counts(a, stream) : launch_exact(a, code, stream);
    }
    size_t smem = screened_smem_bytes(a.max_m, a.P, wmax);
    // approximate mode on a volume: per-voxel c and per-origin box sums of
    // c + c log2 c, in the caller's workspace when given, else in stream-ordered
    // scratch freed after the launch; without either the bounded form runs with
    // a zero bound
    float* aux = nullptr;
    bool aux_owned = false;
    const int* bl = a.block;
    if (a.approx && !a.table && approx_box_shape(a.ndim, bl) && a.inv_scale == 1.0f &&
        a.grid_stride[a.ndim - 1] == 1) {
        int n[3] = {1, 1, 1};
        int64_t nvox = 1;
        for (int d = 0; d < a.ndim; ++d) {
            n[3 - a.ndim + d] = a.counts[d] + a.block[d] - 1;
            nvox *= n[3 - a.ndim + d];
        }
        const int64_t need = nvox * (a.sub ? 4 : 3);
        if (a.aux_ws && a.aux_ws_floats >= need) {
            aux = a.aux_ws;
        } else if (!a.no_alloc) {
            if (cudaMallocAsync(reinterpret_cast<void**>(&aux), static_cast<size_t>(need) * sizeof(float), stream) ==
                cudaSuccess) {
                aux_owned = true;
                note_device_alloc();
            } else {
                (void)cudaGetLastError();
                aux = nullptr;
            }
        }
        if (aux) {
            float* cv = aux;
            float* bv = aux + nvox;
            float* boxb = aux + 2 * nvox;
            float* boxb_sub = a.sub ? aux + 3 * nvox : nullptr;
            int64_t nb = (nvox + 255) / 256;
            if (nb > 152 * 16) nb = 152 * 16;
            // launch checks that release the scratch before reporting a failure
            auto checked = [&](const char* what) -> int32_t {
                note_launch();
                const cudaError_t e = cudaGetLastError();
                if (e == cudaSuccess) return BMND_OK;
                if (aux_owned) (void)cudaFreeAsync(aux, stream);
                return cuda_fail(e, what);
            };
            approx_voxel_kernel<<<static_cast<unsigned>(nb), 256, 0, stream>>>(a.src, a.inv_scale, nvox, cv, bv);
            if (int32_t rc0 = checked("approx_voxel_kernel")) return rc0;
            auto boxes = [&](auto full, auto half) {
                full<<<static_cast<unsigned>(nb), 256, 0, stream>>>(bv, n[0], n[1], n[2], boxb);
                if (boxb_sub) {
                    half<<<static_cast<unsigned>(nb), 256, 0, stream>>>(bv, n[0], n[1], n[2], boxb_sub);
                    note_launch();  // the check below counts the full-box launch
                }
            };
            if (a.ndim == 2)
                boxes(approx_box_kernel<2, 8, 8, 1, 1>, approx_box_kernel<2, 8, 8, 1, 2>);
            else if (bl[0] == 5)
                boxes(approx_box_kernel<3, 5, 5, 5, 1>, approx_box_kernel<3, 5, 5, 5, 2>);
            else
                boxes(approx_box_kernel<3, 4, 4, 4, 1>, approx_box_kernel<3, 4, 4, 4, 2>);
            if (int32_t rc0 = checked("approx_box_kernel")) return rc0;
            a.cv = cv;
            a.boxb = boxb;
            a.boxb_sub = boxb_sub;
        }
    }
    auto run = [&](auto kernel) -> int32_t {
        // persistent CTAs, exactly one resident wave (a partial second wave
        // leaves most SMs idle at the end)
        int sms = 0, per_sm = 0;
        if (int32_t rc = kernel_residency(reinterpret_cast<const void*>(kernel), kSThreads, smem, false, &per_sm,
                                          &sms))
            return rc;
        int64_t blocks = static_cast<int64_t>(sms) * (per_sm > 0 ? per_sm : 1);
        if (blocks > a.n_refs) blocks = a.n_refs;
        kernel<<<static_cast<unsigned>(blocks), kSThreads, smem, stream>>>(a, static_cast<int32_t>(wmax));
        BMND_LAUNCH_CHECK("blockmatch_screened_kernel");
        return BMND_OK;
    };
    int32_t rc;
    if (!a.table && a.ndim == 2 && bl[0] == 8 && bl[1] == 8)
        rc = run(blockmatch_screened_kernel<2, 8, 8, 1>);
    else if (!a.table && a.ndim == 3 && bl[0] == 5 && bl[1] == 5 && bl[2] == 5)
        rc = run(blockmatch_screened_kernel<3, 5, 5, 5>);
    else if (!a.table && a.ndim == 3 && bl[0] == 4 && bl[1] == 4 && bl[2] == 4)
        rc = run(blockmatch_screened_kernel<3, 4, 4, 4>);
    else
        rc = run(blockmatch_screened_kernel<0, 1, 1, 1>);
    if (aux_owned) BMND_CUDA_TRY(cudaFreeAsync(aux, stream));
    a.cv = nullptr;
    a.boxb = nullptr;
    a.boxb_sub = nullptr;
    if (rc) return rc;
    // references that need the best rejected candidates are redone exactly
    MatchArgs fix = a;
    fix.fixup = 1;
    fix.use_table = 0;
    fix.approx = 0;
    return launch_exact(fix, code, stream);
}

int32_t launch_exact(MatchArgs& a, int code, cudaStream_t stream) {
    if (a.n_refs == 0) return BMND_OK;
    size_t smem = match_smem_bytes(a.max_m, a.required, a.P, a.use_table != 0);
    int64_t blocks = (a.n_refs + kWarps - 1) / kWarps;
    // persistent CTAs: each walks references with a grid stride, so per-CTA
    // set-up (offset table, deviance table) is paid once per CTA
    const int64_t cap = 152 * 16;
    if (blocks > cap) blocks = cap;
    dim3 grid(static_cast<unsigned>(blocks));
    switch (code) {
        case BMND_DIST_SSD:
            if (int32_t rc = set_smem_limit(blockmatch_kernel<BMND_DIST_SSD>, smem)) return rc;
            blockmatch_kernel<BMND_DIST_SSD><<<grid, kWarps * 32, smem, stream>>>(a);
            break;
        case BMND_DIST_POISSON_DEVIANCE:
            if (int32_t rc = set_smem_limit(blockmatch_kernel<BMND_DIST_POISSON_DEVIANCE>, smem)) return rc;
            blockmatch_kernel<BMND_DIST_POISSON_DEVIANCE><<<grid, kWarps * 32, smem, stream>>>(a);
            break;
        case BMND_DIST_PEARSON:
            if (int32_t rc = set_smem_limit(blockmatch_kernel<BMND_DIST_PEARSON>, smem)) return rc;
            blockmatch_kernel<BMND_DIST_PEARSON><<<grid, kWarps * 32, smem, stream>>>(a);
            break;
        case BMND_DIST_ANSCOMBE_SSD:
            if (int32_t rc = set_smem_limit(blockmatch_kernel<BMND_DIST_ANSCOMBE_SSD>, smem)) return rc;
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
    // the tabulated path is exact for any data but pays off only for integer counts
    a.use_table = (mp.distance == BMND_DIST_POISSON_DEVIANCE && scale == 1.0 &&
                   mp.precision != BMND_MATCH_REAL_VALUED) ? 1 : 0;
}

}  // namespace

int32_t launch_blockmatch_volume(const BmndMatchParams& mp, const float* volume,
                                 const int32_t* shape, const int32_t* block, const int32_t* refs,
                                 int64_t n_refs, const float* thresholds, float scalar_threshold,
                                 int32_t* sel, int32_t* count, int32_t* accepted,
                                 cudaStream_t stream, const float* thr_dev, const float* noise_ssd,
                                 float gamma, bool allow_alloc, const double* null_moments, int null_max,
                                 bool poisson_bias, float* aux_ws, int64_t aux_ws_floats, char* ssd_ws,
                                 uint64_t ssd_ws_bytes) {
    int32_t rc = validate_match(mp);
    if (rc) return rc;
    if ((noise_ssd || poisson_bias) && mp.distance != BMND_DIST_SSD)
        return fail(BMND_ERR_INVALID_ARG, "the noise-bias correction applies to SSD matching only");
    if (noise_ssd && poisson_bias)
        return fail(BMND_ERR_INVALID_ARG, "one noise-bias correction at a time");
    if (poisson_bias && (!(mp.count_scale > 0.0) || !std::isfinite(mp.count_scale)))
        return fail(BMND_ERR_INVALID_ARG, "poisson_count_scale must be finite and positive");
    if ((noise_ssd || poisson_bias) && (!(gamma >= 0.0f) || !std::isfinite(gamma)))
        return fail(BMND_ERR_INVALID_ARG, "gamma must be finite and non-negative");
    MatchArgs a{};
    fill_common(a, mp);
    a.thr_dev = thr_dev;
    a.noise_ssd = noise_ssd;
    a.gamma = gamma;
    a.poisson_bias = poisson_bias ? 1 : 0;
    a.bias_scale = static_cast<float>(mp.count_scale);  // the Python float meets float32 data
    a.no_alloc = allow_alloc ? 0 : 1;
    a.aux_ws = aux_ws;
    a.aux_ws_floats = aux_ws_floats;
    a.ssd_ws = ssd_ws;
    a.ssd_ws_bytes = ssd_ws_bytes;
    a.null_moments = null_moments;
    a.null_max = null_max;
    if (null_moments && mp.distance == BMND_DIST_SSD)
        return fail(BMND_ERR_INVALID_ARG, "candidate standardisation needs a Poisson distance");
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
    return launch(a, mp.distance, mp.precision, stream);
}

uint64_t ssd_tc_scratch_bytes(const BmndMatchParams& mp, const int32_t* block, int64_t n_refs, bool poisson_bias) {
    if (mp.distance != BMND_DIST_SSD || mp.precision != BMND_MATCH_FAST || poisson_bias || mp.max_matches > 32 ||
        !ssd_screen_shape(mp.ndim, block))
        return 0;
    return ssd_scratch_layout(mp.ndim, mp.counts, block, mp.search_radius, n_refs).bytes;
}

int64_t approx_scratch_floats(const BmndMatchParams& mp, const int32_t* shape, const int32_t* block) {
    const bool approx = mp.precision == BMND_MATCH_APPROX || mp.precision == BMND_MATCH_SUBSAMPLED;
    if (!approx || mp.distance != BMND_DIST_POISSON_DEVIANCE || mp.count_scale != 1.0 ||
        !approx_box_shape(mp.ndim, block))
        return 0;
    int64_t nvox = 1;
    for (int d = 0; d < mp.ndim; ++d) nvox *= shape[d];
    return nvox * (mp.precision == BMND_MATCH_SUBSAMPLED ? 4 : 3);
}

namespace {
// order-preserving min / max of a volume, then the SSD threshold
// float32(t * d * d), d = max - min (1 when d <= 0) (blockmatching.py:168-184)
__global__ void minmax_kernel(const float* __restrict__ x, int64_t n, uint32_t* __restrict__ mm) {
    uint32_t lo = 0xffffffffu, hi = 0u;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const uint32_t b = order_bits(__ldg(x + i));
        lo = min(lo, b);
        hi = max(hi, b);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMin(mm, lo);
        atomicMax(mm + 1, hi);
    }
}

__device__ __forceinline__ float from_order_bits(uint32_t u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

__global__ void ssd_threshold_kernel(const uint32_t* __restrict__ mm, double t, float* __restrict__ thr) {
    float d = from_order_bits(mm[1]) - from_order_bits(mm[0]);
    double ds = d > 0.0f ? static_cast<double>(d) : 1.0;
    *thr = static_cast<float>(t * ds * ds);
}
}  // namespace

namespace {
// reference-finite-count thresholds (blockmatching.py:86-148): per reference,
// mean of the null means + t sqrt(sum of null variances) / P + beta mean^power
// over the reference patch's pooled-count estimates rint(2 r), float64
__global__ void reference_thresholds_kernel(const float* __restrict__ vol, const int32_t* __restrict__ refs,
                                            int64_t n, int ndim, int3 counts, int3 block, int3 vstride,
                                            double count_scale, const double* __restrict__ moments, int max_count,
                                            double t, double beta, double power, float* __restrict__ out) {
    for (int64_t r = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; r < n;
         r += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int c[3] = {refs[r * ndim], ndim > 1 ? refs[r * ndim + 1] : 0, ndim > 2 ? refs[r * ndim + 2] : 0};
        const int b[3] = {block.x, block.y, block.z};
        const int s[3] = {vstride.x, vstride.y, vstride.z};
        int64_t origin = 0;
        int P = 1;
        for (int d = 0; d < ndim; ++d) {
            origin += static_cast<int64_t>(c[d]) * s[d];
            P *= b[d];
        }
        double msum = 0.0, vsum = 0.0, isum = 0.0;
        for (int p = 0; p < P; ++p) {
            int rem = p;
            int64_t off = 0;
            for (int d = ndim - 1; d >= 0; --d) {
                off += static_cast<int64_t>(rem % b[d]) * s[d];
                rem /= b[d];
            }
            double rc = static_cast<double>(vol[origin + off]) / count_scale;
            if (rc < 0.0) rc = 0.0;
            const double pooled = rint(2.0 * rc);
            double m = 1.0, v = 2.0;
            if (pooled <= static_cast<double>(max_count)) {
                const int k = static_cast<int>(pooled);
                m = moments[k];
                v = moments[max_count + 1 + k];
            }
            msum += m;
            vsum += v;
            isum += rc;
        }
        const double pm = msum / P, pv = vsum / (static_cast<double>(P) * P), inten = isum / P;
        out[r] = static_cast<float>(pm + t * sqrt(pv > 0.0 ? pv : 0.0) + beta * pow(inten, power));
    }
}
}  // namespace

int32_t launch_reference_thresholds(const float* volume, const int32_t* refs, int64_t n_refs, int ndim,
                                    const int32_t* counts, const int32_t* block, const int32_t* shape,
                                    double count_scale, const double* moments, int max_count, double t,
                                    double beta, double power, float* out, cudaStream_t stream) {
    if (n_refs == 0) return BMND_OK;
    int st[3] = {1, 1, 1}, bl[3] = {1, 1, 1}, cn[3] = {1, 1, 1};
    int64_t sv = 1;
    for (int d = ndim - 1; d >= 0; --d) {
        st[d] = static_cast<int>(sv);
        sv *= shape[d];
    }
    for (int d = 0; d < ndim; ++d) {
        bl[d] = block[d];
        cn[d] = counts[d];
    }
    int64_t blocks = (n_refs + 127) / 128;
    if (blocks > 152 * 16) blocks = 152 * 16;
    reference_thresholds_kernel<<<static_cast<unsigned>(blocks), 128, 0, stream>>>(
        volume, refs, n_refs, ndim, make_int3(cn[0], cn[1], cn[2]), make_int3(bl[0], bl[1], bl[2]),
        make_int3(st[0], st[1], st[2]), count_scale, moments, max_count, t, beta, power, out);
    BMND_LAUNCH_CHECK("reference_thresholds_kernel");
    return BMND_OK;
}

int32_t launch_ssd_threshold(const float* volume, int64_t n, double t, uint32_t* mm, float* thr,
                             cudaStream_t stream) {
    BMND_CUDA_TRY(cudaMemsetAsync(mm, 0xff, sizeof(uint32_t), stream));
    BMND_CUDA_TRY(cudaMemsetAsync(mm + 1, 0, sizeof(uint32_t), stream));
    int64_t blocks = (n + 255) / 256;
    if (blocks > 152 * 8) blocks = 152 * 8;
    if (blocks < 1) blocks = 1;
    minmax_kernel<<<static_cast<unsigned>(blocks), 256, 0, stream>>>(volume, n, mm);
    BMND_LAUNCH_CHECK("minmax_kernel");
    ssd_threshold_kernel<<<1, 1, 0, stream>>>(mm, t, thr);
    BMND_LAUNCH_CHECK("ssd_threshold_kernel");
    return BMND_OK;
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
    return launch(a, mp.distance, mp.precision, stream);
}

}  // namespace bmnd
