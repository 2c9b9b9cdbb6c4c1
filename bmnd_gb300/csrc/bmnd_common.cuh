// bmnd_common.cuh -- shared device helpers of the GB300 BMND library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstring>
#include <string>

#include "../../include/bmnd_gb300.h"

namespace bmnd {

// internal value of BmndMatchParams.precision: the source is real-valued (a
// pilot estimate), so integer-count tabulation is skipped
constexpr int32_t BMND_MATCH_REAL_VALUED = 100;

// ---------------------------------------------------------------------------
// error reporting (thread-local message behind bmnd_last_error)
// ---------------------------------------------------------------------------
void set_error(const std::string& msg);
void clear_error();
int32_t fail(int32_t code, const std::string& msg);
int32_t cuda_fail(cudaError_t err, const char* what);
// counts kernel launches of this library (bmnd_launch_count)
void note_launch();
// counts the device allocations the library makes itself (fallbacks when a
// caller's workspace has no room for a scratch array)
void note_device_alloc();

#define BMND_CUDA_TRY(expr)                                      \
    do {                                                         \
        cudaError_t _e = (expr);                                 \
        if (_e != cudaSuccess) return ::bmnd::cuda_fail(_e, #expr); \
    } while (0)

// after every kernel launch: counts it and reports a launch error
#define BMND_LAUNCH_CHECK(what)                                   \
    do {                                                          \
        ::bmnd::note_launch();                                    \
        cudaError_t _e = cudaGetLastError();                      \
        if (_e != cudaSuccess) return ::bmnd::cuda_fail(_e, what); \
    } while (0)

// ---------------------------------------------------------------------------
// canonical Poisson distance keys
//
// The reference compares Poisson distances after rounding them to a quantum of
// 32 * 2^-23 * 2^floor(log2(max(|d|, 1))) with round-half-even
// (src/bmnd/blockmatching.py:957-964).  For a float32 d that quantum is a
// power of two, so d / quantum is an exact scaling, rint() is exact in float32
// (the scaled value is below 2^19) and so is the product back: the key is
// computed exactly in float32 here.
// ---------------------------------------------------------------------------
__host__ __device__ inline float canonical_key(float d) {
#ifdef __CUDA_ARCH__
    // e = floor(log2(max(|d|, 1))) from the exponent field; both scalings are
    // by exact powers of two (2^(18-e) <= 2^18, 2^(e-18) >= 2^-18, normal)
    const uint32_t mbits = __float_as_uint(d) & 0x7fffffffu;
    if (mbits >= 0x7f800000u) return d;  // NaN, +-inf
    const int e = mbits >= 0x3f800000u ? static_cast<int>(mbits >> 23) - 127 : 0;
    const float up = __uint_as_float(static_cast<uint32_t>(127 + 18 - e) << 23);
    const float down = __uint_as_float(static_cast<uint32_t>(127 - 18 + e) << 23);
    return __fmul_rn(rintf(__fmul_rn(d, up)), down);
#else
    if (!(d == d) || d == INFINITY || d == -INFINITY) return d;
    float mag = fabsf(d);
    int e = 0;
    if (mag >= 1.0f) {
        int ex;
        frexpf(mag, &ex);  // mag = f * 2^ex, f in [0.5, 1)
        e = ex - 1;
    }
    float scaled = ldexpf(d, 18 - e);
    return ldexpf(rintf(scaled), e - 18);
#endif
}

// q = floor(c / e) for 0 <= c < 2^21 and e >= 1, with inv_e = 1.0f / e:
// (c + 0.5) / e lies at least 0.5 / e away from an integer, and the float32
// evaluation errs by less than 2^-22 (c + 0.5) / e < 0.5 / e
__device__ __forceinline__ int small_div(int c, float inv_e) {
    return __float2int_rz(__fmul_rn(static_cast<float>(c) + 0.5f, inv_e));
}

// order-preserving uint32 image of a float (total order for non-NaN values)
__host__ __device__ inline uint32_t order_bits(float f) {
#ifdef __CUDA_ARCH__
    uint32_t u = __float_as_uint(f);
#else
    uint32_t u;
    memcpy(&u, &f, sizeof(u));
#endif
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

// inverse of order_bits
__device__ __forceinline__ float ordered_float(uint32_t b) {
    return __uint_as_float((b & 0x80000000u) ? (b & 0x7fffffffu) : ~b);
}

__host__ __device__ inline uint64_t composite_key(float key, int32_t lin) {
    return (static_cast<uint64_t>(order_bits(key)) << 32) | static_cast<uint32_t>(lin);
}

// ---------------------------------------------------------------------------
// group-axis transform entries
//
// Hierarchical Haar matrix of a power-of-two size n = 2^L as the reference
// builds it (src/bmnd/transforms.py:393-408): row 0 is s^L, the detail rows
// created at level l (rows [2^(l-1), 2^l)) carry +-s^(L-l+1) on a support of
// 2^(L-l+1) columns.  s^m is the float32 product s*s*...*s evaluated left to
// right, exactly as the repeated kron products produce it.  Other sizes (and
// BMND_GROUP_DCT) use the orthonormal DCT-II evaluated in float64 and rounded
// (transforms.py:424-436).
// ---------------------------------------------------------------------------
__host__ __device__ inline bool is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

__host__ __device__ inline float haar_power(int m) {
    const float s = 0.70710677f;  // float32(1 / sqrt(2))
    float p = 1.0f;
    for (int i = 0; i < m; ++i) p = p * s;
    return p;
}

__host__ __device__ inline int ilog2_floor(int v) {
    int l = 0;
    while ((1 << (l + 1)) <= v) ++l;
    return l;
}

__host__ __device__ inline float haar_entry(int n, int i, int g) {
    int L = ilog2_floor(n);
    if (i == 0) return haar_power(L);
    int l = ilog2_floor(i) + 1;
    int c = 1 << (l - 1);
    int j = i - c;
    int width = n >> (l - 1);
    int start = j * width;
    int half = width >> 1;
    float v = haar_power(L - l + 1);
    if (g >= start && g < start + half) return v;
    if (g >= start + half && g < start + width) return -v;
    return 0.0f;
}

__host__ __device__ inline float dct_entry(int n, int f, int s) {
    const double pi = 3.141592653589793;
    double norm = f == 0 ? sqrt(1.0 / n) : sqrt(2.0 / n);
    return static_cast<float>(norm * cos(pi * (s + 0.5) * f / n));
}

__host__ __device__ inline float group_entry(int kind, int n, int i, int g) {
    if (kind == BMND_GROUP_NONE) return i == g ? 1.0f : 0.0f;
    if (kind == BMND_GROUP_HAAR && is_pow2(n)) return haar_entry(n, i, g);
    return dct_entry(n, i, g);
}

// the n x n group matrices of every group size n = 1 .. BMND_MAX_STACK, one
// after another (group n starts at group_table_offset(n)), as a table the
// filter copies instead of evaluating group_entry per CTA
__host__ __device__ constexpr int group_table_offset(int n) { return (n - 1) * n * (2 * n - 1) / 6; }
constexpr int kGroupTableFloats = group_table_offset(BMND_MAX_STACK + 1);

// exact float32 operations that the compiler must not contract into FMAs
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float div_rn(float a, float b) { return __fdiv_rn(a, b); }

struct Dims {
    int32_t ndim;
    int32_t shape[BMND_MAX_DIMS];
    int32_t block[BMND_MAX_DIMS];
    int32_t counts[BMND_MAX_DIMS];
};

inline int64_t volume_voxels(const BmndStageParams& p) {
    int64_t n = 1;
    for (int d = 0; d < p.ndim; ++d) n *= p.shape[d];
    return n;
}

inline int patch_volume(const BmndStageParams& p) {
    int n = 1;
    for (int d = 0; d < p.ndim; ++d) n *= p.block[d];
    return n;
}

// Layout of the Kronecker table S^T used by the exact variance: lane l of a
// warp owns the KRON_JR(P) consecutive coefficients j = j0 + KRON_JR * l + r,
// so each table row is padded with zeros to a multiple of 32 * KRON_JR floats
// and one vector load per lane fetches all of them.
__host__ __device__ constexpr int kron_jr(int P) { return P <= 32 ? 1 : (P <= 64 ? 2 : 4); }
__host__ __device__ constexpr int kron_stride(int P) {
    return (P + 32 * kron_jr(P) - 1) / (32 * kron_jr(P)) * (32 * kron_jr(P));
}
// floats of the per-stage table region: Kronecker table, risk metric, group matrices
inline uint64_t stage_table_floats(int P) {
    return 2ull * static_cast<uint64_t>(P) * static_cast<uint64_t>(kron_stride(P)) + kGroupTableFloats;
}

// Launch shape of `fn` with `threads` threads and `smem` bytes of dynamic
// shared memory: its resident CTAs per SM and the device's SM count.  Raises the
// kernel's dynamic shared-memory limit to `smem` when needed; with
// fit_carveout the kernel's preferred shared-memory carveout is what its
// resident CTAs need, so the rest of the unified L1 caches global loads.  The
// queries are made once per device, kernel and shape, then served from a cache.
int32_t kernel_residency(const void* fn, int threads, size_t smem, bool fit_carveout, int* per_sm, int* sms);

// launch helpers implemented in the .cu files
int32_t launch_blockmatch_volume(const BmndMatchParams& mp, const float* volume, const int32_t* shape,
                                 const int32_t* block, const int32_t* refs, int64_t n_refs,
                                 const float* thresholds, float scalar_threshold, int32_t* sel,
                                 int32_t* count, int32_t* accepted, cudaStream_t stream,
                                 const float* thr_dev = nullptr, const float* noise_ssd = nullptr,
                                 float gamma = 0.0f, bool allow_alloc = true,
                                 const double* null_moments = nullptr, int null_max = 0,
                                 bool poisson_bias = false, float* aux_ws = nullptr, int64_t aux_ws_floats = 0,
                                 char* ssd_ws = nullptr, uint64_t ssd_ws_bytes = 0);
// squared norm of a patch centred on mu, from its sum of squares s2 and sum s1:
// s2 - 2 mu s1 + P mu^2 (float32, clamped at zero); the screening and the
// selection evaluate it with the same operations
__device__ __forceinline__ float centred_norm(float s2, float s1, float mu, int P) {
    const float v = __fadd_rn(__fsub_rn(s2, __fmul_rn(__fmul_rn(2.0f, mu), s1)),
                              __fmul_rn(__fmul_rn(static_cast<float>(P), mu), mu));
    return v > 0.0f ? v : 0.0f;
}
// bytes of workspace the tensor-core SSD matching of a volume needs (0: it does not apply)
uint64_t ssd_tc_scratch_bytes(const BmndMatchParams& mp, const int32_t* block, int64_t n_refs, bool poisson_bias);
// floats of workspace the approximate screening form of a volume needs (0: none)
int64_t approx_scratch_floats(const BmndMatchParams& mp, const int32_t* shape, const int32_t* block);
int32_t launch_reference_thresholds(const float* volume, const int32_t* refs, int64_t n_refs, int ndim,
                                    const int32_t* counts, const int32_t* block, const int32_t* shape,
                                    double count_scale, const double* moments, int max_count, double t,
                                    double beta, double power, float* out, cudaStream_t stream);
// mm: two uint32 of device scratch; thr: one device float
int32_t launch_ssd_threshold(const float* volume, int64_t n, double t, uint32_t* mm, float* thr,
                             cudaStream_t stream);
int32_t launch_blockmatch_patches(const BmndMatchParams& mp, const float* patches, int32_t patch_vol,
                                  const int32_t* refs, int64_t n_refs, const float* thresholds,
                                  int32_t* sel, int32_t* count, int32_t* accepted,
                                  cudaStream_t stream);
// per-group intermediate arrays of the group filter (bmnd_group_probe); any
// pointer may be null.  Row i of the coefficient-shaped outputs starts at
// i * max_stack * P, of the weights at i * max_stack.
struct GroupProbe {
    int active;
    float* coef;     // forward transform of the observation group
    float* sigma;    // noise standard deviation of every coefficient
    float* atten;    // hard-threshold mask or Wiener gain
    float* weights;  // aggregation weight of every member
    float* filt;     // inverse transform of the shrunk coefficients
};
// exclusive prefix sum of n ints into out[0..n] (out[n] = the total);
// block_sums holds (n + 1023) / 1024 + 1 ints of scratch
int32_t launch_exclusive_scan(const int32_t* in, int64_t n, int32_t* out, int32_t* block_sums,
                              cudaStream_t stream);

// SSD matching on the tensor cores (ssdtc.cu): the screening distances of
// every reference's window candidates, in window order, one row of wmax
// floats per reference
struct SsdScreenArgs {
    const float* src;     // matched volume
    const float* norms;   // per patch origin: sum of squares of its patch (written by the launch)
    const float* sums;    // per patch origin: sum of its patch (written by the launch)
    const float* mu;      // per tile: the mean the tile's patches are centred on (written by the launch)
    float* ref_mu;        // per reference: the mean of its tile (written by the launch)
    int32_t ndim;
    int32_t counts[3], radius[3], block[3];
    int64_t vstride[3];   // voxel offset of one patch-grid step per axis
    const int32_t* refs;  // n_refs x ndim reference positions
    const int32_t* perm;  // references sorted by spatial tile
    const int32_t* tile_start;
    int32_t n_tiles;
    int32_t tile_edge[3], tiles[3];
    float* out;           // n_refs x wmax screening distances
    int64_t wmax;
    int* err;             // set when a bounded wait ran out
};
struct SsdScratchLayout {
    int64_t wmax, n_tiles;
    uint64_t o_norms, o_psum, o_mu, o_rmu, o_rows, o_start, o_cursor, o_sums, o_perm, o_err;
    uint64_t bytes;
};
bool ssd_screen_shape(int ndim, const int32_t* block);
SsdScratchLayout ssd_scratch_layout(int ndim, const int32_t* counts, const int32_t* block, const int32_t* radius,
                                    int64_t n_refs);
int32_t launch_ssd_screen(SsdScreenArgs a, int64_t nvox, int64_t n_refs, char* base, const SsdScratchLayout& L,
                          cudaStream_t stream);

// deterministic aggregation (aggregate.cu): byte offsets of its arrays in a
// 256-byte aligned region, for a stage with n_refs groups
struct AggregationLayout {
    int64_t n_lins;  // patch origins
    uint64_t o_start, o_cursor, o_block_sums, o_entries, o_slot, o_store, o_wstore, o_planes, o_wsum;
    uint64_t bytes;
};
AggregationLayout aggregation_layout(const BmndStageParams& sp, int64_t n_refs);
int64_t agg_row_floats(const BmndStageParams& sp);
// the group filter's output in deterministic mode: member g of group i writes
// its weighted filtered patch to store[slot_of[i * max_stack + g] * row + p]
// and its weight to wstore[slot]
struct AggStore {
    float* store;
    float* wstore;
    const int32_t* slot_of;
    int row;
};
int32_t launch_entry_index(const BmndStageParams& sp, const int32_t* sel, const int32_t* count, int64_t n_refs,
                           char* base, const AggregationLayout& L, cudaStream_t stream);
int32_t launch_gather(const BmndStageParams& sp, const float* noisy, float* out, char* base,
                      const AggregationLayout& L, cudaStream_t stream);
int32_t launch_group_filter(const BmndStageParams& sp, const float* noisy, const float* pilot,
                            const int32_t* sel, const int32_t* count, int64_t n_refs, double* num,
                            double* den, float* st, double* sig_num, cudaStream_t stream,
                            const double* den_ro = nullptr, int* err = nullptr,
                            const GroupProbe* probe = nullptr, const AggStore* store = nullptr);
int32_t launch_finalize_sigma(const BmndStageParams& sp, const double* sig_num, const double* den,
                              float global_sigma, float* out, cudaStream_t stream);
int32_t launch_finalize(const BmndStageParams& sp, const double* num, const double* den,
                        const float* noisy, float* out, cudaStream_t stream);

}  // namespace bmnd
