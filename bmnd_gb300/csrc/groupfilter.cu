// groupfilter.cu -- fused collaborative filtering of matched groups.
//
// One CTA filters one group end to end, with everything staged in shared
// memory:
//   1. gather the N patches of the observation (and of the pilot for Wiener)
//      and of the Poisson variance volume V = max(scale * max(x, 0), floor)
//      (src/bmnd/variance.py:556-598);
//   2. forward separable transform, group axis first then the patch axes
//      (transforms.py:209-255); every axis product accumulates with one fused
//      multiply-add per term in k order, which is how NumPy's sgemm evaluates
//      the reference's matrix products;
//   3. noise standard deviation of every coefficient: the approximate
//      propagation through squared transforms (variance.py:613-623,
//      :1647-1653) and, for the first k group planes, the exact
//      overlap-aware variance sum_v V_v (sum_{e in v} E_e)^2 over the union of
//      overlapping patch voxels (variance.py:758-851, :920-975), then the
//      plane limiting rule (variance.py:1572-1631);
//   4. hard thresholding with the tolerance-aware Poisson mask
//      (bmndalgo.py:460-485, poisson.py:30-46) or the variance-scaled Poisson
//      Wiener gain (wiener.py:24-95, bmndalgo.py:878-894);
//   5. per-patch aggregation weights 1 / (sum_g Ginv[o,g]^2 plane_risk[g] +
//      eps) (aggregationweights.py:213-259, :616-653), or one weight per group
//      from its exact windowed-synthesis risk (wiener.py:638-822);
//   6. inverse transform and weighted Kaiser-window scatter into float64
//      numerator / denominator volumes (patchaggregation.py:170-199).
//
// The union of overlapping voxels is found with a per-group occupancy grid
// holding one bit per group member (N <= 32), so each voxel's entries come out
// in ascending group order and the float32 sums are deterministic.
#include <cuda_runtime.h>
#include <stdint.h>

#include "bmnd_common.cuh"

namespace bmnd {
namespace {

constexpr int kThreads = 256;      // threads per group (CTA)

// Shared-memory plan.  A fixed part holds the group matrix, the transform
// tables, positions and small per-group arrays.  The union region first holds
// the exact-variance phase's occupancy grid and union-voxel lists; once that
// phase is done it holds the group buffers: S (noise sigma), X (noisy
// coefficients) and R (pilot coefficients, Wiener) or V (attenuation, hard
// thresholding).  Transforms run in place, so no scratch buffer is needed.
// With exact risk weights the union-voxel lists are still needed after the
// shrinkage, so they get a region of their own after the group buffers.
struct Layout {
    // byte offsets into dynamic shared memory
    int64_t g, gt, fw, fi, fit, dir, win, mdiag, pos, shf, shl, sg, ex, part, lag, uni, s, x, r, v, grid, lval,
        lstart, lent, scan, plane, wts, misc, risk, total;
};

struct FilterArgs {
    BmndStageParams sp;
    Layout L;
    int32_t P;
    int32_t nmax;
    int32_t kmax;
    int32_t counts[BMND_MAX_DIMS];
    int64_t vstride[BMND_MAX_DIMS];
    const float* noisy;
    const float* pilot;
    const int32_t* sel;
    const int32_t* count;
    int64_t n_refs;
    double* num;
    double* den;
    const float* st;  // S^T: st[p * kron_stride(P) + j] = S[j, p], the Kronecker product of the patch transforms
    double* sig_num;  // optional: sigma-map numerator (sum of sigma x weight x window), else null
    // group-mass conservation, second pass: the first pass's denominator
    // (read only); the kernel then re-aggregates the numerator alone
    const double* den_ro;
    int* err;  // 1: a group's mass correction is undefined; 2: a group was skipped (bad members)
    // group probe: per-group intermediate arrays instead of the aggregation
    GroupProbe probe;
    int64_t n_lins;      // patch-grid positions: a member's lin lies in [0, n_lins)
    int64_t ucells_cap;  // union-box cells the occupancy grid of the layout holds
    AggStore store;      // deterministic aggregation: rows of the entry store, or store.store == null
};

__host__ Layout make_layout(const BmndStageParams& sp, int P, int nmax, int kmax, int64_t ucells, bool sigma) {
    Layout L{};
    int64_t off = 0;
    auto round16 = [](int64_t b) { return (b + 15) & ~int64_t(15); };
    auto take = [&](int64_t bytes) {
        int64_t o = off;
        off += round16(bytes);
        return o;
    };
    const int64_t np = static_cast<int64_t>(nmax) * P;
    const bool wiener = sp.filter == BMND_FILTER_WIENER;
    const int kpad = (kmax + 3) / 4 * 4;
    L.g = take(4 * nmax * nmax);
    L.gt = take(4 * nmax * (kpad > 0 ? kpad : 4));
    L.fw = take(4 * BMND_MAX_DIMS * BMND_MAX_EDGE * BMND_MAX_EDGE);
    L.fi = take(4 * BMND_MAX_DIMS * BMND_MAX_EDGE * BMND_MAX_EDGE);
    // group-mass conservation: transposed inverse spatial matrices, and the
    // per-axis factors of the constant synthesis direction (group axis, patch axes)
    const bool mass = sp.mass_conserve != 0;
    L.fit = take(mass ? 4 * BMND_MAX_DIMS * BMND_MAX_EDGE * BMND_MAX_EDGE : 16);
    L.dir = take(mass ? 4 * (BMND_MAX_STACK + BMND_MAX_DIMS * BMND_MAX_EDGE) : 16);
    L.win = take(4 * P);
    L.mdiag = take(8 * P);
    L.pos = take(4 * nmax * BMND_MAX_DIMS);
    L.shf = take(4 * nmax * BMND_MAX_DIMS);
    L.shl = take(4 * nmax);
    // hard thresholding with a sigma map keeps each coefficient's sigma until the scatter
    L.sg = take(sigma && !wiener ? 4 * np : 16);
    L.ex = take(4 * static_cast<int64_t>(kmax) * P);

    // Gaussian noise: lag index of every member pair (i >= j)
    const bool gauss = sp.noise_model == BMND_NOISE_GAUSSIAN;
    L.lag = take(gauss && kmax > 0 ? 4 * static_cast<int64_t>(nmax) * (nmax + 1) / 2 : 16);
    L.scan = take(8 * (kThreads + 1));
    L.plane = take(8 * (nmax > 40 ? nmax : 40));  // also the mass phase's 8 warps x 5 sums
    L.wts = take(4 * nmax);
    L.misc = take(64);
    L.risk = take(8 * (kThreads / 32 + 1));  // exact risk: per-warp partial sums, then the total
    // union region
    L.uni = off;
    const int64_t buf = round16(4 * np);
    L.s = L.uni;
    L.x = L.s + buf;
    L.r = L.x + buf;  // Wiener: pilot coefficients, then the attenuation
    L.v = L.r;        // hard thresholding: the attenuation
    const int64_t group_bytes = 3 * buf;
    // union-voxel lists of the exact phase (Poisson noise, or white Gaussian
    // noise with exact risk weights), kept apart from the group buffers when
    // the exact risk reads them after the shrinkage
    const bool keep = sp.exact_risk_weights != 0;
    const int kl = (gauss && !keep) ? 0 : kmax;
    const int64_t umax = kl > 0 ? (np < ucells ? np : ucells) : 0;
    L.grid = keep ? L.uni + group_bytes : L.uni;
    L.lval = L.grid + round16(kl > 0 ? 4 * ucells : 0);
    L.lstart = L.lval + round16(4 * umax);
    L.lent = L.lstart + round16(4 * (umax + 1));
    const int64_t list_end = L.lent + round16(kl > 0 ? 4 * np : 0);
    off = keep ? list_end : L.uni + (group_bytes > list_end - L.uni ? group_bytes : list_end - L.uni);
    // exact variance: per-warp partial sums of one tile of 4 planes x 32 JR
    // coefficients (64 for the half-warp form), added in warp order afterwards;
    // they take the occupancy grid's place (free once the lists are built) when
    // it is large enough
    const int tile_w = kron_jr(P) == 2 ? 64 : 32 * kron_jr(P);
    const int64_t part_bytes = 4 * (kThreads / 32) * 4 * static_cast<int64_t>(tile_w);
    if (gauss || kmax <= 0) L.part = L.grid;
    else if (4 * ucells >= part_bytes) L.part = L.grid;
    else L.part = take(part_bytes);
    L.total = off;
    return L;
}

template <typename T>
__device__ __forceinline__ T* sm(unsigned char* base, int64_t off) {
    return reinterpret_cast<T*>(base + off);
}

// Patch geometry: compile-time for the default shapes (ND > 0), runtime otherwise.
template <int ND, int B0, int B1, int B2>
struct Geom {
    int nd_, b_[BMND_MAX_DIMS], P_;
    __device__ explicit Geom(const BmndStageParams& sp) {
        nd_ = sp.ndim;
        P_ = 1;
        for (int d = 0; d < BMND_MAX_DIMS; ++d) {
            b_[d] = d < sp.ndim ? sp.block[d] : 1;
            P_ *= b_[d];
        }
    }
    __device__ __forceinline__ int nd() const { return ND > 0 ? ND : nd_; }
    __device__ __forceinline__ int b(int d) const {
        if (ND > 0) return d == 0 ? B0 : (d == 1 ? B1 : B2);
        return b_[d];
    }
    __device__ __forceinline__ int P() const { return ND > 0 ? B0 * B1 * B2 : P_; }
    // product of the patch extents after axis d
    __device__ __forceinline__ int inner(int d) const {
        int v = 1;
#pragma unroll
        for (int e = 0; e < BMND_MAX_DIMS; ++e)
            if (e > d && e < nd()) v *= b(e);
        return v;
    }
    // voxel offset of element p of the patch whose origin is `org`
    __device__ __forceinline__ int64_t offset(const int* org, int p, const int64_t* vstride) const {
        int64_t off = 0;
#pragma unroll
        for (int d = BMND_MAX_DIMS - 1; d >= 0; --d) {
            if (d < nd()) {
                off += static_cast<int64_t>(org[d] + p % b(d)) * vstride[d];
                p /= b(d);
            }
        }
        return off;
    }
};

// Transforms work in place on an (n, block...) group held in shared memory.
// Every axis product accumulates with one fused multiply-add per term in k
// order, which is how NumPy's sgemm evaluates the reference's products.
//
// Group axis, compile-time size N: out[i, p] = sum_k M[i, k] in[k, p] with
// KIND 0: M = G, KIND 1: M = G^T (the inverse, transforms.py:423, :436),
// KIND 2: M = G o G with each entry rounded as fl(g * g) (the squared
// transform of the variance propagation).  Each thread holds one column in
// registers and produces IC of its N outputs; a round takes whole columns
// (all their chunks) and reads them completely before any thread writes, so
// the product can overwrite its input.  blockDim.x must be a multiple of
// 32 * CH so that each warp holds a single chunk.
template <int KIND>
__device__ __forceinline__ float gmat(const float* G, int N, int i, int k) {
    float m = KIND == 1 ? G[k * N + i] : G[i * N + k];
    return KIND == 2 ? mul_rn(m, m) : m;
}

template <int N, int KIND>
__device__ void group_axis_inplace(float* buf, int P, const float* G) {
    constexpr int IC = N >= 16 ? 8 : N;  // outputs per thread
    constexpr int CH = N / IC;           // threads per column
    // a warp shares one output chunk over 32 consecutive columns: matrix reads
    // are broadcasts, column reads and writes hit consecutive banks
    const int cols = static_cast<int>(blockDim.x) / CH;
    for (int c0 = 0; c0 < P; c0 += cols) {
        const int p = c0 + static_cast<int>(threadIdx.x) % cols;
        const int i0 = (static_cast<int>(threadIdx.x) / cols) * IC;
        const bool act = static_cast<int>(threadIdx.x) < cols * CH && p < P;
        float x[N];
        if (act) {
#pragma unroll
            for (int k = 0; k < N; ++k) x[k] = buf[k * P + p];
        }
        __syncthreads();
        if (act) {
#pragma unroll
            for (int ii = 0; ii < IC; ++ii) {
                const int i = i0 + ii;
                float acc = 0.0f;
                if (KIND != 1 && N % 4 == 0) {
#pragma unroll
                    for (int k = 0; k < N; k += 4) {
                        float4 m = *reinterpret_cast<const float4*>(G + i * N + k);
                        if (KIND == 2) {
                            m.x = mul_rn(m.x, m.x);
                            m.y = mul_rn(m.y, m.y);
                            m.z = mul_rn(m.z, m.z);
                            m.w = mul_rn(m.w, m.w);
                        }
                        acc = fmaf(m.x, x[k], acc);
                        acc = fmaf(m.y, x[k + 1], acc);
                        acc = fmaf(m.z, x[k + 2], acc);
                        acc = fmaf(m.w, x[k + 3], acc);
                    }
                } else {
#pragma unroll
                    for (int k = 0; k < N; ++k) acc = fmaf(gmat<KIND>(G, N, i, k), x[k], acc);
                }
                buf[i * P + p] = acc;
            }
        }
        __syncthreads();
    }
}

// Haar group axis by its sum pyramid (one thread per column, O(N) operations):
// row (l, j) of the orthonormal Haar matrix, block width w = N / 2^(l-1), is
// (first-half sum - second-half sum) / sqrt(w); its elementwise square gives the
// block sum / w; the inverse adds and subtracts the detail down the pyramid.
// The rounding differs from the matrix product, so only the fast path uses it.
template <int N, int KIND>
__device__ __forceinline__ void haar_column(float* buf, int p, int P) {
    {
        float x[N];
#pragma unroll
        for (int k = 0; k < N; ++k) x[k] = buf[k * P + p];
        float out[N];
        if (KIND == 1) {
            // x = H^T c: start from the DC, refine block by block
            out[0] = x[0] * rsqrtf(static_cast<float>(N));
#pragma unroll
            for (int w = N; w >= 2; w >>= 1) {
                const int nb = N / w;
                const float sc = rsqrtf(static_cast<float>(w));
#pragma unroll
                for (int j = nb - 1; j >= 0; --j) {
                    const float d = x[nb + j] * sc;
                    const float a = out[j];
                    out[2 * j + 1] = a - d;
                    out[2 * j] = a + d;
                }
            }
        } else {
            float sm_[N];
#pragma unroll
            for (int k = 0; k < N; ++k) sm_[k] = x[k];
#pragma unroll
            for (int w = 2; w <= N; w <<= 1) {
                const int nb = N / w;
                const float sc = KIND == 2 ? 1.0f / static_cast<float>(w) : rsqrtf(static_cast<float>(w));
#pragma unroll
                for (int j = 0; j < nb; ++j) {
                    const float a = sm_[2 * j], b = sm_[2 * j + 1];
                    out[nb + j] = (KIND == 2 ? a + b : a - b) * sc;
                    sm_[j] = a + b;
                }
            }
            out[0] = sm_[0] * (KIND == 2 ? 1.0f / static_cast<float>(N) : rsqrtf(static_cast<float>(N)));
        }
#pragma unroll
        for (int k = 0; k < N; ++k) buf[k * P + p] = out[k];
    }
}

template <int N, int KIND>
__device__ void haar_axis_fast(float* buf, int P) {
    for (int p = threadIdx.x; p < P; p += blockDim.x) haar_column<N, KIND>(buf, p, P);
    __syncthreads();
}

// the forward Haar group axis of three groups in one sweep: s squared (kind
// 2), x and r (kind 0; r may be null)
template <int N>
__device__ void haar_axis_fast3(float* s, float* x, float* r, int P) {
    for (int p = threadIdx.x; p < P; p += blockDim.x) {
        haar_column<N, 2>(s, p, P);
        haar_column<N, 0>(x, p, P);
        if (r) haar_column<N, 0>(r, p, P);
    }
    __syncthreads();
}

__device__ bool haar_axis_any3(float* s, float* x, float* r, int n, int P) {
    switch (n) {
        case 2: haar_axis_fast3<2>(s, x, r, P); return true;
        case 4: haar_axis_fast3<4>(s, x, r, P); return true;
        case 8: haar_axis_fast3<8>(s, x, r, P); return true;
        case 16: haar_axis_fast3<16>(s, x, r, P); return true;
        case 32: haar_axis_fast3<32>(s, x, r, P); return true;
        default: return false;
    }
}

template <int KIND>
__device__ bool haar_axis_any(float* buf, int n, int P) {
    switch (n) {
        case 2: haar_axis_fast<2, KIND>(buf, P); return true;
        case 4: haar_axis_fast<4, KIND>(buf, P); return true;
        case 8: haar_axis_fast<8, KIND>(buf, P); return true;
        case 16: haar_axis_fast<16, KIND>(buf, P); return true;
        case 32: haar_axis_fast<32, KIND>(buf, P); return true;
        default: return false;
    }
}

// runtime group size (not a power of two): one thread per column
template <int KIND>
__device__ void group_axis_generic(float* buf, int n, int P, const float* G) {
    for (int p = threadIdx.x; p < P; p += blockDim.x) {
        float x[BMND_MAX_STACK];
        for (int k = 0; k < n; ++k) x[k] = buf[k * P + p];
        for (int i = 0; i < n; ++i) {
            float acc = 0.0f;
            for (int k = 0; k < n; ++k) acc = fmaf(gmat<KIND>(G, n, i, k), x[k], acc);
            buf[i * P + p] = acc;
        }
    }
    __syncthreads();
}

template <int KIND>
__device__ void group_axis_any(float* buf, int n, int P, const float* G) {
    switch (n) {
        case 1: group_axis_inplace<1, KIND>(buf, P, G); break;
        case 2: group_axis_inplace<2, KIND>(buf, P, G); break;
        case 4: group_axis_inplace<4, KIND>(buf, P, G); break;
        case 8: group_axis_inplace<8, KIND>(buf, P, G); break;
        case 16: group_axis_inplace<16, KIND>(buf, P, G); break;
        case 32: group_axis_inplace<32, KIND>(buf, P, G); break;
        default: group_axis_generic<KIND>(buf, n, P, G); break;
    }
}

// patch axis d with compile-time edge B and stride INNER: each thread
// transforms whole lines of B values (matrix in registers), so lines never
// share a thread and the product overwrites its input
template <int B, int INNER>
__device__ __forceinline__ void space_line(float* buf, int base, const float (&m)[B * B]) {
    float x[B];
#pragma unroll
    for (int k = 0; k < B; ++k) x[k] = buf[base + k * INNER];
#pragma unroll
    for (int i = 0; i < B; ++i) {
        float acc = 0.0f;
#pragma unroll
        for (int k = 0; k < B; ++k) acc = fmaf(m[i * B + k], x[k], acc);
        buf[base + i * INNER] = acc;
    }
}

template <int B, int INNER>
__device__ void space_axis_reg(float* buf, int total, const float* Msrc, bool square) {
    float m[B * B];
#pragma unroll
    for (int q = 0; q < B * B; ++q) {
        const float v = Msrc[q];
        m[q] = square ? mul_rn(v, v) : v;
    }
    const int lines = total / B;
    for (int line = threadIdx.x; line < lines; line += blockDim.x) {
        const int o = line / INNER;
        const int t = line - o * INNER;
        space_line<B, INNER>(buf, o * B * INNER + t, m);
    }
    __syncthreads();
}

// the same axis of three groups in one sweep: s with the squared matrix, x and
// r (may be null) with the matrix itself
template <int B, int INNER>
__device__ void space_axis_reg3(float* s, float* x, float* r, int total, const float* Msrc) {
    float m[B * B], m2[B * B];
#pragma unroll
    for (int q = 0; q < B * B; ++q) {
        const float v = Msrc[q];
        m[q] = v;
        m2[q] = mul_rn(v, v);
    }
    const int lines = total / B;
    for (int line = threadIdx.x; line < lines; line += blockDim.x) {
        const int o = line / INNER;
        const int t = line - o * INNER;
        const int base = o * B * INNER + t;
        space_line<B, INNER>(s, base, m2);
        space_line<B, INNER>(x, base, m);
        if (r) space_line<B, INNER>(r, base, m);
    }
    __syncthreads();
}

// runtime geometry: one thread per line of edge m along axis d
template <class GM>
__device__ void space_axis_generic(const GM& geo, int d, float* buf, int n, const float* M, bool square) {
    const int m = geo.b(d);
    const int inner = geo.inner(d);
    const int lines = n * geo.P() / m;
    for (int line = threadIdx.x; line < lines; line += blockDim.x) {
        const int o = line / inner;
        const int t = line - o * inner;
        const int base = o * m * inner + t;
        float x[BMND_MAX_EDGE];
        for (int k = 0; k < m; ++k) x[k] = buf[base + k * inner];
        for (int i = 0; i < m; ++i) {
            float acc = 0.0f;
            for (int k = 0; k < m; ++k) {
                float mk = M[i * m + k];
                if (square) mk = mul_rn(mk, mk);
                acc = fmaf(mk, x[k], acc);
            }
            buf[base + i * inner] = acc;
        }
    }
    __syncthreads();
}

template <int ND, int B0, int B1, int B2, int D>
__device__ __forceinline__ void space_axis_fixed(float* buf, int n, const float* M, bool square) {
    constexpr int B = D == 0 ? B0 : (D == 1 ? B1 : B2);
    constexpr int INNER = D == 0 ? (ND > 1 ? B1 : 1) * (ND > 2 ? B2 : 1) : (D == 1 ? (ND > 2 ? B2 : 1) : 1);
    space_axis_reg<B, INNER>(buf, n * B0 * B1 * B2, M, square);
}

template <int ND, int B0, int B1, int B2, int D>
__device__ __forceinline__ void space_axis_fixed3(float* s, float* x, float* r, int n, const float* M) {
    constexpr int B = D == 0 ? B0 : (D == 1 ? B1 : B2);
    constexpr int INNER = D == 0 ? (ND > 1 ? B1 : 1) * (ND > 2 ? B2 : 1) : (D == 1 ? (ND > 2 ? B2 : 1) : 1);
    space_axis_reg3<B, INNER>(s, x, r, n * B0 * B1 * B2, M);
}

// separable transform of an (n, block...) group in place: the group axis
// first, then the patch axes (transforms.py:209-255).  kind: 0 forward,
// 1 inverse, 2 squared forward, 3 transposed inverse (poisson.py:84-114).
template <int ND, int B0, int B1, int B2, class GM>
__device__ void transform_group(const GM& geo, const FilterArgs& a, unsigned char* smem, int n, float* buf,
                                int kind) {
    const float* G = sm<float>(smem, a.L.g);
    const float* F = sm<float>(smem, kind == 1 ? a.L.fi : (kind == 3 ? a.L.fit : a.L.fw));
    const bool fast_haar = a.sp.fast_group_transform && a.sp.group_transform == BMND_GROUP_HAAR &&
                           (kind == 0 ? haar_axis_any<0>(buf, n, geo.P())
                                      : kind == 1 ? haar_axis_any<1>(buf, n, geo.P())
                                                  : kind == 2 ? haar_axis_any<2>(buf, n, geo.P())
                                                              : haar_axis_any<0>(buf, n, geo.P()));
    if (!fast_haar && a.sp.group_transform != BMND_GROUP_NONE) {
        // kind 3 (transposed inverse): the group transforms are orthonormal, so
        // the transposed inverse of the group axis is the forward transform
        if (kind == 0 || kind == 3) group_axis_any<0>(buf, n, geo.P(), G);
        else if (kind == 1) group_axis_any<1>(buf, n, geo.P(), G);
        else group_axis_any<2>(buf, n, geo.P(), G);
    }
    const bool square = kind == 2;
    if constexpr (ND > 0) {
        space_axis_fixed<ND, B0, B1, B2, 0>(buf, n, F, square);
        if constexpr (ND > 1) space_axis_fixed<ND, B0, B1, B2, 1>(buf, n, F + BMND_MAX_EDGE * BMND_MAX_EDGE, square);
        if constexpr (ND > 2)
            space_axis_fixed<ND, B0, B1, B2, 2>(buf, n, F + 2 * BMND_MAX_EDGE * BMND_MAX_EDGE, square);
    } else {
        for (int d = 0; d < geo.nd(); ++d)
            space_axis_generic(geo, d, buf, n, F + d * BMND_MAX_EDGE * BMND_MAX_EDGE, square);
    }
}

// The three forward transforms of the approximate path in one sweep of passes:
// the variance group S squared (kind 2), the observation X and the pilot R
// (kind 0, R may be null).  Only for compile-time patches with the Haar group
// axis by its pyramid and a power-of-two group; returns false, having done
// nothing, otherwise.  Every element goes through the same operations as in
// transform_group, so the results are the same bits.
template <int ND, int B0, int B1, int B2, class GM>
__device__ bool transform_forward3(const GM& geo, const FilterArgs& a, unsigned char* smem, int n, float* S,
                                   float* X, float* R) {
    if constexpr (ND == 0) {
        return false;
    } else {
        if (!(a.sp.fast_group_transform && a.sp.group_transform == BMND_GROUP_HAAR)) return false;
        if (!haar_axis_any3(S, X, R, n, geo.P())) return false;
        const float* F = sm<float>(smem, a.L.fw);
        space_axis_fixed3<ND, B0, B1, B2, 0>(S, X, R, n, F);
        if constexpr (ND > 1) space_axis_fixed3<ND, B0, B1, B2, 1>(S, X, R, n, F + BMND_MAX_EDGE * BMND_MAX_EDGE);
        if constexpr (ND > 2)
            space_axis_fixed3<ND, B0, B1, B2, 2>(S, X, R, n, F + 2 * BMND_MAX_EDGE * BMND_MAX_EDGE);
        return true;
    }
}

// exact float -> double widening on the integer pipe (IEEE 754 binary32 to
// binary64: rebias the exponent by 1023 - 127, shift the fraction by 29);
// zeros keep their sign, subnormals, infinities and NaNs take the hardware
// conversion.  The scatter widens two or three values per entry, and the
// float64 pipe is a small fraction of the FP32 rate on this GPU.
__device__ __forceinline__ double widen_f64(float f) {
    const uint32_t u = __float_as_uint(f);
    const uint32_t e = (u >> 23) & 0xffu;
    const uint64_t sign = static_cast<uint64_t>(u & 0x80000000u) << 32;
    if ((u & 0x7fffffffu) == 0u) return __longlong_as_double(static_cast<long long>(sign));
    if (e == 0u || e == 0xffu) return static_cast<double>(f);
    const uint64_t bits = sign | (static_cast<uint64_t>(e + 896u) << 52) | (static_cast<uint64_t>(u & 0x7fffffu) << 29);
    return __longlong_as_double(static_cast<long long>(bits));
}

__device__ __forceinline__ float variance_of(float x, float scale_f, float floor_f) {
    float nn = x > 0.0f ? x : 0.0f;
    float v = mul_rn(scale_f, nn);
    return v > floor_f ? v : floor_f;
}

// Tolerance-aware hard-threshold mask of the Poisson path (bmndalgo.py:460-485,
// poisson.py:30-46): in count units cc = mag / scale and tc = thr / scale, a
// coefficient is kept iff cc > tc + 128 eps32 max(cc, tc, 1), evaluated in
// float64.  Multiplying through by scale, the real-arithmetic boundary is
// A = thr + 2^-16 max(mag, thr, scale).  Its float32 estimate a is within
// 2^-23 A of it, and the float64 evaluation within ~2^-50 A, so whenever mag
// lies outside a * (1 -+ 2^-20) the float32 comparison gives the float64
// decision; only the band around the boundary (and non-finite inputs) takes the
// float64 path.
__device__ __forceinline__ bool ht_keep_f64(float mag, float thr, double scale) {
    double cc = static_cast<double>(mag) / scale;
    double tc = static_cast<double>(thr) / scale;
    double cs = cc > tc ? cc : tc;
    if (cs < 1.0) cs = 1.0;
    double tol = 128.0 * 1.1920928955078125e-07 * cs;
    return cc > tc + tol;
}

__device__ __forceinline__ bool ht_keep(float mag, float thr, double scale, float scale_f) {
    const float cs = fmaxf(fmaxf(mag, thr), scale_f);
    if (cs >= 1e-30f && cs <= 1e30f) {
        const float a = add_rn(thr, mul_rn(1.52587890625e-05f, cs));  // 2^-16
        if (mag > mul_rn(a, 1.00000095367431640625f)) return true;   // 1 + 2^-20
        if (mag < mul_rn(a, 0.99999904632568359375f)) return false;  // 1 - 2^-20
    }
    return ht_keep_f64(mag, thr, scale);
}

// Exact overlap-aware variance of the first kk group planes (variance.py:950-975):
//   var[i, j] = sum_v V_v c_v[i, j]^2,   c_v[i, j] = sum_{e in v} G[i, g_e] S[j, p_e]
// over the union voxels v, each voxel's entries taken in ascending member order.
// S[j, p] is read from the precomputed S^T, whose entries are the reference's
// float32 Kronecker products.  c and the sum over voxels are accumulated with
// fused multiply-adds (one rounding per term instead of the reference's two).
//
// Work split: warp w takes the voxels whose entry lists start in its 1/nw share
// of all entries, and accumulates every (plane, coefficient) pair over them;
// lane l holds NQ planes (4, or kk when fewer) of the JR consecutive
// coefficients j0 + JR * l + r, so one entry costs three loads (the entry and
// the NQ G values, both warp broadcasts, and one JR-wide vector of S^T) for
// NQ * JR fused multiply-adds.
// The warps' partial sums are then added in warp order, which fixes the result
// independently of scheduling.  An entry packs member g (low byte) and the row
// offset p * kron_stride(P) of S^T (upper bits).
template <int JR>
struct KronVec;
template <>
struct KronVec<1> {
    float v[1];
    __device__ __forceinline__ void load(const float* p) { v[0] = __ldg(p); }
};
template <>
struct KronVec<2> {
    float v[2];
    __device__ __forceinline__ void load(const float* p) {
        const float2 t = __ldg(reinterpret_cast<const float2*>(p));
        v[0] = t.x;
        v[1] = t.y;
    }
};
template <>
struct KronVec<4> {
    float v[4];
    __device__ __forceinline__ void load(const float* p) {
        const float4 t = __ldg(reinterpret_cast<const float4*>(p));
        v[0] = t.x;
        v[1] = t.y;
        v[2] = t.z;
        v[3] = t.w;
    }
};

template <int NQ>
struct PlaneVec {
    float v[NQ];
    __device__ __forceinline__ void load(const float* p) {
        if constexpr (NQ == 4) {
            const float4 t = *reinterpret_cast<const float4*>(p);
            v[0] = t.x;
            v[1] = t.y;
            v[2] = t.z;
            v[3] = t.w;
        } else if constexpr (NQ == 2) {
            const float2 t = *reinterpret_cast<const float2*>(p);
            v[0] = t.x;
            v[1] = t.y;
        } else {
            v[0] = *p;
        }
    }
};

// The warp's (or half-warp's) voxels [u_lo, u_hi) are walked as one stream of
// entries: an entry adds G[i, g] S[j, p] to the running c of its voxel, and the
// first entry of the next voxel first folds V_u c^2 into var.  The loads of
// entry e + 1 are issued before the multiply-adds of entry e, and its entry
// word one step earlier, so the shared-memory and L1 latencies overlap the
// arithmetic across voxel boundaries.  Lane l holds RL coefficients starting
// at j0 + jl (jl = RL l, or RL (l % 16) for the half-warp form).
template <int RL, int NQ>
__device__ __forceinline__ void exact_stream(const float* __restrict__ lval, const int* __restrict__ lstart,
                                             const uint32_t* __restrict__ lent, int u_lo, int u_hi,
                                             const float* __restrict__ gt0, int kpad,
                                             const float* __restrict__ stl, float (&var)[RL][NQ]) {
#pragma unroll
    for (int r = 0; r < RL; ++r)
#pragma unroll
        for (int q = 0; q < NQ; ++q) var[r][q] = 0.0f;
    if (u_lo >= u_hi) return;
    int e = lstart[u_lo];
    const int e_end = lstart[u_hi];
    int u = u_lo;
    int next_start = lstart[u + 1];
    float v = lval[u];
    float c[RL][NQ];
#pragma unroll
    for (int r = 0; r < RL; ++r)
#pragma unroll
        for (int q = 0; q < NQ; ++q) c[r][q] = 0.0f;
    uint32_t ent1 = lent[e];
    PlaneVec<NQ> g0;
    KronVec<RL> s0;
    g0.load(gt0 + (ent1 & 0xffu) * kpad);
    s0.load(stl + (ent1 >> 8));
    ent1 = lent[e + 1 < e_end ? e + 1 : e];
    for (; e < e_end; ++e) {
        // loads of entry e + 1 (harmless repeats of the last entry at the end)
        PlaneVec<NQ> g1;
        KronVec<RL> s1;
        g1.load(gt0 + (ent1 & 0xffu) * kpad);
        s1.load(stl + (ent1 >> 8));
        const uint32_t ent2 = lent[e + 2 < e_end ? e + 2 : e_end - 1];
        if (e == next_start) {
#pragma unroll
            for (int r = 0; r < RL; ++r)
#pragma unroll
                for (int q = 0; q < NQ; ++q) {
                    var[r][q] = fmaf(mul_rn(v, c[r][q]), c[r][q], var[r][q]);
                    c[r][q] = 0.0f;
                }
            ++u;
            v = lval[u];
            next_start = lstart[u + 1];
        }
        // the voxel's first entry: fma(g, s, 0) is the rounded product
#pragma unroll
        for (int r = 0; r < RL; ++r)
#pragma unroll
            for (int q = 0; q < NQ; ++q) c[r][q] = fmaf(g0.v[q], s0.v[r], c[r][q]);
        g0 = g1;
        s0 = s1;
        ent1 = ent2;
    }
#pragma unroll
    for (int r = 0; r < RL; ++r)
#pragma unroll
        for (int q = 0; q < NQ; ++q) var[r][q] = fmaf(mul_rn(v, c[r][q]), c[r][q], var[r][q]);
}

// one tile of NQ planes x 32 JR coefficients over the warp's voxels
template <int JR, int NQ>
__device__ void exact_tile(const float* __restrict__ lval, const int* __restrict__ lstart,
                           const uint32_t* __restrict__ lent, int u_lo, int u_hi,
                           const float* __restrict__ GT, int kpad, int i0,
                           const float* __restrict__ st, int j0, float (&var)[JR][NQ]) {
    const int lane = threadIdx.x & 31;
    exact_stream<JR, NQ>(lval, lstart, lent, u_lo, u_hi, GT + i0, kpad, st + j0 + JR * lane, var);
}

// Patches of 33-64 voxels (JR = 2): the two half-warps take the two halves of
// the warp's voxels and each lane holds 4 coefficients, j = 4 (lane % 16) + r,
// so an entry costs the same three loads for 4 NQ fused multiply-adds instead
// of 2 NQ.  The halves' sums are added at the end (lanes l and l + 16 hold the
// same coefficients).
template <int NQ>
__device__ void exact_tile_hw(const float* __restrict__ lval, const int* __restrict__ lstart,
                              const uint32_t* __restrict__ lent, int u_lo, int u_hi,
                              const float* __restrict__ GT, int kpad, int i0,
                              const float* __restrict__ st, float (&var)[4][NQ]) {
    const int lane = threadIdx.x & 31;
    const int half = lane >> 4;
    // split at the first voxel whose entries start in the second half of the entries
    const int e_mid = (lstart[u_lo] + lstart[u_hi]) >> 1;
    int lo = u_lo, hi = u_hi;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (lstart[mid] < e_mid) lo = mid + 1;
        else hi = mid;
    }
    const int u_mid = lo;
    exact_stream<4, NQ>(lval, lstart, lent, half ? u_mid : u_lo, half ? u_hi : u_mid, GT + i0, kpad,
                        st + 4 * (lane & 15), var);
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int q = 0; q < NQ; ++q) var[r][q] = add_rn(var[r][q], __shfl_xor_sync(0xffffffffu, var[r][q], 16));
}

// all tiles of (NQ planes) x (TW coefficients); EX[i * P + j] receives the
// standard deviation sqrt(max(var, 0)) of planes i < kk.  NQ = 4 in general;
// groups with fewer exact planes (k < 4, or fewer members) use NQ = kk.  Each
// warp leaves its partial sums in `part`; after one barrier every thread adds
// the warps' partials of its (plane, coefficient) pairs in warp order.
template <int JR, int NQ>
__device__ void exact_planes(const float* __restrict__ lval, const int* __restrict__ lstart,
                             const uint32_t* __restrict__ lent, int U, const float* __restrict__ GT,
                             int kpad, int kk, const float* __restrict__ st, int P,
                             float* __restrict__ EX, float* __restrict__ part) {
    constexpr bool kHalf = JR == 2;
    constexpr int RL = kHalf ? 4 : JR;       // coefficients per lane
    constexpr int TW = kHalf ? 64 : 32 * JR;  // coefficients per tile
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nw = blockDim.x >> 5;
    // voxel range of this warp: voxels whose first entry lies in its entry share
    const int E = lstart[U];
    auto first_voxel = [&](int e) {
        int lo = 0, hi = U;  // first u in [0, U] with lstart[u] >= e
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (lstart[mid] < e) lo = mid + 1;
            else hi = mid;
        }
        return lo;
    };
    const int u_lo = first_voxel(static_cast<int>(static_cast<int64_t>(E) * warp / nw));
    const int u_hi = warp == nw - 1 ? U : first_voxel(static_cast<int>(static_cast<int64_t>(E) * (warp + 1) / nw));
    const int jl = kHalf ? 4 * (lane & 15) : JR * lane;
    const bool writer = !kHalf || lane < 16;
    for (int i0 = 0; i0 < kk; i0 += NQ) {
        for (int j0 = 0; j0 < P; j0 += TW) {
            float var[RL][NQ];
            if constexpr (kHalf) exact_tile_hw<NQ>(lval, lstart, lent, u_lo, u_hi, GT, kpad, i0, st, var);
            else exact_tile<JR, NQ>(lval, lstart, lent, u_lo, u_hi, GT, kpad, i0, st, j0, var);
            if (writer) {
#pragma unroll
                for (int q = 0; q < NQ; ++q)
#pragma unroll
                    for (int r = 0; r < RL; ++r) part[(warp * NQ + q) * TW + jl + r] = var[r][q];
            }
            __syncthreads();
            for (int t = threadIdx.x; t < NQ * TW; t += blockDim.x) {
                const int q = t / TW, jj = t - q * TW;
                const int i = i0 + q, j = j0 + jj;
                if (i < kk && j < P) {
                    float v = part[q * TW + jj];
                    for (int w = 1; w < nw; ++w) v = add_rn(v, part[(w * NQ + q) * TW + jj]);
                    EX[i * P + j] = sqrtf(v > 0.0f ? v : 0.0f);
                }
            }
            __syncthreads();
        }
    }
}

template <int JR>
__device__ void exact_planes_any(const float* __restrict__ lval, const int* __restrict__ lstart,
                                 const uint32_t* __restrict__ lent, int U, const float* __restrict__ GT,
                                 int kpad, int kk, const float* __restrict__ st, int P,
                                 float* __restrict__ EX, float* __restrict__ part) {
    if (kk == 1) exact_planes<JR, 1>(lval, lstart, lent, U, GT, kpad, kk, st, P, EX, part);
    else if (kk == 2) exact_planes<JR, 2>(lval, lstart, lent, U, GT, kpad, kk, st, P, EX, part);
    else exact_planes<JR, 4>(lval, lstart, lent, U, GT, kpad, kk, st, P, EX, part);
}

// Exact noise risk of the first kk planes (wiener.py:638-711, :505-535; the
// group metric Ginv^T Ginv of the orthonormal group transforms is the
// identity, the reference's diagonal branch):
//   risk = sum_u V_u sum_{g < kk} f_u[g]^T SM f_u[g],  f_u[g][j] = a[g][j] c_u[g][j],
// c_u as in the exact variance and SM = S_inv^T diag(w^2) S_inv, row p at
// sm + p * kron_stride(P).  Lane l holds coefficients j = JR l + r (P <= 32 JR:
// one tile); (f SM)[j] = sum_p f[p] SM[p][j] takes f[p] from its lane by a
// shuffle.  The voxel terms are float32, their sum over voxels float64.
template <int JR, int NQ>
__device__ double exact_risk_tile(const float* __restrict__ lval, const int* __restrict__ lstart,
                                  const uint32_t* __restrict__ lent, int u_lo, int u_hi,
                                  const float* __restrict__ GT, int kpad, int i0, int kk,
                                  const float* __restrict__ st, const float* __restrict__ smt,
                                  const float* __restrict__ att, int P) {
    const int lane = threadIdx.x & 31;
    const int stride = kron_stride(P);
    const float* stl = st + JR * lane;
    float gq[JR][NQ];
#pragma unroll
    for (int r = 0; r < JR; ++r)
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
            const int j = JR * lane + r, i = i0 + q;
            gq[r][q] = (j < P && i < kk) ? att[i * P + j] : 0.0f;
        }
    const float* gt0 = GT + i0;
    double acc = 0.0;
    for (int u = u_lo; u < u_hi; ++u) {
        int e = lstart[u];
        const int e1 = lstart[u + 1];
        float c[JR][NQ];
        {
            const uint32_t ent = lent[e];
            PlaneVec<NQ> gv;
            gv.load(gt0 + (ent & 0xffu) * kpad);
            KronVec<JR> sv;
            sv.load(stl + (ent >> 8));
#pragma unroll
            for (int r = 0; r < JR; ++r)
#pragma unroll
                for (int q = 0; q < NQ; ++q) c[r][q] = mul_rn(gv.v[q], sv.v[r]);
        }
        for (++e; e < e1; ++e) {
            const uint32_t ent = lent[e];
            PlaneVec<NQ> gv;
            gv.load(gt0 + (ent & 0xffu) * kpad);
            KronVec<JR> sv;
            sv.load(stl + (ent >> 8));
#pragma unroll
            for (int r = 0; r < JR; ++r)
#pragma unroll
                for (int q = 0; q < NQ; ++q) c[r][q] = fmaf(gv.v[q], sv.v[r], c[r][q]);
        }
        float f[JR][NQ], pr[JR][NQ];
#pragma unroll
        for (int r = 0; r < JR; ++r)
#pragma unroll
            for (int q = 0; q < NQ; ++q) {
                f[r][q] = mul_rn(gq[r][q], c[r][q]);
                pr[r][q] = 0.0f;
            }
        for (int sl = 0; sl < 32; ++sl) {
#pragma unroll
            for (int rr = 0; rr < JR; ++rr) {
                const int p = sl * JR + rr;
                if (p < P) {  // the same for every lane
                    float fp[NQ];
#pragma unroll
                    for (int q = 0; q < NQ; ++q) fp[q] = __shfl_sync(0xffffffffu, f[rr][q], sl);
                    KronVec<JR> mv;
                    mv.load(smt + p * stride + JR * lane);
#pragma unroll
                    for (int r = 0; r < JR; ++r)
#pragma unroll
                        for (int q = 0; q < NQ; ++q) pr[r][q] = fmaf(fp[q], mv.v[r], pr[r][q]);
                }
            }
        }
        float t = 0.0f;
#pragma unroll
        for (int r = 0; r < JR; ++r)
#pragma unroll
            for (int q = 0; q < NQ; ++q) t = fmaf(f[r][q], pr[r][q], t);
        acc = fma(static_cast<double>(lval[u]), static_cast<double>(t), acc);
    }
    return acc;
}

// the group's exact noise risk into *out (every thread returns after it is set):
// warp w takes the voxels whose entry lists start in its share of all entries
// (the exact variance's split); lanes, then warps, add in a fixed order
template <int JR, int NQ>
__device__ void exact_risk(const float* __restrict__ lval, const int* __restrict__ lstart,
                           const uint32_t* __restrict__ lent, int U, const float* __restrict__ GT, int kpad,
                           int kk, const float* __restrict__ st, const float* __restrict__ smt,
                           const float* __restrict__ att, int P, double* __restrict__ part) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nw = blockDim.x >> 5;
    const int E = lstart[U];
    auto first_voxel = [&](int e) {
        int lo = 0, hi = U;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (lstart[mid] < e) lo = mid + 1;
            else hi = mid;
        }
        return lo;
    };
    const int u_lo = first_voxel(static_cast<int>(static_cast<int64_t>(E) * warp / nw));
    const int u_hi = warp == nw - 1 ? U : first_voxel(static_cast<int>(static_cast<int64_t>(E) * (warp + 1) / nw));
    double acc = 0.0;
    for (int i0 = 0; i0 < kk; i0 += NQ)
        acc += exact_risk_tile<JR, NQ>(lval, lstart, lent, u_lo, u_hi, GT, kpad, i0, kk, st, smt, att, P);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) part[warp] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < nw; ++w) t += part[w];
        part[nw] = t;
    }
    __syncthreads();
}

template <int JR>
__device__ void exact_risk_any(const float* __restrict__ lval, const int* __restrict__ lstart,
                               const uint32_t* __restrict__ lent, int U, const float* __restrict__ GT, int kpad,
                               int kk, const float* __restrict__ st, const float* __restrict__ smt,
                               const float* __restrict__ att, int P, double* __restrict__ part) {
    if (kk == 1) exact_risk<JR, 1>(lval, lstart, lent, U, GT, kpad, kk, st, smt, att, P, part);
    else if (kk == 2) exact_risk<JR, 2>(lval, lstart, lent, U, GT, kpad, kk, st, smt, att, P, part);
    else exact_risk<JR, 4>(lval, lstart, lent, U, GT, kpad, kk, st, smt, att, P, part);
}

template <int ND, int B0, int B1, int B2, int NT>
__global__ void __launch_bounds__(NT, NT == kThreads ? (ND >= 2 ? 3 : 2) : 1) group_filter_kernel(FilterArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    using GM = Geom<ND, B0, B1, B2>;
    const BmndStageParams& sp = a.sp;
    const GM geo(sp);
    const int64_t gid = blockIdx.x;
    const int tid = threadIdx.x;
    const int P = geo.P();
    const int n = a.count[gid];
    if (n <= 0) return;
    if (n > a.nmax) {
        if (tid == 0 && a.err) atomicExch(a.err, 2);
        return;
    }
    const bool wiener = sp.filter == BMND_FILTER_WIENER;

    float* G = sm<float>(smem, a.L.g);
    float* GT = sm<float>(smem, a.L.gt);
    float* Fw = sm<float>(smem, a.L.fw);
    float* Fi = sm<float>(smem, a.L.fi);
    float* win = sm<float>(smem, a.L.win);
    double* mdiag = sm<double>(smem, a.L.mdiag);
    int* pos = sm<int>(smem, a.L.pos);
    int* shf = sm<int>(smem, a.L.shf);
    float* S = sm<float>(smem, a.L.s);
    float* EX = sm<float>(smem, a.L.ex);
    float* X = sm<float>(smem, a.L.x);
    float* R = sm<float>(smem, a.L.r);
    float* V = sm<float>(smem, a.L.v);  // aliases R: the attenuation
    uint32_t* grid = sm<uint32_t>(smem, a.L.grid);
    float* lval = sm<float>(smem, a.L.lval);
    int* lstart = sm<int>(smem, a.L.lstart);
    uint32_t* lent = sm<uint32_t>(smem, a.L.lent);
    int2* scan = sm<int2>(smem, a.L.scan);
    double* plane = sm<double>(smem, a.L.plane);
    float* wts = sm<float>(smem, a.L.wts);
    int* misc = sm<int>(smem, a.L.misc);

    const int k = sp.variance_k;
    const int kk = k < n ? k : n;
    const int kpad = (a.kmax + 3) / 4 * 4;

    // ---- setup: positions, matrices, window ----
    // a member outside the patch grid skips the group (matching never makes one)
    bool bad_member = false;
    if (tid < n) {
        const int32_t lin = a.sel[gid * sp.max_stack + tid];
        bad_member = lin < 0 || lin >= a.n_lins;
        // lins fit in 31 bits (volumes are limited to 2^31 voxels): 32-bit division
        uint32_t rem = static_cast<uint32_t>(lin);
        for (int d = geo.nd() - 1; d >= 0 && !bad_member; --d) {
            const uint32_t c = static_cast<uint32_t>(a.counts[d]);
            const uint32_t q = rem / c;
            pos[tid * BMND_MAX_DIMS + d] = static_cast<int>(rem - q * c);
            rem = q;
        }
    }
    if (__syncthreads_or(bad_member)) {
        if (tid == 0 && a.err) atomicExch(a.err, 2);
        return;
    }
    {
        const float* gtab = a.st + 2 * static_cast<int64_t>(P) * kron_stride(P) + group_table_offset(n);
        for (int e = tid; e < n * n; e += blockDim.x) G[e] = __ldg(gtab + e);
    }
    // only the b x b entries of each axis are read; the parameters live in the
    // constant bank, where lanes reading different addresses take turns
    for (int d = 0; d < geo.nd(); ++d) {
        const int bb = geo.b(d) * geo.b(d);
        for (int q = tid; q < bb; q += blockDim.x) {
            Fw[d * BMND_MAX_EDGE * BMND_MAX_EDGE + q] = sp.spatial_fwd[d][q];
            Fi[d * BMND_MAX_EDGE * BMND_MAX_EDGE + q] = sp.spatial_inv[d][q];
        }
    }
    for (int e = tid; e < P; e += blockDim.x) win[e] = sp.window[e];
    if (sp.windowed_synthesis)  // the only reader of the metric diagonal
        for (int e = tid; e < P; e += blockDim.x) mdiag[e] = sp.spatial_metric_diag[e];
    if (a.den_ro) {
        // matrices are stored densely, b x b row-major, per axis
        float* Fit = sm<float>(smem, a.L.fit);
        constexpr int EE = BMND_MAX_EDGE * BMND_MAX_EDGE;
        for (int e = tid; e < BMND_MAX_DIMS * EE; e += blockDim.x) {
            const int d = e / EE, q = e % EE;
            const int b = d < geo.nd() ? geo.b(d) : 1;
            const int i = q / b, k = q % b;
            Fit[e] = q < b * b ? sp.spatial_inv[d][k * b + i] : 0.0f;
        }
    }
    __syncthreads();
    // G^T restricted to the exact planes, padded to 4: GT[g * kpad + i] = G[i, g]
    for (int e = tid; e < n * kpad; e += blockDim.x) {
        int g = e / kpad, i = e % kpad;
        GT[e] = i < kk ? G[i * n + g] : 0.0f;
    }
    if (tid < 32) {
        // group origin (min over members), member shifts, union extent, and the
        // patch-linear offset of each shift: element p of member g lies in union
        // cell c with p = lin(c) - shl[g], lin(c) = sum_d c_d inner(d)
        const bool live = tid < n;
        int lin = 0;
        for (int d = 0; d < geo.nd(); ++d) {
            const int v = live ? pos[tid * BMND_MAX_DIMS + d] : 0x7fffffff;
            const int mn = __reduce_min_sync(0xffffffffu, v);
            const int sh = live ? v - mn : 0;
            const int mx = __reduce_max_sync(0xffffffffu, sh);
            if (live) shf[tid * BMND_MAX_DIMS + d] = sh;
            lin += sh * geo.inner(d);
            if (tid == 0) {
                misc[d] = mn;                  // origin
                misc[4 + d] = mx + geo.b(d);   // union extent
            }
        }
        if (live) sm<int>(smem, a.L.shl)[tid] = lin;
    }
    __syncthreads();

    const float scale_f = static_cast<float>(sp.count_scale);
    const float floor_f = static_cast<float>(sp.variance_floor);
    const float* varsrc = (wiener && sp.wiener_variance_source == BMND_SOURCE_PILOT) ? a.pilot : a.noisy;
    const int total = n * P;
    const bool need_approx = (k <= 0) || (kk < n);

    const bool gauss = sp.noise_model == BMND_NOISE_GAUSSIAN;
    const bool exact_risk = sp.exact_risk_weights != 0 && kk > 0;
    if ((!gauss || exact_risk) && kk > 0) {
        // the exact phase's occupancy grid covers a union box of at most
        // ucells_cap cells: members within the search window of their reference
        // always fit; a group spread wider is skipped and reported
        int64_t uc = 1;
        for (int d = 0; d < geo.nd(); ++d) uc *= misc[4 + d];
        if (uc > a.ucells_cap) {
            if (tid == 0 && a.err) atomicExch(a.err, 2);
            return;
        }
    }
    if (gauss) {
        // ---- stationary Gaussian noise (variance.py:2036-2106) ----
        // exact planes g < kk: sum_{i,j} G[g,i] G[g,j] C_c((x_i - x_j) mod domain),
        // C_c the covariance map of spatial coefficient c; the other planes
        // share what is left of n times the patch variance C_c(0)
        int* lag = sm<int>(smem, a.L.lag);
        const int npair = n * (n + 1) / 2;
        if (kk > 0) {
            for (int q = tid; q < npair; q += blockDim.x) {
                int i = static_cast<int>((sqrtf(8.0f * static_cast<float>(q) + 1.0f) - 1.0f) * 0.5f);
                while (i * (i + 1) / 2 > q) --i;
                while ((i + 1) * (i + 2) / 2 <= q) ++i;
                const int j = q - i * (i + 1) / 2;
                int flat = 0;
                for (int d = 0; d < geo.nd(); ++d) {
                    const int D = sp.cov_domain[d];
                    int l = (pos[i * BMND_MAX_DIMS + d] - pos[j * BMND_MAX_DIMS + d]) % D;
                    if (l < 0) l += D;
                    flat = flat * D + l;
                }
                lag[q] = flat;
            }
            __syncthreads();
        }
        const float* cm = sp.cov_maps;
        // one thread per (plane, coefficient): the planes' sums are independent
        for (int t = tid; t < kk * P; t += blockDim.x) {
            const int g = t / P, c = t - g * P;
            const float pv = __ldg(cm + c);  // lag 0: the patch variance of coefficient c
            const float* Gr = G + g * n;
            float value = 0.0f;
            for (int i = 0; i < n; ++i) {
                const float wi = Gr[i];
                if (wi == 0.0f) continue;
                value = add_rn(value, mul_rn(mul_rn(wi, pv), wi));
                const int* lrow = lag + i * (i + 1) / 2;
                for (int j = 0; j < i; ++j) {
                    const float wj = Gr[j];
                    if (wj == 0.0f) continue;
                    const float cv = __ldg(cm + static_cast<int64_t>(lrow[j]) * P + c);
                    value = add_rn(value, mul_rn(mul_rn(wi, wj), add_rn(cv, cv)));
                }
            }
            EX[g * P + c] = fmaxf(value, 0.0f);
        }
        __syncthreads();
        for (int c = tid; c < P; c += blockDim.x) {
            const float pv = __ldg(cm + c);
            float ex_sum = 0.0f;
            for (int g = 0; g < kk; ++g) ex_sum = add_rn(ex_sum, EX[g * P + c]);
            float rest = pv;
            if (kk > 0 && kk < n) {
                rest = div_rn(sub_rn(mul_rn(static_cast<float>(n), pv), ex_sum), static_cast<float>(n - kk));
                rest = fmaxf(rest, 0.0f);
            }
            for (int g = 0; g < n; ++g) {
                const float v = g < kk ? EX[g * P + c] : rest;
                S[g * P + c] = sqrtf(fmaxf(v, 0.0f));
            }
        }
        __syncthreads();
    }

    // ---- union voxels and the exact overlap-aware sigma of the first kk planes ----
    // (with exact risk weights under white Gaussian noise: the union voxels
    // alone, each with the noise variance, variance.py:1451-1496)
    int U = 0;
    if ((!gauss || exact_risk) && kk > 0) {
        int ush[BMND_MAX_DIMS] = {1, 1, 1}, org[BMND_MAX_DIMS] = {0, 0, 0};
        int ucells = 1;
        for (int d = 0; d < geo.nd(); ++d) {
            ush[d] = misc[4 + d];
            org[d] = misc[d];
            ucells *= ush[d];
        }
        for (int c = tid; c < ucells; c += blockDim.x) grid[c] = 0u;
        __syncthreads();
        for (int e = tid; e < total; e += blockDim.x) {
            const int g = e / P;
            int p = e - g * P;
            int cell = 0, mul = 1;
#pragma unroll
            for (int d = BMND_MAX_DIMS - 1; d >= 0; --d) {
                if (d < geo.nd()) {
                    cell += (shf[g * BMND_MAX_DIMS + d] + p % geo.b(d)) * mul;
                    mul *= ush[d];
                    p /= geo.b(d);
                }
            }
            atomicOr(grid + cell, 1u << g);
        }
        __syncthreads();
        // compact occupied cells (ascending) and their entries (ascending
        // member): warp w takes a contiguous 1/nw of the cells, 32 at a time,
        // one cell per lane; voxel ranks come from ballots and entry offsets
        // from a warp scan of the cells' member counts, after the warps'
        // totals are added up in warp order.  The cell index is parked in lval
        // until the variance pass below.
        {
            const int nw = blockDim.x >> 5, warp = tid >> 5, lane = tid & 31;
            const int cpw = (ucells + nw - 1) / nw;
            const int wc0 = min(ucells, warp * cpw), wc1 = min(ucells, wc0 + cpw);
            int wv = 0, wsum = 0;
            for (int base = wc0; base < wc1; base += 32) {
                const int c = base + lane;
                const uint32_t m = c < wc1 ? grid[c] : 0u;
                wv += __popc(__ballot_sync(0xffffffffu, m != 0u));
                wsum += __popc(m);
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) wsum += __shfl_xor_sync(0xffffffffu, wsum, o);
            if (lane == 0) scan[warp] = make_int2(wv, wsum);
            __syncthreads();
            int vbase = 0, ebase = 0, vtot = 0, etot = 0;
            for (int w = 0; w < nw; ++w) {
                const int2 t = scan[w];
                if (w < warp) {
                    vbase += t.x;
                    ebase += t.y;
                }
                vtot += t.x;
                etot += t.y;
            }
            const int* shl = sm<int>(smem, a.L.shl);
            const int kstride = kron_stride(P);
            float inv_ush[BMND_MAX_DIMS];
#pragma unroll
            for (int d = 0; d < BMND_MAX_DIMS; ++d) inv_ush[d] = 1.0f / static_cast<float>(ush[d]);
            const uint32_t below = (1u << lane) - 1u;
            for (int base = wc0; base < wc1; base += 32) {
                const int c = base + lane;
                uint32_t m = c < wc1 ? grid[c] : 0u;
                const uint32_t occ = __ballot_sync(0xffffffffu, m != 0u);
                const int cnt = __popc(m);
                int incl = cnt;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int t = __shfl_up_sync(0xffffffffu, incl, o);
                    if (lane >= o) incl += t;
                }
                if (m) {
                    const int w = vbase + __popc(occ & below);
                    int we = ebase + incl - cnt;
                    // cell -> union-box coordinates -> patch-linear offset
                    int rem = c, lin = 0, cc[BMND_MAX_DIMS] = {0, 0, 0};
#pragma unroll
                    for (int d = BMND_MAX_DIMS - 1; d >= 0; --d) {
                        if (d < geo.nd()) {
                            const int q = d > 0 ? small_div(rem, inv_ush[d]) : 0;
                            cc[d] = rem - q * ush[d];
                            rem = q;
                        }
                    }
#pragma unroll
                    for (int d = 0; d < BMND_MAX_DIMS; ++d)
                        if (d < geo.nd()) lin += cc[d] * geo.inner(d);
                    reinterpret_cast<int*>(lval)[w] = c;
                    lstart[w] = we;
                    while (m) {
                        const int g = __ffs(m) - 1;
                        m &= m - 1;
                        lent[we++] = static_cast<uint32_t>(g) | (static_cast<uint32_t>((lin - shl[g]) * kstride) << 8);
                    }
                }
                vbase += __popc(occ);
                ebase += __shfl_sync(0xffffffffu, incl, 31);
            }
            if (tid == 0) scan[blockDim.x] = make_int2(vtot, etot);
        }
        __syncthreads();
        U = scan[blockDim.x].x;
        if (tid == 0) lstart[U] = scan[blockDim.x].y;
        __syncthreads();
        // variance of every union voxel, all loads in flight together
        for (int u = tid; u < U; u += blockDim.x) {
            if (gauss) {
                lval[u] = sp.exact_source_variance;
                continue;
            }
            int rem = reinterpret_cast<const int*>(lval)[u];
            int64_t vox = 0;
#pragma unroll
            for (int d = BMND_MAX_DIMS - 1; d >= 0; --d) {
                if (d < geo.nd()) {
                    const int q = d > 0 ? small_div(rem, 1.0f / static_cast<float>(ush[d])) : 0;
                    vox += static_cast<int64_t>(rem - q * ush[d] + org[d]) * a.vstride[d];
                    rem = q;
                }
            }
            lval[u] = variance_of(__ldg(varsrc + vox), scale_f, floor_f);
        }
        __syncthreads();
        if (gauss) {
            // sigma comes from the covariance maps
        } else if constexpr (ND > 0) {
            exact_planes_any<kron_jr(B0 * B1 * B2)>(lval, lstart, lent, U, GT, kpad, kk, a.st, P, EX,
                                                    sm<float>(smem, a.L.part));
        } else {
            const int jr = kron_jr(P);
            float* part = sm<float>(smem, a.L.part);
            if (jr == 1) exact_planes_any<1>(lval, lstart, lent, U, GT, kpad, kk, a.st, P, EX, part);
            else if (jr == 2) exact_planes_any<2>(lval, lstart, lent, U, GT, kpad, kk, a.st, P, EX, part);
            else exact_planes_any<4>(lval, lstart, lent, U, GT, kpad, kk, a.st, P, EX, part);
        }
    }

    // ---- approximate sigma from the variance group (squared transforms) ----
    // (after the exact phase: S shares the union region with its lists)
    // The observation (and the pilot) are gathered here too, so the volume the
    // variance comes from is read once (its lists are no longer needed).
    bool gathered = false;
    bool fused = false;  // X and R already forward-transformed with S
    if (!gauss && need_approx) {
        for (int e = tid; e < total; e += blockDim.x) {
            const int g = e / P;
            const int64_t off = geo.offset(pos + g * BMND_MAX_DIMS, e - g * P, a.vstride);
            const float vs = __ldg(varsrc + off);
            S[e] = variance_of(vs, scale_f, floor_f);
            X[e] = varsrc == a.noisy ? vs : __ldg(a.noisy + off);
            if (wiener) R[e] = varsrc == a.pilot ? vs : __ldg(a.pilot + off);
        }
        gathered = true;
        __syncthreads();
        fused = transform_forward3<ND, B0, B1, B2>(geo, a, smem, n, S, X, wiener ? R : nullptr);
        if (!fused) transform_group<ND, B0, B1, B2>(geo, a, smem, n, S, 2);
        for (int e = tid; e < total; e += blockDim.x) {
            const float v = S[e];
            S[e] = sqrtf(v > 0.0f ? v : 0.0f);
        }
        __syncthreads();
    }

    // ---- final sigma in S (plane limiting, variance.py:1572-1631) ----
    if (gauss) {
        // done above
    } else if (k > 0 && kk == n) {
        for (int e = tid; e < total; e += blockDim.x) S[e] = EX[e];
    } else if (k > 0) {
        // TPJ threads per coefficient j (neighbouring lanes), each summing the
        // planes i = sub (mod TPJ); the partial sums are added by shuffles in
        // a fixed order, and each thread rescales its own planes
        const int TPJ = P <= 64 ? 4 : (P <= 128 ? 2 : 1);
        for (int base = 0; base < P * TPJ; base += blockDim.x) {
            const int t = base + tid;
            const int j = t / TPJ, sub = t - j * TPJ;
            const bool live = j < P;
            float sum_a = 0.0f, sum_e = 0.0f, rem_a = 0.0f;
            if (live) {
                for (int i = sub; i < n; i += TPJ) {
                    const float sa = fmaxf(S[i * P + j], 0.0f);
                    const float va = mul_rn(sa, sa);
                    sum_a = add_rn(sum_a, va);
                    if (i >= kk) rem_a = add_rn(rem_a, va);
                }
                for (int i = sub; i < kk; i += TPJ) {
                    const float se = fmaxf(EX[i * P + j], 0.0f);
                    sum_e = add_rn(sum_e, mul_rn(se, se));
                }
            }
            for (int o = 1; o < TPJ; o <<= 1) {
                sum_a = add_rn(sum_a, __shfl_xor_sync(0xffffffffu, sum_a, o));
                sum_e = add_rn(sum_e, __shfl_xor_sync(0xffffffffu, sum_e, o));
                rem_a = add_rn(rem_a, __shfl_xor_sync(0xffffffffu, rem_a, o));
            }
            if (!live) continue;
            float target = sub_rn(sum_a, sum_e);
            if (target < 0.0f) target = 0.0f;
            const float scl = rem_a > 0.0f ? div_rn(target, rem_a) : 0.0f;
            for (int i = sub; i < n; i += TPJ) {
                float v;
                if (i < kk) {
                    const float se = fmaxf(EX[i * P + j], 0.0f);
                    v = mul_rn(se, se);
                } else if (rem_a > 0.0f) {
                    const float sa = fmaxf(S[i * P + j], 0.0f);
                    v = mul_rn(mul_rn(sa, sa), scl);
                } else {
                    v = div_rn(target, static_cast<float>(n - kk));
                }
                S[i * P + j] = sqrtf(v > 0.0f ? v : 0.0f);
            }
        }
    }
    __syncthreads();

    // ---- gather and forward-transform the observation (and the pilot) ----
    if (!gathered) {
        for (int e = tid; e < total; e += blockDim.x) {
            const int g = e / P;
            const int64_t off = geo.offset(pos + g * BMND_MAX_DIMS, e - g * P, a.vstride);
            X[e] = __ldg(a.noisy + off);
            if (wiener) R[e] = __ldg(a.pilot + off);
        }
        __syncthreads();
    }
    if (!fused) {
        transform_group<ND, B0, B1, B2>(geo, a, smem, n, X, 0);
        if (wiener) transform_group<ND, B0, B1, B2>(geo, a, smem, n, R, 0);
    }
    const int64_t probe_base = gid * static_cast<int64_t>(a.nmax) * P;
    if (a.probe.active) {
        for (int e = tid; e < total; e += blockDim.x) {
            if (a.probe.coef) a.probe.coef[probe_base + e] = X[e];
            if (a.probe.sigma) a.probe.sigma[probe_base + e] = S[e];
        }
    }

    // ---- shrinkage: coefficients in X, attenuation in V, and in S each
    // coefficient's aggregation error: a^2 (classic), a^2 sigma^2 (variance) or
    // a^2 sigma^2 + (1 - a)^2 signal power (risk) (aggregationweights.py:213-259) ----
    const float eps_f = static_cast<float>(sp.eps);
    float* SG = sm<float>(smem, a.L.sg);
    float sig_sum = 0.0f;  // Wiener sigma map: this thread's share of the group's sigma sum
    for (int e = tid; e < total; e += blockDim.x) {
        float sig = S[e];
        if (a.sig_num) {
            if (wiener) sig_sum += sig;
            else SG[e] = sig;
        }
        float nv = mul_rn(sig, sig);
        float att;
        float spw = 0.0f;  // Wiener signal power (risk weights)
        if (!wiener && sp.soft_threshold) {
            // soft thresholding (bmndalgo.py:476-486): sign(c) max(|c| - lambda sigma, 0)
            const float thr = mul_rn(sp.ht_lambda, sig);
            const float mag = fabsf(X[e]);
            const float shr = fmaxf(sub_rn(mag, thr), 0.0f);
            att = mag > 0.0f ? div_rn(shr, mag) : 0.0f;
            X[e] = copysignf(shr, X[e]);
            V[e] = att;
            S[e] = sp.weight_model == BMND_WEIGHT_CLASSIC ? att * att : att * att * nv;
            if (exact_risk && e < kk * P) S[e] = 0.0f;  // the exact pass below holds these planes' noise
            continue;
        } else if (!wiener && gauss) {
            // |c| >= lambda sigma, the group DC always kept (bmndalgo.py:462-475)
            float thr = mul_rn(sp.ht_lambda, sig);
            att = (fabsf(X[e]) >= thr || e == 0) ? 1.0f : 0.0f;
        } else if (!wiener) {
            float thr = mul_rn(sp.ht_lambda, sig);
            att = ht_keep(fabsf(X[e]), thr, sp.count_scale, scale_f) ? 1.0f : 0.0f;
        } else if (gauss) {
            // |R|^2 / (|R|^2 + mu^2 max(sigma^2, 1e-8)) (wiener.py:50-69)
            float eff = mul_rn(sp.wiener_scale, fmaxf(nv, fmaxf(eps_f, 1e-8f)));
            float pr = fabsf(R[e]);
            pr = mul_rn(pr, pr);
            float den = add_rn(pr, eff);
            float gain = den > 0.0f ? div_rn(pr, den) : 0.0f;
            att = fminf(fmaxf(gain, 0.0f), 1.0f);
            spw = pr;
        } else {
            // signal power by gain mode (wiener.py:24-47)
            float eff = mul_rn(sp.wiener_scale, nv);
            float pr = fabsf(R[e]);
            pr = mul_rn(pr, pr);
            float spow = pr;
            if (sp.wiener_gain_mode != BMND_GAIN_CLASSIC) {
                spow = sub_rn(pr, sp.wiener_gain_mode == BMND_GAIN_NOISE_FLOOR ? nv : eff);
                if (spow < 0.0f) spow = 0.0f;
            }
            float gain = div_rn(spow, add_rn(add_rn(spow, eff), eps_f));
            att = fminf(fmaxf(gain, 0.0f), 1.0f);
            spw = spow;
        }
        X[e] = mul_rn(X[e], att);
        V[e] = att;
        float err = att * att;
        if (sp.weight_model != BMND_WEIGHT_CLASSIC) err *= nv;
        // exact risk weights: the noise of the first kk planes comes from the
        // exact pass below; their bias term stays (wiener.py:760-797)
        if (exact_risk && e < kk * P) err = 0.0f;
        if (sp.weight_model == BMND_WEIGHT_RISK) {
            const float rj = 1.0f - att;
            err += rj * rj * spw;
        }
        S[e] = err;
    }
    __syncthreads();

    // ---- exact noise risk of the first kk planes (wiener.py:638-711) ----
    // (stages with exact risk weights run the runtime-geometry instantiation,
    // so the specialised ones carry none of this code)
    double* riskp = sm<double>(smem, a.L.risk);
    if constexpr (ND == 0) {
        if (exact_risk) {
            const float* smt = a.st + static_cast<int64_t>(P) * kron_stride(P);
            const int jr = kron_jr(P);
            if (jr == 1) exact_risk_any<1>(lval, lstart, lent, U, GT, kpad, kk, a.st, smt, V, P, riskp);
            else if (jr == 2) exact_risk_any<2>(lval, lstart, lent, U, GT, kpad, kk, a.st, smt, V, P, riskp);
            else exact_risk_any<4>(lval, lstart, lent, U, GT, kpad, kk, a.st, smt, V, P, riskp);
        }
    }

    if (a.probe.active && a.probe.atten)
        for (int e = tid; e < total; e += blockDim.x) a.probe.atten[probe_base + e] = V[e];

    // Wiener sigma map: the group's mean coefficient sigma (bmndalgo.py:874-875),
    // summed per warp and then over warps in warp order
    if (a.sig_num && wiener) {
        float v = sig_sum;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if ((tid & 31) == 0) sm<float>(smem, a.L.scan)[tid >> 5] = v;
        __syncthreads();
        if (tid == 0) {
            float t = 0.0f;
            for (int w = 0; w < static_cast<int>(blockDim.x >> 5); ++w) t += sm<float>(smem, a.L.scan)[w];
            sm<float>(smem, a.L.misc)[12] = t / static_cast<float>(total);
        }
        __syncthreads();
    }

    // ---- aggregation weights (aggregationweights.py:213-259) ----
    // The reference sums the plane risks in float64.  Here the per-coefficient
    // products and sums are float32 (relative error ~P 2^-24 in a weight, far
    // inside the output tolerance): float64 arithmetic runs at a small
    // fraction of the FP32 rate on this GPU and dominated the filter's time.
    {
        const int warp = tid >> 5, lane = tid & 31, nwarps = blockDim.x >> 5;
        for (int g = warp; g < n; g += nwarps) {
            float risk = 0.0f;
            for (int j = lane; j < P; j += 32) {
                float err = S[g * P + j];
                if (sp.windowed_synthesis) err *= static_cast<float>(mdiag[j]);
                risk += err;
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) risk += __shfl_xor_sync(0xffffffffu, risk, o);
            if (lane == 0) plane[g] = static_cast<double>(risk);
        }
    }
    __syncthreads();
    if (tid < n) {
        float risk = 0.0f;
        if (exact_risk) {
            // one weight for the group: its exact risk in float64
            // (wiener.py:760-822, aggregationweights.py:656-676)
            double r = riskp[blockDim.x >> 5];
            for (int g = 0; g < n; ++g) r += plane[g];
            risk = static_cast<float>(r);
        } else if (sp.weight_group_scope) {
            // one weight for the whole group: the summed risk (the group
            // transforms are orthonormal, so the group metric is the identity)
            for (int g = 0; g < n; ++g) risk += static_cast<float>(plane[g]);
        } else {
            for (int g = 0; g < n; ++g) {
                const float gi = G[g * n + tid];  // Ginv[o, g] = G[g, o]
                risk = fmaf(gi * gi, static_cast<float>(plane[g]), risk);
            }
        }
        wts[tid] = (isfinite(risk) && risk >= 0.0f) ? 1.0f / (risk + static_cast<float>(sp.eps)) : 0.0f;
    }
    __syncthreads();

    // ---- group-mass conservation, second pass (poisson.py:161-265) ----
    if (a.den_ro) {
        float* dirv = sm<float>(smem, a.L.dir);  // [n] group axis, then [MAX_DIMS][MAX_EDGE] patch axes
        double* red = sm<double>(smem, a.L.plane);  // reduction scratch: 5 sums per warp
        // constant synthesis direction: per axis solve(inverse, 1) = forward 1
        // (G on the group axis, the forward spatial matrix on each patch axis)
        if (tid < n) {
            float sgv = 0.0f;
            for (int j = 0; j < n; ++j) sgv += G[tid * n + j];
            dirv[tid] = a.sp.group_transform == BMND_GROUP_NONE ? 1.0f : sgv;
        }
        if (tid >= 64 && tid < 64 + BMND_MAX_DIMS * BMND_MAX_EDGE) {
            const int d = (tid - 64) / BMND_MAX_EDGE, k = (tid - 64) % BMND_MAX_EDGE;
            float v = 0.0f;
            if (d < geo.nd() && k < geo.b(d))
                for (int m = 0; m < geo.b(d); ++m) v += Fw[d * BMND_MAX_EDGE * BMND_MAX_EDGE + k * geo.b(d) + m];
            dirv[BMND_MAX_STACK + d * BMND_MAX_EDGE + k] = v;
        }
        // output functional O = w_g win[p] / den (float32 arithmetic, as the
        // reference's gather), into S; the target sum(O x noisy) in float64
        double t_target = 0.0;
        for (int e = tid; e < total; e += blockDim.x) {
            const int g = e / P, p = e - g * P;
            const int64_t off = geo.offset(pos + g * BMND_MAX_DIMS, p, a.vstride);
            const float o = (wts[g] * win[p]) / static_cast<float>(a.den_ro[off]);
            S[e] = o;
            t_target += static_cast<double>(o) * static_cast<double>(__ldg(a.noisy + off));
        }
        __syncthreads();
        transform_group<ND, B0, B1, B2>(geo, a, smem, n, S, 3);  // coefficient functional F
        __syncthreads();
        float dmax_g = 0.0f, dmax_s = 1.0f;
        for (int g = 0; g < n; ++g) dmax_g = fmaxf(dmax_g, fabsf(dirv[g]));
        for (int d = 0; d < geo.nd(); ++d) {
            float m = 0.0f;
            for (int k = 0; k < geo.b(d); ++k) m = fmaxf(m, fabsf(dirv[BMND_MAX_STACK + d * BMND_MAX_EDGE + k]));
            dmax_s *= m;
        }
        const float dmax = dmax_g * dmax_s;
        auto dir_of = [&](int e) -> float {
            const int g = e / P;
            int p = e - g * P;
            float v = dirv[g];
#pragma unroll
            for (int d = BMND_MAX_DIMS - 1; d >= 0; --d) {
                if (d < geo.nd()) {
                    v *= dirv[BMND_MAX_STACK + d * BMND_MAX_EDGE + p % geo.b(d)];
                    p /= geo.b(d);
                }
            }
            return v / dmax;
        };
        double t_cur = 0.0, t_den = 0.0, t_resp = 0.0;
        float t_max = 0.0f;
        for (int e = tid; e < total; e += blockDim.x) {
            const double f = static_cast<double>(S[e]);
            t_cur += f * static_cast<double>(X[e]);
            t_den += f * f;
            t_resp += f * static_cast<double>(dir_of(e));
            t_max = fmaxf(t_max, fabsf(S[e]));
        }
        const int warp = tid >> 5, lane = tid & 31, nwarps = blockDim.x >> 5;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            t_target += __shfl_xor_sync(0xffffffffu, t_target, o);
            t_cur += __shfl_xor_sync(0xffffffffu, t_cur, o);
            t_den += __shfl_xor_sync(0xffffffffu, t_den, o);
            t_resp += __shfl_xor_sync(0xffffffffu, t_resp, o);
            t_max = fmaxf(t_max, __shfl_xor_sync(0xffffffffu, t_max, o));
        }
        __syncthreads();  // red aliases plane[], last read by the weights
        if (lane == 0) {
            red[warp * 5 + 0] = t_target;
            red[warp * 5 + 1] = t_cur;
            red[warp * 5 + 2] = t_den;
            red[warp * 5 + 3] = t_resp;
            red[warp * 5 + 4] = static_cast<double>(t_max);
        }
        __syncthreads();
        if (tid == 0) {
            double target = 0.0, cur = 0.0, fden = 0.0, resp = 0.0, fmx = 0.0;
            for (int w = 0; w < nwarps; ++w) {
                target += red[w * 5 + 0];
                cur += red[w * 5 + 1];
                fden += red[w * 5 + 2];
                resp += red[w * 5 + 3];
                fmx = fmax(fmx, red[w * 5 + 4]);
            }
            double corr = 0.0;
            bool ok = true;
            if (fden <= sp.eps) {
                // rescale a vanishing functional by its largest entry
                if (!(fmx > 0.0) || !isfinite(fmx)) ok = false;
                else {
                    target /= fmx;
                    cur /= fmx;
                    resp /= fmx;
                }
            }
            const double residual = target - cur;
            if (ok && residual != 0.0) {
                if (!(resp != 0.0) || !isfinite(resp)) ok = false;
                else corr = residual / resp;
            }
            if (!ok && a.err) atomicExch(a.err, 1);
            red[0] = ok ? corr : 0.0;
        }
        __syncthreads();
        const double corr = red[0];
        if (corr != 0.0)
            for (int e = tid; e < total; e += blockDim.x)
                X[e] = static_cast<float>(static_cast<double>(X[e]) + corr * static_cast<double>(dir_of(e)));
        __syncthreads();
    }

    // ---- inverse transform and scatter ----
    transform_group<ND, B0, B1, B2>(geo, a, smem, n, X, 1);
    if (a.probe.active) {
        if (a.probe.weights && tid < n) a.probe.weights[gid * static_cast<int64_t>(a.nmax) + tid] = wts[tid];
        if (a.probe.filt)
            for (int e = tid; e < total; e += blockDim.x) a.probe.filt[probe_base + e] = X[e];
        return;
    }
    if (a.store.store) {
        // deterministic aggregation: every member's weighted filtered patch
        // goes to the store row of its entry; the sums happen in aggregate.cu
        int* slot = sm<int>(smem, a.L.shl);  // free after the exact phase
        if (tid < n) {
            const int s = a.store.slot_of[gid * static_cast<int64_t>(sp.max_stack) + tid];
            slot[tid] = s;
            a.store.wstore[s] = wts[tid];
        }
        __syncthreads();
        for (int e = tid; e < total; e += blockDim.x) {
            const int g = e / P;
            const int p = e - g * P;
            a.store.store[static_cast<int64_t>(slot[g]) * a.store.row + p] = mul_rn(X[e], mul_rn(wts[g], win[p]));
        }
        return;
    }
    for (int e = tid; e < total; e += blockDim.x) {
        const int g = e / P;
        const int p = e - g * P;
        const int64_t off = geo.offset(pos + g * BMND_MAX_DIMS, p, a.vstride);
        float ww = mul_rn(wts[g], win[p]);
        atomicAdd(a.num + off, widen_f64(mul_rn(X[e], ww)));
        if (a.den_ro) continue;  // the re-aggregation pass adds to the numerator only
        atomicAdd(a.den + off, widen_f64(ww));
        if (a.sig_num) {
            // sigma map numerator (patchaggregation.py:229-294): per coefficient
            // (hard thresholding) or the group's mean (Wiener)
            const float sv = wiener ? sm<float>(smem, a.L.misc)[12] : SG[e];
            atomicAdd(a.sig_num + off, widen_f64(mul_rn(sv, ww)));
        }
    }
}

// S^T[p * stride + j] = S[j, p] with S = kron(F_0, ..., F_{nd-1}) built axis by
// axis in float32 (fl(fl(F0 * F1) * F2)), as the reference builds its spatial
// matrix (variance.py:744-755); columns j >= P of the padded rows are zero
__global__ void spatial_kron_kernel(BmndStageParams sp, int P, int stride, float* st) {
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < P * stride; idx += gridDim.x * blockDim.x) {
        const int p = idx / stride, j = idx % stride;
        if (j >= P) {
            st[idx] = 0.0f;
            continue;
        }
        int jd[BMND_MAX_DIMS], pd[BMND_MAX_DIMS];
        int rj = j, rp = p;
        for (int d = sp.ndim - 1; d >= 0; --d) {
            jd[d] = rj % sp.block[d];
            rj /= sp.block[d];
            pd[d] = rp % sp.block[d];
            rp /= sp.block[d];
        }
        float v = sp.spatial_fwd[0][jd[0] * sp.block[0] + pd[0]];
        for (int d = 1; d < sp.ndim; ++d) v = mul_rn(v, sp.spatial_fwd[d][jd[d] * sp.block[d] + pd[d]]);
        st[idx] = v;
    }
}

// risk metric SM = S_inv^T diag(w^2) S_inv of the windowed synthesis
// (variance.py:1546-1557): S_inv the Kronecker product of the inverse patch
// matrices (float32 products in axis order, variance.py:744-755), w^2 and
// w^2 S_inv rounded to float32 as the reference's, each entry summed in
// float64 and rounded once.  Row p at sm[p * stride], zero beyond column P.
__global__ void risk_metric_kernel(BmndStageParams sp, int P, int stride, float* sm) {
    auto synth = [&](int x, int c) {
        int xd[BMND_MAX_DIMS], cd[BMND_MAX_DIMS];
        for (int d = sp.ndim - 1; d >= 0; --d) {
            xd[d] = x % sp.block[d];
            x /= sp.block[d];
            cd[d] = c % sp.block[d];
            c /= sp.block[d];
        }
        float v = sp.spatial_inv[0][xd[0] * sp.block[0] + cd[0]];
        for (int d = 1; d < sp.ndim; ++d) v = mul_rn(v, sp.spatial_inv[d][xd[d] * sp.block[d] + cd[d]]);
        return v;
    };
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < P * stride; idx += gridDim.x * blockDim.x) {
        const int p = idx / stride, j = idx % stride;
        if (j >= P) {
            sm[idx] = 0.0f;
            continue;
        }
        double acc = 0.0;
        for (int x = 0; x < P; ++x) {
            const float w2 = mul_rn(sp.window[x], sp.window[x]);
            acc += static_cast<double>(synth(x, p)) * static_cast<double>(mul_rn(w2, synth(x, j)));
        }
        sm[idx] = static_cast<float>(acc);
    }
}

// every group size's group matrix, n = 1 .. BMND_MAX_STACK (group_table_offset)
__global__ void group_table_kernel(int kind, float* __restrict__ gtab) {
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < kGroupTableFloats; idx += gridDim.x * blockDim.x) {
        int n = 1;
        while (group_table_offset(n + 1) <= idx) ++n;
        const int e = idx - group_table_offset(n);
        gtab[idx] = group_entry(kind, n, e / n, e % n);
    }
}

__global__ void finalize_kernel(const double* __restrict__ num, const double* __restrict__ den,
                                const float* __restrict__ noisy, float* __restrict__ out,
                                int64_t n, float eps_f, int no_eps) {
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        float d = static_cast<float>(den[i]);
        // mass conservation divides without eps (bmndalgo.py:617-624)
        out[i] = d > 0.0f ? div_rn(static_cast<float>(num[i]), no_eps ? d : add_rn(d, eps_f)) : noisy[i];
    }
}

// sigma map = sigma_num / den where den > 0, else the global sigma
// (bmndalgo.py:1048-1057)
__global__ void finalize_sigma_kernel(const double* __restrict__ sig_num, const double* __restrict__ den,
                                      float global_sigma, float* __restrict__ out, int64_t n) {
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const float d = static_cast<float>(den[i]);
        out[i] = d > 0.0f ? div_rn(static_cast<float>(sig_num[i]), d) : global_sigma;
    }
}

}  // namespace

int64_t union_cells_bound(const BmndStageParams& sp) {
    int64_t u = 1;
    for (int d = 0; d < sp.ndim; ++d) {
        int counts = sp.shape[d] - sp.block[d] + 1;
        int span = 2 * sp.search_radius[d];
        if (span > counts - 1) span = counts - 1;
        u *= span + sp.block[d];
    }
    return u;
}

int64_t group_filter_smem_bytes(const BmndStageParams& sp) {
    int P = patch_volume(sp);
    int kmax = sp.variance_k < sp.max_stack ? sp.variance_k : sp.max_stack;
    if (kmax < 0) kmax = 0;
    return make_layout(sp, P, sp.max_stack, kmax, union_cells_bound(sp), true).total;
}

int32_t launch_group_filter(const BmndStageParams& sp, const float* noisy, const float* pilot,
                            const int32_t* sel, const int32_t* count, int64_t n_refs, double* num,
                            double* den, float* st, double* sig_num, cudaStream_t stream, const double* den_ro,
                            int* err, const GroupProbe* probe, const AggStore* store) {
    if (n_refs == 0) return BMND_OK;
    {
        const int P = patch_volume(sp);
        const int stride = kron_stride(P);
        spatial_kron_kernel<<<(P * stride + 255) / 256, 256, 0, stream>>>(sp, P, stride, st);
        BMND_LAUNCH_CHECK("spatial_kron_kernel");
        if (sp.exact_risk_weights) {
            risk_metric_kernel<<<(P * stride + 255) / 256, 256, 0, stream>>>(sp, P, stride,
                                                                            st + static_cast<int64_t>(P) * stride);
            BMND_LAUNCH_CHECK("risk_metric_kernel");
        }
        group_table_kernel<<<(kGroupTableFloats + 255) / 256, 256, 0, stream>>>(
            sp.group_transform, st + 2 * static_cast<int64_t>(P) * stride);
        BMND_LAUNCH_CHECK("group_table_kernel");
    }
    FilterArgs a{};
    a.st = st;
    a.sp = sp;
    a.P = patch_volume(sp);
    a.nmax = sp.max_stack;
    a.kmax = sp.variance_k < sp.max_stack ? sp.variance_k : sp.max_stack;
    if (a.kmax < 0) a.kmax = 0;
    int64_t s = 1;
    for (int d = sp.ndim - 1; d >= 0; --d) {
        a.vstride[d] = s;
        s *= sp.shape[d];
    }
    a.n_lins = 1;
    for (int d = 0; d < sp.ndim; ++d) {
        a.counts[d] = sp.shape[d] - sp.block[d] + 1;
        a.n_lins *= a.counts[d];
    }
    a.sig_num = sig_num;
    a.ucells_cap = union_cells_bound(sp);
    a.L = make_layout(sp, a.P, a.nmax, a.kmax, a.ucells_cap, sig_num != nullptr);
    a.noisy = noisy;
    a.pilot = pilot;
    a.sel = sel;
    a.count = count;
    a.n_refs = n_refs;
    a.num = num;
    a.den = den;
    a.den_ro = den_ro;
    a.err = err;
    if (probe) a.probe = *probe;
    if (store) {
        a.store = *store;
        if (sig_num || den_ro) return fail(BMND_ERR_INVALID_ARG, "the entry store excludes sigma maps and mass passes");
    }
    if (a.probe.active && den_ro) return fail(BMND_ERR_INVALID_ARG, "the group probe has no mass-conservation pass");
    if (a.L.total > 227 * 1024)
        return fail(BMND_ERR_UNSUPPORTED, "group filter shared memory exceeds 227 KB for this profile");
    if (n_refs > 0x7fffffffLL) return fail(BMND_ERR_UNSUPPORTED, "too many groups");
    auto run = [&](auto kernel, int threads) -> int32_t {
        // give shared memory only what the resident CTAs need, so the rest of
        // the unified L1 caches the Kronecker table and the volumes
        int per_sm = 0, sms = 0;
        if (int32_t rc = kernel_residency(reinterpret_cast<const void*>(kernel), threads,
                                          static_cast<size_t>(a.L.total), true, &per_sm, &sms))
            return rc;
        kernel<<<static_cast<unsigned>(n_refs), threads, a.L.total, stream>>>(a);
        BMND_LAUNCH_CHECK("group_filter_kernel");
        return BMND_OK;
    };
    // two 256-thread CTAs per SM: one CTA's barrier and serial phases are
    // covered by the other's work (a single 512-thread CTA per SM, which
    // leaves L1 room for the 5x5x5 Kronecker table, measured 16% slower)
    const int* b = sp.block;
    if (sp.exact_risk_weights) return run(group_filter_kernel<0, 0, 0, 0, kThreads>, kThreads);
    if (sp.ndim == 2 && b[0] == 8 && b[1] == 8) return run(group_filter_kernel<2, 8, 8, 1, kThreads>, kThreads);
    if (sp.ndim == 3 && b[0] == 4 && b[1] == 4 && b[2] == 4)
        return run(group_filter_kernel<3, 4, 4, 4, kThreads>, kThreads);
    if (sp.ndim == 3 && b[0] == 5 && b[1] == 5 && b[2] == 5)
        return run(group_filter_kernel<3, 5, 5, 5, kThreads>, kThreads);
    return run(group_filter_kernel<0, 0, 0, 0, kThreads>, kThreads);
}

int32_t launch_finalize_sigma(const BmndStageParams& sp, const double* sig_num, const double* den,
                              float global_sigma, float* out, cudaStream_t stream) {
    int64_t n = volume_voxels(sp);
    if (n == 0) return BMND_OK;
    int64_t blocks = (n + 255) / 256;
    if (blocks > 152 * 16) blocks = 152 * 16;
    finalize_sigma_kernel<<<static_cast<unsigned>(blocks), 256, 0, stream>>>(sig_num, den, global_sigma, out, n);
    BMND_LAUNCH_CHECK("finalize_sigma_kernel");
    return BMND_OK;
}

int32_t launch_finalize(const BmndStageParams& sp, const double* num, const double* den,
                        const float* noisy, float* out, cudaStream_t stream) {
    int64_t n = volume_voxels(sp);
    if (n == 0) return BMND_OK;
    int threads = 256;
    int64_t blocks = (n + threads - 1) / threads;
    if (blocks > 152 * 16) blocks = 152 * 16;
    finalize_kernel<<<static_cast<unsigned>(blocks), threads, 0, stream>>>(num, den, noisy, out, n,
                                                                            static_cast<float>(sp.eps),
                                                                            sp.mass_conserve ? 1 : 0);
    BMND_LAUNCH_CHECK("finalize_kernel");
    return BMND_OK;
}

}  // namespace bmnd
