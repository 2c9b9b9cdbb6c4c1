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
//      eps) (aggregationweights.py:213-259, :616-653);
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

constexpr int kThreads = 256;

struct Layout {
    // byte offsets into dynamic shared memory
    int64_t g, fw, fi, win, mdiag, pos, shf, x, t, v, s, r, a, ex, grid, lcoord, lmask, lval, scan,
        plane, wts, misc, total;
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
};

__host__ Layout make_layout(const BmndStageParams& sp, int P, int nmax, int kmax, int64_t ucells) {
    Layout L{};
    int64_t off = 0;
    auto take = [&](int64_t bytes) {
        int64_t o = off;
        off += (bytes + 15) & ~int64_t(15);
        return o;
    };
    int64_t np = static_cast<int64_t>(nmax) * P;
    L.g = take(4 * nmax * nmax);
    L.fw = take(4 * BMND_MAX_DIMS * BMND_MAX_EDGE * BMND_MAX_EDGE);
    L.fi = take(4 * BMND_MAX_DIMS * BMND_MAX_EDGE * BMND_MAX_EDGE);
    L.win = take(4 * P);
    L.mdiag = take(8 * P);
    L.pos = take(4 * nmax * BMND_MAX_DIMS);
    L.shf = take(4 * nmax * BMND_MAX_DIMS);
    L.x = take(4 * np);
    // t and v are adjacent: the occupancy grid reuses them once both are dead
    L.t = take(4 * np);
    L.v = take(4 * np);
    L.s = take(4 * np);
    L.r = take(sp.filter == BMND_FILTER_WIENER ? 4 * np : 0);
    L.a = take(4 * np);
    L.ex = take(4 * static_cast<int64_t>(kmax) * P);
    if (ucells * 4 <= 8 * np && kmax > 0) {
        L.grid = L.t;
    } else {
        L.grid = take(kmax > 0 ? 4 * ucells : 0);
    }
    int64_t umax = kmax > 0 ? (np < ucells ? np : ucells) : 0;
    L.lcoord = take(4 * umax);
    L.lmask = take(4 * umax);
    L.lval = take(4 * umax);
    L.scan = take(4 * (kThreads + 1));
    L.plane = take(8 * nmax);
    L.wts = take(4 * nmax);
    L.misc = take(64);
    L.total = off;
    return L;
}

template <typename T>
__device__ __forceinline__ T* sm(unsigned char* base, int64_t off) {
    return reinterpret_cast<T*>(base + off);
}

// out = M applied along `axis` of the (nd)-axis tensor `in` (smem), one fused
// multiply-add per term in k order; `square` uses fl(M*M), `transpose` uses M^T
__device__ void apply_axis(const float* in, float* out, const int* dims, int nd, int axis,
                           const float* M, int ld, bool square, bool transpose) {
    int m = dims[axis];
    int inner = 1, total = 1;
    for (int d = axis + 1; d < nd; ++d) inner *= dims[d];
    for (int d = 0; d < nd; ++d) total *= dims[d];
    for (int e = threadIdx.x; e < total; e += blockDim.x) {
        int t = e % inner;
        int rest = e / inner;
        int i = rest % m;
        int o = rest / m;
        const float* col = in + static_cast<int64_t>(o) * m * inner + t;
        float acc = 0.0f;
        for (int k = 0; k < m; ++k) {
            float mk = transpose ? M[k * ld + i] : M[i * ld + k];
            if (square) mk = mul_rn(mk, mk);
            acc = fmaf(mk, col[k * inner], acc);
        }
        out[e] = acc;
    }
    __syncthreads();
}

// separable transform of an (n, block...) group: src -> dst (src may equal
// dst).  The passes alternate between tmp and dst, starting with tmp, so no
// pass reads and writes the same buffer.  kind: 0 forward, 1 inverse,
// 2 squared forward.
__device__ void transform_group(const FilterArgs& a, unsigned char* smem, int n, float* src,
                                float* dst, float* tmp, int kind) {
    const BmndStageParams& sp = a.sp;
    int dims[BMND_MAX_DIMS + 1];
    dims[0] = n;
    for (int d = 0; d < sp.ndim; ++d) dims[1 + d] = sp.block[d];
    const int nd = sp.ndim + 1;
    const float* G = sm<float>(smem, a.L.g);
    const float* Fw = sm<float>(smem, a.L.fw);
    const float* Fi = sm<float>(smem, a.L.fi);
    const float* cur = src;
    float* bufs[2] = {tmp, dst};
    int which = 0;
    if (sp.group_transform != BMND_GROUP_NONE) {
        apply_axis(cur, bufs[which], dims, nd, 0, G, n, kind == 2, kind == 1);
        cur = bufs[which];
        which ^= 1;
    }
    for (int d = 0; d < sp.ndim; ++d) {
        const float* M = (kind == 1 ? Fi : Fw) + d * BMND_MAX_EDGE * BMND_MAX_EDGE;
        apply_axis(cur, bufs[which], dims, nd, d + 1, M, sp.block[d], kind == 2, false);
        cur = bufs[which];
        which ^= 1;
    }
    if (cur != dst) {
        int total = n * a.P;
        for (int e = threadIdx.x; e < total; e += blockDim.x) dst[e] = cur[e];
        __syncthreads();
    }
}

__device__ __forceinline__ float variance_of(float x, float scale_f, float floor_f) {
    float nn = x > 0.0f ? x : 0.0f;
    float v = mul_rn(scale_f, nn);
    return v > floor_f ? v : floor_f;
}

__device__ __forceinline__ bool ht_keep(float mag, float thr, double scale) {
    double cc = static_cast<double>(mag) / scale;
    double tc = static_cast<double>(thr) / scale;
    double cs = cc > tc ? cc : tc;
    if (cs < 1.0) cs = 1.0;
    double tol = 128.0 * 1.1920928955078125e-07 * cs;
    return cc > tc + tol;
}

__global__ void __launch_bounds__(kThreads) group_filter_kernel(FilterArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    const BmndStageParams& sp = a.sp;
    const int64_t gid = blockIdx.x;
    const int tid = threadIdx.x;
    const int P = a.P;
    const int ndim = sp.ndim;
    const int n = a.count[gid];
    if (n <= 0) return;
    const bool wiener = sp.filter == BMND_FILTER_WIENER;

    float* G = sm<float>(smem, a.L.g);
    float* Fw = sm<float>(smem, a.L.fw);
    float* Fi = sm<float>(smem, a.L.fi);
    float* win = sm<float>(smem, a.L.win);
    double* mdiag = sm<double>(smem, a.L.mdiag);
    int* pos = sm<int>(smem, a.L.pos);
    int* shf = sm<int>(smem, a.L.shf);
    float* X = sm<float>(smem, a.L.x);
    float* T = sm<float>(smem, a.L.t);
    float* V = sm<float>(smem, a.L.v);
    float* S = sm<float>(smem, a.L.s);
    float* R = sm<float>(smem, a.L.r);
    float* A = sm<float>(smem, a.L.a);
    float* EX = sm<float>(smem, a.L.ex);
    uint32_t* grid = sm<uint32_t>(smem, a.L.grid);
    uint32_t* lcoord = sm<uint32_t>(smem, a.L.lcoord);
    uint32_t* lmask = sm<uint32_t>(smem, a.L.lmask);
    float* lval = sm<float>(smem, a.L.lval);
    int* scan = sm<int>(smem, a.L.scan);
    double* plane = sm<double>(smem, a.L.plane);
    float* wts = sm<float>(smem, a.L.wts);
    int* misc = sm<int>(smem, a.L.misc);

    // ---- setup: positions, matrices, window ----
    if (tid < n) {
        int64_t rem = a.sel[gid * sp.max_stack + tid];
        for (int d = ndim - 1; d >= 0; --d) {
            pos[tid * BMND_MAX_DIMS + d] = static_cast<int>(rem % a.counts[d]);
            rem /= a.counts[d];
        }
    }
    for (int e = tid; e < n * n; e += blockDim.x) G[e] = group_entry(sp.group_transform, n, e / n, e % n);
    for (int e = tid; e < BMND_MAX_DIMS * BMND_MAX_EDGE * BMND_MAX_EDGE; e += blockDim.x) {
        Fw[e] = sp.spatial_fwd[e / (BMND_MAX_EDGE * BMND_MAX_EDGE)][e % (BMND_MAX_EDGE * BMND_MAX_EDGE)];
        Fi[e] = sp.spatial_inv[e / (BMND_MAX_EDGE * BMND_MAX_EDGE)][e % (BMND_MAX_EDGE * BMND_MAX_EDGE)];
    }
    for (int e = tid; e < P; e += blockDim.x) {
        win[e] = sp.window[e];
        mdiag[e] = sp.spatial_metric_diag[e];
    }
    __syncthreads();
    if (tid == 0) {
        // group origin (min over members) and shifted positions
        for (int d = 0; d < ndim; ++d) {
            int mn = pos[d];
            for (int g = 1; g < n; ++g) mn = min(mn, pos[g * BMND_MAX_DIMS + d]);
            int mx = 0;
            for (int g = 0; g < n; ++g) {
                int s = pos[g * BMND_MAX_DIMS + d] - mn;
                shf[g * BMND_MAX_DIMS + d] = s;
                mx = g == 0 ? s : max(mx, s);
            }
            misc[d] = mn;                  // origin
            misc[4 + d] = mx + sp.block[d];  // union extent
        }
    }
    __syncthreads();

    // ---- gather ----
    const float scale_f = static_cast<float>(sp.count_scale);
    const float floor_f = static_cast<float>(sp.variance_floor);
    const float* varsrc = wiener ? a.pilot : a.noisy;
    const int total = n * P;
    for (int e = tid; e < total; e += blockDim.x) {
        int g = e / P, p = e % P;
        int rem = p;
        int64_t off = 0;
        for (int d = ndim - 1; d >= 0; --d) {
            off += static_cast<int64_t>(pos[g * BMND_MAX_DIMS + d] + rem % sp.block[d]) * a.vstride[d];
            rem /= sp.block[d];
        }
        X[e] = __ldg(a.noisy + off);
        V[e] = variance_of(__ldg(varsrc + off), scale_f, floor_f);
        if (wiener) R[e] = __ldg(a.pilot + off);
    }
    __syncthreads();

    // ---- forward transforms ----
    transform_group(a, smem, n, X, X, T, 0);
    if (wiener) transform_group(a, smem, n, R, R, T, 0);

    // ---- noise standard deviation ----
    const int k = sp.variance_k;
    const int kk = k < n ? k : n;
    const bool need_approx = (k <= 0) || (kk < n);
    if (need_approx) {
        transform_group(a, smem, n, V, V, T, 2);
        for (int e = tid; e < total; e += blockDim.x) {
            float v = V[e];
            A[e] = sqrtf(v > 0.0f ? v : 0.0f);  // approximate sigma
        }
        __syncthreads();
    }
    if (kk > 0) {
        int ush[BMND_MAX_DIMS], org[BMND_MAX_DIMS];
        int64_t ucells = 1;
        for (int d = 0; d < ndim; ++d) {
            ush[d] = misc[4 + d];
            org[d] = misc[d];
            ucells *= ush[d];
        }
        for (int64_t c = tid; c < ucells; c += blockDim.x) grid[c] = 0u;
        __syncthreads();
        for (int e = tid; e < total; e += blockDim.x) {
            int g = e / P, p = e % P;
            int rem = p;
            int64_t cell = 0, mul = 1;
            for (int d = ndim - 1; d >= 0; --d) {
                cell += static_cast<int64_t>(shf[g * BMND_MAX_DIMS + d] + rem % sp.block[d]) * mul;
                mul *= ush[d];
                rem /= sp.block[d];
            }
            atomicOr(grid + cell, 1u << g);
        }
        __syncthreads();
        // compact occupied cells in ascending cell order (block-wide scan)
        int64_t per = (ucells + blockDim.x - 1) / blockDim.x;
        int64_t c0 = tid * per, c1 = min(ucells, c0 + per);
        int mine = 0;
        for (int64_t c = c0; c < c1; ++c) mine += grid[c] != 0u;
        scan[tid] = mine;
        __syncthreads();
        if (tid == 0) {
            int run = 0;
            for (int i = 0; i < static_cast<int>(blockDim.x); ++i) {
                int v = scan[i];
                scan[i] = run;
                run += v;
            }
            scan[blockDim.x] = run;
        }
        __syncthreads();
        int w = scan[tid];
        for (int64_t c = c0; c < c1; ++c) {
            uint32_t m = grid[c];
            if (!m) continue;
            int64_t rem = c;
            uint32_t packed = 0;
            int64_t vox = 0;
            int coords[BMND_MAX_DIMS];
            for (int d = ndim - 1; d >= 0; --d) {
                coords[d] = static_cast<int>(rem % ush[d]);
                rem /= ush[d];
            }
            for (int d = 0; d < ndim; ++d) {
                packed |= static_cast<uint32_t>(coords[d]) << (10 * d);
                vox += static_cast<int64_t>(coords[d] + org[d]) * a.vstride[d];
            }
            lcoord[w] = packed;
            lmask[w] = m;
            lval[w] = variance_of(__ldg(varsrc + vox), scale_f, floor_f);
            ++w;
        }
        __syncthreads();
        const int U = scan[blockDim.x];
        // one coefficient (plane i < kk, spatial j) per thread iteration
        for (int idx = tid; idx < kk * P; idx += blockDim.x) {
            int i = idx / P, j = idx % P;
            int jd[BMND_MAX_DIMS];
            {
                int rem = j;
                for (int d = ndim - 1; d >= 0; --d) {
                    jd[d] = rem % sp.block[d];
                    rem /= sp.block[d];
                }
            }
            float accv = 0.0f;
            for (int u = 0; u < U; ++u) {
                uint32_t m = lmask[u];
                uint32_t pc = lcoord[u];
                float c = 0.0f;
                while (m) {
                    int g = __ffs(m) - 1;
                    m &= m - 1;
                    // kron entry S[j, p] = fl(fl(F0 * F1) * F2), then fl(G * S)
                    float s = 1.0f;
                    for (int d = 0; d < ndim; ++d) {
                        int pd = static_cast<int>((pc >> (10 * d)) & 1023u) - shf[g * BMND_MAX_DIMS + d];
                        float f = Fw[d * BMND_MAX_EDGE * BMND_MAX_EDGE + jd[d] * sp.block[d] + pd];
                        s = d == 0 ? f : mul_rn(s, f);
                    }
                    c = add_rn(c, mul_rn(G[i * n + g], s));
                }
                accv = add_rn(accv, mul_rn(mul_rn(lval[u], c), c));
            }
            EX[idx] = sqrtf(accv > 0.0f ? accv : 0.0f);
        }
        __syncthreads();
    }
    // final sigma into S
    if (k <= 0) {
        for (int e = tid; e < total; e += blockDim.x) S[e] = A[e];
    } else if (kk == n) {
        for (int e = tid; e < total; e += blockDim.x) S[e] = EX[e];
    } else {
        for (int j = tid; j < P; j += blockDim.x) {
            float sum_a = 0.0f, sum_e = 0.0f, rem_a = 0.0f;
            for (int i = 0; i < n; ++i) {
                float s = fmaxf(A[i * P + j], 0.0f);
                sum_a = add_rn(sum_a, mul_rn(s, s));
            }
            for (int i = 0; i < kk; ++i) {
                float s = fmaxf(EX[i * P + j], 0.0f);
                sum_e = add_rn(sum_e, mul_rn(s, s));
            }
            for (int i = kk; i < n; ++i) {
                float s = fmaxf(A[i * P + j], 0.0f);
                rem_a = add_rn(rem_a, mul_rn(s, s));
            }
            float target = sub_rn(sum_a, sum_e);
            if (target < 0.0f) target = 0.0f;
            float scl = rem_a > 0.0f ? div_rn(target, rem_a) : 0.0f;
            for (int i = 0; i < n; ++i) {
                float v;
                if (i < kk) {
                    float s = fmaxf(EX[i * P + j], 0.0f);
                    v = mul_rn(s, s);
                } else if (rem_a > 0.0f) {
                    float s = fmaxf(A[i * P + j], 0.0f);
                    v = mul_rn(mul_rn(s, s), scl);
                } else {
                    v = div_rn(target, static_cast<float>(n - kk));
                }
                S[i * P + j] = sqrtf(v > 0.0f ? v : 0.0f);
            }
        }
    }
    __syncthreads();

    // ---- shrinkage: attenuation into A, noise variance into S ----
    const float eps_f = static_cast<float>(sp.eps);
    for (int e = tid; e < total; e += blockDim.x) {
        float sig = S[e];
        float nv = mul_rn(sig, sig);
        float att;
        if (!wiener) {
            float thr = mul_rn(sp.ht_lambda, sig);
            att = ht_keep(fabsf(X[e]), thr, sp.count_scale) ? 1.0f : 0.0f;
        } else {
            float eff = mul_rn(sp.wiener_scale, nv);
            float pr = fabsf(R[e]);
            pr = mul_rn(pr, pr);
            float spow = sub_rn(pr, eff);
            if (spow < 0.0f) spow = 0.0f;
            float gain = div_rn(spow, add_rn(add_rn(spow, eff), eps_f));
            att = fminf(fmaxf(gain, 0.0f), 1.0f);
        }
        X[e] = mul_rn(X[e], att);
        A[e] = att;
        S[e] = nv;
    }
    __syncthreads();

    // ---- aggregation weights (float64, aggregationweights.py:213-259) ----
    {
        const int warp = tid >> 5, lane = tid & 31, nwarps = blockDim.x >> 5;
        for (int g = warp; g < n; g += nwarps) {
            double risk = 0.0;
            for (int j = lane; j < P; j += 32) {
                double at = static_cast<double>(A[g * P + j]);
                double err = at * at;
                if (sp.weight_model != BMND_WEIGHT_CLASSIC) err *= static_cast<double>(S[g * P + j]);
                if (sp.windowed_synthesis) err *= mdiag[j];
                risk += err;
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) risk += __shfl_xor_sync(0xffffffffu, risk, o);
            if (lane == 0) plane[g] = risk;
        }
    }
    __syncthreads();
    if (tid < n) {
        double risk = 0.0;
        for (int g = 0; g < n; ++g) {
            double gi = static_cast<double>(G[g * n + tid]);  // Ginv[o, g] = G[g, o]
            risk += (gi * gi) * plane[g];
        }
        wts[tid] = (isfinite(risk) && risk >= 0.0) ? static_cast<float>(1.0 / (risk + sp.eps)) : 0.0f;
    }
    __syncthreads();

    // ---- inverse transform and scatter ----
    transform_group(a, smem, n, X, X, T, 1);
    for (int e = tid; e < total; e += blockDim.x) {
        int g = e / P, p = e % P;
        int rem = p;
        int64_t off = 0;
        for (int d = ndim - 1; d >= 0; --d) {
            off += static_cast<int64_t>(pos[g * BMND_MAX_DIMS + d] + rem % sp.block[d]) * a.vstride[d];
            rem /= sp.block[d];
        }
        float ww = mul_rn(wts[g], win[p]);
        atomicAdd(a.num + off, static_cast<double>(mul_rn(X[e], ww)));
        atomicAdd(a.den + off, static_cast<double>(ww));
    }
}

__global__ void finalize_kernel(const double* __restrict__ num, const double* __restrict__ den,
                                const float* __restrict__ noisy, float* __restrict__ out,
                                int64_t n, float eps_f) {
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        float d = static_cast<float>(den[i]);
        out[i] = d > 0.0f ? div_rn(static_cast<float>(num[i]), add_rn(d, eps_f)) : noisy[i];
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
    return make_layout(sp, P, sp.max_stack, kmax, union_cells_bound(sp)).total;
}

int32_t launch_group_filter(const BmndStageParams& sp, const float* noisy, const float* pilot,
                            const int32_t* sel, const int32_t* count, int64_t n_refs, double* num,
                            double* den, cudaStream_t stream) {
    if (n_refs == 0) return BMND_OK;
    FilterArgs a{};
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
    for (int d = 0; d < sp.ndim; ++d) a.counts[d] = sp.shape[d] - sp.block[d] + 1;
    a.L = make_layout(sp, a.P, a.nmax, a.kmax, union_cells_bound(sp));
    a.noisy = noisy;
    a.pilot = pilot;
    a.sel = sel;
    a.count = count;
    a.n_refs = n_refs;
    a.num = num;
    a.den = den;
    if (a.L.total > 227 * 1024)
        return fail(BMND_ERR_UNSUPPORTED, "group filter shared memory exceeds 227 KB for this profile");
    if (n_refs > 0x7fffffffLL) return fail(BMND_ERR_UNSUPPORTED, "too many groups");
    BMND_CUDA_TRY(cudaFuncSetAttribute(group_filter_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(a.L.total)));
    group_filter_kernel<<<static_cast<unsigned>(n_refs), kThreads, a.L.total, stream>>>(a);
    BMND_LAUNCH_CHECK("group_filter_kernel");
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
                                                                            static_cast<float>(sp.eps));
    BMND_LAUNCH_CHECK("finalize_kernel");
    return BMND_OK;
}

}  // namespace bmnd
