// pilotnet.cu -- learned stage-1 pilot: a residual convolution net in the
// Anscombe domain.  This part has no counterpart in the reference; it stands in
// for the hard-thresholding basic estimate on the fast path.
//
//   a   = 2 sqrt(max(x, 0) + 3/8)                   variance-stabilised input
//   h_1 = relu(W_0 * a + b_0)                       1 -> C channels
//   h_l = relu(W_{l-1} * h_{l-1} + b_{l-1})         C -> C, l = 2 .. L-1
//   y   = a + W_{L-1} * h_{L-1} + b_{L-1}           C -> 1, residual
//   pilot = max((y / 2)^2 - 3/8, 0)
//
// 3x3 (2-D) or 3x3x3 (3-D) kernels with zero padding, over a batch of
// volumes.  Weights and hidden activations are BF16; every sum accumulates in
// FP32.  Parameters are kept as an FP32 master copy, flat, layer by layer:
// W_l[tap][ci][co] then b_l[co].
//
// The C -> C layers run on the tensor cores as an implicit GEMM
// (mma.sync m16n8k16, BF16 in, FP32 accumulate): a persistent CTA keeps the
// layer's weights in shared memory, pre-arranged in B-fragment order, and
// walks output tiles of 256 voxels (16 rows of 16 along x).  Each tile's input
// with its one-voxel halo is staged channels-last with rows padded to C + 8
// elements, so the ldmatrix reads of the A fragments are bank-conflict free.
// The same kernel computes a layer's data gradient with the weights flipped
// and transposed and the layer input's ReLU mask in the epilogue.  The
// one-channel layers, the weight gradients and the optimiser run on the CUDA
// cores.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <type_traits>
#include <vector>

#include "bmnd_common.cuh"
#include "tc_common.cuh"

namespace bmnd {
namespace {

typedef __nv_bfloat16 bf16;

struct NetGeo {
    int nb, D, H, W;  // batch, depth (1 in 2-D), height, width
    __host__ __device__ int64_t voxels() const { return static_cast<int64_t>(nb) * D * H * W; }
};

template <int ND>
struct Tile {
    static constexpr int taps = ND == 3 ? 27 : 9;
    static constexpr int tx = 16;                    // voxels per row (one m16 fragment)
    static constexpr int ty = ND == 3 ? 8 : 16;
    static constexpr int tz = ND == 3 ? 2 : 1;       // ty * tz = 16 rows, 256 voxels
    static constexpr int hx = tx + 2, hy = ty + 2, hz = ND == 3 ? tz + 2 : 1;
    static constexpr int halo = hx * hy * hz;
};

// tap t -> offsets (dz, dy, dx) in {-1, 0, 1} (dz = 0 in 2-D), C order, so
// tap taps-1-t has the opposite offsets
template <int ND>
__host__ __device__ __forceinline__ void tap_offsets(int t, int& dz, int& dy, int& dx) {
    if (ND == 3) {
        dz = t / 9 - 1;
        dy = (t / 3) % 3 - 1;
        dx = t % 3 - 1;
    } else {
        dz = 0;
        dy = t / 3 - 1;
        dx = t % 3 - 1;
    }
}

__device__ __forceinline__ int64_t vox_index(const NetGeo& g, int b, int z, int y, int x) {
    return ((static_cast<int64_t>(b) * g.D + z) * g.H + y) * g.W + x;
}

// Hidden activations and their gradients are stored chunk-planar,
// [C / 8][voxel][8 channels]: one 8-channel chunk of a row of voxels is
// contiguous, so a halo row arrives as one TMA row of 16 * hx bytes.
// One-channel tensors (the Anscombe input, the output) are plain [voxel].
template <int CH>
__host__ __device__ __forceinline__ int64_t hid(int64_t v, int c, int64_t nv) {
    return CH < 8 ? v * CH + c : (static_cast<int64_t>(c >> 3) * nv + v) * 8 + (c & 7);
}

__device__ __forceinline__ void vox_decode(const NetGeo& g, int64_t v, int& b, int& z, int& y, int& x) {
    x = static_cast<int>(v % g.W);
    v /= g.W;
    y = static_cast<int>(v % g.H);
    v /= g.H;
    z = static_cast<int>(v % g.D);
    b = static_cast<int>(v / g.D);
}

__device__ __forceinline__ float anscombe(float x) { return 2.0f * sqrtf(fmaxf(x, 0.0f) + 0.375f); }

// ---------------------------------------------------------------------------
// element-wise and one-channel layers (CUDA cores)
// ---------------------------------------------------------------------------
__global__ void anscombe_kernel(const float* __restrict__ x, float* __restrict__ a, int64_t n) {
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x)
        a[i] = anscombe(x[i]);
}

// h[v][c] = relu(b[c] + sum_t w[t][c] a[v + off(t)]), C channels, 16-byte stores.
// A thread computes two voxels (x and x + 1) so each pair of 16-byte weight
// loads from shared memory feeds 16 multiply-adds.
template <int ND, int C>
__global__ void conv_in_kernel(const float* __restrict__ a, const float* __restrict__ w,
                               const float* __restrict__ bias, bf16* __restrict__ h, NetGeo g) {
    constexpr int T = Tile<ND>::taps;
    __shared__ __align__(16) float ws[T * C];
    __shared__ __align__(16) float bs[C];
    for (int i = threadIdx.x; i < T * C; i += blockDim.x) ws[i] = w[i];
    for (int i = threadIdx.x; i < C; i += blockDim.x) bs[i] = bias[i];
    __syncthreads();
    const int wp = (g.W + 1) / 2;  // voxel pairs per row
    const int64_t nv = g.voxels();
    const int64_t npair = static_cast<int64_t>(g.nb) * g.D * g.H * wp;
    for (int64_t q = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; q < npair;
         q += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        int64_t r = q;
        const int x = static_cast<int>(r % wp) * 2;
        r /= wp;
        const int y = static_cast<int>(r % g.H);
        r /= g.H;
        const int z = static_cast<int>(r % g.D);
        const int b = static_cast<int>(r / g.D);
        const bool two = x + 1 < g.W;
        float in0[T], in1[T];
#pragma unroll
        for (int t = 0; t < T; ++t) {
            int dz, dy, dx;
            tap_offsets<ND>(t, dz, dy, dx);
            const int zz = z + dz, yy = y + dy, xa = x + dx, xb = x + 1 + dx;
            const bool row = zz >= 0 && zz < g.D && yy >= 0 && yy < g.H;
            in0[t] = (row && xa >= 0 && xa < g.W) ? a[vox_index(g, b, zz, yy, xa)] : 0.0f;
            in1[t] = (row && xb >= 0 && xb < g.W) ? a[vox_index(g, b, zz, yy, xb)] : 0.0f;
        }
        const int64_t v0 = vox_index(g, b, z, y, x);
#pragma unroll
        for (int c0 = 0; c0 < C; c0 += 8) {
            float acc0[8], acc1[8];
            {
                const float4 b0 = *reinterpret_cast<const float4*>(bs + c0);
                const float4 b1 = *reinterpret_cast<const float4*>(bs + c0 + 4);
                const float bb[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
                for (int j = 0; j < 8; ++j) acc0[j] = acc1[j] = bb[j];
            }
#pragma unroll
            for (int t = 0; t < T; ++t) {
                const float4 w0 = *reinterpret_cast<const float4*>(ws + t * C + c0);
                const float4 w1 = *reinterpret_cast<const float4*>(ws + t * C + c0 + 4);
                const float ww[8] = {w0.x, w0.y, w0.z, w0.w, w1.x, w1.y, w1.z, w1.w};
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    acc0[j] = fmaf(ww[j], in0[t], acc0[j]);
                    acc1[j] = fmaf(ww[j], in1[t], acc1[j]);
                }
            }
            __align__(16) bf16 o[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) o[j] = __float2bfloat16_rn(fmaxf(acc0[j], 0.0f));
            *reinterpret_cast<uint4*>(h + hid<C>(v0, c0, nv)) = *reinterpret_cast<const uint4*>(o);
            if (two) {
#pragma unroll
                for (int j = 0; j < 8; ++j) o[j] = __float2bfloat16_rn(fmaxf(acc1[j], 0.0f));
                *reinterpret_cast<uint4*>(h + hid<C>(v0 + 1, c0, nv)) = *reinterpret_cast<const uint4*>(o);
            }
        }
    }
}

// y[v] = a[v] + b + sum_t sum_c w[t][c] h[v + off(t)][c]; pilot = inverse
// Anscombe.  A CTA of 16 x 8 threads walks OutZ planes of a 16 x 8 tile; the
// three input planes it needs (tile plus one-voxel halo, channels padded to
// C + 8 so the 16-byte reads are free of bank conflicts) rotate through
// shared memory, so every input voxel is read from global memory about once.
template <int ND>
struct OutTile {
    static constexpr int tx = 16, ty = 8, hx = tx + 2, hy = ty + 2;
    static constexpr int planes = ND == 3 ? 3 : 1;
    static constexpr int zb = ND == 3 ? 8 : 1;  // output planes per CTA
};

template <int ND, int C>
__global__ void __launch_bounds__(128) conv_out_kernel(const bf16* __restrict__ h, const float* __restrict__ w,
                                                       const float* __restrict__ bias, const float* __restrict__ a,
                                                       float* __restrict__ y, float* __restrict__ pilot, NetGeo g) {
    using OT = OutTile<ND>;
    constexpr int T = Tile<ND>::taps;
    constexpr int CP = C + 8;
    constexpr int HV = OT::hx * OT::hy;
    constexpr int CH = C / 8;
    extern __shared__ __align__(16) unsigned char out_smem[];
    float* ws = reinterpret_cast<float*>(out_smem);
    bf16* ring = reinterpret_cast<bf16*>(out_smem + static_cast<size_t>(T) * C * 4);
    for (int i = threadIdx.x; i < T * C; i += blockDim.x) ws[i] = w[i];
    const float b0 = bias[0];
    const int64_t nv = g.voxels();
    const int tiles_x = (g.W + OT::tx - 1) / OT::tx;
    const int tiles_y = (g.H + OT::ty - 1) / OT::ty;
    const int zblocks = (g.D + OT::zb - 1) / OT::zb;
    int64_t r = blockIdx.x;
    const int x0 = static_cast<int>(r % tiles_x) * OT::tx;
    r /= tiles_x;
    const int y0 = static_cast<int>(r % tiles_y) * OT::ty;
    r /= tiles_y;
    const int zs = static_cast<int>(r % zblocks) * OT::zb;
    const int b = static_cast<int>(r / zblocks);
    const int ze = min(zs + OT::zb, g.D);
    auto load_plane = [&](int zz, int slot) {
        bf16* dst = ring + static_cast<size_t>(slot) * HV * CP;
        for (int i = threadIdx.x; i < HV * CH; i += blockDim.x) {
            const int ch = i / HV, hv = i - ch * HV;  // chunk-major: a warp reads consecutive voxels
            const int xx = x0 - 1 + hv % OT::hx, yy = y0 - 1 + hv / OT::hx;
            uint4 v = make_uint4(0u, 0u, 0u, 0u);
            if (zz >= 0 && zz < g.D && yy >= 0 && yy < g.H && xx >= 0 && xx < g.W)
                v = *reinterpret_cast<const uint4*>(h + hid<C>(vox_index(g, b, zz, yy, xx), ch * 8, nv));
            *reinterpret_cast<uint4*>(dst + static_cast<size_t>(hv) * CP + ch * 8) = v;
        }
    };
    const int tx = threadIdx.x % OT::tx, ty = threadIdx.x / OT::tx;
    if (ND == 3) {
        load_plane(zs - 1, (zs + 2) % 3);
        load_plane(zs, zs % 3);
    }
    for (int z = zs; z < ze; ++z) {
        if (ND == 3) load_plane(z + 1, (z + 1) % 3);
        else load_plane(z, 0);
        __syncthreads();
        const int xx = x0 + tx, yy = y0 + ty;
        if (xx < g.W && yy < g.H) {
            float acc[8] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};  // eight independent chains
#pragma unroll 1
            for (int t = 0; t < T; ++t) {
                int dz, dy, dx;
                tap_offsets<ND>(t, dz, dy, dx);
                const int slot = ND == 3 ? (z + dz + 3) % 3 : 0;
                const bf16* hv = ring + (static_cast<size_t>(slot) * HV + (ty + 1 + dy) * OT::hx + (tx + 1 + dx)) * CP;
#pragma unroll
                for (int c0 = 0; c0 < C; c0 += 8) {
                    const uint4 raw = *reinterpret_cast<const uint4*>(hv + c0);
                    const bf16* e = reinterpret_cast<const bf16*>(&raw);
                    const float4 w0 = *reinterpret_cast<const float4*>(ws + t * C + c0);
                    const float4 w1 = *reinterpret_cast<const float4*>(ws + t * C + c0 + 4);
                    acc[0] = fmaf(w0.x, __bfloat162float(e[0]), acc[0]);
                    acc[1] = fmaf(w0.y, __bfloat162float(e[1]), acc[1]);
                    acc[2] = fmaf(w0.z, __bfloat162float(e[2]), acc[2]);
                    acc[3] = fmaf(w0.w, __bfloat162float(e[3]), acc[3]);
                    acc[4] = fmaf(w1.x, __bfloat162float(e[4]), acc[4]);
                    acc[5] = fmaf(w1.y, __bfloat162float(e[5]), acc[5]);
                    acc[6] = fmaf(w1.z, __bfloat162float(e[6]), acc[6]);
                    acc[7] = fmaf(w1.w, __bfloat162float(e[7]), acc[7]);
                }
            }
            const float sum = ((acc[0] + acc[1]) + (acc[2] + acc[3])) + ((acc[4] + acc[5]) + (acc[6] + acc[7]));
            const int64_t v = vox_index(g, b, z, yy, xx);
            const float yv = a[v] + (b0 + sum);
            if (y) y[v] = yv;
            if (pilot) {
                const float hh = 0.5f * yv;
                pilot[v] = fmaxf(hh * hh - 0.375f, 0.0f);
            }
        }
        __syncthreads();
    }
}

template <int ND, int C>
constexpr size_t out_smem_bytes() {
    return static_cast<size_t>(Tile<ND>::taps) * C * 4 +
           static_cast<size_t>(OutTile<ND>::planes) * OutTile<ND>::hx * OutTile<ND>::hy * (C + 8) * 2;
}

// loss = mean (y - anscombe(target))^2 and its gradient with respect to y
__global__ void loss_grad_kernel(const float* __restrict__ y, const float* __restrict__ target,
                                 float* __restrict__ gy, int64_t n, double* __restrict__ loss) {
    __shared__ double red[32];
    double local = 0.0;
    const float scale = 2.0f / static_cast<float>(n);
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const float d = y[i] - anscombe(target[i]);
        gy[i] = scale * d;
        local += static_cast<double>(d) * d;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) local += __shfl_xor_sync(0xffffffffu, local, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = local;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int i = 0; i < static_cast<int>(blockDim.x >> 5); ++i) s += red[i];
        atomicAdd(loss, s / static_cast<double>(n));
    }
}

// data gradient of the last layer: gh[u][c] = (h[u][c] > 0) sum_t w[t][c] gy[u - off(t)]
template <int ND, int C>
__global__ void conv_out_dgrad_kernel(const float* __restrict__ gy, const float* __restrict__ w,
                                      const bf16* __restrict__ h, bf16* __restrict__ gh, NetGeo g) {
    constexpr int T = Tile<ND>::taps;
    __shared__ float ws[T * C];
    for (int i = threadIdx.x; i < T * C; i += blockDim.x) ws[i] = w[i];
    __syncthreads();
    const int64_t n = g.voxels();
    for (int64_t u = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; u < n;
         u += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        int b, z, y, x;
        vox_decode(g, u, b, z, y, x);
        float gv[T];
#pragma unroll
        for (int t = 0; t < T; ++t) {
            int dz, dy, dx;
            tap_offsets<ND>(t, dz, dy, dx);
            const int zz = z - dz, yy = y - dy, xx = x - dx;
            const bool inside = zz >= 0 && zz < g.D && yy >= 0 && yy < g.H && xx >= 0 && xx < g.W;
            gv[t] = inside ? gy[vox_index(g, b, zz, yy, xx)] : 0.0f;
        }
#pragma unroll
        for (int c0 = 0; c0 < C; c0 += 8) {
            const uint4 raw = *reinterpret_cast<const uint4*>(h + hid<C>(u, c0, n));
            const bf16* hm = reinterpret_cast<const bf16*>(&raw);
            float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
            for (int t = 0; t < T; ++t)
#pragma unroll
                for (int j = 0; j < 8; ++j) acc[j] = fmaf(ws[t * C + c0 + j], gv[t], acc[j]);
            __align__(16) bf16 o[8];
#pragma unroll
            for (int j = 0; j < 8; ++j)
                o[j] = __float2bfloat16_rn(__bfloat162float(hm[j]) > 0.0f ? acc[j] : 0.0f);
            *reinterpret_cast<uint4*>(gh + hid<C>(u, c0, n)) = *reinterpret_cast<const uint4*>(o);
        }
    }
}

// ---------------------------------------------------------------------------
// C -> C layers on the tensor cores
// ---------------------------------------------------------------------------
__device__ __forceinline__ void ldmatrix_x4(uint32_t addr, uint32_t& r0, uint32_t& r1, uint32_t& r2,
                                            uint32_t& r3) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0, %1, %2, %3}, [%4];\n"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                 : "r"(addr));
}

__device__ __forceinline__ void mma_bf16(float (&c)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                         uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, "
        "{%8, %9}, {%0, %1, %2, %3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

template <int ND, int C>
struct MidSmem {
    static constexpr int taps = Tile<ND>::taps;
    static constexpr int kc = C / 16, nt = C / 8, cp = C + 8;
    static constexpr size_t wfrag = static_cast<size_t>(taps) * kc * nt * 32;  // uint2 per lane
    static constexpr size_t wbytes = wfrag * 8;
    static constexpr size_t tbytes = static_cast<size_t>(Tile<ND>::halo) * cp * 2;
    static constexpr size_t bytes = wbytes + tbytes;
};

// B fragment of mma.m16n8k16 (k16 x n8, "col"): lane (g = lane / 4, q = lane % 4)
// holds B[2q][g], B[2q+1][g] in x and B[2q+8][g], B[2q+9][g] in y.  Forward:
// B[k][n] = W[t][ci = k][co = n]; data gradient: the layer applied backwards,
// B[k][n] = W[taps-1-t][ci = n][co = k].
template <int ND, int C>
__global__ void pack_mid_kernel(const float* __restrict__ W, uint2* __restrict__ out, int backward) {
    using S = MidSmem<ND, C>;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < static_cast<int64_t>(S::wfrag);
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int lane = static_cast<int>(i % 32);
        int64_t r = i / 32;
        const int nt = static_cast<int>(r % S::nt);
        r /= S::nt;
        const int kc = static_cast<int>(r % S::kc);
        const int t = static_cast<int>(r / S::kc);
        const int n = nt * 8 + lane / 4;
        const int k0 = kc * 16 + 2 * (lane % 4);
        auto B = [&](int k) -> float {
            return backward ? W[(static_cast<int64_t>(S::taps - 1 - t) * C + n) * C + k]
                            : W[(static_cast<int64_t>(t) * C + k) * C + n];
        };
        auto pack2 = [](float lo, float hi) -> uint32_t {
            const uint16_t l = __bfloat16_as_ushort(__float2bfloat16_rn(lo));
            const uint16_t h = __bfloat16_as_ushort(__float2bfloat16_rn(hi));
            return static_cast<uint32_t>(l) | (static_cast<uint32_t>(h) << 16);
        };
        out[i] = make_uint2(pack2(B(k0), B(k0 + 1)), pack2(B(k0 + 8), B(k0 + 9)));
    }
}

// out[v][co] = epi(sum_t sum_ci in[v + off(t)][ci] B_t[ci][co]) with
// epi = relu(. + bias) (forward) or (mask[v][co] > 0 ? . : 0) (data gradient)
template <int ND, int C>
__global__ void __launch_bounds__(256, 1) conv_mid_kernel(const bf16* __restrict__ in, const uint2* __restrict__ wpk,
                                                          const float* __restrict__ bias, const bf16* __restrict__ mask,
                                                          bf16* __restrict__ out, NetGeo g) {
    using TL = Tile<ND>;
    using S = MidSmem<ND, C>;
    extern __shared__ __align__(16) unsigned char smem[];
    uint2* wsm = reinterpret_cast<uint2*>(smem);
    bf16* tile = reinterpret_cast<bf16*>(smem + S::wbytes);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    for (int i = tid; i < static_cast<int>(S::wfrag); i += blockDim.x) wsm[i] = wpk[i];

    const int tiles_x = (g.W + TL::tx - 1) / TL::tx;
    const int tiles_y = (g.H + TL::ty - 1) / TL::ty;
    const int tiles_z = (g.D + TL::tz - 1) / TL::tz;
    const int64_t ntiles = static_cast<int64_t>(tiles_x) * tiles_y * tiles_z * g.nb;
    constexpr int chunks = C / 8;  // 16-byte chunks per voxel
    const int64_t nv = g.voxels();
    const uint32_t tile_base = static_cast<uint32_t>(__cvta_generic_to_shared(tile));

    for (int64_t tl = blockIdx.x; tl < ntiles; tl += gridDim.x) {
        int64_t r = tl;
        const int x0 = static_cast<int>(r % tiles_x) * TL::tx;
        r /= tiles_x;
        const int y0 = static_cast<int>(r % tiles_y) * TL::ty;
        r /= tiles_y;
        const int z0 = static_cast<int>(r % tiles_z) * TL::tz;
        const int b = static_cast<int>(r / tiles_z);
        __syncthreads();  // the previous tile is no longer read (and the weights are in place)
        for (int i = tid; i < TL::halo * chunks; i += blockDim.x) {
            const int ch = i / TL::halo, vox = i - ch * TL::halo;  // chunk-major: coalesced reads
            const int hxi = vox % TL::hx, hyi = (vox / TL::hx) % TL::hy, hzi = vox / (TL::hx * TL::hy);
            const int xx = x0 + hxi - 1, yy = y0 + hyi - 1, zz = ND == 3 ? z0 + hzi - 1 : z0;
            uint4 v = make_uint4(0u, 0u, 0u, 0u);
            if (xx >= 0 && xx < g.W && yy >= 0 && yy < g.H && zz >= 0 && zz < g.D)
                v = *reinterpret_cast<const uint4*>(in + hid<C>(vox_index(g, b, zz, yy, xx), ch * 8, nv));
            *reinterpret_cast<uint4*>(tile + static_cast<size_t>(vox) * S::cp + ch * 8) = v;
        }
        __syncthreads();

        float acc[2][S::nt][4];
#pragma unroll
        for (int i = 0; i < 2; ++i)
#pragma unroll
            for (int n = 0; n < S::nt; ++n)
#pragma unroll
                for (int q = 0; q < 4; ++q) acc[i][n][q] = 0.0f;
        int rz[2], ry[2];
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            const int row = 2 * warp + i;
            rz[i] = row / TL::ty;
            ry[i] = row % TL::ty;
        }
#pragma unroll 1
        for (int t = 0; t < S::taps; ++t) {
            int dz, dy, dx;
            tap_offsets<ND>(t, dz, dy, dx);
            uint32_t rowaddr[2];
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                const int hzi = ND == 3 ? rz[i] + dz + 1 : 0;
                const int vox = (hzi * TL::hy + ry[i] + dy + 1) * TL::hx + (lane & 15) + dx + 1;
                rowaddr[i] = tile_base + static_cast<uint32_t>((vox * S::cp + (lane >> 4) * 8) * 2);
            }
#pragma unroll
            for (int kc = 0; kc < S::kc; ++kc) {
                uint2 bf[S::nt];
#pragma unroll
                for (int n = 0; n < S::nt; ++n) bf[n] = wsm[((t * S::kc + kc) * S::nt + n) * 32 + lane];
#pragma unroll
                for (int i = 0; i < 2; ++i) {
                    uint32_t a0, a1, a2, a3;
                    ldmatrix_x4(rowaddr[i] + kc * 32, a0, a1, a2, a3);
#pragma unroll
                    for (int n = 0; n < S::nt; ++n) mma_bf16(acc[i][n], a0, a1, a2, a3, bf[n].x, bf[n].y);
                }
            }
        }
        // epilogue: acc[i][n][q] is (row m = lane/4 + 8 (q/2), channel n*8 + 2 (lane%4) + q%2)
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            const int zz = z0 + rz[i], yy = y0 + ry[i];
            if (zz >= g.D || yy >= g.H) continue;
#pragma unroll
            for (int hh = 0; hh < 2; ++hh) {
                const int xx = x0 + lane / 4 + 8 * hh;
                if (xx >= g.W) continue;
                const int64_t v = vox_index(g, b, zz, yy, xx);
#pragma unroll
                for (int n = 0; n < S::nt; ++n) {
                    const int co = n * 8 + 2 * (lane % 4);
                    float v0 = acc[i][n][2 * hh], v1 = acc[i][n][2 * hh + 1];
                    if (mask) {
                        const __nv_bfloat162 m2 = *reinterpret_cast<const __nv_bfloat162*>(mask + hid<C>(v, co, nv));
                        v0 = __low2float(m2) > 0.0f ? v0 : 0.0f;
                        v1 = __high2float(m2) > 0.0f ? v1 : 0.0f;
                    } else {
                        v0 = fmaxf(v0 + bias[co], 0.0f);
                        v1 = fmaxf(v1 + bias[co + 1], 0.0f);
                    }
                    *reinterpret_cast<__nv_bfloat162*>(out + hid<C>(v, co, nv)) = __floats2bfloat162_rn(v0, v1);
                }
            }
        }
    }
}

// ---------------------------------------------------------------------------
// C -> C layers with tcgen05 (fifth-generation tensor cores, accumulator in
// tensor memory), fed by TMA.
//
// Output tile: one z plane of 16 rows x 8 voxels = the M = 128 rows of one
// tcgen05.mma (kind::f16, BF16 in, FP32 accumulate, N = C, K = 16).  The
// input halo of the tile (10 x 18 voxels, x 3 planes in 3-D) arrives by TMA,
// one 3-D box per 8-channel chunk plane of the chunk-planar activations (each
// box row is 16 * hx contiguous bytes), so shared memory holds it chunk-major:
// [chunk][halo voxel][16 bytes], chunks 128-byte aligned.  For every tap the A
// operand is then a no-swizzle K-major matrix: a core matrix is 8 consecutive
// voxels of one row (128 contiguous bytes), the next 8 rows of M are the next
// halo row (16 * hx bytes on), the second 8 channels of the K = 16 slice are
// the next chunk.  TMA fills the out-of-volume halo with zeros, which is the
// convolution's zero padding.  The weights stay in shared memory for the whole
// launch as B = W_t[ci][co] in the same K-major core-matrix layout.
//
// Warp roles (224 threads, one CTA per SM): warp 0 issues the TMA loads into
// two halo stages; one thread each of warps 1 and 6 issues the MMAs of a tile,
// the first half of the taps and the second, into two partial accumulators in
// tensor memory (one pair per stage), and commits them to mbarriers (stage
// free, accumulator full); warps 2-5 read the accumulator rows they may access
// (tcgen05.ld 32x32b), add the two partials, release them, and apply the
// epilogue.  Loads, MMAs and epilogues of neighbouring tiles overlap.  Two
// issuing threads, because one thread issues a 128 x 48 x 16 MMA about every
// 64 clocks, while the tensor core reads its operands (4 KB of A, 1.5 KB of B
// at 128 bytes per clock) in 44.  Every mbarrier wait is
// bounded: on timeout the kernel records an error, stops issuing work, waits
// (bounded) for its copies and MMAs in flight, and frees its tensor memory.
// ---------------------------------------------------------------------------
// NO: output columns of the MMA, C for the C -> C layers, 16 for the output
// layer (one channel, B padded with zero columns to the smallest N)
template <int ND, int C, int NO = C>
struct TcTile {
    static constexpr int tx = 8, ty = 16;
    static constexpr int hx = tx + 2, hy = ty + 2, hz = ND == 3 ? 3 : 1;
    static constexpr int halo = hx * hy * hz;
    static constexpr int halo_pad = (halo + 7) / 8 * 8;  // chunk stride: 128-byte multiple
    static constexpr int chunks = C / 8;
    static constexpr int taps = ND == 3 ? 27 : 9;
    static constexpr int kc = C / 16;
    static constexpr uint32_t cbytes = static_cast<uint32_t>(halo_pad) * 16;           // one chunk in shared memory
    static constexpr uint32_t box_bytes = static_cast<uint32_t>(halo) * 16;            // one chunk by TMA
    static constexpr uint32_t tbytes = chunks * cbytes;                                 // one halo stage
    static constexpr uint32_t wbytes = static_cast<uint32_t>(taps) * kc * 2 * NO * 16;  // B core matrices
    static constexpr uint32_t bytes = 2 * tbytes + wbytes;
    static constexpr int tsplit = (taps + 1) / 2;  // taps of the first issuing thread
    static constexpr uint32_t acc_cols = NO <= 32 ? 32 : 64;
    static constexpr uint32_t tmem_cols = 4 * acc_cols;  // (stage, half) partial accumulators
    static constexpr int threads = 224;
};

struct TcMaps {
    CUtensorMap m[6];  // one per 8-channel chunk of the input
};

// B for tcgen05: element (t, kc, kk, n, e) = W[t][ci = 16 kc + 8 kk + e][co = n]
// (forward) or W[taps-1-t][ci = n][co = 16 kc + 8 kk + e] (data gradient), BF16
template <int ND, int C>
__global__ void pack_tc_kernel(const float* __restrict__ W, bf16* __restrict__ out, int backward) {
    constexpr int T = Tile<ND>::taps;
    const int64_t total = static_cast<int64_t>(T) * (C / 16) * 2 * C * 8;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < total;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        int64_t r = i;
        const int e = static_cast<int>(r % 8);
        r /= 8;
        const int n = static_cast<int>(r % C);
        r /= C;
        const int kk = static_cast<int>(r % 2);
        r /= 2;
        const int kc = static_cast<int>(r % (C / 16));
        const int t = static_cast<int>(r / (C / 16));
        const int k = 16 * kc + 8 * kk + e;
        const float v = backward ? W[(static_cast<int64_t>(T - 1 - t) * C + n) * C + k]
                                 : W[(static_cast<int64_t>(t) * C + k) * C + n];
        out[i] = __float2bfloat16_rn(v);
    }
}

// c0 is the element offset along a row of the chunk plane (8 per voxel), so
// c0 * 2 bytes is a multiple of 16 for every voxel offset, negative included
// B of the output layer (one output channel) for tcgen05 with N = 16:
// element (t, kc, kk, n, e) = W[t][ci = 16 kc + 8 kk + e] for n = 0, else 0
template <int ND, int C>
__global__ void pack_tc_out_kernel(const float* __restrict__ W, bf16* __restrict__ out) {
    constexpr int T = Tile<ND>::taps;
    const int64_t total = static_cast<int64_t>(T) * (C / 16) * 2 * 16 * 8;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < total;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        int64_t r = i;
        const int e = static_cast<int>(r % 8);
        r /= 8;
        const int n = static_cast<int>(r % 16);
        r /= 16;
        const int kk = static_cast<int>(r % 2);
        r /= 2;
        const int kc = static_cast<int>(r % (C / 16));
        const int t = static_cast<int>(r / (C / 16));
        const int k = 16 * kc + 8 * kk + e;
        out[i] = __float2bfloat16_rn(n == 0 ? W[static_cast<int64_t>(t) * C + k] : 0.0f);
    }
}

__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap* map, int c0, int c1, int c2,
                                            uint32_t mbar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, "
        "%4}], [%5];\n" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(mbar)
        : "memory");
}

// the MMAs of taps T0 .. T1 - 1 of one tile into the accumulator at d_tmem
template <int ND, int C, int NO, int T0, int T1>
__device__ __forceinline__ void issue_conv_taps(uint64_t a_base, uint64_t b_base, uint32_t d_tmem) {
    using TT = TcTile<ND, C, NO>;
    constexpr uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | (static_cast<uint32_t>(NO >> 3) << 17) |
                               (static_cast<uint32_t>(128 >> 4) << 24);
#pragma unroll
    for (int t = T0; t < T1; ++t) {
        const int dz = ND == 3 ? t / 9 : 0;
        const int dy = ND == 3 ? (t / 3) % 3 : t / 3;
        const int dx = t % 3;
        const int vox0 = (dz * TT::hy + dy) * TT::hx + dx;
#pragma unroll
        for (int k = 0; k < TT::kc; ++k) {
            // start-address field += offset / 16 (stays below 2^14: no carry)
            const uint64_t ad = a_base + static_cast<uint64_t>(2 * k * TT::halo_pad + vox0);
            const uint64_t bd = b_base + static_cast<uint64_t>((t * TT::kc + k) * 2 * NO);
            const uint32_t acc = (t != T0 || k != 0) ? 1u : 0u;
            asm volatile(
                "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
                "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
                : "memory");
        }
    }
}

// NO == C: a C -> C layer (bias, ReLU or ReLU mask, BF16 out).  NO == 16: the
// output layer, y = a + b + sum (column 0 of the accumulator), written to y
// and, as the inverse Anscombe transform, to pilot (either may be null).
template <int ND, int C, int NO = C>
__global__ void __launch_bounds__(224, 1) conv_mid_tc_kernel(const __grid_constant__ TcMaps maps,
                                                             const bf16* __restrict__ wtc,
                                                             const float* __restrict__ bias,
                                                             const bf16* __restrict__ mask, bf16* __restrict__ out,
                                                             const float* __restrict__ a_in, float* __restrict__ y_out,
                                                             float* __restrict__ pilot_out, NetGeo g,
                                                             int* __restrict__ err, uint64_t probe_ns) {
    using TT = TcTile<ND, C, NO>;
    constexpr bool kOut = NO != C;
    extern __shared__ __align__(128) unsigned char tc_smem[];
    // full[2] (halo stage landed), empty[2] (stage read by the MMAs), afull[2]
    // (accumulator complete), aempty[2] (accumulator read out), weights, one
    // barrier that nothing completes (the wait probe), drain[2] (an issuing
    // thread's MMAs all done)
    __shared__ __align__(8) uint64_t bars[12];
    __shared__ uint32_t tmem_slot;
    __shared__ int abort_flag;
    volatile int* abort_v = &abort_flag;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t sbase = static_cast<uint32_t>(__cvta_generic_to_shared(tc_smem));
    const uint32_t wsm = sbase + 2 * TT::tbytes;
    const uint32_t bar0 = static_cast<uint32_t>(__cvta_generic_to_shared(bars));
    auto full = [&](int s) { return bar0 + 8u * s; };
    auto empty = [&](int s) { return bar0 + 16u + 8u * s; };
    auto afull = [&](int s) { return bar0 + 32u + 8u * s; };
    auto aempty = [&](int s) { return bar0 + 48u + 8u * s; };
    const uint32_t wbar = bar0 + 64u;
    const uint32_t never = bar0 + 72u;
    auto drain = [&](int k) { return bar0 + 80u + 8u * k; };
    constexpr uint64_t kWaitNs = 1000000000ull;  // one tile takes microseconds

    if (tid == 0) {
        for (int s = 0; s < 2; ++s) {
            mbar_init(full(s), 1);
            mbar_init(empty(s), 2);   // one commit per issuing thread
            mbar_init(afull(s), 2);
            mbar_init(aempty(s), 4);  // one arrival per epilogue warp
            mbar_init(drain(s), 1);
        }
        mbar_init(wbar, 1);
        mbar_init(never, 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        abort_flag = (sbase & 127u) != 0u ? 1 : 0;  // TMA destinations need 128-byte alignment
        if (abort_flag) atomicExch(err, 2);
    }
    if (warp == 1) {
        const uint32_t slot = static_cast<uint32_t>(__cvta_generic_to_shared(&tmem_slot));
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(slot),
                     "r"(TT::tmem_cols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_slot;
    if (probe_ns) {
        // wait probe: a bounded wait on a barrier nothing completes runs out
        // before any copy or product is issued; the launch then stops as on a
        // real timeout (status set, tensor memory freed below)
        if (tid == 0 && !mbar_wait(never, 0, probe_ns)) {
            abort_flag = 1;
            atomicExch(err, 1);
        }
        __syncthreads();
    }

    const int tiles_x = (g.W + TT::tx - 1) / TT::tx;
    const int tiles_y = (g.H + TT::ty - 1) / TT::ty;
    const int64_t ntiles = static_cast<int64_t>(tiles_x) * tiles_y * g.D * g.nb;
    auto decode = [&](int64_t tl, int& b, int& z0, int& y0, int& x0) {
        int64_t r = tl;
        x0 = static_cast<int>(r % tiles_x) * TT::tx;
        r /= tiles_x;
        y0 = static_cast<int>(r % tiles_y) * TT::ty;
        r /= tiles_y;
        z0 = static_cast<int>(r % g.D);
        b = static_cast<int>(r / g.D);
    };
    auto fail = [&](int code) {
        *abort_v = 1;
        atomicExch(err, code);
    };

    if (warp == 0) {
        // ---- producer: weights once, then one halo stage per tile ----
        int issued = 0;
        if (lane == 0 && !*abort_v) {
            mbar_expect_tx(wbar, TT::wbytes);
            asm volatile(
                "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
                    wsm),
                "l"(reinterpret_cast<uint64_t>(wtc)), "r"(TT::wbytes), "r"(wbar)
                : "memory");
            int it = 0;
            for (int64_t tl = blockIdx.x; tl < ntiles; tl += gridDim.x, ++it) {
                const int s = it & 1;
                if (!mbar_wait(empty(s), ((it >> 1) & 1) ^ 1, kWaitNs)) {
                    fail(1);
                    break;
                }
                if (*abort_v) break;
                int b, z0, y0, x0;
                decode(tl, b, z0, y0, x0);
                const int zc = ND == 3 ? b * g.D + z0 - 1 : b;
                mbar_expect_tx(full(s), TT::chunks * TT::box_bytes);
                const uint32_t dst = sbase + static_cast<uint32_t>(s) * TT::tbytes;
#pragma unroll
                for (int ch = 0; ch < TT::chunks; ++ch)
                    tma_load_3d(dst + ch * TT::cbytes, &maps.m[ch], 8 * (x0 - 1), y0 - 1, zc, full(s));
                issued = it + 1;
            }
            if (*abort_v) {
                // copies in flight: wait (bounded) for the last two stages
                for (int j = issued - 2; j < issued; ++j)
                    if (j >= 0) (void)mbar_wait(full(j & 1), (j >> 1) & 1, kWaitNs);
                (void)mbar_wait(wbar, 0, kWaitNs);
            }
        }
        __syncwarp();
    } else if (warp == 1 || warp == 6) {
        // ---- MMA issuers (lane 0): warp 1 the first TT::tsplit taps, warp 6 the
        // rest; each warp zeroes the batch-boundary planes of the stage before
        // its own MMAs (both write the same zeros) ----
        const int k = warp == 6 ? 1 : 0;
        bool ok = !*abort_v;
        if (ok && !mbar_wait(wbar, 0, kWaitNs)) {
            fail(1);
            ok = false;
        }
        int it = 0;
        for (int64_t tl = blockIdx.x; ok && tl < ntiles; tl += gridDim.x, ++it) {
            const int s = it & 1;
            const uint32_t ph = (it >> 1) & 1;
            bool got = true;
            if (lane == 0) got = mbar_wait(full(s), ph, kWaitNs) && mbar_wait(aempty(s), ph ^ 1, kWaitNs);
            got = __shfl_sync(0xffffffffu, got ? 1 : 0, 0) != 0;
            if (!got || *abort_v) {
                if (lane == 0 && !got) fail(1);
                break;
            }
            const uint32_t stage = sbase + static_cast<uint32_t>(s) * TT::tbytes;
            if (ND == 3 && g.nb > 1) {
                // planes of the neighbouring volume in the batch read as zero padding
                int b, z0, y0, x0;
                decode(tl, b, z0, y0, x0);
                const bool below = z0 == 0 && b > 0, above = z0 == g.D - 1 && b < g.nb - 1;
                if (below || above) {
                    constexpr int pv = TT::hx * TT::hy;
                    for (int plane = 0; plane < 3; plane += 2) {
                        if (plane == 0 ? !below : !above) continue;
                        for (int i = lane; i < TT::chunks * pv; i += 32) {
                            const int ch = i / pv, v = plane * pv + i % pv;
                            const uint32_t a = stage + ch * TT::cbytes + static_cast<uint32_t>(v) * 16u;
                            asm volatile("st.shared.v4.u32 [%0], {%1, %1, %1, %1};\n" ::"r"(a), "r"(0) : "memory");
                        }
                    }
                    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
                    __syncwarp();
                }
            }
            tc_fence_after();
            if (lane == 0) {
                const uint64_t a_base = umma_desc(stage, TT::cbytes, TT::hx * 16);
                const uint64_t b_base = umma_desc(wsm, NO * 16, 128);
                const uint32_t d_tmem = tmem + static_cast<uint32_t>(2 * s + k) * TT::acc_cols;
                if (k == 0)
                    issue_conv_taps<ND, C, NO, 0, TT::tsplit>(a_base, b_base, d_tmem);
                else
                    issue_conv_taps<ND, C, NO, TT::tsplit, TT::taps>(a_base, b_base, d_tmem);
                asm volatile(
                    "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(empty(s))
                    : "memory");
                asm volatile(
                    "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(afull(s))
                    : "memory");
            }
            __syncwarp();
        }
        if (lane == 0) {
            // every MMA of this thread done (bounded) before the tensor memory is freed
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                             drain(k))
                         : "memory");
            if (!mbar_wait(drain(k), 0, kWaitNs)) fail(1);
        }
        __syncwarp();
    } else {
        // ---- epilogue: warp w reads tensor-memory lanes 32 (w % 4) .. + 31 ----
        const int q = warp & 3;
        const int m = 32 * q + lane;  // accumulator row = voxel of the tile
        const int64_t nv = g.voxels();
        int it = 0;
        for (int64_t tl = blockIdx.x; tl < ntiles; tl += gridDim.x, ++it) {
            const int s = it & 1;
            if (*abort_v) break;
            bool got = true;
            if (lane == 0) got = mbar_wait(afull(s), (it >> 1) & 1, kWaitNs);
            got = __shfl_sync(0xffffffffu, got ? 1 : 0, 0) != 0;
            if (!got || *abort_v) {
                if (lane == 0 && !got) fail(1);
                break;
            }
            tc_fence_after();
            if constexpr (kOut) {
                // output layer: column 0 of both partial accumulators
                uint32_t p0, p1;
                const uint32_t tbase = tmem + (static_cast<uint32_t>(32 * q) << 16);
                asm volatile("tcgen05.ld.sync.aligned.32x32b.x1.b32 {%0}, [%1];\n"
                             : "=r"(p0)
                             : "r"(tbase + static_cast<uint32_t>(2 * s) * TT::acc_cols));
                asm volatile("tcgen05.ld.sync.aligned.32x32b.x1.b32 {%0}, [%1];\n"
                             : "=r"(p1)
                             : "r"(tbase + static_cast<uint32_t>(2 * s + 1) * TT::acc_cols));
                asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
                tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(aempty(s));
                int b, z0, y0, x0;
                decode(tl, b, z0, y0, x0);
                const int xx = x0 + (m % TT::tx), yy = y0 + m / TT::tx;
                if (xx < g.W && yy < g.H) {
                    const int64_t v = vox_index(g, b, z0, yy, xx);
                    const float yv = a_in[v] + (__ldg(bias) + (__uint_as_float(p0) + __uint_as_float(p1)));
                    if (y_out) y_out[v] = yv;
                    if (pilot_out) {
                        const float hh = 0.5f * yv;
                        pilot_out[v] = fmaxf(hh * hh - 0.375f, 0.0f);
                    }
                }
            } else {
                uint32_t r[C], r2[C];
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    uint32_t* d = h == 0 ? r : r2;
#pragma unroll
                    for (int c0 = 0; c0 < C; c0 += 16) {
                        const uint32_t taddr = tmem + (static_cast<uint32_t>(32 * q) << 16) +
                                               static_cast<uint32_t>(2 * s + h) * TT::acc_cols + c0;
                        asm volatile(
                            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, "
                            "%12, %13, %14, %15}, [%16];\n"
                            : "=r"(d[c0 + 0]), "=r"(d[c0 + 1]), "=r"(d[c0 + 2]), "=r"(d[c0 + 3]), "=r"(d[c0 + 4]),
                              "=r"(d[c0 + 5]), "=r"(d[c0 + 6]), "=r"(d[c0 + 7]), "=r"(d[c0 + 8]), "=r"(d[c0 + 9]),
                              "=r"(d[c0 + 10]), "=r"(d[c0 + 11]), "=r"(d[c0 + 12]), "=r"(d[c0 + 13]), "=r"(d[c0 + 14]),
                              "=r"(d[c0 + 15])
                            : "r"(taddr));
                    }
                }
                asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
                for (int c = 0; c < C; ++c) r[c] = __float_as_uint(__uint_as_float(r[c]) + __uint_as_float(r2[c]));
                tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(aempty(s));
                int b, z0, y0, x0;
                decode(tl, b, z0, y0, x0);
                const int xx = x0 + (m % TT::tx), yy = y0 + m / TT::tx;
                if (xx < g.W && yy < g.H) {
                    const int64_t v = vox_index(g, b, z0, yy, xx);
#pragma unroll
                    for (int c0 = 0; c0 < C; c0 += 8) {
                        __align__(16) bf16 o[8];
                        if (mask) {
                            __align__(16) bf16 mk[8];
                            *reinterpret_cast<uint4*>(mk) = *reinterpret_cast<const uint4*>(mask + hid<C>(v, c0, nv));
#pragma unroll
                            for (int j = 0; j < 8; ++j)
                                o[j] = __float2bfloat16_rn(__bfloat162float(mk[j]) > 0.0f ? __uint_as_float(r[c0 + j])
                                                                                         : 0.0f);
                        } else {
#pragma unroll
                            for (int j = 0; j < 8; ++j)
                                o[j] = __float2bfloat16_rn(
                                    fmaxf(__uint_as_float(r[c0 + j]) + __ldg(bias + c0 + j), 0.0f));
                        }
                        *reinterpret_cast<uint4*>(out + hid<C>(v, c0, nv)) = *reinterpret_cast<const uint4*>(o);
                    }
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 1)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(TT::tmem_cols)
                     : "memory");
}

// ---------------------------------------------------------------------------
// Weight gradients of the C -> C layers on the tensor cores.  For tap t,
//   dW_t[ci][co] = sum_v X[v + off_t][ci] dY[v][co],
// a GEMM with M = ci, N = co and K = the voxels: A is the input halo of a tile
// and B its output-gradient tile, both in shared memory exactly as TMA lands
// them from the chunk-planar tensors, where the 8 channels of a voxel are 16
// contiguous bytes and a tile row holds 8 voxels.  That is the MN-major
// core-matrix layout: 8 K-rows (voxels, 16 bytes apart) of 8 MN elements
// (channels); the MN stride between core matrices is one chunk plane, the K
// stride one tile row (the halo's row pitch for A, 128 bytes for B).  A tap is
// a shift of A's start address, as in the forward kernel.  M is 128 (the
// smallest single-CTA shape): rows C .. 127 read the memory after the C / 8
// chunk planes of the stage, which the layout keeps inside the allocation, and
// are discarded.  The CTAs split the taps into groups of 9, so one group's
// accumulators (9 x C columns) fit the 512 columns of tensor memory, and each
// CTA accumulates its share of the tiles for the whole launch; the per-CTA
// sums are added by reduce_partials_kernel.  Roles: warp 0 issues the TMA
// loads (two stages); one thread each of warps 1 and 2 issues the MMAs of the
// first 5 taps of the group and of the other 4 (one issuing thread cannot keep
// the tensor core busy with MMAs this small); at the end warps 0-1 read
// tensor-memory lanes 0-63.  Every mbarrier wait is bounded.
// ---------------------------------------------------------------------------
template <int ND, int C>
struct WgTile {
    using TT = TcTile<ND, C>;
    static constexpr int taps_per_cta = 9;
    static constexpr int tsplit = 5;  // taps of the first issuing thread
    static constexpr int groups = TT::taps / taps_per_cta;
    static constexpr uint32_t xbytes = TT::tbytes;                                   // one input-halo stage
    static constexpr uint32_t ybytes = TT::chunks * TT::tx * TT::ty * 16;            // one output-gradient stage
    // A of stage 1 reads 16 chunk planes from its start (M = 128)
    static constexpr uint32_t bytes = xbytes + 16 * TT::cbytes > 2 * (xbytes + ybytes)
                                          ? xbytes + 16 * TT::cbytes
                                          : 2 * (xbytes + ybytes);
    static constexpr uint32_t acc_cols = taps_per_cta * C;
    static constexpr int threads = 128;
};

template <int ND, int C>
__global__ void __launch_bounds__(128, 1) wgrad_tc_kernel(const __grid_constant__ TcMaps xmaps,
                                                          const __grid_constant__ TcMaps ymaps,
                                                          float* __restrict__ partial, int64_t nparams, NetGeo g,
                                                          int* __restrict__ err, uint64_t probe_ns) {
    using TT = TcTile<ND, C>;
    using WT = WgTile<ND, C>;
    extern __shared__ __align__(128) unsigned char wg_smem[];
    __shared__ __align__(8) uint64_t bars[6];  // full[2], empty[2], done, never
    __shared__ uint32_t tmem_slot;
    __shared__ int abort_flag;
    volatile int* abort_v = &abort_flag;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t sbase = static_cast<uint32_t>(__cvta_generic_to_shared(wg_smem));
    // stage s: the input halo at xs(s), the output gradient at ys(s)
    auto xs = [&](int st) { return sbase + static_cast<uint32_t>(st) * WT::xbytes; };
    auto ys = [&](int st) { return sbase + 2 * WT::xbytes + static_cast<uint32_t>(st) * WT::ybytes; };
    const uint32_t bar0 = static_cast<uint32_t>(__cvta_generic_to_shared(bars));
    auto full = [&](int st) { return bar0 + 8u * st; };
    auto empty = [&](int st) { return bar0 + 16u + 8u * st; };
    const uint32_t done = bar0 + 32u, never = bar0 + 40u;
    constexpr uint64_t kWaitNs = 1000000000ull;
    const int cpg = static_cast<int>(gridDim.x) / WT::groups;  // CTAs per tap group
    const int group = static_cast<int>(blockIdx.x) / cpg;
    const int gidx = static_cast<int>(blockIdx.x) - group * cpg;

    if (tid == 0) {
        for (int st = 0; st < 2; ++st) {
            mbar_init(full(st), 1);
            mbar_init(empty(st), 2);  // one commit per issuing thread
        }
        mbar_init(done, 2);
        mbar_init(never, 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        abort_flag = ((sbase & 127u) != 0u || group >= WT::groups) ? 1 : 0;
        if ((sbase & 127u) != 0u) atomicExch(err, 2);
    }
    if (warp == 1) {
        const uint32_t slot = static_cast<uint32_t>(__cvta_generic_to_shared(&tmem_slot));
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(slot), "r"(512)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_slot;
    if (probe_ns) {
        if (tid == 0 && !mbar_wait(never, 0, probe_ns)) {
            abort_flag = 1;
            atomicExch(err, 1);
        }
        __syncthreads();
    }

    const int tiles_x = (g.W + TT::tx - 1) / TT::tx;
    const int tiles_y = (g.H + TT::ty - 1) / TT::ty;
    const int64_t ntiles = static_cast<int64_t>(tiles_x) * tiles_y * g.D * g.nb;
    auto decode = [&](int64_t tl, int& b, int& z0, int& y0, int& x0) {
        int64_t r = tl;
        x0 = static_cast<int>(r % tiles_x) * TT::tx;
        r /= tiles_x;
        y0 = static_cast<int>(r % tiles_y) * TT::ty;
        r /= tiles_y;
        z0 = static_cast<int>(r % g.D);
        b = static_cast<int>(r / g.D);
    };
    auto fail = [&](int code) {
        *abort_v = 1;
        atomicExch(err, code);
    };
    if (warp == 0) {
        // ---- producer: one input halo and one output-gradient tile per stage ----
        int issued = 0;
        if (lane == 0 && !*abort_v) {
            int it = 0;
            for (int64_t tl = gidx; tl < ntiles; tl += cpg, ++it) {
                const int st = it & 1;
                if (!mbar_wait(empty(st), ((it >> 1) & 1) ^ 1, kWaitNs)) {
                    fail(1);
                    break;
                }
                if (*abort_v) break;
                int b, z0, y0, x0;
                decode(tl, b, z0, y0, x0);
                mbar_expect_tx(full(st), TT::chunks * (TT::box_bytes + TT::tx * TT::ty * 16));
#pragma unroll
                for (int ch = 0; ch < TT::chunks; ++ch) {
                    tma_load_3d(xs(st) + ch * TT::cbytes, &xmaps.m[ch], 8 * (x0 - 1), y0 - 1,
                                ND == 3 ? b * g.D + z0 - 1 : b, full(st));
                    tma_load_3d(ys(st) + ch * (TT::tx * TT::ty * 16), &ymaps.m[ch], 8 * x0, y0,
                                ND == 3 ? b * g.D + z0 : b, full(st));
                }
                issued = it + 1;
            }
            if (*abort_v) {
                // copies in flight: wait (bounded) for the last two stages
                for (int j = issued - 2; j < issued; ++j)
                    if (j >= 0) (void)mbar_wait(full(j & 1), (j >> 1) & 1, kWaitNs);
            }
        }
        __syncwarp();
    } else if (warp == 1 || warp == 2) {
        // ---- MMA issuers; each warp zeroes the batch-boundary planes before
        // its own MMAs (both write the same zeros) ----
        const int t_lo = warp == 1 ? 0 : WT::tsplit, t_hi = warp == 1 ? WT::tsplit : WT::taps_per_cta;
        constexpr uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | (1u << 15) | (1u << 16) |
                                   (static_cast<uint32_t>(C >> 3) << 17) | (static_cast<uint32_t>(128 >> 4) << 24);
        int it = 0;
        for (int64_t tl = gidx; !*abort_v && tl < ntiles; tl += cpg, ++it) {
            const int st = it & 1;
            bool got = true;
            if (lane == 0) got = mbar_wait(full(st), (it >> 1) & 1, kWaitNs);
            got = __shfl_sync(0xffffffffu, got ? 1 : 0, 0) != 0;
            if (!got || *abort_v) {
                if (lane == 0 && !got) fail(1);
                break;
            }
            if (ND == 3 && g.nb > 1) {
                // planes of the neighbouring volume in the batch read as zero padding
                int b, z0, y0, x0;
                decode(tl, b, z0, y0, x0);
                const bool below = z0 == 0 && b > 0, above = z0 == g.D - 1 && b < g.nb - 1;
                if (below || above) {
                    constexpr int pv = TT::hx * TT::hy;
                    for (int plane = 0; plane < 3; plane += 2) {
                        if (plane == 0 ? !below : !above) continue;
                        for (int i = lane; i < TT::chunks * pv; i += 32) {
                            const int ch = i / pv, v = plane * pv + i % pv;
                            const uint32_t a = xs(st) + ch * TT::cbytes + static_cast<uint32_t>(v) * 16u;
                            asm volatile("st.shared.v4.u32 [%0], {%1, %1, %1, %1};\n" ::"r"(a), "r"(0) : "memory");
                        }
                    }
                    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
                    __syncwarp();
                }
            }
            tc_fence_after();
            if (lane == 0) {
                // A: MN-major, SBO = chunk plane (next 8 input channels), LBO = halo row (next 8 voxels)
                const uint64_t a_base = umma_desc(xs(st), TT::hx * 16, TT::cbytes);
                // B: MN-major, SBO = chunk plane of the gradient tile, LBO = one tile row (128 bytes)
                const uint64_t b_base = umma_desc(ys(st), 128, TT::tx * TT::ty * 16);
#pragma unroll 1
                for (int tt = t_lo; tt < t_hi; ++tt) {
                    const int t = group * WT::taps_per_cta + tt;
                    const int dz = ND == 3 ? t / 9 : 0;
                    const int dy = ND == 3 ? (t / 3) % 3 : t / 3;
                    const int dx = t % 3;
                    const int vox0 = (dz * TT::hy + dy) * TT::hx + dx;
                    const uint32_t d_tmem = tmem + static_cast<uint32_t>(tt * C);
#pragma unroll
                    for (int ks = 0; ks < TT::ty / 2; ++ks) {
                        // K step ks: tile rows 2 ks and 2 ks + 1 (16 voxels)
                        const uint64_t ad = a_base + static_cast<uint64_t>(vox0 + 2 * ks * TT::hx);
                        const uint64_t bd = b_base + static_cast<uint64_t>(2 * ks * TT::tx);
                        const uint32_t acc = (it > 0 || ks > 0) ? 1u : 0u;
                        asm volatile(
                            "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
                            "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
                            : "memory");
                    }
                }
                asm volatile(
                    "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(empty(st))
                    : "memory");
            }
            __syncwarp();
        }
        if (lane == 0) {
            // everything issued (or nothing): the done barrier completes when the products have
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(done)
                         : "memory");
        }
        __syncwarp();
    }
    // ---- read the accumulators out: warp w holds tensor-memory lanes 32 w .. 32 w + 31 ----
    __syncthreads();
    bool got = true;
    if (lane == 0) got = mbar_wait(done, 0, kWaitNs);
    got = __shfl_sync(0xffffffffu, got ? 1 : 0, 0) != 0;
    if (!got && lane == 0) fail(1);
    tc_fence_after();
    if (warp < 2 && got && !*abort_v) {
        const int ci = 32 * warp + lane;
        float* out = partial + static_cast<int64_t>(blockIdx.x) * nparams;
        for (int c0 = 0; c0 < static_cast<int>(WT::acc_cols); c0 += 16) {
            uint32_t r[16];
            const uint32_t taddr = tmem + (static_cast<uint32_t>(32 * warp) << 16) + static_cast<uint32_t>(c0);
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, "
                "%12, %13, %14, %15}, [%16];\n"
                : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                  "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                  "=r"(r[15])
                : "r"(taddr));
            asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
            if (ci < C) {
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    const int col = c0 + j;
                    const int t = group * WT::taps_per_cta + col / C;
                    const int co = col % C;
                    out[(static_cast<int64_t>(t) * C + ci) * C + co] = __uint_as_float(r[j]);
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 1)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(512) : "memory");
}

// bias gradient of a C-channel layer: per-CTA partial sums of the output
// gradient over a contiguous share of the voxels, into the bias slots of the
// partial records; a thread reads the 8 channels of a voxel as 16 bytes
template <int C>
__global__ void __launch_bounds__(256) bias_partial_kernel(const bf16* __restrict__ gout, int64_t nv,
                                                           float* __restrict__ partial, int64_t nparams,
                                                           int64_t wparams) {
    __shared__ float red[8][8];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t per = (nv + gridDim.x - 1) / gridDim.x;
    const int64_t v0 = static_cast<int64_t>(blockIdx.x) * per, v1 = min(nv, v0 + per);
    for (int ch = 0; ch < C / 8; ++ch) {
        const uint4* src = reinterpret_cast<const uint4*>(gout + static_cast<int64_t>(ch) * nv * 8);
        float s[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) s[e] = 0.0f;
        for (int64_t v = v0 + threadIdx.x; v < v1; v += blockDim.x) {
            const uint4 q = src[v];
            const uint32_t w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                s[2 * e] += __uint_as_float(w[e] << 16);
                s[2 * e + 1] += __uint_as_float(w[e] & 0xffff0000u);
            }
        }
#pragma unroll
        for (int e = 0; e < 8; ++e)
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s[e] += __shfl_xor_sync(0xffffffffu, s[e], o);
        if (lane == 0)
#pragma unroll
            for (int e = 0; e < 8; ++e) red[warp][e] = s[e];
        __syncthreads();
        if (threadIdx.x < 8) {
            float t = 0.0f;
            for (int w = 0; w < static_cast<int>(blockDim.x >> 5); ++w) t += red[w][threadIdx.x];
            partial[static_cast<int64_t>(blockIdx.x) * nparams + wparams + ch * 8 + threadIdx.x] = t;
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// weight gradients (CUDA cores): per-CTA partial sums over a tile of 256
// voxels, summed over CTAs by reduce_partials_kernel
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ float to_f(T v);
template <>
__device__ __forceinline__ float to_f<float>(float v) { return v; }
template <>
__device__ __forceinline__ float to_f<bf16>(bf16 v) { return __bfloat162float(v); }

template <int ND, int CIN, int COUT, typename TI, typename TG>
struct WgradSmem {
    static constexpr size_t in_floats = static_cast<size_t>(Tile<ND>::halo) * CIN;
    static constexpr size_t g_floats = 256 * static_cast<size_t>(COUT);
    static constexpr size_t bytes = (in_floats + g_floats) * 4;
};

// partial[cta][p]: p = (t * CIN + ci) * COUT + co for the weights, then
// T * CIN * COUT + co for the bias
template <int ND, int CIN, int COUT, typename TI, typename TG>
__global__ void __launch_bounds__(256) wgrad_kernel(const TI* __restrict__ in, const TG* __restrict__ gout,
                                                    float* __restrict__ partial, NetGeo g) {
    using TL = Tile<ND>;
    constexpr int T = TL::taps;
    constexpr int BI = CIN >= 4 ? 4 : 1, BO = COUT >= 4 ? 4 : 1;
    constexpr int nw_items = T * (CIN / BI) * (COUT / BO);
    constexpr int nitems = nw_items + COUT / BO;
    constexpr int nparams = T * CIN * COUT + COUT;
    extern __shared__ __align__(16) unsigned char smem[];
    float* sin = reinterpret_cast<float*>(smem);
    float* sg = sin + static_cast<size_t>(TL::halo) * CIN;
    const int tiles_x = (g.W + TL::tx - 1) / TL::tx;
    const int tiles_y = (g.H + TL::ty - 1) / TL::ty;
    const int tiles_z = (g.D + TL::tz - 1) / TL::tz;
    int64_t r = blockIdx.x;
    const int x0 = static_cast<int>(r % tiles_x) * TL::tx;
    r /= tiles_x;
    const int y0 = static_cast<int>(r % tiles_y) * TL::ty;
    r /= tiles_y;
    const int z0 = static_cast<int>(r % tiles_z) * TL::tz;
    const int b = static_cast<int>(r / tiles_z);
    const int64_t nv = g.voxels();
    for (int j = threadIdx.x; j < TL::halo * CIN; j += blockDim.x) {
        const int c = j / TL::halo, vox = j - c * TL::halo;  // channel-major: coalesced reads
        const int i = vox * CIN + c;
        const int hxi = vox % TL::hx, hyi = (vox / TL::hx) % TL::hy, hzi = vox / (TL::hx * TL::hy);
        const int xx = x0 + hxi - 1, yy = y0 + hyi - 1, zz = ND == 3 ? z0 + hzi - 1 : z0;
        float v = 0.0f;
        if (xx >= 0 && xx < g.W && yy >= 0 && yy < g.H && zz >= 0 && zz < g.D)
            v = to_f<TI>(in[hid<CIN>(vox_index(g, b, zz, yy, xx), c, nv)]);
        sin[i] = v;
    }
    for (int j = threadIdx.x; j < 256 * COUT; j += blockDim.x) {
        const int c = j / 256, m = j - c * 256;
        const int xx = x0 + m % TL::tx, yy = y0 + (m / TL::tx) % TL::ty, zz = z0 + m / (TL::tx * TL::ty);
        float v = 0.0f;
        if (xx < g.W && yy < g.H && zz < g.D) v = to_f<TG>(gout[hid<COUT>(vox_index(g, b, zz, yy, xx), c, nv)]);
        sg[m * COUT + c] = v;
    }
    __syncthreads();
    float* out = partial + static_cast<int64_t>(blockIdx.x) * nparams;
    for (int item = threadIdx.x; item < nitems; item += blockDim.x) {
        float acc[BI][BO];
#pragma unroll
        for (int i = 0; i < BI; ++i)
#pragma unroll
            for (int o = 0; o < BO; ++o) acc[i][o] = 0.0f;
        if (item < nw_items) {
            const int cob = item % (COUT / BO);
            const int cib = (item / (COUT / BO)) % (CIN / BI);
            const int t = item / ((COUT / BO) * (CIN / BI));
            int dz, dy, dx;
            tap_offsets<ND>(t, dz, dy, dx);
            for (int m = 0; m < 256; ++m) {
                const int mx = m % TL::tx, my = (m / TL::tx) % TL::ty, mz = m / (TL::tx * TL::ty);
                const int hz = ND == 3 ? mz + dz + 1 : 0;
                const int vox = (hz * TL::hy + my + dy + 1) * TL::hx + mx + dx + 1;
                float iv[BI], gv[BO];
#pragma unroll
                for (int i = 0; i < BI; ++i) iv[i] = sin[vox * CIN + cib * BI + i];
#pragma unroll
                for (int o = 0; o < BO; ++o) gv[o] = sg[m * COUT + cob * BO + o];
#pragma unroll
                for (int i = 0; i < BI; ++i)
#pragma unroll
                    for (int o = 0; o < BO; ++o) acc[i][o] = fmaf(iv[i], gv[o], acc[i][o]);
            }
#pragma unroll
            for (int i = 0; i < BI; ++i)
#pragma unroll
                for (int o = 0; o < BO; ++o)
                    out[(t * CIN + cib * BI + i) * COUT + cob * BO + o] = acc[i][o];
        } else {
            const int cob = item - nw_items;
            for (int m = 0; m < 256; ++m)
#pragma unroll
                for (int o = 0; o < BO; ++o) acc[0][o] += sg[m * COUT + cob * BO + o];
#pragma unroll
            for (int o = 0; o < BO; ++o) out[T * CIN * COUT + cob * BO + o] = acc[0][o];
        }
    }
}

// Sums the per-CTA partial records into the gradient.  Block b owns the 32
// parameters 32 b .. 32 b + 31 (lane = parameter, coalesced 128-byte rows);
// warp w adds the records w, w + 32, ... of the range, and the warps' sums are
// added in warp order, so the result does not depend on timing.  With cpg > 0
// (tensor-core weight gradients) parameter p < wparams is summed over the cpg
// records of its tap group, p / group_params; otherwise over all records.
__global__ void __launch_bounds__(1024) reduce_partials_kernel(const float* __restrict__ partial, int64_t nparts,
                                                               int64_t nparams, float* __restrict__ grad, int cpg,
                                                               int64_t group_params, int64_t wparams) {
    __shared__ float red[32][33];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t p0 = static_cast<int64_t>(blockIdx.x) * 32;
    const int64_t p = p0 + lane;
    int64_t c0 = 0, c1 = nparts;
    if (cpg > 0 && p0 < wparams) {  // group_params and wparams are multiples of 32
        c0 = (p0 / group_params) * cpg;
        c1 = c0 + cpg;
    }
    float s = 0.0f;
    if (p < nparams) {
        int64_t c = c0 + warp;
        for (; c + 96 < c1; c += 128) {
            const float a0 = partial[c * nparams + p], a1 = partial[(c + 32) * nparams + p];
            const float a2 = partial[(c + 64) * nparams + p], a3 = partial[(c + 96) * nparams + p];
            s += a0;
            s += a1;
            s += a2;
            s += a3;
        }
        for (; c < c1; c += 32) s += partial[c * nparams + p];
    }
    red[warp][lane] = s;
    __syncthreads();
    if (warp == 0) {
        float t = 0.0f;
        for (int w = 0; w < 32; ++w) t += red[w][lane];
        if (p < nparams) grad[p] = t;
    }
}

__global__ void round_bf16_kernel(const float* __restrict__ src, float* __restrict__ dst, int64_t n) {
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x)
        dst[i] = __bfloat162float(__float2bfloat16_rn(src[i]));
}

// squared L2 norm of the gradient (for clipping), accumulated in float64
__global__ void sumsq_kernel(const float* __restrict__ g, int64_t n, double* __restrict__ out) {
    __shared__ double red[32];
    double local = 0.0;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x)
        local += static_cast<double>(g[i]) * g[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) local += __shfl_xor_sync(0xffffffffu, local, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = local;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int i = 0; i < static_cast<int>(blockDim.x >> 5); ++i) s += red[i];
        atomicAdd(out, s);
    }
}

// Adam on the gradient scaled by min(1, clip / ||g||) when clip > 0
__global__ void adam_kernel(float* __restrict__ p, const float* __restrict__ grad, float* __restrict__ m,
                            float* __restrict__ v, int64_t n, float lr, float b1, float b2, float eps, float bc1,
                            float bc2, float clip, const double* __restrict__ sumsq) {
    float scale = 1.0f;
    if (clip > 0.0f) {
        const double norm = sqrt(*sumsq);
        if (norm > static_cast<double>(clip)) scale = static_cast<float>(static_cast<double>(clip) / norm);
    }
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const float gi = grad[i] * scale;
        const float mi = b1 * m[i] + (1.0f - b1) * gi;
        const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        p[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
    }
}

// ---------------------------------------------------------------------------
// residual check for the per-tile fallback: for each tile of edge `edge`
// (cubes in 3-D, squares in 2-D) the observed Poisson deviance of the input
// against the pilot, sum_v 2 [x ln(x / mu) - (x - mu)], and its expectation and
// variance under Poisson noise of mean mu (interpolated in ln mu from a table
// of n points starting at ln_mu0 with step d_ln).  out[tile] = (observed,
// expected, variance) in float64.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void table_lookup(const float* __restrict__ table, int n, float ln_mu0, float d_ln,
                                             float mu, float& e, float& var) {
    float f = (logf(fmaxf(mu, 1e-30f)) - ln_mu0) / d_ln;
    f = fminf(fmaxf(f, 0.0f), static_cast<float>(n - 1));
    const int i = min(static_cast<int>(f), n - 2);
    const float w = f - static_cast<float>(i);
    e = (1.0f - w) * table[i] + w * table[i + 1];
    var = (1.0f - w) * table[n + i] + w * table[n + i + 1];
}

__global__ void tile_deviance_kernel(const float* __restrict__ x, const float* __restrict__ mu, NetGeo g, int edge,
                                     const float* __restrict__ table, int n, float ln_mu0, float d_ln,
                                     double* __restrict__ out, int tiles_x, int tiles_y, int tiles_z) {
    __shared__ double red[3][32];
    const int tile = blockIdx.x;
    int r = tile;
    const int tx = r % tiles_x;
    r /= tiles_x;
    const int ty = r % tiles_y;
    r /= tiles_y;
    const int tz = r % tiles_z;
    const int b = r / tiles_z;
    const int ez = g.D > 1 ? edge : 1;
    double obs = 0.0, ex = 0.0, va = 0.0;
    for (int i = threadIdx.x; i < ez * edge * edge; i += blockDim.x) {
        const int xx = tx * edge + i % edge, yy = ty * edge + (i / edge) % edge, zz = tz * ez + i / (edge * edge);
        if (xx >= g.W || yy >= g.H || zz >= g.D) continue;
        const int64_t v = vox_index(g, b, zz, yy, xx);
        const float xv = fmaxf(x[v], 0.0f), m = fmaxf(mu[v], 1e-6f);
        const float d = 2.0f * ((xv > 0.0f ? xv * logf(xv / m) : 0.0f) - (xv - m));
        float e, vr;
        table_lookup(table, n, ln_mu0, d_ln, m, e, vr);
        obs += d;
        ex += e;
        va += vr;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        obs += __shfl_xor_sync(0xffffffffu, obs, o);
        ex += __shfl_xor_sync(0xffffffffu, ex, o);
        va += __shfl_xor_sync(0xffffffffu, va, o);
    }
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        red[0][w] = obs;
        red[1][w] = ex;
        red[2][w] = va;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        double s = 0.0;
        for (int i = 0; i < static_cast<int>(blockDim.x >> 5); ++i) s += red[threadIdx.x][i];
        out[static_cast<int64_t>(tile) * 3 + threadIdx.x] = s;
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
struct NetPlan {
    int nd, C, L, taps;
    NetGeo geo;
    // flat FP32 parameter offsets (floats) of W_l and b_l
    std::vector<int64_t> w_off, b_off;
    int64_t nparams;
    // packed buffer offsets (bytes): bf16-rounded FP32 copies of the
    // one-channel layers, fragment-packed BF16 of the mid layers (forward and
    // data gradient), FP32 biases
    uint64_t p_in_w, packed_bytes;
    std::vector<uint64_t> p_mid_fwd, p_mid_bwd;
    uint64_t mid_frag_bytes;
    // the same layers as tcgen05 B operands (forward and data gradient), and
    // the output layer's weights as a B operand of 16 columns
    std::vector<uint64_t> p_tc_fwd, p_tc_bwd;
    uint64_t tc_bytes, p_tc_out, tc_out_bytes;
    int64_t max_layer_params;
};

int32_t make_plan(const BmndPilotNet* net, NetPlan& P) {
    if (!net) return fail(BMND_ERR_INVALID_ARG, "null network descriptor");
    if (net->ndim != 2 && net->ndim != 3) return fail(BMND_ERR_INVALID_ARG, "pilot net ndim must be 2 or 3");
    if (!(net->channels == 32 || net->channels == 48))
        return fail(BMND_ERR_UNSUPPORTED, "pilot net channels must be 32 or 48");
    if (net->layers < 3 || net->layers > 32) return fail(BMND_ERR_INVALID_ARG, "pilot net layers must be in [3, 32]");
    if (net->batch < 1) return fail(BMND_ERR_INVALID_ARG, "pilot net batch must be positive");
    P.nd = net->ndim;
    P.C = net->channels;
    P.L = net->layers;
    P.taps = net->ndim == 3 ? 27 : 9;
    P.geo.nb = net->batch;
    P.geo.D = net->ndim == 3 ? net->shape[0] : 1;
    P.geo.H = net->ndim == 3 ? net->shape[1] : net->shape[0];
    P.geo.W = net->ndim == 3 ? net->shape[2] : net->shape[1];
    if (P.geo.D < 1 || P.geo.H < 1 || P.geo.W < 1) return fail(BMND_ERR_INVALID_ARG, "pilot net shape must be positive");
    if (P.geo.voxels() > (int64_t(1) << 40)) return fail(BMND_ERR_UNSUPPORTED, "pilot net volume too large");
    P.w_off.clear();
    P.b_off.clear();
    int64_t off = 0;
    P.max_layer_params = 0;
    for (int l = 0; l < P.L; ++l) {
        const int cin = l == 0 ? 1 : P.C, cout = l == P.L - 1 ? 1 : P.C;
        P.w_off.push_back(off);
        off += static_cast<int64_t>(P.taps) * cin * cout;
        P.b_off.push_back(off);
        off += cout;
        const int64_t lp = static_cast<int64_t>(P.taps) * cin * cout + cout;
        if (lp > P.max_layer_params) P.max_layer_params = lp;
    }
    P.nparams = off;
    // packed layout
    auto a256 = [](uint64_t v) { return (v + 255) & ~uint64_t(255); };
    uint64_t po = 0;
    P.p_in_w = po;  // bf16-rounded copy of the whole FP32 parameter vector
    po = a256(po + 4ull * static_cast<uint64_t>(P.nparams));
    P.mid_frag_bytes = static_cast<uint64_t>(P.taps) * (P.C / 16) * (P.C / 8) * 32 * 8;
    P.p_mid_fwd.clear();
    P.p_mid_bwd.clear();
    for (int l = 1; l < P.L - 1; ++l) {
        P.p_mid_fwd.push_back(po);
        po = a256(po + P.mid_frag_bytes);
        P.p_mid_bwd.push_back(po);
        po = a256(po + P.mid_frag_bytes);
    }
    P.tc_bytes = static_cast<uint64_t>(P.taps) * (P.C / 16) * 2 * P.C * 16;
    P.p_tc_fwd.clear();
    P.p_tc_bwd.clear();
    for (int l = 1; l < P.L - 1; ++l) {
        P.p_tc_fwd.push_back(po);
        po = a256(po + P.tc_bytes);
        P.p_tc_bwd.push_back(po);
        po = a256(po + P.tc_bytes);
    }
    P.tc_out_bytes = static_cast<uint64_t>(P.taps) * (P.C / 16) * 2 * 16 * 16;
    P.p_tc_out = po;
    po = a256(po + P.tc_out_bytes);
    P.packed_bytes = po;
    return BMND_OK;
}

int launch_blocks(int64_t n, int threads) {
    int64_t blocks = (n + threads - 1) / threads;
    if (blocks > 152 * 32) blocks = 152 * 32;
    if (blocks < 1) blocks = 1;
    return static_cast<int>(blocks);
}

struct Bufs {
    int* err;            // set by a kernel whose bounded wait ran out
    float* a;            // Anscombe input
    float* y;            // network output (Anscombe domain)
    float* gy;           // its gradient
    bf16* act;           // hidden activations, (L - 1) x voxels x C (training) or 2 (inference)
    bf16* grad[2];       // hidden gradients, ping-pong
    float* partial;      // weight-gradient partial sums
    uint64_t bytes;
};

Bufs carve_ws(const NetPlan& P, bool training, void* base) {
    Bufs B{};
    uint64_t off = 0;
    auto take = [&](uint64_t bytes) {
        uint64_t o = off;
        off += (bytes + 255) & ~uint64_t(255);
        return o;
    };
    const uint64_t nv = static_cast<uint64_t>(P.geo.voxels());
    const uint64_t hbytes = nv * P.C * 2;
    const uint64_t o_err = take(sizeof(int));
    const uint64_t o_a = take(nv * 4);
    const uint64_t o_y = take(nv * 4);
    const uint64_t o_gy = training ? take(nv * 4) : 0;
    const uint64_t o_act = take(hbytes * (training ? (P.L - 1) : 2));
    const uint64_t o_g0 = training ? take(hbytes) : 0;
    const uint64_t o_g1 = training ? take(hbytes) : 0;
    const int64_t tiles = [&] {
        const int tx = 16, ty = P.nd == 3 ? 8 : 16, tz = P.nd == 3 ? 2 : 1;
        return static_cast<int64_t>((P.geo.W + tx - 1) / tx) * ((P.geo.H + ty - 1) / ty) *
               ((P.geo.D + tz - 1) / tz) * P.geo.nb;
    }();
    const uint64_t o_part = training ? take(static_cast<uint64_t>(tiles) * P.max_layer_params * 4) : 0;
    B.bytes = off;
    if (base) {
        char* c = static_cast<char*>(base);
        B.err = reinterpret_cast<int*>(c + o_err);
        B.a = reinterpret_cast<float*>(c + o_a);
        B.y = reinterpret_cast<float*>(c + o_y);
        B.gy = training ? reinterpret_cast<float*>(c + o_gy) : nullptr;
        B.act = reinterpret_cast<bf16*>(c + o_act);
        B.grad[0] = training ? reinterpret_cast<bf16*>(c + o_g0) : nullptr;
        B.grad[1] = training ? reinterpret_cast<bf16*>(c + o_g1) : nullptr;
        B.partial = training ? reinterpret_cast<float*>(c + o_part) : nullptr;
    }
    return B;
}

template <int ND, int C>
int32_t run_mid(const bf16* in, const uint2* wpk, const float* bias, const bf16* mask, bf16* out, NetGeo g,
                cudaStream_t stream) {
    using S = MidSmem<ND, C>;
    auto kernel = conv_mid_kernel<ND, C>;
    int sms = 0, per_sm = 0;
    if (int32_t rc = kernel_residency(reinterpret_cast<const void*>(kernel), 256, S::bytes, false, &per_sm, &sms))
        return rc;
    if (per_sm < 1) return fail(BMND_ERR_UNSUPPORTED, "pilot net layer does not fit on an SM");
    using TL = Tile<ND>;
    const int64_t ntiles = static_cast<int64_t>((g.W + TL::tx - 1) / TL::tx) * ((g.H + TL::ty - 1) / TL::ty) *
                           ((g.D + TL::tz - 1) / TL::tz) * g.nb;
    int64_t blocks = static_cast<int64_t>(sms) * per_sm;
    if (blocks > ntiles) blocks = ntiles;
    kernel<<<static_cast<unsigned>(blocks), 256, S::bytes, stream>>>(in, wpk, bias, mask, out, g);
    BMND_LAUNCH_CHECK("conv_mid_kernel");
    return BMND_OK;
}

int g_conv_engine = BMND_CONV_TCGEN05;
uint64_t g_wait_probe_ns = 0;  // see bmnd_pilotnet_set_wait_probe

// One 3-D tensor map per 8-channel chunk plane of a chunk-planar BF16 tensor:
// (8 channels x W voxels as one row of elements, y, z * batch), with a box of
// box_vox = (x, y, z) voxels, so a box row is 16 x bytes contiguous in memory
// and arrives as whole 32-byte sectors; out-of-range elements read as zero.
// The CUDA driver API's tensor-map encoder is fetched through the runtime (no
// link-time dependency on libcuda).
int32_t encode_chunk_maps(const bf16* base, NetGeo g, int C, const uint32_t box_vox[3], TcMaps& maps) {
    memset(&maps, 0, sizeof(maps));
    const cuuint64_t dims[3] = {static_cast<cuuint64_t>(g.W) * 8, static_cast<cuuint64_t>(g.H),
                                static_cast<cuuint64_t>(g.D) * static_cast<cuuint64_t>(g.nb)};
    const cuuint64_t strides[2] = {static_cast<cuuint64_t>(g.W) * 16, static_cast<cuuint64_t>(g.H) * g.W * 16};
    const cuuint32_t box[3] = {box_vox[0] * 8, box_vox[1], box_vox[2]};
    const cuuint32_t estr[3] = {1, 1, 1};
    static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    if (!encode) {
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        void* fn = nullptr;
        BMND_CUDA_TRY(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q));
        if (q != cudaDriverEntryPointSuccess || !fn) return fail(BMND_ERR_CUDA, "cuTensorMapEncodeTiled not available");
        encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    }
    const int64_t nv = g.voxels();
    for (int ch = 0; ch < C / 8; ++ch) {
        const CUresult rc = encode(&maps.m[ch], CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3,
                                   const_cast<bf16*>(base) + static_cast<int64_t>(ch) * nv * 8, dims, strides, box,
                                   estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                   CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (rc != CUDA_SUCCESS) return fail(BMND_ERR_CUDA, "cuTensorMapEncodeTiled failed for a pilot net tensor");
    }
    return BMND_OK;
}

template <int ND, int C>
int32_t run_mid_tc(const bf16* in, const bf16* wtc, const float* bias, const bf16* mask, bf16* out, NetGeo g,
                   int* err, cudaStream_t stream) {
    using TT = TcTile<ND, C>;
    auto kernel = conv_mid_tc_kernel<ND, C>;
    int sms = 0, per_sm = 0;
    if (int32_t rc = kernel_residency(reinterpret_cast<const void*>(kernel), TT::threads, TT::bytes, false, &per_sm,
                                      &sms))
        return rc;
    if ((reinterpret_cast<uintptr_t>(in) & 15u) != 0 || (reinterpret_cast<uintptr_t>(wtc) & 15u) != 0)
        return fail(BMND_ERR_INVALID_ARG, "pilot net buffers must be 16-byte aligned");
    // one map per 8-channel chunk plane, a box of (hx, hy, hz) voxels whose
    // rows are 16 * hx contiguous bytes; out-of-range elements read as zero
    TcMaps maps;
    const uint32_t box[3] = {TT::hx, TT::hy, TT::hz};
    if (int32_t rc = encode_chunk_maps(in, g, C, box, maps)) return rc;
    const int64_t ntiles = static_cast<int64_t>((g.W + TT::tx - 1) / TT::tx) * ((g.H + TT::ty - 1) / TT::ty) * g.D *
                           g.nb;
    // one persistent CTA per SM: the weights fill most of the shared memory
    int64_t blocks = sms;
    if (blocks > ntiles) blocks = ntiles;
    kernel<<<static_cast<unsigned>(blocks), TT::threads, TT::bytes, stream>>>(
        maps, wtc, bias, mask, out, nullptr, nullptr, nullptr, g, err, g_wait_probe_ns);
    BMND_LAUNCH_CHECK("conv_mid_tc_kernel");
    return BMND_OK;
}

// the output layer (C -> 1) on the tensor cores: N = 16 columns, column 0 used
template <int ND, int C>
int32_t run_out_tc(const bf16* in, const bf16* wtc, const float* bias, const float* a, float* y, float* pilot,
                   NetGeo g, int* err, cudaStream_t stream) {
    using TT = TcTile<ND, C, 16>;
    auto kernel = conv_mid_tc_kernel<ND, C, 16>;
    int sms = 0, per_sm = 0;
    if (int32_t rc = kernel_residency(reinterpret_cast<const void*>(kernel), TT::threads, TT::bytes, false, &per_sm,
                                      &sms))
        return rc;
    if ((reinterpret_cast<uintptr_t>(in) & 15u) != 0 || (reinterpret_cast<uintptr_t>(wtc) & 15u) != 0)
        return fail(BMND_ERR_INVALID_ARG, "pilot net buffers must be 16-byte aligned");
    TcMaps maps;
    const uint32_t box[3] = {TT::hx, TT::hy, TT::hz};
    if (int32_t rc = encode_chunk_maps(in, g, C, box, maps)) return rc;
    const int64_t ntiles = static_cast<int64_t>((g.W + TT::tx - 1) / TT::tx) * ((g.H + TT::ty - 1) / TT::ty) * g.D *
                           g.nb;
    int64_t blocks = sms;
    if (blocks > ntiles) blocks = ntiles;
    kernel<<<static_cast<unsigned>(blocks), TT::threads, TT::bytes, stream>>>(
        maps, wtc, bias, nullptr, nullptr, a, y, pilot, g, err, g_wait_probe_ns);
    BMND_LAUNCH_CHECK("conv_mid_tc_kernel");
    return BMND_OK;
}

// one C -> C layer with the selected engine; l is the layer (1 .. L-2)
template <int ND, int C>
int32_t run_layer(const NetPlan& P, const unsigned char* packed, int l, bool backward, const bf16* in,
                  const float* bias, const bf16* mask, bf16* out, const Bufs& B, cudaStream_t stream) {
    if (g_conv_engine == BMND_CONV_TCGEN05) {
        const bf16* w = reinterpret_cast<const bf16*>(packed + (backward ? P.p_tc_bwd : P.p_tc_fwd)[l - 1]);
        return run_mid_tc<ND, C>(in, w, bias, mask, out, P.geo, B.err, stream);
    }
    const uint2* w = reinterpret_cast<const uint2*>(packed + (backward ? P.p_mid_bwd : P.p_mid_fwd)[l - 1]);
    return run_mid<ND, C>(in, w, bias, mask, out, P.geo, stream);
}

template <int ND, int C>
int32_t forward_impl(const NetPlan& P, const unsigned char* packed, const float* noisy, float* pilot, float* y_out,
                     Bufs& B, bool keep_all, cudaStream_t stream) {
    const NetGeo g = P.geo;
    const int64_t nv = g.voxels();
    const float* wr = reinterpret_cast<const float*>(packed + P.p_in_w);  // bf16-rounded parameters
    const int eb = launch_blocks(nv, 256);
    anscombe_kernel<<<eb, 256, 0, stream>>>(noisy, B.a, nv);
    BMND_LAUNCH_CHECK("anscombe_kernel");
    auto act = [&](int l) -> bf16* {  // hidden activation h_{l+1} (output of layer l)
        const int64_t stride = nv * C;
        return B.act + (keep_all ? l : (l & 1)) * stride;
    };
    conv_in_kernel<ND, C><<<launch_blocks((nv + 1) / 2, 256), 256, 0, stream>>>(B.a, wr + P.w_off[0],
                                                                              wr + P.b_off[0], act(0), g);
    BMND_LAUNCH_CHECK("conv_in_kernel");
    for (int l = 1; l < P.L - 1; ++l) {
        int32_t rc = run_layer<ND, C>(P, packed, l, false, act(l - 1), wr + P.b_off[l], nullptr, act(l), B, stream);
        if (rc) return rc;
    }
    if (g_conv_engine == BMND_CONV_TCGEN05) {
        return run_out_tc<ND, C>(act(P.L - 2), reinterpret_cast<const bf16*>(packed + P.p_tc_out),
                                 wr + P.b_off[P.L - 1], B.a, y_out, pilot, g, B.err, stream);
    }
    {
        using OT = OutTile<ND>;
        constexpr size_t smem = out_smem_bytes<ND, C>();
        int sms = 0, per_sm = 0;
        if (int32_t rc = kernel_residency(reinterpret_cast<const void*>(conv_out_kernel<ND, C>), OT::tx * OT::ty,
                                          smem, false, &per_sm, &sms))
            return rc;
        const int64_t blocks = static_cast<int64_t>((g.W + OT::tx - 1) / OT::tx) * ((g.H + OT::ty - 1) / OT::ty) *
                               ((g.D + OT::zb - 1) / OT::zb) * g.nb;
        conv_out_kernel<ND, C><<<static_cast<unsigned>(blocks), OT::tx * OT::ty, smem, stream>>>(
            act(P.L - 2), wr + P.w_off[P.L - 1], wr + P.b_off[P.L - 1], B.a, y_out, pilot, g);
    }
    BMND_LAUNCH_CHECK("conv_out_kernel");
    return BMND_OK;
}

template <int ND, int CIN, int COUT, typename TI, typename TG>
int32_t run_wgrad(const TI* in, const TG* gout, float* partial, float* grad, int64_t tiles, NetGeo g,
                  cudaStream_t stream) {
    using S = WgradSmem<ND, CIN, COUT, TI, TG>;
    auto kernel = wgrad_kernel<ND, CIN, COUT, TI, TG>;
    int sms = 0, per_sm = 0;
    if (int32_t rc = kernel_residency(reinterpret_cast<const void*>(kernel), 256, S::bytes, false, &per_sm, &sms))
        return rc;
    kernel<<<static_cast<unsigned>(tiles), 256, S::bytes, stream>>>(in, gout, partial, g);
    BMND_LAUNCH_CHECK("wgrad_kernel");
    constexpr int64_t np = static_cast<int64_t>(Tile<ND>::taps) * CIN * COUT + COUT;
    reduce_partials_kernel<<<static_cast<unsigned>((np + 31) / 32), 1024, 0, stream>>>(partial, tiles, np, grad, 0,
                                                                                      np, np);
    BMND_LAUNCH_CHECK("reduce_partials_kernel");
    return BMND_OK;
}

// the C -> C weight gradient on the tensor cores; returns BMND_ERR_UNSUPPORTED
// (nothing launched) when the partial records do not fit the workspace
template <int ND, int C>
int32_t run_wgrad_tc(const bf16* in, const bf16* gout, float* partial, int64_t capacity, float* grad, NetGeo g,
                     int* err, cudaStream_t stream) {
    using TT = TcTile<ND, C>;
    using WT = WgTile<ND, C>;
    auto kernel = wgrad_tc_kernel<ND, C>;
    int sms = 0, per_sm = 0;
    if (int32_t rc = kernel_residency(reinterpret_cast<const void*>(kernel), WT::threads, WT::bytes, false, &per_sm,
                                      &sms))
        return rc;
    if (per_sm < 1) return BMND_ERR_UNSUPPORTED;
    if ((reinterpret_cast<uintptr_t>(in) & 15u) != 0 || (reinterpret_cast<uintptr_t>(gout) & 15u) != 0)
        return fail(BMND_ERR_INVALID_ARG, "pilot net buffers must be 16-byte aligned");
    const int64_t ntiles = static_cast<int64_t>((g.W + TT::tx - 1) / TT::tx) * ((g.H + TT::ty - 1) / TT::ty) *
                           g.D * g.nb;
    int64_t cpg = sms / WT::groups;
    if (cpg > ntiles) cpg = ntiles;
    if (cpg * WT::groups > capacity) cpg = capacity / WT::groups;
    if (cpg < 1) return BMND_ERR_UNSUPPORTED;
    TcMaps xmaps, ymaps;
    const uint32_t xbox[3] = {TT::hx, TT::hy, TT::hz};
    const uint32_t ybox[3] = {TT::tx, TT::ty, 1};
    if (int32_t rc = encode_chunk_maps(in, g, C, xbox, xmaps)) return rc;
    if (int32_t rc = encode_chunk_maps(gout, g, C, ybox, ymaps)) return rc;
    constexpr int64_t wparams = static_cast<int64_t>(TT::taps) * C * C;
    constexpr int64_t np = wparams + C;
    const int64_t nparts = cpg * WT::groups;
    kernel<<<static_cast<unsigned>(nparts), WT::threads, WT::bytes, stream>>>(xmaps, ymaps, partial, np, g, err,
                                                                             g_wait_probe_ns);
    BMND_LAUNCH_CHECK("wgrad_tc_kernel");
    bias_partial_kernel<C><<<static_cast<unsigned>(nparts), 256, 0, stream>>>(gout, g.voxels(), partial, np, wparams);
    BMND_LAUNCH_CHECK("bias_partial_kernel");
    reduce_partials_kernel<<<static_cast<unsigned>((np + 31) / 32), 1024, 0, stream>>>(
        partial, nparts, np, grad, static_cast<int>(cpg), static_cast<int64_t>(WT::taps_per_cta) * C * C, wparams);
    BMND_LAUNCH_CHECK("reduce_partials_kernel");
    return BMND_OK;
}

template <int ND, int C>
int32_t gradient_impl(const NetPlan& P, const unsigned char* packed, const float* noisy, const float* target,
                      float* grad, double* loss, Bufs& B, cudaStream_t stream) {
    const NetGeo g = P.geo;
    const int64_t nv = g.voxels();
    int32_t rc = forward_impl<ND, C>(P, packed, noisy, nullptr, B.y, B, true, stream);
    if (rc) return rc;
    const float* wr = reinterpret_cast<const float*>(packed + P.p_in_w);
    const int eb = launch_blocks(nv, 256);
    BMND_CUDA_TRY(cudaMemsetAsync(loss, 0, sizeof(double), stream));
    loss_grad_kernel<<<eb, 256, 0, stream>>>(B.y, target, B.gy, nv, loss);
    BMND_LAUNCH_CHECK("loss_grad_kernel");
    using TL = Tile<ND>;
    const int64_t tiles = static_cast<int64_t>((g.W + TL::tx - 1) / TL::tx) * ((g.H + TL::ty - 1) / TL::ty) *
                          ((g.D + TL::tz - 1) / TL::tz) * g.nb;
    const int64_t stride = nv * C;
    auto act = [&](int l) -> bf16* { return B.act + l * stride; };
    const int L = P.L;
    constexpr int64_t wg_params = static_cast<int64_t>(TL::taps) * C * C + C;  // one C -> C layer
    // last layer: weight gradient from h_{L-1} and gy, data gradient into h_{L-1}
    rc = run_wgrad<ND, C, 1, bf16, float>(act(L - 2), B.gy, B.partial, grad + P.w_off[L - 1], tiles, g, stream);
    if (rc) return rc;
    int cur = 0;
    conv_out_dgrad_kernel<ND, C><<<eb, 256, 0, stream>>>(B.gy, wr + P.w_off[L - 1], act(L - 2), B.grad[cur], g);
    BMND_LAUNCH_CHECK("conv_out_dgrad_kernel");
    // mid layers, last to first: B.grad[cur] is the gradient of layer l's output
    for (int l = L - 2; l >= 1; --l) {
        rc = BMND_ERR_UNSUPPORTED;
        if (g_conv_engine == BMND_CONV_TCGEN05)
            rc = run_wgrad_tc<ND, C>(act(l - 1), B.grad[cur], B.partial, tiles * P.max_layer_params / wg_params,
                                     grad + P.w_off[l], g, B.err, stream);
        if (rc == BMND_ERR_UNSUPPORTED)
            rc = run_wgrad<ND, C, C, bf16, bf16>(act(l - 1), B.grad[cur], B.partial, grad + P.w_off[l], tiles, g,
                                                 stream);
        if (rc) return rc;
        rc = run_layer<ND, C>(P, packed, l, true, B.grad[cur], nullptr, act(l - 1), B.grad[cur ^ 1], B, stream);
        if (rc) return rc;
        cur ^= 1;
    }
    // first layer: weight gradient only
    return run_wgrad<ND, 1, C, float, bf16>(B.a, B.grad[cur], B.partial, grad + P.w_off[0], tiles, g, stream);
}

template <typename F>
int32_t dispatch(const NetPlan& P, F&& f) {
    if (P.nd == 3 && P.C == 48) return f(std::integral_constant<int, 3>{}, std::integral_constant<int, 48>{});
    if (P.nd == 3 && P.C == 32) return f(std::integral_constant<int, 3>{}, std::integral_constant<int, 32>{});
    if (P.nd == 2 && P.C == 48) return f(std::integral_constant<int, 2>{}, std::integral_constant<int, 48>{});
    return f(std::integral_constant<int, 2>{}, std::integral_constant<int, 32>{});
}

}  // namespace
}  // namespace bmnd

using namespace bmnd;

extern "C" {

int32_t bmnd_pilotnet_param_count(const BmndPilotNet* net, int64_t* count) {
    clear_error();
    NetPlan P;
    if (int32_t rc = make_plan(net, P)) return rc;
    if (!count) return fail(BMND_ERR_INVALID_ARG, "null output");
    *count = P.nparams;
    return BMND_OK;
}

int32_t bmnd_pilotnet_packed_bytes(const BmndPilotNet* net, uint64_t* bytes) {
    clear_error();
    NetPlan P;
    if (int32_t rc = make_plan(net, P)) return rc;
    if (!bytes) return fail(BMND_ERR_INVALID_ARG, "null output");
    *bytes = P.packed_bytes;
    return BMND_OK;
}

int32_t bmnd_pilotnet_workspace_bytes(const BmndPilotNet* net, int32_t training, uint64_t* bytes) {
    clear_error();
    NetPlan P;
    if (int32_t rc = make_plan(net, P)) return rc;
    if (!bytes) return fail(BMND_ERR_INVALID_ARG, "null output");
    *bytes = carve_ws(P, training != 0, nullptr).bytes;
    return BMND_OK;
}

int32_t bmnd_pilotnet_set_conv_engine(int32_t engine) {
    clear_error();
    if (engine != BMND_CONV_TCGEN05 && engine != BMND_CONV_MMA_SYNC)
        return fail(BMND_ERR_INVALID_ARG, "unknown convolution engine");
    g_conv_engine = engine;
    return BMND_OK;
}

int32_t bmnd_pilotnet_get_conv_engine(int32_t* engine) {
    clear_error();
    if (!engine) return fail(BMND_ERR_INVALID_ARG, "null output");
    *engine = g_conv_engine;
    return BMND_OK;
}

int32_t bmnd_pilotnet_set_wait_probe(uint64_t ns) {
    clear_error();
    if (ns > 1000000000ull) return fail(BMND_ERR_INVALID_ARG, "the wait probe is at most one second");
    g_wait_probe_ns = ns;
    return BMND_OK;
}

int32_t bmnd_pilotnet_status(const BmndPilotNet* net, const void* d_ws, uint64_t stream_u64) {
    clear_error();
    NetPlan P;
    if (int32_t rc = make_plan(net, P)) return rc;
    if (!d_ws) return fail(BMND_ERR_INVALID_ARG, "null workspace");
    Bufs B = carve_ws(P, false, const_cast<void*>(d_ws));
    int flag = 0;
    cudaStream_t stream = reinterpret_cast<cudaStream_t>(stream_u64);
    BMND_CUDA_TRY(cudaMemcpyAsync(&flag, B.err, sizeof(int), cudaMemcpyDeviceToHost, stream));
    BMND_CUDA_TRY(cudaStreamSynchronize(stream));
    if (flag) return fail(BMND_ERR_TIMEOUT, "a pilot net tensor-core wait ran out of time");
    return BMND_OK;
}

int32_t bmnd_pilotnet_pack(const BmndPilotNet* net, const float* d_params, void* d_packed, uint64_t stream_u64) {
    clear_error();
    NetPlan P;
    if (int32_t rc = make_plan(net, P)) return rc;
    if (!d_params || !d_packed) return fail(BMND_ERR_INVALID_ARG, "null buffer");
    cudaStream_t stream = reinterpret_cast<cudaStream_t>(stream_u64);
    unsigned char* pk = static_cast<unsigned char*>(d_packed);
    round_bf16_kernel<<<launch_blocks(P.nparams, 256), 256, 0, stream>>>(
        d_params, reinterpret_cast<float*>(pk + P.p_in_w), P.nparams);
    BMND_LAUNCH_CHECK("round_bf16_kernel");
    return dispatch(P, [&](auto nd, auto c) -> int32_t {
        constexpr int ND = decltype(nd)::value, C = decltype(c)::value;
        const int64_t nfrag = static_cast<int64_t>(MidSmem<ND, C>::wfrag);
        for (int l = 1; l < P.L - 1; ++l) {
            pack_mid_kernel<ND, C><<<launch_blocks(nfrag, 256), 256, 0, stream>>>(
                d_params + P.w_off[l], reinterpret_cast<uint2*>(pk + P.p_mid_fwd[l - 1]), 0);
            BMND_LAUNCH_CHECK("pack_mid_kernel");
            pack_mid_kernel<ND, C><<<launch_blocks(nfrag, 256), 256, 0, stream>>>(
                d_params + P.w_off[l], reinterpret_cast<uint2*>(pk + P.p_mid_bwd[l - 1]), 1);
            BMND_LAUNCH_CHECK("pack_mid_kernel");
            const int64_t ntc = static_cast<int64_t>(P.tc_bytes / 2);
            for (int dir = 0; dir < 2; ++dir) {
                pack_tc_kernel<ND, C><<<launch_blocks(ntc, 256), 256, 0, stream>>>(
                    d_params + P.w_off[l], reinterpret_cast<bf16*>(pk + (dir ? P.p_tc_bwd : P.p_tc_fwd)[l - 1]), dir);
                BMND_LAUNCH_CHECK("pack_tc_kernel");
            }
        }
        const int64_t nout = static_cast<int64_t>(P.tc_out_bytes / 2);
        pack_tc_out_kernel<ND, C><<<launch_blocks(nout, 256), 256, 0, stream>>>(
            d_params + P.w_off[P.L - 1], reinterpret_cast<bf16*>(pk + P.p_tc_out));
        BMND_LAUNCH_CHECK("pack_tc_out_kernel");
        return BMND_OK;
    });
}

int32_t bmnd_pilotnet_forward(const BmndPilotNet* net, const void* d_packed, const float* d_noisy, float* d_pilot,
                              float* d_y, void* d_ws, uint64_t ws_bytes, uint64_t stream_u64) {
    clear_error();
    NetPlan P;
    if (int32_t rc = make_plan(net, P)) return rc;
    if (!d_packed || !d_noisy || (!d_pilot && !d_y) || !d_ws) return fail(BMND_ERR_INVALID_ARG, "null buffer");
    Bufs B = carve_ws(P, false, nullptr);
    if (ws_bytes < B.bytes) return fail(BMND_ERR_WORKSPACE, "pilot net workspace too small");
    B = carve_ws(P, false, d_ws);
    cudaStream_t stream = reinterpret_cast<cudaStream_t>(stream_u64);
    BMND_CUDA_TRY(cudaMemsetAsync(B.err, 0, sizeof(int), stream));
    const unsigned char* pk = static_cast<const unsigned char*>(d_packed);
    return dispatch(P, [&](auto nd, auto c) -> int32_t {
        return forward_impl<decltype(nd)::value, decltype(c)::value>(P, pk, d_noisy, d_pilot, d_y, B, false, stream);
    });
}

int32_t bmnd_pilotnet_gradient(const BmndPilotNet* net, const void* d_packed, const float* d_noisy,
                               const float* d_target, float* d_grad, double* d_loss, void* d_ws, uint64_t ws_bytes,
                               uint64_t stream_u64) {
    clear_error();
    NetPlan P;
    if (int32_t rc = make_plan(net, P)) return rc;
    if (!d_packed || !d_noisy || !d_target || !d_grad || !d_loss || !d_ws)
        return fail(BMND_ERR_INVALID_ARG, "null buffer");
    Bufs B = carve_ws(P, true, nullptr);
    if (ws_bytes < B.bytes) return fail(BMND_ERR_WORKSPACE, "pilot net workspace too small");
    B = carve_ws(P, true, d_ws);
    cudaStream_t stream = reinterpret_cast<cudaStream_t>(stream_u64);
    BMND_CUDA_TRY(cudaMemsetAsync(B.err, 0, sizeof(int), stream));
    const unsigned char* pk = static_cast<const unsigned char*>(d_packed);
    return dispatch(P, [&](auto nd, auto c) -> int32_t {
        return gradient_impl<decltype(nd)::value, decltype(c)::value>(P, pk, d_noisy, d_target, d_grad, d_loss, B,
                                                                      stream);
    });
}

int32_t bmnd_pilot_tile_deviance(int32_t ndim, int32_t batch, const int32_t* shape, int32_t edge,
                                 const float* d_noisy, const float* d_pilot, const float* d_table, int32_t n_table,
                                 float ln_mu0, float d_ln, double* d_out, uint64_t stream_u64) {
    clear_error();
    if ((ndim != 2 && ndim != 3) || batch < 1 || !shape || edge < 1 || n_table < 2 || !(d_ln > 0.0f))
        return fail(BMND_ERR_INVALID_ARG, "bad tile-deviance arguments");
    if (!d_noisy || !d_pilot || !d_table || !d_out) return fail(BMND_ERR_INVALID_ARG, "null buffer");
    NetGeo g;
    g.nb = batch;
    g.D = ndim == 3 ? shape[0] : 1;
    g.H = ndim == 3 ? shape[1] : shape[0];
    g.W = ndim == 3 ? shape[2] : shape[1];
    if (g.D < 1 || g.H < 1 || g.W < 1) return fail(BMND_ERR_INVALID_ARG, "shape must be positive");
    const int tx = (g.W + edge - 1) / edge, ty = (g.H + edge - 1) / edge;
    const int tz = ndim == 3 ? (g.D + edge - 1) / edge : 1;
    const int64_t tiles = static_cast<int64_t>(tx) * ty * tz * batch;
    if (tiles > 0x7fffffffLL) return fail(BMND_ERR_UNSUPPORTED, "too many tiles");
    cudaStream_t stream = reinterpret_cast<cudaStream_t>(stream_u64);
    tile_deviance_kernel<<<static_cast<unsigned>(tiles), 256, 0, stream>>>(d_noisy, d_pilot, g, edge, d_table, n_table,
                                                                          ln_mu0, d_ln, d_out, tx, ty, tz);
    BMND_LAUNCH_CHECK("tile_deviance_kernel");
    return BMND_OK;
}

int32_t bmnd_pilotnet_adam(int64_t n, float* d_params, const float* d_grad, float* d_m, float* d_v, int32_t step,
                           float lr, float beta1, float beta2, float eps, float clip_norm, double* d_sumsq,
                           uint64_t stream_u64) {
    clear_error();
    if (n < 0 || !d_params || !d_grad || !d_m || !d_v) return fail(BMND_ERR_INVALID_ARG, "bad Adam arguments");
    if (step < 1) return fail(BMND_ERR_INVALID_ARG, "Adam step counts from 1");
    if (clip_norm > 0.0f && !d_sumsq) return fail(BMND_ERR_INVALID_ARG, "clipping needs the norm scratch");
    const float bc1 = 1.0f - powf(beta1, static_cast<float>(step));
    const float bc2 = 1.0f - powf(beta2, static_cast<float>(step));
    cudaStream_t stream = reinterpret_cast<cudaStream_t>(stream_u64);
    if (clip_norm > 0.0f) {
        BMND_CUDA_TRY(cudaMemsetAsync(d_sumsq, 0, sizeof(double), stream));
        sumsq_kernel<<<launch_blocks(n, 256), 256, 0, stream>>>(d_grad, n, d_sumsq);
        BMND_LAUNCH_CHECK("sumsq_kernel");
    }
    adam_kernel<<<launch_blocks(n, 256), 256, 0, stream>>>(d_params, d_grad, d_m, d_v, n, lr, beta1, beta2, eps, bc1,
                                                           bc2, clip_norm, d_sumsq);
    BMND_LAUNCH_CHECK("adam_kernel");
    return BMND_OK;
}

}  // extern "C"
