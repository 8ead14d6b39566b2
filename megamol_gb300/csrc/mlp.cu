// Learned AO: a small MLP that stands in for the cone march.
//
// Input (60): two consecutive mip levels of the AO volume (the levels the cone's first samples read), each
// resampled as a 3x3x3 stencil of trilinear samples 1.5 texels apart centred on the particle's surface
// point (the stencil moves continuously with the point), then the unit normal and the surface point in
// normalised volume coordinates (the cones reach far into the volume, so AO also depends on where in the
// volume the point lies). Network 60 -> 64 -> 64 -> 1, SiLU, SiLU, sigmoid.
// Training: FP32 forward/backward kernels per CTA with a fixed-order reduction of the per-CTA gradients,
// then Adam; pairs come from the plain cone march. Inference: BF16 weights and features, FP32 accumulation
// on the 5th-generation tensor cores (tcgen05.mma, accumulators in TMEM), bias/activations in FP32. A
// particle whose features leave the training range (per feature, with a margin) falls back to the cone
// march.
// No reference counterpart: the reference evaluates AO only by the GLSL cone march / AOSphere taps.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "ao_internal.h"
#include "mlp_internal.h"
#include "p2v_common.cuh"

namespace p2v {

namespace {

__device__ __forceinline__ float silu(float a) {
    return a / (1.0f + __expf(-a));
}

// inference: silu(a) = a * sigmoid(a) with sigmoid(a) = 0.5 tanh(a / 2) + 0.5 from the hardware tanh
// approximation (one special-function operation instead of an exponential and a division; its ~2^-11
// relative error lies below the BF16 rounding the activations receive next)
__device__ __forceinline__ float tanh_approx(float x) {
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float silu_fast(float a) {
    const float h = 0.5f * a;
    return fmaf(h, tanh_approx(h), h);
}

__device__ __forceinline__ float sigmoidf_(float a) {
    return 1.0f / (1.0f + __expf(-a));
}

// 3x3x3 trilinear samples of one mip level at offsets 1.5 (k - 1) texels around normalised point u (the
// extent of a 4x4x4 stencil one texel apart, with 27 samples instead of 64), in the order kz*9 + ky*3 + kx.
// The level is a layered 2D texture of FP16 pairs: layer L holds z slices L - 1 (red) and L (green), so one
// bilinear fetch (GL LINEAR in x and y, CLAMP_TO_BORDER) returns both slices around a sample's z; the z
// interpolation runs in FP32 with the sample's own fraction; slices outside the level are 0, as the border.
// The 27 fetches do not depend on each other. The features feed a BF16 network, so the texture filter's
// 8-bit weight fractions sit below the features' own rounding; training pairs are extracted by the same
// code.
__device__ __forceinline__ void stencil27(unsigned long long tex, const float inv[3], int nz, float ux, float uy,
                                          float uz, float v[MLP_STENCIL]) {
    float px[3], py[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        px[k] = fmaf(1.5f * (float) (k - 1), inv[0], ux);
        py[k] = fmaf(1.5f * (float) (k - 1), inv[1], uy);
    }
#pragma unroll
    for (int kz = 0; kz < 3; ++kz) {
        // texel-space z of the sample minus the half texel: slices z0 and z0 + 1 live in layer z0 + 1
        const float zs = fmaf(uz, (float) nz, 1.5f * (float) (kz - 1) - 0.5f);
        const float z0f = floorf(zs);
        const float fz = zs - z0f;
        const int layer = (int) z0f + 1;
        const bool in = layer >= 0 && layer <= nz;
#pragma unroll
        for (int ky = 0; ky < 3; ++ky)
#pragma unroll
            for (int kx = 0; kx < 3; ++kx) {
                float2 t = make_float2(0.0f, 0.0f);
                if (in)
                    t = tex2DLayered<float2>((cudaTextureObject_t) tex, px[kx], py[ky], layer);
                v[kz * 9 + ky * 3 + kx] = t.x + fz * (t.y - t.x);
            }
    }
}

// Layer L of the paired texture = (slice L - 1, slice L) of level (dx, dy, dz), L in [0, dz].
__global__ void __launch_bounds__(256) fill_stencil_tex_kernel(const float* __restrict__ src, int dx, int dy, int dz,
                                                               float sat, unsigned long long surf) {
    const int64_t n = (int64_t) dx * dy * (dz + 1);
    for (int64_t i = blockIdx.x * (int64_t) blockDim.x + threadIdx.x; i < n; i += (int64_t) gridDim.x * blockDim.x) {
        const int x = (int) (i % dx), y = (int) ((i / dx) % dy), L = (int) (i / ((int64_t) dx * dy));
        float v[2];
#pragma unroll
        for (int c = 0; c < 2; ++c) {
            const int z = L - 1 + c;
            v[c] = 0.0f;
            if (z >= 0 && z < dz) {
                v[c] = src[((int64_t) z * dy + y) * dx + x];
                if (sat > 0.0f)
                    v[c] = fminf(fmaxf(v[c] * sat, 0.0f), 1.0f);
            }
        }
        const __half2 h = __floats2half2_rn(v[0], v[1]);
        surf2DLayeredwrite(*reinterpret_cast<const unsigned int*>(&h), (cudaSurfaceObject_t) surf,
                           x * (int) sizeof(__half2), y, L);
    }
}

// Surface point (normalised volume coordinates) and unit normal; false for a zero normal.
__device__ __forceinline__ bool mlp_point(const ConeParams& cp, const float4 p, const float4 nv, float u[3], float n[3]) {
    const float l2 = nv.x * nv.x + nv.y * nv.y + nv.z * nv.z;
    if (!(l2 > 0.0f))
        return false;
    const float il = rsqrtf(l2);
    n[0] = nv.x * il;
    n[1] = nv.y * il;
    n[2] = nv.z * il;
    const float pc[3] = {p.x, p.y, p.z};
#pragma unroll
    for (int a = 0; a < 3; ++a)
        u[a] = (pc[a] + p.w * n[a] - cp.bmin[a]) * cp.ibsize[a];
    return true;
}

// ---------------------------------------------------------------------------------------------
// training pairs: features of selected particles (sorted positions `sel`) and their cone-march AO
// ---------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(128) mlp_collect_kernel(const ConeParams cp, const uint32_t* __restrict__ order,
    const uint32_t* __restrict__ sel, uint32_t nsel, const float4* __restrict__ xyzr, const float4* __restrict__ nrm,
    const float* __restrict__ ao, float* __restrict__ X, float* __restrict__ T, uint32_t* __restrict__ kept) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nsel)
        return;
    const uint32_t o = order[sel[i]];
    float u[3], n[3];
    const float4 p = xyzr[o];
    if (!(isfinite(p.x) && isfinite(p.y) && isfinite(p.z) && p.w > 0.0f) || !mlp_point(cp, p, nrm[o], u, n)) {
        T[i] = -1.0f;  // marks a pair without features; compacted away on the host side
        return;
    }
    float* x = X + (size_t) i * MLP_IN;
    float v[MLP_STENCIL];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        stencil27(cp.stex[h], cp.sinv[h], cp.lv[cp.stencil_level + h].d[2], u[0], u[1], u[2], v);
        for (int k = 0; k < MLP_STENCIL; ++k)
            x[MLP_STENCIL * h + k] = v[k];
    }
    x[54] = n[0];
    x[55] = n[1];
    x[56] = n[2];
    x[57] = u[0];
    x[58] = u[1];
    x[59] = u[2];
    T[i] = ao[o];
    atomicAdd(kept, 1u);
}

// ---------------------------------------------------------------------------------------------
// training: forward + backward of TS samples per CTA, FP32; per-CTA gradient partials
// ---------------------------------------------------------------------------------------------
constexpr int TS = 32;
constexpr int TT = 256;

__global__ void __launch_bounds__(TT) mlp_train_kernel(const float* __restrict__ P, const float* __restrict__ X,
    const float* __restrict__ T, const uint32_t* __restrict__ idx, int nbatch, float inv_batch,
    float* __restrict__ partial, float* __restrict__ partial_loss) {
    extern __shared__ __align__(16) float sh[];
    float* W1 = sh;                          // [H][IN]
    float* W2 = W1 + MLP_H * MLP_IN;         // [H][H]
    float* Xs = W2 + MLP_H * MLP_H;          // [TS][IN]
    float* A1 = Xs + TS * MLP_IN;            // [TS][H]
    float* H1 = A1 + TS * MLP_H;
    float* A2 = H1 + TS * MLP_H;
    float* H2 = A2 + TS * MLP_H;
    float* D2 = H2 + TS * MLP_H;             // dL/dA2
    float* D1 = D2 + TS * MLP_H;             // dL/dA1
    float* dz = D1 + TS * MLP_H;             // [TS]
    const float* b1 = P + OFF_B1;
    const float* b2 = P + OFF_B2;
    const float* w3 = P + OFF_W3;
    const int t = threadIdx.x;
    const int s0 = blockIdx.x * TS;
    const int ns = min(TS, nbatch - s0);
    for (int k = t; k < MLP_H * MLP_IN; k += TT)
        W1[k] = P[OFF_W1 + k];
    for (int k = t; k < MLP_H * MLP_H; k += TT)
        W2[k] = P[OFF_W2 + k];
    for (int k = t; k < TS * MLP_IN; k += TT) {
        const int s = k / MLP_IN, i = k % MLP_IN;
        Xs[k] = s < ns ? X[(size_t) idx[s0 + s] * MLP_IN + i] : 0.0f;
    }
    __syncthreads();
    for (int o = t; o < TS * MLP_H; o += TT) {
        const int s = o / MLP_H, j = o % MLP_H;
        float a = b1[j];
        for (int i = 0; i < MLP_IN; ++i)
            a = fmaf(W1[j * MLP_IN + i], Xs[s * MLP_IN + i], a);
        A1[o] = a;
        H1[o] = silu(a);
    }
    __syncthreads();
    for (int o = t; o < TS * MLP_H; o += TT) {
        const int s = o / MLP_H, j = o % MLP_H;
        float a = b2[j];
        for (int i = 0; i < MLP_H; ++i)
            a = fmaf(W2[j * MLP_H + i], H1[s * MLP_H + i], a);
        A2[o] = a;
        H2[o] = silu(a);
    }
    __syncthreads();
    if (t < TS) {
        float l = 0.0f, d = 0.0f;
        if (t < ns) {
            float z = P[OFF_B3];
            for (int j = 0; j < MLP_H; ++j)
                z = fmaf(w3[j], H2[t * MLP_H + j], z);
            const float y = sigmoidf_(z);
            const float e = y - T[idx[s0 + t]];
            l = e * e;
            d = 2.0f * e * inv_batch * y * (1.0f - y);
        }
        dz[t] = d;
        // loss partial of this CTA (fixed-order warp reduction)
        for (int off = 16; off > 0; off >>= 1)
            l += __shfl_xor_sync(0xffffffffu, l, off);
        if (t == 0)
            partial_loss[blockIdx.x] = l;
    }
    __syncthreads();
    float* G = partial + (size_t) blockIdx.x * MLP_NPARAM;
    for (int o = t; o < TS * MLP_H; o += TT) {
        const int s = o / MLP_H, j = o % MLP_H;
        const float a = A2[o];
        const float sg = sigmoidf_(a);
        D2[o] = dz[s] * w3[j] * sg * (1.0f + a * (1.0f - sg));
    }
    if (t < MLP_H) {
        float g = 0.0f;
        for (int s = 0; s < TS; ++s)
            g = fmaf(dz[s], H2[s * MLP_H + t], g);
        G[OFF_W3 + t] = g;
    } else if (t == MLP_H) {
        float g = 0.0f;
        for (int s = 0; s < TS; ++s)
            g += dz[s];
        G[OFF_B3] = g;
    }
    __syncthreads();
    for (int o = t; o < MLP_H * MLP_H; o += TT) {
        const int j = o / MLP_H, i = o % MLP_H;
        float g = 0.0f;
        for (int s = 0; s < TS; ++s)
            g = fmaf(D2[s * MLP_H + j], H1[s * MLP_H + i], g);
        G[OFF_W2 + o] = g;
    }
    if (t < MLP_H) {
        float g = 0.0f;
        for (int s = 0; s < TS; ++s)
            g += D2[s * MLP_H + t];
        G[OFF_B2 + t] = g;
    }
    for (int o = t; o < TS * MLP_H; o += TT) {
        const int s = o / MLP_H, i = o % MLP_H;
        float g = 0.0f;
        for (int j = 0; j < MLP_H; ++j)
            g = fmaf(D2[s * MLP_H + j], W2[j * MLP_H + i], g);
        const float a = A1[o];
        const float sg = sigmoidf_(a);
        D1[o] = g * sg * (1.0f + a * (1.0f - sg));
    }
    __syncthreads();
    for (int o = t; o < MLP_H * MLP_IN; o += TT) {
        const int j = o / MLP_IN, i = o % MLP_IN;
        float g = 0.0f;
        for (int s = 0; s < TS; ++s)
            g = fmaf(D1[s * MLP_H + j], Xs[s * MLP_IN + i], g);
        G[OFF_W1 + o] = g;
    }
    if (t < MLP_H) {
        float g = 0.0f;
        for (int s = 0; s < TS; ++s)
            g += D1[s * MLP_H + t];
        G[OFF_B1 + t] = g;
    }
}

// gradient = sum of the CTA partials in CTA order (deterministic)
__global__ void __launch_bounds__(256) mlp_reduce_kernel(const float* __restrict__ partial, int nblk,
    const float* __restrict__ partial_loss, float* __restrict__ grad, float* __restrict__ loss) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < MLP_NPARAM) {
        float g = 0.0f;
        for (int b = 0; b < nblk; ++b)
            g += partial[(size_t) b * MLP_NPARAM + p];
        grad[p] = g;
    }
    if (p == 0) {
        float l = 0.0f;
        for (int b = 0; b < nblk; ++b)
            l += partial_loss[b];
        *loss = l;
    }
}

__global__ void __launch_bounds__(256) mlp_adam_kernel(float* __restrict__ P, const float* __restrict__ g,
    float* __restrict__ m, float* __restrict__ v, float lr, float b1, float b2, float eps, float c1, float c2) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= MLP_NPARAM)
        return;
    const float gp = g[p];
    const float mp = b1 * m[p] + (1.0f - b1) * gp;
    const float vp = b2 * v[p] + (1.0f - b2) * gp * gp;
    m[p] = mp;
    v[p] = vp;
    P[p] -= lr * (mp * c1) / (sqrtf(vp * c2) + eps);
}

// FP32 forward of given features (validation), one thread per sample
__global__ void __launch_bounds__(128) mlp_forward_f32_kernel(const float* __restrict__ P, const float* __restrict__ X,
    const uint32_t* __restrict__ idx, uint32_t n, float* __restrict__ y) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n)
        return;
    const float* x = X + (size_t) (idx ? idx[s] : s) * MLP_IN;
    float h1[MLP_H];
    for (int j = 0; j < MLP_H; ++j) {
        float a = P[OFF_B1 + j];
        for (int i = 0; i < MLP_IN; ++i)
            a = fmaf(P[OFF_W1 + j * MLP_IN + i], x[i], a);
        h1[j] = silu(a);
    }
    float z = P[OFF_B3];
    for (int j = 0; j < MLP_H; ++j) {
        float a = P[OFF_B2 + j];
        for (int i = 0; i < MLP_H; ++i)
            a = fmaf(P[OFF_W2 + j * MLP_H + i], h1[i], a);
        z = fmaf(P[OFF_W3 + j], silu(a), z);
    }
    y[s] = sigmoidf_(z);
}

// per-feature minimum and maximum over the rows idx[0..n) (one block per feature, fixed-order reduction)
__global__ void __launch_bounds__(256) mlp_range_kernel(const float* __restrict__ X, const uint32_t* __restrict__ idx,
    uint32_t n, float margin, float* __restrict__ lo, float* __restrict__ hi) {
    __shared__ float smin[256], smax[256];
    const int f = blockIdx.x;
    float mn = INFINITY, mx = -INFINITY;
    for (uint32_t s = threadIdx.x; s < n; s += blockDim.x) {
        const float v = X[(size_t) idx[s] * MLP_IN + f];
        mn = fminf(mn, v);
        mx = fmaxf(mx, v);
    }
    smin[threadIdx.x] = mn;
    smax[threadIdx.x] = mx;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            smin[threadIdx.x] = fminf(smin[threadIdx.x], smin[threadIdx.x + o]);
            smax[threadIdx.x] = fmaxf(smax[threadIdx.x], smax[threadIdx.x + o]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const float w = smax[0] - smin[0];
        lo[f] = smin[0] - margin * w;
        hi[f] = smax[0] + margin * w;
    }
}

// ---------------------------------------------------------------------------------------------
// inference weights: BF16 copies of W1 (its columns at the K positions of mlp_kpos, zeros between) and W2
// ---------------------------------------------------------------------------------------------
__global__ void mlp_pack_kernel(const float* __restrict__ P, __nv_bfloat16* __restrict__ w1h,
    __nv_bfloat16* __restrict__ w2h) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < MLP_H * MLP_KP; k += gridDim.x * blockDim.x) {
        const int j = k / MLP_KP, i = k % MLP_KP;
        const int f = mlp_feature_at(i);
        w1h[k] = __float2bfloat16_rn(f >= 0 ? P[OFF_W1 + j * MLP_IN + f] : 0.0f);
    }
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < MLP_H * MLP_H; k += gridDim.x * blockDim.x)
        w2h[k] = __float2bfloat16_rn(P[OFF_W2 + k]);
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}

// ---------------------------------------------------------------------------------------------
// Inference on the 5th-generation tensor cores (tcgen05). One CTA of 256 threads takes 128 particles per
// tile. Threads t and t + 128 extract the two stencil levels of particle t straight into the A tile (BF16,
// canonical no-swizzle K-major layout in shared memory; each thread's features fill whole 16-byte chunks, see
// mlp_kpos); one thread issues the layer-1 MMAs (M = 128, N = 64, K = 80) into 64 TMEM columns and commits
// them to an mbarrier. The epilogue reads TMEM
// (warp w: lanes 32 (w % 4).., columns 32 (w / 4)..), adds the bias, applies SiLU and writes the hidden
// layer back into the A tile as layer 2's A operand; layer 2 (K = 64) reuses the TMEM columns, and its
// epilogue finishes layer 3 (64 -> 1) in FP32 with the sigmoid. The accumulators never occupy registers,
// so four CTAs (32 warps, 64 registers each: more warps hide the texture latency better than the few
// spilled registers cost) stay resident per SM. Every mbarrier wait
// is bounded: on timeout the CTA records ERR_MMA_TIMEOUT, drains its MMAs (bounded) and frees TMEM.
// ---------------------------------------------------------------------------------------------
namespace tc {
constexpr int THREADS = 256;
constexpr int M = 128;                         // particles per tile (MMA M, TMEM lanes)
constexpr int KCH1 = MLP_KP / 8;               // 16-byte core-matrix columns of layer 1's K (10)
constexpr int KCH2 = MLP_H / 8;                // of layer 2's K (8)
constexpr int SBO1 = KCH1 * 128;               // bytes between 8-row core-matrix groups, layer 1
constexpr int SBO2 = KCH2 * 128;               // layer 2
constexpr int A_BYTES = (M / 8) * SBO1;        // 20480: features; later the hidden layer (16384 B)
constexpr int W1_BYTES = (MLP_H / 8) * SBO1;   // 10240
constexpr int W2_BYTES = (MLP_H / 8) * SBO2;   // 8192
constexpr int DYN_SMEM = A_BYTES + W1_BYTES + W2_BYTES;
constexpr uint32_t TMEM_COLS = 64;
constexpr uint32_t WAIT_LIMIT = 1u << 20;
// instruction descriptor, kind::f16: D = F32 (bits 4-5), A = B = BF16 (bits 7-9, 10-12), both K-major,
// N >> 3 at bits 17-22, M >> 4 at bits 24-28
constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t) (MLP_H >> 3) << 17) |
                           ((uint32_t) (M >> 4) << 24);
}  // namespace tc

// byte offset of element (row, k) in the canonical K-major layout: 8x8 BF16 core matrices of 128 B (row r
// of a core matrix at 16 r), core matrices along K 128 B apart, 8-row groups `sbo` bytes apart
__device__ __forceinline__ uint32_t canon_off(int row, int k, int sbo) {
    return (uint32_t) ((row >> 3) * sbo + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

// shared-memory matrix descriptor: start address, leading (K) byte offset, stride (8-row) byte offset,
// bits 46-48 = 0b001, base offset 0, no swizzle
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t) ((saddr >> 4) & 0x3FFFu) | ((uint64_t) ((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t) ((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t) __cvta_generic_to_shared(p);
}

__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(tc::IDESC), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void umma_commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
                 : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void tc_fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void fence_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// bounded wait for phase `phase` of an mbarrier; false when the budget ran out
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t phase) {
    for (uint32_t i = 0; i < tc::WAIT_LIMIT; ++i) {
        uint32_t ok;
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.b32 %0, 1, 0, p;\n}\n"
            : "=r"(ok)
            : "r"(mbar), "r"(phase)
            : "memory");
        if (ok)
            return true;
    }
    return false;
}

// 32 consecutive TMEM columns of this thread's lane
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]),
          "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]),
          "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int j = 0; j < 32; ++j)
        v[j] = __uint_as_float(r[j]);
}

__device__ __forceinline__ void st_shared_v4(uint8_t* p, uint32_t a, uint32_t b, uint32_t c, uint32_t d) {
    *reinterpret_cast<uint4*>(p) = make_uint4(a, b, c, d);
}

template<bool FEATURES_IN>
__global__ void __launch_bounds__(tc::THREADS, 4) mlp_infer_tc_kernel(const MlpInferArgs args, const ConeParams cp) {
    extern __shared__ __align__(1024) uint8_t tc_smem[];
    uint8_t* sA = tc_smem;
    uint8_t* sW1 = tc_smem + tc::A_BYTES;
    uint8_t* sW2 = sW1 + tc::W1_BYTES;
    __shared__ float sB1[MLP_H], sB2[MLP_H], sW3[MLP_H];
    // training range per feature pair, rounded outward to BF16 (the features are checked as the BF16 values
    // the network sees)
    __shared__ __nv_bfloat162 sLo2[MLP_KP / 2], sHi2[MLP_KP / 2];
    __shared__ __align__(8) uint64_t s_mbar;
    __shared__ uint32_t s_tmem;
    __shared__ float s_part[tc::M];
    __shared__ uint32_t s_flag[tc::M];

    const int t = threadIdx.x;
    const int row = t & (tc::M - 1), half = t >> 7;
    const int q = (t >> 5) & 3;
    // weights into the canonical layout (16-byte chunks: 8 consecutive k of one output neuron)
    for (int i = t; i < MLP_H * tc::KCH1; i += tc::THREADS) {
        const int n = i / tc::KCH1, c = i % tc::KCH1;
        *reinterpret_cast<uint4*>(sW1 + canon_off(n, 8 * c, tc::SBO1)) =
            *reinterpret_cast<const uint4*>(args.w1h + n * MLP_KP + 8 * c);
    }
    for (int i = t; i < MLP_H * tc::KCH2; i += tc::THREADS) {
        const int n = i / tc::KCH2, c = i % tc::KCH2;
        *reinterpret_cast<uint4*>(sW2 + canon_off(n, 8 * c, tc::SBO2)) =
            *reinterpret_cast<const uint4*>(args.w2h + n * MLP_H + 8 * c);
    }
    for (int k = t; k < MLP_H; k += tc::THREADS) {
        sB1[k] = args.P[OFF_B1 + k];
        sB2[k] = args.P[OFF_B2 + k];
        sW3[k] = args.P[OFF_W3 + k];
    }
    for (int w = t; w < MLP_KP / 2; w += tc::THREADS) {
        float lo[2], hi[2];
        for (int e = 0; e < 2; ++e) {
            const int f = mlp_feature_at(2 * w + e);
            lo[e] = (args.lo && f >= 0) ? args.lo[f] : -INFINITY;
            hi[e] = (args.hi && f >= 0) ? args.hi[f] : INFINITY;
        }
        sLo2[w] = __halves2bfloat162(__float2bfloat16_rd(lo[0]), __float2bfloat16_rd(lo[1]));
        sHi2[w] = __halves2bfloat162(__float2bfloat16_ru(hi[0]), __float2bfloat16_ru(hi[1]));
    }
    const uint32_t mbar = smem_u32(&s_mbar);
    if (t == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (t < 32) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&s_tmem)),
                     "r"(tc::TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_async_smem();  // the weight tiles were written by ordinary stores; the MMA reads them
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = s_tmem;
    const uint32_t taddr = tmem + ((uint32_t) (32 * q) << 16) + (uint32_t) (32 * half);
    const uint32_t a_s = smem_u32(sA), w1_s = smem_u32(sW1), w2_s = smem_u32(sW2);
    const float b3 = args.P[OFF_B3];
    const bool check = args.lo != nullptr && args.hi != nullptr;
    uint32_t phase = 0;
    bool failed = false;
    const uint32_t ntiles = (args.n + tc::M - 1) / tc::M;
    for (uint32_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const uint32_t pi = tile * tc::M + row;
        bool valid = pi < args.n;
        bool oor = false;
        uint32_t o = 0;
        // ---- features: this thread's half of row `row` ----
        auto in_range = [&](int w, __nv_bfloat162 v2) { return __hble2(sLo2[w], v2) && __hble2(v2, sHi2[w]); };
        if (FEATURES_IN) {
            // half h writes the K chunks [5 h, 5 h + 5)
#pragma unroll 1
            for (int c = 0; c < tc::KCH1 / 2; ++c) {
                const int k0 = 8 * (c + half * (tc::KCH1 / 2));
                uint32_t pk[4];
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    const int k = k0 + 2 * e;
                    const int fa = mlp_feature_at(k), fb = mlp_feature_at(k + 1);
                    const float a = (valid && fa >= 0) ? args.X[(size_t) pi * MLP_IN + fa] : 0.0f;
                    const float b = (valid && fb >= 0) ? args.X[(size_t) pi * MLP_IN + fb] : 0.0f;
                    const __nv_bfloat162 v2 = __floats2bfloat162_rn(a, b);
                    if (check && valid)
                        oor |= !in_range(k >> 1, v2);
                    pk[e] = *reinterpret_cast<const uint32_t*>(&v2);
                }
                st_shared_v4(sA + canon_off(row, k0, tc::SBO1), pk[0], pk[1], pk[2], pk[3]);
            }
        } else {
            float u[3] = {0, 0, 0}, nn[3] = {0, 0, 0};
            if (valid) {
                o = args.order ? args.order[pi] : pi;
                const float4 p = args.xyzr[o];
                valid = isfinite(p.x) && isfinite(p.y) && isfinite(p.z) && p.w > 0.0f &&
                        mlp_point(cp, p, args.nrm[o], u, nn);
            }
            // K 64..79 first (the normal and the position are then no longer needed): the normal, the
            // position and zero padding (chunk 8 on half 0, chunk 9 on half 1)
            if (half == 0) {
                const __nv_bfloat162 n01 = __floats2bfloat162_rn(nn[0], nn[1]);
                const __nv_bfloat162 n2u0 = __floats2bfloat162_rn(nn[2], u[0]);
                const __nv_bfloat162 u12 = __floats2bfloat162_rn(u[1], u[2]);
                st_shared_v4(sA + canon_off(row, 64, tc::SBO1), *reinterpret_cast<const uint32_t*>(&n01),
                             *reinterpret_cast<const uint32_t*>(&n2u0), *reinterpret_cast<const uint32_t*>(&u12), 0u);
                if (valid && check)
                    oor |= !(in_range(32, n01) && in_range(33, n2u0) && in_range(34, u12));
            } else {
                st_shared_v4(sA + canon_off(row, 72, tc::SBO1), 0u, 0u, 0u, 0u);
            }
            // this half's stencil level: K 32 h .. 32 h + 26, padded with zeros to 32 h + 31 (chunks 4 h .. 4 h + 3)
            float sv[MLP_STENCIL];
            if (valid)
                stencil27(cp.stex[half], cp.sinv[half], cp.lv[cp.stencil_level + half].d[2], u[0], u[1], u[2], sv);
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                uint32_t pk[4];
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    const int j = 8 * c + 2 * e;
                    const float a = (valid && j < MLP_STENCIL) ? sv[j] : 0.0f;
                    const float b = (valid && j + 1 < MLP_STENCIL) ? sv[j + 1] : 0.0f;
                    const __nv_bfloat162 v2 = __floats2bfloat162_rn(a, b);
                    if (check && valid)
                        oor |= !in_range(16 * half + 4 * c + e, v2);
                    pk[e] = *reinterpret_cast<const uint32_t*>(&v2);
                }
                st_shared_v4(sA + canon_off(row, 32 * half + 8 * c, tc::SBO1), pk[0], pk[1], pk[2], pk[3]);
            }
            oor = oor && valid;
        }
        if (half == 1)
            s_flag[row] = oor ? 1u : 0u;
        fence_async_smem();
        tc_fence_before();
        __syncthreads();
        if (half == 0)
            oor = oor || s_flag[row] != 0u;
        // ---- layer 1: D[128 x 64] = A[128 x 80] W1^T ----
        if (t == 0) {
            tc_fence_after();
#pragma unroll
            for (int kk = 0; kk < tc::KCH1 / 2; ++kk)
                umma_bf16(tmem, umma_desc(a_s + 256u * kk, 128u, tc::SBO1), umma_desc(w1_s + 256u * kk, 128u, tc::SBO1),
                          kk > 0 ? 1u : 0u);
            umma_commit(mbar);
        }
        failed = !mbar_wait(mbar, phase);
        phase ^= 1u;
        tc_fence_after();
        if (__syncthreads_or(failed))
            break;
        float v[32];
        tmem_ld32(taddr, v);
        // hidden layer 1 -> A tile (K = 64 layout): columns 32 half .. 32 half + 31 of row `row`
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            uint32_t pk[4];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int j = 8 * c + 2 * e;
                pk[e] = pack_bf16(silu_fast(v[j] + sB1[32 * half + j]), silu_fast(v[j + 1] + sB1[32 * half + j + 1]));
            }
            st_shared_v4(sA + canon_off(row, 32 * half + 8 * c, tc::SBO2), pk[0], pk[1], pk[2], pk[3]);
        }
        fence_async_smem();
        tc_fence_before();
        __syncthreads();
        // ---- layer 2: D[128 x 64] = H[128 x 64] W2^T (same TMEM columns) ----
        if (t == 0) {
            tc_fence_after();
#pragma unroll
            for (int kk = 0; kk < tc::KCH2 / 2; ++kk)
                umma_bf16(tmem, umma_desc(a_s + 256u * kk, 128u, tc::SBO2), umma_desc(w2_s + 256u * kk, 128u, tc::SBO2),
                          kk > 0 ? 1u : 0u);
            umma_commit(mbar);
        }
        failed = !mbar_wait(mbar, phase);
        phase ^= 1u;
        tc_fence_after();
        if (__syncthreads_or(failed))
            break;
        tmem_ld32(taddr, v);
        // ---- layer 3 (64 -> 1) in FP32: each half sums its 32 columns ----
        float z = 0.0f;
#pragma unroll
        for (int j = 0; j < 32; ++j)
            z = fmaf(silu_fast(v[j] + sB2[32 * half + j]), sW3[32 * half + j], z);
        if (half == 1)
            s_part[row] = z;
        tc_fence_before();
        __syncthreads();
        if (half == 0 && pi < args.n) {
            const float y = sigmoidf_(z + s_part[row] + b3);
            const uint32_t oo = FEATURES_IN ? pi : o;
            if (!FEATURES_IN && !valid) {
                args.y[oo] = 1.0f;  // no normal / invalid particle: unoccluded, as the cone march
            } else if (oor && args.fallback) {
                args.fallback[atomicAdd(args.nfallback, 1u)] = oo;
                if (FEATURES_IN)
                    args.y[oo] = y;
            } else {
                args.y[oo] = y;
            }
        }
    }
    if (failed) {
        if (t == 0 && args.err)
            atomicOr(args.err, ERR_MMA_TIMEOUT);
        // drain: the phase that timed out may still complete; wait for it once more (bounded)
        mbar_wait(mbar, phase ^ 1u);
    }
    tc_fence_before();
    __syncthreads();
    if (t < 32) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(tc::TMEM_COLS)
                     : "memory");
    }
}

}  // namespace

size_t mlp_train_smem_bytes() {
    return sizeof(float) * (MLP_H * MLP_IN + MLP_H * MLP_H + TS * MLP_IN + 6 * TS * MLP_H + TS);
}

cudaError_t StencilTex::ensure(const int dims[3]) {
    if (arr && d[0] == dims[0] && d[1] == dims[1] && d[2] == dims[2])
        return cudaSuccess;
    release();
    cudaChannelFormatDesc fmt = cudaCreateChannelDescHalf2();
    // dims[2] + 1 layers of slice pairs (slice L - 1, slice L)
    cudaError_t e = cudaMalloc3DArray(&arr, &fmt, make_cudaExtent(dims[0], dims[1], dims[2] + 1),
                                      cudaArrayLayered | cudaArraySurfaceLoadStore);
    if (e != cudaSuccess) {
        arr = nullptr;
        return e;
    }
    cudaResourceDesc rd{};
    rd.resType = cudaResourceTypeArray;
    rd.res.array.array = arr;
    cudaTextureDesc td{};
    for (int a = 0; a < 3; ++a)
        td.addressMode[a] = cudaAddressModeBorder;  // CLAMP_TO_BORDER with border colour 0
    td.filterMode = cudaFilterModeLinear;
    td.readMode = cudaReadModeElementType;
    td.normalizedCoords = 1;
    cudaTextureObject_t to = 0;
    cudaSurfaceObject_t so = 0;
    if ((e = cudaCreateTextureObject(&to, &rd, &td, nullptr)) != cudaSuccess ||
        (e = cudaCreateSurfaceObject(&so, &rd)) != cudaSuccess) {
        if (to)
            cudaDestroyTextureObject(to);
        cudaFreeArray(arr);
        arr = nullptr;
        return e;
    }
    tex = to;
    surf = so;
    for (int a = 0; a < 3; ++a)
        d[a] = dims[a];
    return cudaSuccess;
}

void StencilTex::release() {
    if (tex)
        cudaDestroyTextureObject((cudaTextureObject_t) tex);
    if (surf)
        cudaDestroySurfaceObject((cudaSurfaceObject_t) surf);
    if (arr)
        cudaFreeArray(arr);
    arr = nullptr;
    tex = surf = 0;
    d[0] = d[1] = d[2] = 0;
}

cudaError_t launch_fill_stencil_tex(const ConeLevel& L, float sat, const StencilTex& t, cudaStream_t st) {
    const int64_t n = (int64_t) L.d[0] * L.d[1] * (L.d[2] + 1);
    const unsigned grd = (unsigned) std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 16));
    fill_stencil_tex_kernel<<<grd, 256, 0, st>>>(L.v, L.d[0], L.d[1], L.d[2], sat, t.surf);
    return cudaGetLastError();
}

cudaError_t launch_mlp_collect(const ConeParams& cp, const uint32_t* order, const uint32_t* sel, uint32_t nsel,
    const float4* xyzr, const float4* nrm, const float* ao, float* X, float* T, uint32_t* kept, cudaStream_t st) {
    if (nsel == 0)
        return cudaSuccess;
    mlp_collect_kernel<<<ceil_div(nsel, 128), 128, 0, st>>>(cp, order, sel, nsel, xyzr, nrm, ao, X, T, kept);
    return cudaGetLastError();
}

cudaError_t launch_mlp_train_step(const float* P, const float* X, const float* T, const uint32_t* idx, int nbatch,
    float* partial, float* partial_loss, float* grad, float* loss, cudaStream_t st) {
    const int nblk = (nbatch + TS - 1) / TS;
    const size_t smem = mlp_train_smem_bytes();
    cudaError_t e = cudaFuncSetAttribute(mlp_train_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem);
    if (e != cudaSuccess)
        return e;
    mlp_train_kernel<<<nblk, TT, smem, st>>>(P, X, T, idx, nbatch, 1.0f / (float) nbatch, partial, partial_loss);
    mlp_reduce_kernel<<<ceil_div(MLP_NPARAM, 256), 256, 0, st>>>(partial, nblk, partial_loss, grad, loss);
    return cudaGetLastError();
}

cudaError_t launch_mlp_adam(float* P, const float* g, float* m, float* v, float lr, float b1, float b2, float eps,
    int step, cudaStream_t st) {
    const float c1 = 1.0f / (1.0f - powf(b1, (float) step));
    const float c2 = 1.0f / (1.0f - powf(b2, (float) step));
    mlp_adam_kernel<<<ceil_div(MLP_NPARAM, 256), 256, 0, st>>>(P, g, m, v, lr, b1, b2, eps, c1, c2);
    return cudaGetLastError();
}

cudaError_t launch_mlp_forward_f32(const float* P, const float* X, const uint32_t* idx, uint32_t n, float* y,
    cudaStream_t st) {
    if (n == 0)
        return cudaSuccess;
    mlp_forward_f32_kernel<<<ceil_div(n, 128), 128, 0, st>>>(P, X, idx, n, y);
    return cudaGetLastError();
}

cudaError_t launch_mlp_range(const float* X, const uint32_t* idx, uint32_t n, float margin, float* lo, float* hi,
    cudaStream_t st) {
    mlp_range_kernel<<<MLP_IN, 256, 0, st>>>(X, idx, n, margin, lo, hi);
    return cudaGetLastError();
}

cudaError_t launch_mlp_pack(const float* P, __nv_bfloat16* w1h, __nv_bfloat16* w2h, cudaStream_t st) {
    mlp_pack_kernel<<<32, 256, 0, st>>>(P, w1h, w2h);
    return cudaGetLastError();
}

cudaError_t launch_mlp_infer(const MlpInferArgs& a, const ConeParams& cp, bool features_in, int sms, cudaStream_t st) {
    if (a.n == 0)
        return cudaSuccess;
    static_assert(tc::DYN_SMEM <= 227 * 1024, "tensor-core tile does not fit in shared memory");
    const uint32_t ntiles = (a.n + tc::M - 1) / tc::M;
    // four resident CTAs per SM (41 KB of shared memory and 64 registers per thread each; 4 x 64 TMEM
    // columns of 512): one wave
    const unsigned grid = (unsigned) std::min<uint32_t>(ntiles, (uint32_t) sms * 4);
    cudaError_t e;
    if (features_in) {
        e = cudaFuncSetAttribute(mlp_infer_tc_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, tc::DYN_SMEM);
        if (e == cudaSuccess)
            mlp_infer_tc_kernel<true><<<grid, tc::THREADS, tc::DYN_SMEM, st>>>(a, cp);
    } else {
        e = cudaFuncSetAttribute(mlp_infer_tc_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, tc::DYN_SMEM);
        if (e == cudaSuccess)
            mlp_infer_tc_kernel<false><<<grid, tc::THREADS, tc::DYN_SMEM, st>>>(a, cp);
    }
    return e != cudaSuccess ? e : cudaGetLastError();
}

}  // namespace p2v
