// Learned AO: a small MLP that stands in for the cone march.
//
// Input (54): the cone march's own visibility samples, read by the texture units: for each of the 8 cones, in
// the particle's MDAO cone frame, the volume at 6 of the march's steps (spread evenly over the step table),
// each at the step's own mip level (LINEAR_MIPMAP_LINEAR between the two levels around its lod); then the
// unit normal and the surface point in normalised volume coordinates. Network 54 -> 64 -> 64 -> 1, SiLU,
// SiLU, sigmoid: it learns how the march's 32 steps, early exit and cone average turn these samples into AO.
// Training: FP32 forward/backward kernels per CTA with a fixed-order reduction of the per-CTA gradients,
// then Adam; pairs come from the plain cone march. Inference: BF16 weights and features, FP32 accumulation
// on the 5th-generation tensor cores (tcgen05.mma, accumulators in TMEM), bias/activations in FP32. A
// particle whose features leave the training range (per feature, with a margin) falls back to the cone
// march.
// No reference counterpart: the reference evaluates AO only by the GLSL cone march / AOSphere taps
// (plugins/moldyn_gl/shaders/moldyn_gl/sphere_renderer/inc/mdao_deferred_fragment_ambocc.inc.glsl:30-51 is the
// march whose samples the features are).
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "ao_internal.h"
#include "cone_device.cuh"
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

// GL LINEAR sample of one mip level (dz slices) at normalised point q (CLAMP_TO_BORDER with border 0, texel
// centres at (i + 0.5) / N) through its paired-slice layered texture: layer z holds the texels of slices z
// and z + 1 (0 past the last) as two 8-bit UNORM channels (the MDAO volume's own R8 format), so one bilinear
// fetch returns both slices around the sample, x and y weighted by the texture units with 8-bit fractions;
// the z weight is applied in FP32. The features feed a BF16 network and training pairs are extracted by the
// same code (measured on the CPU: the same test RMSE as FP32 texels on the LJ, uniform and mixed-phase frames).
__device__ __forceinline__ float feature_tex_sample(unsigned long long tex, float fdz, int dz, float qx, float qy,
                                                    float qz) {
    const float cz = fmaf(qz, fdz, -0.5f);
    const float z0f = floorf(cz);
    const float fz = cz - z0f;
    const int z0 = (int) z0f;
    // branch-free (every sample fetches, so the fetches of a particle issue back to back): the layer clamped
    // into the texture; below slice 0 the pair is (border 0, slice 0), past the last slice (0, 0)
    const float2 p = tex2DLayered<float2>((cudaTextureObject_t) tex, qx, qy, min(max(z0, 0), dz - 1));
    const bool inside = z0 >= 0 && z0 < dz;
    const float lo = inside ? p.x : 0.0f;
    const float hi = inside ? p.y : (z0 == -1 ? p.x : 0.0f);
    return fmaf(fz, hi - lo, lo);
}

// Feature sample j of a cone with direction dir from normalised point u: the march's step fstep[j] at its
// own lod, blended linearly between the two levels around it (the branch depends on j only, so it is uniform
// across the warp).
__device__ __forceinline__ float feature_sample(const ConeParams& cp, const float dir[3], const float u[3], int j) {
    const int k = cp.fstep[j];
    const float t = cp.t[k], lod = cp.lod[k];
    const float qx = fmaf(t, dir[0], u[0]), qy = fmaf(t, dir[1], u[1]), qz = fmaf(t, dir[2], u[2]);
    const int l0 = min((int) lod, cp.nlevels - 1);
    const float fr = lod - (float) l0;
    float v = feature_tex_sample(cp.ftex[l0], cp.lv[l0].fd[2], cp.lv[l0].d[2], qx, qy, qz);
    if (fr > 0.0f && l0 + 1 < cp.nlevels)
        v = fmaf(fr, feature_tex_sample(cp.ftex[l0 + 1], cp.lv[l0 + 1].fd[2], cp.lv[l0 + 1].d[2], qx, qy, qz) - v, v);
    return v;
}

// The MLP_FSTEPS features of cone c, written to v[0 .. MLP_FSTEPS).
__device__ __forceinline__ void cone_features(const ConeParams& cp, int c, const float u[3], const float nn[3],
                                              const float ex[3], const float ez[3], float* v) {
    float dir[3];
    cone_dir(cp, c, ex, nn, ez, dir);
#pragma unroll
    for (int j = 0; j < MLP_FSTEPS; ++j)
        v[j] = feature_sample(cp, dir, u, j);
}

// Surface point in normalised volume coordinates, unit normal and cone frame of a particle (the plain march's
// own, cone_device.cuh); false for an invalid particle (non-finite position, radius <= 0) or a zero normal.
__device__ __forceinline__ bool particle_frame(const ConeParams& cp, const float4 p, const float4 nv, float u[3],
                                               float nn[3], float ex[3], float ez[3]) {
    if (!(isfinite(p.x) && isfinite(p.y) && isfinite(p.z) && p.w > 0.0f))
        return false;
    float x[3];
    if (!surface_point(p, nv, x, nn))
        return false;
    cone_frame(cp, x, nn, u, ex, ez);
    return true;
}

// Level (dx, dy, dz) into its paired-slice layered texture: texel (x, y) of layer z = the 8-bit UNORM values
// of slices z and z + 1 (0 past the last slice), each texel clamped to [0, 1] (level-0 saturation
// clamp(v * sat, 0, 1) applied first when sat > 0).
__device__ __forceinline__ unsigned char unorm8(float v, float sat) {
    if (sat > 0.0f)
        v = v * sat;
    return (unsigned char) __float2uint_rn(fminf(fmaxf(v, 0.0f), 1.0f) * 255.0f);
}

__global__ void __launch_bounds__(256) fill_feature_tex_kernel(const float* __restrict__ src, int dx, int dy, int dz,
                                                               float sat, unsigned long long surf) {
    const int64_t n = (int64_t) dx * dy * dz;
    const int64_t plane = (int64_t) dx * dy;
    for (int64_t i = blockIdx.x * (int64_t) blockDim.x + threadIdx.x; i < n; i += (int64_t) gridDim.x * blockDim.x) {
        const int x = (int) (i % dx), y = (int) ((i / dx) % dy), z = (int) (i / plane);
        const unsigned char lo = unorm8(src[i], sat);
        const unsigned char hi = z + 1 < dz ? unorm8(src[i + plane], sat) : (unsigned char) 0;
        surf2DLayeredwrite(make_uchar2(lo, hi), (cudaSurfaceObject_t) surf, x * (int) sizeof(uchar2), y, z);
    }
}

// ---------------------------------------------------------------------------------------------
// training pairs: features of selected particles (sorted positions `sel`, read from the sorted copies of the
// positions and normals) and their cone-march AO (input order)
// ---------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(128) mlp_collect_kernel(const ConeParams cp, const uint32_t* __restrict__ order,
    const uint32_t* __restrict__ sel, uint32_t nsel, const float4* __restrict__ xyzr, const float4* __restrict__ nrm,
    const float* __restrict__ ao, float* __restrict__ X, float* __restrict__ T, uint32_t* __restrict__ kept) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nsel)
        return;
    const uint32_t js = sel[i];  // sorted position: positions and normals are read in sorted order
    float u[3], nn[3], ex[3], ez[3];
    if (!particle_frame(cp, xyzr[js], nrm[js], u, nn, ex, ez)) {
        T[i] = -1.0f;  // marks a pair without features; compacted away on the host side
        return;
    }
    float* x = X + (size_t) i * MLP_IN;
    for (int c = 0; c < MLP_CONES; ++c) {
        float v[MLP_FSTEPS];
        cone_features(cp, c, u, nn, ex, ez, v);
#pragma unroll
        for (int j = 0; j < MLP_FSTEPS; ++j)
            x[c * MLP_FSTEPS + j] = v[j];
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        x[MLP_SAMPLES + a] = nn[a];
        x[MLP_SAMPLES + 3 + a] = u[a];
    }
    T[i] = ao[order[js]];
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
// inference weights: BF16 copies of W1 (feature i at K position i, zeros in the padding) and W2
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
// tile. Threads t and t + 128 extract the cone samples of particle t (cones 0-3 and 4-7) straight into the A
// tile (BF16, canonical no-swizzle K-major layout in shared memory, feature i at K position i); one thread
// issues the layer-1 MMAs (M = 128, N = 64, K = 64) into 64 TMEM columns and commits
// them to an mbarrier. The epilogue reads TMEM
// (warp w: lanes 32 (w % 4).., columns 32 (w / 4)..), adds the bias, applies SiLU and writes the hidden
// layer back into the A tile as layer 2's A operand; layer 2 (K = 64) reuses the TMEM columns, and its
// epilogue finishes layer 3 (64 -> 1) in FP32 with the sigmoid. The accumulators never occupy registers,
// so four CTAs (32 warps, 64 registers each: more warps hide the texture latency better than the few
// spilled registers cost) stay resident per SM. Every mbarrier wait
// is bounded: on timeout the CTA records ERR_MMA_TIMEOUT, drains its MMAs (bounded) and frees TMEM. The
// poll count can be lowered (p2v_params.mma_wait_polls), and a test hook (p2v_params.test_hold_mma) leaves layer
// 1 unissued so that its wait, on an arrival that never comes, runs out.
// ---------------------------------------------------------------------------------------------
#ifndef P2V_MLP_PACK_PER_CONE
#define P2V_MLP_PACK_PER_CONE 1  // with an even step count, pack each cone's features as soon as it is sampled
#endif
#ifndef P2V_MLP_CTAS
#define P2V_MLP_CTAS 4  // resident inference CTAs per SM (64 registers per thread at 4)
#endif
namespace tc {
constexpr int THREADS = 256;
constexpr int CTAS = P2V_MLP_CTAS;
constexpr int M = 128;                         // particles per tile (MMA M, TMEM lanes)
constexpr int KCH1 = MLP_KP / 8;               // 16-byte core-matrix columns of layer 1's K (8)
constexpr int KCH2 = MLP_H / 8;                // of layer 2's K (8)
constexpr int SBO1 = KCH1 * 128;               // bytes between 8-row core-matrix groups, layer 1
constexpr int SBO2 = KCH2 * 128;               // layer 2
constexpr int A_BYTES = (M / 8) * SBO1;        // 16384: features; later the hidden layer (16384 B)
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
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t phase, uint32_t limit) {
    for (uint32_t i = 0; i < limit; ++i) {
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

__device__ __forceinline__ void st_shared_v2(uint8_t* p, uint32_t a, uint32_t b) {
    *reinterpret_cast<uint2*>(p) = make_uint2(a, b);
}

// Store the BF16 pairs pk[0 .. NP) at K positions K0, K0 + 2, ... of row `row` (K0 even) with the widest
// aligned shared-memory stores (a pair never straddles a core-matrix row: K0 + 2 e is even).
template<int K0, int NP>
__device__ __forceinline__ void store_pairs(uint8_t* sA, int row, const uint32_t* pk) {
    int k = K0, i = 0;
#pragma unroll
    for (int step = 0; step < NP; ++step) {
        if (i >= NP)
            break;
        if (k % 8 == 0 && NP - i >= 4) {
            st_shared_v4(sA + canon_off(row, k, tc::SBO1), pk[i], pk[i + 1], pk[i + 2], pk[i + 3]);
            k += 8;
            i += 4;
        } else if (k % 4 == 0 && NP - i >= 2) {
            st_shared_v2(sA + canon_off(row, k, tc::SBO1), pk[i], pk[i + 1]);
            k += 4;
            i += 2;
        } else {
            *reinterpret_cast<uint32_t*>(sA + canon_off(row, k, tc::SBO1)) = pk[i];
            k += 2;
            i += 1;
        }
    }
}

template<bool FEATURES_IN>
__global__ void __launch_bounds__(tc::THREADS, tc::CTAS) mlp_infer_tc_kernel(const MlpInferArgs args, const ConeParams cp) {
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
    const uint32_t polls = args.wait_polls ? args.wait_polls : tc::WAIT_LIMIT;
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
            float u[3] = {0, 0, 0}, nn[3] = {0, 0, 0}, ex[3], ez[3];
            if (valid) {
                o = args.order ? args.order[pi] : pi;
                valid = particle_frame(cp, args.xyzr[o], args.nrm[o], u, nn, ex, ez);
            }
            // this half's cones 4 h .. 4 h + 3 = features HALF_F h .. HALF_F (h + 1) - 1 (K positions equal
            // feature indices)
            constexpr int HALF_F = MLP_SAMPLES / 2;  // 24
            uint32_t pk[HALF_F / 2];
            if constexpr (MLP_FSTEPS % 2 == 0 && P2V_MLP_PACK_PER_CONE) {
                // an even step count: a cone's features pair up among themselves, so each cone is packed as soon
                // as it is sampled (fewer live registers)
#pragma unroll
                for (int cc = 0; cc < MLP_CONES / 2; ++cc) {
                    float fv[MLP_FSTEPS];
                    if (valid)
                        cone_features(cp, (MLP_CONES / 2) * half + cc, u, nn, ex, ez, fv);
                    else
#pragma unroll
                        for (int j = 0; j < MLP_FSTEPS; ++j)
                            fv[j] = 0.0f;
#pragma unroll
                    for (int e = 0; e < MLP_FSTEPS / 2; ++e) {
                        const int pe = cc * (MLP_FSTEPS / 2) + e;
                        const __nv_bfloat162 v2 = __floats2bfloat162_rn(fv[2 * e], fv[2 * e + 1]);
                        if (check && valid)
                            oor |= !in_range((HALF_F / 2) * half + pe, v2);
                        pk[pe] = *reinterpret_cast<const uint32_t*>(&v2);
                    }
                }
            } else {
                float fv[HALF_F];
#pragma unroll
                for (int cc = 0; cc < MLP_CONES / 2; ++cc) {
                    if (valid)
                        cone_features(cp, (MLP_CONES / 2) * half + cc, u, nn, ex, ez, fv + cc * MLP_FSTEPS);
                    else
#pragma unroll
                        for (int j = 0; j < MLP_FSTEPS; ++j)
                            fv[cc * MLP_FSTEPS + j] = 0.0f;
                }
#pragma unroll
                for (int e = 0; e < HALF_F / 2; ++e) {
                    const __nv_bfloat162 v2 = __floats2bfloat162_rn(fv[2 * e], fv[2 * e + 1]);
                    if (check && valid)
                        oor |= !in_range((HALF_F / 2) * half + e, v2);
                    pk[e] = *reinterpret_cast<const uint32_t*>(&v2);
                }
            }
            if (half == 0) {
                store_pairs<0, HALF_F / 2>(sA, row, pk);
            } else {
                store_pairs<HALF_F, HALF_F / 2>(sA, row, pk);
                // then the normal, the surface point and two zeros (K MLP_SAMPLES .. MLP_SAMPLES + 7), and zeros up
                // to MLP_KP
                const __nv_bfloat162 n01 = __floats2bfloat162_rn(nn[0], nn[1]);
                const __nv_bfloat162 n2u0 = __floats2bfloat162_rn(nn[2], u[0]);
                const __nv_bfloat162 u12 = __floats2bfloat162_rn(u[1], u[2]);
                st_shared_v4(sA + canon_off(row, MLP_SAMPLES, tc::SBO1), *reinterpret_cast<const uint32_t*>(&n01),
                             *reinterpret_cast<const uint32_t*>(&n2u0), *reinterpret_cast<const uint32_t*>(&u12), 0u);
#pragma unroll
                for (int k = MLP_SAMPLES + 8; k < MLP_KP; k += 8)
                    st_shared_v4(sA + canon_off(row, k, tc::SBO1), 0u, 0u, 0u, 0u);
                if (valid && check)
                    oor |= !(in_range(MLP_SAMPLES / 2, n01) && in_range(MLP_SAMPLES / 2 + 1, n2u0) &&
                             in_range(MLP_SAMPLES / 2 + 2, u12));
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
        // ---- layer 1: D[128 x 64] = A[128 x MLP_KP] W1^T ----
        if (t == 0 && !args.hold_mma) {
            tc_fence_after();
#pragma unroll
            for (int kk = 0; kk < tc::KCH1 / 2; ++kk)
                umma_bf16(tmem, umma_desc(a_s + 256u * kk, 128u, tc::SBO1), umma_desc(w1_s + 256u * kk, 128u, tc::SBO1),
                          kk > 0 ? 1u : 0u);
            umma_commit(mbar);
        }
        failed = !mbar_wait(mbar, phase, polls);
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
        failed = !mbar_wait(mbar, phase, polls);
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
            const uint32_t wo = (!FEATURES_IN && args.out_order) ? args.out_order[oo] : oo;
            if (!FEATURES_IN && !valid) {
                args.y[wo] = 1.0f;  // no normal / invalid particle: unoccluded, as the cone march
            } else if (oor && args.fallback) {
                args.fallback[atomicAdd(args.nfallback, 1u)] = oo;
                if (FEATURES_IN)
                    args.y[wo] = y;
            } else {
                args.y[wo] = y;
            }
        }
    }
    if (failed) {
        if (t == 0 && args.err)
            atomicOr(args.err, ERR_MMA_TIMEOUT);
        // drain: the MMAs of the phase that timed out may still be running; wait for their completion once more
        // with the full budget before TMEM is freed (nothing was issued under the test hook)
        if (!args.hold_mma)
            mbar_wait(mbar, phase ^ 1u, tc::WAIT_LIMIT);
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

cudaError_t FeatureTex::ensure(const int dims[3]) {
    if (arr && d[0] == dims[0] && d[1] == dims[1] && d[2] == dims[2])
        return cudaSuccess;
    release();
    cudaChannelFormatDesc fmt = cudaCreateChannelDesc<uchar2>();
    cudaError_t e = cudaMalloc3DArray(&arr, &fmt, make_cudaExtent(dims[0], dims[1], dims[2]),
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
    td.readMode = cudaReadModeNormalizedFloat;  // 8-bit UNORM texels read as floats in [0, 1]
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

void FeatureTex::release() {
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

cudaError_t launch_fill_feature_tex(const ConeLevel& L, float sat, const FeatureTex& t, cudaStream_t st) {
    const int64_t n = (int64_t) L.d[0] * L.d[1] * L.d[2];
    const unsigned grd = (unsigned) std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 16));
    fill_feature_tex_kernel<<<grd, 256, 0, st>>>(L.v, L.d[0], L.d[1], L.d[2], sat, t.surf);
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
    // tc::CTAS resident CTAs per SM (41 KB of shared memory each, the registers the launch bounds leave, 64 TMEM
    // columns each of 512): one wave
    const unsigned grid = (unsigned) std::min<uint32_t>(ntiles, (uint32_t) sms * tc::CTAS);
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
