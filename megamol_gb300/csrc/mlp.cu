// Learned AO: a small MLP that stands in for the cone march.
//
// Input (131): two consecutive mip levels of the AO volume (the levels the cone's first samples read), each
// resampled as a 4x4x4 stencil of trilinear samples
// centred on the particle's surface point (sample spacing = one texel of that level, so the stencil moves
// continuously with the point), then the unit normal. Network 131 -> 64 -> 64 -> 1, SiLU, SiLU, sigmoid.
// Training: FP32 forward/backward kernels per CTA with a fixed-order reduction of the per-CTA gradients,
// then Adam; pairs come from the plain cone march. Inference: BF16 weights and features, FP32 accumulation
// on the tensor cores (mma.sync m16n8k16), bias/activations in FP32 registers. A particle whose features
// leave the training range (per feature, with a margin) falls back to the cone march.
// No reference counterpart: the reference evaluates AO only by the GLSL cone march / AOSphere taps.
#include <cuda_bf16.h>
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

__device__ __forceinline__ float sigmoidf_(float a) {
    return 1.0f / (1.0f + __expf(-a));
}

__device__ __forceinline__ float lv_fetch(const ConeLevel& L, int x, int y, int z) {
    if ((unsigned) x >= (unsigned) L.d[0] || (unsigned) y >= (unsigned) L.d[1] || (unsigned) z >= (unsigned) L.d[2])
        return 0.0f;  // CLAMP_TO_BORDER, as the cone march samples
    return __ldg(L.v + ((int64_t) z * L.d[1] + y) * L.d[0] + x);
}

// 4x4x4 trilinear samples of level L at texel-spaced offsets (k - 1.5) around normalised point u;
// out[(kz*4 + ky)*4 + kx]. The samples share one 5x5x5 block of texels and one set of weights.
__device__ __forceinline__ void stencil64(const ConeLevel& L, float ux, float uy, float uz, float* out) {
    const float cx = ux * L.fd[0] - 2.0f, cy = uy * L.fd[1] - 2.0f, cz = uz * L.fd[2] - 2.0f;
    const float fx0 = floorf(cx), fy0 = floorf(cy), fz0 = floorf(cz);
    const int x0 = (int) fx0, y0 = (int) fy0, z0 = (int) fz0;
    const float fx = cx - fx0, fy = cy - fy0, fz = cz - fz0;
    float prev[16];
#pragma unroll
    for (int zz = 0; zz < 5; ++zz) {
        float cur[16];
        float rowp[4];
#pragma unroll
        for (int yy = 0; yy < 5; ++yy) {
            float t[5];
#pragma unroll
            for (int xx = 0; xx < 5; ++xx)
                t[xx] = lv_fetch(L, x0 + xx, y0 + yy, z0 + zz);
            float rowc[4];
#pragma unroll
            for (int k = 0; k < 4; ++k)
                rowc[k] = t[k] + fx * (t[k + 1] - t[k]);
            if (yy > 0) {
#pragma unroll
                for (int k = 0; k < 4; ++k)
                    cur[(yy - 1) * 4 + k] = rowp[k] + fy * (rowc[k] - rowp[k]);
            }
#pragma unroll
            for (int k = 0; k < 4; ++k)
                rowp[k] = rowc[k];
        }
        if (zz > 0) {
#pragma unroll
            for (int k = 0; k < 16; ++k)
                out[(zz - 1) * 16 + k] = prev[k] + fz * (cur[k] - prev[k]);
        }
#pragma unroll
        for (int k = 0; k < 16; ++k)
            prev[k] = cur[k];
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
    float f[64];
    float* x = X + (size_t) i * MLP_IN;
    stencil64(cp.lv[cp.stencil_level], u[0], u[1], u[2], f);
#pragma unroll
    for (int k = 0; k < 64; ++k)
        x[k] = f[k];
    stencil64(cp.lv[cp.stencil_level + 1], u[0], u[1], u[2], f);
#pragma unroll
    for (int k = 0; k < 64; ++k)
        x[64 + k] = f[k];
    x[128] = n[0];
    x[129] = n[1];
    x[130] = n[2];
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
// inference: BF16 tensor cores (mma.sync m16n8k16, FP32 accumulate)
// ---------------------------------------------------------------------------------------------
constexpr int W1P = 152;  // smem row pitch (bf16) of W1 and of the feature tile: conflict-free fragment loads
constexpr int W2P = 72;
constexpr int IWARPS = 4;

__global__ void mlp_pack_kernel(const float* __restrict__ P, __nv_bfloat16* __restrict__ w1h,
    __nv_bfloat16* __restrict__ w2h) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < MLP_H * MLP_KP; k += gridDim.x * blockDim.x) {
        const int j = k / MLP_KP, i = k % MLP_KP;
        w1h[k] = __float2bfloat16_rn(i < MLP_IN ? P[OFF_W1 + j * MLP_IN + i] : 0.0f);
    }
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < MLP_H * MLP_H; k += gridDim.x * blockDim.x)
        w2h[k] = __float2bfloat16_rn(P[OFF_W2 + k]);
}

__device__ __forceinline__ void mma_bf16(float* c, uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3, uint32_t b0,
    uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}

// FEATURES_IN: features given in global memory (tests); else extracted from the mip levels.
template<bool FEATURES_IN>
__global__ void __launch_bounds__(IWARPS * 32) mlp_infer_kernel(const MlpInferArgs args, const ConeParams cp) {
    __shared__ __align__(16) __nv_bfloat16 sW1[MLP_H * W1P];
    __shared__ __align__(16) __nv_bfloat16 sW2[MLP_H * W2P];
    __shared__ __align__(16) __nv_bfloat16 sA[IWARPS][16 * W1P];
    __shared__ float sB1[MLP_H], sB2[MLP_H], sW3[MLP_H], sLo[MLP_IN], sHi[MLP_IN];
    const int t = threadIdx.x;
    for (int k = t; k < MLP_H * MLP_KP; k += blockDim.x)
        sW1[(k / MLP_KP) * W1P + k % MLP_KP] = args.w1h[k];
    for (int k = t; k < MLP_H * MLP_H; k += blockDim.x)
        sW2[(k / MLP_H) * W2P + k % MLP_H] = args.w2h[k];
    for (int k = t; k < MLP_H; k += blockDim.x) {
        sB1[k] = args.P[OFF_B1 + k];
        sB2[k] = args.P[OFF_B2 + k];
        sW3[k] = args.P[OFF_W3 + k];
    }
    for (int k = t; k < MLP_IN; k += blockDim.x) {
        sLo[k] = args.lo ? args.lo[k] : -INFINITY;
        sHi[k] = args.hi ? args.hi[k] : INFINITY;
    }
    __syncthreads();
    const float b3 = args.P[OFF_B3];
    const int warp = t >> 5, lane = t & 31;
    const int g = lane >> 2, tg = lane & 3;
    __nv_bfloat16* A = sA[warp];
    const uint32_t ntiles = (args.n + 15) / 16;
    for (uint32_t tile = blockIdx.x * IWARPS + warp; tile < ntiles; tile += gridDim.x * IWARPS) {
        const uint32_t base = tile * 16;
        // ---- features: lane pair (2p, 2p+1) builds particle p's row; lane 2p+l does level l+1 ----
        const int pl = lane >> 1, lev = lane & 1;
        const uint32_t pi = base + pl;
        bool out_of_range = false;
        bool valid = pi < args.n;
        uint32_t o = 0;
        if (FEATURES_IN) {
            for (int k = lev; k < MLP_KP; k += 2) {
                float v = 0.0f;
                if (valid && k < MLP_IN) {
                    v = args.X[(size_t) pi * MLP_IN + k];
                    out_of_range |= !(v >= sLo[k] && v <= sHi[k]);
                }
                A[pl * W1P + k] = __float2bfloat16_rn(v);
            }
        } else {
            float f[64];
            float u[3] = {0, 0, 0}, nn[3] = {0, 0, 0};
            if (valid) {
                o = args.order[pi];
                const float4 p = args.xyzr[o];
                valid = isfinite(p.x) && isfinite(p.y) && isfinite(p.z) && p.w > 0.0f &&
                        mlp_point(cp, p, args.nrm[o], u, nn);
            }
            if (valid) {
                stencil64(cp.lv[cp.stencil_level + lev], u[0], u[1], u[2], f);
            } else {
#pragma unroll
                for (int k = 0; k < 64; ++k)
                    f[k] = 0.0f;
            }
#pragma unroll
            for (int k = 0; k < 64; ++k) {
                const int fi = lev * 64 + k;
                out_of_range |= valid && !(f[k] >= sLo[fi] && f[k] <= sHi[fi]);
                A[pl * W1P + fi] = __float2bfloat16_rn(f[k]);
            }
            if (lev == 0) {
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    out_of_range |= valid && !(nn[c] >= sLo[128 + c] && nn[c] <= sHi[128 + c]);
                    A[pl * W1P + 128 + c] = __float2bfloat16_rn(nn[c]);
                }
            } else {
                for (int k = 131; k < MLP_KP; ++k)
                    A[pl * W1P + k] = __float2bfloat16_rn(0.0f);
            }
        }
        // every lane must execute each shuffle (full mask): no short-circuit around them
        const bool partner_oor = __shfl_xor_sync(0xffffffffu, out_of_range, 1);
        const bool partner_valid = __shfl_xor_sync(0xffffffffu, valid, 1);
        out_of_range = out_of_range || partner_oor;
        const bool pvalid = valid || partner_valid;
        __syncwarp();
        // ---- layer 1: [16 x 144] x [144 x 64] ----
        float acc[8][4];
#pragma unroll
        for (int nt = 0; nt < 8; ++nt)
#pragma unroll
            for (int e = 0; e < 4; ++e)
                acc[nt][e] = 0.0f;
#pragma unroll
        for (int kk = 0; kk < MLP_KP / 16; ++kk) {
            const int c0 = 16 * kk + 2 * tg;
            const uint32_t a0 = *reinterpret_cast<const uint32_t*>(&A[g * W1P + c0]);
            const uint32_t a1 = *reinterpret_cast<const uint32_t*>(&A[(g + 8) * W1P + c0]);
            const uint32_t a2 = *reinterpret_cast<const uint32_t*>(&A[g * W1P + c0 + 8]);
            const uint32_t a3 = *reinterpret_cast<const uint32_t*>(&A[(g + 8) * W1P + c0 + 8]);
#pragma unroll
            for (int nt = 0; nt < 8; ++nt) {
                const __nv_bfloat16* wr = sW1 + (8 * nt + g) * W1P + c0;
                mma_bf16(acc[nt], a0, a1, a2, a3, *reinterpret_cast<const uint32_t*>(wr),
                         *reinterpret_cast<const uint32_t*>(wr + 8));
            }
        }
        // ---- bias + SiLU; the accumulator layout of two n-tiles is the A layout of one k-step ----
        uint32_t h[4][4];
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            const int col = 8 * nt + 2 * tg;
            const float v0 = silu(acc[nt][0] + sB1[col]), v1 = silu(acc[nt][1] + sB1[col + 1]);
            const float v2 = silu(acc[nt][2] + sB1[col]), v3 = silu(acc[nt][3] + sB1[col + 1]);
            h[nt >> 1][(nt & 1) * 2 + 0] = pack_bf16(v0, v1);
            h[nt >> 1][(nt & 1) * 2 + 1] = pack_bf16(v2, v3);
        }
        // ---- layer 2: [16 x 64] x [64 x 64] ----
#pragma unroll
        for (int nt = 0; nt < 8; ++nt)
#pragma unroll
            for (int e = 0; e < 4; ++e)
                acc[nt][e] = 0.0f;
#pragma unroll
        for (int kk = 0; kk < 4; ++kk) {
            const int c0 = 16 * kk + 2 * tg;
#pragma unroll
            for (int nt = 0; nt < 8; ++nt) {
                const __nv_bfloat16* wr = sW2 + (8 * nt + g) * W2P + c0;
                // A regs: a0 = (row g, k c0..), a1 = (row g+8), a2 = (row g, k c0+8..), a3 = (row g+8, ..)
                mma_bf16(acc[nt], h[kk][0], h[kk][1], h[kk][2], h[kk][3], *reinterpret_cast<const uint32_t*>(wr),
                         *reinterpret_cast<const uint32_t*>(wr + 8));
            }
        }
        // ---- layer 3 (64 -> 1) in FP32 on the CUDA cores, sigmoid ----
        float zlo = 0.0f, zhi = 0.0f;
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            const int col = 8 * nt + 2 * tg;
            zlo = fmaf(silu(acc[nt][0] + sB2[col]), sW3[col], zlo);
            zlo = fmaf(silu(acc[nt][1] + sB2[col + 1]), sW3[col + 1], zlo);
            zhi = fmaf(silu(acc[nt][2] + sB2[col]), sW3[col], zhi);
            zhi = fmaf(silu(acc[nt][3] + sB2[col + 1]), sW3[col + 1], zhi);
        }
        zlo += __shfl_xor_sync(0xffffffffu, zlo, 1);
        zlo += __shfl_xor_sync(0xffffffffu, zlo, 2);
        zhi += __shfl_xor_sync(0xffffffffu, zhi, 1);
        zhi += __shfl_xor_sync(0xffffffffu, zhi, 2);
        // flags and output index of rows g and g+8 live on lanes 2g and 2(g+8)
        const bool oor_lo = __shfl_sync(0xffffffffu, out_of_range, 2 * g);
        const bool oor_hi = __shfl_sync(0xffffffffu, out_of_range, (2 * (g + 8)) & 31);
        const bool val_lo = __shfl_sync(0xffffffffu, pvalid, 2 * g);
        const bool val_hi = __shfl_sync(0xffffffffu, pvalid, (2 * (g + 8)) & 31);
        const uint32_t o_lo = __shfl_sync(0xffffffffu, o, 2 * g);
        const uint32_t o_hi = __shfl_sync(0xffffffffu, o, (2 * (g + 8)) & 31);
        if (tg == 0) {
#pragma unroll
            for (int half = 0; half < 2; ++half) {
                const uint32_t row = base + g + 8 * half;
                if (row >= args.n)
                    continue;
                const float y = sigmoidf_((half ? zhi : zlo) + b3);
                const bool oor = half ? oor_hi : oor_lo;
                const bool vv = half ? val_hi : val_lo;
                const uint32_t oo = FEATURES_IN ? row : (half ? o_hi : o_lo);
                if (!FEATURES_IN && !vv) {
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
        __syncwarp();
    }
}

}  // namespace

size_t mlp_train_smem_bytes() {
    return sizeof(float) * (MLP_H * MLP_IN + MLP_H * MLP_H + TS * MLP_IN + 6 * TS * MLP_H + TS);
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
    const uint32_t ntiles = (a.n + 15) / 16;
    const unsigned grid = (unsigned) std::min<uint32_t>(ceil_div(ntiles, IWARPS), (uint32_t) sms * 8);
    if (features_in)
        mlp_infer_kernel<true><<<grid, IWARPS * 32, 0, st>>>(a, cp);
    else
        mlp_infer_kernel<false><<<grid, IWARPS * 32, 0, st>>>(a, cp);
    return cudaGetLastError();
}

}  // namespace p2v
