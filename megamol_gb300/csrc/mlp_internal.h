// Internal interfaces of the learned-AO MLP (not part of the C ABI).
#pragma once

#include <cstdint>

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "ao_internal.h"

namespace p2v {

constexpr int MLP_STENCIL = 27;                // 3x3x3 samples per stencil level
constexpr int MLP_IN = 2 * MLP_STENCIL + 6;    // 60: two stencil levels, 3 normal and 3 position components
// The tensor-core tile keeps each group of features in whole 16-byte chunks: level s at K 0..26, level s + 1
// at K 32..58, normal and position at K 64..69, zeros elsewhere (MLP_KP = 80, five MMAs of K = 16).
constexpr int MLP_KP = 80;
// K position of logical feature i, and the logical feature at K position k (-1: padding)
__host__ __device__ constexpr int mlp_kpos(int i) {
    return i < 27 ? i : (i < 54 ? i + 5 : i + 10);
}
__host__ __device__ constexpr int mlp_feature_at(int k) {
    return k < 27 ? k : (k < 32 ? -1 : (k < 59 ? k - 5 : (k < 64 ? -1 : (k < 70 ? k - 10 : -1))));
}
constexpr int MLP_H = 64;
// parameter vector: W1[H][IN], b1[H], W2[H][H], b2[H], w3[H], b3
constexpr int OFF_W1 = 0;
constexpr int OFF_B1 = OFF_W1 + MLP_H * MLP_IN;
constexpr int OFF_W2 = OFF_B1 + MLP_H;
constexpr int OFF_B2 = OFF_W2 + MLP_H * MLP_H;
constexpr int OFF_W3 = OFF_B2 + MLP_H;
constexpr int OFF_B3 = OFF_W3 + MLP_H;
constexpr int MLP_NPARAM = OFF_B3 + 1;

struct MlpInferArgs {
    const float* P;                 // FP32 parameters (biases, last layer)
    const __nv_bfloat16* w1h;       // [H][KP] BF16
    const __nv_bfloat16* w2h;       // [H][H] BF16
    const float* lo;                // per-feature training range (nullable: no range check)
    const float* hi;
    uint32_t n;
    // extracted features (inference on particles)
    const uint32_t* order;          // sorted position -> particle index
    const float4* xyzr;
    const float4* nrm;
    // given features (tests)
    const float* X;
    float* y;                       // output, indexed by particle (or by row for given features)
    uint32_t* fallback;             // particle indices whose features left the training range (nullable)
    uint32_t* nfallback;
    uint32_t* err;                  // ERR_* bits (the tensor-core kernel's bounded waits)
};

// One mip level of the AO volume as an FP16 layered 2D texture, one layer per z slice (CLAMP_TO_BORDER,
// linear filtering in x and y, normalised coordinates), written through a surface. The learned AO's
// stencil samples it with the texture units.
struct StencilTex {
    cudaArray_t arr = nullptr;
    unsigned long long tex = 0;   // cudaTextureObject_t
    unsigned long long surf = 0;  // cudaSurfaceObject_t
    int d[3] = {0, 0, 0};
    cudaError_t ensure(const int dims[3]);
    void release();
};
// copy level L (level-0 saturation `sat` applied when > 0) into the texture
cudaError_t launch_fill_stencil_tex(const ConeLevel& L, float sat, const StencilTex& t, cudaStream_t st);

size_t mlp_train_smem_bytes();
cudaError_t launch_mlp_collect(const ConeParams& cp, const uint32_t* order, const uint32_t* sel, uint32_t nsel,
    const float4* xyzr, const float4* nrm, const float* ao, float* X, float* T, uint32_t* kept, cudaStream_t st);
cudaError_t launch_mlp_train_step(const float* P, const float* X, const float* T, const uint32_t* idx, int nbatch,
    float* partial, float* partial_loss, float* grad, float* loss, cudaStream_t st);
cudaError_t launch_mlp_adam(float* P, const float* g, float* m, float* v, float lr, float b1, float b2, float eps,
    int step, cudaStream_t st);
cudaError_t launch_mlp_forward_f32(const float* P, const float* X, const uint32_t* idx, uint32_t n, float* y,
    cudaStream_t st);
cudaError_t launch_mlp_range(const float* X, const uint32_t* idx, uint32_t n, float margin, float* lo, float* hi,
    cudaStream_t st);
cudaError_t launch_mlp_pack(const float* P, __nv_bfloat16* w1h, __nv_bfloat16* w2h, cudaStream_t st);
cudaError_t launch_mlp_infer(const MlpInferArgs& a, const ConeParams& cp, bool features_in, int sms, cudaStream_t st);

}  // namespace p2v
