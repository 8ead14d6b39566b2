// Internal interfaces of the learned-AO MLP (not part of the C ABI).
#pragma once

#include <cstdint>

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "../../include/p2v.h"
#include "ao_internal.h"

namespace p2v {

// Features: the cone march's own samples, for each of MLP_CONES cones at MLP_FSTEPS of its steps (cone-major:
// feature c * MLP_FSTEPS + j), then the unit normal and the surface point in normalised volume coordinates.
#ifndef P2V_MLP_FSTEPS_BUILD
#define P2V_MLP_FSTEPS_BUILD P2V_MLP_FSTEPS
#endif
constexpr int MLP_CONES = 8;
constexpr int MLP_FSTEPS = P2V_MLP_FSTEPS_BUILD;
constexpr int MLP_SAMPLES = MLP_CONES * MLP_FSTEPS;   // 48
constexpr int MLP_IN = MLP_SAMPLES + 6;               // 54
static_assert(MLP_FSTEPS <= MAX_FSTEPS, "feature step table too small");
static_assert(MLP_SAMPLES % 8 == 0, "the normal and the surface point start a core-matrix column");
// The tensor-core tile holds feature i at K position i; K MLP_IN .. MLP_KP - 1 are zero (MLP_KP = 64: four MMAs
// of K = 16).
constexpr int MLP_KP = (MLP_IN + 15) / 16 * 16;
__host__ __device__ constexpr int mlp_feature_at(int k) {
    return k < MLP_IN ? k : -1;
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
    const uint32_t* out_order;      // nullable: particle j's output goes to y[out_order[j]] (sorted in, input order out)
    uint32_t* fallback;             // particle indices whose features left the training range (nullable)
    uint32_t* nfallback;
    uint32_t* err;                  // ERR_* bits (the tensor-core kernel's bounded waits)
    uint32_t wait_polls;            // polls of each MMA-completion wait before it gives up (0: the default)
    int hold_mma;                   // test hook: layer 1 is not issued, so its completion wait runs out
};

// One mip level of the AO volume as a paired-slice layered texture: layer z holds slices z and z + 1 as two
// 8-bit UNORM channels (GL LINEAR in x and y, CLAMP_TO_BORDER, normalised coordinates), written through a
// surface; the learned AO's features sample it with the texture units (one bilinear fetch per sample, the z
// weight applied in FP32).
struct FeatureTex {
    cudaArray_t arr = nullptr;
    unsigned long long tex = 0;   // cudaTextureObject_t
    unsigned long long surf = 0;  // cudaSurfaceObject_t
    int d[3] = {0, 0, 0};
    cudaError_t ensure(const int dims[3]);
    void release();
};
// copy level L (level-0 saturation `sat` applied when > 0) into the texture
cudaError_t launch_fill_feature_tex(const ConeLevel& L, float sat, const FeatureTex& t, cudaStream_t st);

size_t mlp_train_smem_bytes();
// xyzr, nrm in sorted order (sel holds sorted positions), ao in input order (order: sorted position -> index)
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
