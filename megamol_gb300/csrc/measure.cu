// Hardware-rate probes for the benchmark's roofline figures (include/p2v_measure.h).
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "p2v.h"
#include "p2v_measure.h"

namespace p2v {
namespace {

constexpr int PROBE_D = 128;     // texels per axis of the probed level (layers = slices)
constexpr int PROBE_R = 64;      // region of the random pattern
constexpr int PROBE_ITERS = 512;  // samples per thread

__device__ __forceinline__ uint32_t mix32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

// Every warp moves a base point by a linear congruential step per sample; a lane's offset from it is fixed.
// Pattern 0: the quad's lanes at the 2 x 2 texels of one layer; pattern 1: every lane its own random offset in
// PROBE_R^3. Coordinates stay inside the texture (base + offset < PROBE_D on every axis).
__global__ void __launch_bounds__(256) texture_rate_kernel(cudaTextureObject_t tex, int pattern, float* sink) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int ox, oy, oz;
    if (pattern == 0) {
        const uint32_t hq = mix32(warp * 131u + (lane >> 2) * 977u + 7u);
        ox = (int) (hq % 4u) + (int) (lane & 1u);
        oy = (int) ((hq >> 8) % 4u) + (int) ((lane >> 1) & 1u);
        oz = (int) ((hq >> 16) % 4u);
    } else {
        const uint32_t hl = mix32(warp * 131u + lane * 977u + 3u);
        ox = (int) (hl % PROBE_R);
        oy = (int) ((hl >> 10) % PROBE_R);
        oz = (int) ((hl >> 20) % PROBE_R);
    }
    const uint32_t span = PROBE_D - PROBE_R;  // base in [0, span)
    uint32_t s = mix32(warp + 12345u);
    const float inv = 1.0f / (float) PROBE_D;
    float acc = 0.0f;
    for (int it = 0; it < PROBE_ITERS; it += 4) {
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            s = s * 1664525u + 1013904223u;
            const int bx = (int) (((s >> 24) * span) >> 8), by = (int) ((((s >> 16) & 255u) * span) >> 8),
                      bz = (int) ((((s >> 8) & 255u) * span) >> 8);
            const float2 v = tex2DLayered<float2>(tex, ((float) (bx + ox) + 0.37f) * inv,
                                                  ((float) (by + oy) + 0.61f) * inv, bz + oz);
            acc += v.x + v.y;
        }
    }
    if (acc == -1.0f)  // never: keeps the fetches
        *sink = acc;
}

}  // namespace
}  // namespace p2v

extern "C" p2v_status p2v_measure_texture_rate(int pattern, double* gsamples_per_s) {
    using namespace p2v;
    if (gsamples_per_s == nullptr || (pattern != 0 && pattern != 1))
        return P2V_EINVAL;
    *gsamples_per_s = 0.0;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return P2V_ECUDA;
    cudaArray_t arr = nullptr;
    cudaTextureObject_t tex = 0;
    float* sink = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    p2v_status st = P2V_ECUDA;
    do {
        const cudaChannelFormatDesc cd = cudaCreateChannelDesc(8, 8, 0, 0, cudaChannelFormatKindUnsigned);
        if (cudaMalloc3DArray(&arr, &cd, make_cudaExtent(PROBE_D, PROBE_D, PROBE_D), cudaArrayLayered) != cudaSuccess)
            break;
        std::vector<uint8_t> h((size_t) PROBE_D * PROBE_D * PROBE_D * 2);
        for (size_t i = 0; i < h.size(); ++i)
            h[i] = (uint8_t) ((i * 2654435761u) >> 24);
        cudaMemcpy3DParms mp = {};
        mp.srcPtr = make_cudaPitchedPtr(h.data(), PROBE_D * 2, PROBE_D, PROBE_D);
        mp.dstArray = arr;
        mp.extent = make_cudaExtent(PROBE_D, PROBE_D, PROBE_D);
        mp.kind = cudaMemcpyHostToDevice;
        if (cudaMemcpy3D(&mp) != cudaSuccess)
            break;
        cudaResourceDesc rd = {};
        rd.resType = cudaResourceTypeArray;
        rd.res.array.array = arr;
        cudaTextureDesc td = {};
        td.addressMode[0] = td.addressMode[1] = td.addressMode[2] = cudaAddressModeClamp;
        td.filterMode = cudaFilterModeLinear;
        td.readMode = cudaReadModeNormalizedFloat;
        td.normalizedCoords = 1;
        if (cudaCreateTextureObject(&tex, &rd, &td, nullptr) != cudaSuccess || cudaMalloc(&sink, sizeof(float)) != cudaSuccess ||
            cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
            break;
        const unsigned blocks = (unsigned) sms * 8u;
        for (int w = 0; w < 2; ++w)
            texture_rate_kernel<<<blocks, 256>>>(tex, pattern, sink);
        cudaEventRecord(e0);
        texture_rate_kernel<<<blocks, 256>>>(tex, pattern, sink);
        cudaEventRecord(e1);
        if (cudaEventSynchronize(e1) != cudaSuccess)
            break;
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess || ms <= 0.0f)
            break;
        *gsamples_per_s = (double) blocks * 256.0 * PROBE_ITERS / (ms * 1e-3) / 1e9;
        st = P2V_OK;
    } while (false);
    if (e0)
        cudaEventDestroy(e0);
    if (e1)
        cudaEventDestroy(e1);
    if (sink)
        cudaFree(sink);
    if (tex)
        cudaDestroyTextureObject(tex);
    if (arr)
        cudaFreeArray(arr);
    return st;
}
