// Shared device/host definitions of libp2v (GB300, sm_103a).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace p2v {

constexpr uint32_t ERR_LOOKBACK_TIMEOUT = 1u;  // radix-sort decoupled look-back waited too long
constexpr uint32_t ERR_GAP_OVERFLOW = 2u;      // cell-start long-gap list overflowed
constexpr uint32_t ERR_STAGE_OVERFLOW = 4u;    // density tile window exceeded the staging tables
constexpr uint32_t ERR_WINDOW_TOO_WIDE = 8u;   // footprint wider than the supported tile window
constexpr uint32_t ERR_MMA_TIMEOUT = 16u;      // a tensor-core MMA completion wait gave up

// Bounded spin budget for device-side waits: a wait that exceeds it records an error and gives up.
constexpr uint32_t SPIN_LIMIT = 1u << 22;

// Geometry of one density grid, with the reference's float quantities (used for every integer
// decision: cell, footprint, wrap) and an accurate spacing (used for distances).
struct GridGeo {
    int32_t s[3];        // resolution (sizex, sizey, sizez)
    int32_t cyc[3];      // cyclic per axis
    float minf[3];       // bbox min (reference origin)
    float hf[3];         // reference spacing: float(range) / float(res-1)
    float hhi[3], hlo[3];// exact spacing (right-left)/(res-1) as an unevaluated float sum
    float ihh[3];        // 1 / hhi
    float sigma;
    int32_t kernel;      // 0 bump, 1 gauss3
    uint32_t nb[3];      // bins per axis = res + 2 (underflow and overflow bins)
    uint32_t nbins;      // nb[0]*nb[1]*nb[2]
    int32_t zlo, zhi;    // the grid planes computed and written: [zlo, zhi) (a z-slab; 0, s[2] = all)
};

// Per-frame device scalars written by the binning stage and read by later stages.
struct FrameScalars {
    uint32_t rmax_bits;     // float bits of the largest valid radius (radii > 0)
    int32_t cmin[3];        // occupied cell range (floor), clamped to +-2^30
    int32_t cmax[3];
    uint32_t n_dropped;
    uint32_t n_valid;
    uint32_t error;         // ERR_* bits
    uint32_t ngaps;
    uint32_t ao_fallback;   // learned AO: particles handed to the cone march
    uint32_t wmax_bits;     // float bits of the largest |weight| (intensity / vector aggregators)
    uint32_t dmin_bits, dmax_bits;  // vector aggregator: density range (float bits, densities >= 0)
    uint32_t vcount;        // vector aggregator: nodes with a non-zero density
    uint32_t bin_maxcount;  // counting sort: particles in the fullest cell (0 when the radix path ran alone)
    uint32_t bin_nmulti;    // counting sort: cells holding two or more particles
    double mass;            // FP64 sum of the raw grid
    float vmin, vmax;       // raw grid min / max
    float out_min, out_max; // after normalisation
    float scale, offset;    // v_out = (v_raw - offset) * scale
    double mass_scale;
};

// Per-CTA partial statistics of the density tiles.
struct TileStats {
    double sum;
    float vmin, vmax;
};

__host__ __device__ inline uint32_t ceil_div(uint32_t a, uint32_t b) {
    return (a + b - 1) / b;
}

}  // namespace p2v

#define P2V_CUDA_TRY(expr)                                                                        \
    do {                                                                                          \
        cudaError_t e_ = (expr);                                                                  \
        if (e_ != cudaSuccess) {                                                                  \
            return fail(P2V_ECUDA, "%s failed: %s (%s:%d)", #expr, cudaGetErrorString(e_), __FILE__, \
                        __LINE__);                                                                \
        }                                                                                         \
    } while (0)
