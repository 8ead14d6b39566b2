// Internal interfaces of the AO stage of libp2v (not part of the C ABI).
#pragma once

#include <cstdint>

#include <cuda_runtime.h>

#include "p2v_common.cuh"

namespace p2v {

constexpr int MAX_CONES = 16;
constexpr int MAX_STEPS = 256;
constexpr int MAX_LEVELS = 12;
constexpr int MAX_FSTEPS = 16;

struct ConeLevel {
    const float* v;
    int d[3];
    float fd[3];
};

// Everything the cone march needs, passed by value (kernel parameter space).
struct ConeParams {
    float bmin[3], ibsize[3];      // volume bounds (normalised coordinates u = (x - bmin) * ibsize)
    float strength;
    float sat;                     // level-0 texel = clamp(v * sat, 0, 1); 0 = raw
    int border;                    // 0 = CLAMP_TO_BORDER, 1 = CLAMP_TO_EDGE
    int early_exit;
    int ncones, nsteps, nlevels;
    float4 dirs[MAX_CONES];        // xyz around +Y, w = cone width
    float t[MAX_STEPS], lod[MAX_STEPS];
    ConeLevel lv[MAX_LEVELS];
    // learned AO: the march steps its features sample (per cone), and 8-bit paired-slice textures of the mip levels
    // those samples read (0 = level not needed)
    int nfsteps;
    int fstep[MAX_FSTEPS];
    unsigned long long ftex[MAX_LEVELS];
};

struct AOSphereParams {
    int s[3], si[3];               // texture size with border, inner size
    float minOS[3], rangeOS[3];    // clip box
    float voxel_vol, gen_fac, eval_fac;
    float origin[3], ext[3], sampd[3];  // posOrigin, posExtents, aoSampDist
    int glsl_rule;                 // deposit: 0 = createVolumeCPU's voxel rule, 1 = createVolumeGLSL's
    int clip;                      // CPU rule: drop particles on the far side of the clip plane
    float clip_plane[4];           // unit normal, d
};

// MDAO occupancy volume geometry (uniforms of mdao_volume.geom/frag.glsl, MDAOVolumeGenerator.cpp:139-164)
struct MdaoParams {
    float bmin[3], inv[3], fd[3], cell[3];  // inBoundsMin, inBoundsSizeInverse, inVolumeSize, cellSize
    float cell_vol, ps_scale, sphere_k;     // cell volume, point-size scale (mdao_volume.geom.glsl:28), 4/3 * 3.14152
    float half_vp[2];                       // half the slice viewport
    int d[3];
    int unorm8;                             // 1 = R8 texel values k/255, 0 = unquantised fractions
};

// ---- the persistent batch AO (p2v_run_batch, cone march on the density) ----
// One frame's deferred AO stage: its cone march (lv[0] = the frame's density grid, lv[1..] mip levels the
// batch kernel builds), its grid geometry for gradient normals, and its particles in sorted order.
struct alignas(16) BatchAoFrame {
    ConeParams cp;
    GridGeo g;
    const float* grid;       // the density grid (level 0 before saturation)
    const float4* xyzr;      // positions and radii, sorted order
    const float4* nrm;       // normals, sorted order; null: -grad(density) at each particle
    const uint32_t* order;   // sorted position -> input index
    float* ao;               // AO in input order
    uint32_t n;
};
static_assert(sizeof(BatchAoFrame) % 16 == 0, "frame descriptors are copied as 16-byte words");

enum : uint32_t { BSEG_MIP = 0, BSEG_AO = 1 };
constexpr uint32_t BATCH_MIP_ITEM = 512;  // voxels of one mip item
constexpr uint32_t BATCH_AO_ITEM = 128;   // particles of one AO item (one per thread)

// A run of work items of one kind and frame. Items are numbered by tickets in queue order; a segment's
// items start once its dependency (an earlier segment) has completed every item.
struct BatchSeg {
    uint32_t first;  // first ticket
    uint32_t count;  // items
    uint32_t frame;
    uint32_t kind;   // BSEG_MIP: build mip level `level` from level - 1; BSEG_AO: cone march
    int32_t level;
    int32_t dep;     // segment index, -1 none
};

struct BatchQueueArgs {
    const BatchAoFrame* frames;
    const BatchSeg* segs;
    uint32_t nseg, total;  // segments, tickets
    uint32_t* words;       // [0] next ticket, [1] error (BATCH_ERR_*), [2 + s] completed items of segment s
    uint32_t wait_polls;   // polls of a dependency before the wait gives up
    int32_t hold_seg;      // test hook: this segment never reports its completion (-1 none)
};
constexpr uint32_t BATCH_ERR_TIMEOUT = 1;
inline size_t batch_queue_words(uint32_t nseg) { return 2 + (size_t) nseg; }
// zeroes the queue words and runs the queue with one resident block per free slot of every SM
cudaError_t launch_batch_ao(const BatchQueueArgs& q, int sms, cudaStream_t st);

// quantize = 1: the levels are R8 textures (texels k/255; out = ((sum k + 4) / 8) / 255)
cudaError_t launch_mip_levels(const float* l0, const int d0[3], float sat_scale, int quantize, int nlevels,
    float* const* out, int (*dims)[3], int sms, cudaStream_t st);
// acc: scratch of 4 (unorm8) or 8 bytes per voxel; vol: level 0 of the MDAO volume (x fastest)
cudaError_t launch_mdao_volume(const MdaoParams& mp, const uint32_t* order, const float4* xyzr, uint32_t n,
    void* acc, float* vol, int sms, cudaStream_t st);
// n_dev (nullable): device-side particle count, at most n (the cone march of the learned-AO fallback list)
// xyzr_s[j] = xyzr[order[j]] (skipped when xyzr is null), nrm_s[j] = nrm[order[j]] (sorted order).
cudaError_t launch_sort_particles(const uint32_t* order, uint32_t n, const float4* xyzr, const float4* nrm,
    float4* xyzr_s, float4* nrm_s, int sms, cudaStream_t st);
// particle i (or list entry i) reads xyzr / nrm at order[i] (or i); its AO goes to ao[out_order[that index]]
// when out_order is given (sorted copies in, input order out), else to ao[that index]
cudaError_t launch_cone_ao(const ConeParams& cp, const uint32_t* order, const float4* xyzr, const float4* nrm,
    uint32_t n, const uint32_t* n_dev, const uint32_t* out_order, float* ao, cudaStream_t st);
// the whole frame with one warp per cone of a particle (the bits of launch_cone_ao)
cudaError_t launch_cone_ao_warp(const ConeParams& cp, const float4* xyzr, const float4* nrm, uint32_t n,
    const uint32_t* out_order, float* ao, int sms, cudaStream_t st);
cudaError_t launch_aosphere(const AOSphereParams& ap, const float4* xyzr, uint32_t n, unsigned long long* acc,
    float* tex, const uint32_t* order, const float4* nrm, int mode, float* ao, int sms, cudaStream_t st);
// unit normals down the density gradient of `grid` (geometry geo) at xyzr[j], into nrm[j] (P2V_NORMALS_GRADIENT)
cudaError_t launch_gradient_normals(const GridGeo& geo, const float* grid, const float4* xyzr, uint32_t n, float4* nrm,
    cudaStream_t st);
// Brick-major order of the cell-sorted particles (bricks of 16 x 4 x 4 cells): cnt needs nseg words, tsum
// ntiles; xyzr_b[j] = xyzr[src], nrm_b[j] = nrm[src] (nrm nullable), order_b[j] = order[src] for the particle
// src of brick order position j. start: the cell start table (nbins + 1 entries); rec_b: the sorted particles'
// gather records (their floor cells).
struct BrickPlan {
    uint32_t nb[3];
    uint64_t nseg, ntiles;
};
BrickPlan brick_plan(const GridGeo& g);
cudaError_t launch_brick_order(const BrickPlan& p, const GridGeo& g, const uint32_t* start, const int4* rec_b,
                               uint32_t n, uint32_t* cnt, uint32_t* tsum, const float4* xyzr, const float4* nrm,
                               const uint32_t* order, float4* xyzr_b, float4* nrm_b, uint32_t* order_b, int sms,
                               cudaStream_t st);
cudaError_t launch_pack_normals(const void* src, uint32_t stride, uint64_t count, uint64_t offset, float4* nrm,
    cudaStream_t st);

}  // namespace p2v
