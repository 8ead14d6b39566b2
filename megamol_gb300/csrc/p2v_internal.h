// Internal launcher interfaces of libp2v (not part of the C ABI).
#pragma once

#include <algorithm>
#include <cstddef>
#include <cstdint>

#include <cuda_runtime.h>

#include "p2v_common.cuh"

namespace p2v {

// One particle list on the device, as the pack kernel reads it.
struct ListDesc {
    const uint8_t* data;
    uint32_t stride;       // bytes, never 0 (packed stride filled in by the host)
    int32_t type;          // p2v_vertex_type
    float global_radius;
    uint64_t count;
    uint64_t offset;       // index of the list's first record in the frame arrays
};

// The counting sort by cell is taken while its count table stays at most this large (near L2-resident).
constexpr uint64_t COUNTING_TABLE_MAX_BYTES = 128ull << 20;

struct SortBuffers {
    uint32_t* keys[2];
    uint32_t* vals[2];
    uint32_t* hist;        // digit histograms + tile counters, sort_hist_words()
    uint32_t* status;      // look-back words, sort_status_words(n)
    uint32_t* err;
    const float4* xyzr_in; // when non-null the last pass writes every particle's gather record
    float4* rec_a;         // (particle_record.cuh) in sorted order, interleaved: rec_b = rec_a + 1, both
    int4* rec_b;           // indexed with REC_STRIDE * position
    float4* xyzr_out;      // nullable: with xyzr_in, the particles' xyzr in sorted order as well (the AO stages)
    GridGeo geo;
    int result;            // index of the buffers holding the sorted output
    bool implicit_vals0;   // vals[0] holds no input values: the first pass takes the identity (indices)
    bool first_pass;       // set by launch_sort for its own bookkeeping
    uint32_t empty_flag = 0;  // key bit of the particles whose support holds no node (radix path), 0 = none
    uint32_t wait_polls = 0;  // polls of a look-back wait before the sort gives up (0: SPIN_LIMIT)
    int32_t hold_tile = -1;   // test hook: this tile of the first pass never publishes its counts (-1 none)
};

// idx (optional) receives the identity order of the packed particles. empty_flag: 0, or the bit that
// sort_empty_flag returns, added to the keys of particles whose support holds no grid node.
cudaError_t launch_pack_keys(const ListDesc& L, const GridGeo& g, float4* xyzr, uint32_t* keys, uint32_t* idx,
    FrameScalars* fs, uint32_t empty_flag, cudaStream_t st);
// The power of two above every cell key (max_key) that marks particles whose support holds no node, or 0 when
// the extra key bit would cost the radix sort a pass.
uint32_t sort_empty_flag(uint32_t max_key);
size_t sort_status_words(uint32_t n);
size_t sort_hist_words();
int sort_passes(uint32_t max_key);
// Stable LSD radix sort of keys[0] / vals[0]; b.result names the buffers holding the output. With a gate
// every kernel returns at once unless the gate's counting sort overflowed; odd: an odd pass count.
cudaError_t launch_sort(SortBuffers& b, uint32_t n, uint32_t max_key, int sms, cudaStream_t st,
    const FrameScalars* gate = nullptr, bool odd = false);
// keys[j] for sorted positions j from the cell start table (the counting sort writes no sorted keys).
cudaError_t launch_keys_from_starts(const uint32_t* start, uint32_t nbins, uint32_t n, uint32_t* keys, int sms,
    cudaStream_t st);
// Words of the status buffer the counting sort's scan needs for nbins + 1 cells.
size_t bin_scan_words(uint32_t nbins);
// The particle binning: the stable sort of the bin keys (keys[0], vals[0] from launch_pack_keys) with the
// gather records, and the cell start table (nbins + 1 entries). counts (nbins + 1 words) selects the
// counting sort by cell, whose per-cell ordering handles cells of up to 32 particles; a fuller cell sends
// the frame through the radix sort on the device. counts == nullptr: the radix sort alone.
// bstart: cell_block_count(nbins) words of scratch (the radix path's start of every 64th cell)
cudaError_t launch_bin_sort(SortBuffers& b, uint32_t n, const GridGeo& g, uint32_t* counts, uint32_t* start,
    uint32_t* bstart, uint4* gaps, uint32_t gap_cap, FrameScalars* fs, int sms, cudaStream_t st);
uint32_t cell_block_count(uint32_t nbins);

// Density gather configuration chosen on the host.
enum GatherMode { GATHER_EXACT = 0, GATHER_KAHAN = 1 };
struct GatherConfig {
    int mode;              // GatherMode
    int tx, ty, tz;        // nodes per tile
    int smax;              // staged particles per chunk
    int rmax;              // row-table entries per plane chunk
};

// Accumulation and per-particle weights of one gather pass: DENSITY (exact fixed point), FIXED (the
// intensity aggregator: weights w[j * wstride] in sorted order, signed fixed point), DOUBLE (the vector
// aggregator: FP64 sums of weights w, or of the plain kernel values when w == nullptr). The output grid is
// written with stride ostride (3 for one component of a vector volume).
struct GatherWeights {
    enum Mode { DENSITY = 0, FIXED = 1, DOUBLE = 2 };
    int mode = DENSITY;
    const float* w = nullptr;
    int wstride = 1;
    int ostride = 1;
};

// Per-particle weight source of one list for the intensity (nc = 1: first colour channel) or vector
// (nc = 3: DIRDATA_FLOAT_XYZ) aggregator; data == nullptr with nc = 1: every particle has global_i.
struct WeightSource {
    const uint8_t* data = nullptr;
    uint32_t stride = 0;
    int ctype = 0;          // p2v_colour_type
    float global_i = 0.0f;
    uint64_t count = 0, offset = 0;
};
cudaError_t launch_pack_weights(const WeightSource& src, int nc, float* w, FrameScalars* fs, int sms, cudaStream_t st);
cudaError_t launch_permute_weights(const uint32_t* order, const float* win, float* wout, uint32_t n, int nc, int sms,
                                   cudaStream_t st);
// vol3 /= weight sums, density range into fs, normalisation constants (ParticlesToDensity.cpp:628-682)
// The vector aggregator's outParticles / outInfo grid: per node the density, the unit direction and the sort
// key ~bits(density) (descending densities in a stable ascending sort) with the node index as value.
struct VectorGridBufs {
    float* dens;       // V
    float* dirs;       // 3 V
    uint32_t* keys;    // V
    uint32_t* vals;    // V
};
// Node positions of the grid: min + h * index in float (ParticlesToDensity.cpp:436-456).
struct VectorGridGeo {
    float minf[3], hf[3];
    int32_t res[3];
    int normalize;
};
// vg == nullptr: the volume only; otherwise also the grid buffers and fs->vcount (non-zero densities).
cudaError_t launch_vector_finish(float* vol3, const float* wsum, int64_t V, FrameScalars* fs, int minmax_normalize,
                                 int sms, cudaStream_t st, const VectorGridBufs* vg = nullptr);
// The first `count` entries of the sorted grid into positions (3), directions (3), colours (1) and info rows
// (7); any output may be null.
cudaError_t launch_vector_grid(const uint32_t* order, const float* dens, const float* dirs, const FrameScalars* fs,
                               const VectorGridGeo& geo, uint32_t count, float* pos, float* dir, float* col, float* info,
                               int sms, cudaStream_t st);

size_t gather_smem_bytes(const GatherConfig& c);
cudaError_t launch_gather(const GatherConfig& c, const GridGeo& g, const float4* rec_a, const int4* rec_b,
    const uint32_t* start, float* grid, TileStats* tiles, FrameScalars* fs, cudaStream_t st,
    const GatherWeights& w = GatherWeights{});
uint32_t gather_tile_count(const GatherConfig& c, const GridGeo& g);
// Reduce the tile statistics (fixed order, FP64 sum) and derive the normalisation of the grid.
cudaError_t launch_finalize(const TileStats* tiles, uint32_t ntiles, FrameScalars* fs, int mass_normalize,
    int minmax_normalize, double n_scale, double voxel_volume, cudaStream_t st);
cudaError_t launch_normalize_modes(float* grid, uint64_t nvox, const FrameScalars* fs, int mass_normalize,
    int minmax_normalize, int sms, cudaStream_t st);

}  // namespace p2v
