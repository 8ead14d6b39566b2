// Cell binning: typed particle lists -> float4 xyzr records + cell keys, their stable sort by cell with
// every particle's gather record in sorted order, and the per-cell start table of the sorted order.
// Two sorts give the same permutation bit for bit: a counting sort by cell (histogram, scan of the cell
// counts = the start table, scatter, and an index-order pass over the cells holding two or more particles;
// taken while no cell holds more than 32 particles) and a stable LSD radix sort (onesweep: one read and
// one write of the keys per 8- or 9-bit digit, decoupled look-back across tiles), which runs alone for
// sparse frames and as the device-side fallback of the counting sort.
//
// Reference semantics (plugins/datatools/src/ParticlesToDensity.cpp):
//   - particle components are read through SimpleSphericalParticles' accessors, i.e. converted to
//     float with static_cast (SimpleSphericalParticles.h:86-130, Accessor.h:33-117); FLOAT_XYZ,
//     DOUBLE_XYZ and SHORT_XYZ lists use the list's global radius (ParticlesToDensity.cpp:460-463,569-571)
//   - the cell of a particle is (p - min) / sliceDist in float (:564-568).
// The bin used for sorting is floor() of that quotient clamped to [-1, res] (one underflow and one
// overflow bin per axis collect everything outside the box); the footprint decisions later use the
// reference's truncation of the same quotient.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "p2v_common.cuh"
#include "p2v_internal.h"
#include "particle_record.cuh"

namespace p2v {

namespace {

template<class T>
__device__ __forceinline__ T load_unaligned(const uint8_t* p) {
    T v;
    uint8_t* d = reinterpret_cast<uint8_t*>(&v);
#pragma unroll
    for (int i = 0; i < (int) sizeof(T); ++i)
        d[i] = p[i];
    return v;
}

template<class T, bool ALIGNED>
__device__ __forceinline__ float load_comp(const uint8_t* p) {
    if (ALIGNED)
        return static_cast<float>(*reinterpret_cast<const T*>(p));
    return static_cast<float>(load_unaligned<T>(p));
}

__device__ __forceinline__ int32_t clamp_cell(float q) {
    // floor of the cell quotient, clamped to +-2^30 so it always fits an int
    float f = floorf(q);
    f = fminf(fmaxf(f, -1073741824.0f), 1073741824.0f);
    return static_cast<int32_t>(f);
}

__device__ __forceinline__ uint32_t lane_id() {
    return threadIdx.x & 31u;
}

// True when the particle's kernel support holds no grid node along some axis, by a margin that the density
// gather's own node ranges cannot contradict: the gather would add nothing for it. q: the particle's position
// in cells, (p - min) / h as the bin key takes it. In node units the nodes around the particle lie at in-cell
// offsets 0 and 1 from its offset phi = q - floor(q); neither is inside the support when phi and 1 - phi both
// exceed eps / h by 1e-3 plus the rounding of q and of a position the gather forms from a cell up to twice the
// grid size away (the gather's exactly rounded in-cell offset differs from phi by less than that).
__device__ __forceinline__ bool support_misses_nodes(const float q[3], float r, const GridGeo& g) {
    const float eps = g.kernel == 0 ? g.sigma * r : 3.0f * (g.sigma * r);
    bool miss = false;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float phi = q[a] - floorf(q[a]);
        const float eh = eps * g.ihh[a];
        const float m = 1e-3f + 1e-6f * static_cast<float>(g.s[a]) + 4e-7f * fabsf(q[a]);
        miss = miss || (phi - eh > m && (1.0f - phi) - eh > m);
    }
    return miss;
}

// Grid-stride over the list: each thread packs several particles and keeps running reductions, so the
// frame-wide maxima and counts cost one atomic per block rather than per 256 particles. empty_flag (a power of
// two above every cell key, or 0): added to the key of a particle whose support holds no node, so that the
// sort puts those particles after every other (in cell order) and the cell start table, which the density
// gather walks, leaves them out.
template<class T, int NC, bool ALIGNED>
__global__ void __launch_bounds__(256) pack_keys_kernel(ListDesc L, GridGeo g, float4* __restrict__ xyzr,
    uint32_t* __restrict__ keys, uint32_t* __restrict__ idx, FrameScalars* __restrict__ fs, uint32_t empty_flag) {
    __shared__ int32_t s_cmin[3][8], s_cmax[3][8];
    __shared__ uint32_t s_rmax[8], s_drop[8];
    int32_t cell[3] = {INT32_MAX, INT32_MAX, INT32_MAX};
    int32_t cellhi[3] = {INT32_MIN, INT32_MIN, INT32_MIN};
    uint32_t rbits = 0u, drop = 0u;
    const uint64_t step = (uint64_t) gridDim.x * blockDim.x;
    for (uint64_t i = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; i < L.count; i += step) {
        const uint8_t* rec = L.data + i * L.stride;
        const float x = load_comp<T, ALIGNED>(rec);
        const float y = load_comp<T, ALIGNED>(rec + sizeof(T));
        const float z = load_comp<T, ALIGNED>(rec + 2 * sizeof(T));
        const float r = NC == 4 ? load_comp<T, ALIGNED>(rec + 3 * sizeof(T)) : L.global_radius;
        const float p[3] = {x, y, z};
        bool valid = isfinite(x) && isfinite(y) && isfinite(z) && isfinite(r) && r > 0.0f;
        uint32_t bin[3];
        int32_t c[3];
        float qa[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const float q = (p[a] - g.minf[a]) / g.hf[a];
            qa[a] = q;
            valid = valid && fabsf(q) < 1073741824.0f;
            c[a] = clamp_cell(q);
            const int32_t b = c[a] < -1 ? -1 : (c[a] > g.s[a] ? g.s[a] : c[a]);
            bin[a] = static_cast<uint32_t>(b + 1);
        }
        uint32_t key = g.nbins;
        if (valid) {
            key = (bin[2] * g.nb[1] + bin[1]) * g.nb[0] + bin[0];
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                cell[a] = min(cell[a], c[a]);
                cellhi[a] = max(cellhi[a], c[a]);
            }
            rbits = max(rbits, __float_as_uint(r));
            if (empty_flag && support_misses_nodes(qa, r, g))
                key |= empty_flag;
        } else {
            ++drop;
        }
        const uint64_t o = L.offset + i;
        xyzr[o] = make_float4(x, y, z, r);
        keys[o] = key;
        if (idx)
            idx[o] = static_cast<uint32_t>(o);
    }
    // block reduction: one atomic per block and quantity
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        rbits = max(rbits, __shfl_xor_sync(0xffffffffu, rbits, o));
        drop += __shfl_xor_sync(0xffffffffu, drop, o);
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            cell[a] = min(cell[a], __shfl_xor_sync(0xffffffffu, cell[a], o));
            cellhi[a] = max(cellhi[a], __shfl_xor_sync(0xffffffffu, cellhi[a], o));
        }
    }
    const int w = threadIdx.x >> 5;
    if (lane_id() == 0) {
        s_rmax[w] = rbits;
        s_drop[w] = drop;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            s_cmin[a][w] = cell[a];
            s_cmax[a][w] = cellhi[a];
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const int nw = blockDim.x >> 5;
        for (int k = 1; k < nw; ++k) {
            s_rmax[0] = max(s_rmax[0], s_rmax[k]);
            s_drop[0] += s_drop[k];
            for (int a = 0; a < 3; ++a) {
                s_cmin[a][0] = min(s_cmin[a][0], s_cmin[a][k]);
                s_cmax[a][0] = max(s_cmax[a][0], s_cmax[a][k]);
            }
        }
        if (s_rmax[0])
            atomicMax(&fs->rmax_bits, s_rmax[0]);
        if (s_drop[0])
            atomicAdd(&fs->n_dropped, s_drop[0]);
        for (int a = 0; a < 3; ++a) {
            if (s_cmin[a][0] != INT32_MAX)
                atomicMin(&fs->cmin[a], s_cmin[a][0]);
            if (s_cmax[a][0] != INT32_MIN)
                atomicMax(&fs->cmax[a], s_cmax[a][0]);
        }
    }
}

// ---------------------------------------------------------------------------------------------
// Onesweep LSD radix sort of (key, value) pairs with 8- or 9-bit digits: a key of B bits takes
// ceil(B / 9) passes (a 256^3 grid's 25-bit bin keys take 9 + 8 + 8 bits, three passes).
// ---------------------------------------------------------------------------------------------
constexpr int SORT_THREADS = 256;
constexpr int SORT_WARPS = SORT_THREADS / 32;
constexpr int SORT_ITEMS = 16;
constexpr int SORT_TILE = SORT_THREADS * SORT_ITEMS;  // 4096 keys per tile
constexpr int MAX_RADIX = 512;
constexpr int MAX_PASSES = 5;
constexpr int HIST_WORDS = MAX_PASSES * MAX_RADIX;    // digit histograms, pass p at p * MAX_RADIX
// after the histograms: one tile counter per radix pass
constexpr int LOOKBACK_WINDOW = 8;  // predecessor tiles a look-back round reads at once (4: 3.55, 16: 3.49 ms)
constexpr uint32_t FLAG_AGG = 1u << 30;
constexpr uint32_t FLAG_PRE = 2u << 30;
constexpr uint32_t FLAG_MASK = 3u << 30;
constexpr uint32_t COUNT_MASK = (1u << 30) - 1u;

struct SortPlan {
    int passes;
    int shift[MAX_PASSES];
    int bits[MAX_PASSES];
};

// odd: an odd number of passes, so the sorted keys end in buffer 1 (8-bit digits where a pass is added)
SortPlan sort_plan(uint32_t max_key, bool odd = false) {
    int nb = 0;
    while (nb < 32 && (max_key >> nb) != 0u)
        ++nb;
    nb = std::max(nb, 1);
    SortPlan pl{};
    pl.passes = (nb + 8) / 9;
    if (odd && (pl.passes & 1) == 0)
        ++pl.passes;
    // the first (nb - 8 * passes) passes take 9 bits, the others 8
    int nine = std::max(0, nb - 8 * pl.passes);
    int sh = 0;
    for (int p = 0; p < pl.passes; ++p) {
        pl.bits[p] = p < nine ? 9 : 8;
        pl.shift[p] = sh;
        sh += pl.bits[p];
    }
    return pl;
}

constexpr uint32_t BIN_CELL_MAX = 32;  // the counting sort orders cells of up to this many particles

// The radix path runs unless the counting sort (count_bins / scan_bins / scatter_bins / order_bins) took the
// frame: with a gate, every radix kernel returns at once when the frame's fullest cell fits the counting
// sort's per-cell ordering.
__device__ __forceinline__ bool radix_skipped(const FrameScalars* gate) {
    return gate != nullptr && gate->bin_maxcount <= BIN_CELL_MAX;
}

__global__ void __launch_bounds__(256) radix_hist_kernel(const uint32_t* __restrict__ keys, uint32_t n, SortPlan pl,
    uint32_t* __restrict__ hist, const FrameScalars* __restrict__ gate) {
    if (radix_skipped(gate))
        return;
    __shared__ uint32_t sh[HIST_WORDS];
    for (int i = threadIdx.x; i < HIST_WORDS; i += blockDim.x)
        sh[i] = 0;
    __syncthreads();
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        const uint32_t k = keys[j];
        for (int p = 0; p < pl.passes; ++p)
            atomicAdd(&sh[p * MAX_RADIX + ((k >> pl.shift[p]) & ((1u << pl.bits[p]) - 1u))], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < pl.passes * MAX_RADIX; i += blockDim.x)
        if (sh[i])
            atomicAdd(&hist[i], sh[i]);
}

// Exclusive scan of each pass' digit histogram (one block of MAX_RADIX threads).
__global__ void __launch_bounds__(MAX_RADIX) radix_scan_kernel(uint32_t* hist, int passes,
                                                                const FrameScalars* __restrict__ gate) {
    if (radix_skipped(gate))
        return;
    __shared__ uint32_t s[MAX_RADIX];
    for (int p = 0; p < passes; ++p) {
        const uint32_t v = hist[p * MAX_RADIX + threadIdx.x];
        s[threadIdx.x] = v;
        __syncthreads();
        for (int o = 1; o < MAX_RADIX; o <<= 1) {
            const uint32_t t = threadIdx.x >= (unsigned) o ? s[threadIdx.x - o] : 0u;
            __syncthreads();
            s[threadIdx.x] += t;
            __syncthreads();
        }
        hist[p * MAX_RADIX + threadIdx.x] = s[threadIdx.x] - v;
        __syncthreads();
    }
}

__device__ __forceinline__ uint32_t ld_volatile(const uint32_t* p) {
    return *reinterpret_cast<const volatile uint32_t*>(p);
}

__device__ __forceinline__ void st_volatile(uint32_t* p, uint32_t v) {
    *reinterpret_cast<volatile uint32_t*>(p) = v;
}

// One pass over digit (key >> shift) & (RADIX - 1). Tiles are taken in launch order from a counter; each
// tile ranks its keys stably (peer lanes from ballots on the digit bits, per-warp digit counters), publishes its digit
// counts, resolves its global offsets by decoupled look-back, stages the tile in digit order in shared
// memory and writes runs of equal digits contiguously.
// The look-back waits are bounded (wait_polls polls of a predecessor that has published nothing). A wait
// that runs out records ERR_LOOKBACK_TIMEOUT; every other wait then stops at its next poll and later passes
// return at once. A tile that gave up adds only the counts it saw, so its destinations stay at or below the
// true ones (inside the output); sort_sanitize_kernel then replaces the unfinished output by a valid one.
template<bool GATHER, int BITS>
__global__ void __launch_bounds__(SORT_THREADS, 3) onesweep_kernel(const uint32_t* __restrict__ keys_in,
    const uint32_t* __restrict__ vals_in, uint32_t* __restrict__ keys_out, uint32_t* __restrict__ vals_out, uint32_t n,
    int shift, const uint32_t* __restrict__ digit_offsets, uint32_t* __restrict__ tile_counter,
    uint32_t* __restrict__ status, uint32_t* __restrict__ err, const float4* __restrict__ xyzr_in,
    float4* __restrict__ rec_a, int4* __restrict__ rec_b, float4* __restrict__ xyzr_out, GridGeo geo,
    const FrameScalars* __restrict__ gate, uint32_t wait_polls, int32_t hold_tile) {
    if (radix_skipped(gate) || (ld_volatile(err) & ERR_LOOKBACK_TIMEOUT))
        return;
    constexpr int RADIX = 1 << BITS;
    constexpr uint32_t DMASK = RADIX - 1u;
    constexpr int DPT = RADIX / SORT_THREADS;  // digits per thread in the per-digit phases
    extern __shared__ __align__(16) uint32_t sort_smem[];
    uint32_t* s_keys = sort_smem;                                                  // [SORT_TILE]
    uint32_t* s_vals = s_keys + SORT_TILE;                                         // [SORT_TILE]
    uint32_t(*s_whist)[RADIX] = reinterpret_cast<uint32_t(*)[RADIX]>(s_vals + SORT_TILE);  // [SORT_WARPS][RADIX]
    uint32_t* s_base = s_vals + SORT_TILE + SORT_WARPS * RADIX;  // global destination of each digit's first item
    uint32_t* s_local = s_base + RADIX;                          // tile-local exclusive offset of each digit
    __shared__ uint32_t s_scan[SORT_WARPS];
    __shared__ uint32_t s_tile;

    const int tid = threadIdx.x;
    const int w = tid >> 5;
    const uint32_t lane = lane_id();
    if (tid == 0)
        s_tile = atomicAdd(tile_counter, 1u);
    for (int i = tid; i < SORT_WARPS * RADIX; i += SORT_THREADS)
        (&s_whist[0][0])[i] = 0u;
    __syncthreads();
    const uint32_t tile = s_tile;
    const uint32_t base = tile * SORT_TILE;

    // warp-striped load: item i of lane l of warp w is element base + w*32*ITEMS + i*32 + l, so the
    // ranking order (i, lane) is the input order within the warp and warps follow each other.
    uint32_t k[SORT_ITEMS], v[SORT_ITEMS], rk[SORT_ITEMS];
    const uint32_t wbase = base + w * 32 * SORT_ITEMS;
#pragma unroll
    for (int i = 0; i < SORT_ITEMS; ++i) {
        const uint32_t j = wbase + i * 32 + lane;
        k[i] = j < n ? keys_in[j] : 0u;
        v[i] = j < n ? (vals_in ? vals_in[j] : j) : 0u;  // no input values: the identity (particle indices)
    }
    const uint32_t lt_mask = (1u << lane) - 1u;
#pragma unroll
    for (int i = 0; i < SORT_ITEMS; ++i) {
        const uint32_t j = wbase + i * 32 + lane;
        const bool valid = j < n;
        const uint32_t d = (k[i] >> shift) & DMASK;
        // the lanes holding the same digit, from one ballot per digit bit and one on validity (cheaper than a
        // warp match: the 64M frame's binning went from 3.59 to 3.34 ms)
        const uint32_t vmask = __ballot_sync(0xffffffffu, valid);
        uint32_t peers = valid ? vmask : (1u << lane);
#pragma unroll
        for (int bit = 0; bit < BITS; ++bit) {
            const bool set = (d >> bit) & 1u;
            const uint32_t bal = __ballot_sync(0xffffffffu, set);
            peers &= set ? bal : ~bal;
        }
        const uint32_t cnt = __popc(peers);
        const uint32_t before = __popc(peers & lt_mask);
        const uint32_t leader = __ffs(peers) - 1;
        uint32_t b = valid ? s_whist[w][d] : 0u;
        __syncwarp();
        if (valid && lane == leader)
            s_whist[w][d] = b + cnt;
        __syncwarp();
        rk[i] = b + before;
    }
    __syncthreads();

    // per digit (thread tid owns digits tid*DPT .. tid*DPT + DPT-1): exclusive offsets over warps, counts
    uint32_t count[DPT];
    uint32_t tsum = 0;
#pragma unroll
    for (int e = 0; e < DPT; ++e) {
        const int d = tid * DPT + e;
        uint32_t run = 0;
#pragma unroll
        for (int ww = 0; ww < SORT_WARPS; ++ww) {
            const uint32_t c = s_whist[ww][d];
            s_whist[ww][d] = run;
            run += c;
        }
        count[e] = run;
        tsum += run;
        // publish the tile aggregate (or the inclusive prefix for tile 0) before looking back
        if ((int32_t) tile != hold_tile)
            st_volatile(status + (size_t) tile * RADIX + d, (tile == 0 ? FLAG_PRE : FLAG_AGG) | run);
    }
    // tile-local exclusive scan over digits (block scan of the per-thread digit sums)
    uint32_t incl = tsum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= (uint32_t) o)
            incl += t;
    }
    if (lane == 31)
        s_scan[w] = incl;
    __syncthreads();
    uint32_t wpre = 0;
    for (int ww = 0; ww < w; ++ww)
        wpre += s_scan[ww];
    uint32_t run = wpre + incl - tsum;
#pragma unroll
    for (int e = 0; e < DPT; ++e) {
        s_local[tid * DPT + e] = run;
        run += count[e];
    }

    // decoupled look-back per digit, LOOKBACK_WINDOW predecessors per round: the window's loads are independent,
    // so a round costs one memory latency however many of its tiles have only published their aggregate (the
    // inclusive prefixes trail the tiles in flight by ~30 tiles on large frames: walking them one load at a time
    // made the look-back the key passes' bottleneck). A round consumes the window's tiles up to the first one
    // that has published nothing; a round that consumes none is a poll of the bounded wait.
#pragma unroll
    for (int e = 0; e < DPT; ++e) {
        const int d = tid * DPT + e;
        uint32_t excl = 0;
        if (tile > 0) {
            int32_t t = (int32_t) tile - 1;
            uint32_t spins = 0;
            bool done = false;
            while (!done) {
                uint32_t sv[LOOKBACK_WINDOW];
#pragma unroll
                for (int q = 0; q < LOOKBACK_WINDOW; ++q)
                    sv[q] = t - q >= 0 ? ld_volatile(status + (size_t) (t - q) * RADIX + d) : FLAG_PRE;
                int used = 0;
#pragma unroll
                for (int q = 0; q < LOOKBACK_WINDOW; ++q) {
                    if (done || used < q || (sv[q] & FLAG_MASK) == 0u)
                        continue;  // stop at the first tile without a published count
                    excl += sv[q] & COUNT_MASK;
                    done = (sv[q] & FLAG_MASK) == FLAG_PRE;
                    used = q + 1;
                }
                if (done)
                    break;
                t -= used;
                if (used == 0) {
                    if (++spins > wait_polls) {
                        atomicOr(err, ERR_LOOKBACK_TIMEOUT);
                        break;
                    }
                    if (ld_volatile(err) & ERR_LOOKBACK_TIMEOUT)
                        break;  // another wait gave up: the pass is void
                }
            }
            if ((int32_t) tile != hold_tile)
                st_volatile(status + (size_t) tile * RADIX + d, FLAG_PRE | (excl + count[e]));
        }
        s_base[d] = digit_offsets[d] + excl;
    }
    __syncthreads();

    // stage the tile in digit order, then write runs of equal digits contiguously
#pragma unroll
    for (int i = 0; i < SORT_ITEMS; ++i) {
        const uint32_t j = wbase + i * 32 + lane;
        if (j < n) {
            const uint32_t dd = (k[i] >> shift) & DMASK;
            const uint32_t lp = s_local[dd] + s_whist[w][dd] + rk[i];
            s_keys[lp] = k[i];
            s_vals[lp] = v[i];
        }
    }
    __syncthreads();
    const uint32_t tile_n = n - base < (uint32_t) SORT_TILE ? n - base : (uint32_t) SORT_TILE;
    if (!GATHER) {
        for (uint32_t j = tid; j < tile_n; j += SORT_THREADS) {
            const uint32_t kk = s_keys[j];
            const uint32_t dd = (kk >> shift) & DMASK;
            const uint32_t dst = s_base[dd] + (j - s_local[dd]);
            keys_out[dst] = kk;
            vals_out[dst] = s_vals[j];
        }
        return;
    }
    // last pass: emit every particle's gather record (and its xyzr) in sorted order. The xyzr reads are
    // scattered (input order): each thread issues GATHER_BATCH of them before it uses the first, so that
    // enough reads are in flight to cover their latency
    constexpr int GATHER_BATCH = 4;
    for (uint32_t j0 = tid; j0 < tile_n; j0 += GATHER_BATCH * SORT_THREADS) {
        uint32_t dst[GATHER_BATCH], vv[GATHER_BATCH];
        float4 p[GATHER_BATCH];
#pragma unroll
        for (int q = 0; q < GATHER_BATCH; ++q) {
            const uint32_t j = j0 + q * SORT_THREADS;
            if (j < tile_n) {
                const uint32_t kk = s_keys[j];
                const uint32_t dd = (kk >> shift) & DMASK;
                dst[q] = s_base[dd] + (j - s_local[dd]);
                vv[q] = s_vals[j];
                keys_out[dst[q]] = kk;
                vals_out[dst[q]] = vv[q];
                p[q] = xyzr_in[vv[q]];
            }
        }
#pragma unroll
        for (int q = 0; q < GATHER_BATCH; ++q) {
            if (j0 + q * SORT_THREADS < tile_n) {
                float4 A;
                int4 B;
                make_record(p[q], geo, A, B);
                rec_a[REC_STRIDE * (size_t) dst[q]] = A;
                rec_b[REC_STRIDE * (size_t) dst[q]] = B;
                if (xyzr_out)
                    xyzr_out[dst[q]] = p[q];
            }
        }
    }
}

// After a radix sort whose look-back gave up: every particle gets the invalid key nbins and the identity
// order, a valid sorted state (an empty grid), so that no later stage indexes with unfinished output. The
// frame reports P2V_ETIMEOUT.
__global__ void __launch_bounds__(256) sort_sanitize_kernel(uint32_t* __restrict__ keys, uint32_t* __restrict__ vals,
    uint32_t n, uint32_t nbins, const uint32_t* __restrict__ err, const FrameScalars* __restrict__ gate) {
    if (radix_skipped(gate) || !(ld_volatile(err) & ERR_LOOKBACK_TIMEOUT))
        return;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        keys[i] = nbins;
        vals[i] = i;
    }
}

// start[c] = first sorted position whose key is >= c, for c in [0, nbins]. Boundary i of the sorted keys
// (between keys[i-1] and keys[i]) starts the cells (keys[i-1], keys[i]]. boundary_starts_kernel<G> writes
// the start of every G-th cell there: out[b] = start[G b] for the b whose cell G b lies in that range; a run
// of more than RUN (64 cells, 32 blocks) is queued in chunks of at most GAP_CHUNK for cell_gap_fill_kernel
// (a sparse grid holds runs of millions of empty cells). Runs are disjoint and longer than RUN, so the
// chunks number at most (nbins / G + 1) (1/GAP_CHUNK + 1/(RUN + 1)), below the nbins / 64 + 2 entries the
// list holds. Dense frames (fewer than 8 cells per particle) take G = 1: the table directly. Sparse frames
// take G = CELL_BLOCK, then cell_starts_kernel: every cell searches the keys of its block, which lie in
// [out[b], out[b+1]) (up to n for the last block), and its thread stores start[c] (coalesced; per-boundary
// threads would write gaps of tens of cells each, one scattered sector per store).
constexpr uint32_t GAP_CHUNK = 8192;
constexpr uint32_t CELL_BLOCK = 64;

template<uint32_t G>
__global__ void __launch_bounds__(256) boundary_starts_kernel(const uint32_t* __restrict__ keys, uint32_t n,
    uint32_t nbins, uint32_t* __restrict__ out, uint4* __restrict__ gaps, uint32_t gap_cap,
    FrameScalars* __restrict__ fs, const FrameScalars* __restrict__ gate) {
    constexpr uint32_t RUN = G == 1 ? 64u : 32u;
    if (radix_skipped(gate))
        return;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i <= n; i += gridDim.x * blockDim.x) {
        const uint32_t lo = i == 0 ? 0u : keys[i - 1] + 1u;
        uint32_t hi = i == n ? nbins : keys[i];
        if (hi > nbins)
            hi = nbins;
        if (lo > hi)
            continue;
        const uint32_t b0 = (uint32_t) (((uint64_t) lo + G - 1) / G), b1 = hi / G;
        if (b0 > b1)
            continue;
        if (b1 - b0 < RUN) {
            for (uint32_t bb = b0; bb <= b1; ++bb)
                out[bb] = i;
        } else {
            const uint32_t nch = (uint32_t) (((uint64_t) b1 - b0 + GAP_CHUNK) / GAP_CHUNK);
            const uint32_t slot = atomicAdd(&fs->ngaps, nch);
            for (uint32_t q = 0; q < nch; ++q) {
                const uint64_t c0 = (uint64_t) b0 + (uint64_t) q * GAP_CHUNK;
                const uint64_t c1 = std::min<uint64_t>(b1, c0 + GAP_CHUNK - 1);
                if ((uint64_t) slot + q < gap_cap)
                    gaps[slot + q] = make_uint4((uint32_t) c0, (uint32_t) c1, i, 0u);
                else
                    atomicOr(&fs->error, ERR_GAP_OVERFLOW);
            }
        }
    }
}

// The dense table (G = 1) with coalesced stores: a warp takes 32 consecutive boundaries, scans the lengths of
// their runs of up to RUN cells, and its lanes then write the cells of all 32 runs together (consecutive lanes,
// consecutive cells; each lane finds the boundary owning its cell by a binary search over the scanned lengths).
// Longer runs go to the gap list as in boundary_starts_kernel. Per-thread run loops stored one scattered
// sector per cell and lane; the cells a boundary owns get longer when particles whose support holds no node
// are sorted behind the others.
__global__ void __launch_bounds__(256) boundary_starts_dense_kernel(const uint32_t* __restrict__ keys, uint32_t n,
    uint32_t nbins, uint32_t* __restrict__ out, uint4* __restrict__ gaps, uint32_t gap_cap,
    FrameScalars* __restrict__ fs, const FrameScalars* __restrict__ gate) {
    constexpr uint32_t RUN = 64u;
    if (radix_skipped(gate))
        return;
    const uint32_t lane = lane_id();
    const uint64_t wstride = (uint64_t) gridDim.x * blockDim.x;
    for (uint64_t base = (uint64_t) blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base <= n; base += wstride) {
        const uint64_t i64 = base + lane;
        uint32_t lo = 1u, hi = 0u;  // empty run
        if (i64 <= n) {
            const uint32_t i = (uint32_t) i64;
            lo = i == 0 ? 0u : keys[i - 1] + 1u;
            hi = i == n ? nbins : keys[i];
            if (hi > nbins)
                hi = nbins;
        }
        uint32_t len = lo <= hi ? hi - lo + 1u : 0u;
        if (len > RUN) {
            const uint32_t i = (uint32_t) i64;
            const uint32_t nch = (uint32_t) (((uint64_t) len - 1 + GAP_CHUNK) / GAP_CHUNK);
            const uint32_t slot = atomicAdd(&fs->ngaps, nch);
            for (uint32_t q = 0; q < nch; ++q) {
                const uint64_t c0 = (uint64_t) lo + (uint64_t) q * GAP_CHUNK;
                const uint64_t c1 = std::min<uint64_t>(hi, c0 + GAP_CHUNK - 1);
                if ((uint64_t) slot + q < gap_cap)
                    gaps[slot + q] = make_uint4((uint32_t) c0, (uint32_t) c1, i, 0u);
                else
                    atomicOr(&fs->error, ERR_GAP_OVERFLOW);
            }
            len = 0u;
        }
        uint32_t incl = len;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= (uint32_t) o)
                incl += t;
        }
        const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
        const uint32_t pre = incl - len;  // first cell slot of this lane's run
        for (uint32_t j0 = 0; j0 < total; j0 += 32) {
            const uint32_t j = j0 + lane;
            // owner: the last lane whose run starts at or before slot j (lanes with empty runs share the next
            // lane's start and are passed over: the search ends on the last of equal starts)
            uint32_t ow = 0;
#pragma unroll
            for (int step = 16; step > 0; step >>= 1) {
                const uint32_t cand = ow + step;
                const uint32_t pc = __shfl_sync(0xffffffffu, pre, cand);
                if (pc <= j)
                    ow = cand;
            }
            const uint32_t olo = __shfl_sync(0xffffffffu, lo, ow);
            const uint32_t opre = __shfl_sync(0xffffffffu, pre, ow);
            if (j < total)
                out[olo + (j - opre)] = (uint32_t) (base + ow);
        }
    }
}

__global__ void __launch_bounds__(256) cell_starts_kernel(const uint32_t* __restrict__ keys, uint32_t n,
    uint32_t nbins, const uint32_t* __restrict__ bstart, uint32_t nblk, uint32_t* __restrict__ start,
    const FrameScalars* __restrict__ gate) {
    if (radix_skipped(gate))
        return;
    const uint64_t c = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x;
    if (c > nbins)
        return;
    const uint32_t b = (uint32_t) (c / CELL_BLOCK);
    uint32_t lo = bstart[b], hi = b + 1 < nblk ? bstart[b + 1] : n;
    while (lo < hi) {
        const uint32_t mid = lo + ((hi - lo) >> 1);
        if ((uint64_t) keys[mid] < c)
            lo = mid + 1;
        else
            hi = mid;
    }
    start[c] = lo;
}

__global__ void __launch_bounds__(256) cell_gap_fill_kernel(const uint4* __restrict__ gaps, uint32_t gap_cap,
    uint32_t* __restrict__ start, const FrameScalars* __restrict__ fs, const FrameScalars* __restrict__ gate) {
    if (radix_skipped(gate))
        return;
    const uint32_t ng = min(fs->ngaps, gap_cap);
    for (uint32_t g = blockIdx.x; g < ng; g += gridDim.x) {
        const uint4 e = gaps[g];
        for (uint32_t c = e.x + threadIdx.x; c <= e.y; c += blockDim.x)
            start[c] = e.z;
    }
}

// ---- counting sort by cell ----
// counts[key] = particles per key, keys in [0, nbins] (nbins: the invalid particles); rank[i] = the
// particle's arrival rank in its cell (its slot there until order_bins_kernel fixes the order)
__global__ void __launch_bounds__(256) count_bins_kernel(const uint32_t* __restrict__ keys, uint32_t n,
                                                         uint32_t* __restrict__ counts, uint32_t* __restrict__ rank) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        rank[i] = atomicAdd(counts + keys[i], 1u);
}

constexpr int SCAN_THREADS = 256, SCAN_ITEMS = 16, SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

// 16 consecutive counts of thread `tid` in tile `tile` (zeros past nb); true when all 16 exist
__device__ __forceinline__ bool load_counts(const uint32_t* __restrict__ counts, uint32_t nb, uint64_t b0,
                                            uint32_t v[SCAN_ITEMS]) {
    const bool full = b0 + SCAN_ITEMS <= nb;
    if (full) {
#pragma unroll
        for (int q = 0; q < SCAN_ITEMS / 4; ++q) {
            const uint4 u = reinterpret_cast<const uint4*>(counts + b0)[q];
            v[4 * q] = u.x;
            v[4 * q + 1] = u.y;
            v[4 * q + 2] = u.z;
            v[4 * q + 3] = u.w;
        }
    } else {
#pragma unroll
        for (int e = 0; e < SCAN_ITEMS; ++e)
            v[e] = b0 + e < nb ? counts[b0 + e] : 0u;
    }
    return full;
}

// Scan of the cell counts in three steps (tile sums, their scan, tile scans): no cross-tile waiting.
// Step 1: the sum of every tile of SCAN_TILE counts, and the largest count (fs->bin_maxcount).
__global__ void __launch_bounds__(SCAN_THREADS) bin_tile_sums_kernel(const uint32_t* __restrict__ counts, uint32_t nb,
    uint32_t* __restrict__ tsum, FrameScalars* __restrict__ fs) {
    __shared__ uint32_t s_sum[SCAN_THREADS / 32], s_max[SCAN_THREADS / 32];
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    uint32_t v[SCAN_ITEMS];
    load_counts(counts, nb, (uint64_t) blockIdx.x * SCAN_TILE + (uint64_t) tid * SCAN_ITEMS, v);
    uint32_t sum = 0, vmax = 0;
#pragma unroll
    for (int e = 0; e < SCAN_ITEMS; ++e) {
        sum += v[e];
        vmax = max(vmax, v[e]);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        sum += __shfl_xor_sync(0xffffffffu, sum, o);
        vmax = max(vmax, __shfl_xor_sync(0xffffffffu, vmax, o));
    }
    if (lane == 0) {
        s_sum[w] = sum;
        s_max[w] = vmax;
    }
    __syncthreads();
    if (tid == 0) {
        for (int k = 1; k < SCAN_THREADS / 32; ++k) {
            sum += s_sum[k];
            vmax = max(vmax, s_max[k]);
        }
        tsum[blockIdx.x] = sum;
        if (vmax > 0)
            atomicMax(&fs->bin_maxcount, vmax);
    }
}

// Step 2: exclusive scan of the tile sums in place (one block).
__global__ void __launch_bounds__(1024) bin_tile_scan_kernel(uint32_t* __restrict__ tsum, uint32_t ntiles) {
    __shared__ uint32_t s_warp[32];
    __shared__ uint32_t s_carry;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    if (tid == 0)
        s_carry = 0;
    __syncthreads();
    for (uint32_t base = 0; base < ntiles; base += 1024) {
        const uint32_t i = base + tid;
        const uint32_t x = i < ntiles ? tsum[i] : 0u;
        uint32_t incl = x;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o)
                incl += t;
        }
        if (lane == 31)
            s_warp[w] = incl;
        __syncthreads();
        if (w == 0) {
            uint32_t ws = s_warp[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t t = __shfl_up_sync(0xffffffffu, ws, o);
                if (lane >= o)
                    ws += t;
            }
            s_warp[lane] = ws;  // inclusive over warps
        }
        __syncthreads();
        const uint32_t carry = s_carry;
        const uint32_t excl = carry + (w > 0 ? s_warp[w - 1] : 0u) + incl - x;
        if (i < ntiles)
            tsum[i] = excl;
        __syncthreads();
        if (tid == 0)
            s_carry = carry + s_warp[31];
        __syncthreads();
    }
}

// Step 3: start[c] = tile prefix + the scan inside the tile, for c in [0, nb); cells holding two or more
// particles are appended to `multi` (their order inside the cell is fixed by order_bins_kernel).
__global__ void __launch_bounds__(SCAN_THREADS) bin_starts_kernel(const uint32_t* __restrict__ counts, uint32_t nb,
    const uint32_t* __restrict__ tsum, uint32_t* __restrict__ start, uint32_t* __restrict__ multi,
    FrameScalars* __restrict__ fs) {
    __shared__ uint32_t s_warp[SCAN_THREADS / 32];
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const uint64_t b0 = (uint64_t) blockIdx.x * SCAN_TILE + (uint64_t) tid * SCAN_ITEMS;
    uint32_t v[SCAN_ITEMS];
    const bool full = load_counts(counts, nb, b0, v);
    uint32_t sum = 0, nm = 0;
#pragma unroll
    for (int e = 0; e < SCAN_ITEMS; ++e) {
        sum += v[e];
        nm += v[e] >= 2u ? 1u : 0u;
    }
    uint32_t incl = sum, mincl = nm;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
        const uint32_t tm = __shfl_up_sync(0xffffffffu, mincl, o);
        if (lane >= o) {
            incl += t;
            mincl += tm;
        }
    }
    if (lane == 31)
        s_warp[w] = incl;
    // the warp's multi-particle cells take consecutive list entries
    const uint32_t mtot = __shfl_sync(0xffffffffu, mincl, 31);
    uint32_t mbase = 0;
    if (lane == 31 && mtot)
        mbase = atomicAdd(&fs->bin_nmulti, mtot);
    mbase = __shfl_sync(0xffffffffu, mbase, 31) + mincl - nm;
    __syncthreads();
    uint32_t wpre = 0;
    for (int k = 0; k < w; ++k)
        wpre += s_warp[k];
    uint32_t run = tsum[blockIdx.x] + wpre + incl - sum;
#pragma unroll
    for (int e = 0; e < SCAN_ITEMS; ++e) {
        if (v[e] >= 2u)
            multi[mbase++] = (uint32_t) (b0 + e);
        const uint32_t x = run;
        run += v[e];
        v[e] = x;
    }
    if (full) {
#pragma unroll
        for (int q = 0; q < SCAN_ITEMS / 4; ++q)
            reinterpret_cast<uint4*>(start + b0)[q] = make_uint4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
    } else {
#pragma unroll
        for (int e = 0; e < SCAN_ITEMS; ++e)
            if (b0 + e < nb)
                start[b0 + e] = v[e];
    }
}

// Each particle takes slot start[key] + rank of its cell (arrival order within the cell, fixed by
// order_bins_kernel) and writes its index and its 32-byte gather record there. The sorted keys are not
// written: the cell starts hold them (keys_from_starts_kernel rebuilds them for the binning readback).
__global__ void __launch_bounds__(256) scatter_bins_kernel(const uint32_t* __restrict__ keys_in,
    const uint32_t* __restrict__ rank, const float4* __restrict__ xyzr, uint32_t n,
    const uint32_t* __restrict__ start, uint32_t* __restrict__ vals_out, float4* __restrict__ rec_a,
    int4* __restrict__ rec_b, float4* __restrict__ xyzr_out, GridGeo geo, const FrameScalars* __restrict__ fs) {
    if (fs->bin_maxcount > BIN_CELL_MAX)
        return;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t slot = start[keys_in[i]] + rank[i];
        vals_out[slot] = i;
        const float4 p = xyzr[i];
        float4 A;
        int4 B;
        make_record(p, geo, A, B);
        rec_a[REC_STRIDE * (size_t) slot] = A;
        rec_b[REC_STRIDE * (size_t) slot] = B;
        if (xyzr_out)
            xyzr_out[slot] = p;
    }
}

// Every cell with two or more particles (the list `multi`) puts them in index order (an insertion sort of
// at most BIN_CELL_MAX entries) and rewrites their values and records: the result is the stable sort by key.
__global__ void __launch_bounds__(256) order_bins_kernel(uint32_t n, uint32_t nbins, const uint32_t* __restrict__ multi,
    uint32_t* __restrict__ vals, const uint32_t* __restrict__ start, const float4* __restrict__ xyzr,
    float4* __restrict__ rec_a, int4* __restrict__ rec_b, float4* __restrict__ xyzr_out, GridGeo geo,
    const FrameScalars* __restrict__ fs) {
    if (fs->bin_maxcount > BIN_CELL_MAX)
        return;
    const uint32_t nm = fs->bin_nmulti;
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < nm; q += gridDim.x * blockDim.x) {
        const uint32_t k = multi[q];
        const uint32_t j = start[k];
        const uint32_t m = (k < nbins ? start[k + 1] : n) - j;
        uint32_t v[BIN_CELL_MAX];
        for (uint32_t a = 0; a < m; ++a) {
            const uint32_t x = vals[j + a];
            uint32_t b = a;
            while (b > 0 && v[b - 1] > x) {
                v[b] = v[b - 1];
                --b;
            }
            v[b] = x;
        }
        for (uint32_t a = 0; a < m; ++a) {
            if (vals[j + a] == v[a])
                continue;
            vals[j + a] = v[a];
            const float4 p = xyzr[v[a]];
            float4 A;
            int4 B;
            make_record(p, geo, A, B);
            rec_a[REC_STRIDE * (size_t) (j + a)] = A;
            rec_b[REC_STRIDE * (size_t) (j + a)] = B;
            if (xyzr_out)
                xyzr_out[j + a] = p;
        }
    }
}

// keys[j] = the cell whose start range holds sorted position j (the counting sort writes no keys)
__global__ void __launch_bounds__(256) keys_from_starts_kernel(const uint32_t* __restrict__ start, uint32_t nbins,
                                                               uint32_t n, uint32_t* __restrict__ keys) {
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k <= nbins; k += gridDim.x * blockDim.x) {
        const uint32_t e = k < nbins ? start[k + 1] : n;
        for (uint32_t j = start[k]; j < e; ++j)
            keys[j] = k;
    }
}

__global__ void count_valid_kernel(const uint32_t* __restrict__ start, uint32_t nbins, FrameScalars* fs) {
    fs->n_valid = start[nbins];
}

}  // namespace

// ---------------------------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------------------------
cudaError_t launch_pack_keys(const ListDesc& L, const GridGeo& g, float4* xyzr, uint32_t* keys, uint32_t* idx,
    FrameScalars* fs, uint32_t empty_flag, cudaStream_t st) {
    if (L.count == 0)
        return cudaSuccess;
    const dim3 block(256);
    // about 8 particles per thread; at most 64 resident-sized blocks per SM
    const dim3 grid((unsigned) std::max<uint64_t>(1, std::min<uint64_t>((L.count + 2047) / 2048, 152ull * 64)));
    const uintptr_t addr = reinterpret_cast<uintptr_t>(L.data);
    switch (L.type) {
    case 1: {  // FLOAT_XYZ
        bool al = (addr % 4 == 0) && (L.stride % 4 == 0);
        if (al)
            pack_keys_kernel<float, 3, true><<<grid, block, 0, st>>>(L, g, xyzr, keys, idx, fs, empty_flag);
        else
            pack_keys_kernel<float, 3, false><<<grid, block, 0, st>>>(L, g, xyzr, keys, idx, fs, empty_flag);
    } break;
    case 2: {  // FLOAT_XYZR
        bool al = (addr % 4 == 0) && (L.stride % 4 == 0);
        if (al)
            pack_keys_kernel<float, 4, true><<<grid, block, 0, st>>>(L, g, xyzr, keys, idx, fs, empty_flag);
        else
            pack_keys_kernel<float, 4, false><<<grid, block, 0, st>>>(L, g, xyzr, keys, idx, fs, empty_flag);
    } break;
    case 3: {  // SHORT_XYZ
        bool al = (addr % 2 == 0) && (L.stride % 2 == 0);
        if (al)
            pack_keys_kernel<uint16_t, 3, true><<<grid, block, 0, st>>>(L, g, xyzr, keys, idx, fs, empty_flag);
        else
            pack_keys_kernel<uint16_t, 3, false><<<grid, block, 0, st>>>(L, g, xyzr, keys, idx, fs, empty_flag);
    } break;
    case 4: {  // DOUBLE_XYZ
        bool al = (addr % 8 == 0) && (L.stride % 8 == 0);
        if (al)
            pack_keys_kernel<double, 3, true><<<grid, block, 0, st>>>(L, g, xyzr, keys, idx, fs, empty_flag);
        else
            pack_keys_kernel<double, 3, false><<<grid, block, 0, st>>>(L, g, xyzr, keys, idx, fs, empty_flag);
    } break;
    default:
        return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

size_t sort_status_words(uint32_t n) {
    return (size_t) ceil_div(n, SORT_TILE) * MAX_RADIX;
}

size_t sort_hist_words() {
    return HIST_WORDS + 8;
}

int sort_passes(uint32_t max_key) {
    return sort_plan(max_key).passes;
}

uint32_t sort_empty_flag(uint32_t max_key) {
    int nb = 0;
    while (nb < 32 && (max_key >> nb) != 0u)
        ++nb;
    if (nb >= 31)
        return 0u;
    const uint32_t flag = 1u << nb;
    return sort_plan(flag | (flag - 1u)).passes == sort_plan(max_key).passes ? flag : 0u;
}

template<bool GATHER, int BITS>
cudaError_t launch_onesweep_bits(uint32_t tiles, SortBuffers& b, int cur, uint32_t n, int shift, const uint32_t* offs,
                                 uint32_t* counter, cudaStream_t st, const FrameScalars* gate) {
    constexpr int RADIX = 1 << BITS;
    const int smem = (int) sizeof(uint32_t) * (2 * SORT_TILE + SORT_WARPS * RADIX + 2 * RADIX);
    const cudaError_t e = cudaFuncSetAttribute(onesweep_kernel<GATHER, BITS>,
                                               cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess)
        return e;
    onesweep_kernel<GATHER, BITS><<<tiles, SORT_THREADS, smem, st>>>(b.keys[cur],
        (cur == 0 && b.implicit_vals0 && b.first_pass) ? nullptr : b.vals[cur], b.keys[cur ^ 1],
        b.vals[cur ^ 1], n, shift, offs, counter, b.status, b.err, GATHER ? b.xyzr_in : nullptr,
        GATHER ? b.rec_a : nullptr, GATHER ? b.rec_b : nullptr, GATHER ? b.xyzr_out : nullptr, b.geo, gate,
        b.wait_polls ? b.wait_polls : SPIN_LIMIT, b.first_pass ? b.hold_tile : -1);
    return cudaSuccess;
}

template<bool GATHER>
cudaError_t launch_onesweep(int bits, uint32_t tiles, SortBuffers& b, int cur, uint32_t n, int shift,
                            const uint32_t* offs, uint32_t* counter, cudaStream_t st, const FrameScalars* gate) {
    return bits == 9 ? launch_onesweep_bits<GATHER, 9>(tiles, b, cur, n, shift, offs, counter, st, gate)
                     : launch_onesweep_bits<GATHER, 8>(tiles, b, cur, n, shift, offs, counter, st, gate);
}

cudaError_t launch_sort(SortBuffers& b, uint32_t n, uint32_t max_key, int sms, cudaStream_t st, const FrameScalars* gate,
                        bool odd) {
    const SortPlan pl = sort_plan(max_key, odd);
    const uint32_t tiles = ceil_div(n, SORT_TILE);
    cudaError_t e = cudaMemsetAsync(b.hist, 0, sizeof(uint32_t) * HIST_WORDS + sizeof(uint32_t) * MAX_PASSES, st);
    if (e != cudaSuccess)
        return e;
    b.result = pl.passes & 1;
    if (n == 0)
        return cudaSuccess;
    const unsigned hgrid = (unsigned) std::min<uint32_t>(ceil_div(n, 256 * 8), (uint32_t) sms * 4);
    radix_hist_kernel<<<hgrid ? hgrid : 1, 256, 0, st>>>(b.keys[0], n, pl, b.hist, gate);
    radix_scan_kernel<<<1, MAX_RADIX, 0, st>>>(b.hist, pl.passes, gate);
    int cur = 0;
    for (int p = 0; p < pl.passes; ++p) {
        b.first_pass = p == 0;
        e = cudaMemsetAsync(b.status, 0, sizeof(uint32_t) * (size_t) tiles * ((size_t) 1 << pl.bits[p]), st);
        if (e != cudaSuccess)
            return e;
        uint32_t* counter = b.hist + HIST_WORDS + p;
        const bool last = p == pl.passes - 1;
        if (last && b.xyzr_in != nullptr)
            e = launch_onesweep<true>(pl.bits[p], tiles, b, cur, n, pl.shift[p], b.hist + p * MAX_RADIX, counter, st,
                                      gate);
        else
            e = launch_onesweep<false>(pl.bits[p], tiles, b, cur, n, pl.shift[p], b.hist + p * MAX_RADIX, counter, st,
                                       gate);
        if (e != cudaSuccess)
            return e;
        cur ^= 1;
    }
    return cudaGetLastError();
}

cudaError_t launch_keys_from_starts(const uint32_t* start, uint32_t nbins, uint32_t n, uint32_t* keys, int sms,
                                    cudaStream_t st) {
    const unsigned grid = (unsigned) std::max<uint32_t>(1u, std::min<uint32_t>(ceil_div(nbins + 1, 256), (uint32_t) sms * 16));
    keys_from_starts_kernel<<<grid, 256, 0, st>>>(start, nbins, n, keys);
    return cudaGetLastError();
}

size_t bin_scan_words(uint32_t nbins) {
    return (size_t) ceil_div(nbins + 1, SCAN_TILE);
}

uint32_t cell_block_count(uint32_t nbins) {
    return (uint32_t) (((uint64_t) nbins + CELL_BLOCK) / CELL_BLOCK);  // blocks of cells 0 .. nbins
}

cudaError_t launch_bin_sort(SortBuffers& b, uint32_t n, const GridGeo& g, uint32_t* counts, uint32_t* start,
                            uint32_t* bstart, uint4* gaps, uint32_t gap_cap, FrameScalars* fs, int sms,
                            cudaStream_t st) {
    const uint32_t nb = g.nbins + 1;
    cudaError_t e;
    const bool counting = counts != nullptr && n > 0;
    if (counting) {
        // counting sort by cell: histogram, scan (= the cell starts), scatter, per-cell index order
        const uint32_t ntiles = (uint32_t) bin_scan_words(g.nbins);
        if ((e = cudaMemsetAsync(counts, 0, sizeof(uint32_t) * nb, st)) != cudaSuccess)
            return e;
        const unsigned pgrid = (unsigned) std::max<uint32_t>(1u, std::min<uint32_t>(ceil_div(n, 256), (uint32_t) sms * 16));
        // ranks in vals[0]: the gated radix sort then takes the identity as its first pass' values
        b.implicit_vals0 = true;
        count_bins_kernel<<<pgrid, 256, 0, st>>>(b.keys[0], n, counts, b.vals[0]);
        // tile sums in the status buffer; the multi-particle cell list in keys[1] (the counting sort writes no
        // sorted keys there)
        bin_tile_sums_kernel<<<ntiles, SCAN_THREADS, 0, st>>>(counts, nb, b.status, fs);
        bin_tile_scan_kernel<<<1, 1024, 0, st>>>(b.status, ntiles);
        bin_starts_kernel<<<ntiles, SCAN_THREADS, 0, st>>>(counts, nb, b.status, start, b.keys[1], fs);
        scatter_bins_kernel<<<pgrid, 256, 0, st>>>(b.keys[0], b.vals[0], b.xyzr_in, n, start, b.vals[1], b.rec_a,
                                                   b.rec_b, b.xyzr_out, b.geo, fs);
        order_bins_kernel<<<pgrid, 256, 0, st>>>(n, g.nbins, b.keys[1], b.vals[1], start, b.xyzr_in, b.rec_a, b.rec_b,
                                                 b.xyzr_out, b.geo, fs);
    }
    // the radix path: alone, or as the fallback (gated) when a cell holds more than BIN_CELL_MAX particles;
    // with the counting sort its pass count is odd so both leave the sorted keys in buffer 1
    const FrameScalars* gate = counting ? fs : nullptr;
    const uint32_t max_key = b.empty_flag ? (b.empty_flag | (b.empty_flag - 1u)) : g.nbins;
    if ((e = launch_sort(b, n, max_key, sms, st, gate, counting)) != cudaSuccess)
        return e;
    const unsigned grid = (unsigned) std::max<uint32_t>(1u, std::min<uint32_t>(ceil_div(n + 1, 256), sms * 8));
    if (n > 0)
        sort_sanitize_kernel<<<grid, 256, 0, st>>>(b.keys[b.result], b.vals[b.result], n, g.nbins, b.err, gate);
    if ((uint64_t) g.nbins < 8ull * n) {
        boundary_starts_dense_kernel<<<grid, 256, 0, st>>>(b.keys[b.result], n, g.nbins, start, gaps, gap_cap, fs, gate);
        cell_gap_fill_kernel<<<sms * 2, 256, 0, st>>>(gaps, gap_cap, start, fs, gate);
    } else {
        const uint32_t nblk = cell_block_count(g.nbins);
        boundary_starts_kernel<CELL_BLOCK><<<grid, 256, 0, st>>>(b.keys[b.result], n, g.nbins, bstart, gaps, gap_cap,
                                                                 fs, gate);
        cell_gap_fill_kernel<<<sms * 2, 256, 0, st>>>(gaps, gap_cap, bstart, fs, gate);
        cell_starts_kernel<<<(unsigned) (((uint64_t) g.nbins + 256) / 256), 256, 0, st>>>(b.keys[b.result], n,
                                                                                          g.nbins, bstart, nblk, start,
                                                                                          gate);
    }
    count_valid_kernel<<<1, 1, 0, st>>>(start, g.nbins, fs);
    return cudaGetLastError();
}

}  // namespace p2v
