// Deterministic cell-ordered density gather, its tile statistics, and the grid normalisation.
//
// Reference: ParticlesToDensity::createVolumeCPU (plugins/datatools/src/ParticlesToDensity.cpp:389-747).
// The reference scatters every particle into the (2f+1)^3 nodes of its footprint [c-f, c+f]
// (c = trunc((p-min)/h), f = ceil(r/h), :562-579), wraps node indices with (h+2s)%s in cyclic axes
// while measuring the distance to the unwrapped node (:583-614), and adds rbf(d, sigma*r) (:472-476).
// Here every node gathers instead: a CTA owns a tile of TX*TY*TZ nodes, each thread owns one x-row of
// TX nodes, and the CTA stages the particles of the cell rows around the tile (per cyclic image of the
// tile) in shared memory with coalesced float4 loads. A thread adds its candidates in a fixed order
// (image, cell row (z,y), sorted particle order) with Kahan-compensated FP32 sums, so the result is
// bitwise reproducible. The node set a particle reaches is the reference's footprint intersected with
// the kernel support; nodes outside the support receive exactly zero in the reference as well.
#include <cuda_runtime.h>

#include <cstdint>

#include "p2v_common.cuh"
#include "p2v_internal.h"
#include "particle_record.cuh"

namespace p2v {

namespace {

constexpr int GATHER_TX = 8;
constexpr int GATHER_TY = 16;
constexpr int GATHER_TZ = 16;
constexpr int MAX_IMAGES = 8;  // cyclic images per axis a tile may visit

// floor(a / b) for b > 0
__device__ __forceinline__ int floor_div(int a, int b) {
    const int q = a / b;
    return (a % b != 0 && a < 0) ? q - 1 : q;
}

struct Extent {
    int L[3], H[3];     // cell-bin rows [u - L, u + H] can hold candidates of node u
    int klo[3], khi[3]; // cyclic images of the tile to visit
    float eps2_max;
    int ok;
};

template<int TX, int TY, int TZ>
__global__ void __launch_bounds__(TY* TZ, 2) gather_kernel(GridGeo g, const float4* __restrict__ rec_a,
    const int4* __restrict__ rec_b, const uint32_t* __restrict__ start, float* __restrict__ grid,
    TileStats* __restrict__ tiles, FrameScalars* __restrict__ fs, int smax, int rmax) {
    constexpr int NT = TY * TZ;
    extern __shared__ __align__(16) unsigned char smem[];
    float* acc_s = reinterpret_cast<float*>(smem);                      // [TX][NT]
    float* acc_c = acc_s + TX * NT;                                      // [TX][NT]
    float4* sp = reinterpret_cast<float4*>(acc_c + TX * NT);             // [smax] phi xyz, support^2
    uint4* sm = reinterpret_cast<uint4*>(sp + smax);                     // [smax] boxes, cells, kernel scale
    uint32_t* row_beg = reinterpret_cast<uint32_t*>(sm + smax);          // [rmax]
    uint32_t* row_off = row_beg + rmax;                                  // [rmax + 1]
    __shared__ double s_dsum[NT / 32];
    __shared__ float s_fmin[NT / 32], s_fmax[NT / 32];
    __shared__ Extent s_ex;

    const int t = threadIdx.x;
    const int ty = t % TY;
    const int tz = t / TY;
    // tiles cover the slab [zlo, zhi) of the grid (z tile index offset by the slab's first tile)
    const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY, z0 = (blockIdx.z + g.zlo / TZ) * TZ;
    const bool row_in = (y0 + ty < g.s[1]) && (z0 + tz >= g.zlo) && (z0 + tz < g.zhi);
    const int T3[3] = {TX, TY, TZ};

#pragma unroll
    for (int k = 0; k < TX; ++k) {
        acc_s[k * NT + t] = 0.0f;
        acc_c[k * NT + t] = 0.0f;
    }

    const bool bump = g.kernel == 0;
    const float E45 = __expf(-4.5f);
    // ---- candidate extents from the largest radius, once per CTA ----
    if (t == 0) {
        const float rmax_r = __uint_as_float(fs->rmax_bits);
        Extent ex;
        ex.ok = rmax_r > 0.0f;
        const float eps_max = bump ? g.sigma * rmax_r : 3.0f * (g.sigma * rmax_r);
        // enlarged slightly so rounding never prunes a contributing cell row
        ex.eps2_max = eps_max * eps_max * 1.0001f;
        const int o3[3] = {x0, y0, z0};
        for (int a = 0; a < 3 && ex.ok; ++a) {
            int E = static_cast<int>(ceilf(eps_max / g.hhi[a] + 1e-3f));
            E = E < 1 ? 1 : E;
            const int F = bump ? static_cast<int>(fminf(ceilf(rmax_r / g.hf[a]), 255.0f)) : E;
            ex.L[a] = bump ? min(E, F + 1) : E;
            ex.H[a] = bump ? min(E - 1, F) : E - 1;
            if (ex.L[a] > 100) {  // staged cell offsets are kept in 8 bits
                atomicOr(&fs->error, ERR_WINDOW_TOO_WIDE);
                ex.L[a] = 100;
                ex.H[a] = min(ex.H[a], 100);
            }
            if (g.cyc[a]) {
                const int s = g.s[a];
                // images k with [o + k s - L, o + T - 1 + k s + H] meeting the occupied cells
                ex.klo[a] = -floor_div(-(fs->cmin[a] - o3[a] - T3[a] + 1 - ex.H[a]), s);
                ex.khi[a] = floor_div(fs->cmax[a] - o3[a] + ex.L[a], s);
                if (ex.khi[a] - ex.klo[a] + 1 > MAX_IMAGES) {
                    atomicOr(&fs->error, ERR_WINDOW_TOO_WIDE);
                    ex.khi[a] = ex.klo[a] + MAX_IMAGES - 1;
                }
            } else {
                ex.klo[a] = 0;
                ex.khi[a] = 0;
            }
        }
        s_ex = ex;
    }
    __syncthreads();
    const Extent ex = s_ex;

    if (ex.ok) {
        for (int kz = ex.klo[2]; kz <= ex.khi[2]; ++kz)
            for (int ky = ex.klo[1]; ky <= ex.khi[1]; ++ky)
                for (int kx = ex.klo[0]; kx <= ex.khi[0]; ++kx) {
                    const int u0[3] = {x0 + kx * g.s[0], y0 + ky * g.s[1], z0 + kz * g.s[2]};
                    int wlo[3], whi[3];
#pragma unroll
                    for (int a = 0; a < 3; ++a) {
                        wlo[a] = min(max(u0[a] - ex.L[a], -1), g.s[a]);
                        whi[a] = max(min(u0[a] + T3[a] - 1 + ex.H[a], g.s[a]), -1);
                    }
                    const int nwy = whi[1] - wlo[1] + 1;
                    const int nwz = whi[2] - wlo[2] + 1;
                    if (nwy > rmax) {
                        if (t == 0)
                            atomicOr(&fs->error, ERR_STAGE_OVERFLOW);
                        continue;
                    }
                    const int planes_per_chunk = rmax / nwy;
                    // This thread's node row (unwrapped) and its candidate cell rows. Each end is first
                    // clamped to the bin range [-1, s]: bins -1 and s hold every particle beyond the box,
                    // so a row range lying wholly outside maps onto them.
                    const int uy = u0[1] + ty, uz = u0[2] + tz;
                    const int ry_lo = max(min(max(uy - ex.L[1], -1), g.s[1]), wlo[1]);
                    const int ry_hi = min(max(min(uy + ex.H[1], g.s[1]), -1), whi[1]);
                    const int rz_lo = max(min(max(uz - ex.L[2], -1), g.s[2]), wlo[2]);
                    const int rz_hi = min(max(min(uz + ex.H[2], g.s[2]), -1), whi[2]);
                    const uint32_t bx_lo = (uint32_t) (wlo[0] + 1), bx_end = (uint32_t) (whi[0] + 2);

                    for (int pz0 = 0; pz0 < nwz; pz0 += planes_per_chunk) {
                        const int pz1 = min(nwz, pz0 + planes_per_chunk);
                        const int nrows = (pz1 - pz0) * nwy;
                        __syncthreads();  // previous users of the row table are done
                        // row table: begin and staged count of every cell row of the chunk
                        for (int r = t; r < nrows; r += NT) {
                            const int zz = wlo[2] + pz0 + r / nwy;
                            const int yy = wlo[1] + r % nwy;
                            const uint32_t rowkey = ((uint32_t) (zz + 1) * g.nb[1] + (uint32_t) (yy + 1)) * g.nb[0];
                            const uint32_t b = start[rowkey + bx_lo];
                            const uint32_t e = start[rowkey + bx_end];
                            row_beg[r] = b;
                            row_off[r + 1] = e - b;
                        }
                        __syncthreads();
                        // exclusive scan of the row counts (one warp)
                        if (t < 32) {
                            uint32_t carry = 0;
                            for (int base = 0; base < nrows; base += 32) {
                                const int r = base + t;
                                uint32_t v = r < nrows ? row_off[r + 1] : 0u;
#pragma unroll
                                for (int o = 1; o < 32; o <<= 1) {
                                    uint32_t u = __shfl_up_sync(0xffffffffu, v, o);
                                    if (t >= o)
                                        v += u;
                                }
                                if (r < nrows)
                                    row_off[r + 1] = carry + v;
                                carry += __shfl_sync(0xffffffffu, v, 31);
                            }
                            if (t == 0)
                                row_off[0] = 0;
                        }
                        __syncthreads();
                        const uint32_t total = row_off[nrows];
                        for (uint32_t cb = 0; cb < total; cb += (uint32_t) smax) {
                            const uint32_t cn = min((uint32_t) smax, total - cb);
                            if (cb > 0)
                                __syncthreads();  // previous chunk fully consumed
                            // ---- stage: coalesced 16-byte loads of the chunk's particle records ----
                            for (uint32_t si = t; si < cn; si += NT) {
                                const uint32_t f = cb + si;
                                int lo = 0, hi = nrows;  // row r with row_off[r] <= f < row_off[r+1]
                                while (hi - lo > 1) {
                                    const int mid = (lo + hi) >> 1;
                                    if (row_off[mid] <= f)
                                        lo = mid;
                                    else
                                        hi = mid;
                                }
                                const uint32_t j = row_beg[lo] + (f - row_off[lo]);
                                const float4 A = rec_a[REC_STRIDE * (size_t) j];
                                const int4 B = rec_b[REC_STRIDE * (size_t) j];
                                const float phi[3] = {A.x, A.y, A.z};
                                const int cf[3] = {B.x, B.y, B.z};
                                const uint32_t meta = (uint32_t) B.w;
                                const float r = A.w;
                                const float eps = bump ? g.sigma * r : 3.0f * (g.sigma * r);
                                int blo[3], bhi[3], crel[3];
                                bool empty = false;
#pragma unroll
                                for (int a = 0; a < 3; ++a) {
                                    const int cr = cf[a] - u0[a];
                                    const float pos = static_cast<float>(cr) + phi[a];
                                    const float eh = eps * g.ihh[a];
                                    // nodes k with |k - pos| < eps / h; a node the rounding drops lies at
                                    // the edge of the support, where the kernel is zero
                                    int lo_a = static_cast<int>(floorf(pos - eh)) + 1;
                                    int hi_a = static_cast<int>(ceilf(pos + eh)) - 1;
                                    if (bump) {
                                        const int f = (int) ((meta >> (8 * a)) & 0xFFu);
                                        const int ctr = cr + (int) ((meta >> (24 + a)) & 1u);
                                        lo_a = max(lo_a, ctr - f);
                                        hi_a = min(hi_a, ctr + f);
                                    }
                                    lo_a = max(lo_a, 0);
                                    hi_a = min(hi_a, T3[a] - 1);
                                    empty = empty || lo_a > hi_a;
                                    blo[a] = lo_a;
                                    bhi[a] = hi_a;
                                    crel[a] = max(min(cr, 120), -120);
                                }
                                uint4 m;
                                if (empty) {
                                    // lo = 127 lies outside every tile, so the y/z box test rejects it
                                    m.x = 0x7Fu | (0x7Fu << 16);
                                    m.y = 0x7Fu;
                                    m.z = 0u;
                                } else {
                                    m.x = (uint32_t) blo[0] | ((uint32_t) (bhi[0] - blo[0]) << 8) |
                                          ((uint32_t) blo[1] << 16) | ((uint32_t) (bhi[1] - blo[1]) << 24);
                                    m.y = (uint32_t) blo[2] | ((uint32_t) (bhi[2] - blo[2]) << 8) |
                                          ((uint32_t) (crel[0] & 0xFF) << 16) | ((uint32_t) (crel[1] & 0xFF) << 24);
                                    m.z = (uint32_t) (crel[2] & 0xFF);
                                }
                                float eps2, inv;
                                if (bump) {
                                    eps2 = eps * eps;
                                    inv = __frcp_rn(eps2);
                                } else {
                                    const float sg = g.sigma * r;
                                    eps2 = 9.0f * sg * sg;
                                    inv = __frcp_rn(2.0f * sg * sg);
                                }
                                m.w = __float_as_uint(inv);
                                sp[si] = make_float4(phi[0], phi[1], phi[2], eps2);
                                sm[si] = m;
                            }
                            __syncthreads();
                            // ---- accumulate: this thread's node row against its candidate rows ----
                            if (row_in) {
                                const int zr_lo = max(rz_lo, wlo[2] + pz0), zr_hi = min(rz_hi, wlo[2] + pz1 - 1);
                                for (int zz = zr_lo; zz <= zr_hi; ++zz) {
                                    // smallest z distance from this node row to cell row zz
                                    const int oz = zz - uz;
                                    const float gz = oz > 0 ? oz * g.hhi[2] : (oz < -1 ? (-oz - 1) * g.hhi[2] : 0.0f);
                                    for (int yy = ry_lo; yy <= ry_hi; ++yy) {
                                        const int oy = yy - uy;
                                        const float gy = oy > 0 ? oy * g.hhi[1] : (oy < -1 ? (-oy - 1) * g.hhi[1] : 0.0f);
                                        // bins -1 and s hold particles from arbitrarily far away: never pruned
                                        if (gy * gy + gz * gz >= ex.eps2_max && yy >= 0 && yy < g.s[1] && zz >= 0 &&
                                            zz < g.s[2])
                                            continue;
                                        const int r = (zz - wlo[2] - pz0) * nwy + (yy - wlo[1]);
                                        uint32_t a0 = row_off[r], a1 = row_off[r + 1];
                                        a0 = max(a0, cb);
                                        a1 = min(a1, cb + cn);
                                        for (uint32_t i = a0; i < a1; ++i) {
                                            const uint32_t li = i - cb;
                                            const uint4 m = sm[li];
                                            const uint32_t ylo = (m.x >> 16) & 0xFFu, yw = m.x >> 24;
                                            const uint32_t zlo = m.y & 0xFFu, zw = (m.y >> 8) & 0xFFu;
                                            if ((uint32_t) (ty - (int) ylo) > yw || (uint32_t) (tz - (int) zlo) > zw)
                                                continue;
                                            const float4 P = sp[li];
                                            const int cy = (int) (int8_t) (m.y >> 24);
                                            const int cz = (int) (int8_t) (m.z & 0xFFu);
                                            const int cx = (int) (int8_t) ((m.y >> 16) & 0xFFu);
                                            const float dy = g.hhi[1] * (static_cast<float>(ty - cy) - P.y);
                                            const float dz = g.hhi[2] * (static_cast<float>(tz - cz) - P.z);
                                            const float dyz = dy * dy + dz * dz;
                                            if (!(dyz < P.w))
                                                continue;
                                            const float inv = __uint_as_float(m.w);
                                            const int xlo = (int) (m.x & 0xFFu);
                                            const int xhi = xlo + (int) ((m.x >> 8) & 0xFFu);
                                            for (int k = xlo; k <= xhi; ++k) {
                                                const float dx = g.hhi[0] * (static_cast<float>(k - cx) - P.x);
                                                const float d2 = __fmaf_rn(dx, dx, dyz);
                                                if (!(d2 < P.w))
                                                    continue;
                                                // __frcp_rn is the correctly rounded reciprocal; __expf's
                                                // relative error stays below 1e-6 over the argument range
                                                // that yields values above 1e-7 of the kernel maximum.
                                                float v;
                                                if (bump) {
                                                    const float w = __fmaf_rn(-d2, inv, 1.0f);
                                                    v = w > 0.0f ? __expf(-__frcp_rn(w)) : 0.0f;
                                                } else {
                                                    v = fmaxf(__expf(-d2 * inv) - E45, 0.0f);
                                                }
                                                float* ps = acc_s + k * NT + t;
                                                float* pcmp = acc_c + k * NT + t;
                                                const float s = *ps;
                                                const float yv = v - *pcmp;
                                                const float tt = s + yv;
                                                *pcmp = (tt - s) - yv;
                                                *ps = tt;
                                            }
                                        }
                                    }
                                }
                            }
                        }
                    }
                }
    }

    // ---- write the tile and its statistics ----
    double dsum = 0.0;
    float vmin = INFINITY, vmax = -INFINITY;
    if (row_in) {
        float* out = grid + ((size_t) (z0 + tz - g.zlo) * g.s[1] + (y0 + ty)) * g.s[0] + x0;
#pragma unroll
        for (int k = 0; k < TX; ++k) {
            if (x0 + k < g.s[0]) {
                const float v = acc_s[k * NT + t] - acc_c[k * NT + t];
                out[k] = v;
                dsum += (double) v;
                vmin = fminf(vmin, v);
                vmax = fmaxf(vmax, v);
            }
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        dsum += __shfl_xor_sync(0xffffffffu, dsum, o);
        vmin = fminf(vmin, __shfl_xor_sync(0xffffffffu, vmin, o));
        vmax = fmaxf(vmax, __shfl_xor_sync(0xffffffffu, vmax, o));
    }
    if ((t & 31) == 0) {
        s_dsum[t >> 5] = dsum;
        s_fmin[t >> 5] = vmin;
        s_fmax[t >> 5] = vmax;
    }
    __syncthreads();
    if (t == 0) {
        for (int w = 1; w < NT / 32; ++w) {
            dsum += s_dsum[w];
            vmin = fminf(vmin, s_fmin[w]);
            vmax = fmaxf(vmax, s_fmax[w]);
        }
        TileStats ts;
        ts.sum = dsum;
        ts.vmin = vmin;
        ts.vmax = vmax;
        tiles[(blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x] = ts;
    }
}

// Candidate extents and cyclic images of one tile (shared by both gather kernels).
__device__ __forceinline__ Extent tile_extent(const GridGeo& g, FrameScalars* fs, const int o3[3], const int T3[3]) {
    const bool bump = g.kernel == 0;
    const float rmax_r = __uint_as_float(fs->rmax_bits);
    Extent ex;
    ex.ok = rmax_r > 0.0f;
    const float eps_max = bump ? g.sigma * rmax_r : 3.0f * (g.sigma * rmax_r);
    ex.eps2_max = eps_max * eps_max * 1.0001f;
    for (int a = 0; a < 3 && ex.ok; ++a) {
        int E = static_cast<int>(ceilf(eps_max / g.hhi[a] + 1e-3f));
        E = E < 1 ? 1 : E;
        const int F = bump ? static_cast<int>(fminf(ceilf(rmax_r / g.hf[a]), 255.0f)) : E;
        ex.L[a] = bump ? min(E, F + 1) : E;
        ex.H[a] = bump ? min(E - 1, F) : E - 1;
        if (ex.L[a] > 100) {
            atomicOr(&fs->error, ERR_WINDOW_TOO_WIDE);
            ex.L[a] = 100;
            ex.H[a] = min(ex.H[a], 100);
        }
        if (g.cyc[a]) {
            const int s = g.s[a];
            ex.klo[a] = -floor_div(-(fs->cmin[a] - o3[a] - T3[a] + 1 - ex.H[a]), s);
            ex.khi[a] = floor_div(fs->cmax[a] - o3[a] + ex.L[a], s);
            if (ex.khi[a] - ex.klo[a] + 1 > MAX_IMAGES) {
                atomicOr(&fs->error, ERR_WINDOW_TOO_WIDE);
                ex.khi[a] = ex.klo[a] + MAX_IMAGES - 1;
            }
        } else {
            ex.klo[a] = 0;
            ex.khi[a] = 0;
        }
    }
    return ex;
}

// One particle's node box as the warp-level walk needs it (held in registers, then published to
// shared memory field by field so that lanes reading different particles never conflict on a bank).
struct WarpPart {
    float d0[3];       // (box corner - particle) in cells, per axis
    float eps2, inv;   // squared support and kernel scale
    float iby;         // 1/by for decoding a box-local row index
    int bx, by;        // box extents in x and y
    int node0;         // tile index of the box corner
    float w;           // the particle's weight (the weighted aggregators)
};
constexpr int WP_FIELDS = 10;

// Fixed-point scale of the exact accumulation: contributions (all below 1) are rounded to multiples of
// 2^-32 and summed as 64-bit integers held in two 32-bit words per node (a 32-bit shared-memory atomic on
// the low word; the thread whose add wraps it carries into the high word), so every voxel holds the exact
// sum of its rounded FP32 contributions, independent of the order in which particles arrive.
constexpr float FIX_SCALE = 4294967296.0f;          // 2^32
constexpr float FIX_INV = 2.3283064365386963e-10f;  // 2^-32

// The float nearest (ties to even) to the fixed-point sum hi:lo times 2^-32, from 32-bit integer operations
// and one exact 32-bit conversion: the same value as __ull2float_rn(hi:lo) * 2^-32, without the 64-bit
// conversion, which like FP64 arithmetic runs on the narrow FP64 pipe of this part. q receives the rounded
// sum (v * 2^32, an integer).
__device__ __forceinline__ float fixed_to_float(uint32_t hi, uint32_t lo, unsigned long long& q) {
    const unsigned long long x = ((unsigned long long) hi << 32) | lo;
    const int sh = 40 - __clzll(x);  // bits below a 24-bit significand (x == 0: -24)
    if (sh <= 0) {
        q = x;  // below 2^24: exact
        return __uint2float_rn(lo) * FIX_INV;
    }
    unsigned long long m = x >> sh;
    const unsigned long long rem = x & ((1ull << sh) - 1ull), half = 1ull << (sh - 1);
    m += (rem > half || (rem == half && (m & 1ull))) ? 1ull : 0ull;  // m <= 2^24
    q = m << sh;
    // m * 2^(sh - 32): the significand converts exactly and the scale is a power of two (sh in [1, 40])
    return __uint2float_rn((uint32_t) m) * __int_as_float((95 + sh) << 23);
}

// Particle-major gather with exact, order-independent accumulation. A CTA owns a tile of TX*TY*TZ
// nodes held as 64-bit fixed-point sums in shared memory; for every cyclic image of the tile it walks
// the sorted particle records of the surrounding cell rows (coalesced 16-byte loads), and each thread
// adds its particle's kernel values to the nodes of the particle's footprint that lie in the tile.
//
// ACC selects the accumulation:
//   ACC_EXACT   the density: contributions < 1 in 2^-32 fixed point (see above);
//   ACC_FIXED_W the intensity aggregator (ParticlesToDensity.cpp:509-519): contribution = kernel value times
//               the particle's weight w (wts[j * wstride], sorted order), rounded to a multiple of 1 / wscale
//               with wscale = 2^31 / 2^ceil(log2 max|w|) and summed as a signed 64-bit integer (exact, order
//               independent; absolute resolution 2^-31 of the largest weight);
//   ACC_DOUBLE  the vector aggregator's direction and weight sums (:492-508): FP64 shared-memory atomics of
//               the FP32 contributions. Its finish divides two sums, so small sums need relative accuracy
//               (a fixed-point quantum would erase voxels reached only by kernel tails); the sums depend on
//               the arrival order only at the 1e-16 level, below the final rounding to FP32.
// The result is written with stride ostride.
constexpr int ACC_EXACT = 0, ACC_FIXED_W = 1, ACC_DOUBLE = 2;

// Sorted position of the f-th staged record: the row r with row_off[r] <= f < row_off[r + 1] holds it.
__device__ __forceinline__ uint32_t locate_record(const uint32_t* row_off, const uint32_t* row_beg, int nrows,
                                                  uint32_t f) {
    int lo = 0, hi = nrows;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (row_off[mid] <= f)
            lo = mid;
        else
            hi = mid;
    }
    return row_beg[lo] + (f - row_off[lo]);
}
template<int TX, int TY, int TZ, int NT, int ACC>
__global__ void __launch_bounds__(NT, 1024 / NT) gather_fixed_kernel(GridGeo g, const float4* __restrict__ rec_a,
    const int4* __restrict__ rec_b, const uint32_t* __restrict__ start, float* __restrict__ grid,
    TileStats* __restrict__ tiles, FrameScalars* __restrict__ fs, int rmax, const float* __restrict__ wts,
    int wstride, int ostride) {
    constexpr int NN = TX * TY * TZ;
    extern __shared__ __align__(16) unsigned char smem[];
    uint32_t* acc_lo = reinterpret_cast<uint32_t*>(smem);  // [NN] low words of the fixed-point sums
    uint32_t* acc_hi = acc_lo + NN;                        // [NN] high words
    unsigned long long* acc64 = reinterpret_cast<unsigned long long*>(smem);  // [NN] ACC_FIXED_W sums (same bytes)
    double* accd = reinterpret_cast<double*>(smem);                          // [NN] ACC_DOUBLE sums (same bytes)
    constexpr bool WEIGHTED = ACC != ACC_EXACT;
    uint32_t* row_beg = acc_hi + NN;                        // [rmax]
    uint32_t* row_off = row_beg + rmax;                                      // [rmax + 1]
    __shared__ double s_dsum[NT / 32];
    __shared__ unsigned long long s_isum[NT / 32], s_fsum[NT / 32];
    __shared__ float s_fmin[NT / 32], s_fmax[NT / 32];
    __shared__ Extent s_ex;
    __shared__ uint32_t s_part[WP_FIELDS][NT];
    __shared__ uint32_t s_pre[NT + 32];

    const int t = threadIdx.x;
    const uint32_t lane = t & 31u;
    const uint32_t warp = t >> 5;
    // tiles cover the slab [zlo, zhi) of the grid (z tile index offset by the slab's first tile)
    const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY, z0 = (blockIdx.z + g.zlo / TZ) * TZ;
    const int T3[3] = {TX, TY, TZ};
    const int o3[3] = {x0, y0, z0};
    for (int n = t; n < NN; n += NT) {
        acc_lo[n] = 0u;
        acc_hi[n] = 0u;
    }
    const bool bump = g.kernel == 0;
    const float E45 = __expf(-4.5f);
    float wscale = 1.0f, winv = 1.0f;
    if (ACC == ACC_FIXED_W) {
        const float wmax = __uint_as_float(fs->wmax_bits);
        if (wmax > 0.0f) {
            int e;
            frexpf(wmax, &e);  // wmax <= 2^e
            e = max(e, -90);
            wscale = ldexpf(1.0f, 31 - e);
            winv = ldexpf(1.0f, e - 31);
        }
    }
    if (t == 0)
        s_ex = tile_extent(g, fs, o3, T3);
    __syncthreads();
    const Extent ex = s_ex;

    if (ex.ok) {
        for (int kz = ex.klo[2]; kz <= ex.khi[2]; ++kz)
            for (int ky = ex.klo[1]; ky <= ex.khi[1]; ++ky)
                for (int kx = ex.klo[0]; kx <= ex.khi[0]; ++kx) {
                    const int u0[3] = {x0 + kx * g.s[0], y0 + ky * g.s[1], z0 + kz * g.s[2]};
                    int wlo[3], whi[3];
#pragma unroll
                    for (int a = 0; a < 3; ++a) {
                        wlo[a] = min(max(u0[a] - ex.L[a], -1), g.s[a]);
                        whi[a] = max(min(u0[a] + T3[a] - 1 + ex.H[a], g.s[a]), -1);
                    }
                    const int nwy = whi[1] - wlo[1] + 1;
                    const int nwz = whi[2] - wlo[2] + 1;
                    if (nwy > rmax) {
                        if (t == 0)
                            atomicOr(&fs->error, ERR_STAGE_OVERFLOW);
                        continue;
                    }
                    const int planes_per_chunk = rmax / nwy;
                    const uint32_t bx_lo = (uint32_t) (wlo[0] + 1), bx_end = (uint32_t) (whi[0] + 2);
                    for (int pz0 = 0; pz0 < nwz; pz0 += planes_per_chunk) {
                        const int pz1 = min(nwz, pz0 + planes_per_chunk);
                        const int nrows = (pz1 - pz0) * nwy;
                        __syncthreads();
                        for (int r = t; r < nrows; r += NT) {
                            const int zz = wlo[2] + pz0 + r / nwy;
                            const int yy = wlo[1] + r % nwy;
                            const uint32_t rowkey = ((uint32_t) (zz + 1) * g.nb[1] + (uint32_t) (yy + 1)) * g.nb[0];
                            const uint32_t b = start[rowkey + bx_lo];
                            row_beg[r] = b;
                            row_off[r + 1] = start[rowkey + bx_end] - b;
                        }
                        __syncthreads();
                        if (t < 32) {
                            uint32_t carry = 0;
                            for (int base = 0; base < nrows; base += 32) {
                                const int r = base + t;
                                uint32_t v = r < nrows ? row_off[r + 1] : 0u;
#pragma unroll
                                for (int o = 1; o < 32; o <<= 1) {
                                    uint32_t u = __shfl_up_sync(0xffffffffu, v, o);
                                    if (t >= o)
                                        v += u;
                                }
                                if (r < nrows)
                                    row_off[r + 1] = carry + v;
                                carry += __shfl_sync(0xffffffffu, v, 31);
                            }
                            if (t == 0)
                                row_off[0] = 0;
                        }
                        __syncthreads();
                        const uint32_t total = row_off[nrows];
                        // Each warp takes 32 consecutive records; every lane derives its particle's node
                        // box, then the warp walks the concatenated boxes 32 nodes at a time (a warp-level
                        // load-balanced search), so all lanes test nodes in lockstep.
                        // the warp's next 32 records are located and loaded one iteration ahead (their
                        // latency overlaps the current batch's nodes)
                        uint32_t jn = 0;
                        float4 An = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                        int4 Bn = make_int4(0, 0, 0, 0);
                        if (warp * 32 + lane < total) {
                            jn = locate_record(row_off, row_beg, nrows, warp * 32 + lane);
                            An = rec_a[REC_STRIDE * (size_t) jn];
                            Bn = rec_b[REC_STRIDE * (size_t) jn];
                        }
                        for (uint32_t base = warp * 32; base < total; base += NT) {
                            const uint32_t f = base + lane;
                            uint32_t nb = 0;
                            WarpPart wp;
                            const uint32_t j = jn;
                            const float4 A = An;
                            const int4 B = Bn;
                            if (f + NT < total) {
                                jn = locate_record(row_off, row_beg, nrows, f + NT);
                                An = rec_a[REC_STRIDE * (size_t) jn];
                                Bn = rec_b[REC_STRIDE * (size_t) jn];
                            }
                            if (f < total) {
                                const float phi[3] = {A.x, A.y, A.z};
                                const int cf[3] = {B.x, B.y, B.z};
                                const uint32_t meta = (uint32_t) B.w;
                                const float r = A.w;
                                const float eps = bump ? g.sigma * r : 3.0f * (g.sigma * r);
                                int blo[3], bw[3];
                                bool empty = false;
#pragma unroll
                                for (int a = 0; a < 3; ++a) {
                                    const int cr = cf[a] - u0[a];
                                    const float pos = static_cast<float>(cr) + phi[a];
                                    const float eh = eps * g.ihh[a];
                                    // nodes k with |k - pos| < eps / h; a node the rounding drops lies at
                                    // the edge of the support, where the kernel is zero
                                    int lo_a = static_cast<int>(floorf(pos - eh)) + 1;
                                    int hi_a = static_cast<int>(ceilf(pos + eh)) - 1;
                                    if (bump) {
                                        const int fa = (int) ((meta >> (8 * a)) & 0xFFu);
                                        const int ctr = cr + (int) ((meta >> (24 + a)) & 1u);
                                        lo_a = max(lo_a, ctr - fa);
                                        hi_a = min(hi_a, ctr + fa);
                                    }
                                    lo_a = max(lo_a, 0);
                                    hi_a = min(hi_a, T3[a] - 1);
                                    empty = empty || lo_a > hi_a;
                                    blo[a] = lo_a;
                                    bw[a] = hi_a - lo_a + 1;
                                    // node offset from the particle, in cells: (k - cr) - phi = (k - lo) + d0
                                    wp.d0[a] = static_cast<float>(lo_a - cr) - phi[a];
                                }
                                if (!empty) {
                                    nb = (uint32_t) (bw[1] * bw[2]);  // x-rows of the box
                                    if (bump) {
                                        wp.eps2 = eps * eps;
                                        wp.inv = __frcp_rn(wp.eps2);
                                    } else {
                                        const float sg = g.sigma * r;
                                        wp.eps2 = 9.0f * sg * sg;
                                        wp.inv = __frcp_rn(2.0f * sg * sg);
                                    }
                                    wp.bx = bw[0];
                                    wp.by = bw[1];
                                    wp.node0 = (blo[2] * TY + blo[1]) * TX + blo[0];
                                    wp.iby = 1.0f / (float) bw[1];
                                    if (WEIGHTED)
                                        wp.w = wts ? __ldg(wts + (size_t) j * wstride) : 1.0f;
                                }
                            }
                            // exclusive prefix of the row counts over the warp
                            uint32_t incl = nb;
#pragma unroll
                            for (int o = 1; o < 32; o <<= 1) {
                                const uint32_t u = __shfl_up_sync(0xffffffffu, incl, o);
                                if (lane >= (uint32_t) o)
                                    incl += u;
                            }
                            const uint32_t wtotal = __shfl_sync(0xffffffffu, incl, 31);
                            if (wtotal == 0)
                                continue;
                            const int wl = warp * 32 + lane;
                            s_part[0][wl] = __float_as_uint(wp.d0[0]);
                            s_part[1][wl] = __float_as_uint(wp.d0[1]);
                            s_part[2][wl] = __float_as_uint(wp.d0[2]);
                            s_part[3][wl] = __float_as_uint(wp.eps2);
                            s_part[4][wl] = __float_as_uint(wp.inv);
                            s_part[5][wl] = __float_as_uint(wp.iby);
                            s_part[6][wl] = (uint32_t) wp.bx;
                            s_part[7][wl] = (uint32_t) wp.by;
                            s_part[8][wl] = (uint32_t) wp.node0;
                            if (WEIGHTED)
                                s_part[9][wl] = __float_as_uint(wp.w);
                            s_pre[wl] = incl - nb;
                            __syncwarp();
                            const uint32_t* pre = s_pre + warp * 32;
                            for (uint32_t j0 = 0; j0 < wtotal; j0 += 32) {
                                const uint32_t jj = j0 + lane;
                                if (jj < wtotal) {
                                    // owner: the last lane whose prefix is <= jj (its box is non-empty)
                                    int o = 0;
#pragma unroll
                                    for (int step = 16; step > 0; step >>= 1)
                                        if (pre[o + step] <= jj)
                                            o += step;
                                    const int ow = warp * 32 + o;
                                    const int local = (int) (jj - pre[o]);
                                    const int by = (int) s_part[7][ow];
                                    const int zl = (int) ((static_cast<float>(local) + 0.5f) * __uint_as_float(s_part[5][ow]));
                                    const int yl = local - zl * by;
                                    const float dy = g.hhi[1] * (static_cast<float>(yl) + __uint_as_float(s_part[1][ow]));
                                    const float dz = g.hhi[2] * (static_cast<float>(zl) + __uint_as_float(s_part[2][ow]));
                                    const float dyz = __fmaf_rn(dy, dy, dz * dz);
                                    const float eps2 = __uint_as_float(s_part[3][ow]);
                                    if (dyz < eps2) {
                                        const float inv = __uint_as_float(s_part[4][ow]);
                                        const float d0x = __uint_as_float(s_part[0][ow]);
                                        const int bx = (int) s_part[6][ow];
                                        const int row = (int) s_part[8][ow] + (zl * TY + yl) * TX;
                                        const float pw = WEIGHTED ? __uint_as_float(s_part[9][ow]) : 0.0f;
                                        for (int xl = 0; xl < bx; ++xl) {
                                            const float dx = g.hhi[0] * (static_cast<float>(xl) + d0x);
                                            const float d2 = __fmaf_rn(dx, dx, dyz);
                                            if (!(d2 < eps2))
                                                continue;
                                            // the hardware reciprocal (__fdividef, within 2 ulp) and exponential:
                                            // the kernel's relative error stays below 1e-6 where it exceeds 1e-7 of
                                            // its peak (at 1/w = 16, e^-16 = 1.1e-7 of the peak, the reciprocal's
                                            // 2.4e-7 relative error moves e^-1/w by 3.8e-6 of itself)
                                            float v;
                                            if (bump) {
                                                const float w = __fmaf_rn(-d2, inv, 1.0f);
                                                v = w > 0.0f ? __expf(-__fdividef(1.0f, w)) : 0.0f;
                                            } else {
                                                v = fmaxf(__expf(-d2 * inv) - E45, 0.0f);
                                            }
                                            if (ACC == ACC_FIXED_W) {
                                                const long long q = __float2ll_rn(__fmul_rn(__fmul_rn(v, pw), wscale));
                                                if (q != 0)
                                                    atomicAdd(acc64 + row + xl, (unsigned long long) q);
                                            } else if (ACC == ACC_DOUBLE) {
                                                const float c = __fmul_rn(v, pw);  // rbf * val, in float
                                                if (c != 0.0f)
                                                    atomicAdd(accd + row + xl, (double) c);
                                            } else {
                                                const uint32_t q = __float2uint_rn(v * FIX_SCALE);
                                                if (q != 0u) {
                                                    const uint32_t old = atomicAdd(acc_lo + row + xl, q);
                                                    if (old + q < old)
                                                        atomicAdd(acc_hi + row + xl, 1u);
                                                }
                                            }
                                        }
                                    }
                                }
                            }
                            __syncwarp();
                        }
                    }
                }
    }
    __syncthreads();

    // ---- write the tile (x fastest, coalesced) and its statistics ----
    // The density's tile sum is exact in integers: every output value is a multiple of 2^-32, and the
    // integer and fractional parts of the rounded sums are added separately (each below 2^44 for a tile), so
    // no node pays an FP64 conversion and add (the FP64 pipe of this part is 1/64 of the FP32 rate).
    double dsum = 0.0;
    unsigned long long isum = 0ull, fsum = 0ull;
    float vmin = INFINITY, vmax = -INFINITY;
    for (int n = t; n < NN; n += NT) {
        const int x = n % TX, y = (n / TX) % TY, z = n / (TX * TY);
        if (x0 + x < g.s[0] && y0 + y < g.s[1] && z0 + z >= g.zlo && z0 + z < g.zhi) {
            float v;
            if (ACC == ACC_EXACT) {
                unsigned long long q;
                v = fixed_to_float(acc_hi[n], acc_lo[n], q);
                isum += q >> 32;
                fsum += q & 0xFFFFFFFFull;
            } else {
                v = ACC == ACC_FIXED_W ? __ll2float_rn((long long) acc64[n]) * winv : __double2float_rn(accd[n]);
                dsum += (double) v;
            }
            grid[(((size_t) (z0 + z - g.zlo) * g.s[1] + (y0 + y)) * g.s[0] + (x0 + x)) * (size_t) ostride] = v;
            vmin = fminf(vmin, v);
            vmax = fmaxf(vmax, v);
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        if (ACC == ACC_EXACT) {
            isum += __shfl_xor_sync(0xffffffffu, isum, o);
            fsum += __shfl_xor_sync(0xffffffffu, fsum, o);
        } else {
            dsum += __shfl_xor_sync(0xffffffffu, dsum, o);
        }
        vmin = fminf(vmin, __shfl_xor_sync(0xffffffffu, vmin, o));
        vmax = fmaxf(vmax, __shfl_xor_sync(0xffffffffu, vmax, o));
    }
    if ((t & 31) == 0) {
        s_dsum[t >> 5] = dsum;
        s_isum[t >> 5] = isum;
        s_fsum[t >> 5] = fsum;
        s_fmin[t >> 5] = vmin;
        s_fmax[t >> 5] = vmax;
    }
    __syncthreads();
    if (t == 0) {
        for (int w = 1; w < NT / 32; ++w) {
            dsum += s_dsum[w];
            isum += s_isum[w];
            fsum += s_fsum[w];
            vmin = fminf(vmin, s_fmin[w]);
            vmax = fmaxf(vmax, s_fmax[w]);
        }
        if (ACC == ACC_EXACT)
            dsum = (double) isum + (double) fsum * 2.3283064365386963e-10;
        TileStats ts;
        ts.sum = dsum;
        ts.vmin = vmin;
        ts.vmax = vmax;
        tiles[(blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x] = ts;
    }
}

// Fixed-order reduction of the tile statistics (one block) and the normalisation constants.
__global__ void __launch_bounds__(1024) finalize_kernel(const TileStats* __restrict__ tiles, uint32_t ntiles,
    FrameScalars* __restrict__ fs, int mass_normalize, int minmax_normalize, double voxel_volume) {
    __shared__ double s_sum[32];
    __shared__ float s_min[32], s_max[32];
    double sum = 0.0;
    float mn = INFINITY, mx = -INFINITY;
    for (uint32_t i = threadIdx.x; i < ntiles; i += blockDim.x) {
        const TileStats ts = tiles[i];
        sum += ts.sum;
        mn = fminf(mn, ts.vmin);
        mx = fmaxf(mx, ts.vmax);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        sum += __shfl_xor_sync(0xffffffffu, sum, o);
        mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    }
    if ((threadIdx.x & 31) == 0) {
        s_sum[threadIdx.x >> 5] = sum;
        s_min[threadIdx.x >> 5] = mn;
        s_max[threadIdx.x >> 5] = mx;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const int nw = blockDim.x >> 5;
        for (int w = 1; w < nw; ++w) {
            sum += s_sum[w];
            mn = fminf(mn, s_min[w]);
            mx = fmaxf(mx, s_max[w]);
        }
        fs->mass = sum;
        fs->vmin = mn;
        fs->vmax = mx;
        double ms = 1.0;
        if (mass_normalize && sum > 0.0)
            ms = (double) fs->n_valid / (sum * voxel_volume);
        fs->mass_scale = ms;
        float lo = mn, hi = mx;
        if (mass_normalize) {
            lo = (float) (mn * ms);
            hi = (float) (mx * ms);
        }
        if (minmax_normalize) {
            // ParticlesToDensity.cpp:676-682: rcp = 1 / (max - min); v = (v - min) * rcp
            fs->offset = lo;
            fs->scale = 1.0f / (hi - lo);
            fs->out_min = 0.0f;
            fs->out_max = 1.0f;
        } else {
            fs->offset = 0.0f;
            fs->scale = 1.0f;
            fs->out_min = lo;
            fs->out_max = hi;
        }
    }
}

__device__ __forceinline__ float normalize_one(float v, float ms, float off, float sc, int mass_normalize,
                                               int minmax_normalize) {
    if (mass_normalize)
        v = v * ms;
    if (minmax_normalize)
        v = (v - off) * sc;
    return v;
}

__global__ void __launch_bounds__(256) normalize_scalar_kernel(float* __restrict__ grid, uint64_t n,
    const FrameScalars* __restrict__ fs, int mass_normalize, int minmax_normalize) {
    const float ms = (float) fs->mass_scale;
    const float off = fs->offset, sc = fs->scale;
    for (uint64_t i = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; i < n; i += (uint64_t) gridDim.x * blockDim.x)
        grid[i] = normalize_one(grid[i], ms, off, sc, mass_normalize, minmax_normalize);
}

// Streams the grid in 16-byte vectors, four per thread per round (many loads in flight); the tail past
// the last whole vector is done element-wise.
__global__ void __launch_bounds__(256) normalize_kernel(float* __restrict__ grid, uint64_t n,
    const FrameScalars* __restrict__ fs, int mass_normalize, int minmax_normalize) {
    const float ms = (float) fs->mass_scale;
    const float off = fs->offset, sc = fs->scale;
    float4* g4 = reinterpret_cast<float4*>(grid);
    const uint64_t n4 = n / 4;
    const uint64_t stride = (uint64_t) gridDim.x * blockDim.x;
    uint64_t i = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x;
    for (; i + 3 * stride < n4; i += 4 * stride) {
        float4 v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u)
            v[u] = g4[i + u * stride];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            v[u].x = normalize_one(v[u].x, ms, off, sc, mass_normalize, minmax_normalize);
            v[u].y = normalize_one(v[u].y, ms, off, sc, mass_normalize, minmax_normalize);
            v[u].z = normalize_one(v[u].z, ms, off, sc, mass_normalize, minmax_normalize);
            v[u].w = normalize_one(v[u].w, ms, off, sc, mass_normalize, minmax_normalize);
            g4[i + u * stride] = v[u];
        }
    }
    for (; i < n4; i += stride) {
        float4 v = g4[i];
        v.x = normalize_one(v.x, ms, off, sc, mass_normalize, minmax_normalize);
        v.y = normalize_one(v.y, ms, off, sc, mass_normalize, minmax_normalize);
        v.z = normalize_one(v.z, ms, off, sc, mass_normalize, minmax_normalize);
        v.w = normalize_one(v.w, ms, off, sc, mass_normalize, minmax_normalize);
        g4[i] = v;
    }
    const uint64_t t = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x;
    if (t < n - 4 * n4)
        grid[4 * n4 + t] = normalize_one(grid[4 * n4 + t], ms, off, sc, mass_normalize, minmax_normalize);
}

}  // namespace

size_t gather_smem_bytes(const GatherConfig& c) {
    if (c.mode == GATHER_EXACT)
        return (size_t) c.tx * c.ty * c.tz * sizeof(unsigned long long) + (size_t) (2 * c.rmax + 1) * sizeof(uint32_t);
    return (size_t) 2 * c.tx * c.ty * c.tz * sizeof(float) + (size_t) c.smax * (sizeof(float4) + sizeof(uint4)) +
           (size_t) (2 * c.rmax + 1) * sizeof(uint32_t);
}

// z tiles of the slab [zlo, zhi): from the tile holding plane zlo to the one holding plane zhi - 1
uint32_t gather_tiles_z(const GatherConfig& c, const GridGeo& g) {
    return ceil_div((uint32_t) g.zhi, (uint32_t) c.tz) - (uint32_t) (g.zlo / c.tz);
}

uint32_t gather_tile_count(const GatherConfig& c, const GridGeo& g) {
    return ceil_div(g.s[0], c.tx) * ceil_div(g.s[1], c.ty) * gather_tiles_z(c, g);
}

namespace {
template<class K>
cudaError_t launch_tiles(K kern, const GatherConfig& c, const GridGeo& g, int nt, size_t smem, cudaStream_t st,
    const float4* rec_a, const int4* rec_b, const uint32_t* start, float* grid, TileStats* tiles, FrameScalars* fs,
    const GatherWeights& w) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem);
    if (e != cudaSuccess)
        return e;
    dim3 grd(ceil_div(g.s[0], c.tx), ceil_div(g.s[1], c.ty), gather_tiles_z(c, g));
    kern<<<grd, nt, smem, st>>>(g, rec_a, rec_b, start, grid, tiles, fs, c.rmax, w.w, w.wstride,
                                w.ostride > 0 ? w.ostride : 1);
    return cudaGetLastError();
}

template<int W>
cudaError_t launch_exact(const GatherConfig& c, const GridGeo& g, size_t smem, cudaStream_t st, const float4* rec_a,
    const int4* rec_b, const uint32_t* start, float* grid, TileStats* tiles, FrameScalars* fs,
    const GatherWeights& w) {
    if (c.tx == 16 && c.ty == 16 && c.tz == 16)
        return launch_tiles(gather_fixed_kernel<16, 16, 16, 256, W>, c, g, 256, smem, st, rec_a, rec_b, start, grid,
                            tiles, fs, w);
    if (c.tx == 16 && c.ty == 8 && c.tz == 8)
        return launch_tiles(gather_fixed_kernel<16, 8, 8, 256, W>, c, g, 256, smem, st, rec_a, rec_b, start, grid,
                            tiles, fs, w);
    if (c.tx == 32 && c.ty == 16 && c.tz == 8)
        return launch_tiles(gather_fixed_kernel<32, 16, 8, 512, W>, c, g, 512, smem, st, rec_a, rec_b, start, grid,
                            tiles, fs, w);
    return cudaErrorInvalidValue;
}
}  // namespace

cudaError_t launch_gather(const GatherConfig& c, const GridGeo& g, const float4* rec_a, const int4* rec_b,
    const uint32_t* start, float* grid, TileStats* tiles, FrameScalars* fs, cudaStream_t st, const GatherWeights& w) {
    const size_t smem = gather_smem_bytes(c);
    if (c.mode == GATHER_EXACT) {
        if (w.mode == GatherWeights::DOUBLE)
            return launch_exact<ACC_DOUBLE>(c, g, smem, st, rec_a, rec_b, start, grid, tiles, fs, w);
        if (w.mode == GatherWeights::FIXED)
            return launch_exact<ACC_FIXED_W>(c, g, smem, st, rec_a, rec_b, start, grid, tiles, fs, w);
        return launch_exact<ACC_EXACT>(c, g, smem, st, rec_a, rec_b, start, grid, tiles, fs, w);
    }
    if (w.mode != GatherWeights::DENSITY)
        return cudaErrorInvalidValue;  // the weighted aggregators use the particle-major gather
    if (c.tx != GATHER_TX || c.ty != GATHER_TY || c.tz != GATHER_TZ)
        return cudaErrorInvalidValue;
    auto kern = gather_kernel<GATHER_TX, GATHER_TY, GATHER_TZ>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem);
    if (e != cudaSuccess)
        return e;
    dim3 grd(ceil_div(g.s[0], c.tx), ceil_div(g.s[1], c.ty), gather_tiles_z(c, g));
    kern<<<grd, c.ty * c.tz, smem, st>>>(g, rec_a, rec_b, start, grid, tiles, fs, c.smax, c.rmax);
    return cudaGetLastError();
}

cudaError_t launch_finalize(const TileStats* tiles, uint32_t ntiles, FrameScalars* fs, int mass_normalize,
    int minmax_normalize, double, double voxel_volume, cudaStream_t st) {
    finalize_kernel<<<1, 1024, 0, st>>>(tiles, ntiles, fs, mass_normalize, minmax_normalize, voxel_volume);
    return cudaGetLastError();
}

cudaError_t launch_normalize_modes(float* grid, uint64_t nvox, const FrameScalars* fs, int mass_normalize,
    int minmax_normalize, int sms, cudaStream_t st) {
    if (!mass_normalize && !minmax_normalize)
        return cudaSuccess;
    // the grid starts 16-byte aligned (cudaMalloc, or a caller's device buffer checked below)
    if (reinterpret_cast<uintptr_t>(grid) % 16 != 0) {
        const unsigned g1 = (unsigned) std::max<uint64_t>(1, std::min<uint64_t>((nvox + 255) / 256, (uint64_t) sms * 16));
        normalize_scalar_kernel<<<g1, 256, 0, st>>>(grid, nvox, fs, mass_normalize, minmax_normalize);
        return cudaGetLastError();
    }
    const unsigned grd = (unsigned) std::max<uint64_t>(1, std::min<uint64_t>((nvox / 4 + 255) / 256, (uint64_t) sms * 8));
    normalize_kernel<<<grd, 256, 0, st>>>(grid, nvox, fs, mass_normalize, minmax_normalize);
    return cudaGetLastError();
}

}  // namespace p2v
