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

namespace p2v {

namespace {

constexpr int GATHER_TX = 8;
constexpr int GATHER_TY = 16;
constexpr int GATHER_TZ = 16;
constexpr int MAX_IMAGES = 8;  // cyclic images per axis a tile may visit

__device__ __forceinline__ int64_t floor_div(int64_t a, int64_t b) {
    int64_t q = a / b;
    return (a % b != 0 && ((a < 0) != (b < 0))) ? q - 1 : q;
}

__device__ __forceinline__ int64_t ceil_div_i(int64_t a, int64_t b) {
    return -floor_div(-a, b);
}

// Fractional position of coordinate p relative to cell cf, in units of the exact spacing
// (hhi + hlo): ((p - min) / h) - cf, accurate to ~1e-7 absolute without FP64.
__device__ __forceinline__ float frac_in_cell(float p, float minf, float hhi, float hlo, int cf) {
    // two-sum: p - minf = ah + al exactly
    const float ah = p - minf;
    const float bb = ah - p;
    const float al = (p - (ah - bb)) + (-minf - bb);
    const float q0 = ah / hhi;
    float rem = __fmaf_rn(-q0, hhi, ah);  // exact remainder of the rounded quotient
    rem = rem + al - q0 * hlo;
    return (q0 - static_cast<float>(cf)) + rem / hhi;
}

struct Extent {
    int L[3], H[3];  // rows [u - L, u + H] of cell bins can hold candidates of node u
    int F[3];        // largest footprint half-width (bump)
};

template<int TX, int TY, int TZ>
__global__ void __launch_bounds__(TY* TZ, 2) gather_kernel(GridGeo g, const float4* __restrict__ xyzr,
    const uint32_t* __restrict__ start, float* __restrict__ grid, TileStats* __restrict__ tiles,
    FrameScalars* __restrict__ fs, int smax, int rmax) {
    constexpr int NT = TY * TZ;
    extern __shared__ __align__(16) unsigned char smem[];
    float* acc_s = reinterpret_cast<float*>(smem);                      // [TX][NT]
    float* acc_c = acc_s + TX * NT;                                      // [TX][NT]
    float4* sp = reinterpret_cast<float4*>(acc_c + TX * NT);             // [smax] phi xyz, eps^2
    uint4* sm = reinterpret_cast<uint4*>(sp + smax);                     // [smax] boxes, cells, inv
    uint32_t* row_beg = reinterpret_cast<uint32_t*>(sm + smax);          // [rmax]
    uint32_t* row_off = row_beg + rmax;                                  // [rmax + 1]
    __shared__ double s_dsum[NT / 32];
    __shared__ float s_fmin[NT / 32], s_fmax[NT / 32];

    const int t = threadIdx.x;
    const int ty = t % TY;
    const int tz = t / TY;
    const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY, z0 = blockIdx.z * TZ;
    const bool row_in = (y0 + ty < g.s[1]) && (z0 + tz < g.s[2]);

#pragma unroll
    for (int k = 0; k < TX; ++k) {
        acc_s[k * NT + t] = 0.0f;
        acc_c[k * NT + t] = 0.0f;
    }

    const float rmax_r = __uint_as_float(fs->rmax_bits);
    const bool bump = g.kernel == 0;
    const float E45 = expf(-4.5f);
    if (rmax_r > 0.0f) {
        // ---- candidate extents from the largest radius ----
        Extent ex;
        const float eps_max = bump ? g.sigma * rmax_r : 3.0f * (g.sigma * rmax_r);
        int64_t klo[3], khi[3];
        const int T3[3] = {TX, TY, TZ};
        const int o3[3] = {x0, y0, z0};
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            int E = static_cast<int>(ceilf(eps_max / g.hhi[a] + 1e-3f));
            E = E < 1 ? 1 : E;
            int F = bump ? static_cast<int>(fminf(ceilf(rmax_r / g.hf[a]), 268435456.0f)) : E;
            ex.F[a] = F;
            ex.L[a] = bump ? min(E, F + 1) : E;
            ex.H[a] = bump ? min(E - 1, F) : E - 1;
            if (ex.L[a] > 100) {  // staged cell offsets are kept in 8 bits
                if (t == 0)
                    atomicOr(&fs->error, ERR_WINDOW_TOO_WIDE);
                ex.L[a] = 100;
                ex.H[a] = min(ex.H[a], 100);
            }
            if (g.cyc[a]) {
                const int64_t s = g.s[a];
                klo[a] = ceil_div_i((int64_t) fs->cmin[a] - o3[a] - T3[a] + 1 - ex.H[a], s);
                khi[a] = floor_div((int64_t) fs->cmax[a] - o3[a] + ex.L[a], s);
                if (khi[a] - klo[a] + 1 > MAX_IMAGES) {
                    if (t == 0)
                        atomicOr(&fs->error, ERR_WINDOW_TOO_WIDE);
                    khi[a] = klo[a] + MAX_IMAGES - 1;
                }
            } else {
                klo[a] = 0;
                khi[a] = 0;
            }
        }

        for (int64_t kz = klo[2]; kz <= khi[2]; ++kz)
            for (int64_t ky = klo[1]; ky <= khi[1]; ++ky)
                for (int64_t kx = klo[0]; kx <= khi[0]; ++kx) {
                    const int u0[3] = {x0 + (int) (kx * g.s[0]), y0 + (int) (ky * g.s[1]), z0 + (int) (kz * g.s[2])};
                    int wlo[3], whi[3];
#pragma unroll
                    for (int a = 0; a < 3; ++a) {
                        wlo[a] = max(u0[a] - ex.L[a], -1);
                        wlo[a] = min(wlo[a], g.s[a]);
                        whi[a] = min(u0[a] + T3[a] - 1 + ex.H[a], g.s[a]);
                        whi[a] = max(whi[a], -1);
                    }
                    const int nwy = whi[1] - wlo[1] + 1;
                    const int nwz = whi[2] - wlo[2] + 1;
                    if (nwy > rmax) {
                        if (t == 0)
                            atomicOr(&fs->error, ERR_STAGE_OVERFLOW);
                        continue;
                    }
                    const int planes_per_chunk = rmax / nwy;
                    // this thread's node (unwrapped) and its relevant rows
                    const int uy = u0[1] + ty, uz = u0[2] + tz;
                    const int ry_lo = max(uy - ex.L[1], wlo[1]), ry_hi = min(uy + ex.H[1], whi[1]);
                    const int rz_lo = max(uz - ex.L[2], wlo[2]), rz_hi = min(uz + ex.H[2], whi[2]);
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
                        // exclusive scan of the row counts (single warp, rows are few)
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
                            // ---- stage: coalesced float4 loads of the chunk's particles ----
                            for (uint32_t si = t; si < cn; si += NT) {
                                const uint32_t f = cb + si;
                                int lo = 0, hi = nrows;  // find row r with row_off[r] <= f < row_off[r+1]
                                while (hi - lo > 1) {
                                    const int mid = (lo + hi) >> 1;
                                    if (row_off[mid] <= f)
                                        lo = mid;
                                    else
                                        hi = mid;
                                }
                                const uint32_t j = row_beg[lo] + (f - row_off[lo]);
                                const float4 p = xyzr[j];
                                const float pc[3] = {p.x, p.y, p.z};
                                const float r = p.w;
                                const float eps = bump ? g.sigma * r : 3.0f * (g.sigma * r);
                                float phi[3];
                                int blo[3], bhi[3], crel[3];
                                bool empty = false;
#pragma unroll
                                for (int a = 0; a < 3; ++a) {
                                    const float q = (pc[a] - g.minf[a]) / g.hf[a];
                                    const int ct = static_cast<int>(q);          // reference cell
                                    const int cf = static_cast<int>(floorf(q));  // bin cell
                                    phi[a] = frac_in_cell(pc[a], g.minf[a], g.hhi[a], g.hlo[a], cf);
                                    const int64_t cr = (int64_t) cf - u0[a];
                                    const float pos = static_cast<float>(cr) + phi[a];
                                    const float eh = eps / g.hhi[a];
                                    int64_t lo_a = (int64_t) floorf(pos - eh);
                                    int64_t hi_a = (int64_t) ceilf(pos + eh);
                                    if (bump) {
                                        const int64_t f = (int64_t) fminf(ceilf(r / g.hf[a]), 268435456.0f);
                                        const int64_t ctr = (int64_t) ct - u0[a];
                                        lo_a = max(lo_a, ctr - f);
                                        hi_a = min(hi_a, ctr + f);
                                    }
                                    lo_a = max(lo_a, (int64_t) 0);
                                    hi_a = min(hi_a, (int64_t) T3[a] - 1);
                                    if (lo_a > hi_a)
                                        empty = true;
                                    blo[a] = (int) lo_a;
                                    bhi[a] = (int) hi_a;
                                    crel[a] = (int) max(min(cr, (int64_t) 120), (int64_t) -120);
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
                                    inv = 1.0f / eps2;
                                } else {
                                    const float sg = g.sigma * r;
                                    eps2 = 9.0f * sg * sg;
                                    inv = 1.0f / (2.0f * sg * sg);
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
                                    for (int yy = ry_lo; yy <= ry_hi; ++yy) {
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
                                                float v;
                                                if (bump) {
                                                    const float w = __fmaf_rn(-d2, inv, 1.0f);
                                                    v = w > 0.0f ? expf(-1.0f / w) : 0.0f;
                                                } else {
                                                    v = fmaxf(expf(-d2 * inv) - E45, 0.0f);
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
        float* out = grid + ((size_t) (z0 + tz) * g.s[1] + (y0 + ty)) * g.s[0] + x0;
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
        // warp 0's values are already in dsum/vmin/vmax of lane 0
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

__global__ void __launch_bounds__(256) normalize_kernel(float* __restrict__ grid, uint64_t n,
    const FrameScalars* __restrict__ fs, int mass_normalize, int minmax_normalize) {
    const float ms = (float) fs->mass_scale;
    const float off = fs->offset, sc = fs->scale;
    for (uint64_t i = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; i < n; i += (uint64_t) gridDim.x * blockDim.x) {
        float v = grid[i];
        if (mass_normalize)
            v = v * ms;
        if (minmax_normalize)
            v = (v - off) * sc;
        grid[i] = v;
    }
}

}  // namespace

size_t gather_smem_bytes(const GatherConfig& c) {
    return (size_t) 2 * c.tx * c.ty * c.tz * sizeof(float) + (size_t) c.smax * (sizeof(float4) + sizeof(uint4)) +
           (size_t) (2 * c.rmax + 1) * sizeof(uint32_t);
}

uint32_t gather_tile_count(const GatherConfig& c, const GridGeo& g) {
    return ceil_div(g.s[0], c.tx) * ceil_div(g.s[1], c.ty) * ceil_div(g.s[2], c.tz);
}

cudaError_t launch_gather(const GatherConfig& c, const GridGeo& g, const float4* xyzr_sorted, const uint32_t* start,
    float* grid, TileStats* tiles, FrameScalars* fs, cudaStream_t st) {
    if (c.tx != GATHER_TX || c.ty != GATHER_TY || c.tz != GATHER_TZ)
        return cudaErrorInvalidValue;
    const size_t smem = gather_smem_bytes(c);
    auto kern = gather_kernel<GATHER_TX, GATHER_TY, GATHER_TZ>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem);
    if (e != cudaSuccess)
        return e;
    dim3 grd(ceil_div(g.s[0], c.tx), ceil_div(g.s[1], c.ty), ceil_div(g.s[2], c.tz));
    kern<<<grd, c.ty * c.tz, smem, st>>>(g, xyzr_sorted, start, grid, tiles, fs, c.smax, c.rmax);
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
    const unsigned grd = (unsigned) std::max<uint64_t>(1, std::min<uint64_t>((nvox + 255) / 256, (uint64_t) sms * 16));
    normalize_kernel<<<grd, 256, 0, st>>>(grid, nvox, fs, mass_normalize, minmax_normalize);
    return cudaGetLastError();
}

}  // namespace p2v
