// Per-particle ambient occlusion: the MDAO mip pyramid and cone march, and the AOSphereRenderer volume.
//
// Reference shaders (all GLSL, restated here as CUDA; the GL sampler semantics are written out by hand):
//   mip build   plugins/moldyn_gl/shaders/moldyn_gl/mdao_volume_generator/mdao_mipmap_compute_main.comp.glsl:8-26
//   cone march  plugins/moldyn_gl/shaders/moldyn_gl/sphere_renderer/inc/mdao_deferred_fragment_ambocc.inc.glsl:9-60
//   AOSphere    plugins/pwdemos_gl/src/AOSphereRenderer.cpp:918-1021 (deposit), :489-514 (uniforms),
//               shaders/pwdemos_gl/AOSphere/snippets/mainaxes_vertex_2.glsl:1-9, mainaxes_fragLightAO_evalAO.glsl:1-8,
//               normals_fragLightAO_evalAO.glsl:1-4
// AO is evaluated once per particle at its surface point p + r * n along the particle's normal n.
// Particles are processed in cell-sorted order so neighbouring threads sample neighbouring texels.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "ao_internal.h"
#include "cone_march.cuh"
#include "p2v_common.cuh"
#include "particle_record.cuh"

namespace p2v {

namespace {

// ---------------------------------------------------------------------------------------------
// mip pyramid: level l+1 voxel = sum of the children 2g .. min(2g+1, N-1), divided by 8 always
// ---------------------------------------------------------------------------------------------
// One thread per voxel of the coarser level in 32-bit index arithmetic (an AO volume holds fewer than 2^31
// texels, so every level above level 0 fewer than 2^28).
// pairs: the finer level's rows have an even length and start 8-byte aligned, so the two children of a voxel
// along x load as one float2 (the same values added in the same order as mip_voxel's loop: the same bits).
__global__ void __launch_bounds__(256) mip_level_kernel(const float* __restrict__ src, int sx, int sy, int sz,
    float* __restrict__ dst, int dx, int dy, int dz, float sat_scale, int quantize, int pairs) {
    const uint32_t n = (uint32_t) dx * (uint32_t) dy * (uint32_t) dz;
    const uint32_t pxy = (uint32_t) dx * (uint32_t) dy;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t z = i / pxy, r = i - z * pxy;
        const uint32_t y = r / (uint32_t) dx, x = r - y * (uint32_t) dx;
        if (pairs && !quantize) {
            const int y1 = min(2 * (int) y + 1, sy - 1), z1 = min(2 * (int) z + 1, sz - 1);
            float acc = 0.0f;
            for (int zz = 2 * (int) z; zz <= z1; ++zz)
                for (int yy = 2 * (int) y; yy <= y1; ++yy) {
                    float2 v = __ldg(reinterpret_cast<const float2*>(src + ((int64_t) zz * sy + yy) * sx + 2 * x));
                    if (sat_scale > 0.0f) {
                        v.x = fminf(fmaxf(__fmul_rn(v.x, sat_scale), 0.0f), 1.0f);
                        v.y = fminf(fmaxf(__fmul_rn(v.y, sat_scale), 0.0f), 1.0f);
                    }
                    acc = __fadd_rn(__fadd_rn(acc, v.x), v.y);
                }
            dst[i] = __fmul_rn(acc, 0.125f);
        } else {
            dst[i] = mip_voxel<true>(src, sx, sy, sz, (int) x, (int) y, (int) z, sat_scale, quantize);
        }
    }
}

// One thread per particle: marches all cones (throughput: millions of particles). Particle i's data are
// read at order[i] (or i) and its AO is written at out_order[i] (or there): the frame's kernels read sorted
// copies and scatter the AO straight to input order.
__global__ void __launch_bounds__(128) cone_ao_kernel(const ConeParams cp, const uint32_t* __restrict__ order,
    const float4* __restrict__ xyzr, const float4* __restrict__ nrm, uint32_t n, const uint32_t* __restrict__ out_order,
    float* __restrict__ ao) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const uint32_t o = order ? order[i] : i;
    const uint32_t w = out_order ? out_order[i] : o;
    ao[w] = cone_ao_at<true>(cp, xyzr[o], nrm[o]);
}

// One warp per cone: a block takes one particle with one warp per cone, and the lanes of a warp take the
// cone's samples (32 at a time: the step positions are tabulated, so all samples load at once). Every lane
// then runs the march's recurrence over the shuffled samples in step order with the same early exit, the
// block's first thread adds the cones in cone order: the result has the bits of cone_ao_kernel. A bounded
// grid strides over the particles: the learned AO's fallback list (list and its device-side length n_dev,
// usually tiny, where latency matters), or a whole frame (no list: particle i; P2V_AO_MARCH_WARP), where
// every lane stays busy whatever step its cone ends at, at the price of the samples past the early exit.
__global__ void __launch_bounds__(32 * MAX_CONES) cone_ao_list_kernel(const ConeParams cp,
    const uint32_t* __restrict__ list, const float4* __restrict__ xyzr, const float4* __restrict__ nrm, uint32_t n,
    const uint32_t* __restrict__ n_dev, const uint32_t* __restrict__ out_order, float* __restrict__ ao) {
    __shared__ float s_acc[MAX_CONES];
    const int lane = threadIdx.x & 31, c = threadIdx.x >> 5;
    if (n_dev)
        n = min(n, *n_dev);
    for (uint32_t i = blockIdx.x; i < n; i += gridDim.x) {
        const uint32_t o = list ? list[i] : i;
        const float4 p = xyzr[o];
        const float4 nv = nrm[o];
        float x[3], nn[3];
        const uint32_t w = out_order ? out_order[o] : o;
        if (!surface_point(p, nv, x, nn)) {  // the whole block takes this branch
            if (threadIdx.x == 0)
                ao[w] = 1.0f;
            continue;
        }
        float u[3], ex[3], ez[3], dir[3];
        cone_frame(cp, x, nn, u, ex, ez);
        cone_dir(cp, c, ex, nn, ez, dir);
        float acc = 0.0f;
        bool done = false;
        for (int k0 = 0; k0 < cp.nsteps && !done; k0 += 32) {
            const float vis = k0 + lane < cp.nsteps ? cone_sample<true>(cp, dir, u, k0 + lane) : 0.0f;
            const int m = min(32, cp.nsteps - k0);
            for (int s = 0; s < m; ++s) {
                acc = __fmaf_rn(__fsub_rn(1.0f, acc), __shfl_sync(0xffffffffu, vis, s), acc);
                if (cp.early_exit && acc > 0.99f) {
                    done = true;
                    break;
                }
            }
        }
        if (lane == 0)
            s_acc[c] = acc;
        __syncthreads();
        if (threadIdx.x == 0) {
            float ambient = 0.0f;
            for (int k = 0; k < cp.ncones; ++k)
                ambient = __fadd_rn(ambient, s_acc[k]);
            ao[w] = cone_combine(cp, ambient);
        }
        __syncthreads();
    }
}

// Positions and normals in sorted (cell) order: the AO kernels then read them coalesced whatever the input
// order was (a streaming kernel keeps many of these scattered reads in flight; inside the latency-bound AO
// kernels they stalled every tile). The AO kernels store each result straight at its input-order index.
__global__ void __launch_bounds__(256) sort_particles_kernel(const uint32_t* __restrict__ order, uint32_t n,
    const float4* __restrict__ xyzr, const float4* __restrict__ nrm, float4* __restrict__ xyzr_s,
    float4* __restrict__ nrm_s) {
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        const uint32_t o = order[j];
        if (xyzr)  // null: the binning's last pass wrote the sorted positions already
            xyzr_s[j] = xyzr[o];
        nrm_s[j] = nrm[o];
    }
}

// Unit normals down the density gradient (P2V_NORMALS_GRADIENT), one thread per particle.
__global__ void __launch_bounds__(256) gradient_normals_kernel(const GridGeo geo, const float* __restrict__ grid,
    const float4* __restrict__ xyzr, uint32_t n, float4* __restrict__ nrm) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n)
        return;
    nrm[j] = gradient_normal<true>(geo, grid, xyzr[j]);
}

// ---------------------------------------------------------------------------------------------
// AOSphere volume: nearest inner voxel, (4/3 pi r^3 / voxel volume) * genFac, summed exactly in
// 64-bit fixed point (2^-32) so the result does not depend on the particle order.
// ---------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(256) aosphere_deposit_kernel(const AOSphereParams ap, const float4* __restrict__ xyzr,
    uint32_t n, unsigned long long* __restrict__ acc) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const float4 p = xyzr[i];
    if (!(isfinite(p.x) && isfinite(p.y) && isfinite(p.z) && isfinite(p.w) && p.w > 0.0f))
        return;
    const float pc[3] = {p.x, p.y, p.z};
    int c[3];
    if (!ap.glsl_rule) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            // AOSphereRenderer.cpp:964-980: int(((p - min) / range) * s_inner), clamped to [0, s_inner - 1]
            const float q = __fmul_rn(__fdiv_rn(__fsub_rn(pc[a], ap.minOS[a]), ap.rangeOS[a]), (float) ap.si[a]);
            const int v = (int) fminf(fmaxf(q, -2147483520.0f), 2147483520.0f);
            c[a] = (v < 0 ? 0 : (v >= ap.si[a] ? ap.si[a] - 1 : v)) + 1;  // inside the one-voxel border
        }
        if (ap.clip) {
            // :982-991: the particle is dropped when dot(pos, n) - d >= 0 (vislib's Dot: a running sum)
            const float od = __fadd_rn(__fadd_rn(__fmul_rn(pc[0], ap.clip_plane[0]), __fmul_rn(pc[1], ap.clip_plane[1])),
                                       __fmul_rn(pc[2], ap.clip_plane[2]));
            if (__fsub_rn(od, ap.clip_plane[3]) >= 0.0f)
                return;
        }
    } else {
        // volume_updateVolume.vert.glsl:22: clamp(floor(((p - min) / range) * s_inner), 0, s_inner) in x and y, the
        // point's pixel (no border offset); z: the host's slice binning (AOSphereRenderer.cpp:1129-1131), layer + 1
#pragma unroll
        for (int a = 0; a < 2; ++a) {
            const float q = __fmul_rn(__fdiv_rn(__fsub_rn(pc[a], ap.minOS[a]), ap.rangeOS[a]), (float) ap.si[a]);
            const float fl = fminf(fmaxf(floorf(q), 0.0f), (float) ap.si[a]);
            c[a] = (int) fl;
        }
        const float qz = __fmul_rn(__fdiv_rn(__fsub_rn(pc[2], ap.minOS[2]), ap.rangeOS[2]), (float) ap.si[2]);
        const int vz = (int) fminf(fmaxf(qz, -2147483520.0f), 2147483520.0f);
        c[2] = max(0, min(vz, ap.si[2] - 1)) + 1;
    }
    // (4/3) pi r^3 (the CPU's float(M_PI) and the shader's 3.14159265 are the same float)
    const float spVol = 4.0f / 3.0f * 3.14159265358979f * p.w * p.w * p.w;
    const float val = (spVol / ap.voxel_vol) * ap.gen_fac;
    const int64_t idx = c[0] + ((int64_t) c[1] + (int64_t) c[2] * ap.s[1]) * ap.s[0];
    atomicAdd(acc + idx, (unsigned long long) __float2ull_rn(val * 4294967296.0f));
}

__global__ void __launch_bounds__(256) fixed_to_float_kernel(const unsigned long long* __restrict__ acc, int64_t n,
    float* __restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t) blockDim.x + threadIdx.x; i < n; i += (int64_t) gridDim.x * blockDim.x)
        out[i] = (float) ((double) acc[i] * 2.3283064365386963e-10);
}

__global__ void __launch_bounds__(128) aosphere_ao_kernel(const AOSphereParams ap, const float* __restrict__ tex,
    const uint32_t* __restrict__ order, const float4* __restrict__ xyzr, const float4* __restrict__ nrm, uint32_t n,
    int mode, float* __restrict__ ao) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const uint32_t o = order ? order[i] : i;
    const float4 p = xyzr[o];
    const float4 nv = nrm[o];
    float x[3], nn[3];
    if (!surface_point(p, nv, x, nn)) {
        ao[o] = 1.0f;
        return;
    }
    ConeLevel T;
    T.v = tex;
    for (int a = 0; a < 3; ++a) {
        T.d[a] = ap.s[a];
        T.fd[a] = (float) ap.s[a];
    }
    if (mode == 0) {
        // taps at p +- (r + aoSampDist) along each axis, combined by n^2 (main axes)
        const float pc[3] = {p.x, p.y, p.z};
        float aop[3], aod[3];
        for (int a = 0; a < 3; ++a) {
            aop[a] = (pc[a] - ap.origin[a]) / ap.ext[a];
            aod[a] = (p.w + ap.sampd[a]) / ap.ext[a];
        }
        float acc = 0.0f;
        for (int a = 0; a < 3; ++a) {
            float q[3] = {aop[0], aop[1], aop[2]};
            q[a] += nn[a] > 0.0f ? aod[a] : -aod[a];
            const float tap = 1.0f - trilinear<true>(T, q[0], q[1], q[2], 1, 0.0f) * ap.eval_fac;
            acc += nn[a] * nn[a] * tap;
        }
        ao[o] = acc;
    } else {
        float q[3];
        for (int a = 0; a < 3; ++a)
            q[a] = (x[a] + nn[a] * ap.sampd[a] - ap.origin[a]) / ap.ext[a];
        ao[o] = 1.0f - trilinear<true>(T, q[0], q[1], q[2], 1, 0.0f) * ap.eval_fac;
    }
}

__global__ void __launch_bounds__(256) pack_normals_kernel(const uint8_t* __restrict__ src, uint32_t stride,
    uint64_t count, uint64_t offset, float4* __restrict__ nrm, int aligned) {
    const uint64_t i = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x;
    if (i >= count)
        return;
    const uint8_t* r = src + i * stride;
    float v[3];
    if (aligned) {
        const float* f = reinterpret_cast<const float*>(r);
        v[0] = f[0];
        v[1] = f[1];
        v[2] = f[2];
    } else {
        for (int c = 0; c < 3; ++c) {
            uint32_t b = (uint32_t) r[4 * c] | ((uint32_t) r[4 * c + 1] << 8) | ((uint32_t) r[4 * c + 2] << 16) |
                         ((uint32_t) r[4 * c + 3] << 24);
            v[c] = __uint_as_float(b);
        }
    }
    nrm[offset + i] = make_float4(v[0], v[1], v[2], 0.0f);
}

// ---------------------------------------------------------------------------------------------
// Brick-major order of the sorted particles (ao_brick_order): bricks of 16 x 4 x 4 cells in (z, y, x) order,
// inside a brick the cells in (z, y, x) order. The cell-sorted particles of one brick row (its 16 cells of one
// (z, y)) are contiguous, so the order is a stable reordering of row segments: segment s = brick * 16 +
// lz * 4 + ly holds the cells x in [16 bx, 16 bx + 16) of row (z, y) = (4 bz + lz, 4 by + ly). Its particles
// lie at [start[k0], start[k0 + 16]) of the cell order; the exclusive scan of the segments' counts gives their
// place in brick order. Particles of the invalid bin (the tail of the cell order) keep their places.
// ---------------------------------------------------------------------------------------------
struct BrickGeo {
    uint32_t nb0, nb1, nb2, nbx, nby;
};

__device__ __forceinline__ bool brick_segment(const BrickGeo& bg, uint32_t s, uint32_t& k0, uint32_t& len) {
    const uint32_t brick = s >> 4, lz = (s >> 2) & 3u, ly = s & 3u;
    const uint32_t bx = brick % bg.nbx, by = (brick / bg.nbx) % bg.nby, bz = brick / (bg.nbx * bg.nby);
    const uint32_t z = 4 * bz + lz, y = 4 * by + ly, x0 = 16 * bx;
    if (z >= bg.nb2 || y >= bg.nb1)
        return false;
    k0 = (z * bg.nb1 + y) * bg.nb0 + x0;
    len = min(16u, bg.nb0 - x0);
    return true;
}

constexpr int BSCAN_THREADS = 256, BSCAN_ITEMS = 16, BSCAN_TILE = BSCAN_THREADS * BSCAN_ITEMS;

// segment counts, and the sum of every tile of BSCAN_TILE segments
__global__ void __launch_bounds__(BSCAN_THREADS) brick_counts_kernel(const uint32_t* __restrict__ start, BrickGeo bg,
    uint32_t nseg, uint32_t* __restrict__ cnt, uint32_t* __restrict__ tsum) {
    __shared__ uint32_t s_sum[BSCAN_THREADS / 32];
    uint32_t sum = 0;
    for (int e = 0; e < BSCAN_ITEMS; ++e) {
        const uint32_t s = blockIdx.x * BSCAN_TILE + e * BSCAN_THREADS + threadIdx.x;
        if (s >= nseg)
            break;
        uint32_t k0, len, c = 0;
        if (brick_segment(bg, s, k0, len))
            c = start[k0 + len] - start[k0];
        cnt[s] = c;
        sum += c;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        sum += __shfl_xor_sync(0xffffffffu, sum, o);
    if ((threadIdx.x & 31) == 0)
        s_sum[threadIdx.x >> 5] = sum;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < BSCAN_THREADS / 32; ++w)
            sum += s_sum[w];
        tsum[blockIdx.x] = sum;
    }
}

// exclusive scan of the tile sums in place (one block)
__global__ void __launch_bounds__(1024) brick_tile_scan_kernel(uint32_t* __restrict__ tsum, uint32_t ntiles) {
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
            s_warp[lane] = ws;
        }
        __syncthreads();
        const uint32_t carry = s_carry;
        if (i < ntiles)
            tsum[i] = carry + (w > 0 ? s_warp[w - 1] : 0u) + incl - x;
        __syncthreads();
        if (tid == 0)
            s_carry = carry + s_warp[31];
        __syncthreads();
    }
}

// the segments' brick-order offsets in place of their counts: the tile's prefix + the scan inside the tile
__global__ void __launch_bounds__(BSCAN_THREADS) brick_offsets_kernel(uint32_t nseg, uint32_t* __restrict__ cnt,
                                                                      const uint32_t* __restrict__ tsum) {
    __shared__ uint32_t s_warp[BSCAN_THREADS / 32];
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    // this thread's segments: BSCAN_ITEMS consecutive ones, so that the in-tile scan is a thread-local run
    const uint32_t s0 = blockIdx.x * BSCAN_TILE + tid * BSCAN_ITEMS;
    uint32_t c[BSCAN_ITEMS], sum = 0;
#pragma unroll
    for (int e = 0; e < BSCAN_ITEMS; ++e) {
        c[e] = s0 + e < nseg ? cnt[s0 + e] : 0u;
        sum += c[e];
    }
    uint32_t incl = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o)
            incl += t;
    }
    if (lane == 31)
        s_warp[w] = incl;
    __syncthreads();
    uint32_t run = tsum[blockIdx.x] + incl - sum;
    for (int k = 0; k < w; ++k)
        run += s_warp[k];
#pragma unroll
    for (int e = 0; e < BSCAN_ITEMS; ++e) {
        if (s0 + e < nseg)
            cnt[s0 + e] = run;
        run += c[e];
    }
}

// One thread per sorted particle (balanced however crowded a cell is): its segment from its record's floor
// cell (the bin key's own cell: clamped to the border cells), its place = the segment's offset + its rank
// in the segment's cell-order run. Particles of the invalid bin (the tail of the cell order) keep theirs.
__global__ void __launch_bounds__(256) brick_scatter_kernel(const uint32_t* __restrict__ start,
    const int4* __restrict__ rec_b, BrickGeo bg, uint32_t nbins, uint32_t n, const uint32_t* __restrict__ off,
    int3 s3, const float4* __restrict__ xyzr, const float4* __restrict__ nrm, const uint32_t* __restrict__ order,
    float4* __restrict__ xyzr_b, float4* __restrict__ nrm_b, uint32_t* __restrict__ order_b) {
    const uint32_t nvalid = start[nbins];
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        uint32_t d = j;
        if (j < nvalid) {
            const int4 B = rec_b[(size_t) REC_STRIDE * j];
            const uint32_t x = (uint32_t) (min(max(B.x, -1), s3.x) + 1);
            const uint32_t y = (uint32_t) (min(max(B.y, -1), s3.y) + 1);
            const uint32_t z = (uint32_t) (min(max(B.z, -1), s3.z) + 1);
            const uint32_t seg = ((((z >> 2) * bg.nby + (y >> 2)) * bg.nbx + (x >> 4)) << 4) | ((z & 3u) << 2) | (y & 3u);
            const uint32_t k0 = (z * bg.nb1 + y) * bg.nb0 + (x & ~15u);
            d = off[seg] + (j - start[k0]);
        }
        xyzr_b[d] = xyzr[j];
        if (nrm)
            nrm_b[d] = nrm[j];
        order_b[d] = order[j];
    }
}

}  // namespace

BrickPlan brick_plan(const GridGeo& g) {
    BrickPlan p{};
    p.nb[0] = g.nb[0];
    p.nb[1] = g.nb[1];
    p.nb[2] = g.nb[2];
    const uint64_t nbx = (g.nb[0] + 15) / 16, nby = (g.nb[1] + 3) / 4, nbz = (g.nb[2] + 3) / 4;
    p.nseg = nbx * nby * nbz * 16;
    p.ntiles = (p.nseg + BSCAN_TILE - 1) / BSCAN_TILE;
    return p;
}

cudaError_t launch_brick_order(const BrickPlan& p, const GridGeo& g, const uint32_t* start, const int4* rec_b,
                               uint32_t n, uint32_t* cnt, uint32_t* tsum, const float4* xyzr, const float4* nrm,
                               const uint32_t* order, float4* xyzr_b, float4* nrm_b, uint32_t* order_b, int sms,
                               cudaStream_t st) {
    if (n == 0)
        return cudaSuccess;
    BrickGeo bg{p.nb[0], p.nb[1], p.nb[2], (p.nb[0] + 15) / 16, (p.nb[1] + 3) / 4};
    const uint32_t nseg = (uint32_t) p.nseg, ntiles = (uint32_t) p.ntiles;
    brick_counts_kernel<<<ntiles, BSCAN_THREADS, 0, st>>>(start, bg, nseg, cnt, tsum);
    brick_tile_scan_kernel<<<1, 1024, 0, st>>>(tsum, ntiles);
    brick_offsets_kernel<<<ntiles, BSCAN_THREADS, 0, st>>>(nseg, cnt, tsum);
    const unsigned grd = (unsigned) std::max<uint32_t>(1u, std::min<uint32_t>(ceil_div(n, 256), (uint32_t) sms * 16));
    brick_scatter_kernel<<<grd, 256, 0, st>>>(start, rec_b, bg, g.nbins, n, cnt, make_int3(g.s[0], g.s[1], g.s[2]),
                                              xyzr, nrm, order, xyzr_b, nrm_b, order_b);
    return cudaGetLastError();
}

cudaError_t launch_mip_levels(const float* l0, const int d0[3], float sat_scale, int quantize, int nlevels,
    float* const* out, int (*dims)[3], int sms, cudaStream_t st) {
    const float* src = l0;
    int sd[3] = {d0[0], d0[1], d0[2]};
    for (int l = 1; l < nlevels; ++l) {
        int dd[3] = {max(1, sd[0] / 2), max(1, sd[1] / 2), max(1, sd[2] / 2)};
        const int64_t nv = (int64_t) dd[0] * dd[1] * dd[2];
        const unsigned grd = (unsigned) std::max<int64_t>(1, std::min<int64_t>((nv + 255) / 256, (int64_t) sms * 32));
        const int pairs = (sd[0] % 2 == 0) && (reinterpret_cast<uintptr_t>(src) % 8 == 0);
        mip_level_kernel<<<grd, 256, 0, st>>>(src, sd[0], sd[1], sd[2], out[l], dd[0], dd[1], dd[2],
                                              l == 1 ? sat_scale : 0.0f, quantize, pairs);
        for (int a = 0; a < 3; ++a)
            dims[l][a] = dd[a];
        src = out[l];
        for (int a = 0; a < 3; ++a)
            sd[a] = dd[a];
    }
    return cudaGetLastError();
}

cudaError_t launch_cone_ao_warp(const ConeParams& cp, const float4* xyzr, const float4* nrm, uint32_t n,
    const uint32_t* out_order, float* ao, int sms, cudaStream_t st) {
    if (n == 0)
        return cudaSuccess;
    const int threads = 32 * cp.ncones;
    const unsigned grd = (unsigned) std::min<uint64_t>(n, (uint64_t) sms * std::max(1, 2048 / threads));
    cone_ao_list_kernel<<<grd, threads, 0, st>>>(cp, nullptr, xyzr, nrm, n, nullptr, out_order, ao);
    return cudaGetLastError();
}

cudaError_t launch_cone_ao(const ConeParams& cp, const uint32_t* order, const float4* xyzr, const float4* nrm,
    uint32_t n, const uint32_t* n_dev, const uint32_t* out_order, float* ao, cudaStream_t st) {
    if (n == 0)
        return cudaSuccess;
    if (n_dev == nullptr) {
        cone_ao_kernel<<<ceil_div(n, 128), 128, 0, st>>>(cp, order, xyzr, nrm, n, out_order, ao);
    } else {
        // the learned AO's fallback list: one block of ncones warps per particle, a bounded grid
        const unsigned grd = (unsigned) std::min<uint32_t>(n, 4096u);
        cone_ao_list_kernel<<<grd, 32 * cp.ncones, 0, st>>>(cp, order, xyzr, nrm, n, n_dev, out_order, ao);
    }
    return cudaGetLastError();
}

cudaError_t launch_aosphere(const AOSphereParams& ap, const float4* xyzr, uint32_t n, unsigned long long* acc, float* tex, const uint32_t* order, const float4* nrm, int mode, float* ao,
    int sms, cudaStream_t st) {
    const int64_t nv = (int64_t) ap.s[0] * ap.s[1] * ap.s[2];
    cudaError_t e = cudaMemsetAsync(acc, 0, sizeof(unsigned long long) * nv, st);
    if (e != cudaSuccess)
        return e;
    if (n > 0)
        aosphere_deposit_kernel<<<ceil_div(n, 256), 256, 0, st>>>(ap, xyzr, n, acc);
    const unsigned grd = (unsigned) std::max<int64_t>(1, std::min<int64_t>((nv + 255) / 256, (int64_t) sms * 16));
    fixed_to_float_kernel<<<grd, 256, 0, st>>>(acc, nv, tex);
    if (n > 0)
        aosphere_ao_kernel<<<ceil_div(n, 128), 128, 0, st>>>(ap, tex, order, xyzr, nrm, n, mode, ao);
    return cudaGetLastError();
}

cudaError_t launch_sort_particles(const uint32_t* order, uint32_t n, const float4* xyzr, const float4* nrm,
                                  float4* xyzr_s, float4* nrm_s, int sms, cudaStream_t st) {
    if (n == 0)
        return cudaSuccess;
    const unsigned grd = (unsigned) std::max<uint32_t>(1u, std::min<uint32_t>(ceil_div(n, 256), (uint32_t) sms * 16));
    sort_particles_kernel<<<grd, 256, 0, st>>>(order, n, xyzr, nrm, xyzr_s, nrm_s);
    return cudaGetLastError();
}

cudaError_t launch_gradient_normals(const GridGeo& geo, const float* grid, const float4* xyzr, uint32_t n, float4* nrm,
                                    cudaStream_t st) {
    if (n == 0)
        return cudaSuccess;
    gradient_normals_kernel<<<ceil_div(n, 256), 256, 0, st>>>(geo, grid, xyzr, n, nrm);
    return cudaGetLastError();
}

cudaError_t launch_pack_normals(const void* src, uint32_t stride, uint64_t count, uint64_t offset, float4* nrm,
    cudaStream_t st) {
    if (count == 0)
        return cudaSuccess;
    const int aligned = (reinterpret_cast<uintptr_t>(src) % 4 == 0) && (stride % 4 == 0);
    pack_normals_kernel<<<(unsigned) ((count + 255) / 256), 256, 0, st>>>(static_cast<const uint8_t*>(src), stride,
                                                                         count, offset, nrm, aligned);
    return cudaGetLastError();
}

}  // namespace p2v
