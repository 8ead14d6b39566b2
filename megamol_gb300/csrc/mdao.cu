// MDAO occupancy voxeliser: the AO volume of moldyn_gl::SphereRenderer's MDAO mode, built with CUDA
// instead of the reference's layered point rasterisation.
//
// The reference (MDAOVolumeGenerator.cpp:117-238 with mdao_volume.vert/geom/frag.glsl) draws every sphere
// as one point sprite per z-slice it touches into an R8 3D texture with additive blending. Here one warp
// takes one sphere: the lanes first compute the slice disks the geometry shader would emit (one disk per
// lane), prefix-sum the pixel counts of their point squares, and then walk the flattened (disk, pixel)
// list 32 fragments at a time. Each fragment evaluates the fragment shader's coverage fraction with
// explicitly rounded FP32 operations in the shader's order, and adds its blend contribution with one
// integer atomic:
//   unorm8: q = round(clamp(frac, 0, 1) * 255) into a 32-bit counter; texel = min(255, sum) / 255. For
//           non-negative contributions the saturating 8-bit blend chain equals this clamped integer sum.
//   fp32:   clamp(frac, 0, 1) in 2^-32 fixed point into a 64-bit counter; texel = min(1, sum).
// Integer sums are independent of the order in which fragments arrive, so the volume is deterministic.
// Saturated voxels (a dense liquid's interior) are recognised by a plain read and skip the atomic.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "ao_internal.h"

namespace p2v {
namespace {

__device__ __forceinline__ float sq_rn(float v) {
    return __fmul_rn(v, v);
}

__device__ __forceinline__ float dot3_rn(float x, float y, float z) {
    return __fadd_rn(__fadd_rn(sq_rn(x), sq_rn(y)), sq_rn(z));
}

// mdao_volume.frag.glsl:9-76 for voxel (i, j, layer) and a sphere with centre c relative to inBoundsMin and
// squared radius w2. Returns -1 for a discarded fragment.
__device__ float mdao_fragment(const MdaoParams& mp, int i, int j, int layer, float cx, float cy, float cz,
                               float w2) {
    const float cm[3] = {__fmul_rn((float) i, mp.cell[0]), __fmul_rn((float) j, mp.cell[1]),
                         __fmul_rn((float) layer, mp.cell[2])};
    const float c[3] = {cx, cy, cz};
    float lo[3], hi[3], fp[3], np[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        lo[a] = __fsub_rn(cm[a], c[a]);
        hi[a] = __fadd_rn(lo[a], mp.cell[a]);
        fp[a] = fmaxf(fabsf(lo[a]), fabsf(hi[a]));
        np[a] = fminf(fabsf(lo[a]), fabsf(hi[a]));
    }
    // the closest cell corner outside the sphere: discard (this also discards spheres lying inside the
    // cell, so the shader's sphere-in-cell branch below is reached only by spheres touching a corner)
    if (__fsub_rn(dot3_rn(np[0], np[1], np[2]), w2) > 0.0f)
        return -1.0f;
    if (__fsub_rn(dot3_rn(fp[0], fp[1], fp[2]), w2) < 0.0f)
        return 1.0f;
    const float radius = __fsqrt_rn(w2);
    if (lo[0] <= -radius && lo[1] <= -radius && lo[2] <= -radius && hi[0] >= radius && hi[1] >= radius &&
        hi[2] >= radius)
        return __fdiv_rn(__fmul_rn(__fmul_rn(mp.sphere_k, w2), radius), mp.cell_vol);
    // 3x3x3 samples at the cell's corners, edge midpoints and centre
    float s[3][3];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int k = 0; k < 3; ++k)
            s[a][k] = sq_rn(__fsub_rn(__fadd_rn(cm[a], __fmul_rn(__fmul_rn(mp.cell[a], (float) k), 0.5f)), c[a]));
    int hits = 0;
#pragma unroll
    for (int x = 0; x < 3; ++x)
#pragma unroll
        for (int y = 0; y < 3; ++y) {
            const float xy = __fadd_rn(s[0][x], s[1][y]);
#pragma unroll
            for (int z = 0; z < 3; ++z)
                hits += __fsub_rn(__fadd_rn(xy, s[2][z]), w2) < 0.0f ? 1 : 0;
        }
    return __fdiv_rn((float) hits, 27.0f);
}

// Pixel centres i + 0.5 in [wc - size/2, wc + size/2), clipped to [0, n). size <= 2^22 keeps both
// subtractions of 0.5 exact.
__device__ __forceinline__ void point_span(float wc, float size, int n, int& i0, int& i1) {
    const float half = 0.5f * size;
    const float lo = __fsub_rn(wc, half), hi = __fadd_rn(wc, half);
    i0 = (int) fminf(fmaxf(ceilf(__fsub_rn(lo, 0.5f)), 0.0f), (float) n);
    i1 = (int) fminf(fmaxf(ceilf(__fsub_rn(hi, 0.5f)), 0.0f), (float) n);
}

template <bool U8>
__global__ void __launch_bounds__(256) mdao_voxelise_kernel(const MdaoParams mp, const uint32_t* __restrict__ order,
                                                            const float4* __restrict__ xyzr, uint32_t n,
                                                            void* __restrict__ accv) {
    const int lane = threadIdx.x & 31;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t k = warp; k < n; k += nwarps) {
        const float4 p = __ldg(xyzr + (order ? __ldg(order + k) : k));
        const float r = p.w;
        // mdao_volume.geom.glsl:72-92; every lane evaluates the same sphere, so branches are warp-uniform
        const float npx = __fmul_rn(__fsub_rn(p.x, mp.bmin[0]), mp.inv[0]);
        const float npy = __fmul_rn(__fsub_rn(p.y, mp.bmin[1]), mp.inv[1]);
        const float npz = __fmul_rn(__fsub_rn(p.z, mp.bmin[2]), mp.inv[2]);
        const float ndx = __fsub_rn(__fmul_rn(npx, 2.0f), 1.0f);
        const float ndy = __fsub_rn(__fmul_rn(npy, 2.0f), 1.0f);
        const float ndz = __fsub_rn(__fmul_rn(npz, 2.0f), 1.0f);
        // a point primitive survives clipping only if its centre vertex lies in the clip volume
        if (!(ndx >= -1.0f && ndx <= 1.0f && ndy >= -1.0f && ndy <= 1.0f && ndz >= -1.0f && ndz <= 1.0f))
            continue;
        const float cx = __fsub_rn(p.x, mp.bmin[0]), cy = __fsub_rn(p.y, mp.bmin[1]), cz = __fsub_rn(p.z, mp.bmin[2]);
        const float w2 = sq_rn(r);
        const float xw = __fadd_rn(__fmul_rn(ndx, mp.half_vp[0]), mp.half_vp[0]);
        const float yw = __fadd_rn(__fmul_rn(ndy, mp.half_vp[1]), mp.half_vp[1]);
        const int ns = (int) fminf(ceilf(__fmul_rn(__fmul_rn(r, mp.inv[2]), mp.fd[2])), (float) (mp.d[2] + 1));
        const float zs = __fmul_rn(npz, mp.fd[2]);
        const int cl = (int) floorf(zs);
        const float thick = __fdiv_rn(1.0f, mp.fd[2]);
        const float zoff = __fdiv_rn(__fsub_rn(zs, floorf(zs)), mp.fd[2]);
        const int ndisk = 1 + 2 * max(ns, 0);
        for (int base = 0; base < ndisk; base += 32) {
            // disk q: 0 = centre slice, 1..ns = negative hemisphere, ns+1..2ns = positive hemisphere. The
            // squared slice radius falls with i, so the shader's `break` equals dropping every disk whose
            // squared radius is negative.
            const int q = base + lane;
            int layer = 0, x0 = 0, x1 = 0, y0 = 0, y1 = 0;
            bool ok = false;
            if (q < ndisk) {
                float disk = r;
                layer = cl;
                ok = true;
                if (q > 0) {
                    const bool pos = q > ns;
                    const int i = pos ? q - ns : q;
                    const float off = pos ? __fsub_rn(thick, zoff) : zoff;
                    const float dist = __fdiv_rn(__fadd_rn(__fdiv_rn((float) (i - 1), mp.fd[2]), off), mp.inv[2]);
                    const float nsq = __fsub_rn(sq_rn(r), sq_rn(dist));
                    ok = !(nsq < 0.0f);
                    disk = __fsqrt_rn(fmaxf(nsq, 0.0f));
                    layer = pos ? cl + i : cl - i;
                }
                ok = ok && layer >= 0 && layer < mp.d[2];
                if (ok) {
                    const float ps = fmaxf(fminf(2.0f * ceilf(__fmul_rn(disk, mp.ps_scale)), 4194304.0f), 1.0f);
                    point_span(xw, ps, mp.d[0], x0, x1);
                    point_span(yw, ps, mp.d[1], y0, y1);
                }
            }
            const int wdt = x1 - x0;
            const int cnt = ok ? wdt * (y1 - y0) : 0;
            int incl = cnt;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int v = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o)
                    incl += v;
            }
            const int total = __shfl_sync(0xffffffffu, incl, 31);
            for (int sb = 0; sb < total; sb += 32) {
                const int s = sb + lane;
                // the disk holding fragment s: the number of disks whose inclusive count is <= s
                int j = 0;
#pragma unroll
                for (int step = 16; step > 0; step >>= 1) {
                    const int v = __shfl_sync(0xffffffffu, incl, j + step - 1);
                    if (v <= s)
                        j += step;
                }
                const int dl = __shfl_sync(0xffffffffu, layer, j);
                const int dx0 = __shfl_sync(0xffffffffu, x0, j);
                const int dy0 = __shfl_sync(0xffffffffu, y0, j);
                const int dw = __shfl_sync(0xffffffffu, wdt, j);
                const int dex = __shfl_sync(0xffffffffu, incl - cnt, j);
                if (s >= total)
                    continue;
                const int local = s - dex;
                const int px = dx0 + local % dw, py = dy0 + local / dw;
                float f = mdao_fragment(mp, px, py, dl, cx, cy, cz, w2);
                if (f < 0.0f)
                    continue;
                f = fminf(fmaxf(f, 0.0f), 1.0f);  // UNORM colour clamp before blending
                const int64_t v = (int64_t) px + ((int64_t) py + (int64_t) dl * mp.d[1]) * mp.d[0];
                if (U8) {
                    unsigned int* acc = static_cast<unsigned int*>(accv) + v;
                    const unsigned int qv = __float2uint_rn(__fmul_rn(f, 255.0f));
                    if (qv != 0u && *(volatile unsigned int*) acc < 255u)
                        atomicAdd(acc, qv);
                } else {
                    unsigned long long* acc = static_cast<unsigned long long*>(accv) + v;
                    const unsigned long long qv = __float2ull_rn(__fmul_rn(f, 4294967296.0f));
                    if (qv != 0ull && *(volatile unsigned long long*) acc < (1ull << 32))
                        atomicAdd(acc, qv);
                }
            }
        }
    }
}

template <bool U8>
__global__ void __launch_bounds__(256) mdao_finish_kernel(const void* __restrict__ accv, int64_t nv,
                                                          float* __restrict__ vol) {
    for (int64_t i = blockIdx.x * (int64_t) blockDim.x + threadIdx.x; i < nv; i += (int64_t) gridDim.x * blockDim.x) {
        if (U8) {
            const unsigned int a = static_cast<const unsigned int*>(accv)[i];
            vol[i] = __fdiv_rn((float) min(a, 255u), 255.0f);
        } else {
            const unsigned long long a = static_cast<const unsigned long long*>(accv)[i];
            vol[i] = a >= (1ull << 32) ? 1.0f : __fmul_rn(__ull2float_rn(a), 1.0f / 4294967296.0f);
        }
    }
}

}  // namespace

cudaError_t launch_mdao_volume(const MdaoParams& mp, const uint32_t* order, const float4* xyzr, uint32_t n,
                               void* acc, float* vol, int sms, cudaStream_t st) {
    const int64_t nv = (int64_t) mp.d[0] * mp.d[1] * mp.d[2];
    cudaError_t e = cudaMemsetAsync(acc, 0, (mp.unorm8 ? sizeof(unsigned int) : sizeof(unsigned long long)) * nv, st);
    if (e != cudaSuccess)
        return e;
    if (n > 0) {
        const unsigned grd = (unsigned) std::max<int64_t>(1, std::min<int64_t>(((int64_t) n + 7) / 8, (int64_t) sms * 16));
        if (mp.unorm8)
            mdao_voxelise_kernel<true><<<grd, 256, 0, st>>>(mp, order, xyzr, n, acc);
        else
            mdao_voxelise_kernel<false><<<grd, 256, 0, st>>>(mp, order, xyzr, n, acc);
    }
    const unsigned grd = (unsigned) std::max<int64_t>(1, std::min<int64_t>((nv + 255) / 256, (int64_t) sms * 16));
    if (mp.unorm8)
        mdao_finish_kernel<true><<<grd, 256, 0, st>>>(acc, nv, vol);
    else
        mdao_finish_kernel<false><<<grd, 256, 0, st>>>(acc, nv, vol);
    return cudaGetLastError();
}

}  // namespace p2v
