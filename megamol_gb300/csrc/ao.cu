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
#include "cone_device.cuh"
#include "p2v_common.cuh"

namespace p2v {

namespace {

// ---------------------------------------------------------------------------------------------
// mip pyramid: level l+1 voxel = sum of the children 2g .. min(2g+1, N-1), divided by 8 always
// ---------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(256) mip_level_kernel(const float* __restrict__ src, int sx, int sy, int sz,
    float* __restrict__ dst, int dx, int dy, int dz, float sat_scale, int quantize) {
    const int64_t n = (int64_t) dx * dy * dz;
    for (int64_t i = blockIdx.x * (int64_t) blockDim.x + threadIdx.x; i < n; i += (int64_t) gridDim.x * blockDim.x) {
        const int x = (int) (i % dx);
        const int y = (int) ((i / dx) % dy);
        const int z = (int) (i / ((int64_t) dx * dy));
        const int x1 = min(2 * x + 1, sx - 1), y1 = min(2 * y + 1, sy - 1), z1 = min(2 * z + 1, sz - 1);
        if (quantize) {
            // R8 levels: children as 8-bit integers, the /8 rule rounded half up, stored as k/255
            int k = 0;
            for (int zz = 2 * z; zz <= z1; ++zz)
                for (int yy = 2 * y; yy <= y1; ++yy)
                    for (int xx = 2 * x; xx <= x1; ++xx)
                        k += __float2int_rn(__ldg(src + ((int64_t) zz * sy + yy) * sx + xx) * 255.0f);
            dst[i] = __fdiv_rn((float) ((k + 4) >> 3), 255.0f);
            continue;
        }
        float acc = 0.0f;
        for (int zz = 2 * z; zz <= z1; ++zz)
            for (int yy = 2 * y; yy <= y1; ++yy)
                for (int xx = 2 * x; xx <= x1; ++xx) {
                    float v = __ldg(src + ((int64_t) zz * sy + yy) * sx + xx);
                    if (sat_scale > 0.0f)
                        v = fminf(fmaxf(v * sat_scale, 0.0f), 1.0f);
                    acc += v;
                }
        dst[i] = acc * 0.125f;
    }
}

using Level = ConeLevel;

// GL LINEAR filtering with texel centres at (i + 0.5) / N. border: 0 = CLAMP_TO_BORDER (0 outside),
// 1 = CLAMP_TO_EDGE. sat > 0 saturates level-0 texels (the level-0 texture holds clamp(v*sat, 0, 1)).
__device__ __forceinline__ float tex_fetch(const Level& L, int x, int y, int z, int border, float sat) {
    if (border == 0) {
        if ((unsigned) x >= (unsigned) L.d[0] || (unsigned) y >= (unsigned) L.d[1] || (unsigned) z >= (unsigned) L.d[2])
            return 0.0f;
    } else {
        x = min(max(x, 0), L.d[0] - 1);
        y = min(max(y, 0), L.d[1] - 1);
        z = min(max(z, 0), L.d[2] - 1);
    }
    const float v = __ldg(L.v + ((int64_t) z * L.d[1] + y) * L.d[0] + x);
    return sat > 0.0f ? fminf(fmaxf(v * sat, 0.0f), 1.0f) : v;
}

__device__ __forceinline__ float lerp_rn(float a, float b, float w) {
    return __fmaf_rn(w, __fsub_rn(b, a), a);
}

__device__ __forceinline__ float saturate_if(float v, float sat) {
    return sat > 0.0f ? fminf(fmaxf(v * sat, 0.0f), 1.0f) : v;
}

// One GL LINEAR sample. When the 2x2x2 block lies inside the level (the common case) the eight texels are
// read from one base pointer without per-texel checks. The base offset and the z stride are 64-bit: a level
// may hold more than 2^31 texels (an AOSphere volume of 2048^3, a density grid above 1290^3).
__device__ __forceinline__ float trilinear(const Level& L, float ux, float uy, float uz, int border, float sat) {
    // explicitly rounded operations: every kernel that inlines this gets the same bits
    const float cx = __fmaf_rn(ux, L.fd[0], -0.5f), cy = __fmaf_rn(uy, L.fd[1], -0.5f);
    const float cz = __fmaf_rn(uz, L.fd[2], -0.5f);
    const float fx0 = floorf(cx), fy0 = floorf(cy), fz0 = floorf(cz);
    const int x0 = (int) fx0, y0 = (int) fy0, z0 = (int) fz0;
    const float fx = __fsub_rn(cx, fx0), fy = __fsub_rn(cy, fy0), fz = __fsub_rn(cz, fz0);
    float c000, c100, c010, c110, c001, c101, c011, c111;
    if (x0 >= 0 && y0 >= 0 && z0 >= 0 && x0 + 1 < L.d[0] && y0 + 1 < L.d[1] && z0 + 1 < L.d[2]) {
        const int sy = L.d[0];
        const int64_t sz = (int64_t) L.d[0] * L.d[1];
        const float* b = L.v + (((int64_t) z0 * L.d[1] + y0) * L.d[0] + x0);
        c000 = saturate_if(__ldg(b), sat);
        c100 = saturate_if(__ldg(b + 1), sat);
        c010 = saturate_if(__ldg(b + sy), sat);
        c110 = saturate_if(__ldg(b + sy + 1), sat);
        c001 = saturate_if(__ldg(b + sz), sat);
        c101 = saturate_if(__ldg(b + sz + 1), sat);
        c011 = saturate_if(__ldg(b + sz + sy), sat);
        c111 = saturate_if(__ldg(b + sz + sy + 1), sat);
    } else {
        c000 = tex_fetch(L, x0, y0, z0, border, sat);
        c100 = tex_fetch(L, x0 + 1, y0, z0, border, sat);
        c010 = tex_fetch(L, x0, y0 + 1, z0, border, sat);
        c110 = tex_fetch(L, x0 + 1, y0 + 1, z0, border, sat);
        c001 = tex_fetch(L, x0, y0, z0 + 1, border, sat);
        c101 = tex_fetch(L, x0 + 1, y0, z0 + 1, border, sat);
        c011 = tex_fetch(L, x0, y0 + 1, z0 + 1, border, sat);
        c111 = tex_fetch(L, x0 + 1, y0 + 1, z0 + 1, border, sat);
    }
    const float c00 = lerp_rn(c000, c100, fx), c10 = lerp_rn(c010, c110, fx);
    const float c01 = lerp_rn(c001, c101, fx), c11 = lerp_rn(c011, c111, fx);
    const float c0 = lerp_rn(c00, c10, fy), c1 = lerp_rn(c01, c11, fy);
    return lerp_rn(c0, c1, fz);
}

// Visibility sample k of a cone: trilinear in the two levels around its lod, blended linearly
// (LINEAR_MIPMAP_LINEAR).
__device__ __forceinline__ float cone_sample(const ConeParams& cp, const float dir[3], const float u[3], int k) {
    const float t = cp.t[k];
    const float lod = cp.lod[k];
    const float qx = __fmaf_rn(t, dir[0], u[0]), qy = __fmaf_rn(t, dir[1], u[1]), qz = __fmaf_rn(t, dir[2], u[2]);
    const int l0 = min((int) lod, cp.nlevels - 1);
    const float fr = __fsub_rn(lod, (float) l0);
    float vis = trilinear(cp.lv[l0], qx, qy, qz, cp.border, l0 == 0 ? cp.sat : 0.0f);
    if (fr > 0.0f && l0 + 1 < cp.nlevels)
        vis = __fmaf_rn(fr, trilinear(cp.lv[l0 + 1], qx, qy, qz, cp.border, 0.0f), __fmul_rn(1.0f - fr, vis));
    return vis;
}

// One cone of the MDAO march (mdao_deferred_fragment_ambocc.inc.glsl:30-51) from normalised point u.
__device__ __forceinline__ float march_cone(const ConeParams& cp, int c, const float u[3], const float ex[3],
                                            const float nn[3], const float ez[3]) {
    float dir[3];
    cone_dir(cp, c, ex, nn, ez, dir);
    float acc = 0.0f;
    for (int k = 0; k < cp.nsteps; ++k) {
        acc = __fmaf_rn(1.0f - acc, cone_sample(cp, dir, u, k), acc);
        if (cp.early_exit && acc > 0.99f)
            break;
    }
    return acc;
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
    const float4 p = xyzr[o];
    const float4 nv = nrm[o];
    float x[3], nn[3];
    if (!surface_point(p, nv, x, nn)) {
        ao[w] = 1.0f;  // no normal: no occlusion
        return;
    }
    float u[3], ex[3], ez[3];
    cone_frame(cp, x, nn, u, ex, ez);
    float ambient = 0.0f;
    for (int c = 0; c < cp.ncones; ++c)
        ambient += march_cone(cp, c, u, ex, nn, ez);
    ao[w] = 1.0f - fminf(fmaxf(cp.strength * ambient / (float) cp.ncones, 0.0f), 1.0f);
}

// The learned AO's fallback list (its length a device-side count, usually tiny): latency matters, so a
// block takes one particle with one warp per cone, and the lanes of a warp take the cone's samples (32 at a
// time: the step positions are tabulated, so all samples load at once). Every lane then runs the march's
// recurrence over the shuffled samples in step order with the same early exit, the block's first thread
// adds the cones in cone order: the result has the bits of cone_ao_kernel. A bounded grid strides over the
// list.
__global__ void __launch_bounds__(32 * MAX_CONES) cone_ao_list_kernel(const ConeParams cp,
    const uint32_t* __restrict__ list, const float4* __restrict__ xyzr, const float4* __restrict__ nrm, uint32_t n,
    const uint32_t* __restrict__ n_dev, const uint32_t* __restrict__ out_order, float* __restrict__ ao) {
    __shared__ float s_acc[MAX_CONES];
    const int lane = threadIdx.x & 31, c = threadIdx.x >> 5;
    n = min(n, *n_dev);
    for (uint32_t i = blockIdx.x; i < n; i += gridDim.x) {
        const uint32_t o = list[i];
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
            const float vis = k0 + lane < cp.nsteps ? cone_sample(cp, dir, u, k0 + lane) : 0.0f;
            const int m = min(32, cp.nsteps - k0);
            for (int s = 0; s < m; ++s) {
                acc = __fmaf_rn(1.0f - acc, __shfl_sync(0xffffffffu, vis, s), acc);
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
                ambient += s_acc[k];
            ao[w] = 1.0f - fminf(fmaxf(cp.strength * ambient / (float) cp.ncones, 0.0f), 1.0f);
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

// Normals from the density grid (P2V_NORMALS_GRADIENT): -grad(rho) at the particle, normalised. grad(rho) at
// node i along axis a is (v[i + 1] - v[i - 1]) / (2 h) with the neighbours wrapped on a cyclic axis, and the
// one-sided first differences (v[1] - v[0]) / h, (v[s-1] - v[s-2]) / h at the faces of an open one; the node
// gradients are interpolated trilinearly at u = (p - min) / h clamped into [0, s - 1].
__device__ __forceinline__ float node_grad(const float* __restrict__ g, int64_t base, int64_t stride, int i, int s,
                                           int cyc, float ih) {
    if (s < 2)
        return 0.0f;
    int lo = i - 1, hi = i + 1;
    float scale = 0.5f * ih;
    if (cyc) {
        lo = lo < 0 ? lo + s : lo;
        hi = hi >= s ? hi - s : hi;
    } else if (i == 0) {
        lo = 0;
        scale = ih;
    } else if (i == s - 1) {
        hi = s - 1;
        scale = ih;
    }
    return (__ldg(g + base + hi * stride) - __ldg(g + base + lo * stride)) * scale;
}

__global__ void __launch_bounds__(256) gradient_normals_kernel(const GridGeo geo, const float* __restrict__ grid,
    const float4* __restrict__ xyzr, uint32_t n, float4* __restrict__ nrm) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n)
        return;
    const float4 p = xyzr[j];
    const float pc[3] = {p.x, p.y, p.z};
    int i0[3], i1[3];
    float f[3], ih[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        ih[a] = 1.0f / geo.hf[a];
        float u = (pc[a] - geo.minf[a]) * ih[a];
        u = fminf(fmaxf(u, 0.0f), (float) (geo.s[a] - 1));  // a NaN coordinate becomes 0 (fmaxf)
        const int k = min((int) u, geo.s[a] - 1);
        i0[a] = k;
        i1[a] = min(k + 1, geo.s[a] - 1);
        f[a] = u - (float) k;
    }
    const int64_t sx = geo.s[0], sxy = (int64_t) geo.s[0] * geo.s[1];
    float gr[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        const int x = (c & 1) ? i1[0] : i0[0], y = (c & 2) ? i1[1] : i0[1], z = (c & 4) ? i1[2] : i0[2];
        const float w = ((c & 1) ? f[0] : 1.0f - f[0]) * ((c & 2) ? f[1] : 1.0f - f[1]) * ((c & 4) ? f[2] : 1.0f - f[2]);
        gr[0] += w * node_grad(grid, z * sxy + y * sx, 1, x, geo.s[0], geo.cyc[0], ih[0]);
        gr[1] += w * node_grad(grid, z * sxy + x, sx, y, geo.s[1], geo.cyc[1], ih[1]);
        gr[2] += w * node_grad(grid, y * sx + x, sxy, z, geo.s[2], geo.cyc[2], ih[2]);
    }
    const float l2 = gr[0] * gr[0] + gr[1] * gr[1] + gr[2] * gr[2];
    float4 out = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (l2 > 0.0f && isfinite(l2)) {
        const float il = -rsqrtf(l2);
        out = make_float4(gr[0] * il, gr[1] * il, gr[2] * il, 0.0f);
    }
    nrm[j] = out;
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
    Level T;
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
            const float tap = 1.0f - trilinear(T, q[0], q[1], q[2], 1, 0.0f) * ap.eval_fac;
            acc += nn[a] * nn[a] * tap;
        }
        ao[o] = acc;
    } else {
        float q[3];
        for (int a = 0; a < 3; ++a)
            q[a] = (x[a] + nn[a] * ap.sampd[a] - ap.origin[a]) / ap.ext[a];
        ao[o] = 1.0f - trilinear(T, q[0], q[1], q[2], 1, 0.0f) * ap.eval_fac;
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

}  // namespace

cudaError_t launch_mip_levels(const float* l0, const int d0[3], float sat_scale, int quantize, int nlevels,
    float* const* out, int (*dims)[3], int sms, cudaStream_t st) {
    const float* src = l0;
    int sd[3] = {d0[0], d0[1], d0[2]};
    for (int l = 1; l < nlevels; ++l) {
        int dd[3] = {max(1, sd[0] / 2), max(1, sd[1] / 2), max(1, sd[2] / 2)};
        const int64_t nv = (int64_t) dd[0] * dd[1] * dd[2];
        const unsigned grd = (unsigned) std::max<int64_t>(1, std::min<int64_t>((nv + 255) / 256, (int64_t) sms * 32));
        mip_level_kernel<<<grd, 256, 0, st>>>(src, sd[0], sd[1], sd[2], out[l], dd[0], dd[1], dd[2],
                                              l == 1 ? sat_scale : 0.0f, quantize);
        for (int a = 0; a < 3; ++a)
            dims[l][a] = dd[a];
        src = out[l];
        for (int a = 0; a < 3; ++a)
            sd[a] = dd[a];
    }
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
