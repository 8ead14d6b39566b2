// Device code of the MDAO cone march, the mip build and the gradient normals, shared by the per-frame
// kernels (ao.cu) and the persistent batch kernel (batch_ao.cu). Every function is written in explicitly
// rounded FP32 (or in operations no compiler contracts), so each kernel that inlines it computes the same
// bits.
//
// NC selects how volume texels are loaded: true reads through the non-coherent path (__ldg), which is
// valid only for data no thread writes during the kernel; false uses plain loads, which the persistent batch
// kernel needs for the mip levels its own items write (an acquire of the level's completion count orders
// them).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "ao_internal.h"
#include "cone_device.cuh"
#include "p2v_common.cuh"

namespace p2v {

template <bool NC>
__device__ __forceinline__ float ld_texel(const float* p) {
    if constexpr (NC)
        return __ldg(p);
    else
        return *p;
}

// Voxel (x, y, z) of mip level l+1 from level l (src, sx x sy x sz): the sum of the children
// 2g .. min(2g+1, N-1), divided by 8 always (mdao_mipmap_compute_main.comp.glsl:8-26). sat_scale > 0
// saturates the children first (level 0 of a density volume as the cone march sees it). quantize: R8
// levels, children as 8-bit integers, the /8 rule rounded half up, stored as k/255.
template <bool NC>
__device__ __forceinline__ float mip_voxel(const float* src, int sx, int sy, int sz, int x, int y, int z,
                                           float sat_scale, int quantize) {
    const int x1 = min(2 * x + 1, sx - 1), y1 = min(2 * y + 1, sy - 1), z1 = min(2 * z + 1, sz - 1);
    if (quantize) {
        int k = 0;
        for (int zz = 2 * z; zz <= z1; ++zz)
            for (int yy = 2 * y; yy <= y1; ++yy)
                for (int xx = 2 * x; xx <= x1; ++xx)
                    k += __float2int_rn(__fmul_rn(ld_texel<NC>(src + ((int64_t) zz * sy + yy) * sx + xx), 255.0f));
        return __fdiv_rn((float) ((k + 4) >> 3), 255.0f);
    }
    float acc = 0.0f;
    for (int zz = 2 * z; zz <= z1; ++zz)
        for (int yy = 2 * y; yy <= y1; ++yy)
            for (int xx = 2 * x; xx <= x1; ++xx) {
                float v = ld_texel<NC>(src + ((int64_t) zz * sy + yy) * sx + xx);
                if (sat_scale > 0.0f)
                    v = fminf(fmaxf(__fmul_rn(v, sat_scale), 0.0f), 1.0f);
                acc = __fadd_rn(acc, v);
            }
    return __fmul_rn(acc, 0.125f);
}

// GL LINEAR filtering with texel centres at (i + 0.5) / N. border: 0 = CLAMP_TO_BORDER (0 outside),
// 1 = CLAMP_TO_EDGE. sat > 0 saturates level-0 texels (the level-0 texture holds clamp(v*sat, 0, 1)).
__device__ __forceinline__ float saturate_if(float v, float sat) {
    return sat > 0.0f ? fminf(fmaxf(__fmul_rn(v, sat), 0.0f), 1.0f) : v;
}

template <bool NC>
__device__ __forceinline__ float tex_fetch(const ConeLevel& L, int x, int y, int z, int border, float sat) {
    if (border == 0) {
        if ((unsigned) x >= (unsigned) L.d[0] || (unsigned) y >= (unsigned) L.d[1] || (unsigned) z >= (unsigned) L.d[2])
            return 0.0f;
    } else {
        x = min(max(x, 0), L.d[0] - 1);
        y = min(max(y, 0), L.d[1] - 1);
        z = min(max(z, 0), L.d[2] - 1);
    }
    return saturate_if(ld_texel<NC>(L.v + ((int64_t) z * L.d[1] + y) * L.d[0] + x), sat);
}

__device__ __forceinline__ float lerp_rn(float a, float b, float w) {
    return __fmaf_rn(w, __fsub_rn(b, a), a);
}

// One GL LINEAR sample. When the 2x2x2 block lies inside the level (the common case) the eight texels are
// read from one base pointer without per-texel checks. The base offset and the z stride are 64-bit: a level
// may hold more than 2^31 texels (an AOSphere volume of 2048^3, a density grid above 1290^3).
template <bool NC>
__device__ __forceinline__ float trilinear(const ConeLevel& L, float ux, float uy, float uz, int border, float sat) {
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
        c000 = saturate_if(ld_texel<NC>(b), sat);
        c100 = saturate_if(ld_texel<NC>(b + 1), sat);
        c010 = saturate_if(ld_texel<NC>(b + sy), sat);
        c110 = saturate_if(ld_texel<NC>(b + sy + 1), sat);
        c001 = saturate_if(ld_texel<NC>(b + sz), sat);
        c101 = saturate_if(ld_texel<NC>(b + sz + 1), sat);
        c011 = saturate_if(ld_texel<NC>(b + sz + sy), sat);
        c111 = saturate_if(ld_texel<NC>(b + sz + sy + 1), sat);
    } else {
        c000 = tex_fetch<NC>(L, x0, y0, z0, border, sat);
        c100 = tex_fetch<NC>(L, x0 + 1, y0, z0, border, sat);
        c010 = tex_fetch<NC>(L, x0, y0 + 1, z0, border, sat);
        c110 = tex_fetch<NC>(L, x0 + 1, y0 + 1, z0, border, sat);
        c001 = tex_fetch<NC>(L, x0, y0, z0 + 1, border, sat);
        c101 = tex_fetch<NC>(L, x0 + 1, y0, z0 + 1, border, sat);
        c011 = tex_fetch<NC>(L, x0, y0 + 1, z0 + 1, border, sat);
        c111 = tex_fetch<NC>(L, x0 + 1, y0 + 1, z0 + 1, border, sat);
    }
    const float c00 = lerp_rn(c000, c100, fx), c10 = lerp_rn(c010, c110, fx);
    const float c01 = lerp_rn(c001, c101, fx), c11 = lerp_rn(c011, c111, fx);
    const float c0 = lerp_rn(c00, c10, fy), c1 = lerp_rn(c01, c11, fy);
    return lerp_rn(c0, c1, fz);
}

// Visibility sample k of a cone: trilinear in the two levels around its lod, blended linearly
// (LINEAR_MIPMAP_LINEAR).
template <bool NC>
__device__ __forceinline__ float cone_sample(const ConeParams& cp, const float dir[3], const float u[3], int k) {
    const float t = cp.t[k];
    const float lod = cp.lod[k];
    const float qx = __fmaf_rn(t, dir[0], u[0]), qy = __fmaf_rn(t, dir[1], u[1]), qz = __fmaf_rn(t, dir[2], u[2]);
    const int l0 = min((int) lod, cp.nlevels - 1);
    const float fr = __fsub_rn(lod, (float) l0);
    float vis = trilinear<NC>(cp.lv[l0], qx, qy, qz, cp.border, l0 == 0 ? cp.sat : 0.0f);
    if (fr > 0.0f && l0 + 1 < cp.nlevels)
        vis = __fmaf_rn(fr, trilinear<NC>(cp.lv[l0 + 1], qx, qy, qz, cp.border, 0.0f),
                        __fmul_rn(__fsub_rn(1.0f, fr), vis));
    return vis;
}

// One cone of the MDAO march (mdao_deferred_fragment_ambocc.inc.glsl:30-51) from normalised point u.
template <bool NC>
__device__ __forceinline__ float march_cone(const ConeParams& cp, int c, const float u[3], const float ex[3],
                                            const float nn[3], const float ez[3]) {
    float dir[3];
    cone_dir(cp, c, ex, nn, ez, dir);
    float acc = 0.0f;
    for (int k = 0; k < cp.nsteps; ++k) {
        acc = __fmaf_rn(__fsub_rn(1.0f, acc), cone_sample<NC>(cp, dir, u, k), acc);
        if (cp.early_exit && acc > 0.99f)
            break;
    }
    return acc;
}

// The AO of one particle (position and radius p, normal nv): 1 - clamp(strength * mean cone occlusion, 0, 1),
// 1 for a particle without a normal.
__device__ __forceinline__ float cone_combine(const ConeParams& cp, float ambient) {
    return __fsub_rn(1.0f, fminf(fmaxf(__fdiv_rn(__fmul_rn(cp.strength, ambient), (float) cp.ncones), 0.0f), 1.0f));
}

template <bool NC>
__device__ __forceinline__ float cone_ao_at(const ConeParams& cp, const float4 p, const float4 nv) {
    float x[3], nn[3];
    if (!surface_point(p, nv, x, nn))
        return 1.0f;  // no normal: no occlusion
    float u[3], ex[3], ez[3];
    cone_frame(cp, x, nn, u, ex, ez);
    float ambient = 0.0f;
    for (int c = 0; c < cp.ncones; ++c)
        ambient = __fadd_rn(ambient, march_cone<NC>(cp, c, u, ex, nn, ez));
    return cone_combine(cp, ambient);
}

// Normals from the density grid (P2V_NORMALS_GRADIENT): -grad(rho) at the particle, normalised. grad(rho) at
// node i along axis a is (v[i + 1] - v[i - 1]) / (2 h) with the neighbours wrapped on a cyclic axis, and the
// one-sided first differences (v[1] - v[0]) / h, (v[s-1] - v[s-2]) / h at the faces of an open one; the node
// gradients are interpolated trilinearly at u = (p - min) / h clamped into [0, s - 1].
template <bool NC>
__device__ __forceinline__ float node_grad(const float* g, int64_t base, int64_t stride, int i, int s, int cyc,
                                           float ih) {
    if (s < 2)
        return 0.0f;
    int lo = i - 1, hi = i + 1;
    float scale = __fmul_rn(0.5f, ih);
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
    return __fmul_rn(__fsub_rn(ld_texel<NC>(g + base + hi * stride), ld_texel<NC>(g + base + lo * stride)), scale);
}

// lo / hi neighbour and scale of node_grad at node i along an axis of s nodes (s >= 2)
__device__ __forceinline__ void grad_stencil(int i, int s, int cyc, float ih, int& lo, int& hi, float& scale) {
    lo = i - 1;
    hi = i + 1;
    scale = __fmul_rn(0.5f, ih);
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
}

template <bool NC>
__device__ __forceinline__ float4 gradient_normal(const GridGeo& geo, const float* grid, const float4 p) {
    const float pc[3] = {p.x, p.y, p.z};
    int i0[3], i1[3];
    float f[3], ih[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        ih[a] = __frcp_rn(geo.hf[a]);
        float u = __fmul_rn(__fsub_rn(pc[a], geo.minf[a]), ih[a]);
        u = fminf(fmaxf(u, 0.0f), (float) (geo.s[a] - 1));  // a NaN coordinate becomes 0 (fmaxf)
        const int k = min((int) u, geo.s[a] - 1);
        i0[a] = k;
        i1[a] = min(k + 1, geo.s[a] - 1);
        f[a] = __fsub_rn(u, (float) k);
    }
    const int64_t sx = geo.s[0], sxy = (int64_t) geo.s[0] * geo.s[1];
    // the common case: along every axis the upper neighbour of node i0 is i1 and the lower one of i1 is i0, so
    // the gradients at the eight corners read the corners themselves plus 24 outer nodes (32 loads instead of
    // 48); the same values and the same operations in the same order as the general case below
    int lo0[3], hi1[3];
    float sc0[3], sc1[3];
    bool fast = true;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        if (geo.s[a] < 2) {
            fast = false;
            break;
        }
        int hi0, lo1;
        grad_stencil(i0[a], geo.s[a], geo.cyc[a], ih[a], lo0[a], hi0, sc0[a]);
        grad_stencil(i1[a], geo.s[a], geo.cyc[a], ih[a], lo1, hi1[a], sc1[a]);
        fast = fast && hi0 == i1[a] && lo1 == i0[a];
    }
    float gr[3] = {0.0f, 0.0f, 0.0f};
    if (fast) {
        const int64_t zr[2] = {i0[2] * sxy, i1[2] * sxy}, yr[2] = {i0[1] * sx, i1[1] * sx};
        const int xs[2] = {i0[0], i1[0]};
        float cv[8];
#pragma unroll
        for (int c = 0; c < 8; ++c)
            cv[c] = ld_texel<NC>(grid + zr[(c >> 2) & 1] + yr[(c >> 1) & 1] + xs[c & 1]);
#pragma unroll
        for (int c = 0; c < 8; ++c) {
            const int cx = c & 1, cy = (c >> 1) & 1, cz = (c >> 2) & 1;
            const float wx = cx ? f[0] : __fsub_rn(1.0f, f[0]);
            const float wy = cy ? f[1] : __fsub_rn(1.0f, f[1]);
            const float wz = cz ? f[2] : __fsub_rn(1.0f, f[2]);
            const float w = __fmul_rn(__fmul_rn(wx, wy), wz);
            // x: corner cx = 0 reads (lo(i0), i1), cx = 1 reads (i0, hi(i1))
            const float xlo = cx ? cv[c ^ 1] : ld_texel<NC>(grid + zr[cz] + yr[cy] + lo0[0]);
            const float xhi = cx ? ld_texel<NC>(grid + zr[cz] + yr[cy] + hi1[0]) : cv[c ^ 1];
            const float ylo = cy ? cv[c ^ 2] : ld_texel<NC>(grid + zr[cz] + lo0[1] * sx + xs[cx]);
            const float yhi = cy ? ld_texel<NC>(grid + zr[cz] + hi1[1] * sx + xs[cx]) : cv[c ^ 2];
            const float zlo = cz ? cv[c ^ 4] : ld_texel<NC>(grid + lo0[2] * sxy + yr[cy] + xs[cx]);
            const float zhi = cz ? ld_texel<NC>(grid + hi1[2] * sxy + yr[cy] + xs[cx]) : cv[c ^ 4];
            gr[0] = __fmaf_rn(w, __fmul_rn(__fsub_rn(xhi, xlo), cx ? sc1[0] : sc0[0]), gr[0]);
            gr[1] = __fmaf_rn(w, __fmul_rn(__fsub_rn(yhi, ylo), cy ? sc1[1] : sc0[1]), gr[1]);
            gr[2] = __fmaf_rn(w, __fmul_rn(__fsub_rn(zhi, zlo), cz ? sc1[2] : sc0[2]), gr[2]);
        }
    } else {
#pragma unroll
        for (int c = 0; c < 8; ++c) {
            const int x = (c & 1) ? i1[0] : i0[0], y = (c & 2) ? i1[1] : i0[1], z = (c & 4) ? i1[2] : i0[2];
            const float wx = (c & 1) ? f[0] : __fsub_rn(1.0f, f[0]);
            const float wy = (c & 2) ? f[1] : __fsub_rn(1.0f, f[1]);
            const float wz = (c & 4) ? f[2] : __fsub_rn(1.0f, f[2]);
            const float w = __fmul_rn(__fmul_rn(wx, wy), wz);
            gr[0] = __fmaf_rn(w, node_grad<NC>(grid, z * sxy + y * sx, 1, x, geo.s[0], geo.cyc[0], ih[0]), gr[0]);
            gr[1] = __fmaf_rn(w, node_grad<NC>(grid, z * sxy + x, sx, y, geo.s[1], geo.cyc[1], ih[1]), gr[1]);
            gr[2] = __fmaf_rn(w, node_grad<NC>(grid, y * sx + x, sxy, z, geo.s[2], geo.cyc[2], ih[2]), gr[2]);
        }
    }
    const float l2 = __fmaf_rn(gr[2], gr[2], __fmaf_rn(gr[1], gr[1], __fmul_rn(gr[0], gr[0])));
    float4 out = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (l2 > 0.0f && isfinite(l2)) {
        const float il = -rsqrtf(l2);
        out = make_float4(__fmul_rn(gr[0], il), __fmul_rn(gr[1], il), __fmul_rn(gr[2], il), 0.0f);
    }
    return out;
}

}  // namespace p2v
