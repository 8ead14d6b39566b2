// Device helpers shared by the cone march (ao.cu) and the learned AO's features (mlp.cu): the surface
// point, the MDAO cone frame and the cone directions, in explicitly rounded FP32 so that every kernel
// inlining them computes the same bits.
#pragma once

#include <cuda_runtime.h>

#include "ao_internal.h"

namespace p2v {

// Surface point x = p + r n and unit normal n of a particle; false for a zero or NaN normal.
__device__ __forceinline__ bool surface_point(const float4 p, const float4 nrm, float x[3], float n[3]) {
    const float l2 = __fmaf_rn(nrm.z, nrm.z, __fmaf_rn(nrm.y, nrm.y, __fmul_rn(nrm.x, nrm.x)));
    if (!(l2 > 0.0f))
        return false;
    const float il = rsqrtf(l2);
    n[0] = __fmul_rn(nrm.x, il);
    n[1] = __fmul_rn(nrm.y, il);
    n[2] = __fmul_rn(nrm.z, il);
    x[0] = __fmaf_rn(p.w, n[0], p.x);
    x[1] = __fmaf_rn(p.w, n[1], p.y);
    x[2] = __fmaf_rn(p.w, n[2], p.z);
    return true;
}

__device__ __forceinline__ void cross_rn(const float a[3], const float b[3], float out[3]) {
    out[0] = __fsub_rn(__fmul_rn(a[1], b[2]), __fmul_rn(a[2], b[1]));
    out[1] = __fsub_rn(__fmul_rn(a[2], b[0]), __fmul_rn(a[0], b[2]));
    out[2] = __fsub_rn(__fmul_rn(a[0], b[1]), __fmul_rn(a[1], b[0]));
}

// Cone c's direction in the particle's frame.
__device__ __forceinline__ void cone_dir(const ConeParams& cp, int c, const float ex[3], const float nn[3],
                                         const float ez[3], float dir[3]) {
    const float4 cd = cp.dirs[c];
#pragma unroll
    for (int a = 0; a < 3; ++a)
        dir[a] = __fmaf_rn(ez[a], cd.z, __fmaf_rn(nn[a], cd.y, __fmul_rn(ex[a], cd.x)));
}

// Cone frame at surface point x with unit normal nn (mdao_deferred_fragment_ambocc.inc.glsl:18-21):
// new_y = n, new_x = cross(n, normalize(objPos)), new_z = cross(new_x, new_y); and x in normalised volume
// coordinates.
__device__ __forceinline__ void cone_frame(const ConeParams& cp, const float x[3], const float nn[3], float u[3],
                                           float ex[3], float ez[3]) {
    float xn[3] = {x[0], x[1], x[2]};
    const float xl2 = __fmaf_rn(xn[2], xn[2], __fmaf_rn(xn[1], xn[1], __fmul_rn(xn[0], xn[0])));
    if (xl2 > 0.0f) {
        const float il = rsqrtf(xl2);
        xn[0] = __fmul_rn(xn[0], il);
        xn[1] = __fmul_rn(xn[1], il);
        xn[2] = __fmul_rn(xn[2], il);
    } else {
        xn[0] = 1.0f;
        xn[1] = xn[2] = 0.0f;
    }
    cross_rn(nn, xn, ex);
    cross_rn(ex, nn, ez);
    u[0] = __fmul_rn(__fsub_rn(x[0], cp.bmin[0]), cp.ibsize[0]);
    u[1] = __fmul_rn(__fsub_rn(x[1], cp.bmin[1]), cp.ibsize[1]);
    u[2] = __fmul_rn(__fsub_rn(x[2], cp.bmin[2]), cp.ibsize[2]);
}

}  // namespace p2v
