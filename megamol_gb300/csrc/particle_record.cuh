// Per-particle record of the density gather, computed once per particle in sorted order.
//
// The reference decides a particle's cell and footprint in float (ParticlesToDensity.cpp:562-575):
// c = (int)((p - min) / sliceDist) (truncation), f = (int)ceil(r / sliceDist). Those integer decisions
// are reproduced here with the same float division. Distances, by contrast, are measured with the exact
// grid spacing: phi is the particle's position inside its floor cell in units of (right-left)/(res-1),
// accurate to ~1e-7 of a cell, so |node - p| = h * |(k - cf) - phi| keeps ~1e-7 relative accuracy where
// the reference's float node positions lose ~1e-5.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "p2v_common.cuh"

namespace p2v {

// The records live interleaved, 32 bytes per particle: A = {phi x, y, z, r} at float4 index 2 j and
// B = {floor cell x, y, z, meta} at 2 j + 1, so one particle's record fills one 32-byte sector. A pointer
// pair (rec_a, rec_b = rec_a + 1) indexed with REC_STRIDE * j addresses them.
constexpr int REC_STRIDE = 2;

struct PRecA {
    float phi[3];
    float r;
};

// meta bits: 0-7 / 8-15 / 16-23 footprint half-width per axis (clamped to 255), 24-26 trunc - floor cell
__device__ __forceinline__ float frac_in_cell(float p, float minf, float hhi, float hlo, int cf) {
    // two-sum: p - minf = ah + al exactly
    const float ah = p - minf;
    const float bb = ah - p;
    const float al = (p - (ah - bb)) + (-minf - bb);
    const float q0 = ah / hhi;
    float rem = __fmaf_rn(-q0, hhi, ah);  // remainder of the rounded quotient, exact
    rem = rem + al - q0 * hlo;
    return (q0 - static_cast<float>(cf)) + rem / hhi;
}

__device__ __forceinline__ void make_record(const float4 p, const GridGeo& g, float4& A, int4& B) {
    const float pc[3] = {p.x, p.y, p.z};
    int cf[3];
    float phi[3];
    uint32_t meta = 0;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float q = (pc[a] - g.minf[a]) / g.hf[a];
        const float qc = fminf(fmaxf(q, -1073741824.0f), 1073741824.0f);
        const int ct = static_cast<int>(qc);
        cf[a] = static_cast<int>(floorf(qc));
        phi[a] = frac_in_cell(pc[a], g.minf[a], g.hhi[a], g.hlo[a], cf[a]);
        uint32_t f = 0;
        if (g.kernel == 0)
            f = static_cast<uint32_t>(fminf(ceilf(p.w / g.hf[a]), 255.0f));
        meta |= f << (8 * a);
        meta |= static_cast<uint32_t>(ct - cf[a]) << (24 + a);
    }
    A = make_float4(phi[0], phi[1], phi[2], p.w);
    B = make_int4(cf[0], cf[1], cf[2], static_cast<int>(meta));
}

}  // namespace p2v
