/*
 * p2v_oracle.cpp — CPU restatement of MegaMol's particle-to-volume path (TEST INFRASTRUCTURE ONLY).
 * See p2v_oracle.h for the cited reference lines and the parity status of each function.
 * Built with -ffp-contract=off so every float expression rounds exactly as written.
 */
#include "p2v_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include <omp.h>

namespace {

// Grid geometry exactly as ParticlesToDensity::createVolumeCPU derives it (ParticlesToDensity.cpp:420-432):
// origin = bbox min, range = Cuboid::Width() (|right-left|), sliceDist = range / (res-1), all in float.
struct Geo {
    int s[3];
    bool cyc[3];
    float minf[3], rangef[3], hf[3];
    double mind[3], hd[3];
};

bool make_geo(const p2vo_grid* g, Geo& o) {
    for (int a = 0; a < 3; ++a) {
        o.s[a] = g->res[a];
        if (o.s[a] < 2)
            return false;
        o.cyc[a] = g->cyclic[a] != 0;
        float lo = g->bbox[a], hi = g->bbox[a + 3];
        o.minf[a] = lo;
        o.rangef[a] = hi > lo ? hi - lo : lo - hi;
        o.hf[a] = o.rangef[a] / static_cast<float>(o.s[a] - 1);
        // Exact spacing of the same grid: the float corners are exact in double.
        o.mind[a] = static_cast<double>(lo);
        o.hd[a] = std::fabs(static_cast<double>(hi) - static_cast<double>(lo)) / static_cast<double>(o.s[a] - 1);
    }
    return true;
}

// Footprint of one particle: the reference's integer decisions, made with its float expressions
// (ParticlesToDensity.cpp:563-575). For the Gaussian the half-width covers 3*sigma*r instead of r.
struct Foot {
    int c[3], f[3];
};

inline Foot footprint(const Geo& G, const float* p, float rad, float sigma, int kernel) {
    Foot ft;
    for (int a = 0; a < 3; ++a) {
        ft.c[a] = static_cast<int>((p[a] - G.minf[a]) / G.hf[a]);
        if (kernel == P2VO_BUMP) {
            ft.f[a] = static_cast<int>(std::ceil(rad / G.hf[a]));
        } else {
            // Gaussian support 3*sigma*r; one extra node of slack so every node inside the sphere is
            // visited for particles left of the origin as well (trunc rounds toward zero there).
            float supp = 3.0f * (sigma * rad);
            ft.f[a] = static_cast<int>(std::ceil(supp / G.hf[a])) + 1;
        }
    }
    return ft;
}

// Wrap or reject one node coordinate (ParticlesToDensity.cpp:583-603). Returns -1 when skipped.
inline int wrap_node(int h, int s, bool cyc) {
    if (cyc)
        return (h + 2 * s) % s;
    return (h < 0 || h > s - 1) ? -1 : h;
}

// The reference bump rbf (ParticlesToDensity.cpp:472-476), float, written as the compiled code
// evaluates it: pow(q, 2) of a float is the correctly rounded q*q.
inline float rbf_f32(float dist, float eps) {
    if (dist >= eps)
        return 0.0f;
    float q = (1.0f / eps) * dist;
    return std::exp(-1.0f / (1.0f - q * q));
}

// Gaussian cut at 3 sigma, shifted by its value at the cut so it reaches zero continuously there:
// g(d) = exp(-d^2 / (2 s^2)) - exp(-9/2) for d < 3 s, else 0.
inline double gauss3_f64(double d2, double sg) {
    double cut2 = 9.0 * sg * sg;
    if (!(d2 < cut2))
        return 0.0;
    return std::exp(-d2 / (2.0 * sg * sg)) - std::exp(-4.5);
}

inline float gauss3_f32(float d2, float sg) {
    float cut2 = 9.0f * sg * sg;
    if (!(d2 < cut2))
        return 0.0f;
    return std::exp(-d2 / (2.0f * sg * sg)) - std::exp(-4.5f);
}

inline bool particle_valid(const float* p) {
    return std::isfinite(p[0]) && std::isfinite(p[1]) && std::isfinite(p[2]) && std::isfinite(p[3]);
}

// Static OpenMP partition as GCC's default `omp parallel for` schedule: contiguous chunks, the first
// n % T threads one longer.
inline void chunk_of(int64_t n, int T, int t, int64_t& b, int64_t& e) {
    int64_t q = n / T, r = n % T;
    b = t * q + std::min<int64_t>(t, r);
    e = b + q + (t < r ? 1 : 0);
}

template<class Acc, class Body>
void for_particles(int64_t n, int T, std::vector<std::vector<Acc>>& grids, Body body) {
    if (T <= 1) {
        for (int64_t j = 0; j < n; ++j)
            body(j, grids[0]);
        return;
    }
#pragma omp parallel num_threads(T)
    {
        int t = omp_get_thread_num();
        int64_t b, e;
        chunk_of(n, T, t, b, e);
        for (int64_t j = b; j < e; ++j)
            body(j, grids[t]);
    }
}

} // namespace

extern "C" int p2vo_density_f32(const float* xyzr, int64_t n, const p2vo_grid* g, int kernel, int nthreads, float* out) {
    Geo G;
    if (!make_geo(g, G))
        return 1;
    const int64_t V = int64_t(G.s[0]) * G.s[1] * G.s[2];
    const int T = std::max(1, nthreads);
    std::vector<std::vector<float>> grids(T, std::vector<float>(V, 0.0f));
    const float sigma = g->sigma;
    for_particles(n, T, grids, [&](int64_t j, std::vector<float>& vol) {
        const float* p = xyzr + 4 * j;
        if (!particle_valid(p))
            return;
        const float rad = p[3];
        Foot ft = footprint(G, p, rad, sigma, kernel);
        for (int hz = ft.c[2] - ft.f[2]; hz <= ft.c[2] + ft.f[2]; ++hz) {
            int wz = wrap_node(hz, G.s[2], G.cyc[2]);
            if (wz < 0)
                continue;
            for (int hy = ft.c[1] - ft.f[1]; hy <= ft.c[1] + ft.f[1]; ++hy) {
                int wy = wrap_node(hy, G.s[1], G.cyc[1]);
                if (wy < 0)
                    continue;
                for (int hx = ft.c[0] - ft.f[0]; hx <= ft.c[0] + ft.f[0]; ++hx) {
                    int wx = wrap_node(hx, G.s[0], G.cyc[0]);
                    if (wx < 0)
                        continue;
                    // ParticlesToDensity.cpp:605-614, unwrapped node position.
                    float xd = static_cast<float>(hx) * G.hf[0] + G.minf[0];
                    xd = std::fabs(xd - p[0]);
                    float yd = static_cast<float>(hy) * G.hf[1] + G.minf[1];
                    yd = std::fabs(yd - p[1]);
                    float zd = static_cast<float>(hz) * G.hf[2] + G.minf[2];
                    zd = std::fabs(zd - p[2]);
                    float d2 = xd * xd + yd * yd + zd * zd;
                    if (rad == 0.0f) // volOp returns early (ParticlesToDensity.cpp:523-524)
                        continue;
                    float v = kernel == P2VO_BUMP ? rbf_f32(std::sqrt(d2), sigma * rad) : gauss3_f32(d2, sigma * rad);
                    vol[wx + (wy + int64_t(wz) * G.s[1]) * G.s[0]] += v;
                }
            }
        }
    });
    // Serial reduction of the thread grids (ParticlesToDensity.cpp:623-626).
    for (int t = 1; t < T; ++t)
        for (int64_t i = 0; i < V; ++i)
            grids[0][i] = grids[t][i] + grids[0][i];
    std::memcpy(out, grids[0].data(), V * sizeof(float));
    return 0;
}

extern "C" int p2vo_density_f64(const float* xyzr, int64_t n, const p2vo_grid* g, int kernel, int nthreads, double* out) {
    Geo G;
    if (!make_geo(g, G))
        return 1;
    const int64_t V = int64_t(G.s[0]) * G.s[1] * G.s[2];
    const int T = std::max(1, nthreads);
    std::vector<std::vector<double>> grids(T, std::vector<double>(V, 0.0));
    const float sigma = g->sigma;
    for_particles(n, T, grids, [&](int64_t j, std::vector<double>& vol) {
        const float* p = xyzr + 4 * j;
        if (!particle_valid(p))
            return;
        const float rad = p[3];
        if (rad == 0.0f)
            return;
        Foot ft = footprint(G, p, rad, sigma, kernel);
        const double eps = static_cast<double>(sigma) * static_cast<double>(rad);
        for (int hz = ft.c[2] - ft.f[2]; hz <= ft.c[2] + ft.f[2]; ++hz) {
            int wz = wrap_node(hz, G.s[2], G.cyc[2]);
            if (wz < 0)
                continue;
            double dz = G.mind[2] + hz * G.hd[2] - static_cast<double>(p[2]);
            for (int hy = ft.c[1] - ft.f[1]; hy <= ft.c[1] + ft.f[1]; ++hy) {
                int wy = wrap_node(hy, G.s[1], G.cyc[1]);
                if (wy < 0)
                    continue;
                double dy = G.mind[1] + hy * G.hd[1] - static_cast<double>(p[1]);
                for (int hx = ft.c[0] - ft.f[0]; hx <= ft.c[0] + ft.f[0]; ++hx) {
                    int wx = wrap_node(hx, G.s[0], G.cyc[0]);
                    if (wx < 0)
                        continue;
                    double dx = G.mind[0] + hx * G.hd[0] - static_cast<double>(p[0]);
                    double d2 = dx * dx + dy * dy + dz * dz;
                    double v;
                    if (kernel == P2VO_BUMP) {
                        double q2 = d2 / (eps * eps);
                        v = q2 < 1.0 ? std::exp(-1.0 / (1.0 - q2)) : 0.0;
                    } else {
                        v = gauss3_f64(d2, eps);
                    }
                    vol[wx + (wy + int64_t(wz) * G.s[1]) * G.s[0]] += v;
                }
            }
        }
    });
    for (int t = 1; t < T; ++t)
        for (int64_t i = 0; i < V; ++i)
            grids[0][i] += grids[t][i];
    std::memcpy(out, grids[0].data(), V * sizeof(double));
    return 0;
}

// ParticlesToDensity.cpp:669-682: min/max over the grid, then (v - min) * (1 / (max - min)) in float.
extern "C" void p2vo_normalize_minmax_f32(float* v, int64_t n, int apply, float* out_min, float* out_max) {
    float mx = -INFINITY, mn = INFINITY;
    if (n > 0) {
        mx = *std::max_element(v, v + n);
        mn = *std::min_element(v, v + n);
    }
    *out_min = mn;
    *out_max = mx;
    if (apply) {
        const float rcp = 1.0f / (mx - mn);
        for (int64_t i = 0; i < n; ++i)
            v[i] = (v[i] - mn) * rcp;
    }
}

/* ------------------------------------------------------------------------------------------------
 * MDAO mip step (mdao_mipmap_compute_main.comp.glsl:8-26): every output voxel sums the children at
 * 2*gid .. min(2*gid+1, inputSize-1) and divides by 8, whatever the child count.
 * ---------------------------------------------------------------------------------------------- */
extern "C" void p2vo_mip_step_f64(const double* src, const int32_t sd[3], double* dst, const int32_t dd[3]) {
    for (int z = 0; z < dd[2]; ++z)
        for (int y = 0; y < dd[1]; ++y)
            for (int x = 0; x < dd[0]; ++x) {
                double acc = 0.0;
                int x1 = std::min(2 * x + 1, sd[0] - 1), y1 = std::min(2 * y + 1, sd[1] - 1),
                    z1 = std::min(2 * z + 1, sd[2] - 1);
                for (int xx = 2 * x; xx <= x1; ++xx)
                    for (int yy = 2 * y; yy <= y1; ++yy)
                        for (int zz = 2 * z; zz <= z1; ++zz)
                            acc += src[xx + (yy + int64_t(zz) * sd[1]) * sd[0]];
                dst[x + (y + int64_t(z) * dd[1]) * dd[0]] = acc / 8.0;
            }
}
