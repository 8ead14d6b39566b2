/*
 * p2v_oracle.cpp — CPU restatement of MegaMol's particle-to-volume path (TEST INFRASTRUCTURE ONLY).
 * See p2v_oracle.h for the cited reference lines and the parity status of each function.
 * Built with -ffp-contract=off so every float expression rounds exactly as written.
 */
#include "p2v_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
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

// FP32 createVolumeCPU (ParticlesToDensity.cpp:389-626): with w == nullptr the density (aggregator 0,
// volOp :520-528); with nc weights per particle the intensity (nc = 1, :509-519) or one direction component
// per pass of the vector aggregator (:492-508): vol += rbf(dis, sigma * rad) * val, in float.
static int density_f32_impl(const float* xyzr, const float* w, int nc, int64_t n, const p2vo_grid* g, int kernel,
                            int nthreads, float* out) {
    Geo G;
    if (!make_geo(g, G))
        return 1;
    const int64_t V = int64_t(G.s[0]) * G.s[1] * G.s[2];
    const int T = std::max(1, nthreads);
    std::vector<std::vector<float>> grids(T, std::vector<float>(V * nc, 0.0f));
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
                    const int64_t idx = wx + (wy + int64_t(wz) * G.s[1]) * G.s[0];
                    if (!w)
                        vol[idx] += v;
                    else
                        for (int c = 0; c < nc; ++c)
                            vol[idx * nc + c] += v * w[j * nc + c];
                }
            }
        }
    });
    // Serial reduction of the thread grids (ParticlesToDensity.cpp:623-626).
    for (int t = 1; t < T; ++t)
        for (int64_t i = 0; i < V * nc; ++i)
            grids[0][i] = grids[t][i] + grids[0][i];
    std::memcpy(out, grids[0].data(), V * nc * sizeof(float));
    return 0;
}

extern "C" int p2vo_density_f32(const float* xyzr, int64_t n, const p2vo_grid* g, int kernel, int nthreads, float* out) {
    return density_f32_impl(xyzr, nullptr, 1, n, g, kernel, nthreads, out);
}

extern "C" int p2vo_density_weighted_f32(const float* xyzr, const float* w, int nc, int64_t n, const p2vo_grid* g,
                                         int kernel, int nthreads, float* out) {
    return density_f32_impl(xyzr, w, nc, n, g, kernel, nthreads, out);
}

static int density_f64_impl(const float* xyzr, const float* w, int nc, int64_t n, const p2vo_grid* g, int kernel,
                            int nthreads, double* out) {
    Geo G;
    if (!make_geo(g, G))
        return 1;
    const int64_t V = int64_t(G.s[0]) * G.s[1] * G.s[2];
    const int T = std::max(1, nthreads);
    std::vector<std::vector<double>> grids(T, std::vector<double>(V * nc, 0.0));
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
                    const int64_t idx = wx + (wy + int64_t(wz) * G.s[1]) * G.s[0];
                    if (!w)
                        vol[idx] += v;
                    else
                        for (int c = 0; c < nc; ++c)
                            vol[idx * nc + c] += v * static_cast<double>(w[j * nc + c]);
                }
            }
        }
    });
    for (int t = 1; t < T; ++t)
        for (int64_t i = 0; i < V * nc; ++i)
            grids[0][i] += grids[t][i];
    std::memcpy(out, grids[0].data(), V * nc * sizeof(double));
    return 0;
}

extern "C" int p2vo_density_f64(const float* xyzr, int64_t n, const p2vo_grid* g, int kernel, int nthreads, double* out) {
    return density_f64_impl(xyzr, nullptr, 1, n, g, kernel, nthreads, out);
}

extern "C" int p2vo_density_weighted_f64(const float* xyzr, const float* w, int nc, int64_t n, const p2vo_grid* g,
                                         int kernel, int nthreads, double* out) {
    return density_f64_impl(xyzr, w, nc, n, g, kernel, nthreads, out);
}

// The vector aggregator's finish (ParticlesToDensity.cpp:628-682), float as the reference: every voxel's
// direction sum divided by its weight sum (1 where that is 0), density = |v|, min / max over the densities
// (max starting at 0), then with `normalize` all three components mapped by (a - min) * (1 / (max - min)).
extern "C" void p2vo_vector_finish_f32(float* vol3, const float* weights, int64_t V, int normalize, float* out_min,
                                       float* out_max) {
    float maxD = 0.0f, minD = std::numeric_limits<float>::max();
    for (int64_t i = 0; i < V; ++i) {
        const float wv = weights[i] == 0.0f ? 1.0f : weights[i];
        vol3[i * 3 + 0] /= wv;
        vol3[i * 3 + 1] /= wv;
        vol3[i * 3 + 2] /= wv;
        const float d = std::sqrt(vol3[i * 3 + 0] * vol3[i * 3 + 0] + vol3[i * 3 + 1] * vol3[i * 3 + 1] +
                                  vol3[i * 3 + 2] * vol3[i * 3 + 2]);
        maxD = std::max(maxD, d);
        minD = std::min(minD, d);
    }
    *out_min = minD;
    *out_max = maxD;
    if (normalize) {
        const float rcp = 1.0f / (maxD - minD);
        for (int64_t i = 0; i < 3 * V; ++i)
            vol3[i] = (vol3[i] - minD) * rcp;
    }
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

/* ------------------------------------------------------------------------------------------------
 * AO restatements
 * ---------------------------------------------------------------------------------------------- */
namespace {

struct Vol {
    const double* v;
    int d[3];
};

// Texel fetch with GL wrap semantics: border (0 outside) or edge (clamped index).
inline double fetch(const Vol& L, int x, int y, int z, int border) {
    if (border == 0) {
        if (x < 0 || y < 0 || z < 0 || x >= L.d[0] || y >= L.d[1] || z >= L.d[2])
            return 0.0;
    } else {
        x = std::min(std::max(x, 0), L.d[0] - 1);
        y = std::min(std::max(y, 0), L.d[1] - 1);
        z = std::min(std::max(z, 0), L.d[2] - 1);
    }
    return L.v[x + (y + int64_t(z) * L.d[1]) * L.d[0]];
}

// GL LINEAR filtering at normalised coordinate u: texel centres at (i + 0.5) / N.
inline double trilinear(const Vol& L, const double u[3], int border) {
    double c[3], f[3];
    int i0[3];
    for (int a = 0; a < 3; ++a) {
        c[a] = u[a] * L.d[a] - 0.5;
        i0[a] = (int) std::floor(c[a]);
        f[a] = c[a] - i0[a];
    }
    double acc = 0.0;
    for (int dz = 0; dz < 2; ++dz)
        for (int dy = 0; dy < 2; ++dy)
            for (int dx = 0; dx < 2; ++dx) {
                double w = (dx ? f[0] : 1 - f[0]) * (dy ? f[1] : 1 - f[1]) * (dz ? f[2] : 1 - f[2]);
                if (w != 0.0)
                    acc += w * fetch(L, i0[0] + dx, i0[1] + dy, i0[2] + dz, border);
            }
    return acc;
}

inline void normalize3(double v[3]) {
    double l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    v[0] /= l;
    v[1] /= l;
    v[2] /= l;
}

inline void cross3(const double a[3], const double b[3], double o[3]) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}

}  // namespace

extern "C" void p2vo_cone_dirs(int K, float apex, float* out) {
    // SphereRenderer.cpp:2572-2587 for K = 3; a regular K-gon ring of the same edge length otherwise.
    const float edge = 2.0f * std::tan(0.5f * apex);
    const float height = std::sqrt(1.0f - edge * edge / 12.0f);
    const float radius = K == 3 ? std::sqrt(3.0f) / 3.0f * edge : edge / (2.0f * std::sin(3.14159265358979f / K));
    for (int i = 0; i < K; ++i) {
        const float angle = static_cast<float>(i) / static_cast<float>(K) * 2.0f * 3.14159265358979f;
        float c[3] = {std::cos(angle) * radius, height, std::sin(angle) * radius};
        const float l = std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
        out[4 * i + 0] = c[0] / l;
        out[4 * i + 1] = c[1] / l;
        out[4 * i + 2] = c[2] / l;
        out[4 * i + 3] = edge;
    }
}

extern "C" int p2vo_cone_steps(const p2vo_cone_params* cp, float w, float* t, float* lod, int cap) {
    int n = 0;
    float tt = cp->offset + 0.0001f;
    float g = 0.0f;
    if (cp->steps > 0)
        g = std::pow(cp->cone_length / tt, 1.0f / static_cast<float>(cp->steps));
    while (n < cap) {
        float l = std::log2(tt * w * cp->shortest_edge);
        l = std::min(std::max(l, 0.0f), cp->max_lod);
        t[n] = tt;
        lod[n] = l;
        ++n;
        if (cp->steps > 0) {
            if (n >= cp->steps)
                break;
            tt = tt * g;
        } else {
            tt += tt * w;  // mdao_deferred_fragment_ambocc.inc.glsl:50
            if (!(tt < cp->cone_length))
                break;
        }
    }
    return n;
}

extern "C" void p2vo_cone_ao_f64(const double* const* levels, const int32_t* ldims, int nlevels, const float* dirs,
    int ncones, const p2vo_cone_params* cp, const float* xyzr, const float* nrm, int64_t n, double* ao) {
    std::vector<Vol> L(nlevels);
    for (int l = 0; l < nlevels; ++l)
        L[l] = Vol{levels[l], {ldims[3 * l], ldims[3 * l + 1], ldims[3 * l + 2]}};
    std::vector<double> sat0;
    if (cp->sat_scale > 0.0f) {  // the level-0 texture holds clamp(v * scale, 0, 1)
        const int64_t nv = int64_t(L[0].d[0]) * L[0].d[1] * L[0].d[2];
        sat0.resize(nv);
        for (int64_t i = 0; i < nv; ++i)
            sat0[i] = std::min(1.0, std::max(0.0, L[0].v[i] * (double) cp->sat_scale));
        L[0].v = sat0.data();
    }
    std::vector<float> ts(256), lods(256);
    const int ns = p2vo_cone_steps(cp, dirs[3], ts.data(), lods.data(), 256);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        const float* p = xyzr + 4 * i;
        double nn[3] = {nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]};
        const double nl = std::sqrt(nn[0] * nn[0] + nn[1] * nn[1] + nn[2] * nn[2]);
        if (!(nl > 0.0)) {
            ao[i] = 1.0;  // no normal: no occlusion
            continue;
        }
        for (double& c : nn)
            c /= nl;
        // evaluation point on the sphere surface along the normal
        double x[3] = {p[0] + p[3] * nn[0], p[1] + p[3] * nn[1], p[2] + p[3] * nn[2]};
        // frame: new_y = n, new_x = cross(new_y, normalize(objPos)), new_z = cross(new_x, new_y) (:18-21)
        double xn[3] = {x[0], x[1], x[2]};
        const double xl = std::sqrt(xn[0] * xn[0] + xn[1] * xn[1] + xn[2] * xn[2]);
        if (xl > 0.0) {
            for (double& c : xn)
                c /= xl;
        } else {
            xn[0] = 1.0;
            xn[1] = xn[2] = 0.0;
        }
        double ex[3], ez[3];
        cross3(nn, xn, ex);
        cross3(ex, nn, ez);
        double u[3];
        for (int a = 0; a < 3; ++a)
            u[a] = (x[a] - (double) cp->bounds_min[a]) / (double) cp->bounds_size[a];
        double ambient = 0.0;
        for (int c = 0; c < ncones; ++c) {
            const float* cd = dirs + 4 * c;
            double dir[3];
            for (int a = 0; a < 3; ++a)
                dir[a] = ex[a] * cd[0] + nn[a] * cd[1] + ez[a] * cd[2];
            double acc = 0.0;
            for (int k = 0; k < ns; ++k) {
                const double t = ts[k];
                const double lod = lods[k];
                double q[3] = {u[0] + t * dir[0], u[1] + t * dir[1], u[2] + t * dir[2]};
                const int l0 = (int) std::floor(lod);
                const double fr = lod - l0;
                double vis = trilinear(L[std::min(l0, nlevels - 1)], q, cp->border);
                if (fr > 0.0 && l0 + 1 < nlevels)
                    vis = (1.0 - fr) * vis + fr * trilinear(L[l0 + 1], q, cp->border);
                acc += (1.0 - acc) * vis;
                if (cp->early_exit && acc > 0.99)
                    break;
            }
            ambient += acc;
        }
        ao[i] = 1.0 - std::min(1.0, std::max(0.0, (double) cp->strength * ambient / ncones));
    }
}

/* ------------------------------------------------------------------------------------------------
 * FP32 cone pipeline (the CPU baseline's timing stand-in for the GLSL march, OpenMP): the MDAO pyramid
 * of a float volume (level 1 built from the saturated texels clamp(v * scale, 0, 1)) and the march in
 * FP32 with the GPU kernel's operation order (fused multiply-adds where it fuses, level 0 saturated on
 * the fly). The error reference stays the FP64 march above.
 * ---------------------------------------------------------------------------------------------- */
extern "C" void p2vo_mip_levels_f32(const float* l0, const int32_t d0[3], float sat_scale, int nlevels,
                                    float* const* out, int nthreads) {
    int sd[3] = {d0[0], d0[1], d0[2]};
    const float* src = l0;
    for (int l = 1; l < nlevels; ++l) {
        const int dd[3] = {std::max(1, sd[0] / 2), std::max(1, sd[1] / 2), std::max(1, sd[2] / 2)};
        float* dst = out[l - 1];
        const bool sat = l == 1 && sat_scale > 0.0f;
#pragma omp parallel for schedule(static) num_threads(nthreads)
        for (int z = 0; z < dd[2]; ++z)
            for (int y = 0; y < dd[1]; ++y)
                for (int x = 0; x < dd[0]; ++x) {
                    float acc = 0.0f;
                    const int x1 = std::min(2 * x + 1, sd[0] - 1), y1 = std::min(2 * y + 1, sd[1] - 1),
                              z1 = std::min(2 * z + 1, sd[2] - 1);
                    for (int zz = 2 * z; zz <= z1; ++zz)
                        for (int yy = 2 * y; yy <= y1; ++yy)
                            for (int xx = 2 * x; xx <= x1; ++xx) {
                                float v = src[xx + (yy + int64_t(zz) * sd[1]) * sd[0]];
                                if (sat)
                                    v = std::min(std::max(v * sat_scale, 0.0f), 1.0f);
                                acc += v;
                            }
                    dst[x + (y + int64_t(z) * dd[1]) * dd[0]] = acc * 0.125f;
                }
        src = dst;
        for (int a = 0; a < 3; ++a)
            sd[a] = dd[a];
    }
}

namespace {

struct VolF {
    const float* v;
    int d[3];
    float fd[3];
};

inline float fetch_f32(const VolF& L, int x, int y, int z, float sat) {
    if (x < 0 || y < 0 || z < 0 || x >= L.d[0] || y >= L.d[1] || z >= L.d[2])
        return 0.0f;  // CLAMP_TO_BORDER
    const float v = L.v[x + (y + int64_t(z) * L.d[1]) * L.d[0]];
    return sat > 0.0f ? std::min(std::max(v * sat, 0.0f), 1.0f) : v;
}

inline float lerp_f32(float a, float b, float w) {
    return std::fma(w, b - a, a);
}

inline float trilinear_f32(const VolF& L, float ux, float uy, float uz, float sat) {
    const float cx = std::fma(ux, L.fd[0], -0.5f), cy = std::fma(uy, L.fd[1], -0.5f), cz = std::fma(uz, L.fd[2], -0.5f);
    const float fx0 = std::floor(cx), fy0 = std::floor(cy), fz0 = std::floor(cz);
    const int x0 = (int) fx0, y0 = (int) fy0, z0 = (int) fz0;
    const float fx = cx - fx0, fy = cy - fy0, fz = cz - fz0;
    const float c00 = lerp_f32(fetch_f32(L, x0, y0, z0, sat), fetch_f32(L, x0 + 1, y0, z0, sat), fx);
    const float c10 = lerp_f32(fetch_f32(L, x0, y0 + 1, z0, sat), fetch_f32(L, x0 + 1, y0 + 1, z0, sat), fx);
    const float c01 = lerp_f32(fetch_f32(L, x0, y0, z0 + 1, sat), fetch_f32(L, x0 + 1, y0, z0 + 1, sat), fx);
    const float c11 = lerp_f32(fetch_f32(L, x0, y0 + 1, z0 + 1, sat), fetch_f32(L, x0 + 1, y0 + 1, z0 + 1, sat), fx);
    return lerp_f32(lerp_f32(c00, c10, fy), lerp_f32(c01, c11, fy), fz);
}

inline void cross_f32(const float a[3], const float b[3], float o[3]) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}

}  // namespace

extern "C" void p2vo_cone_ao_f32(const float* const* levels, const int32_t* ldims, int nlevels, const float* dirs,
    int ncones, const p2vo_cone_params* cp, const float* xyzr, const float* nrm, int64_t n, int nthreads, float* ao) {
    std::vector<VolF> L(nlevels);
    for (int l = 0; l < nlevels; ++l) {
        L[l].v = levels[l];
        for (int a = 0; a < 3; ++a) {
            L[l].d[a] = ldims[3 * l + a];
            L[l].fd[a] = (float) ldims[3 * l + a];
        }
    }
    std::vector<float> ts(256), lods(256);
    const int ns = p2vo_cone_steps(cp, dirs[3], ts.data(), lods.data(), 256);
    float bmin[3], ibs[3];
    for (int a = 0; a < 3; ++a) {
        bmin[a] = cp->bounds_min[a];
        ibs[a] = (float) (1.0 / (double) cp->bounds_size[a]);
    }
#pragma omp parallel for schedule(dynamic, 256) num_threads(nthreads)
    for (int64_t i = 0; i < n; ++i) {
        const float* p = xyzr + 4 * i;
        const float* nv = nrm + 3 * i;
        const float l2 = std::fma(nv[2], nv[2], std::fma(nv[1], nv[1], nv[0] * nv[0]));
        if (!(l2 > 0.0f)) {
            ao[i] = 1.0f;  // no normal: no occlusion
            continue;
        }
        const float il = 1.0f / std::sqrt(l2);
        const float nn[3] = {nv[0] * il, nv[1] * il, nv[2] * il};
        const float x[3] = {std::fma(p[3], nn[0], p[0]), std::fma(p[3], nn[1], p[1]), std::fma(p[3], nn[2], p[2])};
        float xn[3] = {x[0], x[1], x[2]};
        const float xl2 = std::fma(xn[2], xn[2], std::fma(xn[1], xn[1], xn[0] * xn[0]));
        if (xl2 > 0.0f) {
            const float ixl = 1.0f / std::sqrt(xl2);
            for (float& c : xn)
                c *= ixl;
        } else {
            xn[0] = 1.0f;
            xn[1] = xn[2] = 0.0f;
        }
        float ex[3], ez[3];
        cross_f32(nn, xn, ex);
        cross_f32(ex, nn, ez);
        const float u[3] = {(x[0] - bmin[0]) * ibs[0], (x[1] - bmin[1]) * ibs[1], (x[2] - bmin[2]) * ibs[2]};
        float ambient = 0.0f;
        for (int c = 0; c < ncones; ++c) {
            const float* cd = dirs + 4 * c;
            float dir[3];
            for (int a = 0; a < 3; ++a)
                dir[a] = std::fma(ez[a], cd[2], std::fma(nn[a], cd[1], ex[a] * cd[0]));
            float acc = 0.0f;
            for (int k = 0; k < ns; ++k) {
                const float t = ts[k], lod = lods[k];
                const float qx = std::fma(t, dir[0], u[0]), qy = std::fma(t, dir[1], u[1]), qz = std::fma(t, dir[2], u[2]);
                const int l0 = std::min((int) lod, nlevels - 1);
                const float fr = lod - (float) l0;
                float vis = trilinear_f32(L[l0], qx, qy, qz, l0 == 0 ? cp->sat_scale : 0.0f);
                if (fr > 0.0f && l0 + 1 < nlevels)
                    vis = std::fma(fr, trilinear_f32(L[l0 + 1], qx, qy, qz, 0.0f), (1.0f - fr) * vis);
                acc = std::fma(1.0f - acc, vis, acc);
                if (cp->early_exit && acc > 0.99f)
                    break;
            }
            ambient += acc;
        }
        ao[i] = 1.0f - std::min(std::max(cp->strength * ambient / (float) ncones, 0.0f), 1.0f);
    }
}

/* ------------------------------------------------------------------------------------------------
 * Normals down the density gradient (the library's P2V_NORMALS_GRADIENT, restated in FP32 with OpenMP):
 * -grad(rho) at each particle from the node grid's central differences (periodic along cyclic axes,
 * one-sided first differences at the faces of open ones), trilinear at u = (p - min) / h clamped into the
 * node range, normalised; zero where the gradient vanishes.
 * ---------------------------------------------------------------------------------------------- */
namespace {
inline float node_grad_f32(const float* g, int64_t base, int64_t stride, int i, int s, int cyc, float ih) {
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
    return (g[base + hi * stride] - g[base + lo * stride]) * scale;
}
}  // namespace

extern "C" void p2vo_gradient_normals_f32(const float* grid, const int32_t res[3], const int32_t cyc[3],
    const float minf[3], const float h[3], const float* xyzr, int64_t n, int nthreads, float* out3) {
#pragma omp parallel for schedule(static) num_threads(nthreads)
    for (int64_t j = 0; j < n; ++j) {
        const float* p = xyzr + 4 * j;
        int i0[3], i1[3];
        float f[3], ih[3];
        for (int a = 0; a < 3; ++a) {
            ih[a] = 1.0f / h[a];
            float u = (p[a] - minf[a]) * ih[a];
            u = std::min(std::max(u, 0.0f), (float) (res[a] - 1));
            if (!(u == u))
                u = 0.0f;
            const int k = std::min((int) u, res[a] - 1);
            i0[a] = k;
            i1[a] = std::min(k + 1, res[a] - 1);
            f[a] = u - (float) k;
        }
        const int64_t sx = res[0], sxy = (int64_t) res[0] * res[1];
        float gr[3] = {0.0f, 0.0f, 0.0f};
        for (int c = 0; c < 8; ++c) {
            const int x = (c & 1) ? i1[0] : i0[0], y = (c & 2) ? i1[1] : i0[1], z = (c & 4) ? i1[2] : i0[2];
            const float w = ((c & 1) ? f[0] : 1.0f - f[0]) * ((c & 2) ? f[1] : 1.0f - f[1]) * ((c & 4) ? f[2] : 1.0f - f[2]);
            gr[0] += w * node_grad_f32(grid, z * sxy + y * sx, 1, x, res[0], cyc[0], ih[0]);
            gr[1] += w * node_grad_f32(grid, z * sxy + x, sx, y, res[1], cyc[1], ih[1]);
            gr[2] += w * node_grad_f32(grid, y * sx + x, sxy, z, res[2], cyc[2], ih[2]);
        }
        const float l2 = gr[0] * gr[0] + gr[1] * gr[1] + gr[2] * gr[2];
        float* o = out3 + 3 * j;
        if (l2 > 0.0f && std::isfinite(l2)) {
            const float il = -1.0f / std::sqrt(l2);
            o[0] = gr[0] * il;
            o[1] = gr[1] * il;
            o[2] = gr[2] * il;
        } else {
            o[0] = o[1] = o[2] = 0.0f;
        }
    }
}

extern "C" void p2vo_aosphere_volume_ex_f64(const float* xyzr, int64_t n, const float clip[6], const int32_t s[3],
    float gen_fac, int glsl_rule, int use_clip, const float plane[4], double* tex) {
    // AOSphereRenderer.cpp:918-1021 (CPU rule) and :1026-1221 with volume_updateVolume.vert.glsl:22-46 (GLSL
    // rule): inner grid s-2, every voxel decision in float as the reference makes it
    const int sx = s[0] - 2, sy = s[1] - 2, sz = s[2] - 2;
    const float minOS[3] = {clip[0], clip[1], clip[2]};
    const float rangeOS[3] = {std::fabs(clip[3] - clip[0]), std::fabs(clip[4] - clip[1]), std::fabs(clip[5] - clip[2])};
    const int si[3] = {sx, sy, sz};
    const double voxelVol = ((double) rangeOS[0] / sx) * ((double) rangeOS[1] / sy) * ((double) rangeOS[2] / sz);
    std::memset(tex, 0, sizeof(double) * (size_t) s[0] * s[1] * s[2]);
    for (int64_t i = 0; i < n; ++i) {
        const float* p = xyzr + 4 * i;
        int c[3];
        if (!glsl_rule) {
            for (int a = 0; a < 3; ++a) {
                int v = static_cast<int>(((p[a] - minOS[a]) / rangeOS[a]) * static_cast<float>(si[a]));
                c[a] = (v < 0 ? 0 : (v >= si[a] ? si[a] - 1 : v)) + 1;
            }
            if (use_clip) {  // :982-991, vislib's Dot as a running float sum
                float od = 0.0f;
                for (int a = 0; a < 3; ++a)
                    od += p[a] * plane[a];
                if (od - plane[3] >= 0.0f)
                    continue;
            }
        } else {
            for (int a = 0; a < 2; ++a) {
                const float q = std::floor(((p[a] - minOS[a]) / rangeOS[a]) * static_cast<float>(si[a]));
                c[a] = (int) std::min(std::max(q, 0.0f), (float) si[a]);
            }
            int vz = static_cast<int>(((p[2] - minOS[2]) / rangeOS[2]) * static_cast<float>(sz));
            c[2] = std::max(0, std::min(vz, sz - 1)) + 1;
        }
        const double r = p[3];
        const double spVol = 4.0 / 3.0 * 3.14159265358979323846 * r * r * r;
        tex[c[0] + (c[1] + int64_t(c[2]) * s[1]) * s[0]] += spVol / voxelVol * gen_fac;
    }
}

extern "C" void p2vo_aosphere_volume_f64(const float* xyzr, int64_t n, const float clip[6], const int32_t s[3],
    float gen_fac, double* tex) {
    p2vo_aosphere_volume_ex_f64(xyzr, n, clip, s, gen_fac, 0, 0, nullptr, tex);
}

extern "C" void p2vo_aosphere_ao_f64(const double* tex, const int32_t s[3], const float clip[6], float step_len,
    float eval_fac, const float* xyzr, const float* nrm, int64_t n, int mode, double* ao) {
    // uniforms of AOSphereRenderer::renderParticles (AOSphereRenderer.cpp:489-514)
    double origin[3], ext[3], sampd[3];
    for (int a = 0; a < 3; ++a) {
        const double range = std::fabs((double) clip[a + 3] - (double) clip[a]);
        ext[a] = range / (1.0 - 2.0 / s[a]);
        origin[a] = (double) clip[a] - ext[a] / s[a];
        sampd[a] = (double) step_len * (range / s[a]);
    }
    Vol T{tex, {s[0], s[1], s[2]}};
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        const float* p = xyzr + 4 * i;
        double nn[3] = {nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]};
        const double nl = std::sqrt(nn[0] * nn[0] + nn[1] * nn[1] + nn[2] * nn[2]);
        if (!(nl > 0.0)) {
            ao[i] = 1.0;
            continue;
        }
        for (double& c : nn)
            c /= nl;
        if (mode == 0) {
            // mainaxes_vertex_2.glsl:1-9 and mainaxes_fragLightAO_evalAO.glsl:1-8
            double aop[3], aod[3];
            for (int a = 0; a < 3; ++a) {
                aop[a] = (p[a] - origin[a]) / ext[a];
                aod[a] = ((double) p[3] + sampd[a]) / ext[a];
            }
            double acc = 0.0;
            for (int a = 0; a < 3; ++a) {
                double q[3] = {aop[0], aop[1], aop[2]};
                q[a] += nn[a] > 0.0 ? aod[a] : -aod[a];
                const double tap = 1.0 - trilinear(T, q, 1) * eval_fac;
                acc += nn[a] * nn[a] * tap;
            }
            ao[i] = acc;
        } else {
            // normals_fragLightAO_evalAO.glsl:1-4 at the surface point p + r n
            double q[3];
            for (int a = 0; a < 3; ++a)
                q[a] = ((p[a] + p[3] * nn[a]) + nn[a] * sampd[a] - origin[a]) / ext[a];
            ao[i] = 1.0 - trilinear(T, q, 1) * eval_fac;
        }
    }
}

/* ------------------------------------------------------------------------------------------------
 * Learned-AO MLP, FP64 forward and backward (the check of the GPU training kernels)
 * ---------------------------------------------------------------------------------------------- */
extern "C" void p2vo_mlp_f64(const double* P, const float* x, const float* t, int64_t n, double* grads, double* loss,
    double* y) {
    const int IN = 54, H = 64;
    const double* W1 = P;
    const double* b1 = W1 + H * IN;
    const double* W2 = b1 + H;
    const double* b2 = W2 + H * H;
    const double* w3 = b2 + H;
    const double b3 = w3[H];
    const int64_t np = (int64_t) H * IN + H + H * H + H + H + 1;
    std::vector<double> g(grads ? np : 0, 0.0);
    double L = 0.0;
    std::vector<double> a1(H), h1(H), a2(H), h2(H), dh2(H), da2(H), dh1(H), da1(H);
    auto sig = [](double v) { return 1.0 / (1.0 + std::exp(-v)); };
    for (int64_t s = 0; s < n; ++s) {
        const float* xs = x + s * IN;
        for (int j = 0; j < H; ++j) {
            double acc = b1[j];
            for (int i = 0; i < IN; ++i)
                acc += W1[j * IN + i] * xs[i];
            a1[j] = acc;
            h1[j] = acc * sig(acc);
        }
        for (int j = 0; j < H; ++j) {
            double acc = b2[j];
            for (int i = 0; i < H; ++i)
                acc += W2[j * H + i] * h1[i];
            a2[j] = acc;
            h2[j] = acc * sig(acc);
        }
        double z = b3;
        for (int j = 0; j < H; ++j)
            z += w3[j] * h2[j];
        const double ys = sig(z);
        if (y)
            y[s] = ys;
        const double e = ys - (t ? t[s] : 0.0);
        L += e * e;
        if (!grads)
            continue;
        const double dz = 2.0 * e / n * ys * (1.0 - ys);
        double* gW1 = g.data();
        double* gb1 = gW1 + H * IN;
        double* gW2 = gb1 + H;
        double* gb2 = gW2 + H * H;
        double* gw3 = gb2 + H;
        for (int j = 0; j < H; ++j) {
            gw3[j] += dz * h2[j];
            dh2[j] = dz * w3[j];
            const double sg = sig(a2[j]);
            da2[j] = dh2[j] * sg * (1.0 + a2[j] * (1.0 - sg));
            gb2[j] += da2[j];
            for (int i = 0; i < H; ++i)
                gW2[j * H + i] += da2[j] * h1[i];
        }
        gw3[H] += dz;
        for (int i = 0; i < H; ++i) {
            double acc = 0.0;
            for (int j = 0; j < H; ++j)
                acc += da2[j] * W2[j * H + i];
            dh1[i] = acc;
            const double sg = sig(a1[i]);
            da1[i] = acc * sg * (1.0 + a1[i] * (1.0 - sg));
            gb1[i] += da1[i];
            for (int k = 0; k < IN; ++k)
                gW1[i * IN + k] += da1[i] * xs[k];
        }
    }
    if (loss)
        *loss = n ? L / n : 0.0;
    if (grads)
        std::memcpy(grads, g.data(), sizeof(double) * np);
}

/* ------------------------------------------------------------------------------------------------
 * MDAO occupancy volume. FP32 throughout, in the shaders' operation order, compiled without fused
 * multiply-adds, so the GPU voxeliser (which uses explicitly rounded operations) matches it bit for bit.
 * ---------------------------------------------------------------------------------------------- */
extern "C" void p2vo_mdao_dims(const float clip[6], int vol_size, int32_t dims[3], float* shortest, float* max_lod) {
    // SphereRenderer.cpp:2463-2476; Cuboid::Width/Height/Depth are absolute edge lengths and
    // Dimension::Scale multiplies in double (AbstractDimensionImpl.h:183-187)
    float size[3];
    for (int a = 0; a < 3; ++a)
        size[a] = clip[a + 3] > clip[a] ? clip[a + 3] - clip[a] : clip[a] - clip[a + 3];
    const float w = size[0], h = size[1], d = size[2];
    const float longest = ((w > h) && (w > d)) ? w : ((h > d) ? h : d);  // AbstractCuboid.h:412-417
    const double f = static_cast<double>(static_cast<float>(vol_size) / longest);
    float dm[3];
    for (int a = 0; a < 3; ++a)
        dm[a] = static_cast<float>(f * static_cast<double>(size[a]));
    dm[0] = std::ceil(dm[0] / 4.0f) * 4.0f;
    dm[1] = std::ceil(dm[1]);
    dm[2] = std::ceil(dm[2]);
    for (int a = 0; a < 3; ++a)
        dims[a] = static_cast<int32_t>(dm[a]);
    *shortest = std::min(dm[0], std::min(dm[1], dm[2]));
    *max_lod = std::ceil(std::log2(static_cast<float>(vol_size))) - 1.0f;
}

namespace {

struct MdaoGeo {
    float bmin[3], inv[3], fd[3], cell[3];
    float cell_vol, ps_scale, sphere_k, half_vp[2];
    int d[3];
};

MdaoGeo mdao_geo(const float clip[6], const int32_t dims[3]) {
    MdaoGeo g{};
    for (int a = 0; a < 3; ++a) {
        const float size = clip[a + 3] > clip[a] ? clip[a + 3] - clip[a] : clip[a] - clip[a + 3];
        g.bmin[a] = clip[a];             // StartInsertion: inBoundsMin (MDAOVolumeGenerator.cpp:145-146)
        g.inv[a] = 1.0f / size;          // inBoundsSizeInverse (:139-143)
        g.fd[a] = static_cast<float>(dims[a]);
        g.d[a] = dims[a];
        g.cell[a] = 1.0f / (g.fd[a] * g.inv[a]);  // mdao_volume.frag.glsl:12
    }
    g.cell_vol = (g.cell[0] * g.cell[1]) * g.cell[2];                                 // frag:50
    g.ps_scale = std::max(g.inv[0] * g.fd[0], g.inv[1] * g.fd[1]);                    // mdao_volume.geom.glsl:28
    g.sphere_k = 4.0f / 3.0f * 3.14152f;                                              // frag:49 (sic)
    g.half_vp[0] = 0.5f * g.fd[0];  // viewport = one slice (MDAOVolumeGenerator.cpp:164)
    g.half_vp[1] = 0.5f * g.fd[1];
    return g;
}

inline float mdao_dot(const float* v) {
    return (v[0] * v[0] + v[1] * v[1]) + v[2] * v[2];
}

// mdao_volume.frag.glsl:9-76 for voxel (i, j, layer) and a sphere with centre c (relative to inBoundsMin)
// and squared radius w2; -1 = discarded fragment.
float mdao_fragment(const MdaoGeo& g, int i, int j, int layer, const float c[3], float w2) {
    const float cm[3] = {static_cast<float>(i) * g.cell[0], static_cast<float>(j) * g.cell[1],
                         static_cast<float>(layer) * g.cell[2]};
    float lo[3], hi[3], fp[3], cp[3];
    for (int a = 0; a < 3; ++a) {
        lo[a] = cm[a] - c[a];
        hi[a] = (cm[a] - c[a]) + g.cell[a];
        fp[a] = std::max(std::fabs(lo[a]), std::fabs(hi[a]));
        cp[a] = std::min(std::fabs(lo[a]), std::fabs(hi[a]));
    }
    if (mdao_dot(cp) - w2 > 0.0f)
        return -1.0f;
    if (mdao_dot(fp) - w2 < 0.0f)
        return 1.0f;
    const float radius = std::sqrt(w2);
    if (lo[0] <= -radius && lo[1] <= -radius && lo[2] <= -radius && hi[0] >= radius && hi[1] >= radius &&
        hi[2] >= radius)
        return (g.sphere_k * w2 * radius) / g.cell_vol;
    int hits = 0;
    for (int x = 0; x < 3; ++x)
        for (int y = 0; y < 3; ++y)
            for (int z = 0; z < 3; ++z) {
                const int k[3] = {x, y, z};
                float t[3];
                for (int a = 0; a < 3; ++a)
                    t[a] = (cm[a] + (g.cell[a] * static_cast<float>(k[a])) * 0.5f) - c[a];
                if (mdao_dot(t) - w2 < 0.0f)
                    ++hits;
            }
    return static_cast<float>(hits) / 27.0f;
}

// Covered pixel range of a point of `size` pixels centred at window coordinate `wc`: pixel centres
// i + 0.5 in [wc - size/2, wc + size/2), clipped to [0, n). For |wc|, size < 2^22 both subtractions of
// 0.5 are exact, so the ceilings give the first centre at or above each bound.
void mdao_point_span(float wc, float size, int n, int& i0, int& i1) {
    const float lo = wc - 0.5f * size, hi = wc + 0.5f * size;
    const float a = std::min(std::max(std::ceil(lo - 0.5f), 0.0f), static_cast<float>(n));
    const float b = std::min(std::max(std::ceil(hi - 0.5f), 0.0f), static_cast<float>(n));
    i0 = static_cast<int>(a);
    i1 = static_cast<int>(b);
}

}  // namespace

extern "C" void p2vo_mdao_volume_f32(const float* xyzr, int64_t n, const float clip[6], const int32_t dims[3],
    int unorm8, float* out) {
    const MdaoGeo g = mdao_geo(clip, dims);
    const int64_t nv = (int64_t) dims[0] * dims[1] * dims[2];
    std::vector<uint64_t> acc((size_t) nv, 0);
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t k = 0; k < n; ++k) {
        const float* p = xyzr + 4 * k;
        const float r = p[3];
        float np[3], c[3];
        bool inside = true;
        for (int a = 0; a < 3; ++a) {
            np[a] = (p[a] - g.bmin[a]) * g.inv[a];  // geom:72
            const float ndc = np[a] * 2.0f - 1.0f;  // geom:79; a point is clipped by its centre vertex
            inside = inside && (ndc >= -1.0f && ndc <= 1.0f);
            c[a] = p[a] - g.bmin[a];                // geom:30
        }
        if (!inside)
            continue;
        const float w2 = r * r;
        const float xw = (np[0] * 2.0f - 1.0f) * g.half_vp[0] + g.half_vp[0];  // viewport transform
        const float yw = (np[1] * 2.0f - 1.0f) * g.half_vp[1] + g.half_vp[1];
        auto emit = [&](int layer, float disk) {  // geom:24-34 + rasterisation of the point
            if (layer < 0 || layer >= g.d[2])
                return;
            // gl_PointSize = int(2 ceil(disk * scale)), at least one pixel; sizes beyond 2^22 pixels cover
            // the whole slice anyway and are capped so the span arithmetic stays exact
            const float ps = std::max(std::min(2.0f * std::ceil(disk * g.ps_scale), 4194304.0f), 1.0f);
            int x0, x1, y0, y1;
            mdao_point_span(xw, ps, g.d[0], x0, x1);
            mdao_point_span(yw, ps, g.d[1], y0, y1);
            for (int j = y0; j < y1; ++j)
                for (int i = x0; i < x1; ++i) {
                    float f = mdao_fragment(g, i, j, layer, c, w2);
                    if (f < 0.0f)
                        continue;
                    f = std::min(std::max(f, 0.0f), 1.0f);  // UNORM colour clamp before blending
                    const uint64_t q = unorm8 ? (uint64_t) std::nearbyint(f * 255.0f)
                                              : (uint64_t) std::llrint((double) (f * 4294967296.0f));
                    const int64_t v = (int64_t) i + ((int64_t) j + (int64_t) layer * g.d[1]) * g.d[0];
#pragma omp atomic
                    acc[(size_t) v] += q;
                }
        };
        // geom:76-92
        // slices beyond the volume's depth emit layers outside it: cap the count there
        const int numSlices =
            static_cast<int>(std::min(std::ceil(r * g.inv[2] * g.fd[2]), static_cast<float>(g.d[2] + 1)));
        const float zs = np[2] * g.fd[2];
        const int centerLayer = static_cast<int>(std::floor(zs));
        emit(centerLayer, r);
        const float sliceThickness = 1.0f / g.fd[2];
        const float zOffset = (zs - std::floor(zs)) / g.fd[2];
        for (int side = 0; side < 2; ++side) {  // geom:39-57, negative then positive hemisphere
            const int step = side == 0 ? -1 : 1;
            const float offset = side == 0 ? zOffset : sliceThickness - zOffset;
            for (int i = 1; i <= numSlices; ++i) {
                const float dist = (static_cast<float>(i - 1) / g.fd[2] + offset) / g.inv[2];
                const float nsq = r * r - dist * dist;
                if (nsq < 0.0f)
                    break;
                emit(centerLayer + step * i, std::sqrt(nsq));
            }
        }
    }
    for (int64_t v = 0; v < nv; ++v) {
        if (unorm8)
            out[v] = static_cast<float>(std::min<uint64_t>(acc[(size_t) v], 255)) / 255.0f;
        else
            out[v] = acc[(size_t) v] >= (1ull << 32) ? 1.0f
                                                     : static_cast<float>(acc[(size_t) v]) * (1.0f / 4294967296.0f);
    }
}

extern "C" void p2vo_mdao_mip_u8(const float* src, const int32_t sd[3], float* dst, const int32_t dd[3]) {
    for (int z = 0; z < dd[2]; ++z)
        for (int y = 0; y < dd[1]; ++y)
            for (int x = 0; x < dd[0]; ++x) {
                int sum = 0;
                const int x1 = std::min(2 * x + 1, sd[0] - 1), y1 = std::min(2 * y + 1, sd[1] - 1),
                          z1 = std::min(2 * z + 1, sd[2] - 1);
                for (int zz = 2 * z; zz <= z1; ++zz)
                    for (int yy = 2 * y; yy <= y1; ++yy)
                        for (int xx = 2 * x; xx <= x1; ++xx)
                            sum += (int) std::lrint(src[xx + (yy + int64_t(zz) * sd[1]) * sd[0]] * 255.0f);
                dst[x + (y + int64_t(z) * dd[1]) * dd[0]] = static_cast<float>((sum + 4) / 8) / 255.0f;
            }
}
