/*
 * p2v_oracle.h — CPU restatement of MegaMol's particle-to-volume path, used ONLY to check results.
 *
 * TEST INFRASTRUCTURE. Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load
 * this library. The shipped GPU library never calls it.
 *
 * Every function restates a cited piece of the reference (paths relative to the MegaMol tree):
 *  - density: plugins/datatools/src/ParticlesToDensity.cpp:389-747 (createVolumeCPU, bump rbf :472-476)
 *  - MDAO mip: plugins/moldyn_gl/shaders/moldyn_gl/mdao_volume_generator/mdao_mipmap_compute_main.comp.glsl:8-26
 *  - cone march: plugins/moldyn_gl/shaders/moldyn_gl/sphere_renderer/inc/mdao_deferred_fragment_ambocc.inc.glsl:9-60
 *  - cone directions: plugins/moldyn_gl/src/rendering/SphereRenderer.cpp:2572-2587
 *  - AOSphere deposit: plugins/pwdemos_gl/src/AOSphereRenderer.cpp:918-1021, sampling uniforms :489-514,
 *    taps shaders/pwdemos_gl/AOSphere/snippets/mainaxes_vertex_2.glsl:1-9,
 *    mainaxes_fragLightAO_evalAO.glsl:1-8, normals_fragLightAO_evalAO.glsl:1-4
 *  - MDAO voxeliser: plugins/moldyn_gl/shaders/moldyn_gl/mdao_volume_generator/mdao_volume.geom.glsl:24-93,
 *    mdao_volume.frag.glsl:9-76
 *
 * Parity status: density is pinned bit-exactly against the reference's own compiled
 * ParticlesToDensity.cpp (see oracle/Makefile, target `ref`). The AO functions restate GLSL that
 * cannot run here (no graphics stack): their parity is UNPINNED by any reference output.
 */
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Grid description shared by the density functions. bbox = {left, bottom, back, right, top, front}. */
typedef struct {
    float bbox[6];
    int32_t res[3];
    int32_t cyclic[3];
    float sigma;
} p2vo_grid;

/* Kernel selector: 0 = reference bump rbf, 1 = Gaussian (sigma*r) cut at 3 sigma. */
enum { P2VO_BUMP = 0, P2VO_GAUSS3 = 1 };

/* FP32, same operation order as ParticlesToDensity::createVolumeCPU for aggregator 0. With
 * nthreads == 1 the summation order is the particle order, as the reference with one OpenMP thread.
 * With nthreads > 1 each thread owns a private grid and the grids are summed serially afterwards,
 * like the reference (ParticlesToDensity.cpp:401-410,561,623-626). `xyzr` is n float4 records. */
int p2vo_density_f32(const float* xyzr, int64_t n, const p2vo_grid* g, int kernel, int nthreads, float* out);

/* FP64 restatement: the reference's integer decisions (cell, footprint, wrap) made with its float
 * expressions, every value (node positions, distances, kernel) evaluated in double with the exact
 * grid spacing (right-left)/(res-1). The GPU path's error is measured against this. */
int p2vo_density_f64(const float* xyzr, int64_t n, const p2vo_grid* g, int kernel, int nthreads, double* out);

/* Weighted createVolumeCPU: nc weights per particle (w[j * nc + c]); out holds nc interleaved components.
 * nc = 1 with intensities: the IColToSingleCell aggregator; the direction components: the
 * IVecToSingleCell aggregator's sums (its weight grid is the plain density). */
int p2vo_density_weighted_f32(const float* xyzr, const float* w, int nc, int64_t n, const p2vo_grid* g, int kernel,
    int nthreads, float* out);
int p2vo_density_weighted_f64(const float* xyzr, const float* w, int nc, int64_t n, const p2vo_grid* g, int kernel,
    int nthreads, double* out);
/* The vector aggregator's finish in float (ParticlesToDensity.cpp:628-682), in place on vol3 (3 per voxel). */
void p2vo_vector_finish_f32(float* vol3, const float* weights, int64_t V, int normalize, float* out_min,
    float* out_max);

/* MDAO 2x2x2 mip step, FP64: dst[i] = sum of the up-to-8 children clamped to the source size, / 8. */
void p2vo_mip_step_f64(const double* src, const int32_t sdim[3], double* dst, const int32_t ddim[3]);

/* Cone-marched AO (MDAO evaluateAmbientOcclusion, mdao_deferred_fragment_ambocc.inc.glsl:9-60).
 * levels[l] is mip level l in FP64 (dims ldims[3l..3l+2], x fastest). The sample positions use the
 * step table of p2vo_cone_steps (float, shared with the GPU so loop lengths agree); everything else is
 * evaluated in double. */
typedef struct {
    float bounds_min[3];
    float bounds_size[3];
    float offset, strength, cone_length, shortest_edge, max_lod;
    int32_t steps;      /* 0 = the reference's geometric stepping t += t*w until cone_length */
    int32_t early_exit; /* 1 = stop a cone once it exceeds 0.99, as the reference */
    int32_t border;     /* 0 = CLAMP_TO_BORDER (0), 1 = CLAMP_TO_EDGE */
    float sat_scale;    /* level-0 texel = clamp(v * sat_scale, 0, 1); <= 0 keeps v */
} p2vo_cone_params;

/* Cone directions around +Y (vec4: xyz direction, w = cone width 2 tan(apex/2)); K = 3 is
 * SphereRenderer::generate3ConeDirections (SphereRenderer.cpp:2572-2587), other K the same ring
 * construction with the K-gon circumradius. Float, as the reference. */
void p2vo_cone_dirs(int K, float apex_rad, float* out4);

/* Step table (t, lod) of one cone of width w; returns the number of samples (<= cap). */
int p2vo_cone_steps(const p2vo_cone_params* cp, float w, float* t, float* lod, int cap);

/* FP32 cone pipeline with OpenMP (nthreads): the MDAO pyramid of a float volume (out[l - 1] receives level l,
 * l = 1 .. nlevels - 1; level 1 from the texels clamp(v * sat_scale, 0, 1) when sat_scale > 0) and the march in
 * FP32 in the GPU kernel's operation order, level 0 saturated on the fly. The CPU baseline's timing stand-in. */
void p2vo_mip_levels_f32(const float* l0, const int32_t d0[3], float sat_scale, int nlevels, float* const* out,
    int nthreads);
void p2vo_cone_ao_f32(const float* const* levels, const int32_t* ldims, int nlevels, const float* dirs, int ncones,
    const p2vo_cone_params* cp, const float* xyzr, const float* nrm, int64_t n, int nthreads, float* ao);
void p2vo_cone_ao_f64(const double* const* levels, const int32_t* ldims, int nlevels, const float* dirs, int ncones,
    const p2vo_cone_params* cp, const float* xyzr, const float* nrm, int64_t n, double* ao);

/* AOSphereRenderer volume deposit (AOSphereRenderer.cpp:918-1021): s = "vol::size" including the
 * 1-voxel zero border; tex gets (4/3 pi r^3 / voxel volume) * genFac in the inner voxel of each particle. */
/* The library's gradient normals (P2V_NORMALS_GRADIENT) in FP32 with OpenMP: -grad(rho) / |grad(rho)| at each
 * particle (out3: n x 3 floats) from the node grid (x fastest, res), cyclic flags, node origin minf and the
 * reference spacing h per axis. */
void p2vo_gradient_normals_f32(const float* grid, const int32_t res[3], const int32_t cyc[3], const float minf[3],
    const float h[3], const float* xyzr, int64_t n, int nthreads, float* out3);
/* AOSphere volume deposit with the renderer's two rules: glsl_rule 0 = createVolumeCPU (inner voxel +1, optional
 * clip-plane discard of particles with dot(p, n) - d >= 0), 1 = createVolumeGLSL (x, y: floor clamped to
 * [0, s_inner] without the border offset; z: slice trunc clamped to [0, s_inner - 1], + 1; no clip). */
void p2vo_aosphere_volume_ex_f64(const float* xyzr, int64_t n, const float clip[6], const int32_t s[3], float gen_fac,
    int glsl_rule, int use_clip, const float plane[4], double* tex);
void p2vo_aosphere_volume_f64(const float* xyzr, int64_t n, const float clip[6], const int32_t s[3], float gen_fac,
    double* tex);
/* AOSphere sampling: mode 0 = main axes (mainaxes_vertex_2.glsl + mainaxes_fragLightAO_evalAO.glsl),
 * mode 1 = normal tap (normals_fragLightAO_evalAO.glsl), uniforms as AOSphereRenderer.cpp:489-514. */
void p2vo_aosphere_ao_f64(const double* tex, const int32_t s[3], const float clip[6], float step_len, float eval_fac,
    const float* xyzr, const float* nrm, int64_t n, int mode, double* ao);

/* Learned-AO MLP 54 -> 64 -> 64 -> 1 (SiLU, SiLU, sigmoid), FP64 reference for gradient checks.
 * params: W1[64][54], b1[64], W2[64][64], b2[64], w3[64], b3 (7745 values). Loss = mean((y - t)^2).
 * grads (may be NULL) receives dLoss/dparams; y (may be NULL) the predictions. */
void p2vo_mlp_f64(const double* params, const float* x, const float* t, int64_t n, double* grads, double* loss,
    double* y);

/* MDAO occupancy volume (the AO volume of moldyn_gl::SphereRenderer's MDAO mode).
 * Dimensions (SphereRenderer.cpp:2463-2476): longest clip-box edge -> vol_size voxels, x rounded up to a
 * multiple of 4; shortest = min(dims); max_lod = ceil(log2(vol_size)) - 1. */
void p2vo_mdao_dims(const float clip[6], int vol_size, int32_t dims[3], float* shortest, float* max_lod);
/* Voxelisation (mdao_volume.vert.glsl:9-14, mdao_volume.geom.glsl:24-93, mdao_volume.frag.glsl:9-76) with
 * the additive blend of MDAOVolumeGenerator.cpp:151-153 into an R8 texture: each voxel receives, per
 * covering sphere, the fragment value q = round(clamp(frac, 0, 1) * 255) and keeps min(255, sum q); out =
 * that / 255 (unorm8 = 1). unorm8 = 0 keeps the fractions unquantised: out = min(1, sum of clamp(frac))
 * summed in 2^-32 fixed point. FP32 with the shaders' operation order, no fused multiply-adds.
 * xyzr holds the particles to insert (radius = w). */
void p2vo_mdao_volume_f32(const float* xyzr, int64_t n, const float clip[6], const int32_t dims[3], int unorm8,
    float* out);
/* One MDAO mip step of an R8 volume (mdao_mipmap_compute_main.comp.glsl:8-26 with an R8 store): children
 * as 8-bit integers k, out = ((sum k + 4) / 8) / 255 (the /8 rule, rounded half up). */
void p2vo_mdao_mip_u8(const float* src, const int32_t sdim[3], float* dst, const int32_t ddim[3]);

#ifdef __cplusplus
}
#endif
