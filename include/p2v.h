/*
 * p2v.h — C ABI of the GB300-native particle-to-volume library (libp2v.so).
 *
 * Drop-in boundary for one MegaMol hot path: a MultiParticleDataCall frame in, a VolumetricDataCall
 * density grid and a per-particle ambient-occlusion (AO) attribute out. The entry points replace:
 *
 *   p2v_set_params   <- the ParamSlots of datatools::ParticlesToDensity
 *                       (plugins/datatools/src/ParticlesToDensity.cpp:59-152) plus the AO parameters of
 *                       AOSphereRenderer (plugins/pwdemos_gl/src/AOSphereRenderer.cpp:83-124) and of the
 *                       SphereRenderer MDAO mode (plugins/moldyn_gl/src/rendering/SphereRenderer.cpp:193-214)
 *   p2v_run_frame    <- ParticlesToDensity::getDataCallback + createVolumeCPU
 *                       (ParticlesToDensity.cpp:210-383, :389-747) and the AO evaluation of
 *                       AOSphereRenderer / MDAO (see p2v_params.ao_mode)
 *   p2v_volume       <- VolumetricMetadata_t + VolumetricDataCall::SetData
 *                       (plugins/geometry_calls/include/geometry_calls/VolumetricDataCallTypes.h:32-134,
 *                       VolumetricDataCall.h:285-288)
 *   p2v_particle_list<- SimpleSphericalParticles vertex / direction / colour data
 *                       (plugins/geometry_calls/include/geometry_calls/SimpleSphericalParticles.h:27-58,475-589)
 *
 * Conventions: every call returns a p2v_status; nothing throws across the boundary. A context is bound
 * to one device and must be used by one host thread at a time. Output buffers are caller-allocated.
 * Pointers flagged P2V_MEM_DEVICE are CUDA device pointers on the context's device.
 */
#ifndef P2V_H
#define P2V_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define P2V_ABI_VERSION 10

#if defined(__GNUC__)
#define P2V_API __attribute__((visibility("default")))
#else
#define P2V_API
#endif

typedef enum p2v_status {
    P2V_OK = 0,
    P2V_EINVAL = 1,       /* invalid argument or parameter */
    P2V_ENOMEM = 2,       /* device or host allocation failed */
    P2V_ECUDA = 3,        /* a CUDA runtime call failed */
    P2V_ETIMEOUT = 4,     /* a bounded device-side wait gave up (the results of that call are invalid) */
    P2V_EDOMAIN = 5,      /* input outside the supported domain (see p2v_stats) */
    P2V_EUNSUPPORTED = 6  /* parameter combination not implemented */
} p2v_status;

/* SimpleSphericalParticles::VertexDataType (SimpleSphericalParticles.h:27-33) */
typedef enum p2v_vertex_type {
    P2V_VERTDATA_NONE = 0,
    P2V_VERTDATA_FLOAT_XYZ = 1,  /* global radius */
    P2V_VERTDATA_FLOAT_XYZR = 2,
    P2V_VERTDATA_SHORT_XYZ = 3,  /* unsigned short components, read as their integer value; global radius */
    P2V_VERTDATA_DOUBLE_XYZ = 4  /* global radius */
} p2v_vertex_type;

typedef enum p2v_mem { P2V_MEM_HOST = 0, P2V_MEM_DEVICE = 1 } p2v_mem;

/* Density kernel. BUMP is the reference's rbf exp(-1/(1-(d/eps)^2)), eps = sigma*r, with its
 * footprint ceil(r/h) (ParticlesToDensity.cpp:472-476,573-575). GAUSS3 is a Gaussian of standard
 * deviation sigma*r cut at 3 sigma, shifted by its value at the cut so it ends continuously at zero. */
typedef enum p2v_kernel { P2V_KERNEL_BUMP = 0, P2V_KERNEL_GAUSS3 = 1 } p2v_kernel;

/* Voxel accumulation. EXACT: every FP32 contribution is rounded to a multiple of 2^-32 and summed in
 * 64-bit integers, i.e. the exact, order-independent sum, rounded once to FP32 (particle-major scatter
 * into shared-memory tiles; the fast path). KAHAN: each voxel gathers its contributions in cell order
 * with a Kahan-compensated FP32 sum (node-major). Both are deterministic run to run. */
typedef enum p2v_accumulate { P2V_ACCUM_EXACT = 0, P2V_ACCUM_KAHAN = 1 } p2v_accumulate;

/* AO evaluated per particle at the surface point p + r*n (n = the particle's normal). */
typedef enum p2v_ao_mode {
    P2V_AO_NONE = 0,
    P2V_AO_CONE = 1,            /* cone march through a mip pyramid (MDAO evaluateAmbientOcclusion) */
    P2V_AO_AOSPHERE_AXES = 2,   /* AOSphereRenderer main-axes mode: 6 taps combined by n^2 */
    P2V_AO_AOSPHERE_NORMAL = 3, /* AOSphereRenderer normal-based mode: 1 tap along n */
    P2V_AO_LEARNED = 4          /* MLP stand-in for CONE, cone-march fallback outside its training range */
} p2v_ao_mode;

/* Volume the cone march samples. */
typedef enum p2v_ao_volume {
    P2V_AOVOL_DENSITY = 0, /* the density grid of this call, times ao_volume_scale, saturated to [0,1] */
    P2V_AOVOL_MDAO = 1     /* MDAO occupancy voxelisation (mdao_volume.geom/frag.glsl) */
} p2v_ao_volume;

/* Colour data types, values of SimpleSphericalParticles::ColourDataType (SimpleSphericalParticles.h:41-50). */
typedef enum p2v_colour_type {
    P2V_COLDATA_NONE = 0,        /* global colour */
    P2V_COLDATA_UINT8_RGB = 1,
    P2V_COLDATA_UINT8_RGBA = 2,
    P2V_COLDATA_FLOAT_RGB = 3,
    P2V_COLDATA_FLOAT_RGBA = 4,
    P2V_COLDATA_FLOAT_I = 5,
    P2V_COLDATA_USHORT_RGBA = 6,
    P2V_COLDATA_DOUBLE_I = 7
} p2v_colour_type;

typedef struct p2v_particle_list {
    int32_t vertex_type;        /* p2v_vertex_type */
    uint32_t vertex_stride;     /* bytes between records, 0 = packed */
    const void* vertex_data;
    uint64_t count;
    float global_radius;
    int32_t mem;                /* p2v_mem of vertex_data, normals, colour_data and ao_out */
    const float* normals;       /* optional: per-particle direction (DIRDATA_FLOAT_XYZ layout): the AO modes'
                                   normals, the vector aggregator's directions */
    uint32_t normal_stride;     /* bytes, 0 = packed (12) */
    float* ao_out;              /* optional: per-particle AO (COLDATA_FLOAT_I), count floats */
    int32_t colour_type;        /* p2v_colour_type of colour_data (the intensity aggregator reads its first
                                   channel, as SimpleSphericalParticles' GetCRAcc) */
    uint32_t colour_stride;     /* bytes, 0 = packed */
    const void* colour_data;
    uint8_t global_colour[4];   /* RGBA for P2V_COLDATA_NONE (channel value / 255 as the intensity) */
} p2v_particle_list;

typedef struct p2v_frame {
    float bbox[6];     /* ObjectSpaceBBox: left, bottom, back, right, top, front */
    float clipbox[6];  /* ObjectSpaceClipBox (bounds of the AOSphere / MDAO AO volumes) */
    uint32_t frame_id;
    uint32_t list_count;
    const p2v_particle_list* lists;
} p2v_frame;

typedef struct p2v_volume {
    float* data;          /* out: resolution product * components floats, x fastest; may be NULL */
    int32_t mem;          /* p2v_mem of data */
    uint64_t capacity;    /* floats available at data */
    /* filled by p2v_run_frame, as ParticlesToDensity::getDataCallback fills VolumetricMetadata_t
     * (ParticlesToDensity.cpp:249-293) */
    uint64_t resolution[3];
    uint64_t components;
    float slice_dists[3];
    float origin[3];
    float extents[3];
    double min_value, max_value;
    float bbox[6];        /* bounding box the grid spans (differs from the input with forSurfaceReconstruction) */
    uint64_t data_hash;   /* bumped on every recomputation, as the module's datahash */
} p2v_volume;

typedef struct p2v_params {
    uint32_t struct_size; /* sizeof(p2v_params); set by p2v_params_default */
    /* --- ParticlesToDensity slots (ParticlesToDensity.cpp:59-152) --- */
    int32_t aggregator;   /* 0 = PosToSingleCell_Volume (density), 1 = IColToSingleCell_Volume (first colour
                             channel), 2 = IVecToSingleCell_Volume (normals as DIRDATA_FLOAT_XYZ; 3 components) */
    int32_t sizex, sizey, sizez;
    int32_t cyclX, cyclY, cyclZ;
    int32_t normalize;    /* min-max to [0,1] after accumulation (ParticlesToDensity.cpp:676-682) */
    float sigma;
    int32_t forSurfaceReconstruction;
    /* --- extensions --- */
    int32_t kernel;         /* p2v_kernel */
    int32_t mass_normalize; /* scale so that sum(grid) * voxel volume == particle count (FP64 sum); before `normalize` */
    int32_t accumulate;     /* p2v_accumulate: how each voxel sums its FP32 contributions */
    /* --- AO --- */
    int32_t ao_mode;        /* p2v_ao_mode */
    int32_t ao_volume;      /* p2v_ao_volume, for P2V_AO_CONE / P2V_AO_LEARNED */
    float ao_volume_scale;  /* density -> occlusion scale for P2V_AOVOL_DENSITY */
    int32_t ao_cones;       /* 3 = the MDAO direction set (SphereRenderer.cpp:2572-2587) */
    int32_t ao_steps;       /* 0 = MDAO geometric stepping t += t*w until cone_length; >0 = that many samples */
    int32_t ao_levels;      /* mip levels sampled (level 0 = the volume); 0 = density: ceil(log2(longest edge)),
                               MDAO: maxLod + 1 = ceil(log2(mdao_volume_size)) (SphereRenderer.cpp:2476) */
    float ao_apex_deg;      /* "ambient occlusion::apex" (50) */
    float ao_offset;        /* "ambient occlusion::offset" (0.01) */
    float ao_strength;      /* "ambient occlusion::strength" (1) */
    float ao_cone_length;   /* "ambient occlusion::coneLength" (0.8), normalised volume coordinates */
    int32_t ao_early_exit;  /* stop a cone at 0.99 occlusion, as the reference (1) */
    int32_t mdao_volume_size; /* "ambient occlusion::volumeSize" (128): voxels along the longest edge */
    int32_t mdao_unorm8;    /* store the MDAO volume and its mips as 8-bit UNORM like the reference's R8 */
    /* AOSphereRenderer (AOSphereRenderer.cpp:83-124) */
    int32_t aos_sizex, aos_sizey, aos_sizez; /* "vol::sizex/y/z" (32) including the 1-voxel border */
    float aos_step_len;     /* "ao::stepLen" (0.5) */
    float aos_gen_fac;      /* "vol::genFac" (1) */
    float aos_eval_fac;     /* "ao::evalFac" (1) */
    /* --- execution --- */
    int32_t tile_x, tile_y, tile_z; /* density tile; 0 = the autotuned tile (p2v_autotune_batch) or 16^3 */
    int32_t batch_lanes;    /* p2v_run_batch: concurrent frame pipelines; 0 = the autotuned count or 4 */
    int32_t batch_graph;    /* p2v_run_batch: capture the batch as a CUDA graph and replay it while the batch's
                               shape (frames, sizes, pointers, parameters) repeats (1) */
    /* --- outputs --- */
    int32_t vector_grid;    /* aggregator 2: also build the outParticles / outInfo grid of p2v_get_vector_grid (0) */
    /* --- AOSphereRenderer volume deposit (appended; AOSphereRenderer.cpp:83-124, 918-1221) --- */
    int32_t aos_deposit;    /* p2v_aos_deposit: the CPU rule of createVolumeCPU (0) or the GLSL rule of createVolumeGLSL */
    int32_t aos_clip;       /* "ao::clipData": the CPU rule drops particles with dot(p, n) - d >= 0 (0) */
    float aos_clip_plane[4];/* the clip plane as the renderer's clipDat: unit normal n and d = dot(point, n) (0) */
    int32_t ao_normals;     /* p2v_ao_normals: where the AO modes take each particle's normal (P2V_NORMALS_LIST) */
    /* --- bounded device waits --- */
    int32_t mma_wait_polls; /* polls of the learned AO's tensor-core completion waits before the call gives up with
                               P2V_ETIMEOUT; 0 = the default (2^20, about a second) */
    int32_t test_hold_mma;  /* test hook: the learned AO's first MMA is not issued, so its bounded wait runs out and
                               the call returns P2V_ETIMEOUT with the context still usable (0) */
    /* --- z-slab output (a rank's share of one large frame) --- */
    int32_t slab_z0, slab_z1; /* compute and return only grid planes [slab_z0, slab_z1) of the sizez planes; both 0 =
                                 the whole grid. The node positions stay those of the whole grid; the returned volume
                                 holds the slab (resolution z = slab_z1 - slab_z0, origin z moved to plane slab_z0),
                                 its statistics and normalisation cover the slab only. Density and intensity
                                 aggregators without AO (0, 0) */
    /* --- the persistent batch AO (appended) --- */
    int32_t batch_persistent; /* p2v_run_batch with the cone march on the density (ao_mode P2V_AO_CONE, ao_volume
                                 P2V_AOVOL_DENSITY, ao_march P2V_AO_MARCH_THREAD, aggregator 0 or 1): 1 = the
                                 lanes run every frame up to its normalised grid, then ONE persistent launch
                                 builds every frame's mip levels and marches every frame's cones from a
                                 device-side work queue; 0 = each lane runs its frames' AO kernels itself
                                 (overlapping them with other frames' binning and density); -1 = the choice of
                                 p2v_autotune_batch, 0 before it has run (-1) */
    int32_t queue_wait_polls; /* polls of a queue item's dependency wait in that launch before the call gives up
                                 with P2V_ETIMEOUT; 0 = the default (2^22, a second or more) */
    int32_t test_hold_queue;  /* test hook: the first mip level the queue builds never reports its completion, so
                                 the items that need it wait until queue_wait_polls runs out (0) */
    int32_t sort_wait_polls;  /* polls of the binning radix sort's decoupled look-back before the frame gives up
                                 with P2V_ETIMEOUT (the frame's grid is then empty); 0 = the default (2^22) */
    int32_t test_hold_sort;   /* test hook: the second tile of the binning's first radix pass never publishes its
                                 digit counts, so the tiles after it wait until sort_wait_polls runs out (0) */
    int32_t ao_march;         /* p2v_ao_march: the kernel of the plain cone march (P2V_AO_MARCH_THREAD) */
    int32_t ao_brick_order;   /* 1: the cone march and the learned AO take the particles in brick-major order (bricks
                                 of 16 x 4 x 4 cells) instead of cell order, so that neighbouring threads sample
                                 neighbouring texels along all three axes; 0: cell order; -1: brick order for the
                                 plain cone march only (14 % faster on the LJ frame, 1 % on the mixed-phase
                                 frame, slower on blob trajectories). The same AO bits either way (0) */
} p2v_params;

/* AOSphere volume deposit rule: which voxel a particle's volume goes to. CPU (createVolumeCPU,
 * AOSphereRenderer.cpp:918-1021): inner voxel trunc(u * s_inner) clamped to [0, s_inner - 1], stored at +1 inside
 * the one-voxel border, with the optional clip-plane discard. GLSL (createVolumeGLSL, :1026-1221, and
 * volume_updateVolume.vert.glsl:22-46): x and y floor(u * s_inner) clamped to [0, s_inner] written without the
 * +1 (the point lands on a pixel corner; a fragment is taken for the pixel centre on the square's lower edge),
 * z binned on the host into slice trunc(u * s_inner) (at most s_inner - 1; below the box: slice 0) + 1; no clip. */
typedef enum p2v_aos_deposit { P2V_AOS_DEPOSIT_CPU = 0, P2V_AOS_DEPOSIT_GLSL = 1 } p2v_aos_deposit;

/* Normals of the AO modes. LIST: the lists' per-particle directions (DIRDATA_FLOAT_XYZ, p2v_particle_list.normals).
 * GRADIENT: computed on the device from this frame's density grid, for particle data without directions: the
 * unit vector down the density gradient, -grad(rho) / |grad(rho)|, with grad(rho) the node grid's central
 * differences (periodic along cyclic axes, one-sided first differences at the faces of open ones) interpolated
 * trilinearly at the particle's position (clamped into the node range); a vanishing gradient gives a zero
 * normal (AO 1). Needs a scalar grid (aggregator 0 or 1). */
typedef enum p2v_ao_normals { P2V_NORMALS_LIST = 0, P2V_NORMALS_GRADIENT = 1 } p2v_ao_normals;
/* The plain cone march's kernel (both give the same bits): one thread marches all cones of a particle, or
 * one warp per cone of a particle with its lanes taking the cone's steps. */
typedef enum p2v_ao_march { P2V_AO_MARCH_THREAD = 0, P2V_AO_MARCH_WARP = 1 } p2v_ao_march;

typedef struct p2v_stats {
    uint64_t particles_in;       /* records presented */
    uint64_t particles_binned;   /* records that can contribute */
    uint64_t particles_dropped;  /* NaN/Inf coordinates or radius, radius <= 0, or farther than 2^30 cells */
    float radius_max;
    int32_t cell_min[3], cell_max[3]; /* occupied cell range (floor((p-min)/h)) */
    double mass_sum;             /* FP64 sum of the raw grid */
    double ms_upload, ms_binning, ms_density, ms_normalize, ms_ao, ms_download, ms_total; /* CUDA events */
    uint32_t device_error;       /* nonzero: a bounded device wait gave up (status P2V_ETIMEOUT) */
    uint32_t ao_fallback;        /* learned AO: particles that fell back to the cone march */
    uint32_t cell_max_count;     /* binning: particles in the fullest cell when the counting sort by cell was
                                    tried (it takes frames whose cells hold at most 32), 0 = radix sort only */
    uint32_t ao_fetches;         /* learned AO: texture fetches per particle of its inference kernel (0 otherwise) */
    double ms_ao_kernel;         /* CUDA events around the AO stage's main kernel alone (the learned AO's inference
                                    or the plain cone march; 0 for other AO modes or untimed frames) */
} p2v_stats;

/* Learned AO (no counterpart in the reference: its AO is the GLSL cone march). Features per particle: the
 * cone march's own visibility samples (mdao_deferred_fragment_ambocc.inc.glsl:30-51), filtered by the texture
 * units: for each of P2V_MLP_CONES cones, in the particle's cone frame, the AO volume at P2V_MLP_FSTEPS of the
 * march's steps (step round(j (steps - 1) / (P2V_MLP_FSTEPS - 1)) for feature j), each at the step's own mip
 * level (linear between the two levels around its lod); cone-major (feature c * P2V_MLP_FSTEPS + j). Then the
 * unit normal and the surface point in normalised volume coordinates; P2V_MLP_INPUTS values. The learned AO
 * therefore needs ao_cones = P2V_MLP_CONES. Network 54 -> 64 -> 64 -> 1 with SiLU, SiLU, sigmoid. Parameter
 * vector: W1[64][54], b1[64], W2[64][64], b2[64], w3[64], b3. */
#define P2V_MLP_CONES 8
#define P2V_MLP_FSTEPS 6
#define P2V_MLP_INPUTS 54
#define P2V_MLP_HIDDEN 64
#define P2V_MLP_PARAMS 7745

typedef struct p2v_train_params {
    uint32_t struct_size;   /* sizeof(p2v_train_params); set by p2v_train_params_default */
    int32_t epochs;
    int32_t batch;
    float lr, beta1, beta2, eps;   /* Adam */
    float lr_decay;         /* lr multiplied by this after every epoch */
    float val_fraction;     /* pairs held out for validation */
    float range_margin;     /* fallback when a feature leaves [lo - m(hi-lo), hi + m(hi-lo)] of the training pairs */
    uint64_t seed;          /* initialisation and batch order */
} p2v_train_params;

typedef struct p2v_train_report {
    uint64_t pairs_train, pairs_val;
    int32_t steps;
    float final_loss;       /* training MSE of the last epoch's last batch */
    float val_rmse, val_max_err;   /* FP32 network vs cone-march targets on the held-out pairs */
    double ms;
} p2v_train_report;

typedef struct p2v_ctx p2v_ctx;

P2V_API int p2v_abi_version(void);
P2V_API void p2v_params_default(p2v_params* p);

P2V_API p2v_status p2v_create(p2v_ctx** ctx, int device);
P2V_API void p2v_destroy(p2v_ctx* ctx);

P2V_API p2v_status p2v_set_params(p2v_ctx* ctx, const p2v_params* p);
/* Current parameters; forSurfaceReconstruction rewrites sizex/sizey as the reference module does. */
P2V_API p2v_status p2v_get_params(const p2v_ctx* ctx, p2v_params* p);

/* Compute the density grid (and AO when ao_mode != NONE) of one frame. Synchronous on `stream`
 * (a cudaStream_t, NULL = the context's stream): on return `vol` is filled and every host output is
 * written. Mirrors ParticlesToDensity::getDataCallback for IDX_GET_DATA. */
P2V_API p2v_status p2v_run_frame(p2v_ctx* ctx, const p2v_frame* frame, p2v_volume* vol, void* stream);

/* AO of a frame's particles against a density grid the caller supplies (sizex * sizey * sizez floats, x fastest,
 * the nodes of the frame's box as p2v_run_frame places them; host or device memory per mem) instead of the grid
 * of the frame's own particles: the grid the cone march and the AOSphere taps sample, and the gradient normals'
 * grid. For a rank that holds only part of a frame's particles but the frame's whole (gathered) grid, and for
 * callers that already hold a volume. No counterpart in the reference, whose AO samples a volume it builds itself
 * (MDAOVolumeGenerator, AOSphereRenderer). Needs an AO mode, aggregator 0 and no z-slab; writes each list's
 * ao_out. Synchronous on `stream` as p2v_run_frame. */
P2V_API p2v_status p2v_run_ao_on_grid(p2v_ctx* ctx, const p2v_frame* frame, const float* grid, int32_t mem,
                                      void* stream);

/* Device pointer of the last density grid (valid until the next call on this context); the reference's
 * VolumetricDataCall cannot carry one, so this is an addition of this library. */
P2V_API p2v_status p2v_get_device_volume(p2v_ctx* ctx, const float** dptr, uint64_t resolution[3]);

/* Level `level` of the last cone-march pyramid (P2V_AO_CONE / P2V_AO_LEARNED): level 0 is the density grid
 * (before the ao_volume_scale saturation) or the MDAO occupancy volume, whose R8 texture the reference
 * keeps in GL (MDAOVolumeGenerator::GetVolumeTextureHandle, MDAOVolumeGenerator.cpp:46-48). dims receives
 * the level's size (x, y, z); with out == NULL only dims is written. Otherwise copies the texels (x fastest)
 * into out (host or device memory per mem, capacity in floats). Synchronises the device. */
P2V_API p2v_status p2v_get_ao_volume(p2v_ctx* ctx, int32_t level, float* out, uint64_t capacity, int32_t mem,
                                     int32_t dims[3]);

/* The binning of the last p2v_run_frame (replaces ParticlesToDensity.cpp:561-568, which computes each
 * particle's cell on the fly): the bin keys in sorted order, the stable sort permutation (sorted position ->
 * particle index over the concatenated lists) and the first sorted position of every bin (nbins + 1
 * entries). A bin is the particle's floor cell per axis clamped to [-1, size] (one underflow and one
 * overflow bin per axis), key = (bz * (sy + 2) + by) * (sx + 2) + bx with b = cell + 1; particles with
 * non-finite coordinates or radius <= 0 carry key nbins and sort last. Any output pointer may be NULL;
 * count and nbins (nullable) receive the sizes. Synchronises the device. */
P2V_API p2v_status p2v_get_binning(p2v_ctx* ctx, uint32_t* keys, uint32_t* order, uint64_t capacity,
                                   uint32_t* cell_start, uint64_t start_capacity, uint32_t* count, uint32_t* nbins);

/* The vector aggregator's two extra outputs (ParticlesToDensity.cpp:306-380, 436-456, 628-727) of the last
 * p2v_run_frame with aggregator 2 and vector_grid set: the grid nodes whose average direction is non-zero,
 * sorted by its length (the "density") descending, equal densities in node order. Per entry: the node
 * position (3 floats, min + slice distance * index), the unit direction (3), the colour
 * (density - min) / (max - min) (the outParticles list: VERTDATA_FLOAT_XYZ, DIRDATA_FLOAT_XYZ,
 * COLDATA_FLOAT_I), and the outInfo row of 7 floats (PositionX/Y/Z, VelocityX/Y/Z, VelocityMag = the colour
 * when normalising, else the density). meta receives the entry count, outParticles' global radius (bbox
 * width / sizex / 5) and the 7 columns' minimum / maximum values. Each output pointer may be NULL; the
 * others need capacity >= count entries, in host or device memory per mem. Synchronises the device. */
typedef struct p2v_vector_grid_info {
    uint64_t count;
    float global_radius;
    float col_min[7], col_max[7];
} p2v_vector_grid_info;

P2V_API p2v_status p2v_get_vector_grid(p2v_ctx* ctx, float* positions, float* directions, float* colours,
                                       float* info, uint64_t capacity, int32_t mem, p2v_vector_grid_info* meta);

P2V_API p2v_status p2v_get_stats(const p2v_ctx* ctx, p2v_stats* st);
/* Last error message of this context ("" if none); returns the message length. */
P2V_API size_t p2v_get_last_error(const p2v_ctx* ctx, char* buf, size_t len);

/* ---- dat/raw output ----
 * Writes a volume as MegaMol's volume::DatRawWriter does (plugins/volume/src/DatRawWriter.cpp:58-186):
 * <prefix><frame, 4 digits zero-filled>.dat, a text header (ObjectFileName = the raw file's name, Format
 * FLOAT, GridType EQUIDISTANT, Components, Dimensions 3, TimeSteps 1, ByteOrder LITTLE_ENDIAN, Resolution,
 * SliceThickness - x, y and y again, as the reference writes it -, Origin, Time = frame), and
 * <prefix><frame>.raw, the voxels x fastest with interleaved components. vol is a volume p2v_run_frame
 * described (resolution, components, slice distances, origin); its data in host or device memory per
 * vol->mem, or vol->data == NULL for the context's device grid of the last frame. A device volume streams
 * through two pinned buffers, copy and file write overlapped. ctx may be NULL for host data. frame_count > 0
 * rejects frame >= frame_count as the reference does; the prefix may not be empty or end in '/'. */
P2V_API p2v_status p2v_write_datraw(p2v_ctx* ctx, const char* prefix, uint32_t frame, uint32_t frame_count,
                                    const p2v_volume* vol);

/* ---- batched frames ----
 * No counterpart in the reference, whose ParticlesToDensity computes one frame per GET_DATA call. A batch
 * runs many frames (a trajectory's, of uneven particle counts and grid sizes) with the current parameters:
 * the frames are spread over batch_lanes concurrent pipelines (largest first, onto the least-loaded lane),
 * nothing waits for the device until the whole batch is queued, and with batch_graph the queued batch is
 * captured once as a CUDA graph and replayed by one launch while its shape repeats. With the cone march
 * on the density and batch_persistent, every frame's AO stage (mip levels, gradient normals, cones) runs
 * in one persistent launch over a device-side work queue after the lanes. Each frame's results equal those
 * of p2v_run_frame on the same frame bit for bit. */
typedef struct p2v_batch_item {
    const p2v_frame* frame;
    p2v_volume* volume;  /* the frame's grid and metadata; NULL or data == NULL: not returned */
    int32_t size[3];     /* grid resolution of this frame; 0 = the parameters' sizex / sizey / sizez */
} p2v_batch_item;

/* stats (nullable) receives count per-frame statistics (stage times are not split per frame in a batch:
 * p2v_get_stats afterwards reports the whole batch's device time in ms_total). */
P2V_API p2v_status p2v_run_batch(p2v_ctx* ctx, const p2v_batch_item* items, uint32_t count, p2v_stats* stats,
                                 void* stream);

#define P2V_TUNE_MAX 32
typedef struct p2v_tune_report {
    uint32_t struct_size;
    int32_t tile[3];                  /* chosen density tile (exact accumulation) */
    int32_t lanes;                    /* chosen batch_lanes */
    float ms_best;                    /* device time of one batch with the chosen configuration */
    int32_t candidates;
    int32_t cand_tile[P2V_TUNE_MAX][3];
    int32_t cand_lanes[P2V_TUNE_MAX];
    float cand_ms[P2V_TUNE_MAX];
    int32_t persistent;               /* chosen batch AO: 1 the persistent launch, 0 the lanes' own kernels */
    int32_t cand_persistent[P2V_TUNE_MAX];
} p2v_tune_report;

/* Time every compiled density tile x lane count (x, where the persistent batch AO applies, both batch AO
 * forms) on this batch (CUDA events, one warm-up run each) and keep the fastest for later calls whose
 * tile_x / batch_lanes are 0 and batch_persistent is -1. rep (nullable) receives the table. */
P2V_API p2v_status p2v_autotune_batch(p2v_ctx* ctx, const p2v_batch_item* items, uint32_t count,
                                      p2v_tune_report* rep);

/* ---- MMPLD files ----
 * The reader of MegaMol's particle list files (plugins/moldyn/src/io/MMPLDDataSource.cpp:50-220, header
 * :335-420): versions 1.0-1.3, a frame table of file offsets, per frame a timestamp (1.2+) and lists of
 * interleaved vertex + colour records with a global radius / colour, an intensity range and (1.3) a per-list
 * box. Frames are read with positional reads, so several threads may read different frames of one open
 * file at once. The caller provides the frame buffer (host memory; a pinned buffer from p2v_host_alloc lets
 * p2v_run_frame upload it asynchronously); the lists point into it. */
typedef struct p2v_mmpld p2v_mmpld;

typedef struct p2v_mmpld_info {
    uint32_t version;   /* 100..103 */
    uint32_t frames;
    float bbox[6];
    float clipbox[6];
} p2v_mmpld_info;

typedef struct p2v_mmpld_list_info {
    float intensity_range[2];  /* colour map index values (FLOAT_I / DOUBLE_I lists; else 0, 1) */
    float bbox[6];             /* the list's box (version 1.3), else the file's */
    uint32_t clusters;         /* version 1.1 cluster count (the cluster data are skipped) */
} p2v_mmpld_list_info;

P2V_API p2v_status p2v_mmpld_open(const char* path, p2v_mmpld** file, p2v_mmpld_info* info);
P2V_API void p2v_mmpld_close(p2v_mmpld* file);
/* Bytes of frame `frame` (the buffer p2v_mmpld_read_frame needs). */
P2V_API p2v_status p2v_mmpld_frame_size(p2v_mmpld* file, uint32_t frame, uint64_t* bytes);
/* Read frame `frame` into buffer and describe its lists: at most max_lists entries of lists (mem = host,
 * pointers into buffer) and list_info (nullable); *nlists receives the frame's list count, *timestamp (nullable)
 * its time (the frame index before version 1.2). Lists without vertex data keep P2V_VERTDATA_NONE. */
P2V_API p2v_status p2v_mmpld_read_frame(p2v_mmpld* file, uint32_t frame, void* buffer, uint64_t capacity,
                                        p2v_particle_list* lists, p2v_mmpld_list_info* list_info, uint32_t max_lists,
                                        uint32_t* nlists, float* timestamp);
/* Pinned host memory for frame buffers (cudaMallocHost / cudaFreeHost). */
P2V_API void* p2v_host_alloc(uint64_t bytes);
P2V_API void p2v_host_free(void* ptr);

/* ---- learned AO ---- */
P2V_API void p2v_train_params_default(p2v_train_params* tp);
/* Run the frame with the plain cone march (current AO parameters, ao_mode forced to P2V_AO_CONE) and add
 * up to max_pairs (feature, cone-march AO) pairs, drawn uniformly with `seed`, to the training set.
 * *total receives the training-set size. The frame's lists must carry normals. */
P2V_API p2v_status p2v_mlp_collect(p2v_ctx* ctx, const p2v_frame* frame, uint32_t max_pairs, uint64_t seed,
                                   uint64_t* total);
P2V_API p2v_status p2v_mlp_clear(p2v_ctx* ctx);
/* The collected training pairs in collection order (P2V_MLP_INPUTS features and the cone-march AO per
 * pair; a pair without features, from a particle with a zero normal, has target -1). *count receives the
 * number of pairs; x (count x P2V_MLP_INPUTS) and t (count) are host arrays of capacity pairs, each
 * nullable. With max_pairs >= the frame's binned particles, p2v_mlp_collect takes every particle in the
 * sorted order of p2v_get_binning. */
P2V_API p2v_status p2v_mlp_get_pairs(p2v_ctx* ctx, float* x, float* t, uint64_t capacity, uint64_t* count);
/* Train the MLP on the collected pairs with FP32 forward/backward kernels and Adam. */
P2V_API p2v_status p2v_mlp_train(p2v_ctx* ctx, const p2v_train_params* tp, p2v_train_report* rep);
/* Flat binary file: header (magic, version, sizes, seed, Adam step), FP32 parameters, Adam moments,
 * feature ranges. */
P2V_API p2v_status p2v_mlp_save(p2v_ctx* ctx, const char* path);
P2V_API p2v_status p2v_mlp_load(p2v_ctx* ctx, const char* path);
/* FP32 parameters (P2V_MLP_PARAMS values). Setting them clears the feature ranges (no fallback). */
P2V_API p2v_status p2v_mlp_get_weights(p2v_ctx* ctx, float* out, uint64_t count);
P2V_API p2v_status p2v_mlp_set_weights(p2v_ctx* ctx, const float* in, uint64_t count);
/* One forward + backward pass of the training kernels on n given pairs (host arrays): gradient of
 * mean((y - t)^2) with respect to the parameters, and the loss. */
P2V_API p2v_status p2v_mlp_gradients(p2v_ctx* ctx, const float* x, const float* t, uint32_t n, float* grad,
                                     float* loss);
/* Tensor-core (BF16 x BF16 -> FP32) inference on n given feature rows (host arrays). */
P2V_API p2v_status p2v_mlp_infer(p2v_ctx* ctx, const float* x, uint32_t n, float* y);

/* ---- allocation-free AOSphere AO ----
 * No counterpart in the reference. For callers that cannot allocate device memory while computing AO
 * (a renderer recording its frame into a CUDA graph, a host that fixed the library's memory budget up
 * front, or a frame callback where cudaMalloc would stall the device). It computes what p2v_run_frame
 * computes for ao_mode P2V_AO_AOSPHERE_AXES / P2V_AO_AOSPHERE_NORMAL, from caller-provided device
 * buffers only: xyzr = count float4 (x, y, z, radius), normals = count float4 (x, y, z, unused),
 * ao_out = count floats, clipbox = ObjectSpaceClipBox, vol_size = "vol::sizex/y/z" including the border.
 * Its scratch is a static device array of P2V_NOALLOC_MAX_VOXELS voxels (3 MB, held by every GPU that
 * loads the library); larger volumes are rejected with P2V_EINVAL. The first call on a device looks up
 * that array's address (make it before any stream capture). Calls share the array: calls that overlap on
 * the GPU race. Asynchronous on `stream` (a cudaStream_t, NULL = the legacy default stream). */
#define P2V_NOALLOC_MAX_VOXELS 262144 /* 64^3 */
P2V_API p2v_status p2v_aosphere_ao_noalloc(const float* xyzr, const float* normals, uint64_t count,
                                           const float clipbox[6], const int32_t vol_size[3], float step_len,
                                           float gen_fac, float eval_fac, int32_t mode, float* ao_out, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* P2V_H */
