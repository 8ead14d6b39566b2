// C ABI of libp2v: context, parameters and the per-frame pipeline
// (pack + cell keys -> radix sort -> cell starts -> density gather -> statistics -> normalisation).
//
// Host-side semantics follow datatools::ParticlesToDensity (plugins/datatools/src/ParticlesToDensity.cpp):
// parameter defaults (:59-152), the surface-reconstruction box adjustment modifyBBox (:749-799), the
// grid geometry (:420-432) and the metadata it publishes (:249-293).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <memory>
#include <numeric>
#include <random>
#include <string>
#include <vector>

#include "../../include/p2v.h"
#include "p2v_common.cuh"
#include "ao_internal.h"
#include "mlp_internal.h"
#include "p2v_internal.h"

using namespace p2v;

namespace {

struct DevBuf {
    void* ptr = nullptr;
    size_t bytes = 0;
    cudaError_t ensure(size_t need) {
        if (need <= bytes)
            return cudaSuccess;
        if (ptr)
            cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
        size_t cap = need + need / 4 + 256;
        cudaError_t e = cudaMalloc(&ptr, cap);
        if (e == cudaSuccess)
            bytes = cap;
        return e;
    }
    void release() {
        if (ptr)
            cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
    }
    template<class T>
    T* as() const {
        return reinterpret_cast<T*>(ptr);
    }
};

enum Ev { EV_START, EV_UPLOAD, EV_BIN, EV_DENSITY, EV_NORM, EV_AO, EV_DOWN, EV_AOK0, EV_AOK1, EV_COUNT };
// fork/join events of a pipe's side stream: the normals upload runs under binning and density, the grid
// download under AO
enum SideEv { SEV_FORK, SEV_NRM, SEV_GRID, SEV_JOIN, SEV_COUNT };

// Scratch of one frame pipeline: every device buffer a frame touches, the stage timing events and the
// pinned mirror of the frame scalars. A context owns one pipe for p2v_run_frame and one per lane of
// p2v_run_batch; frames on different pipes may run concurrently.
struct Pipe {
    DevBuf raw, xyzr, rec_a, keys0, keys1, vals0, vals1, status, hist, cstart, gaps, grid, tiles, scal;
    DevBuf nrm, ao, mips, aos_acc, aos_tex, mdao_acc, mdao_vol, fb_list, wts, wsorted, wsum;
    DevBuf vdens, vdirs, vkeys0, vkeys1, vvals0, vvals1, vout;  // the vector aggregator's grid outputs
    DevBuf bcount;                         // particles per cell (the counting sort)
    DevBuf bstart;                         // start of every 64th cell (the radix path's cell starts)
    DevBuf xyzr_s, nrm_s;                  // positions and normals in sorted order (the cone AO stages)
    DevBuf bk0, bk1, xyzr_b, nrm_b, ord_b;  // the AO stages' brick order (ao_brick_order)
    bool xyzr_sorted = false;              // the binning of this frame wrote xyzr_s
    bool timing = false;                   // this frame records stage events
    bool aok = false;                      // EV_AOK0 / EV_AOK1 bracket this frame's main AO kernel
    uint32_t ao_fetches = 0;               // texture fetches per particle of the learned AO's inference
    FeatureTex ftex[MAX_LEVELS];           // the learned AO's feature levels as paired-slice textures
    cudaEvent_t ev[EV_COUNT] = {};
    cudaEvent_t sev[SEV_COUNT] = {};
    FrameScalars* h_scal = nullptr;        // pinned mirror of the last frame's scalars
    cudaStream_t stream = nullptr;         // the stream of a batch lane
    cudaStream_t side = nullptr;           // copies that overlap the frame's kernels
    ConeParams last_cp{};
    const float* last_grid = nullptr;
    const uint32_t* last_order = nullptr;  // sorted position -> particle index of the last frame
    const uint32_t* last_keys = nullptr;   // sorted bin keys of the last frame
    uint32_t last_n = 0, last_nbins = 0;
    uint64_t last_res[3] = {0, 0, 0};
    // the vector grid of the last frame (aggregator 2 with vector_grid)
    const uint32_t* vg_order = nullptr;
    VectorGridGeo vg_geo{};
    uint32_t vg_count = 0;
    float vg_radius = 0.0f, vg_bbox[6] = {}, vg_range[2] = {0.0f, 0.0f};

    cudaError_t init(bool with_stream) {
        for (auto& e : ev) {
            const cudaError_t r = cudaEventCreate(&e);
            if (r != cudaSuccess)
                return r;
        }
        for (auto& e : sev) {
            const cudaError_t r = cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
            if (r != cudaSuccess)
                return r;
        }
        {
            const cudaError_t r = cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking);
            if (r != cudaSuccess)
                return r;
        }
        if (with_stream) {
            const cudaError_t r = cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking);
            if (r != cudaSuccess)
                return r;
        }
        return cudaMallocHost(&h_scal, sizeof(FrameScalars));
    }
    void release() {
        if (stream)
            cudaStreamSynchronize(stream);
        for (DevBuf* b : {&raw, &xyzr, &rec_a, &keys0, &keys1, &vals0, &vals1, &status, &hist, &cstart, &gaps,
                          &grid, &tiles, &scal, &nrm, &ao, &mips, &aos_acc, &aos_tex, &mdao_acc, &mdao_vol, &fb_list,
                          &wts, &wsorted, &wsum, &vdens, &vdirs, &vkeys0, &vkeys1, &vvals0, &vvals1, &vout, &bcount, &bstart, &xyzr_s, &nrm_s, &bk0, &bk1, &xyzr_b, &nrm_b,
                          &ord_b})
            b->release();
        for (FeatureTex& t : ftex)
            t.release();
        if (side)
            cudaStreamSynchronize(side);
        for (auto& e : ev)
            if (e)
                cudaEventDestroy(e);
        for (auto& e : sev)
            if (e)
                cudaEventDestroy(e);
        if (h_scal)
            cudaFreeHost(h_scal);
        if (stream)
            cudaStreamDestroy(stream);
        if (side)
            cudaStreamDestroy(side);
        side = nullptr;
        h_scal = nullptr;
        stream = nullptr;
        last_grid = nullptr;
        last_order = nullptr;
        vg_order = nullptr;
    }
};

// One frame's buffers in a persistent batch: what the batch AO launch reads once every lane has finished
// (the lane's own buffers serve its next frame meanwhile), and the frame's descriptor for that launch.
struct BatchSlot {
    DevBuf xyzr_s, order, nrm_s, ao, grid, mips;
    DevBuf xyzr_b, ord_b, nrm_b;   // the march's brick order (ao_brick_order)
    BatchAoFrame* desc = nullptr;  // this frame's entry of the pinned descriptor table
    bool deferred = false;         // the frame's AO stage was left to the batch launch
    void release() {
        for (DevBuf* b : {&xyzr_s, &order, &nrm_s, &ao, &grid, &mips, &xyzr_b, &ord_b, &nrm_b})
            b->release();
    }
};

// Host-side state of a frame between its enqueue and its completion.
struct FrameJob {
    uint64_t N = 0;
    int32_t res[3] = {0, 0, 0};
    int32_t zlo = 0, zcount = 0;    // the z-slab the grid holds (zcount = res[2]: the whole grid)
    float bb[6] = {};
    const float* dgrid = nullptr;
    const uint32_t* order = nullptr;
    const uint32_t* keys = nullptr;
    uint32_t nbins = 0;
    int components = 1;
    const uint32_t* vg_order = nullptr;  // sorted vector grid (aggregator 2 with vector_grid), else null
    VectorGridGeo vg_geo{};
    FrameScalars* h_out = nullptr;  // pinned slot that receives the frame's scalars
    bool timed = false;             // stage events were recorded
    bool aok = false;               // the main AO kernel was bracketed by events
    uint32_t ao_fetches = 0;
};

__global__ void init_scalars_kernel(FrameScalars* fs) {
    FrameScalars z{};
    for (int a = 0; a < 3; ++a) {
        z.cmin[a] = INT32_MAX;
        z.cmax[a] = INT32_MIN;
    }
    z.dmin_bits = 0x7f7fffffu;  // FLT_MAX, as the vector aggregator's minDens starts
    *fs = z;
}

}  // namespace

struct p2v_ctx {
    int device = 0;
    int sms = 152;
    cudaStream_t own_stream = nullptr;
    p2v_params prm{};
    std::string err;
    p2v_stats stats{};
    uint64_t datahash = 0;

    Pipe main;                                  // p2v_run_frame
    std::vector<std::unique_ptr<Pipe>> lanes;   // p2v_run_batch
    // batches: pinned per-frame scalars, fork/join events, the captured graph and the shape it was captured for
    FrameScalars* b_scal = nullptr;
    size_t b_scal_cap = 0;
    std::vector<cudaEvent_t> b_events;
    cudaEvent_t b_t0 = nullptr, b_t1 = nullptr;
    cudaGraphExec_t b_exec = nullptr;
    std::vector<uint8_t> b_graph_sig, b_eager_sig;
    std::vector<FrameJob> b_jobs;
    std::vector<int> b_lane_of;
    // the persistent batch AO: per-frame buffers, pinned descriptor and segment tables, their device copies,
    // the queue words and the pinned mirror of the queue's error word
    std::vector<std::unique_ptr<BatchSlot>> b_slots;
    BatchAoFrame* b_frames_h = nullptr;
    size_t b_frames_cap = 0;
    BatchSeg* b_segs_h = nullptr;
    size_t b_segs_cap = 0;
    DevBuf b_frames_d, b_segs_d, b_words;
    uint32_t* b_err_h = nullptr;
    // autotuned choices (0 = none)
    int tuned_tile[3] = {0, 0, 0};
    int tuned_lanes = 0;
    int tuned_persistent = 0;
    // learned AO
    // p2v_run_ao_on_grid: the density grid the AO stage reads instead of this frame's own (null: none)
    const float* ext_grid = nullptr;
    int ext_grid_mem = P2V_MEM_HOST;
    DevBuf mlp_P, mlp_m, mlp_v, mlp_g, mlp_part, mlp_ploss, mlp_loss, mlp_w1h, mlp_w2h, mlp_lo, mlp_hi, mlp_idx,
        mlp_y;
    DevBuf tX, tT;                       // collected training pairs
    uint64_t t_pairs = 0, t_cap = 0;
    std::vector<uint32_t> t_valid;       // indices of pairs with features
    std::vector<float> t_host_T;         // targets on the host (validation error)
    bool mlp_ready = false, mlp_has_range = false;
    int mlp_step = 0;
    uint64_t mlp_seed = 0;

    p2v_status fail(p2v_status s, const char* fmt, ...) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        std::vsnprintf(buf, sizeof(buf), fmt, ap);
        va_end(ap);
        err = buf;
        return s;
    }

    p2v_status run_frame(const p2v_frame* fr, p2v_volume* vol, cudaStream_t st);
    p2v_status enqueue_frame(Pipe& pp, const p2v_frame* fr, p2v_volume* vol, cudaStream_t st, FrameScalars* h_out,
                             bool timed, FrameJob& job, BatchSlot* slot = nullptr);
    p2v_status finish_frame(Pipe& pp, const FrameJob& job, p2v_volume* vol, p2v_stats& out);
    p2v_status run_ao(Pipe& pp, const p2v_frame* fr, const GridGeo& g, const float* dgrid, const float bb[6],
                      uint32_t n, const uint32_t* order, cudaStream_t st, BatchSlot* slot);
    p2v_status build_cone(Pipe& pp, const p2v_frame* fr, const GridGeo& g, const float* dgrid, const float bb[6],
                          uint32_t n, const uint32_t* order, ConeParams& cp, cudaStream_t st, BatchSlot* slot);
    p2v_status enqueue_batch_ao(const p2v_batch_item* items, uint32_t count, const std::vector<uint32_t>& byw,
                                cudaStream_t st);
    p2v_status mlp_alloc();
    p2v_status prepare_features(Pipe& pp, ConeParams& cp, cudaStream_t st);
    p2v_status run_batch(const p2v_batch_item* items, uint32_t count, p2v_stats* out, cudaStream_t st,
                         bool allow_graph, float* ms_out);
    // the AO stage of a batch can run as the persistent launch (cone march of the density, one thread per
    // particle, a scalar grid)
    bool batch_persistent_possible() const {
        return prm.ao_mode == P2V_AO_CONE && prm.ao_volume == P2V_AOVOL_DENSITY && prm.ao_march == P2V_AO_MARCH_THREAD &&
               (prm.aggregator == 0 || prm.aggregator == 1);
    }
    bool batch_persistent_applies() const {
        const bool want = prm.batch_persistent < 0 ? tuned_persistent > 0 : prm.batch_persistent != 0;
        return want && batch_persistent_possible();
    }
    void drop_graph() {
        if (b_exec)
            cudaGraphExecDestroy(b_exec);
        b_exec = nullptr;
        b_graph_sig.clear();
    }
    void mlp_init_params(uint64_t seed, float bias3);
};

namespace {

// ParticlesToDensity::modifyBBox (ParticlesToDensity.cpp:749-799), in the same float arithmetic:
// grow the box by 10% plus two voxels in z, make voxels cubic and rewrite sizex / sizey. Returns false
// where the reference's float-to-int conversions would be undefined (a non-finite box, a box without
// depth, sizez < 1, or a width or height of 2^30 voxels or more); the caller reports the error.
bool modify_bbox(float bb[6], int32_t& sx, int32_t& sy, int32_t sz) {
    for (int a = 0; a < 6; ++a)
        if (!std::isfinite(bb[a]))
            return false;
    float rangeOSx = std::fabs(bb[3] - bb[0]), rangeOSy = std::fabs(bb[4] - bb[1]), rangeOSz = std::fabs(bb[5] - bb[2]);
    if (sz < 1 || !(rangeOSz > 0.0f))
        return false;
    float general_box_scaling = 1.1f;
    float spacing = (rangeOSz * general_box_scaling) / sz;
    float newDepth = (rangeOSz * general_box_scaling) + 2 * spacing;
    spacing = newDepth / sz;
    float newWidth = (rangeOSx * general_box_scaling) + 2 * spacing;
    const float qx = newWidth / spacing;  // the reference evaluates this quotient twice, with the same result
    if (!(qx < 1073741824.0f))
        return false;
    int resolutionX = static_cast<int>(qx);
    float rest = qx - static_cast<float>(resolutionX);
    newWidth += (1 - rest) * spacing;
    resolutionX += 1;
    sx = resolutionX;
    float newHeight = (rangeOSy * general_box_scaling) + 2 * spacing;
    const float qy = newHeight / spacing;
    if (!(qy < 1073741824.0f))
        return false;
    int resolutionY = static_cast<int>(qy);
    rest = qy - static_cast<float>(resolutionY);
    newHeight += (1 - rest) * spacing;
    resolutionY += 1;
    sy = resolutionY;
    float minOSx = bb[0], minOSy = bb[1], minOSz = bb[2], maxOSx = bb[3], maxOSy = bb[4], maxOSz = bb[5];
    bb[0] = minOSx - (newWidth - rangeOSx) / 2;
    bb[1] = minOSy - (newHeight - rangeOSy) / 2;
    bb[2] = minOSz - (newDepth - rangeOSz) / 2;
    bb[3] = maxOSx + (newWidth - rangeOSx) / 2;
    bb[4] = maxOSy + (newHeight - rangeOSy) / 2;
    bb[5] = maxOSz + (newDepth - rangeOSz) / 2;
    return true;
}

// SphereRenderer::generate3ConeDirections (SphereRenderer.cpp:2572-2587) for K = 3; other K use the
// same ring construction with the circumradius of a regular K-gon of that edge length.
void cone_directions(int K, float apex, float4* out) {
    const float edge = 2.0f * std::tan(0.5f * apex);
    const float height = std::sqrt(1.0f - edge * edge / 12.0f);
    const float radius = K == 3 ? std::sqrt(3.0f) / 3.0f * edge : edge / (2.0f * std::sin(3.14159265358979f / K));
    for (int i = 0; i < K; ++i) {
        const float angle = static_cast<float>(i) / static_cast<float>(K) * 2.0f * 3.14159265358979f;
        float c[3] = {std::cos(angle) * radius, height, std::sin(angle) * radius};
        const float l = std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
        out[i] = make_float4(c[0] / l, c[1] / l, c[2] / l, edge);
    }
}

// Sample distances and mip levels along a cone (mdao_deferred_fragment_ambocc.inc.glsl:35-51): t starts at
// offset + 1e-4 and grows by t*w until cone_length, or (steps > 0) follows a geometric sequence of that
// many samples ending below cone_length. lod = clamp(log2(t * w * shortestEdge), 0, maxLod).
int cone_steps(float offset, float cone_length, int steps, float w, float shortest, float max_lod, float* t,
               float* lod, int cap) {
    int n = 0;
    float tt = offset + 0.0001f;
    float gq = 0.0f;
    if (steps > 0)
        gq = std::pow(cone_length / tt, 1.0f / static_cast<float>(steps));
    while (n < cap) {
        float l = std::log2(tt * w * shortest);
        l = std::min(std::max(l, 0.0f), max_lod);
        t[n] = tt;
        lod[n] = l;
        ++n;
        if (steps > 0) {
            if (n >= steps)
                break;
            tt = tt * gq;
        } else {
            tt += tt * w;
            if (!(tt < cone_length))
                break;
        }
    }
    return n;
}

// bytes of one colour record (SimpleSphericalParticles.h:124-175); 0 = no per-particle colour
uint32_t colour_bytes(int type) {
    switch (type) {
    case P2V_COLDATA_UINT8_RGB: return 3;
    case P2V_COLDATA_UINT8_RGBA: return 4;
    case P2V_COLDATA_FLOAT_RGB: return 12;
    case P2V_COLDATA_FLOAT_RGBA: return 16;
    case P2V_COLDATA_FLOAT_I: return 4;
    case P2V_COLDATA_USHORT_RGBA: return 8;
    case P2V_COLDATA_DOUBLE_I: return 8;
    default: return 0;
    }
}

uint32_t record_bytes(int type) {
    switch (type) {
    case P2V_VERTDATA_FLOAT_XYZ: return 12;
    case P2V_VERTDATA_FLOAT_XYZR: return 16;
    case P2V_VERTDATA_SHORT_XYZ: return 6;
    case P2V_VERTDATA_DOUBLE_XYZ: return 24;
    default: return 0;
    }
}

}  // namespace

p2v_status p2v_ctx::run_frame(const p2v_frame* fr, p2v_volume* vol, cudaStream_t st) {
    P2V_CUDA_TRY(cudaSetDevice(device));
    FrameJob job;
    const p2v_status es = enqueue_frame(main, fr, vol, st, main.h_scal, true, job);
    if (es != P2V_OK)
        return es;
    P2V_CUDA_TRY(cudaStreamSynchronize(st));
    return finish_frame(main, job, vol, stats);
}

// Validate the frame and queue its whole pipeline on `st` using the buffers of `pp`; the frame scalars are
// copied to the pinned slot h_out at the end. Nothing here waits for the device.
p2v_status p2v_ctx::enqueue_frame(Pipe& pp, const p2v_frame* fr, p2v_volume* vol, cudaStream_t st,
                                  FrameScalars* h_out, bool timed, FrameJob& job, BatchSlot* slot) {
    DevBuf &raw = pp.raw, &xyzr = pp.xyzr, &rec_a = pp.rec_a, &keys0 = pp.keys0,
           &keys1 = pp.keys1, &vals0 = pp.vals0, &vals1 = pp.vals1, &status = pp.status, &hist = pp.hist,
           &cstart = pp.cstart, &gaps = pp.gaps, &grid = pp.grid, &tiles = pp.tiles, &scal = pp.scal, &nrm = pp.nrm,
           &ao = pp.ao;
    cudaEvent_t* ev = pp.ev;
    const p2v_params& P = prm;
    // aggregator: 0 PosToSingleCell_Volume, 1 IColToSingleCell_Volume, 2 IVecToSingleCell_Volume
    // (ParticlesToDensity.cpp:78-81)
    if (P.aggregator < 0 || P.aggregator > 2)
        return fail(P2V_EINVAL, "aggregator %d is not 0, 1 or 2", P.aggregator);
    const int agg = P.aggregator;
    const int wnc = agg == 1 ? 1 : (agg == 2 ? 3 : 0);      // weights per particle
    const int comps = agg == 2 ? 3 : 1;                       // volume components
    if (agg != 0 && P.accumulate != P2V_ACCUM_EXACT)
        return fail(P2V_EUNSUPPORTED, "aggregator %d needs the exact accumulation", agg);
    if (agg != 0 && P.mass_normalize)
        return fail(P2V_EINVAL, "mass normalisation applies to the density aggregator only");
    if (agg == 2 && P.ao_mode != P2V_AO_NONE && P.ao_volume == P2V_AOVOL_DENSITY)
        return fail(P2V_EUNSUPPORTED, "the cone-march AO of a density volume needs a scalar grid (aggregator 0/1)");
    if (!(P.sigma > 0.0f) || !std::isfinite(P.sigma))
        return fail(P2V_EINVAL, "sigma must be a positive finite number");
    if (P.kernel != P2V_KERNEL_BUMP && P.kernel != P2V_KERNEL_GAUSS3)
        return fail(P2V_EINVAL, "unknown kernel %d", P.kernel);
    if (fr->list_count > 0 && fr->lists == nullptr)
        return fail(P2V_EINVAL, "frame has lists but no list array");

    float bb[6];
    std::memcpy(bb, fr->bbox, sizeof(bb));
    int32_t res[3] = {P.sizex, P.sizey, P.sizez};
    if (P.forSurfaceReconstruction) {
        if (!modify_bbox(bb, res[0], res[1], res[2]))
            return fail(P2V_EINVAL, "forSurfaceReconstruction needs a finite box with depth and sizez >= 1, and at "
                                    "most 2^30 voxels along x and y");
        prm.sizex = res[0];
        prm.sizey = res[1];
    }
    GridGeo g{};
    uint64_t nb = 1;
    for (int a = 0; a < 3; ++a) {
        if (res[a] < 2 || res[a] > 4096)
            return fail(P2V_EINVAL, "size%c = %d: every resolution must lie in [2, 4096]", "xyz"[a], res[a]);
        if (!std::isfinite(bb[a]) || !std::isfinite(bb[a + 3]))
            return fail(P2V_EINVAL, "bounding box is not finite");
        g.s[a] = res[a];
        g.cyc[a] = (a == 0 ? P.cyclX : a == 1 ? P.cyclY : P.cyclZ) ? 1 : 0;
        const float lo = bb[a], hi = bb[a + 3];
        const float rangef = hi > lo ? hi - lo : lo - hi;  // vislib Cuboid::Width()
        if (!(rangef > 0.0f))
            return fail(P2V_EINVAL, "bounding box has zero extent along %c", "xyz"[a]);
        g.minf[a] = lo;
        g.hf[a] = rangef / static_cast<float>(res[a] - 1);
        const double hd = std::fabs((double) hi - (double) lo) / (double) (res[a] - 1);
        g.hhi[a] = (float) hd;
        g.hlo[a] = (float) (hd - (double) g.hhi[a]);
        g.ihh[a] = (float) (1.0 / (double) g.hhi[a]);
        g.nb[a] = (uint32_t) res[a] + 2u;
        nb *= g.nb[a];
    }
    if (nb >= 0xFFFFFFF0ull)
        return fail(P2V_EINVAL, "grid too large for 32-bit cell keys");
    g.nbins = (uint32_t) nb;
    g.sigma = P.sigma;
    g.kernel = P.kernel;
    // the planes computed: a z-slab of the grid, or all of it
    g.zlo = 0;
    g.zhi = res[2];
    if (P.slab_z0 != 0 || P.slab_z1 != 0) {
        if (P.slab_z0 < 0 || P.slab_z1 <= P.slab_z0 || P.slab_z1 > res[2])
            return fail(P2V_EINVAL, "slab [%d, %d) is not a non-empty range of the %d planes", P.slab_z0, P.slab_z1,
                        res[2]);
        if (agg == 2 || P.ao_mode != P2V_AO_NONE)
            return fail(P2V_EUNSUPPORTED, "a z-slab serves the density and intensity aggregators without AO");
        g.zlo = P.slab_z0;
        g.zhi = P.slab_z1;
    }
    const uint64_t V = (uint64_t) res[0] * res[1] * (uint64_t) (g.zhi - g.zlo);
    const uint64_t VC = V * (uint64_t) comps;

    uint64_t N = 0;
    for (uint32_t l = 0; l < fr->list_count; ++l) {
        const p2v_particle_list& L = fr->lists[l];
        if (L.vertex_type == P2V_VERTDATA_NONE)
            continue;
        if (record_bytes(L.vertex_type) == 0)
            return fail(P2V_EINVAL, "list %u: unknown vertex type %d", l, L.vertex_type);
        if (L.count > 0 && L.vertex_data == nullptr)
            return fail(P2V_EINVAL, "list %u: no vertex data", l);
        N += L.count;
    }
    if (N >= (1ull << 30))
        return fail(P2V_EINVAL, "%llu particles: at most 2^30 - 1 per frame", (unsigned long long) N);

    // ---- buffers ----
    const uint32_t n = (uint32_t) N;
    GatherConfig gc{};
    if (P.accumulate == P2V_ACCUM_KAHAN) {
        gc = GatherConfig{GATHER_KAHAN, 8, 16, 16, 2048, 1024};
    } else if (P.accumulate == P2V_ACCUM_EXACT) {
        gc = GatherConfig{GATHER_EXACT, 16, 16, 16, 0, 1024};
        if (P.tile_x > 0 || P.tile_y > 0 || P.tile_z > 0)
            gc = GatherConfig{GATHER_EXACT, P.tile_x, P.tile_y, P.tile_z, 0, 1024};
        else if (tuned_tile[0] > 0)
            gc = GatherConfig{GATHER_EXACT, tuned_tile[0], tuned_tile[1], tuned_tile[2], 0, 1024};
    } else {
        return fail(P2V_EINVAL, "unknown accumulate mode %d", P.accumulate);
    }
    const uint32_t ntiles = gather_tile_count(gc, g);
    const uint32_t gap_cap = g.nbins / 64 + 2;
    P2V_CUDA_TRY(xyzr.ensure(sizeof(float4) * (N + 1)));
    P2V_CUDA_TRY(rec_a.ensure(2 * sizeof(float4) * (N + 1)));  // interleaved 32-byte records
    P2V_CUDA_TRY(keys0.ensure(4 * (N + 1)));
    P2V_CUDA_TRY(keys1.ensure(4 * (N + 1)));
    P2V_CUDA_TRY(vals0.ensure(4 * (N + 1)));
    P2V_CUDA_TRY(vals1.ensure(4 * (N + 1)));
    // the counting sort by cell while its cell table stays near L2-resident: it passes over the table about
    // four times (16 bytes per cell) and scatters every particle by a table lookup and an atomic, cheap while
    // the table sits in L2; a table of hundreds of MB turns every lookup into a DRAM sector, where the radix
    // sort's streaming passes (~150 bytes per particle) win
    const bool counting = n > 0 && (uint64_t) g.nbins + 1 <= 64ull * n &&
                          4ull * ((uint64_t) g.nbins + 1) <= COUNTING_TABLE_MAX_BYTES;
    if (counting)
        P2V_CUDA_TRY(pp.bcount.ensure(4 * ((size_t) g.nbins + 1)));
    // the radix path sorts particles whose support holds no node after all others (a key bit above the cells),
    // so the density gather never visits them; the AO stages' brick order reads the cell table for every
    // particle and keeps plain cell keys
    const uint32_t empty_flag = (!counting && P.ao_brick_order == 0) ? sort_empty_flag(g.nbins) : 0u;
    P2V_CUDA_TRY(status.ensure(4 * (std::max(sort_status_words(n), bin_scan_words(g.nbins)) + 256)));
    P2V_CUDA_TRY(hist.ensure(4 * sort_hist_words()));
    P2V_CUDA_TRY(cstart.ensure(4 * ((size_t) g.nbins + 1)));
    P2V_CUDA_TRY(gaps.ensure(sizeof(uint4) * gap_cap));
    P2V_CUDA_TRY(tiles.ensure(sizeof(TileStats) * ntiles));
    P2V_CUDA_TRY(scal.ensure(sizeof(FrameScalars)));
    float* dgrid;
    const bool direct = vol && vol->data && vol->mem == P2V_MEM_DEVICE && vol->capacity >= VC;
    if (direct) {
        dgrid = vol->data;
    } else if (slot) {  // read by the batch AO launch after the lane has moved on
        P2V_CUDA_TRY(slot->grid.ensure(sizeof(float) * VC));
        dgrid = slot->grid.as<float>();
    } else {
        P2V_CUDA_TRY(grid.ensure(sizeof(float) * VC));
        dgrid = grid.as<float>();
    }
    if (vol && vol->data && vol->capacity < VC)
        return fail(P2V_EINVAL, "output capacity %llu < %llu floats", (unsigned long long) vol->capacity,
                    (unsigned long long) VC);
    if (wnc) {
        P2V_CUDA_TRY(pp.wts.ensure(sizeof(float) * wnc * (N + 1)));
        P2V_CUDA_TRY(pp.wsorted.ensure(sizeof(float) * wnc * (N + 1)));
        if (agg == 2)
            P2V_CUDA_TRY(pp.wsum.ensure(sizeof(float) * V));
    }
    const bool vgrid = agg == 2 && P.vector_grid;
    if (vgrid) {
        if (V >= (1ull << 31))
            return fail(P2V_EINVAL, "the vector grid holds at most 2^31 - 1 nodes");
        P2V_CUDA_TRY(pp.vdens.ensure(sizeof(float) * V));
        P2V_CUDA_TRY(pp.vdirs.ensure(sizeof(float) * 3 * V));
        P2V_CUDA_TRY(pp.vkeys0.ensure(sizeof(uint32_t) * V));
        P2V_CUDA_TRY(pp.vkeys1.ensure(sizeof(uint32_t) * V));
        P2V_CUDA_TRY(pp.vvals0.ensure(sizeof(uint32_t) * V));
        P2V_CUDA_TRY(pp.vvals1.ensure(sizeof(uint32_t) * V));
        P2V_CUDA_TRY(status.ensure(4 * (sort_status_words((uint32_t) V) + 256)));
    }

    FrameScalars* fs = scal.as<FrameScalars>();
    if (timed)
        P2V_CUDA_TRY(cudaEventRecord(ev[EV_START], st));
    init_scalars_kernel<<<1, 1, 0, st>>>(fs);

    // ---- upload + pack + keys ----
    uint64_t raw_need = 0;
    for (uint32_t l = 0; l < fr->list_count; ++l) {
        const p2v_particle_list& L = fr->lists[l];
        if (L.vertex_type == P2V_VERTDATA_NONE || L.count == 0 || L.mem == P2V_MEM_DEVICE)
            continue;
        const uint32_t stride = L.vertex_stride ? L.vertex_stride : record_bytes(L.vertex_type);
        raw_need += (L.count - 1) * (uint64_t) stride + record_bytes(L.vertex_type) + 16;
        if ((P.ao_mode != P2V_AO_NONE || agg == 2) && L.normals != nullptr) {
            const uint32_t ns = L.normal_stride ? L.normal_stride : 12u;
            raw_need += 2 * ((L.count - 1) * (uint64_t) ns + 12 + 16);
        }
        if (agg == 1 && L.colour_data != nullptr && colour_bytes(L.colour_type) > 0) {
            const uint32_t cs = L.colour_stride ? L.colour_stride : colour_bytes(L.colour_type);
            raw_need += (L.count - 1) * (uint64_t) cs + colour_bytes(L.colour_type) + 16;
        }
    }
    if (raw_need)
        P2V_CUDA_TRY(raw.ensure(raw_need));
    uint64_t raw_off = 0, off = 0;
    for (uint32_t l = 0; l < fr->list_count; ++l) {
        const p2v_particle_list& L = fr->lists[l];
        if (L.vertex_type == P2V_VERTDATA_NONE)
            continue;
        const uint32_t rb = record_bytes(L.vertex_type);
        const uint32_t stride = L.vertex_stride ? L.vertex_stride : rb;
        if (stride < rb)
            return fail(P2V_EINVAL, "list %u: stride %u shorter than a record (%u)", l, stride, rb);
        ListDesc d{};
        d.stride = stride;
        d.type = L.vertex_type;
        d.global_radius = L.global_radius;
        d.count = L.count;
        d.offset = off;
        if (L.count > 0) {
            if (L.mem == P2V_MEM_DEVICE) {
                d.data = static_cast<const uint8_t*>(L.vertex_data);
            } else {
                const uint64_t bytes = (L.count - 1) * (uint64_t) stride + rb;
                uint8_t* dst = raw.as<uint8_t>() + raw_off;
                P2V_CUDA_TRY(cudaMemcpyAsync(dst, L.vertex_data, bytes, cudaMemcpyHostToDevice, st));
                d.data = dst;
                raw_off += (bytes + 15) & ~uint64_t(15);
            }
        }
        P2V_CUDA_TRY(launch_pack_keys(d, g, xyzr.as<float4>(), keys0.as<uint32_t>(), nullptr, fs, empty_flag, st));
        off += L.count;
    }
    if (timed)
        P2V_CUDA_TRY(cudaEventRecord(ev[EV_UPLOAD], st));
    // ---- normals for AO, on the side stream: needed only by the AO stage ----
    const bool want_ao = P.ao_mode != P2V_AO_NONE;
    const bool list_normals = P.ao_normals == P2V_NORMALS_LIST;  // else computed from the grid in the AO stage
    cudaStream_t side = pp.side;
    if (want_ao) {
        if (P.ao_normals != P2V_NORMALS_LIST && P.ao_normals != P2V_NORMALS_GRADIENT)
            return fail(P2V_EINVAL, "ao_normals %d is not a p2v_ao_normals", P.ao_normals);
        if (!list_normals && agg == 2)
            return fail(P2V_EINVAL, "gradient normals need a scalar grid (aggregator 0 or 1)");
        P2V_CUDA_TRY(nrm.ensure(sizeof(float4) * (N + 1)));
        P2V_CUDA_TRY(ao.ensure(sizeof(float) * (N + 1)));
        // every check before the fork: an error return must not leave work on the side stream
        uint64_t nbytes = 0;
        for (uint32_t l = 0; l < fr->list_count && list_normals; ++l) {
            const p2v_particle_list& L = fr->lists[l];
            if (L.vertex_type == P2V_VERTDATA_NONE || L.count == 0)
                continue;
            if (L.normals == nullptr)
                return fail(P2V_EINVAL, "list %u: AO needs per-particle normals", l);
            const uint32_t ns = L.normal_stride ? L.normal_stride : 12u;
            if (ns < 12u)
                return fail(P2V_EINVAL, "list %u: normal stride %u < 12", l, ns);
            if (L.mem != P2V_MEM_DEVICE)
                nbytes += (((L.count - 1) * (uint64_t) ns + 12) + 15) & ~uint64_t(15);
        }
        if (raw_off + nbytes > raw.bytes)
            return fail(P2V_EINVAL, "normals larger than the staging buffer");
        // ordered after everything queued on st so far (the previous frame's AO still reads nrm and raw)
        P2V_CUDA_TRY(cudaEventRecord(pp.sev[SEV_FORK], st));
        P2V_CUDA_TRY(cudaStreamWaitEvent(side, pp.sev[SEV_FORK], 0));
        uint64_t noff = 0;
        for (uint32_t l = 0; l < fr->list_count && list_normals; ++l) {
            const p2v_particle_list& L = fr->lists[l];
            if (L.vertex_type == P2V_VERTDATA_NONE)
                continue;
            if (L.count > 0) {
                const uint32_t ns = L.normal_stride ? L.normal_stride : 12u;
                const void* src = L.normals;
                if (L.mem != P2V_MEM_DEVICE) {
                    const uint64_t bytes = (L.count - 1) * (uint64_t) ns + 12;
                    uint8_t* dst = raw.as<uint8_t>() + raw_off;
                    P2V_CUDA_TRY(cudaMemcpyAsync(dst, L.normals, bytes, cudaMemcpyHostToDevice, side));
                    src = dst;
                    raw_off += (bytes + 15) & ~uint64_t(15);
                }
                P2V_CUDA_TRY(launch_pack_normals(src, ns, L.count, noff, nrm.as<float4>(), side));
            }
            noff += L.count;
        }
        P2V_CUDA_TRY(cudaEventRecord(pp.sev[SEV_NRM], side));
    }

    // ---- weights of the intensity / vector aggregators ----
    if (wnc) {
        uint64_t woff = 0;
        for (uint32_t l = 0; l < fr->list_count; ++l) {
            const p2v_particle_list& L = fr->lists[l];
            if (L.vertex_type == P2V_VERTDATA_NONE)
                continue;
            if (L.count > 0) {
                WeightSource ws{};
                ws.count = L.count;
                ws.offset = woff;
                const void* src = agg == 1 ? L.colour_data : static_cast<const void*>(L.normals);
                uint32_t rb = agg == 1 ? colour_bytes(L.colour_type) : 12u;
                uint32_t stride = agg == 1 ? (L.colour_stride ? L.colour_stride : rb) : (L.normal_stride ? L.normal_stride : 12u);
                if (agg == 2 && src == nullptr)
                    return fail(P2V_EINVAL, "list %u: the vector aggregator needs directions (normals)", l);
                if (agg == 1 && (src == nullptr || rb == 0)) {
                    src = nullptr;  // the global colour's red channel, normalised (Accessor_Val<uchar, true>)
                    ws.global_i = static_cast<float>(L.global_colour[0]) / static_cast<float>(255);
                }
                if (src != nullptr && L.mem != P2V_MEM_DEVICE) {
                    const uint64_t bytes = (L.count - 1) * (uint64_t) stride + rb;
                    uint8_t* dst = raw.as<uint8_t>() + raw_off;
                    if (raw_off + bytes > raw.bytes)
                        return fail(P2V_EINVAL, "list %u: weight data larger than the staging buffer", l);
                    P2V_CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st));
                    src = dst;
                    raw_off += (bytes + 15) & ~uint64_t(15);
                }
                ws.data = static_cast<const uint8_t*>(src);
                ws.stride = stride;
                ws.ctype = L.colour_type;
                P2V_CUDA_TRY(launch_pack_weights(ws, wnc, pp.wts.as<float>(), fs, sms, st));
            }
            woff += L.count;
        }
    }

    // ---- sort + cell starts ----
    SortBuffers sb{};
    sb.keys[0] = keys0.as<uint32_t>();
    sb.keys[1] = keys1.as<uint32_t>();
    sb.vals[0] = vals0.as<uint32_t>();
    sb.vals[1] = vals1.as<uint32_t>();
    sb.implicit_vals0 = true;  // no index list was packed: the first radix pass takes the identity
    sb.empty_flag = empty_flag;
    sb.hist = hist.as<uint32_t>();
    sb.status = status.as<uint32_t>();
    sb.err = &fs->error;
    sb.xyzr_in = xyzr.as<float4>();
    sb.rec_a = rec_a.as<float4>();
    sb.rec_b = reinterpret_cast<int4*>(rec_a.as<float4>() + 1);
    // the cone-march stages read the positions in sorted order: the binning's last pass writes them
    pp.xyzr_sorted = P.ao_mode == P2V_AO_CONE || P.ao_mode == P2V_AO_LEARNED;
    if (pp.xyzr_sorted) {
        DevBuf& xs = slot ? slot->xyzr_s : pp.xyzr_s;
        P2V_CUDA_TRY(xs.ensure(sizeof(float4) * ((size_t) n + 1)));
        sb.xyzr_out = xs.as<float4>();
    }
    sb.geo = g;
    if (P.sort_wait_polls < 0)
        return fail(P2V_EINVAL, "sort_wait_polls must be >= 0");
    sb.wait_polls = (uint32_t) P.sort_wait_polls;
    sb.hold_tile = P.test_hold_sort ? 1 : -1;
    P2V_CUDA_TRY(pp.bstart.ensure(4 * ((size_t) cell_block_count(g.nbins) + 1)));
    P2V_CUDA_TRY(launch_bin_sort(sb, n, g, counting ? pp.bcount.as<uint32_t>() : nullptr, cstart.as<uint32_t>(),
                                 pp.bstart.as<uint32_t>(), gaps.as<uint4>(), gap_cap, fs, sms, st));
    const uint32_t* skeys = sb.keys[sb.result];
    if (slot) {
        slot->deferred = false;
        if (want_ao && n > 0) {  // the sorted order outlives the lane's sort buffers
            P2V_CUDA_TRY(slot->order.ensure(sizeof(uint32_t) * ((size_t) n + 1)));
            P2V_CUDA_TRY(cudaMemcpyAsync(slot->order.ptr, sb.vals[sb.result], sizeof(uint32_t) * n,
                                         cudaMemcpyDeviceToDevice, st));
        }
    }
    if (timed)
        P2V_CUDA_TRY(cudaEventRecord(ev[EV_BIN], st));

    // ---- density ----
    if (wnc)
        P2V_CUDA_TRY(launch_permute_weights(sb.vals[sb.result], pp.wts.as<float>(), pp.wsorted.as<float>(), n, wnc, sms,
                                            st));
    if (ext_grid) {
        // p2v_run_ao_on_grid: the caller's grid stands in for this frame's density (no gather, no statistics)
        P2V_CUDA_TRY(cudaMemcpyAsync(dgrid, ext_grid, sizeof(float) * V,
                                     ext_grid_mem == P2V_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                                     st));
    } else {
        // aggregator 0: the density; 1: the intensity-weighted sums; 2: three direction-weighted passes into
        // the interleaved vector volume and the plain kernel sums (the weights) into wsum
        const int passes = agg == 2 ? 4 : 1;
        for (int pass = 0; pass < passes; ++pass) {
            GatherWeights gw{};
            float* out = dgrid;
            if (agg == 1) {
                gw.mode = GatherWeights::FIXED;
                gw.w = pp.wsorted.as<float>();
            } else if (agg == 2 && pass < 3) {
                gw.mode = GatherWeights::DOUBLE;
                gw.w = pp.wsorted.as<float>() + pass;
                gw.wstride = 3;
                gw.ostride = 3;
                out = dgrid + pass;
            } else if (agg == 2) {
                gw.mode = GatherWeights::DOUBLE;  // the weights: plain kernel sums in FP64
                out = pp.wsum.as<float>();
            }
            const cudaError_t ge = launch_gather(gc, g, sb.rec_a, sb.rec_b, cstart.as<uint32_t>(),
                                                 out, tiles.as<TileStats>(), fs, st, gw);
            if (ge == cudaErrorInvalidValue)
                return fail(P2V_EUNSUPPORTED, "density tile %dx%dx%d is not compiled for accumulate=%d", gc.tx, gc.ty,
                            gc.tz, P.accumulate);
            P2V_CUDA_TRY(ge);
        }
    }
    if (timed)
        P2V_CUDA_TRY(cudaEventRecord(ev[EV_DENSITY], st));
    const double voxel_volume = (double) g.hhi[0] * g.hhi[1] * g.hhi[2];
    const uint32_t* vg_order = nullptr;
    if (agg == 2) {
        VectorGridBufs vb{pp.vdens.as<float>(), pp.vdirs.as<float>(), pp.vkeys0.as<uint32_t>(),
                          pp.vvals0.as<uint32_t>()};
        P2V_CUDA_TRY(launch_vector_finish(dgrid, pp.wsum.as<float>(), (int64_t) V, fs, P.normalize, sms, st,
                                          vgrid ? &vb : nullptr));
        P2V_CUDA_TRY(launch_normalize_modes(dgrid, VC, fs, 0, P.normalize, sms, st));
        if (vgrid) {
            // densities descending, equal densities in node order: a stable sort of ~bits(density)
            SortBuffers vs{};
            vs.keys[0] = pp.vkeys0.as<uint32_t>();
            vs.keys[1] = pp.vkeys1.as<uint32_t>();
            vs.vals[0] = pp.vvals0.as<uint32_t>();
            vs.vals[1] = pp.vvals1.as<uint32_t>();
            vs.hist = hist.as<uint32_t>();
            vs.status = status.as<uint32_t>();
            vs.err = &fs->error;
            P2V_CUDA_TRY(launch_sort(vs, (uint32_t) V, 0xFFFFFFFFu, sms, st));
            vg_order = vs.vals[vs.result];
        }
    } else if (!ext_grid) {
        P2V_CUDA_TRY(launch_finalize(tiles.as<TileStats>(), ntiles, fs, P.mass_normalize, P.normalize, 0.0, voxel_volume,
                                     st));
        P2V_CUDA_TRY(launch_normalize_modes(dgrid, V, fs, P.mass_normalize, P.normalize, sms, st));
    }
    if (timed)
        P2V_CUDA_TRY(cudaEventRecord(ev[EV_NORM], st));
    // the grid is final here and AO only reads it: with AO its download runs on the side stream meanwhile
    const bool grid_out = vol && vol->data && !direct;
    const cudaMemcpyKind grid_kind = vol && vol->mem == P2V_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    if (want_ao) {
        if (grid_out) {
            P2V_CUDA_TRY(cudaEventRecord(pp.sev[SEV_GRID], st));
            P2V_CUDA_TRY(cudaStreamWaitEvent(side, pp.sev[SEV_GRID], 0));
            P2V_CUDA_TRY(cudaMemcpyAsync(vol->data, dgrid, sizeof(float) * VC, grid_kind, side));
        }
        P2V_CUDA_TRY(cudaEventRecord(pp.sev[SEV_JOIN], side));
        P2V_CUDA_TRY(cudaStreamWaitEvent(st, pp.sev[SEV_NRM], 0));
        pp.timing = timed && !slot;
        pp.aok = false;
        pp.ao_fetches = 0;
        const p2v_status as = run_ao(pp, fr, g, dgrid, bb, n, sb.vals[sb.result], st, slot);
        if (as != P2V_OK) {
            cudaStreamWaitEvent(st, pp.sev[SEV_JOIN], 0);  // no side work left outside st (graph capture)
            return as;
        }
    }
    if (timed)
        P2V_CUDA_TRY(cudaEventRecord(ev[EV_AO], st));

    // ---- outputs ----
    if (grid_out && !want_ao)
        P2V_CUDA_TRY(cudaMemcpyAsync(vol->data, dgrid, sizeof(float) * VC, grid_kind, st));
    if (want_ao && !(slot && slot->deferred)) {  // a deferred frame's AO is copied out after the batch launch
        uint64_t aoff = 0;
        for (uint32_t l = 0; l < fr->list_count; ++l) {
            const p2v_particle_list& L = fr->lists[l];
            if (L.vertex_type == P2V_VERTDATA_NONE)
                continue;
            if (L.ao_out && L.count > 0)
                P2V_CUDA_TRY(cudaMemcpyAsync(L.ao_out, ao.as<float>() + aoff, sizeof(float) * L.count,
                                             L.mem == P2V_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                                             st));
            aoff += L.count;
        }
    }
    if (want_ao)
        P2V_CUDA_TRY(cudaStreamWaitEvent(st, pp.sev[SEV_JOIN], 0));
    P2V_CUDA_TRY(cudaMemcpyAsync(h_out, fs, sizeof(FrameScalars), cudaMemcpyDeviceToHost, st));
    if (timed)
        P2V_CUDA_TRY(cudaEventRecord(ev[EV_DOWN], st));
    job.N = N;
    for (int a = 0; a < 3; ++a)
        job.res[a] = res[a];
    job.zlo = g.zlo;
    job.zcount = g.zhi - g.zlo;
    std::memcpy(job.bb, bb, sizeof(bb));
    job.dgrid = dgrid;
    job.order = sb.vals[sb.result];
    job.keys = skeys;
    job.nbins = g.nbins;
    job.components = comps;
    job.vg_order = vg_order;
    for (int a = 0; a < 3; ++a) {
        job.vg_geo.minf[a] = g.minf[a];
        job.vg_geo.hf[a] = g.hf[a];
        job.vg_geo.res[a] = res[a];
    }
    job.vg_geo.normalize = P.normalize ? 1 : 0;
    job.h_out = h_out;
    job.timed = timed;
    job.aok = want_ao && pp.aok;
    job.ao_fetches = want_ao ? pp.ao_fetches : 0u;
    return P2V_OK;
}

// Statistics, metadata and error status of a completed frame (its stream has been synchronised).
p2v_status p2v_ctx::finish_frame(Pipe& pp, const FrameJob& job, p2v_volume* vol, p2v_stats& stats) {
    const uint64_t N = job.N;
    const int32_t* res = job.res;
    const float* bb = job.bb;
    const float* dgrid = job.dgrid;
    cudaEvent_t* ev = pp.ev;
    auto& last_grid = pp.last_grid;
    auto& last_order = pp.last_order;
    auto& last_res = pp.last_res;
    const FrameScalars& hs = *job.h_out;
    last_grid = dgrid;
    last_order = job.order;
    // the vector grid: ParticlesToDensity.cpp:306-323 (global radius = bbox width / sizex / 5) and :358-377
    // (column ranges: the bbox, [-1, 1] for the directions, the published density range)
    pp.vg_order = job.vg_order;
    pp.vg_geo = job.vg_geo;
    pp.vg_count = job.vg_order ? job.h_out->vcount : 0u;
    std::memcpy(pp.vg_bbox, bb, sizeof(pp.vg_bbox));
    {
        const float w = bb[3] > bb[0] ? bb[3] - bb[0] : bb[0] - bb[3];
        pp.vg_radius = w / static_cast<float>(res[0]) / 5.0f;
    }
    pp.vg_range[0] = job.h_out->out_min;
    pp.vg_range[1] = job.h_out->out_max;
    pp.last_keys = job.keys;
    pp.last_n = (uint32_t) job.N;
    pp.last_nbins = job.nbins;
    for (int a = 0; a < 3; ++a)
        last_res[a] = (uint64_t) res[a];
    last_res[2] = (uint64_t) job.zcount;  // the planes the grid holds (a z-slab or all)
    stats = p2v_stats{};
    stats.particles_in = N;
    stats.particles_binned = hs.n_valid;
    stats.particles_dropped = hs.n_dropped;
    std::memcpy(&stats.radius_max, &hs.rmax_bits, sizeof(float));
    for (int a = 0; a < 3; ++a) {
        stats.cell_min[a] = hs.cmin[a];
        stats.cell_max[a] = hs.cmax[a];
    }
    stats.mass_sum = hs.mass;
    float ms = 0.0f;
    if (job.timed) {
    cudaEventElapsedTime(&ms, ev[EV_START], ev[EV_UPLOAD]);
    stats.ms_upload = ms;
    cudaEventElapsedTime(&ms, ev[EV_UPLOAD], ev[EV_BIN]);
    stats.ms_binning = ms;
    cudaEventElapsedTime(&ms, ev[EV_BIN], ev[EV_DENSITY]);
    stats.ms_density = ms;
    cudaEventElapsedTime(&ms, ev[EV_DENSITY], ev[EV_NORM]);
    stats.ms_normalize = ms;
    cudaEventElapsedTime(&ms, ev[EV_NORM], ev[EV_AO]);
    stats.ms_ao = ms;
    cudaEventElapsedTime(&ms, ev[EV_AO], ev[EV_DOWN]);
    stats.ms_download = ms;
    cudaEventElapsedTime(&ms, ev[EV_START], ev[EV_DOWN]);
    stats.ms_total = ms;
    if (job.aok && cudaEventElapsedTime(&ms, ev[EV_AOK0], ev[EV_AOK1]) == cudaSuccess)
        stats.ms_ao_kernel = ms;
    }
    stats.ao_fetches = job.ao_fetches;
    stats.device_error = hs.error;
    stats.ao_fallback = hs.ao_fallback;
    stats.cell_max_count = hs.bin_maxcount;

    if (vol) {
        for (int a = 0; a < 3; ++a) {
            vol->resolution[a] = (uint64_t) res[a];
            const float rangef = std::fabs(bb[a + 3] - bb[a]);
            vol->extents[a] = rangef;
            vol->slice_dists[a] = rangef / static_cast<float>(res[a] - 1);
            vol->origin[a] = bb[a];
        }
        if (job.zcount != res[2]) {  // a z-slab: its planes, first plane and extent
            vol->resolution[2] = (uint64_t) job.zcount;
            vol->origin[2] = bb[2] + static_cast<float>(job.zlo) * vol->slice_dists[2];
            vol->extents[2] = static_cast<float>(job.zcount - 1) * vol->slice_dists[2];
        }
        std::memcpy(vol->bbox, bb, sizeof(float) * 6);
        vol->components = (uint64_t) job.components;
        vol->min_value = hs.out_min;
        vol->max_value = hs.out_max;
        vol->data_hash = ++datahash;
    }
    if (hs.error & ERR_LOOKBACK_TIMEOUT)
        return fail(P2V_ETIMEOUT, "radix sort look-back wait gave up (device error 0x%x)", hs.error);
    if (hs.error & ERR_MMA_TIMEOUT)
        return fail(P2V_ETIMEOUT, "tensor-core MMA wait gave up (device error 0x%x)", hs.error);
    if (hs.error)
        return fail(P2V_EDOMAIN, "input outside the supported domain (device error 0x%x)", hs.error);
    err.clear();
    return P2V_OK;
}

// MDAO volume size for a clip box (SphereRenderer.cpp:2463-2476): the longest edge gets vol_size voxels,
// x is rounded up to a multiple of 4; Cuboid edges are absolute and Dimension::Scale multiplies in double.
void mdao_dims(const float clip[6], int vol_size, int dims[3], float& shortest, float& max_lod) {
    float size[3];
    for (int a = 0; a < 3; ++a)
        size[a] = std::fabs(clip[a + 3] - clip[a]);
    const float w = size[0], h = size[1], d = size[2];
    const float longest = ((w > h) && (w > d)) ? w : ((h > d) ? h : d);
    const double f = static_cast<double>(static_cast<float>(vol_size) / longest);
    float dm[3];
    for (int a = 0; a < 3; ++a)
        dm[a] = static_cast<float>(f * static_cast<double>(size[a]));
    dm[0] = std::ceil(dm[0] / 4.0f) * 4.0f;
    dm[1] = std::ceil(dm[1]);
    dm[2] = std::ceil(dm[2]);
    for (int a = 0; a < 3; ++a)
        dims[a] = static_cast<int>(dm[a]);
    shortest = std::min(dm[0], std::min(dm[1], dm[2]));
    max_lod = std::ceil(std::log2(static_cast<float>(vol_size))) - 1.0f;
}

p2v_status p2v_ctx::build_cone(Pipe& pp, const p2v_frame* fr, const GridGeo& g, const float* dgrid,
                               const float bb[6], uint32_t n, const uint32_t* order, ConeParams& cp, cudaStream_t st,
                               BatchSlot* slot) {
    DevBuf &xyzr = pp.xyzr, &mips = slot ? slot->mips : pp.mips, &mdao_acc = pp.mdao_acc, &mdao_vol = pp.mdao_vol;
    const p2v_params& P = prm;
    if (P.ao_volume != P2V_AOVOL_DENSITY && P.ao_volume != P2V_AOVOL_MDAO)
        return fail(P2V_EINVAL, "ao_volume %d is not a p2v_ao_volume", P.ao_volume);
    if (P.ao_cones < 1 || P.ao_cones > MAX_CONES)
        return fail(P2V_EINVAL, "ao_cones must lie in [1, %d]", MAX_CONES);
    cp = ConeParams{};
    const bool mdao = P.ao_volume == P2V_AOVOL_MDAO;
    if (mdao && slot)
        return fail(P2V_EUNSUPPORTED, "the batch AO launch marches the density, not the MDAO volume");
    int d0[3];
    float shortest = 0.0f, max_lod = 0.0f;
    int L = 0;
    const float* level0 = dgrid;
    if (mdao) {
        // the occupancy voxelisation of the clip box (MDAOVolumeGenerator); its texture spans the clip box
        if (P.mdao_volume_size < 1 || P.mdao_volume_size > 4096)
            return fail(P2V_EINVAL, "mdao_volume_size must lie in [1, 4096]");
        for (int a = 0; a < 3; ++a)
            if (!(std::fabs(fr->clipbox[a + 3] - fr->clipbox[a]) > 0.0f) ||
                !std::isfinite(fr->clipbox[a]) || !std::isfinite(fr->clipbox[a + 3]))
                return fail(P2V_EINVAL, "clip box must have a finite, non-zero extent along %c (MDAO volume)",
                            "xyz"[a]);
        mdao_dims(fr->clipbox, P.mdao_volume_size, d0, shortest, max_lod);
        const uint64_t nv = (uint64_t) d0[0] * d0[1] * d0[2];
        if (nv > (1ull << 31))
            return fail(P2V_EINVAL, "MDAO volume %dx%dx%d is too large", d0[0], d0[1], d0[2]);
        MdaoParams mp{};
        for (int a = 0; a < 3; ++a) {
            const float size = std::fabs(fr->clipbox[a + 3] - fr->clipbox[a]);
            mp.bmin[a] = fr->clipbox[a];
            mp.inv[a] = 1.0f / size;
            mp.fd[a] = static_cast<float>(d0[a]);
            mp.d[a] = d0[a];
            mp.cell[a] = 1.0f / (mp.fd[a] * mp.inv[a]);
            cp.bmin[a] = mp.bmin[a];
            cp.ibsize[a] = mp.inv[a];
        }
        mp.cell_vol = (mp.cell[0] * mp.cell[1]) * mp.cell[2];
        mp.ps_scale = std::max(mp.inv[0] * mp.fd[0], mp.inv[1] * mp.fd[1]);
        mp.sphere_k = 4.0f / 3.0f * 3.14152f;
        mp.half_vp[0] = 0.5f * mp.fd[0];
        mp.half_vp[1] = 0.5f * mp.fd[1];
        mp.unorm8 = P.mdao_unorm8 ? 1 : 0;
        P2V_CUDA_TRY(mdao_acc.ensure((mp.unorm8 ? 4 : 8) * nv));
        P2V_CUDA_TRY(mdao_vol.ensure(sizeof(float) * nv));
        P2V_CUDA_TRY(launch_mdao_volume(mp, order, xyzr.as<float4>(), n, mdao_acc.ptr, mdao_vol.as<float>(), sms, st));
        level0 = mdao_vol.as<float>();
        // the reference's texture holds every level down to 1x1x1; the lod clamp is maxLod
        const int smax = std::max(d0[0], std::max(d0[1], d0[2]));
        const int full = (int) std::floor(std::log2((double) smax)) + 1;
        L = P.ao_levels > 0 ? P.ao_levels : std::min(full, (int) max_lod + 1);
        L = std::max(1, std::min(L, MAX_LEVELS));
        max_lod = std::min(max_lod, (float) (L - 1));
        cp.sat = 0.0f;
    } else {
        for (int a = 0; a < 3; ++a)
            d0[a] = g.s[a];
        const int smax = std::max(g.s[0], std::max(g.s[1], g.s[2]));
        shortest = (float) std::min(g.s[0], std::min(g.s[1], g.s[2]));
        L = P.ao_levels > 0 ? P.ao_levels : (int) std::ceil(std::log2((double) smax));
        L = std::max(1, std::min(L, MAX_LEVELS));
        max_lod = (float) (L - 1);
        // the density grid is node-centred: as a texture it spans [min - h/2, max + h/2]
        for (int a = 0; a < 3; ++a) {
            const double hd = std::fabs((double) bb[a + 3] - (double) bb[a]) / (double) (g.s[a] - 1);
            cp.bmin[a] = (float) ((double) bb[a] - 0.5 * hd);
            cp.ibsize[a] = (float) (1.0 / (g.s[a] * hd));
        }
        cp.sat = P.ao_volume_scale;
    }
    cp.strength = P.ao_strength;
    cp.border = 0;  // CLAMP_TO_BORDER (MDAOVolumeGenerator.cpp:58-60)
    cp.early_exit = P.ao_early_exit ? 1 : 0;
    cp.ncones = P.ao_cones;
    cone_directions(P.ao_cones, P.ao_apex_deg * 3.14159265358979f / 180.0f, cp.dirs);
    cp.nsteps = cone_steps(P.ao_offset, P.ao_cone_length, P.ao_steps, cp.dirs[0].w, shortest, max_lod, cp.t, cp.lod,
                           MAX_STEPS);
    if (P.ao_steps > MAX_STEPS || (P.ao_steps <= 0 && cp.nsteps >= MAX_STEPS))
        return fail(P2V_EUNSUPPORTED, "more than %d samples per cone", MAX_STEPS);
    cp.nlevels = L;
    // the samplers address texels with 32-bit offsets
    if ((uint64_t) d0[0] * d0[1] * d0[2] >= (1ull << 31))
        return fail(P2V_EUNSUPPORTED, "AO volume %dx%dx%d exceeds 2^31 texels", d0[0], d0[1], d0[2]);
    // level 0 is the density grid (saturated on the fly) or the MDAO volume; levels 1.. are built here
    // each level starts on a 128-byte boundary
    size_t need = 0;
    int d[MAX_LEVELS][3];
    for (int a = 0; a < 3; ++a)
        d[0][a] = d0[a];
    for (int l = 1; l < L; ++l) {
        for (int a = 0; a < 3; ++a)
            d[l][a] = std::max(1, d[l - 1][a] / 2);
        need += ((size_t) d[l][0] * d[l][1] * d[l][2] + 31) & ~size_t(31);
    }
    P2V_CUDA_TRY(mips.ensure(sizeof(float) * (need + 1)));
    float* lvp[MAX_LEVELS];
    lvp[0] = const_cast<float*>(level0);
    size_t off = 0;
    for (int l = 1; l < L; ++l) {
        lvp[l] = mips.as<float>() + off;
        off += ((size_t) d[l][0] * d[l][1] * d[l][2] + 31) & ~size_t(31);
    }
    int dims[MAX_LEVELS][3];
    if (!slot)  // a batch frame's levels are built by the batch AO launch
        P2V_CUDA_TRY(launch_mip_levels(level0, d0, cp.sat, mdao && P.mdao_unorm8 ? 1 : 0, L, lvp, dims, sms, st));
    for (int l = 0; l < L; ++l) {
        cp.lv[l].v = lvp[l];
        for (int a = 0; a < 3; ++a) {
            cp.lv[l].d[a] = d[l][a];
            cp.lv[l].fd[a] = (float) d[l][a];
        }
    }
    pp.last_cp = cp;
    return P2V_OK;
}

// The learned AO's feature samples: MLP_FSTEPS steps spread evenly over the cone's step table (step
// round(j (nsteps - 1) / (MLP_FSTEPS - 1)) for feature j), each at its own lod. Copy every mip level those
// samples read (level 0 of a density volume saturated as the cone march sees it) into its paired-slice
// texture and hand the texture objects to the kernels.
p2v_status p2v_ctx::prepare_features(Pipe& pp, ConeParams& cp, cudaStream_t st) {
    if (cp.ncones != MLP_CONES)
        return fail(P2V_EINVAL, "learned AO: its features read %d cones (ao_cones is %d)", MLP_CONES, cp.ncones);
    if (cp.nsteps < 1)
        return fail(P2V_EINVAL, "learned AO: empty cone step table");
    cp.nfsteps = MLP_FSTEPS;
    bool need[MAX_LEVELS] = {};
    for (int j = 0; j < MLP_FSTEPS; ++j) {
        const int k = (int) std::lround((double) j * (cp.nsteps - 1) / (double) (MLP_FSTEPS - 1));
        cp.fstep[j] = k;
        const int l0 = std::min((int) cp.lod[k], cp.nlevels - 1);
        need[l0] = true;
        if (cp.lod[k] - (float) l0 > 0.0f && l0 + 1 < cp.nlevels)
            need[l0 + 1] = true;
    }
    for (int l = 0; l < MAX_LEVELS; ++l) {
        cp.ftex[l] = 0;
        if (l >= cp.nlevels || !need[l])
            continue;
        const ConeLevel& L = cp.lv[l];
        // the feature textures are layered (one layer per z slice): the device's layer limit bounds sizez
        int max_layers = 0, max_w = 0;
        P2V_CUDA_TRY(cudaDeviceGetAttribute(&max_layers, cudaDevAttrMaxTexture2DLayeredLayers, device));
        P2V_CUDA_TRY(cudaDeviceGetAttribute(&max_w, cudaDevAttrMaxTexture2DLayeredWidth, device));
        if (L.d[2] > max_layers || L.d[0] > max_w || L.d[1] > max_w)
            return fail(P2V_EUNSUPPORTED, "learned AO: mip level %d is %dx%dx%d; its feature texture allows at most %d "
                        "slices of %d x %d texels", l, L.d[0], L.d[1], L.d[2], max_layers, max_w, max_w);
        P2V_CUDA_TRY(pp.ftex[l].ensure(L.d));
        P2V_CUDA_TRY(launch_fill_feature_tex(L, l == 0 ? cp.sat : 0.0f, pp.ftex[l], st));
        cp.ftex[l] = pp.ftex[l].tex;
    }
    return P2V_OK;
}

p2v_status p2v_ctx::run_ao(Pipe& pp, const p2v_frame* fr, const GridGeo& g, const float* dgrid, const float bb[6],
                           uint32_t n, const uint32_t* order, cudaStream_t st, BatchSlot* slot) {
    DevBuf &xyzr = pp.xyzr, &nrm = pp.nrm, &ao = pp.ao, &scal = pp.scal, &fb_list = pp.fb_list,
           &aos_acc = pp.aos_acc, &aos_tex = pp.aos_tex;
    const p2v_params& P = prm;
    // the cone-march stages run on sorted copies of the positions and normals (coalesced whatever the input
    // order) and scatter the AO back to input order at the end
    // (the binning's last pass wrote the sorted positions when it knew the frame would march cones); gradient
    // normals are computed in sorted order from the sorted positions
    auto to_sorted = [&]() -> cudaError_t {
        cudaError_t e = pp.xyzr_s.ensure(sizeof(float4) * ((size_t) n + 1));
        if (e == cudaSuccess)
            e = pp.nrm_s.ensure(sizeof(float4) * ((size_t) n + 1));
        if (e != cudaSuccess)
            return e;
        if (P.ao_normals == P2V_NORMALS_GRADIENT) {
            if (!pp.xyzr_sorted)
                e = launch_sort_particles(order, n, xyzr.as<float4>(), nrm.as<float4>(), pp.xyzr_s.as<float4>(),
                                          pp.nrm_s.as<float4>(), sms, st);
            if (e == cudaSuccess)
                e = launch_gradient_normals(g, dgrid, pp.xyzr_s.as<float4>(), n, pp.nrm_s.as<float4>(), st);
            return e;
        }
        return launch_sort_particles(order, n, pp.xyzr_sorted ? nullptr : xyzr.as<float4>(), nrm.as<float4>(),
                                     pp.xyzr_s.as<float4>(), pp.nrm_s.as<float4>(), sms, st);
    };
    // the cone-march stages can take the sorted particles in brick-major order (bricks of 16 x 4 x 4 cells):
    // neighbouring threads then sample neighbouring texels along all three axes. ao_brick_order -1: for the
    // plain march only (faster on uniform frames; the learned AO's texture fetches gained nothing)
    const float4* axyzr = nullptr;
    const float4* anrm = nullptr;
    const uint32_t* aorder = order;
    auto ao_inputs = [&]() -> cudaError_t {
        axyzr = pp.xyzr_s.as<float4>();
        anrm = pp.nrm_s.as<float4>();
        aorder = order;
        const bool bricks = P.ao_brick_order > 0 || (P.ao_brick_order < 0 && P.ao_mode == P2V_AO_CONE);
        if (!bricks || n == 0)
            return cudaSuccess;
        const BrickPlan bp = brick_plan(g);
        if (bp.nseg >= (1ull << 32))
            return cudaErrorInvalidValue;
        cudaError_t e = pp.bk0.ensure(sizeof(uint32_t) * (bp.nseg + 1));
        if (e == cudaSuccess)
            e = pp.bk1.ensure(sizeof(uint32_t) * (bp.ntiles + 1));
        if (e == cudaSuccess)
            e = pp.ord_b.ensure(sizeof(uint32_t) * ((size_t) n + 1));
        if (e == cudaSuccess)
            e = pp.xyzr_b.ensure(sizeof(float4) * ((size_t) n + 1));
        if (e == cudaSuccess)
            e = pp.nrm_b.ensure(sizeof(float4) * ((size_t) n + 1));
        if (e == cudaSuccess)
            e = launch_brick_order(bp, g, pp.cstart.as<uint32_t>(), reinterpret_cast<const int4*>(pp.rec_a.as<float4>() + 1),
                                   n, pp.bk0.as<uint32_t>(), pp.bk1.as<uint32_t>(), pp.xyzr_s.as<float4>(),
                                   pp.nrm_s.as<float4>(), order, pp.xyzr_b.as<float4>(), pp.nrm_b.as<float4>(),
                                   pp.ord_b.as<uint32_t>(), sms, st);
        axyzr = pp.xyzr_b.as<float4>();
        anrm = pp.nrm_b.as<float4>();
        aorder = pp.ord_b.as<uint32_t>();
        return e;
    };
    if (P.ao_mode == P2V_AO_CONE) {
        ConeParams cp{};
        const p2v_status bs = build_cone(pp, fr, g, dgrid, bb, n, order, cp, st, slot);
        if (bs != P2V_OK)
            return bs;
        if (slot) {
            // the batch AO launch builds the levels and marches the cones (gradient normals computed there)
            const bool list = P.ao_normals == P2V_NORMALS_LIST;
            if (list && n > 0) {
                P2V_CUDA_TRY(slot->nrm_s.ensure(sizeof(float4) * ((size_t) n + 1)));
                P2V_CUDA_TRY(launch_sort_particles(order, n, nullptr, nrm.as<float4>(), nullptr,
                                                   slot->nrm_s.as<float4>(), sms, st));
            }
            P2V_CUDA_TRY(slot->ao.ensure(sizeof(float) * ((size_t) n + 1)));
            BatchAoFrame& d = *slot->desc;
            d = BatchAoFrame{};
            d.cp = cp;
            d.g = g;
            d.grid = dgrid;
            d.xyzr = slot->xyzr_s.as<float4>();
            d.nrm = list ? slot->nrm_s.as<float4>() : nullptr;
            d.order = slot->order.as<uint32_t>();
            d.ao = slot->ao.as<float>();
            d.n = n;
            if (P.ao_brick_order != 0 && n > 0) {  // the march in brick order (the same bits)
                const BrickPlan bp = brick_plan(g);
                P2V_CUDA_TRY(pp.bk0.ensure(sizeof(uint32_t) * (bp.nseg + 1)));
                P2V_CUDA_TRY(pp.bk1.ensure(sizeof(uint32_t) * (bp.ntiles + 1)));
                P2V_CUDA_TRY(slot->xyzr_b.ensure(sizeof(float4) * ((size_t) n + 1)));
                P2V_CUDA_TRY(slot->ord_b.ensure(sizeof(uint32_t) * ((size_t) n + 1)));
                if (list)
                    P2V_CUDA_TRY(slot->nrm_b.ensure(sizeof(float4) * ((size_t) n + 1)));
                P2V_CUDA_TRY(launch_brick_order(bp, g, pp.cstart.as<uint32_t>(),
                                                reinterpret_cast<const int4*>(pp.rec_a.as<float4>() + 1), n,
                                                pp.bk0.as<uint32_t>(), pp.bk1.as<uint32_t>(), slot->xyzr_s.as<float4>(),
                                                d.nrm, slot->order.as<uint32_t>(), slot->xyzr_b.as<float4>(),
                                                list ? slot->nrm_b.as<float4>() : nullptr, slot->ord_b.as<uint32_t>(),
                                                sms, st));
                d.xyzr = slot->xyzr_b.as<float4>();
                d.nrm = list ? slot->nrm_b.as<float4>() : nullptr;
                d.order = slot->ord_b.as<uint32_t>();
            }
            slot->deferred = true;
            return P2V_OK;
        }
        P2V_CUDA_TRY(to_sorted());
        P2V_CUDA_TRY(ao_inputs());
        if (pp.timing)
            P2V_CUDA_TRY(cudaEventRecord(pp.ev[EV_AOK0], st));
        if (P.ao_march == P2V_AO_MARCH_WARP)
            P2V_CUDA_TRY(launch_cone_ao_warp(cp, axyzr, anrm, n, aorder, ao.as<float>(), sms, st));
        else
            P2V_CUDA_TRY(launch_cone_ao(cp, nullptr, axyzr, anrm, n, nullptr, aorder, ao.as<float>(), st));
        if (pp.timing) {
            P2V_CUDA_TRY(cudaEventRecord(pp.ev[EV_AOK1], st));
            pp.aok = true;
        }
        return P2V_OK;
    }
    if (P.ao_mode == P2V_AO_LEARNED) {
        if (!mlp_ready)
            return fail(P2V_EINVAL, "learned AO: no trained network (p2v_mlp_train or p2v_mlp_load first)");
        ConeParams cp{};
        const p2v_status bs = build_cone(pp, fr, g, dgrid, bb, n, order, cp, st, nullptr);
        if (bs != P2V_OK)
            return bs;
        const p2v_status ps = prepare_features(pp, cp, st);
        if (ps != P2V_OK)
            return ps;
        P2V_CUDA_TRY(fb_list.ensure(sizeof(uint32_t) * ((size_t) n + 1)));
        FrameScalars* fs = scal.as<FrameScalars>();
        MlpInferArgs a{};
        a.P = mlp_P.as<float>();
        a.w1h = mlp_w1h.as<__nv_bfloat16>();
        a.w2h = mlp_w2h.as<__nv_bfloat16>();
        a.lo = mlp_has_range ? mlp_lo.as<float>() : nullptr;
        a.hi = mlp_has_range ? mlp_hi.as<float>() : nullptr;
        P2V_CUDA_TRY(to_sorted());
        P2V_CUDA_TRY(ao_inputs());
        a.n = n;
        a.order = nullptr;  // sorted copies: position j is sorted position j
        a.xyzr = axyzr;
        a.nrm = anrm;
        a.y = ao.as<float>();
        a.out_order = aorder;
        a.fallback = fb_list.as<uint32_t>();
        a.nfallback = &fs->ao_fallback;
        a.err = &fs->error;
        if (P.mma_wait_polls < 0)
            return fail(P2V_EINVAL, "mma_wait_polls must be >= 0");
        a.wait_polls = (uint32_t) P.mma_wait_polls;
        a.hold_mma = P.test_hold_mma ? 1 : 0;
        // texture fetches per particle: one per feature sample, two where the sample's lod lies between levels
        pp.ao_fetches = 0;
        for (int j = 0; j < MLP_FSTEPS; ++j) {
            const float lod = cp.lod[cp.fstep[j]];
            const int l0 = std::min((int) lod, cp.nlevels - 1);
            pp.ao_fetches += (uint32_t) MLP_CONES * ((lod - (float) l0 > 0.0f && l0 + 1 < cp.nlevels) ? 2u : 1u);
        }
        if (pp.timing)
            P2V_CUDA_TRY(cudaEventRecord(pp.ev[EV_AOK0], st));
        P2V_CUDA_TRY(launch_mlp_infer(a, cp, false, sms, st));
        if (pp.timing) {
            P2V_CUDA_TRY(cudaEventRecord(pp.ev[EV_AOK1], st));
            pp.aok = true;
        }
        // the plain cone march for every particle whose features left the training range
        P2V_CUDA_TRY(launch_cone_ao(cp, fb_list.as<uint32_t>(), axyzr, anrm, n, &fs->ao_fallback, aorder,
                                    ao.as<float>(), st));
        return P2V_OK;
    }
    if (P.ao_mode == P2V_AO_AOSPHERE_AXES || P.ao_mode == P2V_AO_AOSPHERE_NORMAL) {
        AOSphereParams ap{};
        const int sz3[3] = {P.aos_sizex, P.aos_sizey, P.aos_sizez};
        for (int a = 0; a < 3; ++a) {
            if (sz3[a] < 3 || sz3[a] > 2048)
                return fail(P2V_EINVAL, "aos_size%c must lie in [3, 2048]", "xyz"[a]);
            ap.s[a] = sz3[a];
            ap.si[a] = sz3[a] - 2;
            ap.minOS[a] = fr->clipbox[a];
            ap.rangeOS[a] = std::fabs(fr->clipbox[a + 3] - fr->clipbox[a]);
            if (!(ap.rangeOS[a] > 0.0f))
                return fail(P2V_EINVAL, "clip box has zero extent along %c", "xyz"[a]);
            // AOSphereRenderer.cpp:496-513
            const float ext = ap.rangeOS[a] / (1.0f - 2.0f / static_cast<float>(sz3[a]));
            ap.ext[a] = ext;
            ap.origin[a] = ap.minOS[a] - ext / static_cast<float>(sz3[a]);
            ap.sampd[a] = P.aos_step_len * (ap.rangeOS[a] / static_cast<float>(sz3[a]));
        }
        ap.voxel_vol = (ap.rangeOS[0] / static_cast<float>(ap.si[0])) * (ap.rangeOS[1] / static_cast<float>(ap.si[1])) *
                       (ap.rangeOS[2] / static_cast<float>(ap.si[2]));
        ap.gen_fac = P.aos_gen_fac;
        ap.eval_fac = P.aos_eval_fac;
        if (P.aos_deposit != P2V_AOS_DEPOSIT_CPU && P.aos_deposit != P2V_AOS_DEPOSIT_GLSL)
            return fail(P2V_EINVAL, "aos_deposit %d is not a p2v_aos_deposit", P.aos_deposit);
        ap.glsl_rule = P.aos_deposit == P2V_AOS_DEPOSIT_GLSL ? 1 : 0;
        ap.clip = P.aos_clip && !ap.glsl_rule ? 1 : 0;  // createVolumeGLSL has no clip discard
        for (int k = 0; k < 4; ++k)
            ap.clip_plane[k] = P.aos_clip_plane[k];
        const size_t nv = (size_t) ap.s[0] * ap.s[1] * ap.s[2];
        if (P.ao_normals == P2V_NORMALS_GRADIENT)  // the taps read the normals in input order
            P2V_CUDA_TRY(launch_gradient_normals(g, dgrid, xyzr.as<float4>(), n, nrm.as<float4>(), st));
        P2V_CUDA_TRY(aos_acc.ensure(sizeof(unsigned long long) * nv));
        P2V_CUDA_TRY(aos_tex.ensure(sizeof(float) * nv));
        P2V_CUDA_TRY(launch_aosphere(ap, xyzr.as<float4>(), n, aos_acc.as<unsigned long long>(), aos_tex.as<float>(),
                                     order, nrm.as<float4>(), P.ao_mode == P2V_AO_AOSPHERE_AXES ? 0 : 1,
                                     ao.as<float>(), sms, st));
        return P2V_OK;
    }
    return fail(P2V_EUNSUPPORTED, "ao_mode %d is not implemented", P.ao_mode);
}

namespace {

void sig_put(std::vector<uint8_t>& v, const void* p, size_t n) {
    const uint8_t* b = static_cast<const uint8_t*>(p);
    v.insert(v.end(), b, b + n);
}

// true when host memory p can take part in a captured graph's copies (pinned, or device / managed)
bool graph_safe_host(const void* p) {
    if (!p)
        return true;
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type != cudaMemoryTypeUnregistered;
}

}  // namespace

// The persistent batch AO (after every lane has finished its frames): the work queue of every deferred
// frame, mip levels first (level 1 of every frame, then level 2, ...; a level's segment depends on the level
// below it), then each frame's cone march (depending on its last level), largest frames first; the tables
// are uploaded from pinned memory, the queue runs in one launch, and the frames' AO is copied to the lists'
// outputs.
p2v_status p2v_ctx::enqueue_batch_ao(const p2v_batch_item* items, uint32_t count, const std::vector<uint32_t>& byw,
                                     cudaStream_t st) {
    if (prm.queue_wait_polls < 0)
        return fail(P2V_EINVAL, "queue_wait_polls must be >= 0");
    std::vector<BatchSeg> segs;
    std::vector<std::array<int, MAX_LEVELS>> seg_of(count);
    int maxL = 0;
    for (uint32_t f = 0; f < count; ++f) {
        seg_of[f].fill(-1);
        const BatchSlot& sl = *b_slots[f];
        if (sl.deferred && sl.desc->n > 0)
            maxL = std::max(maxL, sl.desc->cp.nlevels);
    }
    uint32_t tick = 0;
    for (int l = 1; l < maxL; ++l)
        for (uint32_t f : byw) {
            const BatchSlot& sl = *b_slots[f];
            if (!sl.deferred || sl.desc->n == 0 || l >= sl.desc->cp.nlevels)
                continue;
            const ConeLevel& lv = sl.desc->cp.lv[l];
            const uint64_t nv = (uint64_t) lv.d[0] * lv.d[1] * lv.d[2];
            const uint32_t cnt = (uint32_t) ((nv + BATCH_MIP_ITEM - 1) / BATCH_MIP_ITEM);
            seg_of[f][l] = (int) segs.size();
            segs.push_back(BatchSeg{tick, cnt, f, BSEG_MIP, l, l >= 2 ? seg_of[f][l - 1] : -1});
            tick += cnt;
        }
    const int hold = prm.test_hold_queue && !segs.empty() ? 0 : -1;
    for (uint32_t f : byw) {
        const BatchSlot& sl = *b_slots[f];
        if (!sl.deferred || sl.desc->n == 0)
            continue;
        const uint32_t cnt = (sl.desc->n + BATCH_AO_ITEM - 1) / BATCH_AO_ITEM;
        const int L = sl.desc->cp.nlevels;
        segs.push_back(BatchSeg{tick, cnt, f, BSEG_AO, 0, L >= 2 ? seg_of[f][L - 1] : -1});
        tick += cnt;
    }
    if (b_segs_cap < segs.size()) {
        P2V_CUDA_TRY(cudaStreamSynchronize(st));
        if (b_segs_h)
            cudaFreeHost(b_segs_h);
        b_segs_h = nullptr;
        b_segs_cap = 0;
        P2V_CUDA_TRY(cudaMallocHost(&b_segs_h, sizeof(BatchSeg) * segs.size()));
        b_segs_cap = segs.size();
    }
    if (!segs.empty())
        std::memcpy(b_segs_h, segs.data(), sizeof(BatchSeg) * segs.size());
    P2V_CUDA_TRY(b_frames_d.ensure(sizeof(BatchAoFrame) * count));
    P2V_CUDA_TRY(b_segs_d.ensure(sizeof(BatchSeg) * (segs.size() + 1)));
    P2V_CUDA_TRY(b_words.ensure(sizeof(uint32_t) * batch_queue_words((uint32_t) segs.size())));
    P2V_CUDA_TRY(cudaMemcpyAsync(b_frames_d.ptr, b_frames_h, sizeof(BatchAoFrame) * count, cudaMemcpyHostToDevice, st));
    if (!segs.empty())
        P2V_CUDA_TRY(cudaMemcpyAsync(b_segs_d.ptr, b_segs_h, sizeof(BatchSeg) * segs.size(), cudaMemcpyHostToDevice,
                                     st));
    BatchQueueArgs q{};
    q.frames = b_frames_d.as<BatchAoFrame>();
    q.segs = b_segs_d.as<BatchSeg>();
    q.nseg = (uint32_t) segs.size();
    q.total = tick;
    q.words = b_words.as<uint32_t>();
    q.wait_polls = prm.queue_wait_polls > 0 ? (uint32_t) prm.queue_wait_polls : (1u << 22);
    q.hold_seg = hold;
    P2V_CUDA_TRY(launch_batch_ao(q, sms, st));
    P2V_CUDA_TRY(cudaMemcpyAsync(b_err_h, b_words.as<uint32_t>() + 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    for (uint32_t f = 0; f < count; ++f) {
        const BatchSlot& sl = *b_slots[f];
        if (!sl.deferred)
            continue;
        const p2v_frame* fr = items[f].frame;
        uint64_t aoff = 0;
        for (uint32_t l = 0; l < fr->list_count; ++l) {
            const p2v_particle_list& Lst = fr->lists[l];
            if (Lst.vertex_type == P2V_VERTDATA_NONE)
                continue;
            if (Lst.ao_out && Lst.count > 0)
                P2V_CUDA_TRY(cudaMemcpyAsync(Lst.ao_out, sl.ao.as<float>() + aoff, sizeof(float) * Lst.count,
                                             Lst.mem == P2V_MEM_DEVICE ? cudaMemcpyDeviceToDevice
                                                                       : cudaMemcpyDeviceToHost,
                                             st));
            aoff += Lst.count;
        }
    }
    return P2V_OK;
}

// A batch: frames sorted by work (particles plus a share of the grid) and dealt, largest first, to the
// least-loaded of L lanes; every lane queues its frames on its own stream, forked from and joined back into
// `st`. When the batch's shape (every pointer, count, size and parameter) equals that of the previous eager
// run, the queueing is captured as a CUDA graph (all buffers already have their sizes, so nothing is
// allocated during capture) and later calls with the same shape replay it with a single launch.
p2v_status p2v_ctx::run_batch(const p2v_batch_item* items, uint32_t count, p2v_stats* out, cudaStream_t st,
                              bool allow_graph, float* ms_out) {
    P2V_CUDA_TRY(cudaSetDevice(device));
    if (count == 0)
        return P2V_OK;
    if (!items)
        return fail(P2V_EINVAL, "no batch items");
    int L = prm.batch_lanes > 0 ? prm.batch_lanes : (tuned_lanes > 0 ? tuned_lanes : 4);
    L = std::max(1, std::min(L, 16));
    L = (int) std::min<uint32_t>((uint32_t) L, count);
    while ((int) lanes.size() < L) {
        auto pp = std::make_unique<Pipe>();
        if (pp->init(true) != cudaSuccess) {
            pp->release();
            return fail(P2V_ECUDA, "batch lane creation failed");
        }
        lanes.push_back(std::move(pp));
    }
    while ((int) b_events.size() < L + 1) {
        cudaEvent_t e;
        P2V_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        b_events.push_back(e);
    }
    if (!b_t0) {
        P2V_CUDA_TRY(cudaEventCreate(&b_t0));
        P2V_CUDA_TRY(cudaEventCreate(&b_t1));
    }
    if (b_scal_cap < count) {
        if (b_scal) {
            P2V_CUDA_TRY(cudaStreamSynchronize(st));
            cudaFreeHost(b_scal);
            b_scal = nullptr;
        }
        P2V_CUDA_TRY(cudaMallocHost(&b_scal, sizeof(FrameScalars) * count));
        b_scal_cap = count;
        drop_graph();  // the graph copies into the old slots
    }
    // ---- schedule ----
    std::vector<uint32_t> byw(count);
    std::vector<double> work(count);
    bool pinned = true;
    for (uint32_t f = 0; f < count; ++f) {
        const p2v_batch_item& it = items[f];
        if (!it.frame)
            return fail(P2V_EINVAL, "batch item %u has no frame", f);
        uint64_t n = 0;
        for (uint32_t l = 0; l < it.frame->list_count; ++l) {
            const p2v_particle_list& Lst = it.frame->lists[l];
            n += Lst.count;
            if (Lst.mem != P2V_MEM_DEVICE)
                pinned = pinned && graph_safe_host(Lst.vertex_data) && graph_safe_host(Lst.normals) &&
                         graph_safe_host(Lst.ao_out);
        }
        const int32_t sz[3] = {it.size[0] > 0 ? it.size[0] : prm.sizex, it.size[1] > 0 ? it.size[1] : prm.sizey,
                               it.size[2] > 0 ? it.size[2] : prm.sizez};
        work[f] = (double) n + 0.25 * (double) sz[0] * sz[1] * sz[2];
        if (it.volume && it.volume->data && it.volume->mem != P2V_MEM_DEVICE)
            pinned = pinned && graph_safe_host(it.volume->data);
        byw[f] = f;
    }
    std::stable_sort(byw.begin(), byw.end(), [&](uint32_t a, uint32_t b) { return work[a] > work[b]; });
    std::vector<int> lane_of(count);
    std::vector<double> load(L, 0.0);
    for (uint32_t k = 0; k < count; ++k) {
        const int l = (int) (std::min_element(load.begin(), load.end()) - load.begin());
        lane_of[byw[k]] = l;
        load[l] += work[byw[k]];
    }
    // ---- shape signature ----
    std::vector<uint8_t> sig;
    sig_put(sig, &prm, sizeof(prm));
    sig_put(sig, tuned_tile, sizeof(tuned_tile));
    sig_put(sig, &L, sizeof(L));
    sig_put(sig, &st, sizeof(st));
    for (uint32_t f = 0; f < count; ++f) {
        const p2v_batch_item& it = items[f];
        sig_put(sig, it.size, sizeof(it.size));
        sig_put(sig, it.frame->bbox, sizeof(it.frame->bbox));
        sig_put(sig, it.frame->clipbox, sizeof(it.frame->clipbox));
        sig_put(sig, &it.frame->list_count, sizeof(it.frame->list_count));
        for (uint32_t l = 0; l < it.frame->list_count; ++l)
            sig_put(sig, &it.frame->lists[l], sizeof(p2v_particle_list));
        const p2v_volume* v = it.volume;
        const void* vd = v ? v->data : nullptr;
        const int32_t vm = v ? v->mem : -1;
        const uint64_t vc = v ? v->capacity : 0;
        sig_put(sig, &vd, sizeof(vd));
        sig_put(sig, &vm, sizeof(vm));
        sig_put(sig, &vc, sizeof(vc));
    }
    const bool use_graph = allow_graph && prm.batch_graph != 0 && pinned;
    const bool replay = use_graph && b_exec && sig == b_graph_sig;
    const bool pers = batch_persistent_applies();
    if (pers && !replay) {
        // per-frame buffers and the pinned descriptor table (sized before any capture begins)
        while (b_slots.size() < count)
            b_slots.push_back(std::make_unique<BatchSlot>());
        if (b_frames_cap < count) {
            P2V_CUDA_TRY(cudaStreamSynchronize(st));
            if (b_frames_h)
                cudaFreeHost(b_frames_h);
            b_frames_h = nullptr;
            b_frames_cap = 0;
            P2V_CUDA_TRY(cudaMallocHost(&b_frames_h, sizeof(BatchAoFrame) * count));
            b_frames_cap = count;
        }
        if (!b_err_h)
            P2V_CUDA_TRY(cudaMallocHost(&b_err_h, sizeof(uint32_t)));
        for (uint32_t f = 0; f < count; ++f) {
            b_slots[f]->desc = b_frames_h + f;
            b_slots[f]->deferred = false;
        }
    }
    P2V_CUDA_TRY(cudaEventRecord(b_t0, st));
    if (replay) {
        P2V_CUDA_TRY(cudaGraphLaunch(b_exec, st));
    } else {
        // an eager run may grow (reallocate) buffers a captured graph points to: a graph is replayed only
        // while no other batch ran since its capture
        drop_graph();
        const bool capture = use_graph && sig == b_eager_sig;
        if (capture)
            P2V_CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        b_jobs.assign(count, FrameJob{});
        p2v_status es = P2V_OK;
        cudaError_t ce = cudaEventRecord(b_events[L], st);
        for (int l = 0; l < L && ce == cudaSuccess; ++l)
            ce = cudaStreamWaitEvent(lanes[l]->stream, b_events[L], 0);
        const p2v_params saved = prm;
        for (uint32_t k = 0; k < count && ce == cudaSuccess && es == P2V_OK; ++k) {
            const uint32_t f = byw[k];
            const p2v_batch_item& it = items[f];
            if (it.size[0] > 0)
                prm.sizex = it.size[0];
            if (it.size[1] > 0)
                prm.sizey = it.size[1];
            if (it.size[2] > 0)
                prm.sizez = it.size[2];
            Pipe& pp = *lanes[lane_of[f]];
            es = enqueue_frame(pp, it.frame, it.volume, pp.stream, b_scal + f, false, b_jobs[f],
                               pers ? b_slots[f].get() : nullptr);
            prm = saved;
        }
        for (int l = 0; l < L && ce == cudaSuccess; ++l) {
            ce = cudaEventRecord(b_events[l], lanes[l]->stream);
            if (ce == cudaSuccess)
                ce = cudaStreamWaitEvent(st, b_events[l], 0);
        }
        if (pers && es == P2V_OK && ce == cudaSuccess)
            es = enqueue_batch_ao(items, count, byw, st);
        if (capture) {
            cudaGraph_t g = nullptr;
            const cudaError_t ee = cudaStreamEndCapture(st, &g);
            if (es == P2V_OK && ce == cudaSuccess && ee == cudaSuccess) {
                ce = cudaGraphInstantiate(&b_exec, g, 0);
                if (ce == cudaSuccess) {
                    b_graph_sig = sig;
                    ce = cudaGraphLaunch(b_exec, st);
                } else {
                    b_exec = nullptr;
                }
            } else if (ce == cudaSuccess) {
                ce = ee;
            }
            if (g)
                cudaGraphDestroy(g);
        } else {
            b_eager_sig = sig;
        }
        if (es != P2V_OK) {
            cudaStreamSynchronize(st);
            return es;
        }
        P2V_CUDA_TRY(ce);
        b_lane_of = lane_of;
    }
    P2V_CUDA_TRY(cudaEventRecord(b_t1, st));
    P2V_CUDA_TRY(cudaStreamSynchronize(st));
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, b_t0, b_t1);
    if (ms_out)
        *ms_out = ms;
    // ---- per-frame results ----
    p2v_status first_err = P2V_OK;
    std::string first_msg;
    if (pers && *b_err_h != 0) {
        first_err = P2V_ETIMEOUT;
        first_msg = "batch AO queue: a work item's dependency wait gave up (queue_wait_polls " +
                    std::to_string(prm.queue_wait_polls) + "); the batch's AO is invalid";
    }
    uint64_t parts = 0;
    for (uint32_t f = 0; f < count; ++f) {
        p2v_stats fsx{};
        const p2v_status fs = finish_frame(*lanes[b_lane_of[f]], b_jobs[f], items[f].volume, fsx);
        parts += fsx.particles_in;
        if (out)
            out[f] = fsx;
        if (fs != P2V_OK && first_err == P2V_OK) {
            first_err = fs;
            first_msg = err;
        }
    }
    stats = p2v_stats{};
    stats.particles_in = parts;
    stats.ms_total = ms;
    if (first_err != P2V_OK) {
        err = first_msg;
        return first_err;
    }
    err.clear();
    return P2V_OK;
}

p2v_status p2v_ctx::mlp_alloc() {
    P2V_CUDA_TRY(mlp_P.ensure(sizeof(float) * MLP_NPARAM));
    P2V_CUDA_TRY(mlp_m.ensure(sizeof(float) * MLP_NPARAM));
    P2V_CUDA_TRY(mlp_v.ensure(sizeof(float) * MLP_NPARAM));
    P2V_CUDA_TRY(mlp_g.ensure(sizeof(float) * MLP_NPARAM));
    P2V_CUDA_TRY(mlp_loss.ensure(sizeof(float) * 4));
    P2V_CUDA_TRY(mlp_w1h.ensure(sizeof(__nv_bfloat16) * MLP_H * MLP_KP));
    P2V_CUDA_TRY(mlp_w2h.ensure(sizeof(__nv_bfloat16) * MLP_H * MLP_H));
    P2V_CUDA_TRY(mlp_lo.ensure(sizeof(float) * MLP_IN));
    P2V_CUDA_TRY(mlp_hi.ensure(sizeof(float) * MLP_IN));
    return P2V_OK;
}

// Uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)) weights, zero biases, last bias `bias3`; Adam state cleared.
void p2v_ctx::mlp_init_params(uint64_t seed, float bias3) {
    std::vector<float> h(MLP_NPARAM, 0.0f);
    std::mt19937_64 rng(seed);
    auto fill = [&](int off, int count, int fan_in) {
        std::uniform_real_distribution<float> u(-1.0f / std::sqrt((float) fan_in), 1.0f / std::sqrt((float) fan_in));
        for (int k = 0; k < count; ++k)
            h[off + k] = u(rng);
    };
    fill(OFF_W1, MLP_H * MLP_IN, MLP_IN);
    fill(OFF_W2, MLP_H * MLP_H, MLP_H);
    fill(OFF_W3, MLP_H, MLP_H);
    h[OFF_B3] = bias3;
    cudaMemcpy(mlp_P.ptr, h.data(), sizeof(float) * MLP_NPARAM, cudaMemcpyHostToDevice);
    cudaMemset(mlp_m.ptr, 0, sizeof(float) * MLP_NPARAM);
    cudaMemset(mlp_v.ptr, 0, sizeof(float) * MLP_NPARAM);
    mlp_step = 0;
    mlp_seed = seed;
}

namespace {
// Grow a device buffer keeping its first `used` bytes.
cudaError_t grow_keep(DevBuf& b, size_t need, size_t used) {
    if (need <= b.bytes)
        return cudaSuccess;
    DevBuf nb;
    cudaError_t e = nb.ensure(need);
    if (e != cudaSuccess)
        return e;
    if (used && b.ptr)
        e = cudaMemcpy(nb.ptr, b.ptr, used, cudaMemcpyDeviceToDevice);
    b.release();
    b = nb;
    return e;
}

constexpr char MLP_MAGIC[8] = {'P', '2', 'V', 'M', 'L', 'P', '0', '3'};
#if P2V_MLP_FSTEPS_BUILD == P2V_MLP_FSTEPS  // (an experimental build may change the step count)
static_assert(P2V_MLP_INPUTS == MLP_IN && P2V_MLP_HIDDEN == MLP_H && P2V_MLP_PARAMS == MLP_NPARAM &&
                  P2V_MLP_CONES == MLP_CONES && P2V_MLP_FSTEPS == MLP_FSTEPS,
              "the header's MLP sizes differ from the kernels'");
#endif
}  // namespace

extern "C" {

int p2v_abi_version(void) {
    return P2V_ABI_VERSION;
}

void p2v_params_default(p2v_params* p) {
    if (!p)
        return;
    std::memset(p, 0, sizeof(*p));
    p->struct_size = sizeof(p2v_params);
    p->aggregator = 0;
    p->sizex = p->sizey = p->sizez = 16;  // ParticlesToDensity.cpp:126-131
    p->cyclX = p->cyclY = p->cyclZ = 1;   // :133-138
    p->normalize = 1;                     // :140
    p->sigma = 1.0f;                      // :143-144
    p->forSurfaceReconstruction = 0;      // :147
    p->kernel = P2V_KERNEL_BUMP;
    p->mass_normalize = 0;
    p->accumulate = P2V_ACCUM_EXACT;
    p->ao_mode = P2V_AO_NONE;
    p->ao_volume = P2V_AOVOL_DENSITY;
    p->ao_volume_scale = 1.0f;
    p->ao_cones = 3;                      // SphereRenderer.cpp:2572-2587
    p->ao_steps = 0;
    p->ao_levels = 0;                     // 0: ceil(log2(volume size)) levels (SphereRenderer.cpp:2476)
    p->ao_apex_deg = 50.0f;               // SphereRenderer.cpp:202
    p->ao_offset = 0.01f;                 // :205
    p->ao_strength = 1.0f;                // :208
    p->ao_cone_length = 0.8f;             // :211
    p->ao_early_exit = 1;
    p->mdao_volume_size = 128;            // :199
    p->mdao_unorm8 = 1;
    p->aos_sizex = p->aos_sizey = p->aos_sizez = 32;  // AOSphereRenderer.cpp:83-124
    p->aos_step_len = 0.5f;
    p->aos_gen_fac = 1.0f;
    p->aos_eval_fac = 1.0f;
    p->batch_lanes = 0;
    p->batch_graph = 1;
    p->vector_grid = 0;
    p->aos_deposit = P2V_AOS_DEPOSIT_CPU;  // AOSphereRenderer "vol::gen" (0 = CPU)
    p->aos_clip = 0;                       // "ao::clipData" (false)
    for (float& c : p->aos_clip_plane)
        c = 0.0f;
    p->ao_normals = P2V_NORMALS_LIST;
    p->mma_wait_polls = 0;
    p->test_hold_mma = 0;
    p->slab_z0 = p->slab_z1 = 0;
    p->batch_persistent = -1;
    p->queue_wait_polls = 0;
    p->test_hold_queue = 0;
    p->sort_wait_polls = 0;
    p->test_hold_sort = 0;
    p->ao_march = P2V_AO_MARCH_THREAD;
    p->ao_brick_order = 0;
}

p2v_status p2v_create(p2v_ctx** out, int device) {
    if (!out)
        return P2V_EINVAL;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev)
        return P2V_ECUDA;
    auto* c = new (std::nothrow) p2v_ctx();
    if (!c)
        return P2V_ENOMEM;
    c->device = device;
    p2v_params_default(&c->prm);
    if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete c;
        return P2V_ECUDA;
    }
    cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, device);
    if (c->main.init(false) != cudaSuccess) {
        p2v_destroy(c);
        return P2V_ENOMEM;
    }
    *out = c;
    return P2V_OK;
}

void p2v_destroy(p2v_ctx* c) {
    if (!c)
        return;
    cudaSetDevice(c->device);
    if (c->own_stream)
        cudaStreamSynchronize(c->own_stream);
    c->drop_graph();
    for (auto e : c->b_events)
        cudaEventDestroy(e);
    if (c->b_t0)
        cudaEventDestroy(c->b_t0);
    if (c->b_t1)
        cudaEventDestroy(c->b_t1);
    if (c->b_scal)
        cudaFreeHost(c->b_scal);
    c->main.release();
    for (auto& l : c->lanes)
        l->release();
    c->lanes.clear();
    for (auto& sl : c->b_slots)
        sl->release();
    c->b_slots.clear();
    for (DevBuf* b : {&c->b_frames_d, &c->b_segs_d, &c->b_words})
        b->release();
    if (c->b_frames_h)
        cudaFreeHost(c->b_frames_h);
    if (c->b_segs_h)
        cudaFreeHost(c->b_segs_h);
    if (c->b_err_h)
        cudaFreeHost(c->b_err_h);
    for (DevBuf* b : {&c->mlp_P, &c->mlp_m, &c->mlp_v, &c->mlp_g, &c->mlp_part, &c->mlp_ploss, &c->mlp_loss,
                      &c->mlp_w1h, &c->mlp_w2h, &c->mlp_lo, &c->mlp_hi, &c->mlp_idx, &c->mlp_y, &c->tX, &c->tT})
        b->release();
    if (c->own_stream)
        cudaStreamDestroy(c->own_stream);
    delete c;
}

p2v_status p2v_set_params(p2v_ctx* c, const p2v_params* p) {
    if (!c || !p)
        return P2V_EINVAL;
    if (p->struct_size != sizeof(p2v_params))
        return c->fail(P2V_EINVAL, "p2v_params.struct_size %u != %zu (ABI mismatch)", p->struct_size, sizeof(p2v_params));
    c->prm = *p;
    return P2V_OK;
}

p2v_status p2v_get_params(const p2v_ctx* c, p2v_params* p) {
    if (!c || !p)
        return P2V_EINVAL;
    *p = c->prm;
    return P2V_OK;
}

p2v_status p2v_run_frame(p2v_ctx* c, const p2v_frame* fr, p2v_volume* vol, void* stream) {
    if (!c || !fr)
        return P2V_EINVAL;
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : c->own_stream;
    return c->run_frame(fr, vol, st);
}

p2v_status p2v_run_ao_on_grid(p2v_ctx* c, const p2v_frame* fr, const float* grid, int32_t mem, void* stream) {
    if (!c || !fr || !grid || (mem != P2V_MEM_HOST && mem != P2V_MEM_DEVICE))
        return P2V_EINVAL;
    if (c->prm.ao_mode == P2V_AO_NONE || c->prm.aggregator != 0 || c->prm.slab_z0 != 0 || c->prm.slab_z1 != 0)
        return c->fail(P2V_EINVAL, "p2v_run_ao_on_grid needs an AO mode, the density aggregator and no z-slab");
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : c->own_stream;
    c->ext_grid = grid;
    c->ext_grid_mem = mem;
    const p2v_status s = c->run_frame(fr, nullptr, st);
    c->ext_grid = nullptr;
    return s;
}

p2v_status p2v_run_batch(p2v_ctx* c, const p2v_batch_item* items, uint32_t count, p2v_stats* stats, void* stream) {
    if (!c || (count > 0 && !items))
        return P2V_EINVAL;
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : c->own_stream;
    return c->run_batch(items, count, stats, st, true, nullptr);
}

p2v_status p2v_autotune_batch(p2v_ctx* c, const p2v_batch_item* items, uint32_t count, p2v_tune_report* rep) {
    if (!c || count == 0 || !items)
        return P2V_EINVAL;
    if (rep && rep->struct_size != sizeof(p2v_tune_report))
        return c->fail(P2V_EINVAL, "p2v_tune_report.struct_size %u != %zu", rep->struct_size, sizeof(p2v_tune_report));
    if (c->prm.accumulate != P2V_ACCUM_EXACT)
        return c->fail(P2V_EUNSUPPORTED, "the autotuner chooses tiles of the exact accumulation");
    static const int tiles[][3] = {{16, 16, 16}, {16, 8, 8}, {32, 16, 8}};
    static const int lane_opts[] = {1, 2, 4, 8};
    const p2v_params saved = c->prm;
    const int saved_tile[3] = {c->tuned_tile[0], c->tuned_tile[1], c->tuned_tile[2]};
    const int saved_lanes = c->tuned_lanes;
    const int npers = c->batch_persistent_possible() ? 2 : 1;
    float best = INFINITY;
    int bt = -1, bl = -1, bp = 0, nc = 0;
    p2v_status st = P2V_OK;
    for (int t = 0; t < 3 && st == P2V_OK; ++t)
        for (int l : lane_opts)
            for (int pers = 0; pers < npers && st == P2V_OK; ++pers) {
                c->prm.tile_x = c->prm.tile_y = c->prm.tile_z = 0;
                c->prm.batch_lanes = l;
                c->prm.batch_persistent = pers;
                c->tuned_tile[0] = tiles[t][0];
                c->tuned_tile[1] = tiles[t][1];
                c->tuned_tile[2] = tiles[t][2];
                float ms = 0.0f;
                st = c->run_batch(items, count, nullptr, c->own_stream, false, nullptr);  // warm-up, sizes buffers
                if (st == P2V_OK)
                    st = c->run_batch(items, count, nullptr, c->own_stream, false, &ms);
                if (st != P2V_OK)
                    break;
                if (rep && nc < P2V_TUNE_MAX) {
                    for (int a = 0; a < 3; ++a)
                        rep->cand_tile[nc][a] = tiles[t][a];
                    rep->cand_lanes[nc] = l;
                    rep->cand_ms[nc] = ms;
                    rep->cand_persistent[nc] = pers;
                }
                ++nc;
                if (ms < best) {
                    best = ms;
                    bt = t;
                    bl = l;
                    bp = pers;
                }
            }
    c->prm = saved;
    if (st != P2V_OK || bt < 0) {
        c->tuned_tile[0] = saved_tile[0];
        c->tuned_tile[1] = saved_tile[1];
        c->tuned_tile[2] = saved_tile[2];
        c->tuned_lanes = saved_lanes;
        return st != P2V_OK ? st : c->fail(P2V_ECUDA, "autotune measured nothing");
    }
    for (int a = 0; a < 3; ++a)
        c->tuned_tile[a] = tiles[bt][a];
    c->tuned_lanes = bl;
    c->tuned_persistent = bp;
    c->drop_graph();
    if (rep) {
        for (int a = 0; a < 3; ++a)
            rep->tile[a] = tiles[bt][a];
        rep->lanes = bl;
        rep->persistent = bp;
        rep->ms_best = best;
        rep->candidates = std::min(nc, P2V_TUNE_MAX);
    }
    return P2V_OK;
}

p2v_status p2v_get_device_volume(p2v_ctx* c, const float** dptr, uint64_t resolution[3]) {
    if (!c || !dptr)
        return P2V_EINVAL;
    if (!c->main.last_grid)
        return c->fail(P2V_EINVAL, "no volume computed yet");
    *dptr = c->main.last_grid;
    if (resolution)
        for (int a = 0; a < 3; ++a)
            resolution[a] = c->main.last_res[a];
    return P2V_OK;
}

p2v_status p2v_get_ao_volume(p2v_ctx* c, int32_t level, float* out, uint64_t capacity, int32_t mem,
                             int32_t dims[3]) {
    if (!c || level < 0)
        return P2V_EINVAL;
    const ConeParams& cp = c->main.last_cp;
    if (cp.nlevels < 1 || !cp.lv[0].v)
        return c->fail(P2V_EINVAL, "no cone-march volume computed yet");
    if (level >= cp.nlevels)
        return c->fail(P2V_EINVAL, "level %d does not exist (the last pyramid has %d levels)", level, cp.nlevels);
    const ConeLevel& L = cp.lv[level];
    if (dims)
        for (int a = 0; a < 3; ++a)
            dims[a] = L.d[a];
    if (!out)
        return P2V_OK;
    const uint64_t nv = (uint64_t) L.d[0] * L.d[1] * L.d[2];
    if (capacity < nv)
        return c->fail(P2V_EINVAL, "output capacity %llu < %llu texels", (unsigned long long) capacity,
                       (unsigned long long) nv);
    if (mem != P2V_MEM_HOST && mem != P2V_MEM_DEVICE)
        return c->fail(P2V_EINVAL, "mem must be P2V_MEM_HOST or P2V_MEM_DEVICE");
    cudaError_t e = cudaSetDevice(c->device);
    if (e == cudaSuccess)
        e = cudaDeviceSynchronize();
    if (e == cudaSuccess)
        e = cudaMemcpy(out, L.v, sizeof(float) * nv,
                       mem == P2V_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost);
    if (e != cudaSuccess)
        return c->fail(P2V_ECUDA, "AO volume copy failed: %s", cudaGetErrorString(e));
    return P2V_OK;
}

p2v_status p2v_get_binning(p2v_ctx* c, uint32_t* keys, uint32_t* order, uint64_t capacity, uint32_t* cell_start,
                           uint64_t start_capacity, uint32_t* count, uint32_t* nbins) {
    if (!c)
        return P2V_EINVAL;
    const Pipe& pp = c->main;
    if (!pp.last_keys)
        return c->fail(P2V_EINVAL, "no frame binned yet");
    if (count)
        *count = pp.last_n;
    if (nbins)
        *nbins = pp.last_nbins;
    if ((keys || order) && capacity < pp.last_n)
        return c->fail(P2V_EINVAL, "capacity %llu < %u particles", (unsigned long long) capacity, pp.last_n);
    if (cell_start && start_capacity < (uint64_t) pp.last_nbins + 1)
        return c->fail(P2V_EINVAL, "start capacity %llu < %u bins + 1", (unsigned long long) start_capacity,
                       pp.last_nbins);
    cudaError_t e = cudaSetDevice(c->device);
    if (e == cudaSuccess)
        e = cudaDeviceSynchronize();
    // the counting sort by cell writes no sorted keys: rebuild them from the cell starts
    const bool counted = c->stats.cell_max_count > 0 && c->stats.cell_max_count <= 32;
    if (e == cudaSuccess && keys && pp.last_n && counted) {
        e = launch_keys_from_starts(pp.cstart.as<uint32_t>(), pp.last_nbins, pp.last_n,
                                    const_cast<uint32_t*>(pp.last_keys), c->sms, 0);
        if (e == cudaSuccess)
            e = cudaDeviceSynchronize();
    }
    if (e == cudaSuccess && keys && pp.last_n)
        e = cudaMemcpy(keys, pp.last_keys, sizeof(uint32_t) * pp.last_n, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && order && pp.last_n)
        e = cudaMemcpy(order, pp.last_order, sizeof(uint32_t) * pp.last_n, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && cell_start)
        e = cudaMemcpy(cell_start, pp.cstart.ptr, sizeof(uint32_t) * ((size_t) pp.last_nbins + 1),
                       cudaMemcpyDeviceToHost);
    if (e != cudaSuccess)
        return c->fail(P2V_ECUDA, "binning copy failed: %s", cudaGetErrorString(e));
    return P2V_OK;
}

p2v_status p2v_get_vector_grid(p2v_ctx* c, float* positions, float* directions, float* colours, float* info,
                               uint64_t capacity, int32_t mem, p2v_vector_grid_info* meta) {
    if (!c)
        return P2V_EINVAL;
    Pipe& pp = c->main;
    if (!pp.vg_order)
        return c->fail(P2V_EINVAL, "no vector grid: run a frame with aggregator 2 and vector_grid set");
    const uint32_t n = pp.vg_count;
    if (meta) {
        meta->count = n;
        meta->global_radius = pp.vg_radius;
        for (int a = 0; a < 3; ++a) {  // vislib Cuboid Left/Right, Bottom/Top, Back/Front
            meta->col_min[a] = pp.vg_bbox[a];
            meta->col_max[a] = pp.vg_bbox[a + 3];
            meta->col_min[3 + a] = -1.0f;
            meta->col_max[3 + a] = 1.0f;
        }
        meta->col_min[6] = pp.vg_range[0];
        meta->col_max[6] = pp.vg_range[1];
    }
    if (!positions && !directions && !colours && !info)
        return P2V_OK;
    if (capacity < n)
        return c->fail(P2V_EINVAL, "capacity %llu < %u grid entries", (unsigned long long) capacity, n);
    if (mem != P2V_MEM_HOST && mem != P2V_MEM_DEVICE)
        return c->fail(P2V_EINVAL, "mem must be P2V_MEM_HOST or P2V_MEM_DEVICE");
    cudaError_t e = cudaSetDevice(c->device);
    if (e == cudaSuccess)
        e = cudaDeviceSynchronize();
    if (e != cudaSuccess)
        return c->fail(P2V_ECUDA, "vector grid: %s", cudaGetErrorString(e));
    if (n == 0)
        return P2V_OK;
    float* d_out[4] = {positions, directions, colours, info};
    const int width[4] = {3, 3, 1, 7};
    if (mem == P2V_MEM_HOST) {  // staged in device memory, then copied
        uint64_t off = 0;
        uint64_t offs[4];
        for (int k = 0; k < 4; ++k) {
            offs[k] = off;
            if (d_out[k])
                off += (uint64_t) width[k] * n;
        }
        e = pp.vout.ensure(sizeof(float) * off);
        if (e != cudaSuccess)
            return c->fail(P2V_ENOMEM, "vector grid staging: %s", cudaGetErrorString(e));
        for (int k = 0; k < 4; ++k)
            d_out[k] = d_out[k] ? pp.vout.as<float>() + offs[k] : nullptr;
    }
    e = launch_vector_grid(pp.vg_order, pp.vdens.as<float>(), pp.vdirs.as<float>(), pp.scal.as<FrameScalars>(),
                           pp.vg_geo, n, d_out[0], d_out[1], d_out[2], d_out[3], c->sms, 0);
    if (e == cudaSuccess)
        e = cudaDeviceSynchronize();
    float* h_out[4] = {positions, directions, colours, info};
    for (int k = 0; k < 4 && e == cudaSuccess && mem == P2V_MEM_HOST; ++k)
        if (h_out[k])
            e = cudaMemcpy(h_out[k], d_out[k], sizeof(float) * width[k] * n, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess)
        return c->fail(P2V_ECUDA, "vector grid: %s", cudaGetErrorString(e));
    return P2V_OK;
}

p2v_status p2v_get_stats(const p2v_ctx* c, p2v_stats* st) {
    if (!c || !st)
        return P2V_EINVAL;
    *st = c->stats;
    return P2V_OK;
}

size_t p2v_get_last_error(const p2v_ctx* c, char* buf, size_t len) {
    if (!c)
        return 0;
    if (buf && len) {
        std::strncpy(buf, c->err.c_str(), len - 1);
        buf[len - 1] = '\0';
    }
    return c->err.size();
}

}  // extern "C"

extern "C" {

void p2v_train_params_default(p2v_train_params* tp) {
    if (!tp)
        return;
    std::memset(tp, 0, sizeof(*tp));
    tp->struct_size = sizeof(p2v_train_params);
    tp->epochs = 16;
    tp->batch = 2048;
    tp->lr = 3e-3f;
    tp->beta1 = 0.9f;
    tp->beta2 = 0.999f;
    tp->eps = 1e-8f;
    tp->lr_decay = 0.8f;
    tp->val_fraction = 0.05f;
    tp->range_margin = 0.05f;
    tp->seed = 12345;
}

p2v_status p2v_mlp_clear(p2v_ctx* c) {
    if (!c)
        return P2V_EINVAL;
    c->t_pairs = 0;
    c->t_valid.clear();
    c->t_host_T.clear();
    return P2V_OK;
}

p2v_status p2v_mlp_collect(p2v_ctx* c, const p2v_frame* fr, uint32_t max_pairs, uint64_t seed, uint64_t* total) {
    if (!c || !fr)
        return P2V_EINVAL;
    const p2v_params saved = c->prm;
    c->prm.ao_mode = P2V_AO_CONE;
    p2v_status st = c->run_frame(fr, nullptr, c->own_stream);
    c->prm = saved;
    if (st != P2V_OK)
        return st;
    const uint32_t nvalid = (uint32_t) c->stats.particles_binned;
    const uint32_t nsel = std::min(max_pairs, nvalid);
    if (nsel > 0) {
        const p2v_status ps = c->prepare_features(c->main, c->main.last_cp, c->own_stream);
        if (ps != P2V_OK)
            return ps;
        std::vector<uint32_t> sel(nvalid);
        std::iota(sel.begin(), sel.end(), 0u);
        if (nsel < nvalid) {
            std::mt19937_64 rng(seed);
            for (uint32_t i = 0; i < nsel; ++i) {
                std::uniform_int_distribution<uint32_t> d(i, nvalid - 1);
                std::swap(sel[i], sel[d(rng)]);
            }
            sel.resize(nsel);
            std::sort(sel.begin(), sel.end());
        }
        if (cudaSetDevice(c->device) != cudaSuccess)
            return c->fail(P2V_ECUDA, "cudaSetDevice failed");
        const uint64_t newp = c->t_pairs + nsel;
        if (grow_keep(c->tX, sizeof(float) * newp * MLP_IN, sizeof(float) * c->t_pairs * MLP_IN) != cudaSuccess ||
            grow_keep(c->tT, sizeof(float) * newp, sizeof(float) * c->t_pairs) != cudaSuccess ||
            c->mlp_idx.ensure(sizeof(uint32_t) * (nsel + 4)) != cudaSuccess)
            return c->fail(P2V_ENOMEM, "training buffer of %llu pairs", (unsigned long long) newp);
        uint32_t* d_sel = c->mlp_idx.as<uint32_t>();
        uint32_t* d_kept = d_sel + nsel;
        cudaMemcpyAsync(d_sel, sel.data(), sizeof(uint32_t) * nsel, cudaMemcpyHostToDevice, c->own_stream);
        cudaMemsetAsync(d_kept, 0, sizeof(uint32_t), c->own_stream);
        cudaError_t e = launch_mlp_collect(c->main.last_cp, c->main.last_order, d_sel, nsel, c->main.xyzr_s.as<float4>(),
                                           c->main.nrm_s.as<float4>(), c->main.ao.as<float>(),
                                           c->tX.as<float>() + c->t_pairs * MLP_IN, c->tT.as<float>() + c->t_pairs,
                                           d_kept, c->own_stream);
        if (e != cudaSuccess)
            return c->fail(P2V_ECUDA, "collect: %s", cudaGetErrorString(e));
        std::vector<float> ht(nsel);
        cudaMemcpyAsync(ht.data(), c->tT.as<float>() + c->t_pairs, sizeof(float) * nsel, cudaMemcpyDeviceToHost,
                        c->own_stream);
        if ((e = cudaStreamSynchronize(c->own_stream)) != cudaSuccess)
            return c->fail(P2V_ECUDA, "collect: %s", cudaGetErrorString(e));
        c->t_host_T.resize(newp);
        for (uint32_t i = 0; i < nsel; ++i) {
            c->t_host_T[c->t_pairs + i] = ht[i];
            if (ht[i] >= 0.0f)
                c->t_valid.push_back((uint32_t) (c->t_pairs + i));
        }
        c->t_pairs = newp;
    }
    if (total)
        *total = c->t_valid.size();
    return P2V_OK;
}

p2v_status p2v_mlp_get_pairs(p2v_ctx* c, float* x, float* t, uint64_t capacity, uint64_t* count) {
    if (!c)
        return P2V_EINVAL;
    if (count)
        *count = c->t_pairs;
    if (!x && !t)
        return P2V_OK;
    if (capacity < c->t_pairs)
        return c->fail(P2V_EINVAL, "capacity %llu < %llu pairs", (unsigned long long) capacity,
                       (unsigned long long) c->t_pairs);
    cudaError_t e = cudaSetDevice(c->device);
    if (e == cudaSuccess)
        e = cudaDeviceSynchronize();
    if (e == cudaSuccess && x && c->t_pairs)
        e = cudaMemcpy(x, c->tX.as<float>(), sizeof(float) * MLP_IN * c->t_pairs, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && t && c->t_pairs)
        e = cudaMemcpy(t, c->tT.as<float>(), sizeof(float) * c->t_pairs, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess)
        return c->fail(P2V_ECUDA, "pairs copy failed: %s", cudaGetErrorString(e));
    return P2V_OK;
}

p2v_status p2v_mlp_train(p2v_ctx* c, const p2v_train_params* tp, p2v_train_report* rep) {
    if (!c || !tp)
        return P2V_EINVAL;
    if (tp->struct_size != sizeof(p2v_train_params))
        return c->fail(P2V_EINVAL, "p2v_train_params.struct_size mismatch");
    if (tp->epochs < 1 || tp->batch < 1 || tp->batch > (1 << 20) || !(tp->lr > 0.0f))
        return c->fail(P2V_EINVAL, "invalid training parameters");
    if (c->t_valid.size() < 2)
        return c->fail(P2V_EINVAL, "no training pairs (p2v_mlp_collect first)");
    const auto t0 = std::chrono::steady_clock::now();
    if (cudaSetDevice(c->device) != cudaSuccess)
        return c->fail(P2V_ECUDA, "cudaSetDevice failed");
    p2v_status ps = c->mlp_alloc();
    if (ps != P2V_OK)
        return ps;
    std::vector<uint32_t> all = c->t_valid;
    std::mt19937_64 rng(tp->seed);
    std::shuffle(all.begin(), all.end(), rng);
    size_t nval = (size_t) std::floor(tp->val_fraction * (double) all.size());
    nval = std::min(nval, all.size() - 1);
    std::vector<uint32_t> val(all.begin(), all.begin() + nval), train(all.begin() + nval, all.end());
    std::sort(val.begin(), val.end());
    double mean = 0.0;
    for (uint32_t i : train)
        mean += c->t_host_T[i];
    mean /= (double) train.size();
    mean = std::min(std::max(mean, 1e-3), 1.0 - 1e-3);
    c->mlp_init_params(tp->seed, (float) std::log(mean / (1.0 - mean)));

    const int batch = tp->batch;
    const int nblk = (batch + 31) / 32;
    if (c->mlp_idx.ensure(sizeof(uint32_t) * (train.size() + val.size() + 8)) != cudaSuccess ||
        c->mlp_part.ensure(sizeof(float) * (size_t) nblk * MLP_NPARAM) != cudaSuccess ||
        c->mlp_ploss.ensure(sizeof(float) * nblk) != cudaSuccess ||
        c->mlp_y.ensure(sizeof(float) * (val.size() + 1)) != cudaSuccess)
        return c->fail(P2V_ENOMEM, "training buffers");
    uint32_t* d_idx = c->mlp_idx.as<uint32_t>();
    uint32_t* d_val = d_idx + train.size();
    cudaStream_t st = c->own_stream;
    // feature ranges of the training pairs (the learned path falls back outside them)
    cudaMemcpyAsync(d_idx, train.data(), sizeof(uint32_t) * train.size(), cudaMemcpyHostToDevice, st);
    cudaError_t e = launch_mlp_range(c->tX.as<float>(), d_idx, (uint32_t) train.size(), tp->range_margin,
                                     c->mlp_lo.as<float>(), c->mlp_hi.as<float>(), st);
    if (e != cudaSuccess)
        return c->fail(P2V_ECUDA, "range: %s", cudaGetErrorString(e));
    float lr = tp->lr;
    int steps = 0;
    for (int ep = 0; ep < tp->epochs; ++ep) {
        std::mt19937_64 er(tp->seed + 1 + (uint64_t) ep);
        std::shuffle(train.begin(), train.end(), er);
        cudaMemcpyAsync(d_idx, train.data(), sizeof(uint32_t) * train.size(), cudaMemcpyHostToDevice, st);
        for (size_t b0 = 0; b0 < train.size(); b0 += (size_t) batch) {
            const int nb = (int) std::min<size_t>((size_t) batch, train.size() - b0);
            e = launch_mlp_train_step(c->mlp_P.as<float>(), c->tX.as<float>(), c->tT.as<float>(), d_idx + b0, nb,
                                      c->mlp_part.as<float>(), c->mlp_ploss.as<float>(), c->mlp_g.as<float>(),
                                      c->mlp_loss.as<float>(), st);
            if (e == cudaSuccess)
                e = launch_mlp_adam(c->mlp_P.as<float>(), c->mlp_g.as<float>(), c->mlp_m.as<float>(),
                                    c->mlp_v.as<float>(), lr, tp->beta1, tp->beta2, tp->eps, ++c->mlp_step, st);
            if (e != cudaSuccess)
                return c->fail(P2V_ECUDA, "train step: %s", cudaGetErrorString(e));
            ++steps;
        }
        lr *= tp->lr_decay;
    }
    float last_loss = 0.0f;
    cudaMemcpyAsync(&last_loss, c->mlp_loss.ptr, sizeof(float), cudaMemcpyDeviceToHost, st);
    const size_t last_nb = train.size() % (size_t) batch ? train.size() % (size_t) batch : (size_t) batch;
    float val_rmse = 0.0f, val_max = 0.0f;
    if (!val.empty()) {
        cudaMemcpyAsync(d_val, val.data(), sizeof(uint32_t) * val.size(), cudaMemcpyHostToDevice, st);
        launch_mlp_forward_f32(c->mlp_P.as<float>(), c->tX.as<float>(), d_val, (uint32_t) val.size(),
                               c->mlp_y.as<float>(), st);
        std::vector<float> y(val.size());
        cudaMemcpyAsync(y.data(), c->mlp_y.ptr, sizeof(float) * val.size(), cudaMemcpyDeviceToHost, st);
        if ((e = cudaStreamSynchronize(st)) != cudaSuccess)
            return c->fail(P2V_ECUDA, "validation: %s", cudaGetErrorString(e));
        double se = 0.0;
        for (size_t k = 0; k < val.size(); ++k) {
            const double d = (double) y[k] - c->t_host_T[val[k]];
            se += d * d;
            val_max = std::max(val_max, (float) std::fabs(d));
        }
        val_rmse = (float) std::sqrt(se / (double) val.size());
    }
    e = launch_mlp_pack(c->mlp_P.as<float>(), c->mlp_w1h.as<__nv_bfloat16>(), c->mlp_w2h.as<__nv_bfloat16>(), st);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(st);
    if (e != cudaSuccess)
        return c->fail(P2V_ECUDA, "pack: %s", cudaGetErrorString(e));
    c->mlp_ready = true;
    c->mlp_has_range = true;
    if (rep) {
        rep->pairs_train = train.size();
        rep->pairs_val = val.size();
        rep->steps = steps;
        rep->final_loss = last_loss / (float) last_nb;
        rep->val_rmse = val_rmse;
        rep->val_max_err = val_max;
        rep->ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }
    return P2V_OK;
}

p2v_status p2v_mlp_get_weights(p2v_ctx* c, float* out, uint64_t count) {
    if (!c || !out || count < (uint64_t) MLP_NPARAM)
        return P2V_EINVAL;
    if (!c->mlp_P.ptr)
        return c->fail(P2V_EINVAL, "no network");
    cudaSetDevice(c->device);
    if (cudaMemcpy(out, c->mlp_P.ptr, sizeof(float) * MLP_NPARAM, cudaMemcpyDeviceToHost) != cudaSuccess)
        return c->fail(P2V_ECUDA, "copy failed");
    return P2V_OK;
}

p2v_status p2v_mlp_set_weights(p2v_ctx* c, const float* in, uint64_t count) {
    if (!c || !in || count < (uint64_t) MLP_NPARAM)
        return P2V_EINVAL;
    cudaSetDevice(c->device);
    p2v_status ps = c->mlp_alloc();
    if (ps != P2V_OK)
        return ps;
    if (cudaMemcpy(c->mlp_P.ptr, in, sizeof(float) * MLP_NPARAM, cudaMemcpyHostToDevice) != cudaSuccess ||
        launch_mlp_pack(c->mlp_P.as<float>(), c->mlp_w1h.as<__nv_bfloat16>(), c->mlp_w2h.as<__nv_bfloat16>(),
                        nullptr) != cudaSuccess ||
        cudaDeviceSynchronize() != cudaSuccess)
        return c->fail(P2V_ECUDA, "set weights failed");
    cudaMemset(c->mlp_m.ptr, 0, sizeof(float) * MLP_NPARAM);
    cudaMemset(c->mlp_v.ptr, 0, sizeof(float) * MLP_NPARAM);
    c->mlp_step = 0;
    c->mlp_ready = true;
    c->mlp_has_range = false;
    return P2V_OK;
}

p2v_status p2v_mlp_gradients(p2v_ctx* c, const float* x, const float* t, uint32_t n, float* grad, float* loss) {
    if (!c || !x || !t || !grad || n == 0 || !c->mlp_P.ptr)
        return P2V_EINVAL;
    cudaSetDevice(c->device);
    const int nblk = (int) ((n + 31) / 32);
    DevBuf dx, dt, di;
    if (dx.ensure(sizeof(float) * (size_t) n * MLP_IN) != cudaSuccess || dt.ensure(sizeof(float) * n) != cudaSuccess ||
        di.ensure(sizeof(uint32_t) * n) != cudaSuccess ||
        c->mlp_part.ensure(sizeof(float) * (size_t) nblk * MLP_NPARAM) != cudaSuccess ||
        c->mlp_ploss.ensure(sizeof(float) * nblk) != cudaSuccess) {
        dx.release();
        dt.release();
        di.release();
        return c->fail(P2V_ENOMEM, "gradient buffers");
    }
    std::vector<uint32_t> idx(n);
    std::iota(idx.begin(), idx.end(), 0u);
    cudaMemcpy(dx.ptr, x, sizeof(float) * (size_t) n * MLP_IN, cudaMemcpyHostToDevice);
    cudaMemcpy(dt.ptr, t, sizeof(float) * n, cudaMemcpyHostToDevice);
    cudaMemcpy(di.ptr, idx.data(), sizeof(uint32_t) * n, cudaMemcpyHostToDevice);
    cudaError_t e = launch_mlp_train_step(c->mlp_P.as<float>(), dx.as<float>(), dt.as<float>(), di.as<uint32_t>(),
                                          (int) n, c->mlp_part.as<float>(), c->mlp_ploss.as<float>(),
                                          c->mlp_g.as<float>(), c->mlp_loss.as<float>(), nullptr);
    float l = 0.0f;
    if (e == cudaSuccess)
        e = cudaMemcpy(grad, c->mlp_g.ptr, sizeof(float) * MLP_NPARAM, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess)
        e = cudaMemcpy(&l, c->mlp_loss.ptr, sizeof(float), cudaMemcpyDeviceToHost);
    dx.release();
    dt.release();
    di.release();
    if (e != cudaSuccess)
        return c->fail(P2V_ECUDA, "gradients: %s", cudaGetErrorString(e));
    if (loss)
        *loss = l / (float) n;
    return P2V_OK;
}

p2v_status p2v_mlp_infer(p2v_ctx* c, const float* x, uint32_t n, float* y) {
    if (!c || !x || !y || n == 0)
        return P2V_EINVAL;
    if (!c->mlp_ready)
        return c->fail(P2V_EINVAL, "no trained network");
    cudaSetDevice(c->device);
    DevBuf dx, dy;
    // dy holds the n outputs and, after them, the kernel's error word
    if (dx.ensure(sizeof(float) * (size_t) n * MLP_IN) != cudaSuccess ||
        dy.ensure(sizeof(float) * ((size_t) n + 1)) != cudaSuccess) {
        dx.release();
        dy.release();
        return c->fail(P2V_ENOMEM, "inference buffers");
    }
    cudaError_t e = cudaMemcpy(dx.ptr, x, sizeof(float) * (size_t) n * MLP_IN, cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemset(dy.as<float>() + n, 0, sizeof(uint32_t));
    MlpInferArgs a{};
    a.P = c->mlp_P.as<float>();
    a.w1h = c->mlp_w1h.as<__nv_bfloat16>();
    a.w2h = c->mlp_w2h.as<__nv_bfloat16>();
    a.n = n;
    a.X = dx.as<float>();
    a.y = dy.as<float>();
    a.err = reinterpret_cast<uint32_t*>(dy.as<float>() + n);
    if (e == cudaSuccess)
        e = launch_mlp_infer(a, c->main.last_cp, true, c->sms, nullptr);
    uint32_t derr = 0;
    if (e == cudaSuccess)
        e = cudaMemcpy(y, dy.ptr, sizeof(float) * n, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess)
        e = cudaMemcpy(&derr, a.err, sizeof(uint32_t), cudaMemcpyDeviceToHost);
    dx.release();
    dy.release();
    if (e != cudaSuccess)
        return c->fail(P2V_ECUDA, "infer: %s", cudaGetErrorString(e));
    if (derr & ERR_MMA_TIMEOUT)
        return c->fail(P2V_ETIMEOUT, "tensor-core MMA wait gave up (device error 0x%x)", derr);
    return P2V_OK;
}

p2v_status p2v_mlp_save(p2v_ctx* c, const char* path) {
    if (!c || !path || !c->mlp_ready)
        return c ? c->fail(P2V_EINVAL, "no trained network to save") : P2V_EINVAL;
    cudaSetDevice(c->device);
    std::vector<float> P(MLP_NPARAM), m(MLP_NPARAM), v(MLP_NPARAM), lo(MLP_IN, -INFINITY), hi(MLP_IN, INFINITY);
    cudaMemcpy(P.data(), c->mlp_P.ptr, sizeof(float) * MLP_NPARAM, cudaMemcpyDeviceToHost);
    cudaMemcpy(m.data(), c->mlp_m.ptr, sizeof(float) * MLP_NPARAM, cudaMemcpyDeviceToHost);
    cudaMemcpy(v.data(), c->mlp_v.ptr, sizeof(float) * MLP_NPARAM, cudaMemcpyDeviceToHost);
    if (c->mlp_has_range) {
        cudaMemcpy(lo.data(), c->mlp_lo.ptr, sizeof(float) * MLP_IN, cudaMemcpyDeviceToHost);
        cudaMemcpy(hi.data(), c->mlp_hi.ptr, sizeof(float) * MLP_IN, cudaMemcpyDeviceToHost);
    }
    FILE* f = std::fopen(path, "wb");
    if (!f)
        return c->fail(P2V_EINVAL, "cannot open %s", path);
    const int32_t hdr[7] = {2, MLP_IN, MLP_H, MLP_NPARAM, c->mlp_step, c->mlp_has_range ? 1 : 0, MLP_FSTEPS};
    bool ok = std::fwrite(MLP_MAGIC, 1, 8, f) == 8 && std::fwrite(hdr, sizeof(hdr), 1, f) == 1 &&
              std::fwrite(&c->mlp_seed, sizeof(uint64_t), 1, f) == 1 &&
              std::fwrite(P.data(), sizeof(float), MLP_NPARAM, f) == (size_t) MLP_NPARAM &&
              std::fwrite(m.data(), sizeof(float), MLP_NPARAM, f) == (size_t) MLP_NPARAM &&
              std::fwrite(v.data(), sizeof(float), MLP_NPARAM, f) == (size_t) MLP_NPARAM &&
              std::fwrite(lo.data(), sizeof(float), MLP_IN, f) == (size_t) MLP_IN &&
              std::fwrite(hi.data(), sizeof(float), MLP_IN, f) == (size_t) MLP_IN;
    ok = (std::fclose(f) == 0) && ok;
    return ok ? P2V_OK : c->fail(P2V_EINVAL, "write to %s failed", path);
}

p2v_status p2v_mlp_load(p2v_ctx* c, const char* path) {
    if (!c || !path)
        return P2V_EINVAL;
    FILE* f = std::fopen(path, "rb");
    if (!f)
        return c->fail(P2V_EINVAL, "cannot open %s", path);
    char magic[8];
    int32_t hdr[7];
    uint64_t seed = 0;
    std::vector<float> P(MLP_NPARAM), m(MLP_NPARAM), v(MLP_NPARAM), lo(MLP_IN), hi(MLP_IN);
    bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, MLP_MAGIC, 8) == 0 &&
              std::fread(hdr, sizeof(hdr), 1, f) == 1 && hdr[0] == 2 && hdr[1] == MLP_IN && hdr[2] == MLP_H &&
              hdr[3] == MLP_NPARAM && hdr[6] == MLP_FSTEPS && std::fread(&seed, sizeof(uint64_t), 1, f) == 1 &&
              std::fread(P.data(), sizeof(float), MLP_NPARAM, f) == (size_t) MLP_NPARAM &&
              std::fread(m.data(), sizeof(float), MLP_NPARAM, f) == (size_t) MLP_NPARAM &&
              std::fread(v.data(), sizeof(float), MLP_NPARAM, f) == (size_t) MLP_NPARAM &&
              std::fread(lo.data(), sizeof(float), MLP_IN, f) == (size_t) MLP_IN &&
              std::fread(hi.data(), sizeof(float), MLP_IN, f) == (size_t) MLP_IN;
    std::fclose(f);
    if (!ok)
        return c->fail(P2V_EINVAL, "%s is not a p2v MLP file of this version", path);
    p2v_status ps = p2v_mlp_set_weights(c, P.data(), MLP_NPARAM);
    if (ps != P2V_OK)
        return ps;
    cudaMemcpy(c->mlp_m.ptr, m.data(), sizeof(float) * MLP_NPARAM, cudaMemcpyHostToDevice);
    cudaMemcpy(c->mlp_v.ptr, v.data(), sizeof(float) * MLP_NPARAM, cudaMemcpyHostToDevice);
    c->mlp_step = hdr[4];
    c->mlp_seed = seed;
    c->mlp_has_range = hdr[5] != 0;
    if (c->mlp_has_range) {
        cudaMemcpy(c->mlp_lo.ptr, lo.data(), sizeof(float) * MLP_IN, cudaMemcpyHostToDevice);
        cudaMemcpy(c->mlp_hi.ptr, hi.data(), sizeof(float) * MLP_IN, cudaMemcpyHostToDevice);
    }
    return P2V_OK;
}

}  // extern "C"
