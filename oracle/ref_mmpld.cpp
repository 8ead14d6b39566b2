// Test-only harness that drives MegaMol's own, unmodified moldyn::io::MMPLDDataSource
// (plugins/moldyn/src/io/MMPLDDataSource.cpp) headless through its slots: the "filename" parameter is set
// and its update callback run (filenameChanged, :283-420), then the MultiParticleDataCall GetExtent and
// GetData callbacks of "getdata" are invoked (:426-467) and the lists the module publishes are copied out.
// vislib's String, File/BufferedFile, RawStorage and SystemInformation are compiled from the reference tree;
// the frame cache base class is a synchronous stand-in (shim/mmstd/data/AnimDataModule.h).
//
// This file is ORACLE infrastructure: it is built by oracle/Makefile into oracle/_ref/ (never committed)
// and is called only by tests and by the fixture generator.
#include <cstdint>
#include <cstring>
#include <memory>

#include "io/MMPLDDataSource.h"
#include "mmcore/param/FilePathParam.h"

using namespace megamol;

extern "C" {

// What the module publishes for one list of a frame (SimpleSphericalParticles getters).
struct ref_mmpld_list {
    int32_t vert_type;      // SimpleSphericalParticles::VertexDataType
    int32_t col_type;       // SimpleSphericalParticles::ColourDataType
    uint64_t count;
    float global_radius;
    uint8_t global_colour[4];
    float col_min, col_max; // colour map index values
    uint32_t vert_stride, col_stride; // as the getters report them: 0 for packed records
    float bbox[6];          // GetBBox(): the list's box (version 1.3)
    uint32_t clusters;      // version 1.1 cluster count, 0 without cluster infos
    uint64_t cluster_bytes;
};

struct ref_mmpld_extent {
    uint32_t frames;
    float bbox[6], clipbox[6];
};

} // extern "C"

namespace {

struct Session {
    std::unique_ptr<moldyn::io::MMPLDDataSource> mod;
    geocalls::MultiParticleDataCall call;
    ~Session() {
        call.Unlock();
        if (mod)
            mod->Release();
    }
};

core::CalleeSlot* getdata(Session& S) {
    return dynamic_cast<core::CalleeSlot*>(S.mod->FindSlot("getdata"));
}

void box6(const vislib::math::Cuboid<float>& b, float* out) {
    out[0] = b.Left();
    out[1] = b.Bottom();
    out[2] = b.Back();
    out[3] = b.Right();
    out[4] = b.Top();
    out[5] = b.Front();
}

} // namespace

extern "C" {

// Opens `path` through the module and runs GetExtent; *session receives the handle. Returns 0, or 1 when the
// GetExtent callback failed. A file the module cannot parse is not an error here: the module logs it and
// publishes one frame of the default box (-1..1), as it does in a MegaMol graph.
int ref_mmpld_open(const char* path, void** session, ref_mmpld_extent* ext) {
    auto* S = new Session();
    S->mod = std::make_unique<moldyn::io::MMPLDDataSource>();
    S->mod->Create();
    auto* fn = dynamic_cast<core::param::ParamSlot*>(S->mod->FindSlot("filename"));
    fn->Param<core::param::FilePathParam>()->SetValue(std::filesystem::path(path));
    fn->Update();
    bool ok = getdata(*S)->InCall(geocalls::MultiParticleDataCall::ClassName(),
        geocalls::MultiParticleDataCall::FunctionName(1), S->call);
    ext->frames = S->call.FrameCount();
    box6(S->call.AccessBoundingBoxes().ObjectSpaceBBox(), ext->bbox);
    box6(S->call.AccessBoundingBoxes().ObjectSpaceClipBox(), ext->clipbox);
    *session = S;
    return ok ? 0 : 1;
}

// GetData for frame `frame` (forced, as a renderer stepping through a trajectory requests it); fills at
// most `cap` list descriptions and *n_lists with the frame's list count. Returns 0, or 1 on failure.
int ref_mmpld_frame(void* session, uint32_t frame, ref_mmpld_list* lists, uint32_t cap, uint32_t* n_lists) {
    auto& S = *static_cast<Session*>(session);
    S.call.SetFrameID(frame, true);
    if (!getdata(S)->InCall(geocalls::MultiParticleDataCall::ClassName(),
            geocalls::MultiParticleDataCall::FunctionName(0), S.call))
        return 1;
    const uint32_t n = S.call.GetParticleListCount();
    *n_lists = n;
    for (uint32_t i = 0; i < n && i < cap; ++i) {
        auto& p = S.call.AccessParticles(i);
        ref_mmpld_list& L = lists[i];
        std::memset(&L, 0, sizeof(L));
        L.vert_type = static_cast<int32_t>(p.GetVertexDataType());
        L.col_type = static_cast<int32_t>(p.GetColourDataType());
        L.count = p.GetCount();
        L.global_radius = p.GetGlobalRadius();
        std::memcpy(L.global_colour, p.GetGlobalColour(), 4);
        L.col_min = p.GetMinColourIndexValue();
        L.col_max = p.GetMaxColourIndexValue();
        L.vert_stride = p.GetVertexDataStride();
        L.col_stride = p.GetColourDataStride();
        box6(p.GetBBox(), L.bbox);
        if (auto* ci = p.GetClusterInfos()) {
            L.clusters = ci->numClusters;
            L.cluster_bytes = ci->sizeofPlainData;
        }
    }
    return 0;
}

// Copies the vertex and colour records of list `i` of the last frame, `vert_bytes` / `col_bytes` bytes per
// particle (the record sizes of its types), into packed arrays (either may be null). The getters report a
// stride of 0 for packed records (SimpleSphericalParticles.h:325-327,435-437).
int ref_mmpld_list_data(void* session, uint32_t i, uint32_t vert_bytes, void* vert_out, uint32_t col_bytes,
    void* col_out) {
    auto& S = *static_cast<Session*>(session);
    if (i >= S.call.GetParticleListCount())
        return 1;
    auto& p = S.call.AccessParticles(i);
    const auto* v = static_cast<const uint8_t*>(p.GetVertexData());
    const auto* c = static_cast<const uint8_t*>(p.GetColourData());
    const uint64_t vs = p.GetVertexDataStride() ? p.GetVertexDataStride() : vert_bytes;
    const uint64_t cs = p.GetColourDataStride() ? p.GetColourDataStride() : col_bytes;
    for (uint64_t k = 0; k < p.GetCount(); ++k) {
        if (vert_out && v)
            std::memcpy(static_cast<uint8_t*>(vert_out) + k * vert_bytes, v + k * vs, vert_bytes);
        if (col_out && c)
            std::memcpy(static_cast<uint8_t*>(col_out) + k * col_bytes, c + k * cs, col_bytes);
    }
    return 0;
}

void ref_mmpld_close(void* session) {
    delete static_cast<Session*>(session);
}

} // extern "C"
