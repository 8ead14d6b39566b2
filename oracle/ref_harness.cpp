// Test-only harness that drives MegaMol's own, unmodified datatools::ParticlesToDensity module
// (plugins/datatools/src/ParticlesToDensity.cpp) headless, through the same slots a MegaMol graph
// uses: parameters are set by slot name, the MultiParticleDataCall is connected to "inData", and the
// VolumetricDataCall GET_DATA callback of "outData" is invoked (ParticlesToDensity.cpp:94-112,210-304).
//
// This file is ORACLE infrastructure: it is built by oracle/Makefile into oracle/_ref/ (never
// committed) and is called only by tests and by bench.py's CPU-baseline leg.
#include <chrono>
#include <cstdint>
#include <cstring>
#include <memory>

#include "ParticlesToDensity.h"
#include "mmcore/param/BoolParam.h"
#include "mmcore/param/EnumParam.h"
#include "mmcore/param/FloatParam.h"
#include "mmcore/param/IntParam.h"

using namespace megamol;

namespace {

template<class P, class V>
void set_param(core::Module& m, const char* name, V v) {
    auto* slot = dynamic_cast<core::param::ParamSlot*>(m.FindSlot(name));
    slot->Param<P>()->SetValue(v);
}

} // namespace

extern "C" {

// Describes one particle list, mirroring SimpleSphericalParticles' vertex/colour/direction setters
// (SimpleSphericalParticles.h:475-483,582-589).
struct ref_p2d_list {
    int vert_type;        // SimpleSphericalParticles::VertexDataType
    const void* vert;     // vertex data
    uint32_t vert_stride; // bytes, 0 = packed
    float global_radius;
    uint64_t count;
    const float* icol;    // COLDATA_FLOAT_I (aggregator 1) or nullptr
    const float* dir;     // DIRDATA_FLOAT_XYZ (aggregator 2) or nullptr
};

struct ref_p2d_params {
    int aggregator, sizex, sizey, sizez, cyclX, cyclY, cyclZ, normalize, surface;
    float sigma;
};

struct ref_p2d_result {
    uint64_t resolution[3];
    uint64_t components;
    float slice_dists[3];
    float origin[3];
    float extents[3];
    double min_value, max_value;
    double millis; // wall time of the GET_DATA call (createVolumeCPU + metadata)
    uint64_t needed_floats;
};

// Runs the reference module once. `out` receives the volume when `out_cap` floats suffice; the
// call returns 0 on success, 1 if the module reported failure, 2 if `out_cap` was too small (the
// result then holds the required size in needed_floats).
int ref_p2d_run(const ref_p2d_list* lists, int n_lists, const float bbox[6], const ref_p2d_params* prm,
    float* out, uint64_t out_cap, ref_p2d_result* res) {
    auto mod = std::make_unique<datatools::ParticlesToDensity>();
    mod->Create();
    set_param<core::param::EnumParam>(*mod, "aggregator", prm->aggregator);
    set_param<core::param::IntParam>(*mod, "sizex", prm->sizex);
    set_param<core::param::IntParam>(*mod, "sizey", prm->sizey);
    set_param<core::param::IntParam>(*mod, "sizez", prm->sizez);
    set_param<core::param::BoolParam>(*mod, "cyclX", prm->cyclX != 0);
    set_param<core::param::BoolParam>(*mod, "cyclY", prm->cyclY != 0);
    set_param<core::param::BoolParam>(*mod, "cyclZ", prm->cyclZ != 0);
    set_param<core::param::BoolParam>(*mod, "normalize", prm->normalize != 0);
    set_param<core::param::FloatParam>(*mod, "sigma", prm->sigma);
    set_param<core::param::BoolParam>(*mod, "forSurfaceReconstruction", prm->surface != 0);

    geocalls::MultiParticleDataCall mpdc;
    mpdc.SetParticleListCount(static_cast<unsigned int>(n_lists));
    for (int i = 0; i < n_lists; ++i) {
        auto& p = mpdc.AccessParticles(static_cast<unsigned int>(i));
        p.SetCount(lists[i].count);
        p.SetGlobalRadius(lists[i].global_radius);
        p.SetVertexData(static_cast<geocalls::SimpleSphericalParticles::VertexDataType>(lists[i].vert_type),
            lists[i].vert, lists[i].vert_stride);
        if (lists[i].icol != nullptr)
            p.SetColourData(geocalls::SimpleSphericalParticles::COLDATA_FLOAT_I, lists[i].icol);
        if (lists[i].dir != nullptr)
            p.SetDirData(geocalls::SimpleSphericalParticles::DIRDATA_FLOAT_XYZ, lists[i].dir);
    }
    mpdc.AccessBoundingBoxes().SetObjectSpaceBBox(bbox[0], bbox[1], bbox[2], bbox[3], bbox[4], bbox[5]);
    mpdc.AccessBoundingBoxes().SetObjectSpaceClipBox(bbox[0], bbox[1], bbox[2], bbox[3], bbox[4], bbox[5]);

    auto* in = dynamic_cast<core::CallerSlot*>(mod->FindSlot("inData"));
    in->ConnectCall(&mpdc);
    auto* outSlot = dynamic_cast<core::CalleeSlot*>(mod->FindSlot("outData"));

    geocalls::VolumetricDataCall vdc;
    vdc.SetFrameID(0);
    auto t0 = std::chrono::steady_clock::now();
    bool ok = outSlot->InCall(geocalls::VolumetricDataCall::ClassName(),
        geocalls::VolumetricDataCall::FunctionName(geocalls::VolumetricDataCall::IDX_GET_DATA), vdc);
    auto t1 = std::chrono::steady_clock::now();
    if (!ok)
        return 1;

    const auto* md = vdc.GetMetadata();
    std::memset(res, 0, sizeof(*res));
    for (int a = 0; a < 3; ++a) {
        res->resolution[a] = md->Resolution[a];
        res->slice_dists[a] = md->SliceDists[a][0];
        res->origin[a] = md->Origin[a];
        res->extents[a] = md->Extents[a];
    }
    res->components = md->Components;
    res->min_value = md->MinValues[0];
    res->max_value = md->MaxValues[0];
    res->millis = std::chrono::duration<double, std::milli>(t1 - t0).count();
    res->needed_floats = md->Resolution[0] * md->Resolution[1] * md->Resolution[2] * md->Components;
    if (res->needed_floats > out_cap)
        return 2;
    std::memcpy(out, vdc.GetData(), res->needed_floats * sizeof(float));
    mod->Release();
    return 0;
}

} // extern "C"
