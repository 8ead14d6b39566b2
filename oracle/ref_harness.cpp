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
#include "datatools/table/TableDataCall.h"
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
    // any other colour data (used when icol is null and has_col is set): type, data, stride (0 = packed) and
    // the global colour, set before the colour data as MMPLDDataSource does (MMPLDDataSource.cpp:164-196)
    int has_col;
    int col_type;         // SimpleSphericalParticles::ColourDataType
    const void* col;
    uint32_t col_stride;
    uint8_t global_colour[4];
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

struct ref_p2d_vgrid {
    uint64_t count;       // entries of the outParticles list / rows of the outInfo table
    uint64_t info_cols;
    float global_radius;  // outParticles' global radius
    float col_min[7], col_max[7];
};

} // extern "C"

namespace {

// One configured module with its input call; both live until the session ends, as in a MegaMol graph.
struct Session {
    std::unique_ptr<datatools::ParticlesToDensity> mod;
    geocalls::MultiParticleDataCall mpdc;
    ~Session() {
        if (mod)
            mod->Release();
    }
};

void setup(Session& S, const ref_p2d_list* lists, int n_lists, const float bbox[6], const ref_p2d_params* prm) {
    S.mod = std::make_unique<datatools::ParticlesToDensity>();
    auto& mod = S.mod;
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

    auto& mpdc = S.mpdc;
    mpdc.SetParticleListCount(static_cast<unsigned int>(n_lists));
    for (int i = 0; i < n_lists; ++i) {
        auto& p = mpdc.AccessParticles(static_cast<unsigned int>(i));
        p.SetCount(lists[i].count);
        p.SetGlobalRadius(lists[i].global_radius);
        p.SetVertexData(static_cast<geocalls::SimpleSphericalParticles::VertexDataType>(lists[i].vert_type),
            lists[i].vert, lists[i].vert_stride);
        if (lists[i].icol != nullptr) {
            p.SetColourData(geocalls::SimpleSphericalParticles::COLDATA_FLOAT_I, lists[i].icol);
        } else if (lists[i].has_col) {
            const uint8_t* g = lists[i].global_colour;
            p.SetGlobalColour(g[0], g[1], g[2], g[3]);
            p.SetColourData(static_cast<geocalls::SimpleSphericalParticles::ColourDataType>(lists[i].col_type),
                lists[i].col, lists[i].col_stride);
        }
        if (lists[i].dir != nullptr)
            p.SetDirData(geocalls::SimpleSphericalParticles::DIRDATA_FLOAT_XYZ, lists[i].dir);
    }
    mpdc.AccessBoundingBoxes().SetObjectSpaceBBox(bbox[0], bbox[1], bbox[2], bbox[3], bbox[4], bbox[5]);
    mpdc.AccessBoundingBoxes().SetObjectSpaceClipBox(bbox[0], bbox[1], bbox[2], bbox[3], bbox[4], bbox[5]);
    auto* in = dynamic_cast<core::CallerSlot*>(mod->FindSlot("inData"));
    in->ConnectCall(&mpdc);
}

// GET_DATA on "outData" (ParticlesToDensity.cpp:94-112,210-304); returns 0, 1 (module failure) or 2 (out_cap
// too small).
int get_volume(Session& S, float* out, uint64_t out_cap, ref_p2d_result* res) {
    auto* outSlot = dynamic_cast<core::CalleeSlot*>(S.mod->FindSlot("outData"));
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
    return 0;
}

} // namespace

extern "C" {

// Runs the reference module once. `out` receives the volume when `out_cap` floats suffice; the
// call returns 0 on success, 1 if the module reported failure, 2 if `out_cap` was too small (the
// result then holds the required size in needed_floats).
int ref_p2d_run(const ref_p2d_list* lists, int n_lists, const float bbox[6], const ref_p2d_params* prm,
    float* out, uint64_t out_cap, ref_p2d_result* res) {
    Session S;
    setup(S, lists, n_lists, bbox, prm);
    return get_volume(S, out, out_cap, res);
}

// The vector aggregator's two extra outputs after the volume: GET_DATA on "outParticles" (the compacted
// grid as a particle list: positions, directions, colours; ParticlesToDensity.cpp:306-323) and on "outInfo"
// (the 7-column table; :325-380). Entries are copied when `cap` suffices (return 3 otherwise, with the
// count in vg).
int ref_p2d_run_vector(const ref_p2d_list* lists, int n_lists, const float bbox[6], const ref_p2d_params* prm,
    float* out, uint64_t out_cap, ref_p2d_result* res, float* pos, float* dir, float* col, float* info,
    uint64_t cap, ref_p2d_vgrid* vg) {
    Session S;
    setup(S, lists, n_lists, bbox, prm);
    const int rc = get_volume(S, out, out_cap, res);
    if (rc != 0)
        return rc;
    std::memset(vg, 0, sizeof(*vg));
    geocalls::MultiParticleDataCall grid;
    grid.SetFrameID(0);
    auto* ps = dynamic_cast<core::CalleeSlot*>(S.mod->FindSlot("outParticles"));
    if (!ps->InCall(geocalls::MultiParticleDataCall::ClassName(), geocalls::MultiParticleDataCall::FunctionName(0),
            grid))
        return 1;
    datatools::table::TableDataCall table;
    auto* ts = dynamic_cast<core::CalleeSlot*>(S.mod->FindSlot("outInfo"));
    if (!ts->InCall(datatools::table::TableDataCall::ClassName(), datatools::table::TableDataCall::FunctionName(0),
            table))
        return 1;
    const auto& p = grid.AccessParticles(0);
    vg->count = p.GetCount();
    vg->global_radius = p.GetGlobalRadius();
    vg->info_cols = table.GetColumnsCount();
    for (size_t c = 0; c < 7 && c < table.GetColumnsCount(); ++c) {
        vg->col_min[c] = table.GetColumnsInfos()[c].MinimumValue();
        vg->col_max[c] = table.GetColumnsInfos()[c].MaximumValue();
    }
    if (table.GetRowsCount() != vg->count)
        return 1;
    if (vg->count > cap)
        return 3;
    if (vg->count > 0) {
        std::memcpy(pos, p.GetVertexData(), vg->count * 3 * sizeof(float));
        std::memcpy(dir, p.GetDirData(), vg->count * 3 * sizeof(float));
        std::memcpy(col, p.GetColourData(), vg->count * sizeof(float));
        std::memcpy(info, table.GetData(), vg->count * table.GetColumnsCount() * sizeof(float));
    }
    return 0;
}

} // extern "C"
