// Test-only harness that drives MegaMol's own, unmodified volume::DatRawWriter
// (plugins/volume/src/DatRawWriter.cpp) headless: its parameters are set by slot name, a
// VolumetricDataCall holding the given volume and metadata is connected to its "data" slot, and its
// run() writes <prefix><frame:04>.dat / .raw (DatRawWriter.cpp:58-186).
//
// This file is ORACLE infrastructure: oracle/Makefile builds it into oracle/_ref/ (never committed);
// only tests call it.
#include <cstdint>
#include <cstring>

#include "DatRawWriter.h"
#include "mmcore/param/FilePathParam.h"
#include "mmcore/param/IntParam.h"

using namespace megamol;

extern "C" {

// scalar_type / grid_type: the reference's ScalarType_t / GridType_t values (VolumetricDataCallTypes.h:16-19).
int ref_datraw_write(const char* prefix, unsigned int frame, unsigned int frame_count, const uint64_t res[3],
    uint64_t components, int scalar_type, uint64_t scalar_length, int grid_type, const float slice[3],
    const float origin[3], const void* data) {
    volume::DatRawWriter w;
    w.Create();
    dynamic_cast<core::param::ParamSlot*>(w.FindSlot("filepathPrefix"))
        ->Param<core::param::FilePathParam>()
        ->SetValue(std::filesystem::path(prefix));
    dynamic_cast<core::param::ParamSlot*>(w.FindSlot("frameID"))
        ->Param<core::param::IntParam>()
        ->SetValue(static_cast<int>(frame));

    geocalls::VolumetricDataCall::Metadata md{};
    float sd[3] = {slice[0], slice[1], slice[2]};
    md.Components = components;
    md.ScalarType = static_cast<geocalls::ScalarType_t>(scalar_type);
    md.ScalarLength = scalar_length;
    md.GridType = static_cast<geocalls::GridType_t>(grid_type);
    for (int a = 0; a < 3; ++a) {
        md.Resolution[a] = res[a];
        md.SliceDists[a] = &sd[a];
        md.Origin[a] = origin[a];
        md.IsUniform[a] = true;
    }
    md.NumberOfFrames = frame_count;
    geocalls::VolumetricDataCall vdc;
    vdc.SetData(const_cast<void*>(data));
    vdc.SetMetadata(&md);
    vdc.SetFrameCount(frame_count);
    dynamic_cast<core::CallerSlot*>(w.FindSlot("data"))->ConnectCall(&vdc);
    const bool ok = w.Run();
    // the metadata is stack memory: detach it before the call goes out of scope
    vdc.SetMetadata(nullptr);
    return ok ? 0 : 1;
}

} // extern "C"
