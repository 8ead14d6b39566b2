// Stand-in for MegaMol's volume metadata (plugins/geometry_calls/include/geometry_calls/VolumetricDataCallTypes.h:
// 16-134), for building the MegaMol adapter where the MegaMol tree is absent. The enumerators and the metadata
// fields carry the reference's names and meanings.
#pragma once

#include <cstddef>

namespace megamol::geocalls {

enum GridType_t { NONE, CARTESIAN, RECTILINEAR, TETRAHEDRAL };
enum ScalarType_t { UNKNOWN, SIGNED_INTEGER, UNSIGNED_INTEGER, FLOATING_POINT, BITS };
enum MemoryLocation { VRAM, RAM };

struct VolumetricMetadata_t {
    GridType_t GridType = NONE;
    size_t Resolution[3] = {0, 0, 0};
    ScalarType_t ScalarType = UNKNOWN;
    size_t ScalarLength = 0;
    size_t Components = 0;
    float* SliceDists[3] = {nullptr, nullptr, nullptr};
    float Origin[3] = {0, 0, 0};
    bool IsUniform[3] = {true, true, true};
    size_t NumberOfFrames = 0;
    float Extents[3] = {0, 0, 0};
    double* MinValues = nullptr;
    double* MaxValues = nullptr;
    MemoryLocation MemLoc = RAM;
};

}  // namespace megamol::geocalls
