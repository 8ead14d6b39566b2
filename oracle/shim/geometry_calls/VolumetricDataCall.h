// Minimal stand-in for MegaMol's VolumetricDataCall (plugins/geometry_calls/include/geometry_calls/
// VolumetricDataCall.h:21-326, src/VolumetricDataCall.cpp:80-110), oracle build only. The metadata
// struct is the reference's own VolumetricMetadata_t (VolumetricDataCallTypes.h:32-134).
#pragma once

#include "geometry_calls/VolumetricDataCallTypes.h"
#include "mmcore/factories/CallAutoDescription.h"
#include "mmstd/data/AbstractGetData3DCall.h"

namespace megamol::geocalls {

class VolumetricDataCall : public core::AbstractGetData3DCall {
public:
    typedef VolumetricMetadata_t Metadata;
    typedef ScalarType_t ScalarType;
    typedef GridType_t GridType;

    static const unsigned int IDX_GET_EXTENTS = 0;
    static const unsigned int IDX_GET_DATA = 1;
    static const unsigned int IDX_GET_METADATA = 2;
    static const unsigned int IDX_START_ASYNC = 3;
    static const unsigned int IDX_STOP_ASYNC = 4;
    static const unsigned int IDX_TRY_GET_DATA = 5;

    static const char* ClassName() {
        return "VolumetricDataCall";
    }
    static const char* FunctionName(unsigned int idx) {
        static const char* names[] = {
            "GetExtents", "GetData", "GetMetadata", "StartAsync", "StopAsync", "TryGetData"};
        return idx < 6 ? names[idx] : "";
    }

    void SetData(void* d) {
        data_ = d;
    }
    void* GetData() const {
        return data_;
    }
    void SetMetadata(const Metadata* m) {
        meta_ = m;
    }
    const Metadata* GetMetadata() const {
        return meta_;
    }
    // VolumetricDataCall.h:245-247 and VolumetricDataCall.cpp:201-211
    size_t GetVoxelSize() const {
        return meta_ ? meta_->ScalarLength * meta_->Components : 0;
    }
    size_t GetVoxelsPerFrame() const {
        return meta_ ? meta_->Resolution[0] * meta_->Resolution[1] * meta_->Resolution[2] : 0;
    }

private:
    void* data_ = nullptr;
    const Metadata* meta_ = nullptr;
};

typedef core::factories::CallAutoDescription<VolumetricDataCall> VolumetricDataCallDescription;

} // namespace megamol::geocalls
