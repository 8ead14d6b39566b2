// Minimal stand-in for MegaMol's core::view::CallClipPlane (plugins/mmstd/include/mmstd/renderer/CallClipPlane.h:
// 20-148), oracle and adapter builds only: a call carrying one clipping plane and its colour.
#pragma once

#include "mmcore/Call.h"
#include "mmcore/factories/CallAutoDescription.h"
#include "vislib/math/Plane.h"

namespace megamol::core::view {

class CallClipPlane : public Call {
public:
    static const char* ClassName() {
        return "CallClipPlane";
    }
    static unsigned int FunctionCount() {
        return 1;
    }
    static const char* FunctionName(unsigned int) {
        return "GetPlane";
    }
    const vislib::math::Plane<float>& GetPlane() const {
        return plane_;
    }
    const unsigned char* GetColour() const {
        return colour_;
    }
    void SetPlane(const vislib::math::Plane<float>& p) {
        plane_ = p;
    }

private:
    vislib::math::Plane<float> plane_;
    unsigned char colour_[4] = {192, 192, 192, 255};
};

typedef factories::CallAutoDescription<CallClipPlane> CallClipPlaneDescription;

} // namespace megamol::core::view
