// Minimal stand-in for MegaMol's data-call base classes (plugins/mmstd/include/mmstd/data/
// AbstractGetDataCall.h:54,73,89-105 and AbstractGetData3DCall.h:18,31,40,49,126-129), oracle build
// only: frame ID (and whether it is forced), frame count, data hash, the unlocker of the data the call
// points to, and the object-space bounding/clip boxes.
#pragma once

#include <memory>

#include "mmcore/Call.h"
#include "vislib/math/Cuboid.h"

namespace megamol::core {

class BoundingBoxes {
public:
    const vislib::math::Cuboid<float>& ObjectSpaceBBox() const {
        return osbb_;
    }
    const vislib::math::Cuboid<float>& ObjectSpaceClipBox() const {
        return oscb_;
    }
    void SetObjectSpaceBBox(const vislib::math::Cuboid<float>& b) {
        osbb_ = b;
    }
    void SetObjectSpaceBBox(float l, float b, float k, float r, float t, float f) {
        osbb_.Set(l, b, k, r, t, f);
    }
    void SetObjectSpaceClipBox(const vislib::math::Cuboid<float>& b) {
        oscb_ = b;
    }
    void SetObjectSpaceClipBox(float l, float b, float k, float r, float t, float f) {
        oscb_.Set(l, b, k, r, t, f);
    }
    void MakeScaledWorld(float) {}
    void Clear() {
        osbb_ = vislib::math::Cuboid<float>();
        oscb_ = vislib::math::Cuboid<float>();
    }

private:
    vislib::math::Cuboid<float> osbb_, oscb_;
};

class AbstractGetData3DCall : public Call {
public:
    // AbstractGetDataCall::Unlocker: releases the source's lock on the data the call points to
    class Unlocker {
    public:
        virtual ~Unlocker() = default;
        virtual void Unlock() = 0;
    };

    ~AbstractGetData3DCall() override {
        Unlock();
    }

    void SetFrameID(unsigned int id, bool force = false) {
        frame_ = id;
        forced_ = force;
    }
    unsigned int FrameID() const {
        return frame_;
    }
    bool IsFrameForced() const {
        return forced_;
    }
    void SetFrameCount(unsigned int n) {
        frames_ = n;
    }
    unsigned int FrameCount() const {
        return frames_;
    }
    void SetDataHash(size_t h) {
        hash_ = h;
    }
    size_t DataHash() const {
        return hash_;
    }
    void SetUnlocker(Unlocker* u, bool unlockOld = true) {
        if (unlockOld)
            Unlock();
        unlocker_.reset(u);
    }
    void Unlock() {
        if (unlocker_) {
            unlocker_->Unlock();
            unlocker_.reset();
        }
    }

    BoundingBoxes& AccessBoundingBoxes() {
        return bboxs_;
    }
    const BoundingBoxes& GetBoundingBoxes() const {
        return bboxs_;
    }

private:
    std::unique_ptr<Unlocker> unlocker_;
    bool forced_ = false;
    unsigned int frame_ = 0, frames_ = 1;
    size_t hash_ = 0;
    BoundingBoxes bboxs_;
};

} // namespace megamol::core
