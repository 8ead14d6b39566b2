// Minimal stand-in for MegaMol's core::view::AnimDataModule (plugins/mmstd/include/mmstd/data/
// AnimDataModule.h, plugins/mmstd/src/data/AnimDataModule.cpp:108-186), oracle build only.
// The reference keeps a cache of frames that a loader thread fills around the last requested index;
// requestLockedFrame(idx, true) waits until frame idx is in the cache (an index past the end is clamped
// to the last frame). This stand-in keeps one frame and loads the requested index synchronously through
// the module's loadFrame(), which gives the same frame contents without the thread.
#pragma once

#include <memory>

#include "mmcore/Module.h"

namespace megamol::core::view {

class AnimDataModule : public Module {
public:
    ~AnimDataModule() override = default;

    unsigned int FrameCount() const {
        return frameCnt_;
    }

protected:
    class Frame {
    public:
        explicit Frame(AnimDataModule& owner) : frame(0), owner_(owner) {}
        virtual ~Frame() = default;
        unsigned int FrameNumber() const {
            return frame;
        }
        bool IsLocked() const {
            return locked_;
        }
        void Unlock() {
            locked_ = false;
        }

    protected:
        unsigned int frame;

    private:
        friend class AnimDataModule;
        AnimDataModule& owner_;
        bool locked_ = false;
    };

    AnimDataModule() = default;

    unsigned int CacheSize() const {
        return cacheSize_;
    }

    virtual Frame* constructFrame() const = 0;
    virtual void loadFrame(Frame* frame, unsigned int idx) = 0;

    void initFrameCache(unsigned int cacheSize) {
        cacheSize_ = cacheSize;
        cache_.reset(constructFrame());
    }

    Frame* requestLockedFrame(unsigned int idx, bool forceIdx = false) {
        if (!cache_)
            return nullptr;
        if (idx >= frameCnt_)
            idx = frameCnt_ - 1;  // AnimDataModule.cpp:168-173
        (void) forceIdx;
        loadFrame(cache_.get(), idx);
        cache_->locked_ = true;
        return cache_.get();
    }

    void resetFrameCache() {
        cache_.reset();
    }

    void setFrameCount(unsigned int cnt) {
        frameCnt_ = cnt;
    }

private:
    unsigned int frameCnt_ = 0, cacheSize_ = 0;
    std::unique_ptr<Frame> cache_;
};

} // namespace megamol::core::view
