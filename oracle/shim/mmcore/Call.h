// Minimal stand-in for MegaMol's core::Call (core/include/mmcore/Call.h:35-149), written for the
// oracle build only: it lets the reference module's unmodified source compile and run headless.
// Calling a call with a function index runs a hook the test harness installs; by default it
// returns true, which is what a connected upstream module reports when its data is ready.
#pragma once

#include <functional>

namespace megamol::core {

class Call {
public:
    virtual ~Call() = default;

    bool operator()(unsigned int func = 0) {
        return hook_ ? hook_(*this, func) : true;
    }

    void SetHook(std::function<bool(Call&, unsigned int)> h) {
        hook_ = std::move(h);
    }

private:
    std::function<bool(Call&, unsigned int)> hook_;
};

} // namespace megamol::core
