// Minimal stand-in for MegaMol's core::CallerSlot (core/include/mmcore/CallerSlot.h:58-60,70-108),
// oracle build only. CallAs<T>() returns the call the harness connected, cast to T.
#pragma once

#include "mmcore/Module.h"

namespace megamol::core {

class CallerSlot : public AbstractSlot {
public:
    CallerSlot(const char* name, const char* desc) : AbstractSlot(name, desc) {}

    template<class D>
    void SetCompatibleCall() {}

    void ConnectCall(Call* c) {
        call_ = c;
    }

    template<class T>
    T* CallAs() {
        return dynamic_cast<T*>(call_);
    }

private:
    Call* call_ = nullptr;
};

} // namespace megamol::core
