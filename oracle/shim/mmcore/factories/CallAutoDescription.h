// Minimal stand-in for MegaMol's call description template
// (core/include/mmcore/factories/CallAutoDescription.h), oracle build only.
#pragma once

namespace megamol::core::factories {

template<class C>
class CallAutoDescription {
public:
    static const char* ClassName() {
        return C::ClassName();
    }
};

} // namespace megamol::core::factories
