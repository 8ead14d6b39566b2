// Minimal stand-in for MegaMol's core::CalleeSlot (core/include/mmcore/CalleeSlot.h:57,105-137),
// oracle build only. SetCallback() stores member-function callbacks keyed by (call class, function
// name); InCall() dispatches to them on the owning module, as CalleeSlot::InCall does.
#pragma once

#include <functional>
#include <map>
#include <string>
#include <utility>

#include "mmcore/Module.h"

namespace megamol::core {

class CalleeSlot : public AbstractSlot {
public:
    CalleeSlot(const char* name, const char* desc) : AbstractSlot(name, desc) {}

    template<class C>
    void SetCallback(const char* callName, const char* funcName, bool (C::*func)(Call&)) {
        cbs_[{callName, funcName}] = [func](Module* m, Call& c) { return (static_cast<C*>(m)->*func)(c); };
    }

    bool InCall(const std::string& callName, const std::string& funcName, Call& c) {
        auto it = cbs_.find({callName, funcName});
        if (it == cbs_.end() || Owner() == nullptr)
            return false;
        return it->second(Owner(), c);
    }

private:
    std::map<std::pair<std::string, std::string>, std::function<bool(Module*, Call&)>> cbs_;
};

} // namespace megamol::core
