// Minimal stand-in for MegaMol's core::Module and slot registry (core/include/mmcore/Module.h,
// core/src/Module.cpp:44,97), for the oracle build only. A module registers its slots with
// MakeSlotAvailable(); the harness finds them again by name, the way a MegaMol graph does.
#pragma once

#include <map>
#include <string>

#include "mmcore/Call.h"

namespace megamol::core {

class Module;

class AbstractSlot {
public:
    AbstractSlot(const char* name, const char* desc) : name_(name), desc_(desc) {}
    virtual ~AbstractSlot() = default;
    const std::string& Name() const {
        return name_;
    }
    Module* Owner() const {
        return owner_;
    }
    void SetOwner(Module* m) {
        owner_ = m;
    }

private:
    std::string name_, desc_;
    Module* owner_ = nullptr;
};

class Module {
public:
    virtual ~Module() = default;

    void MakeSlotAvailable(AbstractSlot* slot) {
        slot->SetOwner(this);
        slots_[slot->Name()] = slot;
    }

    AbstractSlot* FindSlot(const std::string& name) const {
        auto it = slots_.find(name);
        return it == slots_.end() ? nullptr : it->second;
    }

    bool Create() {
        return create();
    }

    void Release() {
        if (!released_) {
            released_ = true;
            release();
        }
    }

protected:
    virtual bool create() = 0;
    virtual void release() = 0;

private:
    std::map<std::string, AbstractSlot*> slots_;
    bool released_ = false;
};

} // namespace megamol::core
