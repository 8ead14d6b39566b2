// Minimal stand-ins for MegaMol's parameter slots and parameter types
// (core/include/mmcore/param/ParamSlot.h:28, AbstractParamSlot.h:33,80), oracle build only.
// A parameter is dirty after construction and after every SetValue(), until ResetDirty().
// SetUpdateCallback() stores the module's update callback (ParamSlot.h SetUpdateCallback); the harness
// runs it with Update() after it changed the value, as the core does when a parameter changes.
#pragma once

#include <functional>
#include <map>
#include <memory>
#include <string>

#include "mmcore/Module.h"

namespace megamol::core::param {

class AbstractParam {
public:
    virtual ~AbstractParam() = default;
    bool dirty = true;
};

class ParamSlot : public AbstractSlot {
public:
    ParamSlot(const char* name, const char* desc) : AbstractSlot(name, desc) {}

    template<class P>
    ParamSlot& operator<<(P* p) {
        param_.reset(p);
        return *this;
    }

    void SetParameter(AbstractParam* p) {
        param_.reset(p);
    }

    template<class T>
    T* Param() const {
        return dynamic_cast<T*>(param_.get());
    }

    bool IsDirty() const {
        return param_ && param_->dirty;
    }

    void ResetDirty() {
        if (param_)
            param_->dirty = false;
    }

    template<class C>
    void SetUpdateCallback(bool (C::*func)(ParamSlot&)) {
        update_ = [func](Module* m, ParamSlot& s) { return (static_cast<C*>(m)->*func)(s); };
    }

    bool Update() {
        return update_ && Owner() ? update_(Owner(), *this) : true;
    }

private:
    std::unique_ptr<AbstractParam> param_;
    std::function<bool(Module*, ParamSlot&)> update_;
};

template<class T>
class ValueParam : public AbstractParam {
public:
    explicit ValueParam(T v) : value_(v) {}
    T Value() const {
        return value_;
    }
    void SetValue(T v, bool setDirty = true) {
        if (v != value_ && setDirty)
            dirty = true;
        value_ = v;
    }

private:
    T value_;
};

class IntParam : public ValueParam<int> {
public:
    explicit IntParam(int v, int = 0, int = 0) : ValueParam<int>(v) {}
};

class BoolParam : public ValueParam<bool> {
public:
    explicit BoolParam(bool v) : ValueParam<bool>(v) {}
};

class FloatParam : public ValueParam<float> {
public:
    explicit FloatParam(float v, float = 0.0f, float = 0.0f) : ValueParam<float>(v) {}
};

class EnumParam : public ValueParam<int> {
public:
    explicit EnumParam(int v) : ValueParam<int>(v) {}
    EnumParam* SetTypePair(int v, const char* name) {
        names_[v] = name;
        return this;
    }

private:
    std::map<int, std::string> names_;
};

} // namespace megamol::core::param
