// Minimal stand-in for MegaMol's MultiParticleDataCall (plugins/geometry_calls/include/
// geometry_calls/MultiParticleDataCall.h:22-56, AbstractParticleDataCall.h:23,61-83), oracle build
// only. The particle lists are the reference's own SimpleSphericalParticles, so every accessor the
// module reads through is the reference's code.
#pragma once

#include <vector>

#include "geometry_calls/SimpleSphericalParticles.h"
#include "mmcore/factories/CallAutoDescription.h"
#include "mmstd/data/AbstractGetData3DCall.h"

namespace megamol::geocalls {

class MultiParticleDataCall : public core::AbstractGetData3DCall {
public:
    typedef SimpleSphericalParticles Particles;

    static const char* ClassName() {
        return "MultiParticleDataCall";
    }
    static const char* FunctionName(unsigned int idx) {
        return idx == 0 ? "GetData" : "GetExtent";
    }

    void SetParticleListCount(unsigned int n) {
        lists_.resize(n);
    }
    unsigned int GetParticleListCount() const {
        return static_cast<unsigned int>(lists_.size());
    }
    Particles& AccessParticles(unsigned int i) {
        return lists_[i];
    }
    const Particles& AccessParticles(unsigned int i) const {
        return lists_[i];
    }

private:
    std::vector<Particles> lists_;
};

typedef core::factories::CallAutoDescription<MultiParticleDataCall> MultiParticleDataCallDescription;

} // namespace megamol::geocalls
