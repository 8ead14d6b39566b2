/*
 * ParticlesToDensityGPU — MegaMol module that drops in for datatools::ParticlesToDensity
 * (plugins/datatools/src/ParticlesToDensity.h:32-145) and computes the volume with libp2v on a GB300.
 *
 * Slots and parameters keep the reference module's names and defaults ("aggregator", "sizex/y/z",
 * "cyclX/Y/Z", "normalize", "sigma", "forSurfaceReconstruction"; callee "outData" answering all six
 * VolumetricDataCall functions; callees "outParticles" (MultiParticleDataCall) and "outInfo"
 * (TableDataCall) carrying the vector aggregator's grid; caller "inData" for a MultiParticleDataCall).
 * Added: "outAO", a
 * MultiParticleDataCall whose lists carry the input particles with COLDATA_FLOAT_I = ambient occlusion,
 * and the AO / kernel parameters of p2v_params.
 */
#pragma once

#include <array>
#include <string>
#include <vector>

#include "datatools/table/TableDataCall.h"
#include "geometry_calls/MultiParticleDataCall.h"
#include "geometry_calls/VolumetricDataCall.h"
#include "mmcore/CalleeSlot.h"
#include "mmcore/CallerSlot.h"
#include "mmcore/Module.h"
#include "mmcore/param/ParamSlot.h"

#include "p2v.h"

namespace megamol::p2v_gb300 {

class ParticlesToDensityGPU : public core::Module {
public:
    static const char* ClassName() {
        return "ParticlesToDensityGPU";
    }
    static const char* Description() {
        return "Computes a density volume and per-particle ambient occlusion from particles on the GPU";
    }
    static bool IsAvailable() {
        return true;
    }

    ParticlesToDensityGPU();
    ~ParticlesToDensityGPU() override;

protected:
    bool create() override;
    void release() override;

private:
    bool getDataCallback(core::Call& c);
    bool getExtentCallback(core::Call& c);
    bool dummyCallback(core::Call& c);
    bool getAODataCallback(core::Call& c);
    bool getAOExtentCallback(core::Call& c);

    bool pullFrame(geocalls::MultiParticleDataCall* in, unsigned int frame);
    bool fetchVectorGrid();
    bool recompute(geocalls::MultiParticleDataCall* in);
    bool anythingDirty() const;
    void resetDirty();

    // ParticlesToDensity's parameters (ParticlesToDensity.cpp:59-152)
    core::param::ParamSlot aggregatorSlot, xResSlot, yResSlot, zResSlot, cyclXSlot, cyclYSlot, cyclZSlot,
        normalizeSlot, sigmaSlot, surfaceSlot;
    // additions of this module
    core::param::ParamSlot kernelSlot, massNormSlot, aoModeSlot, aoConesSlot, aoStepsSlot, aoLevelsSlot, aoApexSlot,
        aoOffsetSlot, aoStrengthSlot, aoConeLengthSlot;
    // the AO source: the volume the cone march samples, its scale, the normals, the learned AO's network file
    core::param::ParamSlot aoVolumeSlot, aoVolumeScaleSlot, aoNormalsSlot, aoModelSlot;
    // MDAO (SphereRenderer.cpp:193-214): "ambient occlusion::volumeSize", "ambient occlusion::highPrecisionTexture"
    core::param::ParamSlot mdaoVolSizeSlot, mdaoHighPrecisionSlot;
    // AOSphereRenderer (AOSphereRenderer.cpp:57-124): "vol::sizex/y/z", "vol::gen", "ao::stepLen", "vol::genFac",
    // "ao::evalFac", "ao::clipData"
    core::param::ParamSlot aosSizeXSlot, aosSizeYSlot, aosSizeZSlot, aosGenSlot, aosStepLenSlot, aosGenFacSlot,
        aosEvalFacSlot, aosClipDataSlot;
    core::CallerSlot getClipPlaneSlot;  // "getclipplane" (AOSphereRenderer.cpp:54,273-287)
    std::string loadedModel;

    core::CalleeSlot outDataSlot;
    core::CalleeSlot outParticlesSlot;
    core::CalleeSlot outInfoSlot;
    core::CalleeSlot outAOSlot;
    core::CallerSlot inDataSlot;

    p2v_ctx* ctx = nullptr;
    std::vector<float> volume;
    std::vector<std::vector<float>> ao;
    geocalls::VolumetricDataCall::Metadata metadata;
    std::array<float, 3> sliceDists{};
    double minValues[3] = {0.0, 0.0, 0.0}, maxValues[3] = {0.0, 0.0, 0.0};
    // the vector aggregator's grid (ParticlesToDensity.h:115-126): positions, directions, colours, info rows
    std::vector<float> grid, directions, colors, infoData;
    float gridRadius = 0.0f;
    std::array<datatools::table::TableDataCall::ColumnInfo, 7> info;
    bool hasData = false;
    unsigned int time = static_cast<unsigned int>(-1);
    size_t inDataHash = static_cast<size_t>(-1);
    size_t dataHash = 0;
};

} // namespace megamol::p2v_gb300
