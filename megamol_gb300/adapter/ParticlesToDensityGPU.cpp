/*
 * ParticlesToDensityGPU — see the header. The callback structure follows
 * ParticlesToDensity::getDataCallback / getExtentCallback (ParticlesToDensity.cpp:163-304); the volume and
 * AO are computed by p2v_run_frame.
 */
#include "ParticlesToDensityGPU.h"

#include <algorithm>
#include <limits>

#include "mmcore/param/BoolParam.h"
#include "mmcore/param/EnumParam.h"
#include "mmcore/param/FilePathParam.h"
#include "mmcore/param/FloatParam.h"
#include "mmcore/param/IntParam.h"
#include "mmcore/utility/log/Log.h"
#include "mmstd/renderer/CallClipPlane.h"

using namespace megamol;
using namespace megamol::p2v_gb300;
using core::param::BoolParam;
using core::param::EnumParam;
using core::param::FilePathParam;
using core::param::FloatParam;
using core::param::IntParam;

ParticlesToDensityGPU::ParticlesToDensityGPU()
        : aggregatorSlot("aggregator", "algorithm for the aggregation")
        , xResSlot("sizex", "The size of the volume in numbers of voxels")
        , yResSlot("sizey", "The size of the volume in numbers of voxels")
        , zResSlot("sizez", "The size of the volume in numbers of voxels")
        , cyclXSlot("cyclX", "Considers cyclic boundary conditions in X direction")
        , cyclYSlot("cyclY", "Considers cyclic boundary conditions in Y direction")
        , cyclZSlot("cyclZ", "Considers cyclic boundary conditions in Z direction")
        , normalizeSlot("normalize", "Normalize the output volume")
        , sigmaSlot("sigma", "Sigma for Gauss in multiple of rad")
        , surfaceSlot("forSurfaceReconstruction", "Set true if this volume is used for surface reconstruction")
        , kernelSlot("kernel", "Density kernel: reference bump, or Gaussian cut at 3 sigma")
        , massNormSlot("massNormalize", "Scale the grid so that it integrates to the particle count")
        , aoModeSlot("ao::mode", "Per-particle ambient occlusion")
        , aoConesSlot("ao::cones", "Number of cones")
        , aoStepsSlot("ao::steps", "Samples per cone (0 = geometric steps until the cone length)")
        , aoLevelsSlot("ao::levels", "Mip levels (0 = log2 of the longest edge)")
        , aoApexSlot("ao::apex", "Cone apex angle in degrees")
        , aoOffsetSlot("ao::offset", "Offset from the surface")
        , aoStrengthSlot("ao::strength", "Strength")
        , aoConeLengthSlot("ao::coneLength", "Cone length")
        , aoVolumeSlot("ao::volume", "Volume the cone march samples: the density grid or MDAO's occupancy volume")
        , aoVolumeScaleSlot("ao::volumeScale", "Density to occlusion scale of the density grid (saturated at 1)")
        , aoNormalsSlot("ao::normals", "Particle normals: the input's directions or the density gradient")
        , aoModelSlot("ao::model", "Network file of the learned AO (p2v_mlp_save)")
        , mdaoVolSizeSlot("ambient occlusion::volumeSize", "Ambient Occlusion: Longest volume edge")
        , mdaoHighPrecisionSlot("ambient occlusion::highPrecisionTexture", "Ambient Occlusion: Use high precision textures")
        , aosSizeXSlot("vol::sizex", "The size of the volume in numbers of voxels")
        , aosSizeYSlot("vol::sizey", "The size of the volume in numbers of voxels")
        , aosSizeZSlot("vol::sizez", "The size of the volume in numbers of voxels")
        , aosGenSlot("vol::gen", "The generation method")
        , aosStepLenSlot("ao::stepLen", "The access step length in voxels")
        , aosGenFacSlot("vol::genFac", "The generation factor (influence factor of a single sphere on a voxel)")
        , aosEvalFacSlot("ao::evalFac", "The evaluation factor (influence factor of a single voxel on a sphere)")
        , aosClipDataSlot("ao::clipData", "Clip ao data")
        , getClipPlaneSlot("getclipplane", "Connects to a clipping plane module")
        , outDataSlot("outData", "Provides a density volume for the particles")
        , outParticlesSlot("outParticles", "Provides particles forming a regular grid with the sampled values")
        , outInfoSlot("outInfo", "Provides information which can be used for visualization and filtering")
        , outAOSlot("outAO", "Provides the particles with their ambient occlusion as intensity colour")
        , inDataSlot("inData", "Takes the particle data") {
    auto* ep = new EnumParam(0);
    ep->SetTypePair(0, "PosToSingleCell_Volume");
    ep->SetTypePair(1, "IColToSingleCell_Volume");
    ep->SetTypePair(2, "IVecToSingleCell_Volume");
    aggregatorSlot << ep;
    MakeSlotAvailable(&aggregatorSlot);
    xResSlot << new IntParam(16);
    MakeSlotAvailable(&xResSlot);
    yResSlot << new IntParam(16);
    MakeSlotAvailable(&yResSlot);
    zResSlot << new IntParam(16);
    MakeSlotAvailable(&zResSlot);
    cyclXSlot.SetParameter(new BoolParam(true));
    MakeSlotAvailable(&cyclXSlot);
    cyclYSlot.SetParameter(new BoolParam(true));
    MakeSlotAvailable(&cyclYSlot);
    cyclZSlot.SetParameter(new BoolParam(true));
    MakeSlotAvailable(&cyclZSlot);
    normalizeSlot << new BoolParam(true);
    MakeSlotAvailable(&normalizeSlot);
    sigmaSlot << new FloatParam(1.0f, std::numeric_limits<float>::min(), std::numeric_limits<float>::max());
    MakeSlotAvailable(&sigmaSlot);
    surfaceSlot << new BoolParam(false);
    MakeSlotAvailable(&surfaceSlot);

    auto* kp = new EnumParam(P2V_KERNEL_BUMP);
    kp->SetTypePair(P2V_KERNEL_BUMP, "Bump (reference)");
    kp->SetTypePair(P2V_KERNEL_GAUSS3, "Gaussian, 3 sigma");
    kernelSlot << kp;
    MakeSlotAvailable(&kernelSlot);
    massNormSlot << new BoolParam(false);
    MakeSlotAvailable(&massNormSlot);
    auto* am = new EnumParam(P2V_AO_NONE);
    am->SetTypePair(P2V_AO_NONE, "None");
    am->SetTypePair(P2V_AO_CONE, "Cone march (MDAO)");
    am->SetTypePair(P2V_AO_AOSPHERE_AXES, "AOSphere main axes");
    am->SetTypePair(P2V_AO_AOSPHERE_NORMAL, "AOSphere normal");
    am->SetTypePair(P2V_AO_LEARNED, "Learned (MLP, cone-march fallback)");
    aoModeSlot << am;
    MakeSlotAvailable(&aoModeSlot);
    aoConesSlot << new IntParam(3, 1, 16);
    MakeSlotAvailable(&aoConesSlot);
    aoStepsSlot << new IntParam(0, 0, 256);
    MakeSlotAvailable(&aoStepsSlot);
    aoLevelsSlot << new IntParam(0, 0, 12);
    MakeSlotAvailable(&aoLevelsSlot);
    aoApexSlot << new FloatParam(50.0f, 1.0f, 90.0f);
    MakeSlotAvailable(&aoApexSlot);
    aoOffsetSlot << new FloatParam(0.01f, 0.0f, 0.2f);
    MakeSlotAvailable(&aoOffsetSlot);
    aoStrengthSlot << new FloatParam(1.0f, 0.1f, 20.0f);
    MakeSlotAvailable(&aoStrengthSlot);
    aoConeLengthSlot << new FloatParam(0.8f, 0.01f, 1.0f);
    MakeSlotAvailable(&aoConeLengthSlot);
    auto* av = new EnumParam(P2V_AOVOL_DENSITY);
    av->SetTypePair(P2V_AOVOL_DENSITY, "Density grid");
    av->SetTypePair(P2V_AOVOL_MDAO, "MDAO occupancy");
    aoVolumeSlot << av;
    MakeSlotAvailable(&aoVolumeSlot);
    aoVolumeScaleSlot << new FloatParam(1.0f, 0.0f);
    MakeSlotAvailable(&aoVolumeScaleSlot);
    auto* an = new EnumParam(P2V_NORMALS_LIST);
    an->SetTypePair(P2V_NORMALS_LIST, "Input directions");
    an->SetTypePair(P2V_NORMALS_GRADIENT, "Density gradient");
    aoNormalsSlot << an;
    MakeSlotAvailable(&aoNormalsSlot);
    aoModelSlot << new FilePathParam("");
    MakeSlotAvailable(&aoModelSlot);
    // SphereRenderer.cpp:205,214
    mdaoVolSizeSlot << new IntParam(128, 1, 1024);
    MakeSlotAvailable(&mdaoVolSizeSlot);
    mdaoHighPrecisionSlot << new BoolParam(false);
    MakeSlotAvailable(&mdaoHighPrecisionSlot);
    // AOSphereRenderer.cpp:86-118
    aosSizeXSlot << new IntParam(32, 4);
    MakeSlotAvailable(&aosSizeXSlot);
    aosSizeYSlot << new IntParam(32, 4);
    MakeSlotAvailable(&aosSizeYSlot);
    aosSizeZSlot << new IntParam(32, 4);
    MakeSlotAvailable(&aosSizeZSlot);
    auto* gen = new EnumParam(P2V_AOS_DEPOSIT_CPU);
    gen->SetTypePair(P2V_AOS_DEPOSIT_CPU, "CPU");
    gen->SetTypePair(P2V_AOS_DEPOSIT_GLSL, "GPU (GLSL)");
    aosGenSlot << gen;
    MakeSlotAvailable(&aosGenSlot);
    aosStepLenSlot << new FloatParam(0.5f, 0.0f);
    MakeSlotAvailable(&aosStepLenSlot);
    aosGenFacSlot << new FloatParam(1.0f, 0.0f);
    MakeSlotAvailable(&aosGenFacSlot);
    aosEvalFacSlot << new FloatParam(1.0f, 0.0f);
    MakeSlotAvailable(&aosEvalFacSlot);
    aosClipDataSlot << new BoolParam(false);
    MakeSlotAvailable(&aosClipDataSlot);
    getClipPlaneSlot.SetCompatibleCall<core::view::CallClipPlaneDescription>();
    MakeSlotAvailable(&getClipPlaneSlot);

    using VDC = geocalls::VolumetricDataCall;
    outDataSlot.SetCallback(VDC::ClassName(), VDC::FunctionName(VDC::IDX_GET_DATA),
        &ParticlesToDensityGPU::getDataCallback);
    outDataSlot.SetCallback(VDC::ClassName(), VDC::FunctionName(VDC::IDX_GET_EXTENTS),
        &ParticlesToDensityGPU::getExtentCallback);
    outDataSlot.SetCallback(VDC::ClassName(), VDC::FunctionName(VDC::IDX_GET_METADATA),
        &ParticlesToDensityGPU::getExtentCallback);
    outDataSlot.SetCallback(VDC::ClassName(), VDC::FunctionName(VDC::IDX_START_ASYNC),
        &ParticlesToDensityGPU::dummyCallback);
    outDataSlot.SetCallback(VDC::ClassName(), VDC::FunctionName(VDC::IDX_STOP_ASYNC),
        &ParticlesToDensityGPU::dummyCallback);
    outDataSlot.SetCallback(VDC::ClassName(), VDC::FunctionName(VDC::IDX_TRY_GET_DATA),
        &ParticlesToDensityGPU::dummyCallback);
    MakeSlotAvailable(&outDataSlot);

    using MPDC = geocalls::MultiParticleDataCall;
    using TDC = datatools::table::TableDataCall;
    // as the reference, one data and one extent callback serve the volume, the grid and the table
    // (ParticlesToDensity.cpp:114-124)
    outParticlesSlot.SetCallback(MPDC::ClassName(), MPDC::FunctionName(0), &ParticlesToDensityGPU::getDataCallback);
    outParticlesSlot.SetCallback(MPDC::ClassName(), MPDC::FunctionName(1), &ParticlesToDensityGPU::getExtentCallback);
    MakeSlotAvailable(&outParticlesSlot);
    outInfoSlot.SetCallback(TDC::ClassName(), TDC::FunctionName(0), &ParticlesToDensityGPU::getDataCallback);
    outInfoSlot.SetCallback(TDC::ClassName(), TDC::FunctionName(1), &ParticlesToDensityGPU::getExtentCallback);
    MakeSlotAvailable(&outInfoSlot);

    outAOSlot.SetCallback(MPDC::ClassName(), MPDC::FunctionName(0), &ParticlesToDensityGPU::getAODataCallback);
    outAOSlot.SetCallback(MPDC::ClassName(), MPDC::FunctionName(1), &ParticlesToDensityGPU::getAOExtentCallback);
    MakeSlotAvailable(&outAOSlot);

    inDataSlot.SetCompatibleCall<geocalls::MultiParticleDataCallDescription>();
    MakeSlotAvailable(&inDataSlot);
}

ParticlesToDensityGPU::~ParticlesToDensityGPU() {
    Release();
}

bool ParticlesToDensityGPU::create() {
    // one GPU, device 0, as MegaMol's CUDA service creates its context (frontend/services/cuda/CUDA_Service.cpp:30-56)
    if (p2v_create(&ctx, 0) != P2V_OK) {
        core::utility::log::Log::DefaultLog.WriteError("ParticlesToDensityGPU: no CUDA device for libp2v");
        return false;
    }
    return true;
}

void ParticlesToDensityGPU::release() {
    p2v_destroy(ctx);
    ctx = nullptr;
}

bool ParticlesToDensityGPU::anythingDirty() const {
    for (auto* s : {&aggregatorSlot, &xResSlot, &yResSlot, &zResSlot, &cyclXSlot, &cyclYSlot, &cyclZSlot,
             &normalizeSlot, &sigmaSlot, &kernelSlot, &massNormSlot, &aoModeSlot, &aoConesSlot, &aoStepsSlot,
             &aoLevelsSlot, &aoApexSlot, &aoOffsetSlot, &aoStrengthSlot, &aoConeLengthSlot, &aoVolumeSlot,
             &aoVolumeScaleSlot, &aoNormalsSlot, &aoModelSlot, &mdaoVolSizeSlot, &mdaoHighPrecisionSlot, &aosSizeXSlot,
             &aosSizeYSlot, &aosSizeZSlot, &aosGenSlot, &aosStepLenSlot, &aosGenFacSlot, &aosEvalFacSlot,
             &aosClipDataSlot})
        if (s->IsDirty())
            return true;
    return false;
}

void ParticlesToDensityGPU::resetDirty() {
    for (auto* s : {&aggregatorSlot, &xResSlot, &yResSlot, &zResSlot, &cyclXSlot, &cyclYSlot, &cyclZSlot,
             &normalizeSlot, &sigmaSlot, &kernelSlot, &massNormSlot, &aoModeSlot, &aoConesSlot, &aoStepsSlot,
             &aoLevelsSlot, &aoApexSlot, &aoOffsetSlot, &aoStrengthSlot, &aoConeLengthSlot, &aoVolumeSlot,
             &aoVolumeScaleSlot, &aoNormalsSlot, &aoModelSlot, &mdaoVolSizeSlot, &mdaoHighPrecisionSlot, &aosSizeXSlot,
             &aosSizeYSlot, &aosSizeZSlot, &aosGenSlot, &aosStepLenSlot, &aosGenFacSlot, &aosEvalFacSlot,
             &aosClipDataSlot})
        s->ResetDirty();
}

bool ParticlesToDensityGPU::getExtentCallback(core::Call& c) {
    auto* out = dynamic_cast<geocalls::VolumetricDataCall*>(&c);
    auto* outGrid = dynamic_cast<geocalls::MultiParticleDataCall*>(&c);
    auto* outInfo = dynamic_cast<datatools::table::TableDataCall*>(&c);
    auto* in = inDataSlot.CallAs<geocalls::MultiParticleDataCall>();
    if (in == nullptr)
        return false;
    in->SetFrameID(out != nullptr ? out->FrameID() : (outGrid != nullptr ? outGrid->FrameID() : 0), true);
    if (!(*in)(1))
        return false;
    if (out != nullptr) {
        out->AccessBoundingBoxes().SetObjectSpaceBBox(in->GetBoundingBoxes().ObjectSpaceBBox());
        out->AccessBoundingBoxes().SetObjectSpaceClipBox(in->GetBoundingBoxes().ObjectSpaceClipBox());
        out->AccessBoundingBoxes().MakeScaledWorld(1.0f);
        out->SetFrameCount(in->FrameCount());
    }
    if (outGrid != nullptr) {
        outGrid->AccessBoundingBoxes().SetObjectSpaceBBox(in->GetBoundingBoxes().ObjectSpaceBBox());
        outGrid->AccessBoundingBoxes().SetObjectSpaceClipBox(in->GetBoundingBoxes().ObjectSpaceClipBox());
        outGrid->AccessBoundingBoxes().MakeScaledWorld(1.0f);
        outGrid->SetFrameCount(in->FrameCount());
    }
    if (outInfo != nullptr) {
        outInfo->SetDataHash(dataHash);
        outInfo->SetUnlocker(nullptr);
        outInfo->SetFrameCount(in->FrameCount());
    }
    return true;
}

bool ParticlesToDensityGPU::dummyCallback(core::Call&) {
    return true;
}

bool ParticlesToDensityGPU::pullFrame(geocalls::MultiParticleDataCall* in, unsigned int frame) {
    do { // ParticlesToDensity.cpp:222-232
        in->SetFrameID(frame, true);
        if (!(*in)(1) || !(*in)(0)) {
            core::utility::log::Log::DefaultLog.WriteError("ParticlesToDensityGPU: unable to get frame %u", frame);
            return false;
        }
    } while (in->FrameID() != frame);
    if (time != in->FrameID() || inDataHash != in->DataHash() || anythingDirty()) {
        if (!recompute(in))
            return false;
        time = in->FrameID();
        inDataHash = in->DataHash();
        ++dataHash;
        resetDirty();
    }
    return true;
}

bool ParticlesToDensityGPU::recompute(geocalls::MultiParticleDataCall* in) {
    p2v_params prm;
    p2v_params_default(&prm);
    prm.aggregator = aggregatorSlot.Param<EnumParam>()->Value();
    prm.sizex = xResSlot.Param<IntParam>()->Value();
    prm.sizey = yResSlot.Param<IntParam>()->Value();
    prm.sizez = zResSlot.Param<IntParam>()->Value();
    prm.cyclX = cyclXSlot.Param<BoolParam>()->Value();
    prm.cyclY = cyclYSlot.Param<BoolParam>()->Value();
    prm.cyclZ = cyclZSlot.Param<BoolParam>()->Value();
    prm.normalize = normalizeSlot.Param<BoolParam>()->Value();
    prm.sigma = sigmaSlot.Param<FloatParam>()->Value();
    prm.forSurfaceReconstruction = surfaceSlot.Param<BoolParam>()->Value();
    prm.kernel = kernelSlot.Param<EnumParam>()->Value();
    prm.mass_normalize = massNormSlot.Param<BoolParam>()->Value();
    prm.ao_mode = aoModeSlot.Param<EnumParam>()->Value();
    prm.ao_cones = aoConesSlot.Param<IntParam>()->Value();
    prm.ao_steps = aoStepsSlot.Param<IntParam>()->Value();
    prm.ao_levels = aoLevelsSlot.Param<IntParam>()->Value();
    prm.ao_apex_deg = aoApexSlot.Param<FloatParam>()->Value();
    prm.ao_offset = aoOffsetSlot.Param<FloatParam>()->Value();
    prm.ao_strength = aoStrengthSlot.Param<FloatParam>()->Value();
    prm.ao_cone_length = aoConeLengthSlot.Param<FloatParam>()->Value();
    prm.ao_volume = aoVolumeSlot.Param<EnumParam>()->Value();
    prm.ao_volume_scale = aoVolumeScaleSlot.Param<FloatParam>()->Value();
    prm.ao_normals = aoNormalsSlot.Param<EnumParam>()->Value();
    prm.mdao_volume_size = mdaoVolSizeSlot.Param<IntParam>()->Value();
    prm.mdao_unorm8 = mdaoHighPrecisionSlot.Param<BoolParam>()->Value() ? 0 : 1;  // R8 unless high precision
    prm.aos_sizex = aosSizeXSlot.Param<IntParam>()->Value();
    prm.aos_sizey = aosSizeYSlot.Param<IntParam>()->Value();
    prm.aos_sizez = aosSizeZSlot.Param<IntParam>()->Value();
    prm.aos_deposit = aosGenSlot.Param<EnumParam>()->Value();
    prm.aos_step_len = aosStepLenSlot.Param<FloatParam>()->Value();
    prm.aos_gen_fac = aosGenFacSlot.Param<FloatParam>()->Value();
    prm.aos_eval_fac = aosEvalFacSlot.Param<FloatParam>()->Value();
    prm.aos_clip = aosClipDataSlot.Param<BoolParam>()->Value();
    // the clip plane as AOSphereRenderer reads it (:273-287): unit normal and d = dot(point, normal), all zeros
    // without a connected clip-plane module
    auto* ccp = getClipPlaneSlot.CallAs<core::view::CallClipPlane>();
    if (ccp != nullptr && (*ccp)(0)) {
        const auto& pl = ccp->GetPlane();
        const auto n = pl.Normal();
        const auto pt = pl.Point();
        prm.aos_clip_plane[0] = n.X();
        prm.aos_clip_plane[1] = n.Y();
        prm.aos_clip_plane[2] = n.Z();
        prm.aos_clip_plane[3] = pt.X() * n.X() + pt.Y() * n.Y() + pt.Z() * n.Z();
    }
    prm.vector_grid = prm.aggregator == 2;
    if (p2v_set_params(ctx, &prm) != P2V_OK)
        return false;
    // the learned AO's network, loaded when the file parameter names a new file
    const std::string model = aoModelSlot.Param<FilePathParam>()->Value().string();
    if (!model.empty() && model != loadedModel) {
        if (p2v_mlp_load(ctx, model.c_str()) != P2V_OK) {
            char msg[512];
            p2v_get_last_error(ctx, msg, sizeof(msg));
            core::utility::log::Log::DefaultLog.WriteError("ParticlesToDensityGPU: %s", msg);
            return false;
        }
        loadedModel = model;
    }

    const unsigned int nl = in->GetParticleListCount();
    std::vector<p2v_particle_list> lists(nl);
    ao.resize(nl);
    for (unsigned int i = 0; i < nl; ++i) {
        auto& p = in->AccessParticles(i);
        p2v_particle_list& L = lists[i];
        L = p2v_particle_list{};
        L.vertex_type = static_cast<int32_t>(p.GetVertexDataType());
        L.vertex_data = p.GetVertexData();
        L.vertex_stride = p.GetVertexDataStride();
        L.count = p.GetCount();
        L.global_radius = p.GetGlobalRadius();
        L.mem = P2V_MEM_HOST;
        // the intensity aggregator reads the first colour channel, or the global colour's red
        L.colour_type = static_cast<int32_t>(p.GetColourDataType());
        L.colour_data = p.GetColourData();
        L.colour_stride = p.GetColourDataStride();
        std::copy(p.GetGlobalColour(), p.GetGlobalColour() + 4, L.global_colour);
        // the vector aggregator's directions: DIRDATA_FLOAT_XYZ
        if (prm.aggregator == 2 && p.GetDirDataType() == geocalls::SimpleSphericalParticles::DIRDATA_FLOAT_XYZ) {
            L.normals = static_cast<const float*>(p.GetDirData());
            L.normal_stride = p.GetDirDataStride();
        }
        if (prm.ao_mode != P2V_AO_NONE) {
            if (prm.ao_normals == P2V_NORMALS_LIST) {
                L.normals = static_cast<const float*>(p.GetDirData());
                L.normal_stride = p.GetDirDataStride();
            }
            ao[i].resize(p.GetCount());
            L.ao_out = ao[i].data();
        }
    }
    p2v_frame fr{};
    const auto& bb = in->AccessBoundingBoxes().ObjectSpaceBBox();
    const auto& cb = in->AccessBoundingBoxes().ObjectSpaceClipBox();
    const float box[6] = {bb.Left(), bb.Bottom(), bb.Back(), bb.Right(), bb.Top(), bb.Front()};
    const float clip[6] = {cb.Left(), cb.Bottom(), cb.Back(), cb.Right(), cb.Top(), cb.Front()};
    std::copy(box, box + 6, fr.bbox);
    std::copy(clip, clip + 6, fr.clipbox);
    fr.frame_id = in->FrameID();
    fr.list_count = nl;
    fr.lists = lists.data();

    // the grid size is only final after the surface-reconstruction box adjustment: ask the library first
    p2v_volume v{};
    if (prm.forSurfaceReconstruction) {
        if (p2v_run_frame(ctx, &fr, &v, nullptr) != P2V_OK)
            return false;
    } else {
        v.resolution[0] = prm.sizex;
        v.resolution[1] = prm.sizey;
        v.resolution[2] = prm.sizez;
    }
    const int comps = prm.aggregator == 2 ? 3 : 1;
    volume.resize(v.resolution[0] * v.resolution[1] * v.resolution[2] * comps);
    v.data = volume.data();
    v.mem = P2V_MEM_HOST;
    v.capacity = volume.size();
    if (p2v_run_frame(ctx, &fr, &v, nullptr) != P2V_OK) {
        char msg[512];
        p2v_get_last_error(ctx, msg, sizeof(msg));
        core::utility::log::Log::DefaultLog.WriteError("ParticlesToDensityGPU: %s", msg);
        return false;
    }
    if (prm.forSurfaceReconstruction) {
        // mirror the parameter rewrite of modifyBBox (ParticlesToDensity.cpp:772,779)
        xResSlot.Param<IntParam>()->SetValue(static_cast<int>(v.resolution[0]), false);
        yResSlot.Param<IntParam>()->SetValue(static_cast<int>(v.resolution[1]), false);
    }
    metadata.Components = comps;
    metadata.GridType = geocalls::CARTESIAN;
    metadata.ScalarType = geocalls::FLOATING_POINT;
    metadata.ScalarLength = sizeof(float);
    metadata.NumberOfFrames = 1;
    for (int a = 0; a < 3; ++a) {
        metadata.Resolution[a] = v.resolution[a];
        metadata.Extents[a] = v.extents[a];
        metadata.Origin[a] = v.origin[a];
        sliceDists[a] = v.slice_dists[a];
        metadata.SliceDists[a] = &sliceDists[a];
        metadata.IsUniform[a] = true;
    }
    // every component carries the published range (ParticlesToDensity.cpp:259-270)
    for (int k = 0; k < 3; ++k) {
        minValues[k] = v.min_value;
        maxValues[k] = v.max_value;
    }
    metadata.MinValues = minValues;
    metadata.MaxValues = maxValues;
    hasData = true;
    return prm.aggregator != 2 || fetchVectorGrid();
}

bool ParticlesToDensityGPU::fetchVectorGrid() {
    p2v_vector_grid_info vg{};
    if (p2v_get_vector_grid(ctx, nullptr, nullptr, nullptr, nullptr, 0, P2V_MEM_HOST, &vg) != P2V_OK)
        return false;
    grid.resize(3 * vg.count);
    directions.resize(3 * vg.count);
    colors.resize(vg.count);
    infoData.resize(7 * vg.count);
    if (p2v_get_vector_grid(ctx, grid.data(), directions.data(), colors.data(), infoData.data(), vg.count,
            P2V_MEM_HOST, &vg) != P2V_OK)
        return false;
    gridRadius = vg.global_radius;
    static const char* names[7] = {
        "PositionX", "PositionY", "PositionZ", "VelocityX", "VelocityY", "VelocityZ", "VelocityMag"};
    for (int k = 0; k < 7; ++k) {  // ParticlesToDensity.cpp:327-377
        info[k].SetName(names[k]);
        info[k].SetType(datatools::table::TableDataCall::ColumnType::QUANTITATIVE);
        info[k].SetMinimumValue(vg.col_min[k]);
        info[k].SetMaximumValue(vg.col_max[k]);
    }
    return true;
}

bool ParticlesToDensityGPU::getDataCallback(core::Call& c) {
    auto* in = inDataSlot.CallAs<geocalls::MultiParticleDataCall>();
    auto* out = dynamic_cast<geocalls::VolumetricDataCall*>(&c);
    auto* outGrid = dynamic_cast<geocalls::MultiParticleDataCall*>(&c);
    auto* outInfo = dynamic_cast<datatools::table::TableDataCall*>(&c);
    if (in == nullptr)
        return false;
    // the volume and the grid pull the frame; the table serves the last result (ParticlesToDensity.cpp:220-245)
    if (out != nullptr || outGrid != nullptr)
        if (!pullFrame(in, out != nullptr ? out->FrameID() : outGrid->FrameID()))
            return false;
    const bool isVector = aggregatorSlot.Param<EnumParam>()->Value() == 2;
    if (out != nullptr) {
        out->SetFrameID(time);
        out->SetData(volume.data());
        out->SetMetadata(&metadata);
        out->SetDataHash(dataHash);
    }
    if (outGrid != nullptr && isVector) {  // ParticlesToDensity.cpp:306-323
        outGrid->SetFrameID(time);
        outGrid->SetDataHash(dataHash);
        outGrid->SetParticleListCount(1);
        auto& p = outGrid->AccessParticles(0);
        p.SetCount(colors.size());
        if (p.GetCount() > 0) {
            p.SetVertexData(geocalls::SimpleSphericalParticles::VERTDATA_FLOAT_XYZ, grid.data());
            p.SetDirData(geocalls::SimpleSphericalParticles::DIRDATA_FLOAT_XYZ, directions.data());
            p.SetColourData(geocalls::SimpleSphericalParticles::COLDATA_FLOAT_I, colors.data());
            p.SetGlobalRadius(gridRadius);
        }
    }
    if (outInfo != nullptr && isVector) {  // ParticlesToDensity.cpp:325-380
        if (!hasData) {
            infoData.clear();
            outInfo->SetDataHash(0);
        } else {
            outInfo->SetDataHash(dataHash);
        }
        outInfo->Set(info.size(), infoData.size() / info.size(), info.data(), infoData.data());
    }
    return true;
}

bool ParticlesToDensityGPU::getAOExtentCallback(core::Call& c) {
    auto* out = dynamic_cast<geocalls::MultiParticleDataCall*>(&c);
    auto* in = inDataSlot.CallAs<geocalls::MultiParticleDataCall>();
    if (out == nullptr || in == nullptr)
        return false;
    in->SetFrameID(out->FrameID(), true);
    if (!(*in)(1))
        return false;
    out->AccessBoundingBoxes().SetObjectSpaceBBox(in->GetBoundingBoxes().ObjectSpaceBBox());
    out->AccessBoundingBoxes().SetObjectSpaceClipBox(in->GetBoundingBoxes().ObjectSpaceClipBox());
    out->SetFrameCount(in->FrameCount());
    return true;
}

bool ParticlesToDensityGPU::getAODataCallback(core::Call& c) {
    auto* out = dynamic_cast<geocalls::MultiParticleDataCall*>(&c);
    auto* in = inDataSlot.CallAs<geocalls::MultiParticleDataCall>();
    if (out == nullptr || in == nullptr || aoModeSlot.Param<EnumParam>()->Value() == P2V_AO_NONE)
        return false;
    if (!pullFrame(in, out->FrameID()))
        return false;
    out->SetFrameID(time);
    out->SetDataHash(dataHash);
    out->SetParticleListCount(in->GetParticleListCount());
    for (unsigned int i = 0; i < in->GetParticleListCount(); ++i) {
        auto& src = in->AccessParticles(i);
        auto& dst = out->AccessParticles(i);
        dst.SetCount(src.GetCount());
        dst.SetGlobalRadius(src.GetGlobalRadius());
        dst.SetVertexData(src.GetVertexDataType(), src.GetVertexData(), src.GetVertexDataStride());
        dst.SetDirData(src.GetDirDataType(), src.GetDirData(), src.GetDirDataStride());
        dst.SetColourData(geocalls::SimpleSphericalParticles::COLDATA_FLOAT_I, ao[i].data());
        dst.SetColourMapIndexValues(0.0f, 1.0f);
    }
    return true;
}
