// Drives the MegaMol module ParticlesToDensityGPU (megamol_gb300/adapter) the way a MegaMol graph does: a particle
// source connected to "inData", a clip-plane module to "getclipplane", parameters set by slot name, and the
// callee slots "outData" (VolumetricDataCall GetExtents / GetData) and "outAO" (MultiParticleDataCall GetData)
// called by name. Every result is compared with p2v_run_frame called directly with the same parameters: the
// volume, its metadata and the AO must be identical. Exit status 0 when all cases agree; one line per case.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "ParticlesToDensityGPU.h"
#include "mmstd/renderer/CallClipPlane.h"

using namespace megamol;
using core::param::BoolParam;
using core::param::EnumParam;
using core::param::FloatParam;
using core::param::IntParam;

namespace {

int failures = 0;

void check(bool ok, const char* what) {
    std::printf("%s %s\n", ok ? "ok  " : "FAIL", what);
    if (!ok)
        ++failures;
}

template<class P, class V>
void set(core::Module& m, const char* name, V v) {
    auto* s = dynamic_cast<core::param::ParamSlot*>(m.FindSlot(name));
    if (s == nullptr || s->Param<P>() == nullptr) {
        std::printf("FAIL no parameter %s\n", name);
        ++failures;
        return;
    }
    s->Param<P>()->SetValue(v);
}

struct Frame {
    std::vector<float> xyzr, nrm;
    float bbox[6] = {0, 0, 0, 30, 30, 30};
};

Frame make_frame(size_t n) {
    Frame f;
    uint64_t s = 0x9E3779B97F4A7C15ull;
    auto rnd = [&]() {
        s = s * 6364136223846793005ull + 1442695040888963407ull;
        return (float) ((s >> 40) * (1.0 / 16777216.0));
    };
    f.xyzr.resize(4 * n);
    f.nrm.resize(3 * n);
    for (size_t i = 0; i < n; ++i) {
        for (int a = 0; a < 3; ++a)
            f.xyzr[4 * i + a] = 30.0f * rnd();
        f.xyzr[4 * i + 3] = 0.4f + 0.4f * rnd();
        float v[3], l = 0;
        for (int a = 0; a < 3; ++a) {
            v[a] = 2.0f * rnd() - 1.0f;
            l += v[a] * v[a];
        }
        l = std::sqrt(l) + 1e-6f;
        for (int a = 0; a < 3; ++a)
            f.nrm[3 * i + a] = v[a] / l;
    }
    return f;
}

// the direct call: the same frame through p2v_run_frame with the parameters the module should have set
bool direct(const p2v_params& prm, const Frame& f, bool with_normals, std::vector<float>& vol, std::vector<float>& ao,
            p2v_volume& meta) {
    p2v_ctx* ctx = nullptr;
    if (p2v_create(&ctx, 0) != P2V_OK)
        return false;
    bool ok = p2v_set_params(ctx, &prm) == P2V_OK;
    const size_t n = f.xyzr.size() / 4;
    p2v_particle_list L{};
    L.vertex_type = P2V_VERTDATA_FLOAT_XYZR;
    L.vertex_data = f.xyzr.data();
    L.count = n;
    L.mem = P2V_MEM_HOST;
    if (with_normals)
        L.normals = f.nrm.data();
    ao.assign(n, -1.0f);
    if (prm.ao_mode != P2V_AO_NONE)
        L.ao_out = ao.data();
    p2v_frame fr{};
    std::memcpy(fr.bbox, f.bbox, sizeof(fr.bbox));
    std::memcpy(fr.clipbox, f.bbox, sizeof(fr.clipbox));
    fr.list_count = 1;
    fr.lists = &L;
    vol.assign((size_t) prm.sizex * prm.sizey * prm.sizez, 0.0f);
    meta = p2v_volume{};
    meta.data = vol.data();
    meta.mem = P2V_MEM_HOST;
    meta.capacity = vol.size();
    ok = ok && p2v_run_frame(ctx, &fr, &meta, nullptr) == P2V_OK;
    p2v_destroy(ctx);
    return ok;
}

}  // namespace

int main() {
    const size_t n = 20000;
    Frame f = make_frame(n);

    // upstream particle source: one FLOAT_XYZR list with DIRDATA normals, frame 0 of 3
    geocalls::MultiParticleDataCall in;
    in.SetParticleListCount(1);
    auto& L = in.AccessParticles(0);
    L.SetCount(n);
    L.SetVertexData(geocalls::SimpleSphericalParticles::VERTDATA_FLOAT_XYZR, f.xyzr.data());
    L.SetDirData(geocalls::SimpleSphericalParticles::DIRDATA_FLOAT_XYZ, f.nrm.data());
    in.AccessBoundingBoxes().SetObjectSpaceBBox(f.bbox[0], f.bbox[1], f.bbox[2], f.bbox[3], f.bbox[4], f.bbox[5]);
    in.AccessBoundingBoxes().SetObjectSpaceClipBox(f.bbox[0], f.bbox[1], f.bbox[2], f.bbox[3], f.bbox[4], f.bbox[5]);
    in.SetFrameCount(3);
    in.SetDataHash(7);
    // the clip plane module: a plane through the box centre, normal (1, 2, 2) / 3
    core::view::CallClipPlane clip;
    clip.SetPlane(vislib::math::Plane<float>(15.0f, 15.0f, 15.0f, 1.0f, 2.0f, 2.0f));

    p2v_gb300::ParticlesToDensityGPU m;
    dynamic_cast<core::CallerSlot*>(m.FindSlot("inData"))->ConnectCall(&in);
    dynamic_cast<core::CallerSlot*>(m.FindSlot("getclipplane"))->ConnectCall(&clip);
    if (!m.Create()) {
        std::printf("FAIL create (no CUDA device?)\n");
        return 2;
    }
    auto* outData = dynamic_cast<core::CalleeSlot*>(m.FindSlot("outData"));
    auto* outAO = dynamic_cast<core::CalleeSlot*>(m.FindSlot("outAO"));

    // ---- getExtentCallback: box, clip box and frame count forwarded (ParticlesToDensity.cpp:163-208) ----
    geocalls::VolumetricDataCall vdc;
    vdc.SetFrameID(0);
    check(outData->InCall("VolumetricDataCall", "GetExtents", vdc), "GetExtents answered");
    const auto& bb = vdc.AccessBoundingBoxes().ObjectSpaceBBox();
    check(bb.Left() == f.bbox[0] && bb.Right() == f.bbox[3] && bb.Front() == f.bbox[5] && vdc.FrameCount() == 3,
          "GetExtents forwards the box and the frame count");

    struct Case {
        const char* name;
        int ao_mode, normals, aos_gen, clip;
    };
    const Case cases[] = {{"density + cone AO (list normals)", P2V_AO_CONE, P2V_NORMALS_LIST, 0, 0},
                          {"density + cone AO (gradient normals, no DIRDATA read)", P2V_AO_CONE, P2V_NORMALS_GRADIENT, 0, 0},
                          {"AOSphere main axes, CPU deposit with ao::clipData", P2V_AO_AOSPHERE_AXES, P2V_NORMALS_LIST, 0, 1},
                          {"AOSphere normal tap, GLSL deposit", P2V_AO_AOSPHERE_NORMAL, P2V_NORMALS_LIST, 1, 0}};
    for (const Case& c : cases) {
        set<IntParam>(m, "sizex", 40);
        set<IntParam>(m, "sizey", 36);
        set<IntParam>(m, "sizez", 32);
        set<BoolParam>(m, "normalize", true);
        set<EnumParam>(m, "ao::mode", c.ao_mode);
        set<IntParam>(m, "ao::cones", 8);
        set<IntParam>(m, "ao::steps", 32);
        set<IntParam>(m, "ao::levels", 3);
        set<EnumParam>(m, "ao::normals", c.normals);
        set<IntParam>(m, "vol::sizex", 20);
        set<IntParam>(m, "vol::sizey", 22);
        set<IntParam>(m, "vol::sizez", 18);
        set<EnumParam>(m, "vol::gen", c.aos_gen);
        set<BoolParam>(m, "ao::clipData", c.clip != 0);
        in.SetDataHash(in.DataHash() + 1);

        geocalls::VolumetricDataCall v;
        v.SetFrameID(0);
        const bool got = outData->InCall("VolumetricDataCall", "GetData", v);
        geocalls::MultiParticleDataCall aoc;
        aoc.SetFrameID(0);
        const bool got_ao = outAO->InCall("MultiParticleDataCall", "GetData", aoc);

        p2v_params prm;
        p2v_params_default(&prm);
        prm.sizex = 40, prm.sizey = 36, prm.sizez = 32;
        prm.normalize = 1;
        prm.ao_mode = c.ao_mode;
        prm.ao_cones = 8, prm.ao_steps = 32, prm.ao_levels = 3;
        prm.ao_normals = c.normals;
        prm.aos_sizex = 20, prm.aos_sizey = 22, prm.aos_sizez = 18;
        prm.aos_deposit = c.aos_gen;
        prm.aos_clip = c.clip;
        if (c.clip) {  // what the module reads from the clip-plane call: unit normal, d = dot(point, normal)
            const auto nv = clip.GetPlane().Normal();
            const auto pt = clip.GetPlane().Point();
            prm.aos_clip_plane[0] = nv.X();
            prm.aos_clip_plane[1] = nv.Y();
            prm.aos_clip_plane[2] = nv.Z();
            prm.aos_clip_plane[3] = pt.X() * nv.X() + pt.Y() * nv.Y() + pt.Z() * nv.Z();
        }
        std::vector<float> vol, ao;
        p2v_volume meta{};
        const bool ref_ok = direct(prm, f, c.normals == P2V_NORMALS_LIST, vol, ao, meta);
        char what[256];
        std::snprintf(what, sizeof(what), "%s: GetData answered, direct call ran", c.name);
        check(got && got_ao && ref_ok && v.GetData() != nullptr && v.GetMetadata() != nullptr, what);
        if (!(got && got_ao && ref_ok && v.GetData() && v.GetMetadata()))
            continue;
        const auto* md = v.GetMetadata();
        std::snprintf(what, sizeof(what), "%s: metadata (resolution, slice distances, origin, range)", c.name);
        check(md->Resolution[0] == 40 && md->Resolution[1] == 36 && md->Resolution[2] == 32 && md->Components == 1 &&
                  *md->SliceDists[0] == meta.slice_dists[0] && md->Origin[2] == meta.origin[2] &&
                  md->MinValues[0] == meta.min_value && md->MaxValues[0] == meta.max_value,
              what);
        std::snprintf(what, sizeof(what), "%s: volume identical to p2v_run_frame", c.name);
        check(std::memcmp(v.GetData(), vol.data(), vol.size() * sizeof(float)) == 0, what);
        const auto& P = aoc.AccessParticles(0);
        std::snprintf(what, sizeof(what), "%s: outAO carries the AO as COLDATA_FLOAT_I, identical", c.name);
        check(aoc.GetParticleListCount() == 1 && P.GetCount() == n &&
                  P.GetColourDataType() == geocalls::SimpleSphericalParticles::COLDATA_FLOAT_I &&
                  std::memcmp(P.GetColourData(), ao.data(), n * sizeof(float)) == 0,
              what);
    }
    m.Release();
    std::printf("%d failures\n", failures);
    return failures == 0 ? 0 : 1;
}
