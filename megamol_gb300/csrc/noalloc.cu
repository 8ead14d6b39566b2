// Allocation-free AOSphere AO.
//
// Some callers cannot allocate device memory while they compute AO: a renderer that records its frame
// into a CUDA graph (allocation is not capturable), a host application that hands this library a fixed
// memory budget and forbids later growth, or code running where cudaMalloc would synchronise the device
// in the middle of a frame. p2v_aosphere_ao_noalloc serves them: the caller passes device inputs and the
// output buffer, and the only scratch (the AO volume and its fixed-point accumulator) lives in the
// file-scope arrays below, sized for at most P2V_NOALLOC_MAX_VOXELS voxels. Every GPU that loads the
// library holds these 3 MB until the process exits.
//
// The arrays are shared by every call on a device and keep the last call's contents; the accumulator is
// cleared at the start of each call. Calls that overlap on the GPU (two streams, two host threads) race
// on the arrays and must be serialised by the caller.
#include <cuda_runtime.h>

#include <cstdint>
#include <cmath>
#include <mutex>

#include "../../include/p2v.h"
#include "ao_internal.h"

namespace {

constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned long long g_aos_acc[P2V_NOALLOC_MAX_VOXELS];
__device__ __align__(256) float g_aos_tex[P2V_NOALLOC_MAX_VOXELS];

struct Scratch {
    bool ready = false;
    unsigned long long* acc = nullptr;
    float* tex = nullptr;
    int sms = 0;
};

std::mutex g_mutex;
Scratch g_scratch[kMaxDevices];

// Device addresses of the scratch arrays on the current device. In host code the array names are
// host-side stand-ins, not device addresses: the kernel must receive the address looked up here. The
// lookup runs once per device, on the first call made with that device current.
p2v_status scratch_for_current_device(Scratch& out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
        return P2V_ECUDA;
    std::lock_guard<std::mutex> lock(g_mutex);
    Scratch& s = g_scratch[dev];
    if (!s.ready) {
        void* acc = nullptr;
        void* tex = nullptr;
        if (cudaGetSymbolAddress(&acc, g_aos_acc) != cudaSuccess)
            return P2V_ECUDA;
        if (cudaGetSymbolAddress(&tex, g_aos_tex) != cudaSuccess)
            return P2V_ECUDA;
        int sms = 0;
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
            return P2V_ECUDA;
        s.acc = static_cast<unsigned long long*>(acc);
        s.tex = static_cast<float*>(tex);
        s.sms = sms;
        s.ready = true;
    }
    out = s;
    return P2V_OK;
}

}  // namespace

extern "C" p2v_status p2v_aosphere_ao_noalloc(const float* xyzr, const float* normals, uint64_t count,
    const float clipbox[6], const int32_t vol_size[3], float step_len, float gen_fac, float eval_fac, int32_t mode,
    float* ao_out, void* stream) {
    if ((count > 0 && (xyzr == nullptr || normals == nullptr || ao_out == nullptr)) || clipbox == nullptr ||
        vol_size == nullptr || (mode != P2V_AO_AOSPHERE_AXES && mode != P2V_AO_AOSPHERE_NORMAL))
        return P2V_EINVAL;
    if (count >= (1ull << 31))
        return P2V_EINVAL;
    // Checked after every factor, so the product cannot wrap: each axis is at most the maximum, and a
    // running product above it is rejected before the next multiplication.
    uint64_t voxels = 1;
    for (int a = 0; a < 3; ++a) {
        if (vol_size[a] < 3 || vol_size[a] > P2V_NOALLOC_MAX_VOXELS)
            return P2V_EINVAL;
        voxels *= (uint64_t) vol_size[a];
        if (voxels > (uint64_t) P2V_NOALLOC_MAX_VOXELS)
            return P2V_EINVAL;  // beyond the static scratch; use p2v_run_frame, which allocates what it needs
    }
    p2v::AOSphereParams ap{};
    for (int a = 0; a < 3; ++a) {
        ap.s[a] = vol_size[a];
        ap.si[a] = vol_size[a] - 2;
        ap.minOS[a] = clipbox[a];
        ap.rangeOS[a] = std::fabs(clipbox[a + 3] - clipbox[a]);
        if (!(ap.rangeOS[a] > 0.0f))
            return P2V_EINVAL;
        // AOSphereRenderer.cpp:496-513
        const float ext = ap.rangeOS[a] / (1.0f - 2.0f / static_cast<float>(vol_size[a]));
        ap.ext[a] = ext;
        ap.origin[a] = ap.minOS[a] - ext / static_cast<float>(vol_size[a]);
        ap.sampd[a] = step_len * (ap.rangeOS[a] / static_cast<float>(vol_size[a]));
    }
    ap.voxel_vol = (ap.rangeOS[0] / static_cast<float>(ap.si[0])) * (ap.rangeOS[1] / static_cast<float>(ap.si[1])) *
                   (ap.rangeOS[2] / static_cast<float>(ap.si[2]));
    ap.gen_fac = gen_fac;
    ap.eval_fac = eval_fac;
    Scratch s;
    const p2v_status ps = scratch_for_current_device(s);
    if (ps != P2V_OK)
        return ps;
    const cudaError_t e = p2v::launch_aosphere(ap, reinterpret_cast<const float4*>(xyzr), (uint32_t) count, s.acc,
                                               s.tex, nullptr, reinterpret_cast<const float4*>(normals),
                                               mode == P2V_AO_AOSPHERE_AXES ? 0 : 1, ao_out, s.sms,
                                               static_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? P2V_OK : P2V_ECUDA;
}
