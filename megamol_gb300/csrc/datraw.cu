// Dat/raw writer: the file pair of MegaMol's volume::DatRawWriter (plugins/volume/src/DatRawWriter.cpp:
// 58-186), host code. A device volume streams to the raw file through two pinned staging buffers on a
// stream of its own: the device-to-host copy of chunk k + 1 runs while chunk k is written.
#include <cuda_runtime.h>

#include <fcntl.h>
#include <unistd.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>

#include "../../include/p2v.h"

namespace {

constexpr uint64_t CHUNK_BYTES = 32ull << 20;

bool write_all(int fd, const void* p, uint64_t bytes) {
    const uint8_t* s = static_cast<const uint8_t*>(p);
    while (bytes > 0) {
        const ssize_t w = ::write(fd, s, std::min<uint64_t>(bytes, 1ull << 30));
        if (w <= 0)
            return false;
        s += w;
        bytes -= static_cast<uint64_t>(w);
    }
    return true;
}

// std::ostream's default formatting of a float (6 significant digits, %g), as the reference's << prints
std::string fmt(float v) {
    char b[64];
    std::snprintf(b, sizeof(b), "%g", static_cast<double>(v));
    return b;
}

// The .dat text of DatRawWriter::writeFrame (:113-166): FLOAT scalars on an EQUIDISTANT grid; the slice
// thickness line repeats the y spacing in place of z, as the reference writes it.
std::string dat_text(const std::string& raw_name, const p2v_volume& v, uint32_t frame) {
    std::string s;
    s += "ObjectFileName: " + raw_name + "\n";
    s += "Format:         FLOAT\n";
    s += "GridType:       EQUIDISTANT\n";
    s += "Components:     " + std::to_string(v.components) + "\n";
    s += "Dimensions:     3\n";
    s += "TimeSteps:      1\n";
    s += "ByteOrder:      LITTLE_ENDIAN\n";
    s += "Resolution:     " + std::to_string(v.resolution[0]) + " " + std::to_string(v.resolution[1]) + " " +
         std::to_string(v.resolution[2]) + "\n";
    s += "SliceThickness: " + fmt(v.slice_dists[0]) + " " + fmt(v.slice_dists[1]) + " " + fmt(v.slice_dists[1]) +
         "\n";
    s += "Origin:         " + fmt(v.origin[0]) + " " + fmt(v.origin[1]) + " " + fmt(v.origin[2]) + "\n";
    s += "Time:           " + std::to_string(frame) + "\n";
    return s;
}

p2v_status stream_device(int fd, const float* dsrc, uint64_t bytes) {
    cudaStream_t st = nullptr;
    void* buf[2] = {nullptr, nullptr};
    cudaEvent_t done[2] = {nullptr, nullptr};
    const uint64_t chunk = std::min(bytes, CHUNK_BYTES);
    cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    for (int k = 0; k < 2 && e == cudaSuccess; ++k) {
        e = cudaMallocHost(&buf[k], chunk);
        if (e == cudaSuccess)
            e = cudaEventCreateWithFlags(&done[k], cudaEventDisableTiming);
    }
    bool io_ok = true;
    const uint64_t nchunks = (bytes + chunk - 1) / chunk;
    const uint8_t* src = reinterpret_cast<const uint8_t*>(dsrc);
    auto issue = [&](uint64_t k) {
        const uint64_t off = k * chunk, n = std::min(chunk, bytes - off);
        cudaError_t r = cudaMemcpyAsync(buf[k & 1], src + off, n, cudaMemcpyDeviceToHost, st);
        return r == cudaSuccess ? cudaEventRecord(done[k & 1], st) : r;
    };
    if (e == cudaSuccess && nchunks > 0)
        e = issue(0);
    for (uint64_t k = 0; k < nchunks && e == cudaSuccess && io_ok; ++k) {
        if (k + 1 < nchunks)
            e = issue(k + 1);  // buffer (k + 1) & 1 was written out in iteration k - 1
        if (e == cudaSuccess)
            e = cudaEventSynchronize(done[k & 1]);
        if (e == cudaSuccess)
            io_ok = write_all(fd, buf[k & 1], std::min(chunk, bytes - k * chunk));
    }
    if (st)
        cudaStreamSynchronize(st);
    for (int k = 0; k < 2; ++k) {
        if (done[k])
            cudaEventDestroy(done[k]);
        if (buf[k])
            cudaFreeHost(buf[k]);
    }
    if (st)
        cudaStreamDestroy(st);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return P2V_ECUDA;
    }
    return io_ok ? P2V_OK : P2V_EINVAL;
}

}  // namespace

extern "C" p2v_status p2v_write_datraw(p2v_ctx* ctx, const char* prefix, uint32_t frame, uint32_t frame_count,
                                       const p2v_volume* vol) {
    // DatRawWriter::run (:58-105): a file prefix (not a bare directory), an available frame
    if (!prefix || !vol || prefix[0] == '\0')
        return P2V_EINVAL;
    const std::string pre(prefix);
    if (pre.back() == '/')
        return P2V_EINVAL;
    if (frame_count > 0 && frame >= frame_count)
        return P2V_EINVAL;
    const float* data = vol->data;
    int32_t mem = vol->mem;
    if (data == nullptr) {  // the context's device grid of the last frame
        uint64_t r[3];
        if (!ctx || p2v_get_device_volume(ctx, &data, r) != P2V_OK)
            return P2V_EINVAL;
        for (int a = 0; a < 3; ++a)
            if (r[a] != vol->resolution[a])
                return P2V_EINVAL;
        mem = P2V_MEM_DEVICE;
    }
    if (mem != P2V_MEM_HOST && mem != P2V_MEM_DEVICE)
        return P2V_EINVAL;
    const uint64_t comps = vol->components ? vol->components : 1;
    const uint64_t floats = vol->resolution[0] * vol->resolution[1] * vol->resolution[2] * comps;
    if (vol->data && vol->capacity < floats)
        return P2V_EINVAL;
    // <prefix><frame as 4 digits, zero filled>.dat / .raw (:97-101)
    char num[16];
    std::snprintf(num, sizeof(num), "%04u", frame);
    const std::string datpath = pre + num + ".dat", rawpath = pre + num + ".raw";
    const size_t slash = rawpath.find_last_of("/\\");
    const std::string raw_name = slash == std::string::npos ? rawpath : rawpath.substr(slash + 1);
    p2v_volume v = *vol;
    v.components = comps;
    const std::string text = dat_text(raw_name, v, frame);
    int fd = ::open(datpath.c_str(), O_WRONLY | O_CREAT | O_TRUNC, 0644);
    if (fd < 0)
        return P2V_EINVAL;
    bool ok = write_all(fd, text.data(), text.size());
    ::close(fd);
    if (!ok)
        return P2V_EINVAL;
    fd = ::open(rawpath.c_str(), O_WRONLY | O_CREAT | O_TRUNC, 0644);
    if (fd < 0)
        return P2V_EINVAL;
    p2v_status s = P2V_OK;
    if (mem == P2V_MEM_HOST)
        s = write_all(fd, data, floats * sizeof(float)) ? P2V_OK : P2V_EINVAL;
    else
        s = stream_device(fd, data, floats * sizeof(float));
    if (::close(fd) != 0 && s == P2V_OK)
        s = P2V_EINVAL;
    return s;
}
