// MMPLD reader: MegaMol's particle list file format (plugins/moldyn/src/io/MMPLDDataSource.cpp), host code.
//
// File: "MMPLD\0", uint16 version (100..103), uint32 frame count, float bbox[6], float clipbox[6],
// uint64 frame offsets[frames + 1] (MMPLDDataSource.cpp:386-401). Frame (:64-204): float timestamp
// (version >= 102), uint32 list count, then per list uint8 vertex type, uint8 colour type, a global radius
// (vertex types 1, 3, 4), a global RGBA colour (colour type 0) or an intensity range (colour types 3, 7),
// uint64 count, a float box[6] (version >= 103), count interleaved vertex + colour records, and in version
// 101 a cluster block (uint32 count, uint64 byte size, bytes).
//
// Frames are read with pread, so concurrent reads of different frames of one open file need no lock; the
// parsed lists point into the caller's buffer (host memory, pinned when it comes from p2v_host_alloc).
#include <cuda_runtime.h>

#include <fcntl.h>
#include <sys/stat.h>
#include <unistd.h>

#include <cstdint>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/p2v.h"

struct p2v_mmpld {
    int fd = -1;
    uint32_t version = 0, frames = 0;
    float bbox[6] = {}, clipbox[6] = {};
    std::vector<uint64_t> offsets;  // frames + 1
    uint64_t file_size = 0;
};

namespace {

bool read_at(int fd, void* dst, uint64_t bytes, uint64_t off) {
    uint8_t* d = static_cast<uint8_t*>(dst);
    while (bytes > 0) {
        const ssize_t r = ::pread(fd, d, bytes, static_cast<off_t>(off));
        if (r <= 0)
            return false;
        d += r;
        off += static_cast<uint64_t>(r);
        bytes -= static_cast<uint64_t>(r);
    }
    return true;
}

// MMPLD vertex type -> bytes per vertex (MMPLDDataSource.cpp:95-117); the types share the MegaMol numbering
uint32_t vertex_bytes(uint8_t t) {
    switch (t) {
    case 1: return 12;
    case 2: return 16;
    case 3: return 6;
    case 4: return 24;
    default: return 0;
    }
}

// MMPLD colour type -> (bytes, MegaMol colour type) (MMPLDDataSource.cpp:118-155)
void colour_of(uint8_t t, uint32_t& bytes, int32_t& type) {
    switch (t) {
    case 1: bytes = 3; type = P2V_COLDATA_UINT8_RGB; break;
    case 2: bytes = 4; type = P2V_COLDATA_UINT8_RGBA; break;
    case 3: bytes = 4; type = P2V_COLDATA_FLOAT_I; break;
    case 4: bytes = 12; type = P2V_COLDATA_FLOAT_RGB; break;
    case 5: bytes = 16; type = P2V_COLDATA_FLOAT_RGBA; break;
    case 6: bytes = 8; type = P2V_COLDATA_USHORT_RGBA; break;
    case 7: bytes = 8; type = P2V_COLDATA_DOUBLE_I; break;
    default: bytes = 0; type = P2V_COLDATA_NONE; break;
    }
}

struct Cursor {
    const uint8_t* base;
    uint64_t size, p = 0;
    bool ok = true;
    template<class T>
    T get() {
        T v{};
        if (p + sizeof(T) > size) {
            ok = false;
            return v;
        }
        std::memcpy(&v, base + p, sizeof(T));
        p += sizeof(T);
        return v;
    }
    void skip(uint64_t n) {
        if (n > size - p)
            ok = false;
        else
            p += n;
    }
};

}  // namespace

extern "C" {

p2v_status p2v_mmpld_open(const char* path, p2v_mmpld** out, p2v_mmpld_info* info) {
    if (!path || !out)
        return P2V_EINVAL;
    *out = nullptr;
    const int fd = ::open(path, O_RDONLY);
    if (fd < 0)
        return P2V_EINVAL;
    auto* f = new (std::nothrow) p2v_mmpld();
    if (!f) {
        ::close(fd);
        return P2V_ENOMEM;
    }
    f->fd = fd;
    struct stat sb {};
    uint8_t head[6 + 2 + 4 + 24 + 24];
    bool ok = ::fstat(fd, &sb) == 0 && read_at(fd, head, sizeof(head), 0) && std::memcmp(head, "MMPLD", 6) == 0;
    if (ok) {
        f->file_size = static_cast<uint64_t>(sb.st_size);
        uint16_t ver;
        std::memcpy(&ver, head + 6, 2);
        std::memcpy(&f->frames, head + 8, 4);
        std::memcpy(f->bbox, head + 12, 24);
        std::memcpy(f->clipbox, head + 36, 24);
        f->version = ver;
        ok = ver >= 100 && ver <= 103 && f->frames > 0 && f->frames < (1u << 30);
    }
    if (ok) {
        f->offsets.resize((size_t) f->frames + 1);
        ok = read_at(fd, f->offsets.data(), 8ull * (f->frames + 1), sizeof(head));
        const uint64_t data0 = sizeof(head) + 8ull * (f->frames + 1);
        for (uint32_t i = 0; ok && i < f->frames; ++i)
            ok = f->offsets[i] >= data0 && f->offsets[i] <= f->offsets[i + 1] && f->offsets[i + 1] <= f->file_size;
    }
    if (!ok) {
        p2v_mmpld_close(f);
        return P2V_EINVAL;
    }
    if (info) {
        info->version = f->version;
        info->frames = f->frames;
        std::memcpy(info->bbox, f->bbox, sizeof(f->bbox));
        std::memcpy(info->clipbox, f->clipbox, sizeof(f->clipbox));
    }
    *out = f;
    return P2V_OK;
}

void p2v_mmpld_close(p2v_mmpld* f) {
    if (!f)
        return;
    if (f->fd >= 0)
        ::close(f->fd);
    delete f;
}

p2v_status p2v_mmpld_frame_size(p2v_mmpld* f, uint32_t frame, uint64_t* bytes) {
    if (!f || !bytes || frame >= f->frames)
        return P2V_EINVAL;
    *bytes = f->offsets[frame + 1] - f->offsets[frame];
    return P2V_OK;
}

p2v_status p2v_mmpld_read_frame(p2v_mmpld* f, uint32_t frame, void* buffer, uint64_t capacity,
                                p2v_particle_list* lists, p2v_mmpld_list_info* list_info, uint32_t max_lists,
                                uint32_t* nlists, float* timestamp) {
    if (!f || frame >= f->frames || (!buffer && f->offsets[frame + 1] > f->offsets[frame]))
        return P2V_EINVAL;
    const uint64_t size = f->offsets[frame + 1] - f->offsets[frame];
    if (capacity < size)
        return P2V_EINVAL;
    if (size == 0) {  // an empty frame: no lists (MMPLDDataSource.cpp:66-69)
        if (nlists)
            *nlists = 0;
        if (timestamp)
            *timestamp = static_cast<float>(frame);
        return P2V_OK;
    }
    if (!read_at(f->fd, buffer, size, f->offsets[frame]))
        return P2V_EINVAL;
    Cursor c{static_cast<const uint8_t*>(buffer), size};
    // a frame before version 1.2 carries no time: the reference uses the frame index (:73-80)
    const float ts = f->version >= 102 ? c.get<float>() : static_cast<float>(frame);
    const uint32_t plc = c.get<uint32_t>();
    for (uint32_t i = 0; c.ok && i < plc; ++i) {
        p2v_particle_list L{};
        p2v_mmpld_list_info li{};
        const uint8_t vt = c.get<uint8_t>();
        const uint8_t ct = c.get<uint8_t>();
        const uint32_t vb = vertex_bytes(vt);
        uint32_t cb = 0;
        int32_t ctype = P2V_COLDATA_NONE;
        if (vb != 0)
            colour_of(ct, cb, ctype);
        const uint32_t stride = vb + cb;
        L.vertex_type = vb ? static_cast<int32_t>(vt) : static_cast<int32_t>(P2V_VERTDATA_NONE);
        L.global_radius = (vt == 1 || vt == 3 || vt == 4) ? c.get<float>() : 0.05f;
        // the raw colour byte decides what follows (:164-177), whatever the vertex type
        L.global_colour[0] = L.global_colour[1] = L.global_colour[2] = 192;
        L.global_colour[3] = 255;
        li.intensity_range[0] = 0.0f;
        li.intensity_range[1] = 1.0f;
        if (ct == 0) {
            const uint32_t rgba = c.get<uint32_t>();
            std::memcpy(L.global_colour, &rgba, 3);
        } else if (ct == 3 || ct == 7) {
            li.intensity_range[0] = c.get<float>();
            li.intensity_range[1] = c.get<float>();
        }
        L.count = c.get<uint64_t>();
        if (f->version >= 103) {
            for (int a = 0; a < 6; ++a)
                li.bbox[a] = c.get<float>();
        } else {
            std::memcpy(li.bbox, f->bbox, sizeof(li.bbox));
        }
        if (!c.ok || (stride && L.count > (size - c.p) / stride)) {
            c.ok = false;
            break;
        }
        L.vertex_stride = stride;
        L.vertex_data = stride ? static_cast<const uint8_t*>(buffer) + c.p : nullptr;
        L.colour_type = ctype;
        L.colour_stride = stride;
        L.colour_data = cb ? static_cast<const uint8_t*>(buffer) + c.p + vb : nullptr;
        L.mem = P2V_MEM_HOST;
        c.skip(stride * L.count);
        if (f->version == 101) {  // cluster infos (:190-202): skipped
            li.clusters = c.get<uint32_t>();
            c.skip(c.get<uint64_t>());
        }
        if (i < max_lists) {
            if (lists)
                lists[i] = L;
            if (list_info)
                list_info[i] = li;
        }
    }
    if (!c.ok)
        return P2V_EINVAL;
    if (nlists)
        *nlists = plc;
    if (timestamp)
        *timestamp = ts;
    return P2V_OK;
}

void* p2v_host_alloc(uint64_t bytes) {
    void* p = nullptr;
    if (cudaMallocHost(&p, bytes) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return p;
}

void p2v_host_free(void* p) {
    if (p)
        cudaFreeHost(p);
}

}  // extern "C"
