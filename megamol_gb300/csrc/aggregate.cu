// The intensity and vector aggregators of ParticlesToDensity (aggregator 1 = IColToSingleCell_Volume,
// 2 = IVecToSingleCell_Volume; ParticlesToDensity.cpp:490-519, 628-682): per-particle weights, their
// sorted copy for the weighted gather, and the vector volume's finish.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "../../include/p2v.h"
#include "p2v_common.cuh"
#include "p2v_internal.h"

namespace p2v {
namespace {

template<class T>
__device__ __forceinline__ T load_any(const uint8_t* p) {
    T v;
    uint8_t* d = reinterpret_cast<uint8_t*>(&v);
#pragma unroll
    for (int i = 0; i < (int) sizeof(T); ++i)
        d[i] = p[i];
    return v;
}

// The first colour channel as the reference's GetCRAcc()->Get_f reads it (SimpleSphericalParticles.h:
// 124-175, Accessor.h): a static_cast<float> of the stored value; the global colour (COLDATA_NONE) is the
// normalised unsigned char r / 255.
__device__ __forceinline__ float intensity_of(const uint8_t* rec, int ctype, float global_i) {
    switch (ctype) {
    case P2V_COLDATA_UINT8_RGB:
    case P2V_COLDATA_UINT8_RGBA: return static_cast<float>(rec[0]);
    case P2V_COLDATA_FLOAT_RGB:
    case P2V_COLDATA_FLOAT_RGBA:
    case P2V_COLDATA_FLOAT_I: return load_any<float>(rec);
    case P2V_COLDATA_USHORT_RGBA: return static_cast<float>(load_any<uint16_t>(rec));
    case P2V_COLDATA_DOUBLE_I: return static_cast<float>(load_any<double>(rec));
    default: return global_i;
    }
}

// Weights of one list into w (input order): NC = 1 the intensity, NC = 3 the direction (DIRDATA_FLOAT_XYZ).
// Non-finite weights count as 0. The largest |w| of the frame goes to fs->wmax_bits.
template<int NC>
__global__ void __launch_bounds__(256) pack_weights_kernel(WeightSource src, float* __restrict__ w,
                                                           FrameScalars* __restrict__ fs) {
    __shared__ uint32_t s_max[8];
    uint32_t mbits = 0u;
    const uint64_t step = (uint64_t) gridDim.x * blockDim.x;
    for (uint64_t i = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; i < src.count; i += step) {
        float v[NC];
        if (NC == 1) {
            v[0] = src.data ? intensity_of(src.data + i * src.stride, src.ctype, src.global_i) : src.global_i;
        } else {
            const uint8_t* r = src.data + i * src.stride;
#pragma unroll
            for (int c = 0; c < NC; ++c)
                v[c] = load_any<float>(r + 4 * c);
        }
#pragma unroll
        for (int c = 0; c < NC; ++c) {
            if (!isfinite(v[c]))
                v[c] = 0.0f;
            w[(src.offset + i) * NC + c] = v[c];
            mbits = max(mbits, __float_as_uint(fabsf(v[c])));
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        mbits = max(mbits, __shfl_xor_sync(0xffffffffu, mbits, o));
    if ((threadIdx.x & 31) == 0)
        s_max[threadIdx.x >> 5] = mbits;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < (int) (blockDim.x >> 5); ++k)
            mbits = max(mbits, s_max[k]);
        if (mbits)
            atomicMax(&fs->wmax_bits, mbits);
    }
}

__global__ void __launch_bounds__(256) permute_weights_kernel(const uint32_t* __restrict__ order,
                                                              const float* __restrict__ win, float* __restrict__ wout,
                                                              uint32_t n, int nc) {
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        const uint32_t o = order[j];
        for (int c = 0; c < nc; ++c)
            wout[(size_t) j * nc + c] = win[(size_t) o * nc + c];
    }
}

// ParticlesToDensity.cpp:628-652 per voxel: v /= (w == 0 ? 1 : w); density = sqrt(x*x + y*y + z*z), in
// float without contraction; the density range (max starting at 0, min at FLT_MAX) by atomics on the bits
// of the non-negative densities. With the grid buffers also the density, the unit direction v / density
// (0 where the density is 0), the descending sort key and the count of non-zero densities.
__global__ void __launch_bounds__(256) vector_finish_kernel(float* __restrict__ vol3, const float* __restrict__ wsum,
                                                            int64_t V, FrameScalars* __restrict__ fs,
                                                            VectorGridBufs vg) {
    __shared__ uint32_t s_lo[8], s_hi[8], s_nz[8];
    uint32_t lo = 0x7f7fffffu, hi = 0u, nz = 0u;
    for (int64_t i = blockIdx.x * (int64_t) blockDim.x + threadIdx.x; i < V; i += (int64_t) gridDim.x * blockDim.x) {
        const float wv = wsum[i] == 0.0f ? 1.0f : wsum[i];
        float v[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            v[c] = __fdiv_rn(vol3[i * 3 + c], wv);
            vol3[i * 3 + c] = v[c];
        }
        const float d =
            __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(v[0], v[0]), __fmul_rn(v[1], v[1])), __fmul_rn(v[2], v[2])));
        if (d == d) {
            lo = min(lo, __float_as_uint(d));
            hi = max(hi, __float_as_uint(d));
        }
        if (vg.dens) {
            vg.dens[i] = d;
#pragma unroll
            for (int c = 0; c < 3; ++c)
                vg.dirs[i * 3 + c] = d == 0.0f ? 0.0f : __fdiv_rn(v[c], d);
            vg.keys[i] = ~__float_as_uint(d);
            vg.vals[i] = (uint32_t) i;
            nz += d != 0.0f ? 1u : 0u;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
        nz += __shfl_xor_sync(0xffffffffu, nz, o);
    }
    if ((threadIdx.x & 31) == 0) {
        s_lo[threadIdx.x >> 5] = lo;
        s_hi[threadIdx.x >> 5] = hi;
        s_nz[threadIdx.x >> 5] = nz;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < (int) (blockDim.x >> 5); ++k) {
            lo = min(lo, s_lo[k]);
            hi = max(hi, s_hi[k]);
            nz += s_nz[k];
        }
        atomicMin(&fs->dmin_bits, lo);
        atomicMax(&fs->dmax_bits, hi);
        if (nz)
            atomicAdd(&fs->vcount, nz);
    }
}

// ParticlesToDensity.cpp:436-456, 653-668, 685-727: entry j of the sorted, compacted grid. The node position
// is min + h * index, the colour (density - min) / (max - min) with the densities' range, the info row the
// position, the direction and the colour when normalising, else the density.
__global__ void __launch_bounds__(256) vector_grid_kernel(const uint32_t* __restrict__ order,
                                                          const float* __restrict__ dens,
                                                          const float* __restrict__ dirs,
                                                          const FrameScalars* __restrict__ fs, VectorGridGeo geo,
                                                          uint32_t count, float* __restrict__ pos,
                                                          float* __restrict__ dir, float* __restrict__ col,
                                                          float* __restrict__ info) {
    const float mn = __uint_as_float(fs->dmin_bits), mx = __uint_as_float(fs->dmax_bits);
    const float range = __fsub_rn(mx, mn);
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < count; j += gridDim.x * blockDim.x) {
        const uint32_t idx = order[j];
        const uint32_t sx = (uint32_t) geo.res[0], sy = (uint32_t) geo.res[1];
        const uint32_t xyz[3] = {idx % sx, (idx / sx) % sy, idx / (sx * sy)};
        float p[3], u[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            p[a] = __fadd_rn(geo.minf[a], __fmul_rn(geo.hf[a], static_cast<float>(xyz[a])));
            u[a] = dirs[(size_t) idx * 3 + a];
        }
        const float d = dens[idx];
        const float c = __fdiv_rn(__fsub_rn(d, mn), range);
        if (pos)
#pragma unroll
            for (int a = 0; a < 3; ++a)
                pos[(size_t) j * 3 + a] = p[a];
        if (dir)
#pragma unroll
            for (int a = 0; a < 3; ++a)
                dir[(size_t) j * 3 + a] = u[a];
        if (col)
            col[j] = c;
        if (info) {
            float* r = info + (size_t) j * 7;
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                r[a] = p[a];
                r[3 + a] = u[a];
            }
            r[6] = geo.normalize ? c : d;
        }
    }
}

// ParticlesToDensity.cpp:669-682 with the densities' range: every component maps by (a - min) * (1 /
// (max - min)) when normalising; the published range is the densities'.
__global__ void vector_range_kernel(FrameScalars* fs, int minmax_normalize) {
    const float mn = __uint_as_float(fs->dmin_bits), mx = __uint_as_float(fs->dmax_bits);
    fs->vmin = mn;
    fs->vmax = mx;
    fs->mass_scale = 1.0;
    if (minmax_normalize) {
        fs->offset = mn;
        fs->scale = 1.0f / (mx - mn);
        fs->out_min = 0.0f;
        fs->out_max = 1.0f;
    } else {
        fs->offset = 0.0f;
        fs->scale = 1.0f;
        fs->out_min = mn;
        fs->out_max = mx;
    }
}

}  // namespace

cudaError_t launch_pack_weights(const WeightSource& src, int nc, float* w, FrameScalars* fs, int sms, cudaStream_t st) {
    if (src.count == 0)
        return cudaSuccess;
    const unsigned grd = (unsigned) std::max<uint64_t>(1, std::min<uint64_t>((src.count + 1023) / 1024, (uint64_t) sms * 8));
    if (nc == 1)
        pack_weights_kernel<1><<<grd, 256, 0, st>>>(src, w, fs);
    else
        pack_weights_kernel<3><<<grd, 256, 0, st>>>(src, w, fs);
    return cudaGetLastError();
}

cudaError_t launch_permute_weights(const uint32_t* order, const float* win, float* wout, uint32_t n, int nc, int sms,
                                   cudaStream_t st) {
    if (n == 0)
        return cudaSuccess;
    const unsigned grd = (unsigned) std::max<uint32_t>(1, std::min<uint32_t>(ceil_div(n, 256), (uint32_t) sms * 16));
    permute_weights_kernel<<<grd, 256, 0, st>>>(order, win, wout, n, nc);
    return cudaGetLastError();
}

cudaError_t launch_vector_finish(float* vol3, const float* wsum, int64_t V, FrameScalars* fs, int minmax_normalize,
                                 int sms, cudaStream_t st, const VectorGridBufs* vg) {
    const unsigned grd = (unsigned) std::max<int64_t>(1, std::min<int64_t>((V + 255) / 256, (int64_t) sms * 16));
    vector_finish_kernel<<<grd, 256, 0, st>>>(vol3, wsum, V, fs, vg ? *vg : VectorGridBufs{});
    vector_range_kernel<<<1, 1, 0, st>>>(fs, minmax_normalize);
    return cudaGetLastError();
}

cudaError_t launch_vector_grid(const uint32_t* order, const float* dens, const float* dirs, const FrameScalars* fs,
                               const VectorGridGeo& geo, uint32_t count, float* pos, float* dir, float* col, float* info,
                               int sms, cudaStream_t st) {
    if (count == 0)
        return cudaSuccess;
    const unsigned grd = (unsigned) std::max<uint32_t>(1, std::min<uint32_t>(ceil_div(count, 256), (uint32_t) sms * 16));
    vector_grid_kernel<<<grd, 256, 0, st>>>(order, dens, dirs, fs, geo, count, pos, dir, col, info);
    return cudaGetLastError();
}

}  // namespace p2v
