// The persistent batch AO of p2v_run_batch: one launch builds every frame's mip pyramid and marches every
// frame's cones, taking work items from a device-side queue.
//
// The queue is a list of segments (BatchSeg): runs of items of one kind (a mip level of a frame in 512-voxel
// items, or a frame's particles in 128-particle items), numbered by tickets in queue order. A block takes the
// next ticket with an atomic add, waits until the segment its item depends on has completed (a mip level
// needs the level below it, a frame's cone march needs its last level), runs the item and adds one to its
// segment's completion count. Every dependency points to an earlier segment, so the item a block waits on
// was taken before by a block that is running: the queue makes progress whether or not every block of the
// grid is resident. Each wait is bounded (a poll budget the host sets); when it runs out the block records
// BATCH_ERR_TIMEOUT, every other block stops at its next ticket or wait, and the host reports P2V_ETIMEOUT.
//
// The items compute with the device functions of the per-frame kernels (mip_level_kernel, cone_ao_kernel,
// gradient_normals_kernel): the same operations in the same order, so a frame's AO has the bits it has
// from p2v_run_frame. Mip levels written by this launch are read with plain (coherent) loads; the density
// grid, written before the launch, through the read-only path.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "ao_internal.h"
#include "cone_march.cuh"
#include "p2v_common.cuh"

namespace p2v {

namespace {

__device__ __forceinline__ uint32_t ld_acquire_gpu(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ uint32_t ld_volatile(const uint32_t* p) {
    return *reinterpret_cast<const volatile uint32_t*>(p);
}

__global__ void __launch_bounds__(BATCH_AO_ITEM) batch_ao_kernel(const BatchQueueArgs q) {
    __shared__ BatchAoFrame s_f;
    __shared__ uint32_t s_ticket, s_seg;
    uint32_t* const next = q.words;
    uint32_t* const err = q.words + 1;
    uint32_t* const done = q.words + 2;
    int cur = -1;  // the frame held in s_f
    for (;;) {
        if (threadIdx.x == 0) {
            uint32_t t = atomicAdd(next, 1u);
            uint32_t sg = 0;
            if (t >= q.total || ld_volatile(err) != 0) {
                t = ~0u;
            } else {
                uint32_t lo = 0, hi = q.nseg - 1;  // the last segment starting at or before t
                while (lo < hi) {
                    const uint32_t mid = (lo + hi + 1) >> 1;
                    if (q.segs[mid].first <= t)
                        lo = mid;
                    else
                        hi = mid - 1;
                }
                sg = lo;
                const int dep = q.segs[sg].dep;
                if (dep >= 0) {
                    const uint32_t need = q.segs[dep].count;
                    uint32_t polls = 0;
                    while (ld_acquire_gpu(done + dep) < need) {
                        if (ld_volatile(err) != 0 || ++polls > q.wait_polls) {
                            atomicCAS(err, 0u, BATCH_ERR_TIMEOUT);
                            t = ~0u;
                            break;
                        }
                        __nanosleep(128);
                    }
                }
            }
            s_ticket = t;
            s_seg = sg;
        }
        __syncthreads();
        const uint32_t t = s_ticket, sg = s_seg;
        if (t == ~0u)
            break;
        const BatchSeg S = q.segs[sg];
        if ((int) S.frame != cur) {
            const int4* src = reinterpret_cast<const int4*>(q.frames + S.frame);
            int4* dst = reinterpret_cast<int4*>(&s_f);
            for (uint32_t i = threadIdx.x; i < sizeof(BatchAoFrame) / 16; i += blockDim.x)
                dst[i] = __ldg(src + i);
            __syncthreads();
            cur = (int) S.frame;
        }
        const uint32_t k = t - S.first;
        if (S.kind == BSEG_MIP) {
            const ConeLevel& sl = s_f.cp.lv[S.level - 1];
            const ConeLevel& dl = s_f.cp.lv[S.level];
            float* out = const_cast<float*>(dl.v);
            const int64_t nv = (int64_t) dl.d[0] * dl.d[1] * dl.d[2];
            const int64_t end = std::min<int64_t>(nv, (int64_t) (k + 1) * BATCH_MIP_ITEM);
            for (int64_t i = (int64_t) k * BATCH_MIP_ITEM + threadIdx.x; i < end; i += blockDim.x) {
                const int x = (int) (i % dl.d[0]);
                const int y = (int) ((i / dl.d[0]) % dl.d[1]);
                const int z = (int) (i / ((int64_t) dl.d[0] * dl.d[1]));
                out[i] = S.level == 1 ? mip_voxel<true>(sl.v, sl.d[0], sl.d[1], sl.d[2], x, y, z, s_f.cp.sat, 0)
                                      : mip_voxel<false>(sl.v, sl.d[0], sl.d[1], sl.d[2], x, y, z, 0.0f, 0);
            }
        } else {
            const uint32_t j = k * BATCH_AO_ITEM + threadIdx.x;
            if (j < s_f.n) {
                const float4 p = __ldg(s_f.xyzr + j);
                const float4 nv = s_f.nrm ? __ldg(s_f.nrm + j) : gradient_normal<true>(s_f.g, s_f.grid, p);
                s_f.ao[__ldg(s_f.order + j)] = cone_ao_at<false>(s_f.cp, p, nv);
            }
        }
        __syncthreads();  // every thread's results are written
        if (threadIdx.x == 0 && (int32_t) sg != q.hold_seg) {
            __threadfence();
            atomicAdd(done + sg, 1u);
        }
    }
}

}  // namespace

cudaError_t launch_batch_ao(const BatchQueueArgs& q, int sms, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(q.words, 0, sizeof(uint32_t) * batch_queue_words(q.nseg), st);
    if (e != cudaSuccess || q.total == 0)
        return e;
    static int per_sm = 0;
    if (per_sm == 0) {
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch_ao_kernel, BATCH_AO_ITEM, 0);
        if (e != cudaSuccess)
            return e;
        per_sm = std::max(per_sm, 1);
    }
    const uint32_t grid = (uint32_t) std::min<uint64_t>((uint64_t) sms * per_sm, q.total);
    batch_ao_kernel<<<grid, BATCH_AO_ITEM, 0, st>>>(q);
    return cudaGetLastError();
}

}  // namespace p2v
