// trace.cu — k_trace_closest: closest hits for a batch of rays
// (KDTree::intersect / Scene::intersect, kdtree.cpp:349-353, scene.cpp:102-113).
//
// Persistent warps (the loop of wr_warp_trace.cuh): the grid is sized to fill
// every SM once; lanes refill from a global ray counter.  Per-thread
// traversal stacks live in shared memory, column-major (entry k of thread t
// at k * blockDim.x + t) so a warp's pushes hit 32 distinct banks.
#include <cuda_runtime.h>

#include <algorithm>

#include "../../include/walkray.h"
#include "trace_launch.h"
#include "wr_warp_trace.cuh"

namespace wr {

// rays from a (n x 6) array, hits to wr_hit records
struct BatchSrc {
    const DevTree& T;
    const float* __restrict__ rays;
    const int32_t* __restrict__ inside;
    const int32_t* __restrict__ contact;
    wr_hit* __restrict__ hits;
    bool filtered;

    __device__ __forceinline__ void load(uint64_t id, TraceLane& L, uint32_t* stack, int stride) {
        const float* r = rays + 6 * id;
        L.pairs = T.pairs;
        L.tris = T.tris;
        L.q = make_rayq(mk(r[0], r[1], r[2]), mk(r[3], r[4], r[5]), T.scene_mag);
        L.filt = filtered;
        L.inside = filtered ? inside[id] : -1;
        L.contact = filtered ? contact[id] : -1;
        lane_start(L, root_box(T), T.root_w0, T.root_w1, stack, stride);
    }
    __device__ __forceinline__ void store(uint64_t id, const TraceLane& L) {
        uint4 out = make_uint4(WR_NO_HIT, __float_as_uint(-1.f), 0u, 0u);
        if (L.h.slot >= 0) {
            float u1, u2;
            uint32_t gid;
            hit_barycentrics(T, L.h.slot, L.q, L.h.t, &u1, &u2, &gid);
            out = make_uint4(gid, __float_as_uint(L.h.t), __float_as_uint(u1), __float_as_uint(u2));
        }
        reinterpret_cast<uint4*>(hits)[id] = out;
    }
};

// MINB > 0: compiled for at least MINB resident CTAs per SM (a register cap)
template <bool PRUNE, int MINB>
__global__ void __launch_bounds__(128, MINB > 0 ? MINB : 1) k_trace_closest(DevTree T, const float* __restrict__ rays, uint64_t n,
                                                         const int32_t* __restrict__ inside,
                                                         const int32_t* __restrict__ contact, wr_hit* __restrict__ hits,
                                                         unsigned long long* __restrict__ counter, int stack_cap,
                                                         TraceTune tune, unsigned int* __restrict__ err) {
    extern __shared__ uint32_t s_stack[];
    BatchSrc src{T, rays, inside, contact, hits, inside != nullptr};
    warp_trace<PRUNE, false>(src, n, counter, tune, s_stack + threadIdx.x, blockDim.x, stack_cap, err);
}

cudaError_t launch_trace_closest(const DevTree& T, const float* d_rays, uint64_t n, const int32_t* d_inside,
                                 const int32_t* d_contact, wr_hit* d_hits, unsigned long long* d_counter,
                                 unsigned int* d_err, int num_sms, bool prune, cudaStream_t stream,
                                 int* launched_blocks, const TraceTune* tune, int ctas_per_sm) {
    const int block = 128;
    const int stack_cap = (int)T.max_depth + 3;
    const size_t smem = (size_t)stack_cap * block * sizeof(uint32_t);
    if (smem > 200 * 1024) return cudaErrorInvalidValue;
    cudaError_t e = cudaMemsetAsync(d_counter, 0, sizeof(unsigned long long), stream);
    if (e != cudaSuccess) return e;
    // blocks per SM from the occupancy calculator for this stack size
    int per_sm = 1;
    // default: the 7-CTA variant (72 registers), fastest on the kd workload (six steps per
    // turn: 4810 Mrays/s against 4691 with 8 CTAs and 4775 with 6)
    const int variant = ctas_per_sm ? ctas_per_sm : 7;
    void (*kern)(DevTree, const float*, uint64_t, const int32_t*, const int32_t*, wr_hit*, unsigned long long*, int,
                 TraceTune, unsigned int*) =
        variant >= 8   ? (prune ? k_trace_closest<true, 8> : k_trace_closest<false, 8>)
        : variant >= 7 ? (prune ? k_trace_closest<true, 7> : k_trace_closest<false, 7>)
        : variant >= 6 ? (prune ? k_trace_closest<true, 6> : k_trace_closest<false, 6>)
                           : (prune ? k_trace_closest<true, 0> : k_trace_closest<false, 0>);
    if (smem > 48 * 1024) {
        e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, block, smem);
    if (e != cudaSuccess) return e;
    if (ctas_per_sm > 0) per_sm = std::min(per_sm, ctas_per_sm);
    if (per_sm < 1) per_sm = 1;
    uint64_t need_blocks = (n + block - 1) / block;
    int grid = num_sms * per_sm;
    if ((uint64_t)grid > need_blocks) grid = (int)(need_blocks ? need_blocks : 1);
    if (launched_blocks) *launched_blocks = grid;
    const TraceTune tt = tune ? *tune : default_trace_tune();
    kern<<<grid, block, smem, stream>>>(T, d_rays, n, d_inside, d_contact, d_hits, d_counter, stack_cap, tt, d_err);
    return cudaGetLastError();
}

}  // namespace wr
