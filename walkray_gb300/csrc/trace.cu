// trace.cu — k_trace_closest: closest hits for a batch of rays
// (KDTree::intersect / Scene::intersect, kdtree.cpp:349-353, scene.cpp:102-113).
//
// Persistent warps: the grid is sized to fill every SM once; each warp keeps
// its 32 lanes busy by refilling finished lanes from a global ray counter
// (one atomicAdd per warp per refill, lanes ranked with __ballot_sync).
// Per-thread traversal stacks live in shared memory, column-major
// (entry k of thread t at k * blockDim.x + t) so a warp's pushes hit 32
// distinct banks.
#include <cuda_runtime.h>

#include "../../include/walkray.h"
#include "trace_launch.h"
#include "wr_traverse.cuh"

namespace wr {

constexpr int TRACE_STEPS = 8;  // traversal steps between refill checks

template <bool FILTERED, bool PRUNE>
__global__ void __launch_bounds__(256) k_trace_closest(DevTree T, const float* __restrict__ rays, uint64_t n,
                                                         const int32_t* __restrict__ inside,
                                                         const int32_t* __restrict__ contact, wr_hit* __restrict__ hits,
                                                         unsigned long long* __restrict__ counter, int stack_cap,
                                                         unsigned int* __restrict__ err) {
    extern __shared__ uint32_t s_stack[];
    uint32_t* stack = s_stack + threadIdx.x;
    const int stride = blockDim.x;
    const unsigned lane = threadIdx.x & 31u;
    const unsigned lt_mask = (1u << lane) - 1u;

    bool active = false, exhausted = false;
    uint64_t ray_id = 0;
    RayQ q;
    int in_obj = -1, ct_obj = -1;
    Hit h;
    int sp = 0;

    for (;;) {
        const unsigned need = __ballot_sync(0xffffffffu, !active && !exhausted);
        if (need) {
            const int leader = __ffs(need) - 1;
            unsigned long long base = 0;
            if ((int)lane == leader) base = atomicAdd(counter, (unsigned long long)__popc(need));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (!active && !exhausted) {
                const uint64_t id = base + __popc(need & lt_mask);
                if (id < n) {
                    ray_id = id;
                    const float* r = rays + 6 * id;
                    q = make_rayq(mk(r[0], r[1], r[2]), mk(r[3], r[4], r[5]), T.scene_mag);
                    if (FILTERED) {
                        in_obj = inside[id];
                        ct_obj = contact[id];
                    }
                    h.t = __int_as_float(0x7f800000);
                    h.slot = -1;
                    sp = 0;
                    float tn;
                    if (box_pred(root_box(T), q, &tn)) {
                        if (T.root_w1 & LEAF_FLAG)
                            leaf_test<FILTERED>(T, T.root_w0, T.root_w1 & ~LEAF_FLAG, q, in_obj, ct_obj, h);
                        else
                            stack[(sp++) * stride] = T.root_w0;
                    }
                    active = true;
                } else {
                    exhausted = true;
                }
            }
        }
        if (__all_sync(0xffffffffu, !active)) break;
        if (active) {
            for (int it = 0; it < TRACE_STEPS && sp > 0; ++it) {
                const uint32_t pi = stack[(--sp) * stride];
                const NodePair* P = T.pairs + pi;
                const float4 A = ldg4(&P->a), B = ldg4(&P->b), C = ldg4(&P->c);
                const uint4 W = ldg4u(&P->t);
                float tl, tr;
                bool hl = box_pred(Box{A.x, A.y, A.z, A.w, B.x, B.y}, q, &tl);
                bool hr = box_pred(Box{B.z, B.w, C.x, C.y, C.z, C.w}, q, &tr);
                if (PRUNE) {
                    const float lim = h.t * q.pf + q.M;
                    hl = hl && !(tl > lim);
                    hr = hr && !(tr > lim);
                }
                if (hl && (W.y & LEAF_FLAG)) {
                    leaf_test<FILTERED>(T, W.x, W.y & ~LEAF_FLAG, q, in_obj, ct_obj, h);
                    hl = false;
                }
                if (hr && (W.w & LEAF_FLAG)) {
                    leaf_test<FILTERED>(T, W.z, W.w & ~LEAF_FLAG, q, in_obj, ct_obj, h);
                    hr = false;
                }
                if (sp + 2 > stack_cap) {  // cannot happen for a correctly sized stack; never write past it
                    atomicOr(err, 1u);
                    sp = 0;
                    break;
                }
                if (hl && hr) {
                    const bool lnear = tl <= tr;
                    stack[(sp++) * stride] = lnear ? W.z : W.x;
                    stack[(sp++) * stride] = lnear ? W.x : W.z;
                } else if (hl) {
                    stack[(sp++) * stride] = W.x;
                } else if (hr) {
                    stack[(sp++) * stride] = W.z;
                }
            }
            if (sp == 0) {
                wr_hit out;
                if (h.slot >= 0) {
                    float u1, u2;
                    uint32_t gid;
                    hit_barycentrics(T, h.slot, q, h.t, &u1, &u2, &gid);
                    out.tri = gid;
                    out.t = h.t;
                    out.b1 = u1;
                    out.b2 = u2;
                } else {
                    out.tri = WR_NO_HIT;
                    out.t = -1.f;
                    out.b1 = 0.f;
                    out.b2 = 0.f;
                }
                reinterpret_cast<uint4*>(hits)[ray_id] =
                    make_uint4(out.tri, __float_as_uint(out.t), __float_as_uint(out.b1), __float_as_uint(out.b2));
                active = false;
            }
        }
    }
}

cudaError_t launch_trace_closest(const DevTree& T, const float* d_rays, uint64_t n, const int32_t* d_inside,
                                 const int32_t* d_contact, wr_hit* d_hits, unsigned long long* d_counter,
                                 unsigned int* d_err, int num_sms, bool prune, cudaStream_t stream,
                                 int* launched_blocks) {
    const int block = 128;
    const int stack_cap = (int)T.max_depth + 3;
    const size_t smem = (size_t)stack_cap * block * sizeof(uint32_t);
    if (smem > 200 * 1024) return cudaErrorInvalidValue;
    cudaError_t e = cudaMemsetAsync(d_counter, 0, sizeof(unsigned long long), stream);
    if (e != cudaSuccess) return e;
    // blocks per SM from the occupancy calculator for this stack size
    int per_sm = 1;
    const bool filtered = d_inside != nullptr;
    void (*kern)(DevTree, const float*, uint64_t, const int32_t*, const int32_t*, wr_hit*, unsigned long long*, int,
                 unsigned int*) = filtered ? (prune ? k_trace_closest<true, true> : k_trace_closest<true, false>)
                                           : (prune ? k_trace_closest<false, true> : k_trace_closest<false, false>);
    if (smem > 48 * 1024) {
        e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, block, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    uint64_t need_blocks = (n + block - 1) / block;
    int grid = num_sms * per_sm;
    if ((uint64_t)grid > need_blocks) grid = (int)(need_blocks ? need_blocks : 1);
    if (launched_blocks) *launched_blocks = grid;
    kern<<<grid, block, smem, stream>>>(T, d_rays, n, d_inside, d_contact, d_hits, d_counter, stack_cap, d_err);
    return cudaGetLastError();
}

}  // namespace wr
