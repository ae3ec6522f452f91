// wavefront.cu — kernels and driver of the wavefront renderer (see
// wavefront.h for the stage structure).
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstring>
#include <map>

#include "wavefront.h"
#include "wr_warp_trace.cuh"

namespace wr {

constexpr uint32_t WF_MAX_JOBS = 256;
constexpr uint32_t WF_MAX_SCENES = 64;

uint32_t wf_max_jobs() { return WF_MAX_JOBS; }

// ---------------------------------------------------------------------------
// state load / store
// ---------------------------------------------------------------------------
struct WfPath {
    PRay cur;
    f3 color, prev_d;
    uint32_t depth;
    InsideStack st;
    uint32_t pixel, sample, dim;
    int job;
    float mis_pdf;  // density of the current ray's scatter (WR_RENDER_NEE_MIS)
    f3 acc;         // light connections counted so far (WR_RENDER_NEE_MIS)
};

__device__ __forceinline__ int4 as_i4(float4 v) {
    return make_int4(__float_as_int(v.x), __float_as_int(v.y), __float_as_int(v.z), __float_as_int(v.w));
}
__device__ __forceinline__ float4 as_f4(int4 v) {
    return make_float4(__int_as_float(v.x), __int_as_float(v.y), __int_as_float(v.z), __int_as_float(v.w));
}

__device__ __forceinline__ void wf_load(const WfSide& X, uint32_t i, WfPath& p) {
    const float4* r = X.rec + (size_t)WF_REC * i;
    const float4 a0 = r[WF_O], a1 = r[WF_D], a2 = r[WF_RAD], a3 = r[WF_COL];
    const int4 ids = as_i4(r[WF_IDS]), misc = as_i4(r[WF_MISC]), stk = as_i4(r[WF_STK]);
    p.cur = ray_default();
    p.cur.o = mk(a0.x, a0.y, a0.z);
    p.cur.oP = a0.w;
    p.cur.d = mk(a1.x, a1.y, a1.z);
    p.cur.dP = a1.w;
    p.cur.rad = mk(a2.x, a2.y, a2.z);
    p.cur.cnorm = mk(a2.w, a3.w, __int_as_float(misc.w));
    p.color = mk(a3.x, a3.y, a3.z);
    p.cur.inside = ids.x;
    p.cur.contact = ids.y;
    p.job = ids.z;
    p.pixel = (uint32_t)ids.w;
    p.sample = (uint32_t)misc.x;
    p.dim = (uint32_t)misc.y;
    p.depth = (uint32_t)misc.z & 0xffffu;
    p.st.n = (int)((uint32_t)misc.z >> 16);
    p.st.v0 = stk.x;
    p.st.v1 = stk.y;
    p.st.v2 = stk.z;
    p.st.v3 = stk.w;
    const float4 a4 = r[WF_PREV];
    p.prev_d = mk(a4.x, a4.y, a4.z);
    p.mis_pdf = a4.w;
    p.acc = mk(0, 0, 0);
}

__device__ __forceinline__ void wf_load_acc(const WfSide& X, uint32_t i, WfPath& p) {
    const float4 a5 = X.a5[i];
    p.acc = mk(a5.x, a5.y, a5.z);
}

__device__ __forceinline__ void wf_store(const WfSide& Y, uint32_t j, const WfPath& p) {
    float4* r = Y.rec + (size_t)WF_REC * j;
    r[WF_O] = make_float4(p.cur.o.x, p.cur.o.y, p.cur.o.z, p.cur.oP);
    r[WF_D] = make_float4(p.cur.d.x, p.cur.d.y, p.cur.d.z, p.cur.dP);
    r[WF_IDS] = as_f4(make_int4(p.cur.inside, p.cur.contact, p.job, (int)p.pixel));
    r[WF_MISC] = as_f4(make_int4((int)p.sample, (int)p.dim, (int)(p.depth | ((uint32_t)p.st.n << 16)),
                                 __float_as_int(p.cur.cnorm.z)));
    r[WF_RAD] = make_float4(p.cur.rad.x, p.cur.rad.y, p.cur.rad.z, p.cur.cnorm.x);
    r[WF_COL] = make_float4(p.color.x, p.color.y, p.color.z, p.cur.cnorm.y);
    r[WF_STK] = as_f4(make_int4(p.st.v0, p.st.v1, p.st.v2, p.st.v3));
    r[WF_PREV] = make_float4(p.prev_d.x, p.prev_d.y, p.prev_d.z, p.mis_pdf);
}

// The same record written into row `row` of a shared-memory tile of 128-byte
// rows in the 128-byte swizzle of the tensor-memory-access unit (16-byte
// chunk c of row r at chunk c ^ (r & 7)): eight consecutive rows' stores of
// one field then fall on eight different bank groups, and the bulk tensor
// store writes the rows to global memory unswizzled.
__device__ __forceinline__ void wf_store_tile(float4* tile, uint32_t row, const WfPath& p) {
    float4* r = tile + (size_t)WF_REC * row;
    const uint32_t x = row & 7u;
    r[WF_O ^ x] = make_float4(p.cur.o.x, p.cur.o.y, p.cur.o.z, p.cur.oP);
    r[WF_D ^ x] = make_float4(p.cur.d.x, p.cur.d.y, p.cur.d.z, p.cur.dP);
    r[WF_IDS ^ x] = as_f4(make_int4(p.cur.inside, p.cur.contact, p.job, (int)p.pixel));
    r[WF_MISC ^ x] = as_f4(make_int4((int)p.sample, (int)p.dim, (int)(p.depth | ((uint32_t)p.st.n << 16)),
                                     __float_as_int(p.cur.cnorm.z)));
    r[WF_RAD ^ x] = make_float4(p.cur.rad.x, p.cur.rad.y, p.cur.rad.z, p.cur.cnorm.x);
    r[WF_COL ^ x] = make_float4(p.color.x, p.color.y, p.color.z, p.cur.cnorm.y);
    r[WF_STK ^ x] = as_f4(make_int4(p.st.v0, p.st.v1, p.st.v2, p.st.v3));
    r[WF_PREV ^ x] = make_float4(p.prev_d.x, p.prev_d.y, p.prev_d.z, p.mis_pdf);
}

__device__ __forceinline__ void wf_store_acc(const WfSide& Y, uint32_t j, const WfPath& p) {
    Y.a5[j] = make_float4(p.acc.x, p.acc.y, p.acc.z, 0.f);
}

// warp-aggregated append: returns this lane's position (valid if `want`)
__device__ __forceinline__ uint32_t warp_append(unsigned int* counter, bool want, uint32_t offset) {
    const unsigned lane = threadIdx.x & 31u;
    const unsigned m = __ballot_sync(0xffffffffu, want);
    uint32_t base = 0;
    if (m) {
        const int leader = __ffs(m) - 1;
        if ((int)lane == leader) base = atomicAdd(counter, (unsigned)__popc(m));
        base = __shfl_sync(0xffffffffu, base, leader);
    }
    return offset + base + __popc(m & ((1u << lane) - 1u));
}

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------
__global__ void k_wf_reset(WfSide Y, unsigned long long* work, unsigned int* shadow_count, WfSort B) {
    Y.counts[0] = 0;
    Y.counts[1] = 0;
    work[0] = 0;  // the extend stage's ray counter
    work[1] = 0;  // the shadow stage's
    *shadow_count = 0;
    for (int k = 0; k < WF_SORT_KEYS; k++) B.counts[k] = 0;
}

// sort: bucket the queue by shading material (warp-aggregated appends)
__global__ void __launch_bounds__(256) k_wf_sort(const RenderScene* __restrict__ scenes,
                                                   const WfJob* __restrict__ jobs, WfSide X,
                                                   const int2* __restrict__ hits, WfSort B, uint32_t capacity) {
    const uint32_t n = X.counts[0] + X.counts[1];
    const uint32_t step = gridDim.x * blockDim.x;
    const unsigned lane = threadIdx.x & 31u;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += step) {  // warp-uniform trip count
        const uint32_t i = base + threadIdx.x;
        const bool valid = i < n;
        int key = 0;
        if (valid) {
            const int slot = hits[i].x;
            if (slot >= 0) {
                const int4 ids = as_i4(X.rec[(size_t)WF_REC * i + WF_IDS]);
                const RenderScene& S = scenes[jobs[ids.z].scene];
                const int self = ids.x >= 0 ? ids.x : (int)__float_as_uint(__ldg(&S.tree.tris[slot].v1.w));
                key = 1 + (int)obj_type(S, self);
                key = key < WF_SORT_KEYS ? key : WF_SORT_KEYS - 1;
            }
        }
        const unsigned vm = __ballot_sync(0xffffffffu, valid);
        if (valid) {
            const unsigned peers = __match_any_sync(vm, key);
            const int leader = __ffs(peers) - 1;
            unsigned int b = 0;
            if ((int)lane == leader) b = atomicAdd(&B.counts[key], (unsigned)__popc(peers));
            b = __shfl_sync(peers, b, leader);
            B.idx[(size_t)key * capacity + b + __popc(peers & ((1u << lane) - 1u))] = i;
        }
    }
}

// film update of a finished path: isLegalColor, fixVignetting, FP32 atomics
__device__ __forceinline__ void film_add(const WfJob& J, uint32_t pixel, f3 result) {
    if (!legal(result)) result = mk(0, 0, 0);
    const f3 c = fix_vignetting(J.cam, result, pixel);
    float* f = J.film + 3 * (size_t)pixel;
    atomicAdd(f + 0, c.x);
    atomicAdd(f + 1, c.y);
    atomicAdd(f + 2, c.z);
    if (J.film2) {
        float* f2 = J.film2 + 3 * (size_t)pixel;
        atomicAdd(f2 + 0, c.x * c.x);
        atomicAdd(f2 + 1, c.y * c.y);
        atomicAdd(f2 + 2, c.z * c.z);
    }
}

// shadow stage, second half: with the closest hit of every NEE connection
// and light connection (WF_SHADOW_*) from k_wf_shadow_trace, the visible
// contributions go to the film or to their path
__global__ void __launch_bounds__(128) k_wf_shadow(const RenderScene* __restrict__ scenes,
                                                     const WfJob* __restrict__ jobs, WfShadow Q,
                                                     const int2* __restrict__ hits, WfSide Y) {
    const uint32_t n = *Q.count;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 o = Q.o[i], d = Q.d[i], c = Q.c[i];
        const int4 ids = Q.ids[i];
        const WfJob& J = jobs[ids.z];
        const RenderScene& S = scenes[J.scene];
        const int2 hv = hits[i];
        Hit h;
        h.slot = hv.x;
        h.t = __int_as_float(hv.y);
        const int kind = __float_as_int(c.w);
        const f3 contrib = mk(c.x, c.y, c.z);
        if (kind == WF_SHADOW_NEE) {
            if (nee_visible(h, o.w)) film_add(J, (uint32_t)ids.w, contrib);
            continue;
        }
        LightReq lr;
        lr.dist = o.w;
        lr.light = __float_as_int(d.w);
        const bool vis = light_req_visible(S, h, lr);
        const float4 r = Q.r[i];
        if (kind == WF_SHADOW_MIS_KEEP) {
            if (vis) {
                const int t = __float_as_int(r.w);
                float4 a = Y.a5[t];
                a.x += contrib.x;
                a.y += contrib.y;
                a.z += contrib.z;
                Y.a5[t] = a;
            }
        } else {
            f3 tot = mk(r.x, r.y, r.z);
            if (vis) tot = tot + contrib;
            if (tot.x != 0.f || tot.y != 0.f || tot.z != 0.f) film_add(J, (uint32_t)ids.w, tot);
        }
    }
}

// extend: closest hit of every queued ray; the eye ray (contact == camera)
// without a filter, all others with NoSelfCondition.  Rays of different jobs
// (and scenes) share the queue; each lane follows its own ray's tree.
struct ExtendSrc {
    const RenderScene* __restrict__ scenes;
    const WfJob* __restrict__ jobs;
    WfSide X;
    int2* __restrict__ hits;
    unsigned long long n_rays, n_box, n_tri;  // this thread's work counts (profiling launches)

    __device__ __forceinline__ void load(uint64_t id, TraceLane& L, uint32_t* stack, int stride) {
        const float4* r = X.rec + (size_t)WF_REC * id;
        const float4 a0 = r[WF_O], a1 = r[WF_D];
        const int4 ids = as_i4(r[WF_IDS]);
        const WfJob& J = jobs[ids.z];
        const DevTree& T = scenes[J.scene].tree;
        L.pairs = T.pairs;
        L.tris = T.tris;
        L.q = make_rayq(mk(a0.x, a0.y, a0.z), mk(a1.x, a1.y, a1.z), T.scene_mag);
        L.q.pf = prune_factor(J.flags);
        L.inside = ids.x;
        L.contact = ids.y;
        L.filt = ids.y != CAMERA_OBJ;
        const Box root{T.root_lo[0], T.root_lo[1], T.root_lo[2], T.root_hi[0], T.root_hi[1], T.root_hi[2]};
        lane_start(L, root, T.root_w0, T.root_w1, stack, stride);
    }
    __device__ __forceinline__ void store(uint64_t id, const TraceLane& L) {
        hits[id] = make_int2(L.h.slot, __float_as_int(L.h.t));
        n_rays += 1;
        n_box += L.n_box;
        n_tri += L.n_tri;
    }
};

// adds the warp's sum of v to *dst (one atomic per warp)
__device__ __forceinline__ void warp_add(unsigned long long* dst, unsigned long long v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31u) == 0 && v) atomicAdd(dst, v);
}

// MINB > 0: compiled for at least MINB resident CTAs of 128 threads per SM
// (a register cap), chosen by the configuration's ctas_per_sm
#define WR_EXTEND_BOUNDS(MINB) __launch_bounds__(128, (MINB) > 0 ? (MINB) : 1)

template <bool STATS, int MINB>
__global__ void WR_EXTEND_BOUNDS(MINB) k_wf_extend(const RenderScene* __restrict__ scenes,
                                                     const WfJob* __restrict__ jobs, WfSide X, int2* __restrict__ hits,
                                                     unsigned long long* __restrict__ work, int stack_cap,
                                                     TraceTune tune, unsigned int* __restrict__ err,
                                                     unsigned long long* __restrict__ stats) {
    extern __shared__ uint32_t s_stack[];
    const uint64_t n = (uint64_t)X.counts[0] + X.counts[1];
    ExtendSrc src{scenes, jobs, X, hits, 0ull, 0ull, 0ull};
    warp_trace<true, STATS>(src, n, work, tune, s_stack + threadIdx.x, blockDim.x, stack_cap, err);
    if (STATS) {
        warp_add(stats + 0, src.n_rays);
        warp_add(stats + 1, src.n_box);
        warp_add(stats + 2, src.n_tri);
    }
}

using ExtendKernel = void (*)(const RenderScene*, const WfJob*, WfSide, int2*, unsigned long long*, int, TraceTune,
                              unsigned int*, unsigned long long*);

// shadow stage, first half: the closest hit of every connection in the
// shadow queue, through the same warp-persistent loop as extend (filtered by
// the connection's inside / contact objects, as trace_closest<true, true>)
struct ShadowSrc {
    const RenderScene* __restrict__ scenes;
    const WfJob* __restrict__ jobs;
    WfShadow Q;
    int2* __restrict__ hits;

    __device__ __forceinline__ void load(uint64_t id, TraceLane& L, uint32_t* stack, int stride) {
        const float4 o = Q.o[id], d = Q.d[id];
        const int4 ids = Q.ids[id];
        const WfJob& J = jobs[ids.z];
        const DevTree& T = scenes[J.scene].tree;
        L.pairs = T.pairs;
        L.tris = T.tris;
        L.q = make_rayq(mk(o.x, o.y, o.z), mk(d.x, d.y, d.z), T.scene_mag);
        L.q.pf = prune_factor(J.flags);
        L.inside = ids.x;
        L.contact = ids.y;
        L.filt = true;
        const Box root{T.root_lo[0], T.root_lo[1], T.root_lo[2], T.root_hi[0], T.root_hi[1], T.root_hi[2]};
        lane_start(L, root, T.root_w0, T.root_w1, stack, stride);
    }
    __device__ __forceinline__ void store(uint64_t id, const TraceLane& L) {
        hits[id] = make_int2(L.h.slot, __float_as_int(L.h.t));
    }
};

template <int MINB>
__global__ void WR_EXTEND_BOUNDS(MINB)
    k_wf_shadow_trace(const RenderScene* __restrict__ scenes, const WfJob* __restrict__ jobs, WfShadow Q,
                      int2* __restrict__ hits, unsigned long long* __restrict__ work, int stack_cap, TraceTune tune,
                      unsigned int* __restrict__ err) {
    extern __shared__ uint32_t s_stack[];
    const uint64_t n = *Q.count;
    ShadowSrc src{scenes, jobs, Q, hits};
    warp_trace<true, false>(src, n, work, tune, s_stack + threadIdx.x, blockDim.x, stack_cap, err);
}

using ShadowTraceKernel = void (*)(const RenderScene*, const WfJob*, WfShadow, int2*, unsigned long long*, int,
                                   TraceTune, unsigned int*);

// the shadow traversal for a configuration: the extend stage's register cap
static ShadowTraceKernel shadow_trace_kernel(int ctas_per_sm) {
    if (ctas_per_sm == 0) ctas_per_sm = 6;
    if (ctas_per_sm >= 8) return k_wf_shadow_trace<8>;
    if (ctas_per_sm >= 7) return k_wf_shadow_trace<7>;
    if (ctas_per_sm >= 6) return k_wf_shadow_trace<6>;
    return k_wf_shadow_trace<0>;
}

// the extend kernel for a configuration: register cap from ctas_per_sm
// (0 = the 6-CTA variant, fastest on the mixed-material scene)
static ExtendKernel extend_kernel(int ctas_per_sm, bool stats) {
    if (ctas_per_sm == 0) ctas_per_sm = 6;
    if (ctas_per_sm >= 8) return stats ? k_wf_extend<true, 8> : k_wf_extend<false, 8>;
    if (ctas_per_sm >= 7) return stats ? k_wf_extend<true, 7> : k_wf_extend<false, 7>;
    if (ctas_per_sm >= 6) return stats ? k_wf_extend<true, 6> : k_wf_extend<false, 6>;
    return stats ? k_wf_extend<true, 0> : k_wf_extend<false, 0>;
}

// shade: one bounce per path; survivors compacted into Y, finished paths to
// the film.  MIS: compiled with the WR_RENDER_NEE_MIS code (launched while a
// job with that flag is in the table).
template <bool MIS>
__global__ void __launch_bounds__(128, 4) k_wf_shade(const RenderScene* __restrict__ scenes,
                                                    const WfJob* __restrict__ jobs,
                                                    WfJobCounters* __restrict__ counters, WfSide X,
                                                    const int2* __restrict__ hits, WfSide Y, WfShadow Q, WfSort B,
                                                    uint32_t capacity) {
    __shared__ uint32_t s_first[WF_SORT_KEYS + 1];  // first queue position of each bucket
    if (threadIdx.x == 0) {
        uint32_t a = 0;
        for (int k = 0; k < WF_SORT_KEYS; k++) {
            s_first[k] = a;
            a += B.counts[k];
        }
        s_first[WF_SORT_KEYS] = a;
    }
    __syncthreads();
    const uint32_t n = s_first[WF_SORT_KEYS];
    const uint32_t step = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += step) {  // warp-uniform trip count
        const uint32_t j = base + threadIdx.x;
        const bool valid = j < n;
        uint32_t i = 0;
        if (valid) {  // the j-th path in bucket order
            int k = 0;
#pragma unroll
            for (int kk = 1; kk < WF_SORT_KEYS; kk++) k = j >= s_first[kk] ? kk : k;
            i = B.idx[(size_t)k * capacity + (j - s_first[k])];
        }
        WfPath p;
        bool keep = false, done = false, shadow = false, has_lr = false, mis = false;
        f3 result = mk(0, 0, 0);
        ShadowReq sr;
        LightReq lr;
        if (valid) {
            wf_load(X, i, p);
            const WfJob& J = jobs[p.job];
            const RenderScene& S = scenes[J.scene];
            mis = MIS && (J.flags & WR_RENDER_NEE_MIS) != 0;
            if (mis) wf_load_acc(X, i, p);
            const int2 hv = hits[i];
            Hit h;
            h.slot = hv.x;
            h.t = __int_as_float(hv.y);
            const bool nee = (J.flags & WR_RENDER_NEE) != 0;
            bool nee_here = false;
            PathRng g;
            g.init(J.seed, p.pixel, p.sample, p.dim);
            if (h.slot < 0 && p.cur.contact != CAMERA_OBJ) {
                done = true;  // a scattered ray that escapes ends with zero radiance
                nee_here = nee;
            } else {
                set_hit(S, p.cur, h);
                done = path_advance<MIS>(S, p.cur, p.color, p.prev_d, p.depth, p.st, g, J.max_path_len, J.flags,
                                         result, nee_here, p.mis_pdf, lr, has_lr);
            }
            if (nee_here) shadow = nee_prepare(S, p.cur, p.prev_d, p.color, g, sr);
            p.dim = g.dim;
            keep = !done;
            if (done) {
                if (!legal(result)) result = mk(0, 0, 0);
                result = result + p.acc;  // light connections of earlier vertices
                if (!shadow && !has_lr && (result.x != 0.f || result.y != 0.f || result.z != 0.f))
                    film_add(J, p.pixel, result);
            }
        }
        // survivors, compacted into Y
        const uint32_t out = warp_append(&Y.counts[0], keep, 0);
        if (keep) {
            wf_store(Y, out, p);
            if (mis) wf_store_acc(Y, out, p);
        }
        // connections whose visibility the shadow stage decides
        {
            const bool any = shadow || has_lr;
            const uint32_t k = warp_append(Q.count, any, 0);
            if (shadow) {
                Q.o[k] = make_float4(sr.o.x, sr.o.y, sr.o.z, sr.dist);
                Q.d[k] = make_float4(sr.d.x, sr.d.y, sr.d.z, 0.f);
                Q.c[k] = make_float4(sr.contrib.x, sr.contrib.y, sr.contrib.z, __int_as_float(WF_SHADOW_NEE));
                Q.ids[k] = make_int4(sr.inside, sr.contact, p.job, (int)p.pixel);
            } else if (has_lr) {
                Q.o[k] = make_float4(lr.o.x, lr.o.y, lr.o.z, lr.dist);
                Q.d[k] = make_float4(lr.d.x, lr.d.y, lr.d.z, __int_as_float(lr.light));
                Q.c[k] = make_float4(lr.contrib.x, lr.contrib.y, lr.contrib.z,
                                     __int_as_float(keep ? WF_SHADOW_MIS_KEEP : WF_SHADOW_MIS_DONE));
                Q.r[k] = make_float4(result.x, result.y, result.z, __int_as_float((int)out));
                Q.ids[k] = make_int4(lr.inside, lr.contact, p.job, (int)p.pixel);
            }
        }
        // finished-path counts per job, aggregated over the lanes sharing a job
        {
            const unsigned dm = __ballot_sync(0xffffffffu, done);
            if (done) {
                const unsigned same = __match_any_sync(dm, p.job);
                if ((threadIdx.x & 31u) == (unsigned)(__ffs(same) - 1))
                    atomicAdd(&counters[p.job].finished, (unsigned long long)__popc(same));
            }
        }
    }
}

// drain: the last paths of a render, each finished by one thread (trace,
// bounce, NEE connection) without returning to the bounce loop.  Once nothing
// is left to generate, the loop's iterations each cost about the latency of
// their slowest ray however few rays remain; here the remaining paths run
// side by side instead.  Same paths, draws and film additions as the loop.
__global__ void __launch_bounds__(128) k_wf_drain(const RenderScene* __restrict__ scenes,
                                                    const WfJob* __restrict__ jobs,
                                                    WfJobCounters* __restrict__ counters, WfSide X, int stack_cap,
                                                    unsigned int* __restrict__ err) {
    extern __shared__ uint32_t s_stack[];
    uint32_t* stack = s_stack + threadIdx.x;
    const uint32_t n = X.counts[0] + X.counts[1];
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    WfPath p;
    wf_load(X, i, p);
    const WfJob& J = jobs[p.job];
    const RenderScene& S = scenes[J.scene];
    if (J.flags & WR_RENDER_NEE_MIS) wf_load_acc(X, i, p);
    PathRng g;
    g.init(J.seed, p.pixel, p.sample, p.dim);
    const bool nee = (J.flags & WR_RENDER_NEE) != 0;
    const float pf = prune_factor(J.flags);
    bool filtered = p.cur.contact != CAMERA_OBJ, nee_here = false, has_lr = false;
    f3 result = mk(0, 0, 0);
    LightReq lr;
    for (;;) {
        RayQ q = make_rayq(p.cur.o, p.cur.d, S.tree.scene_mag);
        q.pf = pf;
        const Hit h = filtered ? trace_closest<true, true>(S.tree, q, p.cur.inside, p.cur.contact, stack,
                                                           blockDim.x, stack_cap, err)
                               : trace_closest<false, true>(S.tree, q, -1, -1, stack, blockDim.x, stack_cap, err);
        if (h.slot < 0 && filtered) {  // a scattered ray that escapes ends with zero radiance
            nee_here = nee;
            break;
        }
        set_hit(S, p.cur, h);
        filtered = true;
        const bool done = path_advance<true>(S, p.cur, p.color, p.prev_d, p.depth, p.st, g, J.max_path_len,
                                             J.flags, result, nee_here, p.mis_pdf, lr, has_lr);
        if (has_lr) {
            RayQ lq = make_rayq(lr.o, lr.d, S.tree.scene_mag);
            lq.pf = pf;
            const Hit lh = trace_closest<true, true>(S.tree, lq, lr.inside, lr.contact, stack, blockDim.x, stack_cap,
                                                     err);
            if (light_req_visible(S, lh, lr)) p.acc = p.acc + lr.contrib;
        }
        if (done) break;
    }
    if (nee_here) {
        ShadowReq sr;
        result = mk(0, 0, 0);
        if (nee_prepare(S, p.cur, p.prev_d, p.color, g, sr)) {
            RayQ q = make_rayq(sr.o, sr.d, S.tree.scene_mag);
            q.pf = pf;
            const Hit h = trace_closest<true, true>(S.tree, q, sr.inside, sr.contact, stack, blockDim.x, stack_cap, err);
            if (nee_visible(h, sr.dist)) result = sr.contrib;
        }
    }
    if (!legal(result)) result = mk(0, 0, 0);
    result = result + p.acc;
    if (result.x != 0.f || result.y != 0.f || result.z != 0.f) film_add(J, p.pixel, result);
    const unsigned same = __match_any_sync(__activemask(), p.job);
    if ((threadIdx.x & 31u) == (unsigned)(__ffs(same) - 1))
        atomicAdd(&counters[p.job].finished, (unsigned long long)__popc(same));
}

// plan: how the free slots of Y are shared out among the jobs this turn.
// One block, one thread per listed job (`order`: admission order).  Each job
// with paths left gets an equal share of the free slots (processor sharing:
// a small request admitted behind a large one starts at once), capped by what
// it has left; slots nobody's share used go to the jobs in admission order.
// With `equal_share` off, every slot goes in admission order (first come,
// first served).  The queue is filled up to *live_cap paths (at most its
// capacity): a word in device memory, so that the serving loop can shorten
// the queue without recapturing the bounce loop.  The plan reserves each job's index range [first, first +
// quota) by advancing its claim counter; the generate kernel then maps queue
// position t to a job and a path index without atomics.  Which paths a job
// renders does not depend on the plan, only when.
__device__ __forceinline__ unsigned long long block_excl_scan(unsigned long long v, unsigned long long* buf) {
    const int k = threadIdx.x;
    buf[k] = v;
    __syncthreads();
    for (int d = 1; d < (int)blockDim.x; d <<= 1) {
        const unsigned long long add = k >= d ? buf[k - d] : 0ull;
        __syncthreads();
        buf[k] += add;
        __syncthreads();
    }
    const unsigned long long incl = buf[k];
    __syncthreads();
    return incl - v;
}

__global__ void __launch_bounds__(WF_MAX_JOBS) k_wf_plan(const WfJob* __restrict__ jobs, const int* __restrict__ order,
                                                          WfJobCounters* __restrict__ counters, WfSide Y,
                                                          uint32_t capacity, const uint32_t* __restrict__ live_cap,
                                                          int equal_share, WfPlan P) {
    __shared__ unsigned long long buf[WF_MAX_JOBS];
    __shared__ unsigned long long s_total_q;
    const int n = order[0];
    const int k = threadIdx.x;
    const uint32_t survivors = Y.counts[0];
    const uint32_t cap = min(capacity, *live_cap);
    const unsigned long long free_slots = cap > survivors ? cap - survivors : 0u;
    int j = -1;
    unsigned long long rem = 0, claimed = 0;
    if (k < n) {
        j = order[1 + k];
        const WfJob& J = jobs[j];
        claimed = counters[j].claimed;
        rem = (J.active && claimed < J.total) ? J.total - claimed : 0ull;
    }
    const int active = __syncthreads_count(rem > 0);
    const unsigned long long share = (equal_share && active) ? free_slots / (unsigned long long)active : 0ull;
    const unsigned long long q = rem < share ? rem : share;
    const unsigned long long q_before = block_excl_scan(q, buf);
    if (k == (int)blockDim.x - 1) s_total_q = q_before + q;
    __syncthreads();
    const unsigned long long leftover = free_slots - s_total_q;
    unsigned long long need = rem - q;
    need = need < free_slots ? need : free_slots;
    const unsigned long long need_before = block_excl_scan(need, buf);
    unsigned long long extra = leftover > need_before ? leftover - need_before : 0ull;
    extra = extra < need ? extra : need;
    const unsigned long long quota = q + extra;
    const unsigned long long off = block_excl_scan(quota, buf);
    if (k < n) {
        P.slot[k] = j;
        P.first[k] = claimed;
        P.off[k] = (uint32_t)off;
        if (quota) counters[j].claimed = claimed + quota;
    }
    if (k == n - 1 || (n == 0 && k == 0)) {
        const uint32_t total = n ? (uint32_t)(off + quota) : 0u;
        P.off[n] = total;
        *P.n = n;
        Y.counts[1] = total;
    }
}

// Pixel of the k-th camera path of a sample when paths are generated tile by
// tile: bands of `tile` rows, each cut into tiles of `tile` columns (the last
// band and the last tile of a band may be smaller), rows within a tile.  A
// bijection of [0, W*H); tile 0 is row order.  Neighbouring queue entries
// then hold neighbouring pixels, whose first bounces visit the same nodes.
__device__ __forceinline__ uint32_t tile_pixel(uint32_t k, uint32_t W, uint32_t H, uint32_t tile) {
    if (tile == 0 || tile >= W) return k;
    const uint32_t band = k / (W * tile);
    const uint32_t y0 = band * tile;
    const uint32_t bh = min(tile, H - y0);  // rows in this band
    const uint32_t r = k - band * W * tile;
    const uint32_t tc = r / (tile * bh);     // tile column (the last one may be narrower)
    const uint32_t x0 = tc * tile;
    const uint32_t tw = min(tile, W - x0);
    const uint32_t q = r - tc * tile * bh;
    return (y0 + q / tw) * W + x0 + q % tw;
}

// generate: new camera paths into the free slots of Y as the plan shares
// them out: queue position survivors + t belongs to the job whose planned
// range holds t; the list lives in device memory so the captured graph does
// not change when jobs come and go
// Each block builds WF_GEN_ROWS consecutive records at a time in a
// shared-memory tile and one thread writes the tile with a bulk tensor store
// (cp.async.bulk.tensor through `tmap`, the side's records as a 2-D tensor of
// 32 floats x capacity rows): full 128-byte lines instead of eight 16-byte
// pieces per record from every thread.  The tile's rows past the last new
// path hold stale data and land past the queue's end, which nothing reads;
// the tensor's bounds clip rows past the capacity.
constexpr uint32_t WF_GEN_ROWS = 128;  // = the generate kernel's block size

__global__ void __launch_bounds__(WF_GEN_ROWS) k_wf_generate(const WfJob* __restrict__ jobs, WfPlan P, WfSide Y,
                                                             const __grid_constant__ CUtensorMap tmap) {
    __shared__ __align__(1024) float4 s_tile[WF_GEN_ROWS * WF_REC];  // 16 KiB, 128-byte swizzle
    __shared__ uint32_t s_off[WF_MAX_JOBS + 1];
    __shared__ int s_slot[WF_MAX_JOBS];
    __shared__ unsigned long long s_first[WF_MAX_JOBS];
    const int n = *P.n;
    for (int k = threadIdx.x; k <= n; k += blockDim.x) {
        s_off[k] = P.off[k];
        if (k < n) {
            s_slot[k] = P.slot[k];
            s_first[k] = P.first[k];
        }
    }
    __syncthreads();
    const uint32_t total = s_off[n];
    const uint32_t survivors = Y.counts[0];
    const uint32_t tile_addr = (uint32_t)__cvta_generic_to_shared(s_tile);
    for (uint32_t base = blockIdx.x * WF_GEN_ROWS; base < total; base += gridDim.x * WF_GEN_ROWS) {  // block-uniform
        const uint32_t t = base + threadIdx.x;
        if (t < total) {
            int lo = 0, hi = n - 1;  // the last k with s_off[k] <= t (its range is not empty)
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (s_off[mid] <= t) lo = mid;
                else hi = mid - 1;
            }
            const int jid = s_slot[lo];
            const unsigned long long idx = s_first[lo] + (t - s_off[lo]);
            const WfJob& J = jobs[jid];
            WfPath p;
            p.job = jid;
            p.pixel = tile_pixel((uint32_t)(idx % J.npix), J.cam.width, J.cam.height, J.tile);
            p.sample = J.s0 + (uint32_t)(idx / J.npix);
            PathRng g;
            g.init(J.seed, p.pixel, p.sample);
            p.cur = camera_ray(J.cam, p.pixel, g);
            p.dim = g.dim;
            p.color = mk(1, 1, 1);
            p.prev_d = mk(0, 0, 0);
            p.depth = 0;
            p.st.reset(p.cur.inside);
            p.mis_pdf = 0.f;
            p.acc = mk(0, 0, 0);
            wf_store_tile(s_tile, threadIdx.x, p);
            if (J.flags & WR_RENDER_NEE_MIS) wf_store_acc(Y, survivors + t, p);
        }
        // the tile's generic-proxy writes before the tensor unit reads it
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (threadIdx.x == 0) {
            // row survivors + base, column 0: a 16-byte-aligned start (x = 0)
            asm volatile(
                "cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%1, %2}], [%3];\n\t"
                "cp.async.bulk.commit_group;\n\t"
                "cp.async.bulk.wait_group.read 0;"
                :
                : "l"(reinterpret_cast<uint64_t>(&tmap)), "r"(0), "r"((int)(survivors + base)), "r"(tile_addr)
                : "memory");
        }
        __syncthreads();  // the tile may be written again
    }
    if (threadIdx.x == 0) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
}

// ---------------------------------------------------------------------------
// engine
// ---------------------------------------------------------------------------
struct WfEngine {
    WfConfig cfg;
    DeviceBuffer side_mem[2], hits, scenes, jobs, order, counters, work, err_word, shadow_mem, sort_mem, plan_mem;
    WfSide side[2];
    CUtensorMap rec_map[2];  // each side's records as a 2-D tensor (k_wf_generate's bulk stores)
    WfPlan plan{};
    int equal_share = 1;  // the plan's policy (captured into the graph)
    DeviceBuffer live_cap;     // uint32: paths the plan fills the queue up to
    uint32_t live_cap_host = 0;
    WfShadow shadow{};
    WfSort sort{};
    int grid_sort = 0;
    int grid_shadow = 0;
    std::vector<const RenderData*> scene_of;  // host mirror of the scene table
    std::vector<RenderScene> scene_tab;
    std::vector<WfJob> job_tab;               // host mirror of the job slots
    std::vector<int> order_host;               // [n, slot...]
    int stack_cap = 0;
    int grid_extend = 0, grid_shade = 0, grid_gen = 0;
    size_t smem_extend = 0;
    cudaGraphExec_t graph = nullptr;
    int graph_stack = -1;
    bool mis_any = false;  // a job in the table has WR_RENDER_NEE_MIS: the shade stage with that code
    bool conn_any = true;  // a job in the table connects to lights (NEE or MIS): the shadow stage is in the loop
    int launches_per_iteration() const { return conn_any ? 8 : 6; }
    WfJobCounters* host_counters = nullptr;  // pinned
    ~WfEngine() {
        if (graph) cudaGraphExecDestroy(graph);
        if (host_counters) cudaFreeHost(host_counters);
    }
};

const WfConfig& wf_config(const WfEngine* E) { return E->cfg; }

// side k's records as a tensor of 32 floats x capacity rows (128-byte rows),
// written in WF_GEN_ROWS x 32 boxes from 128-byte-swizzled shared memory
static PFN_cuTensorMapEncodeTiled_v12000 lookup_encode_tiled() {
    cudaDriverEntryPointQueryResult q{};
    void* fn = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
        return nullptr;
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
}

static int map_side(wr_ctx* ctx, WfEngine* E, int k) {
    static const PFN_cuTensorMapEncodeTiled_v12000 encode = lookup_encode_tiled();  // once, thread-safe
    if (!encode) return set_error(ctx, WR_ERR_UNSUPPORTED, "the driver has no cuTensorMapEncodeTiled");
    const cuuint64_t dims[2] = {4 * WF_REC, E->cfg.capacity};
    const cuuint64_t strides[1] = {sizeof(float4) * WF_REC};
    const cuuint32_t box[2] = {4 * WF_REC, WF_GEN_ROWS};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult r = encode(&E->rec_map[k], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, E->side[k].rec, dims, strides, box,
                              estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                              CU_TENSOR_MAP_L2_PROMOTION_NONE, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_error(ctx, WR_ERR_INTERNAL, "cuTensorMapEncodeTiled failed for the path records");
    return WR_OK;
}

static int alloc_side(wr_ctx* ctx, WfEngine* E, int k) {
    const size_t Q = E->cfg.capacity;
    const size_t bytes = Q * (WF_REC + 1) * sizeof(float4) + 256;
    WR_CUDA(ctx, E->side_mem[k].reserve(bytes));
    char* p = E->side_mem[k].as<char>();
    WfSide& S = E->side[k];
    S.rec = reinterpret_cast<float4*>(p);
    S.a5 = S.rec + (size_t)WF_REC * Q;
    S.counts = reinterpret_cast<unsigned int*>(S.a5 + Q);
    WR_CUDA(ctx, cudaMemset(S.counts, 0, 2 * sizeof(unsigned int)));
    return WR_OK;
}

int wf_engine_get(wr_ctx* ctx, const WfConfig& cfg, WfEngine** out) {
    // one engine per context, rebuilt when the configuration changes
    WfEngine* cur = static_cast<WfEngine*>(ctx->wavefront.get());
    if (cur && cur->cfg.capacity == cfg.capacity && cur->cfg.extend_block == cfg.extend_block &&
        cur->cfg.shade_block == cfg.shade_block && cur->cfg.ctas_per_sm == cfg.ctas_per_sm &&
        cur->cfg.iters_per_graph == cfg.iters_per_graph && cur->cfg.trace.refill_min == cfg.trace.refill_min &&
        cur->cfg.trace.steps == cfg.trace.steps &&
        cur->cfg.trace.leaf_min == cfg.trace.leaf_min) {
        cur->cfg.drain_paths = cfg.drain_paths;  // host-side only
        cur->cfg.pixel_tile = cfg.pixel_tile;    // a job field, set when jobs are written
        *out = cur;
        return WR_OK;
    }
    if (cur) {
        WR_CUDA(ctx, cudaDeviceSynchronize());
        ctx->wavefront.reset();
    }
    auto E = std::make_shared<WfEngine>();
    E->cfg = cfg;
    for (int k = 0; k < 2; k++) {
        int rc = alloc_side(ctx, E.get(), k);
        if (rc == WR_OK) rc = map_side(ctx, E.get(), k);
        if (rc != WR_OK) return rc;
    }
    WR_CUDA(ctx, E->hits.reserve(sizeof(int2) * (size_t)cfg.capacity));
    WR_CUDA(ctx, E->sort_mem.reserve(sizeof(uint32_t) * ((size_t)WF_SORT_KEYS * cfg.capacity + 64)));
    E->sort.counts = E->sort_mem.as<unsigned int>();
    E->sort.idx = E->sort.counts + 64;
    WR_CUDA(ctx, cudaMemset(E->sort.counts, 0, sizeof(unsigned int) * WF_SORT_KEYS));
    E->grid_sort = ctx->num_sms * 4;
    {
        const size_t Q = cfg.capacity;
        WR_CUDA(ctx, E->shadow_mem.reserve(Q * (4 * sizeof(float4) + sizeof(int4)) + 256));
        char* p = E->shadow_mem.as<char>();
        E->shadow.o = reinterpret_cast<float4*>(p);
        E->shadow.d = E->shadow.o + Q;
        E->shadow.c = E->shadow.d + Q;
        E->shadow.r = E->shadow.c + Q;
        E->shadow.ids = reinterpret_cast<int4*>(E->shadow.r + Q);
        E->shadow.count = reinterpret_cast<unsigned int*>(E->shadow.ids + Q);
        WR_CUDA(ctx, cudaMemset(E->shadow.count, 0, sizeof(unsigned int)));
    }
    WR_CUDA(ctx, E->scenes.reserve(sizeof(RenderScene) * WF_MAX_SCENES));
    WR_CUDA(ctx, E->jobs.reserve(sizeof(WfJob) * WF_MAX_JOBS));
    WR_CUDA(ctx, cudaMemset(E->jobs.p, 0, sizeof(WfJob) * WF_MAX_JOBS));
    WR_CUDA(ctx, E->order.reserve(sizeof(int) * (WF_MAX_JOBS + 1)));
    WR_CUDA(ctx, cudaMemset(E->order.p, 0, sizeof(int) * (WF_MAX_JOBS + 1)));
    WR_CUDA(ctx, E->plan_mem.reserve(sizeof(unsigned long long) * WF_MAX_JOBS + sizeof(int) * WF_MAX_JOBS +
                                     sizeof(uint32_t) * (WF_MAX_JOBS + 1) + 64));
    E->plan.first = E->plan_mem.as<unsigned long long>();
    E->plan.slot = reinterpret_cast<int*>(E->plan.first + WF_MAX_JOBS);
    E->plan.off = reinterpret_cast<uint32_t*>(E->plan.slot + WF_MAX_JOBS);
    E->plan.n = reinterpret_cast<int*>(E->plan.off + WF_MAX_JOBS + 1);
    WR_CUDA(ctx, E->counters.reserve(sizeof(WfJobCounters) * WF_MAX_JOBS));
    WR_CUDA(ctx, cudaMemset(E->counters.p, 0, sizeof(WfJobCounters) * WF_MAX_JOBS));
    WR_CUDA(ctx, E->work.reserve(2 * sizeof(unsigned long long)));
    WR_CUDA(ctx, E->err_word.reserve(sizeof(unsigned int)));
    WR_CUDA(ctx, E->live_cap.reserve(sizeof(uint32_t)));
    E->live_cap_host = cfg.capacity;
    WR_CUDA(ctx, cudaMemcpy(E->live_cap.p, &E->live_cap_host, sizeof(uint32_t), cudaMemcpyHostToDevice));
    WR_CUDA(ctx, cudaMemset(E->err_word.p, 0, sizeof(unsigned int)));
    // the job counters, then one extra record for the queue counts of side 0
    WR_CUDA(ctx, cudaMallocHost(&E->host_counters, sizeof(WfJobCounters) * (WF_MAX_JOBS + 1)));
    E->job_tab.assign(WF_MAX_JOBS, WfJob{});
    E->order_host.assign(1, 0);
    // persistent grids from the occupancy calculator
    int per_sm = 0;
    WR_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_wf_shade<false>, cfg.shade_block, 0));
    if (cfg.ctas_per_sm > 0) per_sm = std::min(per_sm, cfg.ctas_per_sm);
    E->grid_shade = ctx->num_sms * std::max(1, per_sm);
    WR_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_wf_generate, WF_GEN_ROWS, 0));
    E->grid_gen = ctx->num_sms * std::max(1, per_sm);
    *out = E.get();
    ctx->wavefront = E;
    return WR_OK;
}

int wf_set_config(wr_ctx* ctx, const WfConfig& cfg) {
    WfEngine* E = nullptr;
    return wf_engine_get(ctx, cfg, &E);
}

// slot of a scene in the device scene table (nullptr entries are free)
static int scene_slot(wr_ctx* ctx, WfEngine* E, const RenderData* rd, int* slot) {
    for (size_t k = 0; k < E->scene_of.size(); k++)
        if (E->scene_of[k] == rd) {
            *slot = (int)k;
            return WR_OK;
        }
    for (size_t k = 0; k < E->scene_of.size(); k++)
        if (!E->scene_of[k]) {
            E->scene_of[k] = rd;
            *slot = (int)k;
            return WR_OK;
        }
    if (E->scene_of.size() >= WF_MAX_SCENES) return set_error(ctx, WR_ERR_BUSY, "too many scenes in flight");
    E->scene_of.push_back(rd);
    *slot = (int)E->scene_of.size() - 1;
    return WR_OK;
}

// a released scene must not stay in the table: a later scene could be
// allocated at the same host address and match the stale device entry
void wf_forget_scene(wr_ctx* ctx, const RenderData* rd) {
    WfEngine* E = static_cast<WfEngine*>(ctx->wavefront.get());
    if (!E || !rd) return;
    for (auto& p : E->scene_of)
        if (p == rd) p = nullptr;
}

int wf_update_jobs(wr_ctx* ctx, WfEngine* E, const std::vector<WfSlotUpdate>& updates, const std::vector<int>& order,
                   cudaStream_t s) {
    if (order.size() > WF_MAX_JOBS) return set_error(ctx, WR_ERR_BUSY, "too many jobs in flight");
    bool scenes_changed = false;
    for (const WfSlotUpdate& u : updates) {
        if (u.slot < 0 || u.slot >= (int)WF_MAX_JOBS) return set_error(ctx, WR_ERR_INTERNAL, "bad job slot");
        WfJob j = u.jh.job;
        j.tile = (uint32_t)std::max(0, E->cfg.pixel_tile);
        if (u.jh.rd) {
            int rc = scene_slot(ctx, E, u.jh.rd, &j.scene);
            if (rc != WR_OK) return rc;
            scenes_changed = true;  // (re)copy the entry: its RenderData may be new at a reused address
        } else {
            j.scene = E->job_tab[u.slot].scene;
        }
        E->job_tab[u.slot] = j;
        WR_CUDA(ctx, cudaMemcpyAsync(E->jobs.as<WfJob>() + u.slot, &E->job_tab[u.slot], sizeof(WfJob),
                                     cudaMemcpyHostToDevice, s));
        if (u.reset_counters)
            WR_CUDA(ctx, cudaMemsetAsync(E->counters.as<WfJobCounters>() + u.slot, 0, sizeof(WfJobCounters), s));
    }
    if (scenes_changed) {
        E->scene_tab.resize(E->scene_of.size());
        int cap = 8;
        for (size_t k = 0; k < E->scene_of.size(); k++) {
            if (!E->scene_of[k]) {
                std::memset(&E->scene_tab[k], 0, sizeof(RenderScene));
                continue;
            }
            E->scene_tab[k] = RenderDataView::scene(E->scene_of[k]);
            cap = std::max(cap, (int)E->scene_tab[k].tree.max_depth + 3);
        }
        WR_CUDA(ctx, cudaMemcpyAsync(E->scenes.p, E->scene_tab.data(), sizeof(RenderScene) * E->scene_tab.size(),
                                     cudaMemcpyHostToDevice, s));
        if (cap > E->stack_cap) {
            E->stack_cap = cap;
            E->smem_extend = (size_t)cap * E->cfg.extend_block * sizeof(uint32_t);
            if (E->smem_extend > 200 * 1024) return set_error(ctx, WR_ERR_UNSUPPORTED, "tree too deep for the stack");
            if (E->smem_extend > 48 * 1024) {
                for (bool st : {false, true})
                    WR_CUDA(ctx, cudaFuncSetAttribute(extend_kernel(E->cfg.ctas_per_sm, st),
                                                      cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                      (int)E->smem_extend));
            }
            int per_sm = 0;
            WR_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                             &per_sm, extend_kernel(E->cfg.ctas_per_sm, false), E->cfg.extend_block, E->smem_extend));
            if (E->cfg.ctas_per_sm > 0) per_sm = std::min(per_sm, E->cfg.ctas_per_sm);
            E->grid_extend = ctx->num_sms * std::max(1, per_sm);
            if (E->smem_extend > 48 * 1024)
                WR_CUDA(ctx, cudaFuncSetAttribute(shadow_trace_kernel(E->cfg.ctas_per_sm),
                                                  cudaFuncAttributeMaxDynamicSharedMemorySize, (int)E->smem_extend));
            WR_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_wf_shadow, 128, 0));
            E->grid_shadow = ctx->num_sms * std::max(1, per_sm);
        }
    }
    // the shade stage compiled with the light-connection code only while a job needs it
    // and the shadow stage only while a job can queue a connection
    bool mis_any = false, conn_any = false;
    for (int slot : order) {
        if (!E->job_tab[slot].active) continue;
        if (E->job_tab[slot].flags & WR_RENDER_NEE_MIS) mis_any = true;
        if (E->job_tab[slot].flags & (WR_RENDER_NEE | WR_RENDER_NEE_MIS)) conn_any = true;
    }
    if (mis_any != E->mis_any || conn_any != E->conn_any) {
        E->mis_any = mis_any;
        E->conn_any = conn_any;
        if (E->graph) {
            WR_CUDA(ctx, cudaStreamSynchronize(s));
            cudaGraphExecDestroy(E->graph);
            E->graph = nullptr;
        }
    }
    E->order_host.assign(1, (int)order.size());
    E->order_host.insert(E->order_host.end(), order.begin(), order.end());
    WR_CUDA(ctx, cudaMemcpyAsync(E->order.p, E->order_host.data(), sizeof(int) * E->order_host.size(),
                                 cudaMemcpyHostToDevice, s));
    // the host mirrors must stay alive until the copies ran
    WR_CUDA(ctx, cudaStreamSynchronize(s));
    return WR_OK;
}

// one bounce iteration; `ev` (5 events, profiling only) brackets the stages
static void enqueue_iteration(WfEngine* E, int x, cudaStream_t s, cudaEvent_t* ev = nullptr,
                              unsigned long long* stats = nullptr) {
    const int y = 1 - x;
    const RenderScene* scenes = E->scenes.as<RenderScene>();
    const WfJob* jobs = E->jobs.as<WfJob>();
    WfJobCounters* cnt = E->counters.as<WfJobCounters>();
    k_wf_reset<<<1, 1, 0, s>>>(E->side[y], E->work.as<unsigned long long>(), E->shadow.count, E->sort);
    if (ev) cudaEventRecord(ev[0], s);
    extend_kernel(E->cfg.ctas_per_sm, stats != nullptr)<<<E->grid_extend, E->cfg.extend_block, E->smem_extend, s>>>(
        scenes, jobs, E->side[x], E->hits.as<int2>(), E->work.as<unsigned long long>(), E->stack_cap, E->cfg.trace,
        E->err_word.as<unsigned int>(), stats);
    if (ev) cudaEventRecord(ev[1], s);
    k_wf_sort<<<E->grid_sort, 256, 0, s>>>(scenes, jobs, E->side[x], E->hits.as<int2>(), E->sort, E->cfg.capacity);
    (E->mis_any ? k_wf_shade<true> : k_wf_shade<false>)<<<E->grid_shade, E->cfg.shade_block, 0, s>>>(scenes, jobs, cnt, E->side[x], E->hits.as<int2>(),
                                                            E->side[y], E->shadow, E->sort, E->cfg.capacity);
    if (ev) cudaEventRecord(ev[2], s);
    if (E->conn_any) {  // the connections' closest hits go into E->hits, which shade has read
        shadow_trace_kernel(E->cfg.ctas_per_sm)<<<E->grid_extend, E->cfg.extend_block, E->smem_extend, s>>>(
            scenes, jobs, E->shadow, E->hits.as<int2>(), E->work.as<unsigned long long>() + 1, E->stack_cap,
            E->cfg.trace, E->err_word.as<unsigned int>());
        k_wf_shadow<<<E->grid_shadow, 128, 0, s>>>(scenes, jobs, E->shadow, E->hits.as<int2>(), E->side[y]);
    }
    if (ev) cudaEventRecord(ev[3], s);
    k_wf_plan<<<1, WF_MAX_JOBS, 0, s>>>(jobs, E->order.as<int>(), cnt, E->side[y], E->cfg.capacity,
                                        E->live_cap.as<uint32_t>(), E->equal_share,
                                        E->plan);
    k_wf_generate<<<E->grid_gen, WF_GEN_ROWS, 0, s>>>(jobs, E->plan, E->side[y], E->rec_map[y]);
    if (ev) cudaEventRecord(ev[4], s);
}

// wr_profile_render: the render of render_wavefront with eager launches
int profile_wavefront(wr_ctx* ctx, RenderData& rd, const RenderParams& P, uint32_t spp_offset, uint32_t spp,
                      float* film, wr_render_profile* out) {
    if (ctx->serving) return set_error(ctx, WR_ERR_BUSY, "the serving loop owns the wavefront queues");
    WfEngine* E = nullptr;
    int rc = wf_engine_get(ctx, wf_tuned_config(ctx), &E);
    if (rc != WR_OK) return rc;
    cudaStream_t s = ctx->stream;
    if ((rc = wf_set_live_cap(ctx, E, wf_config(E).capacity, s)) != WR_OK) return rc;
    const RenderScene& S = RenderDataView::scene(&rd);
    WfSlotUpdate u;
    u.slot = 0;
    u.jh.rd = &rd;
    u.jh.job = make_job(S, S.cam, P.seed, spp_offset, spp, P.max_path_len, P.flags, film, nullptr);
    u.reset_counters = true;
    if ((rc = wf_update_jobs(ctx, E, {u}, {0}, s)) != WR_OK) return rc;
    if ((rc = wf_reset_queues(ctx, E, s)) != WR_OK) return rc;
    DeviceBuffer st;
    WR_CUDA(ctx, st.reserve(4 * sizeof(unsigned long long)));
    WR_CUDA(ctx, cudaMemsetAsync(st.p, 0, 4 * sizeof(unsigned long long), s));
    cudaEvent_t ev[5], t0, t1;
    for (auto& e : ev) WR_CUDA(ctx, cudaEventCreate(&e));
    WR_CUDA(ctx, cudaEventCreate(&t0));
    WR_CUDA(ctx, cudaEventCreate(&t1));
    std::memset(out, 0, sizeof *out);
    std::vector<WfJobCounters> c;
    const unsigned long long total = u.jh.job.total;
    cudaEventRecord(t0, s);
    int x = 0;
    uint32_t queued = 0;  // rays waiting in side x
    for (uint64_t it = 0;; it++) {
        enqueue_iteration(E, x, s, ev, st.as<unsigned long long>());
        ctx->kernel_launches += E->launches_per_iteration();
        x = 1 - x;
        WR_CUDA(ctx, cudaEventSynchronize(ev[4]));
        float a = 0, b = 0, cc = 0, d = 0;
        cudaEventElapsedTime(&a, ev[0], ev[1]);
        cudaEventElapsedTime(&b, ev[1], ev[2]);
        cudaEventElapsedTime(&cc, ev[2], ev[3]);
        cudaEventElapsedTime(&d, ev[3], ev[4]);
        out->ms_extend += a;
        out->ms_shade += b;
        out->ms_shadow += cc;
        out->ms_generate += d;
        if (it < 32) {
            out->iter_rays[it] = queued;
            out->iter_extend_ms[it] = a;
            out->iter_shade_ms[it] = b;
        }
        out->iterations++;
        uint32_t waiting = 0;
        if ((rc = wf_read_counters(ctx, E, c, s, &waiting, x)) != WR_OK) break;
        queued = waiting;
        if (c[0].finished >= total) break;
        if (c[0].claimed >= total && waiting <= E->cfg.drain_threshold()) {
            cudaEventRecord(ev[0], s);
            if ((rc = wf_drain(ctx, E, x, waiting, s)) != WR_OK) break;
            cudaEventRecord(ev[1], s);
            WR_CUDA(ctx, cudaEventSynchronize(ev[1]));
            float dm = 0;
            cudaEventElapsedTime(&dm, ev[0], ev[1]);
            out->ms_drain = dm;
            out->drained_paths = waiting;
            if ((rc = wf_read_counters(ctx, E, c, s)) != WR_OK) break;
            if (c[0].finished < total) rc = set_error(ctx, WR_ERR_INTERNAL, "wavefront drain left paths");
            break;
        }
        if (it > 100000) {
            rc = set_error(ctx, WR_ERR_TIMEOUT, "wavefront did not drain");
            break;
        }
    }
    cudaEventRecord(t1, s);
    cudaEventSynchronize(t1);
    float tot = 0;
    cudaEventElapsedTime(&tot, t0, t1);
    out->ms_total = tot;
    unsigned long long h[4] = {0, 0, 0, 0};
    cudaMemcpy(h, st.p, sizeof h, cudaMemcpyDeviceToHost);
    out->rays = h[0];
    out->box_tests = h[1];
    out->tri_tests = h[2];
    out->paths = total;
    for (auto& e : ev) cudaEventDestroy(e);
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    u.jh.job.active = 0;
    u.reset_counters = false;
    if (rc == WR_OK) rc = wf_update_jobs(ctx, E, {u}, {}, s);
    return rc;
}

int wf_launch(wr_ctx* ctx, WfEngine* E, cudaStream_t s) {
    if (E->stack_cap == 0) return set_error(ctx, WR_ERR_INTERNAL, "wavefront launched without a scene");
    if (!E->graph || E->graph_stack != E->stack_cap) {
        if (E->graph) {
            cudaGraphExecDestroy(E->graph);
            E->graph = nullptr;
        }
        cudaStream_t cap;
        WR_CUDA(ctx, cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            for (int it = 0; it < E->cfg.iters_per_graph; it++) {
                enqueue_iteration(E, 0, cap);
                enqueue_iteration(E, 1, cap);
            }
            e = cudaStreamEndCapture(cap, &g);
        }
        cudaStreamDestroy(cap);
        if (e != cudaSuccess) return cuda_error(ctx, e, "capturing the bounce loop");
        e = cudaGraphInstantiate(&E->graph, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return cuda_error(ctx, e, "instantiating the bounce loop");
        E->graph_stack = E->stack_cap;
    }
    WR_CUDA(ctx, cudaGraphLaunch(E->graph, s));
    // reset, extend, sort, shade, [shadow trace, shadow,] plan, generate
    ctx->kernel_launches += (uint64_t)E->launches_per_iteration() * 2 * E->cfg.iters_per_graph;
    return WR_OK;
}

int wf_read_counters(wr_ctx* ctx, WfEngine* E, std::vector<WfJobCounters>& out, cudaStream_t s, uint32_t* waiting,
                     int side) {
    out.resize(WF_MAX_JOBS);
    WR_CUDA(ctx, cudaMemcpyAsync(E->host_counters, E->counters.p, sizeof(WfJobCounters) * WF_MAX_JOBS,
                                 cudaMemcpyDeviceToHost, s));
    unsigned int* q = reinterpret_cast<unsigned int*>(E->host_counters + WF_MAX_JOBS);
    if (waiting)
        WR_CUDA(ctx, cudaMemcpyAsync(q, E->side[side].counts, 2 * sizeof(unsigned int), cudaMemcpyDeviceToHost, s));
    WR_CUDA(ctx, cudaStreamSynchronize(s));
    std::memcpy(out.data(), E->host_counters, sizeof(WfJobCounters) * WF_MAX_JOBS);
    if (waiting) *waiting = q[0] + q[1];
    return WR_OK;
}

int wf_drain(wr_ctx* ctx, WfEngine* E, int side, uint32_t n, cudaStream_t s) {
    if (n == 0) return WR_OK;
    const int block = 128;
    const size_t smem = (size_t)E->stack_cap * block * sizeof(uint32_t);
    if (smem > 48 * 1024)
        WR_CUDA(ctx, cudaFuncSetAttribute(k_wf_drain, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_wf_drain<<<(n + block - 1) / block, block, smem, s>>>(E->scenes.as<RenderScene>(), E->jobs.as<WfJob>(),
                                                           E->counters.as<WfJobCounters>(), E->side[side],
                                                           E->stack_cap, E->err_word.as<unsigned int>());
    WR_CUDA(ctx, cudaGetLastError());
    ctx->kernel_launches++;
    return WR_OK;
}

int wf_error_word(wr_ctx* ctx, WfEngine* E, unsigned int* herr, cudaStream_t s) {
    WR_CUDA(ctx, cudaMemcpyAsync(herr, E->err_word.p, sizeof(unsigned int), cudaMemcpyDeviceToHost, s));
    WR_CUDA(ctx, cudaStreamSynchronize(s));
    return WR_OK;
}

int wf_set_equal_share(wr_ctx* ctx, WfEngine* E, bool on) {
    (void)ctx;
    if (E->equal_share != (int)on) {
        E->equal_share = on;
        if (E->graph) {  // the policy is a kernel argument of the captured loop
            cudaGraphExecDestroy(E->graph);
            E->graph = nullptr;
        }
    }
    return WR_OK;
}

int wf_set_live_cap(wr_ctx* ctx, WfEngine* E, uint32_t paths, cudaStream_t s) {
    paths = std::max<uint32_t>(1, std::min(paths, E->cfg.capacity));
    if (paths == E->live_cap_host) return WR_OK;
    E->live_cap_host = paths;
    // from pageable memory: the call has read `paths` when it returns
    WR_CUDA(ctx, cudaMemcpyAsync(E->live_cap.p, &paths, sizeof(uint32_t), cudaMemcpyHostToDevice, s));
    return WR_OK;
}

uint32_t wf_live_cap(const WfEngine* E) { return E->live_cap_host; }

int wf_reset_queues(wr_ctx* ctx, WfEngine* E, cudaStream_t s) {
    for (int k = 0; k < 2; k++) WR_CUDA(ctx, cudaMemsetAsync(E->side[k].counts, 0, 2 * sizeof(unsigned int), s));
    return WR_OK;
}

WfJob make_job(const RenderScene& S, const CamParams& cam, uint64_t seed, uint32_t s0, uint32_t spp,
               uint32_t max_path_len, uint32_t flags, float* film, float* film2) {
    WfJob j;
    std::memset(&j, 0, sizeof j);
    (void)S;
    j.active = 1;
    j.cam = cam;
    j.seed = seed;
    j.s0 = s0;
    j.spp = spp;
    j.max_path_len = max_path_len;
    j.flags = flags;
    j.npix = cam.width * cam.height;
    j.total = (unsigned long long)j.npix * spp;
    j.film = film;
    j.film2 = film2;
    return j;
}

int render_wavefront(wr_ctx* ctx, RenderData& rd, const RenderParams& P, uint32_t spp_offset, uint32_t spp,
                     float* film, float* film2, cudaStream_t s) {
    if (ctx->serving) return set_error(ctx, WR_ERR_BUSY, "the serving loop owns the wavefront queues");
    WfEngine* E = nullptr;
    int rc = wf_engine_get(ctx, wf_tuned_config(ctx), &E);
    if (rc != WR_OK) return rc;
    if ((rc = wf_set_live_cap(ctx, E, wf_config(E).capacity, s)) != WR_OK) return rc;  // the whole queue
    const RenderScene& S = RenderDataView::scene(&rd);
    WfSlotUpdate u;
    u.slot = 0;
    u.jh.rd = &rd;
    u.jh.job = make_job(S, S.cam, P.seed, spp_offset, spp, P.max_path_len, P.flags, film, film2);
    u.reset_counters = true;
    rc = wf_update_jobs(ctx, E, {u}, {0}, s);
    if (rc != WR_OK) return rc;
    if ((rc = wf_reset_queues(ctx, E, s)) != WR_OK) return rc;
    // replay the captured bounce loop until every path of the job has reached the film
    std::vector<WfJobCounters> c;
    const unsigned long long total = u.jh.job.total;
    const uint64_t max_launches =
        1 + (total / std::max<uint32_t>(1, E->cfg.capacity) + 4) * (uint64_t)(P.max_path_len + 4) * 4;
    const uint32_t drain_at = E->cfg.drain_threshold();
    for (uint64_t l = 0;; l++) {
        if ((rc = wf_launch(ctx, E, s)) != WR_OK) return rc;
        uint32_t waiting = 0;
        if ((rc = wf_read_counters(ctx, E, c, s, &waiting)) != WR_OK) return rc;
        if (c[0].finished >= total) break;
        if (c[0].claimed >= total && waiting <= drain_at) {
            // every path is generated and few remain: finish them one per thread
            if ((rc = wf_drain(ctx, E, 0, waiting, s)) != WR_OK) return rc;
            if ((rc = wf_read_counters(ctx, E, c, s)) != WR_OK) return rc;
            if (c[0].finished < total) return set_error(ctx, WR_ERR_INTERNAL, "wavefront drain left paths");
            break;
        }
        if (l > max_launches) return set_error(ctx, WR_ERR_TIMEOUT, "wavefront did not drain");
    }
    // retire the job so a later render starts from an empty table
    u.jh.job.active = 0;
    u.reset_counters = false;
    if ((rc = wf_update_jobs(ctx, E, {u}, {}, s)) != WR_OK) return rc;
    unsigned int herr = 0;
    if ((rc = wf_error_word(ctx, E, &herr, s)) != WR_OK) return rc;
    if (herr) return set_error(ctx, WR_ERR_INTERNAL, "traversal stack overflow");
    return WR_OK;
}

}  // namespace wr
