// wr_warp_trace.cuh — the warp-persistent closest-hit loop shared by the
// batch kernel (k_trace_closest) and the wavefront extend stage.
//
// Same result as trace_closest() (wr_traverse.cuh): the same box predicate
// decides every descent and the winner is order-free ("smallest t, then
// largest slot"), so visiting order and the moment a leaf is tested do not
// change it.  What changes is how a warp's 32 lanes are kept busy:
//
//  * postponed leaves: a lane that reaches leaves parks them and waits; once
//    `leaf_min` lanes hold leaves (or no lane is left searching) the warp
//    tests them together, so the triangle test runs once for many lanes
//    instead of once per divergent branch;
//  * ray refill: lanes whose ray is finished fetch new rays from a global
//    counter (one atomicAdd per warp) as soon as `refill_min` of them are
//    idle, instead of waiting for the whole warp;
//  * the box predicate (wr_traverse.cuh) is straight-line code but for the
//    rare exact face test, which both children share.
//
// A source class supplies the rays: `load(id, lane, stack, stride)` fills the
// lane's ray and tree and calls lane_start(); `store(id, lane)` writes the
// result.
#pragma once

#include "wr_traverse.cuh"

namespace wr {

struct TraceLane {
    const NodePair* pairs;
    const TriRec* tris;
    RayQ q;
    int inside, contact;  // NoSelfCondition object ids (used when filt)
    bool filt;
    Hit h;
    int sp;               // stack entries
    int npend;            // postponed leaves (0..2)
    uint32_t lf0, lc0, lf1, lc1;  // postponed leaves: first slot and triangle count
    uint32_t n_box, n_tri;        // work counters (profiling only)
};

// Starts a ray: the root's box test; the root pair goes on the stack, or a
// root leaf is postponed.
__device__ __forceinline__ void lane_start(TraceLane& L, const Box& root, uint32_t w0, uint32_t w1, uint32_t* stack,
                                           int stride) {
    L.h.t = __int_as_float(0x7f800000);
    L.h.slot = -1;
    L.sp = 0;
    L.npend = 0;
    L.n_box = 1;
    L.n_tri = 0;
    float tn;
    if (box_pred(root, L.q, &tn)) {
        if (w1 & LEAF_FLAG) {
            L.lf0 = w0;
            L.lc0 = w1 & ~LEAF_FLAG;
            L.npend = 1;
        } else {
            stack[(L.sp++) * stride] = w0;
        }
    }
}

// One traversal step of a searching lane (npend == 0, sp > 0): pop a pair,
// test both children, postpone leaf children, push internal ones far-first.
template <bool PRUNE, bool STATS>
__device__ __forceinline__ void lane_step(TraceLane& L, uint32_t* stack, int stride, int cap, unsigned int* err) {
    const uint32_t pi = stack[(--L.sp) * stride];
    const NodePair* P = L.pairs + pi;
    const float4 A = ldg4(&P->a), B = ldg4(&P->b), C = ldg4(&P->c);
    const uint4 W = ldg4u(&P->t);
    float tl, tr;
    bool hl, hr;
    pair_pred(Box{A.x, A.y, A.z, A.w, B.x, B.y}, Box{B.z, B.w, C.x, C.y, C.z, C.w}, L.q, &hl, &hr, &tl, &tr);
    if (STATS) L.n_box += 2;
    if (PRUNE) {
        const float lim = L.h.t * L.q.pf + L.q.M;
        hl = hl && !(tl > lim);
        hr = hr && !(tr > lim);
    }
    const bool ll = hl && (W.y & LEAF_FLAG), lr = hr && (W.w & LEAF_FLAG);
    L.lf0 = ll ? W.x : W.z;
    L.lc0 = (ll ? W.y : W.w) & ~LEAF_FLAG;
    L.lf1 = W.z;
    L.lc1 = W.w & ~LEAF_FLAG;
    L.npend = (int)ll + (int)lr;
    hl = hl && !ll;
    hr = hr && !lr;
    if (L.sp + 2 > cap) {  // cannot happen for a stack of tree depth + 3; never write past it
        atomicOr(err, 1u);
        L.sp = 0;
        return;
    }
    if (hl && hr) {
        const bool lnear = tl <= tr;
        stack[(L.sp++) * stride] = lnear ? W.z : W.x;
        stack[(L.sp++) * stride] = lnear ? W.x : W.z;
    } else if (hl) {
        stack[(L.sp++) * stride] = W.x;
    } else if (hr) {
        stack[(L.sp++) * stride] = W.z;
    }
}

// The postponed leaves of a lane, through one code path for the warp.
template <bool PRUNE, bool STATS>
__device__ __forceinline__ void lane_leaves(TraceLane& L) {
    for (int k = 0; k < L.npend; ++k) {
        const uint32_t first = k ? L.lf1 : L.lf0, count = k ? L.lc1 : L.lc0;
        if (STATS) L.n_tri += count;
        leaf_test_dyn<PRUNE>(L.tris, first, count, L.q, L.filt, L.inside, L.contact, L.h);
    }
    L.npend = 0;
}

// Traces rays [0, n) of `src`, handing out ray ids from *counter (which
// starts at 0).  Every lane of the warp must call it.  Each turn the warp
// does one thing for the lanes it concerns: tests the postponed leaves (once
// `leaf_min` lanes hold some, or no lane is left searching) or takes one
// traversal step (or up to `steps` of them); lanes that finish store their
// hit, and idle lanes refill once `refill_min` of them are idle.
template <bool PRUNE, bool STATS, class Src>
__device__ __forceinline__ void warp_trace(Src& src, uint64_t n, unsigned long long* counter, TraceTune tune,
                                           uint32_t* stack, int stride, int cap, unsigned int* err) {
    constexpr unsigned FULL = 0xffffffffu;
    const unsigned lane = threadIdx.x & 31u;
    const unsigned lt_mask = (1u << lane) - 1u;
    bool active = false, exhausted = false;
    uint64_t id = 0;
    TraceLane L;
    L.sp = 0;
    L.npend = 0;
    for (;;) {
        const bool want = !active && !exhausted;
        const unsigned need = __ballot_sync(FULL, want);
        const unsigned busy = __ballot_sync(FULL, active);
        if (need && (busy == 0 || __popc(need) >= tune.refill_min)) {
            const int leader = __ffs(need) - 1;
            unsigned long long base = 0;
            if ((int)lane == leader) base = atomicAdd(counter, (unsigned long long)__popc(need));
            base = __shfl_sync(FULL, base, leader);
            if (want) {
                id = base + __popc(need & lt_mask);
                if (id < n) {
                    src.load(id, L, stack, stride);
                    active = true;
                } else {
                    exhausted = true;
                }
            }
        }
        if (__ballot_sync(FULL, active) == 0) {
            if (__ballot_sync(FULL, !exhausted) == 0) break;
            continue;
        }
        const bool searching = active && L.npend == 0 && L.sp > 0;
        const bool pending = active && L.npend > 0;
        const unsigned sm = __ballot_sync(FULL, searching), pm = __ballot_sync(FULL, pending);
        if (pm && (sm == 0 || __popc(pm) >= tune.leaf_min)) {
            if (pending) lane_leaves<PRUNE, STATS>(L);
        } else if (searching) {
            // up to tune.steps steps before the warp looks at its lanes again:
            // fewer ballots per step, at the price of lanes that reach leaves
            // early waiting for the others
            lane_step<PRUNE, STATS>(L, stack, stride, cap, err);
            for (int k = 1; k < tune.steps && L.npend == 0 && L.sp > 0; ++k)
                lane_step<PRUNE, STATS>(L, stack, stride, cap, err);
        }
        if (active && L.sp == 0 && L.npend == 0) {
            src.store(id, L);
            active = false;
        }
    }
}

}  // namespace wr
