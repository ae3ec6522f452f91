// wr_traverse.cuh — closest-hit traversal of the reference tree on sm_103a.
//
// Result contract: identical triangle id (and t) to KDTree::intersect
// (kdtree.cpp:308-353) with NoSelfCondition (noself.cpp:13-20) when filtered.
//
// How the reference's semantics are kept while the GPU is free to reorder:
//  * The reference descends every child whose box passes its predicate
//    (BoundingBox::intersect, kdtree.cpp:46-64), so its candidate set is "all
//    triangles under passing boxes".  The same predicate decides here, so the
//    candidate set is the same whatever the visiting order.
//  * Its winner is the smallest t, ties to the right child / first in a leaf;
//    with the slot layout of wr_device.cuh that is "smallest t, then largest
//    slot", an order-free rule.
//  * The predicate itself is evaluated cheaply, by two slab tests: one on the
//    box grown by a margin M, one on the box shrunk by M.  M (about 33 units
//    of FP32 rounding of the coordinates involved) is larger than the error
//    of the reference's face test and of the slab tests themselves, so:
//      - a ray that misses the grown box fails all six reference face tests
//        (each of them needs a plane point within rounding of the box);
//      - a ray that passes the shrunk box, and whose entry axis is
//        unambiguous (the grown-box entry distance T1 = max of the grown
//        near distances is at least the shrunk near distance of every other
//        axis), enters the real box through a point at least ~M inside the
//        entry face on both other axes, at a distance >= 0; the reference's
//        test of that face therefore passes.  With the origin inside (T1 <
//        0) the same holds for the exit face (U1 = min of the grown far
//        distances at most the shrunk far distance of every other axis).
//    Everything else (a ray within ~M of an edge, a box thinner than 2M,
//    a NaN) runs the reference's face test itself: the likely face first,
//    all six if that one fails.
//    Rays must be finite; a NaN or infinite direction gets no hit here, as
//    in the reference (its triangle test fails for it).
//    The shrunk distances are the grown ones moved by 2M|inv| per axis
//    (q.sm: the grown near plane is M outside the box, the shrunk one M
//    inside, so their distances differ by exactly 2M|inv|), one FP32
//    addition each instead of a subtraction and a product: their rounding
//    stays within ~4 eps (B + |o|) |inv|, far inside the margin.  A ray with
//    a zero (or subnormal) direction component has a non-finite 2M|inv|; its
//    q.sm is NaN, so its shrunk test never passes and every box it grazes is
//    decided by the face test.
//  * Optional pruning (PRUNE, used by the renderers and wr_trace_closest): a
//    child whose grown-box entry distance exceeds q.pf times the best hit
//    (plus M) is skipped.  A triangle lies inside its box (boxes are the
//    bounds of their triangles' vertices), so its hit distance is at least
//    the box's entry distance up to the triangle test's rounding, which is
//    relative and bounded unless the ray grazes the triangle's plane (|n.d|
//    small).  A hit accepted with |n.d| < 2^-5 |d| therefore switches pruning
//    off for the rest of that ray (q.pf = inf): near-grazing rays see every
//    box the reference sees.
#pragma once

#include "wr_device.cuh"

namespace wr {

struct RayQ {
    f3 o, d, inv;
    // per axis, with s = +1 where the direction is positive (inv > 0), else -1:
    // gno = o + s M and gfo = o - s M.  (near corner - gno) * inv is the
    // grown-box near distance, (far corner - gfo) * inv the grown-box far
    // one; the shrunk box's are those -/+ sm = 2 M |inv| (NaN: never sure).
    f3 gno, gfo, sm;
    float M;      // box margin for this ray
    float pf;     // pruning: boxes entered beyond pf * (closest hit) + M are skipped
};

// below this |n.d| / |d| an accepted hit turns pruning off for its ray
constexpr float GRAZE_COS = 0.03125f;

__device__ __forceinline__ RayQ make_rayq(f3 o, f3 d, float scene_mag) {
    RayQ q;
    q.o = o;
    q.d = d;
    q.inv = mk(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
    float om = fmaxf(fabsf(o.x), fmaxf(fabsf(o.y), fabsf(o.z)));
    // reference predicate rounding <= ~4.1 eps (B + |o|), slab test rounding
    // <= ~4 eps (B + |o|) (eps = 2^-24); 2e-6 is ~33 eps
    q.M = 2e-6f * (scene_mag + om) + 1e-30f;
    const float lo_x = o.x + q.M, lo_y = o.y + q.M, lo_z = o.z + q.M;
    const float hi_x = o.x - q.M, hi_y = o.y - q.M, hi_z = o.z - q.M;
    q.gno = mk(q.inv.x > 0.f ? lo_x : hi_x, q.inv.y > 0.f ? lo_y : hi_y, q.inv.z > 0.f ? lo_z : hi_z);
    q.gfo = mk(q.inv.x > 0.f ? hi_x : lo_x, q.inv.y > 0.f ? hi_y : lo_y, q.inv.z > 0.f ? hi_z : lo_z);
    const float m2 = 2.f * q.M;
    q.sm = mk(m2 * fabsf(q.inv.x), m2 * fabsf(q.inv.y), m2 * fabsf(q.inv.z));
    if (!(isfinite(q.sm.x) && isfinite(q.sm.y) && isfinite(q.sm.z))) q.sm = mk(NAN, NAN, NAN);
    q.pf = 1.001f;
    return q;
}

struct Box {
    float lx, ly, lz, hx, hy, hz;
};
template <int K>
__device__ __forceinline__ float lo_(const Box& b) { return K == 0 ? b.lx : (K == 1 ? b.ly : b.lz); }
template <int K>
__device__ __forceinline__ float hi_(const Box& b) { return K == 0 ? b.hx : (K == 1 ? b.hy : b.hz); }
template <int K>
__device__ __forceinline__ float c_(f3 v) { return K == 0 ? v.x : (K == 1 ? v.y : v.z); }

// One reference face test (kdtree.cpp:50-63), face I in 0..5 of the box.
template <int I>
__device__ __forceinline__ bool face_pass(const Box& bx, const RayQ& q) {
    constexpr int A = I % 3, B = (I + 1) % 3, C = (I + 2) % 3;
    const float dA = c_<A>(q.d);
    if (dA == 0.f) return false;
    const float plane = I < 3 ? lo_<A>(bx) : hi_<A>(bx);
    const float dist = div_x(sub_x(plane, c_<A>(q.o)), dA);
    const float pb = add_x(c_<B>(q.o), mul_x(dist, c_<B>(q.d)));
    const float pc = add_x(c_<C>(q.o), mul_x(dist, c_<C>(q.d)));
    return dist >= 0.f && lo_<B>(bx) <= pb && hi_<B>(bx) >= pb && lo_<C>(bx) <= pc && hi_<C>(bx) >= pc;
}

__device__ __forceinline__ bool all_faces(const Box& bx, const RayQ& q) {
    return face_pass<0>(bx, q) || face_pass<1>(bx, q) || face_pass<2>(bx, q) || face_pass<3>(bx, q) ||
           face_pass<4>(bx, q) || face_pass<5>(bx, q);
}

__device__ __forceinline__ float pick3(int k, float x, float y, float z) { return k == 0 ? x : (k == 1 ? y : z); }

// The reference face test on the face given at run time (axis `a`, max plane
// if `hi`), with register selects instead of a per-lane switch so that lanes
// testing different faces do not diverge.  Same operations as face_pass<I>.
__device__ __forceinline__ bool face_pass_sel(int a, bool hi, const Box& bx, const RayQ& q) {
    const int b = a == 2 ? 0 : a + 1, c = b == 2 ? 0 : b + 1;
    const float dA = pick3(a, q.d.x, q.d.y, q.d.z);
    const float oA = pick3(a, q.o.x, q.o.y, q.o.z);
    const float plane = hi ? pick3(a, bx.hx, bx.hy, bx.hz) : pick3(a, bx.lx, bx.ly, bx.lz);
    const float oB = pick3(b, q.o.x, q.o.y, q.o.z), dB = pick3(b, q.d.x, q.d.y, q.d.z);
    const float oC = pick3(c, q.o.x, q.o.y, q.o.z), dC = pick3(c, q.d.x, q.d.y, q.d.z);
    const float loB = pick3(b, bx.lx, bx.ly, bx.lz), hiB = pick3(b, bx.hx, bx.hy, bx.hz);
    const float loC = pick3(c, bx.lx, bx.ly, bx.lz), hiC = pick3(c, bx.hx, bx.hy, bx.hz);
    // a zero direction component skips the face (kdtree.cpp:51); the division
    // is still evaluated so that every lane runs the same instructions
    const float dist = div_x(sub_x(plane, oA), dA);
    const float pb = add_x(oB, mul_x(dist, dB));
    const float pc = add_x(oC, mul_x(dist, dC));
    return (dA != 0.f) & (dist >= 0.f) & (loB <= pb) & (hiB >= pb) & (loC <= pc) & (hiC >= pc);
}

// The reference's test run on the likely face (entry face, or the exit face
// when the grown-box entry is behind the origin), on all six if that fails:
// exactly BoundingBox::intersect's pass/fail.
__device__ __forceinline__ bool box_exact(const Box& bx, const RayQ& q) {
    const bool px = q.inv.x > 0.f, py = q.inv.y > 0.f, pz = q.inv.z > 0.f;
    const float nx = ((px ? bx.lx : bx.hx) - q.gno.x) * q.inv.x, fx = ((px ? bx.hx : bx.lx) - q.gfo.x) * q.inv.x;
    const float ny = ((py ? bx.ly : bx.hy) - q.gno.y) * q.inv.y, fy = ((py ? bx.hy : bx.ly) - q.gfo.y) * q.inv.y;
    const float nz = ((pz ? bx.lz : bx.hz) - q.gno.z) * q.inv.z, fz = ((pz ? bx.hz : bx.lz) - q.gfo.z) * q.inv.z;
    const bool entry = fmaxf(nx, fmaxf(ny, nz)) >= 0.f;
    const int ea = (nx >= ny && nx >= nz) ? 0 : (ny >= nz ? 1 : 2);
    const int xa = (fx <= fy && fx <= fz) ? 0 : (fy <= fz ? 1 : 2);
    const int a = entry ? ea : xa;
    const bool pos = pick3(a, q.d.x, q.d.y, q.d.z) > 0.f;
    if (face_pass_sel(a, entry ? !pos : pos, bx, q)) return true;
    return all_faces(bx, q);
}

enum : int { BOX_MISS = 0, BOX_HIT = 1, BOX_UNSURE = 2 };

// The two slab tests of the header: BOX_MISS and BOX_HIT are the reference's
// answer, BOX_UNSURE needs box_exact().  *tnear = grown-box entry distance.
__device__ __forceinline__ int box_classify(const Box& bx, const RayQ& q, float* tnear) {
    const bool px = q.inv.x > 0.f, py = q.inv.y > 0.f, pz = q.inv.z > 0.f;
    const float cnx = px ? bx.lx : bx.hx, cfx = px ? bx.hx : bx.lx;
    const float cny = py ? bx.ly : bx.hy, cfy = py ? bx.hy : bx.ly;
    const float cnz = pz ? bx.lz : bx.hz, cfz = pz ? bx.hz : bx.lz;
    // grown box; fmaxf/fminf drop a NaN (0 * inf: parallel ray on a plane)
    const float gnx = (cnx - q.gno.x) * q.inv.x, gfx = (cfx - q.gfo.x) * q.inv.x;
    const float gny = (cny - q.gno.y) * q.inv.y, gfy = (cfy - q.gfo.y) * q.inv.y;
    const float gnz = (cnz - q.gno.z) * q.inv.z, gfz = (cfz - q.gfo.z) * q.inv.z;
    // shrunk box (empty, so never "sure", when thinner than 2M)
    const float snx = gnx + q.sm.x, sfx = gfx - q.sm.x;
    const float sny = gny + q.sm.y, sfy = gfy - q.sm.y;
    const float snz = gnz + q.sm.z, sfz = gfz - q.sm.z;
    const float T1 = fmaxf(gnx, fmaxf(gny, gnz)), U1 = fminf(gfx, fminf(gfy, gfz));
    const float T2 = fmaxf(snx, fmaxf(sny, snz)), U2 = fminf(sfx, fminf(sfy, sfz));
    *tnear = T1;
    const bool grown = (T1 <= U1) & (U1 >= 0.f);
    const bool shrunk = (T2 <= U2) & (U2 >= 0.f);
    const int cin = (int)(snx > T1) + (int)(sny > T1) + (int)(snz > T1);
    const int cout = (int)(sfx < U1) + (int)(sfy < U1) + (int)(sfz < U1);
    const bool sure = shrunk & ((T1 >= 0.f) ? (cin <= 1) : (cout <= 1));
    return grown ? (sure ? BOX_HIT : BOX_UNSURE) : BOX_MISS;
}

// The reference box predicate; *tnear gets the grown-box entry distance.
__device__ __forceinline__ bool box_pred(const Box& bx, const RayQ& q, float* tnear) {
    const int c = box_classify(bx, q, tnear);
    if (c == BOX_UNSURE) return box_exact(bx, q);
    return c == BOX_HIT;
}

// Both children of a pair: the rare exact tests share one code path.
__device__ __forceinline__ void pair_pred(const Box& L, const Box& R, const RayQ& q, bool* hl, bool* hr, float* tl,
                                          float* tr) {
    int cl = box_classify(L, q, tl), cr = box_classify(R, q, tr);
    const bool el = cl == BOX_UNSURE, er = cr == BOX_UNSURE;
    for (int k = 0, nk = (int)el + (int)er; k < nk; ++k) {
        const bool right = k == 1 || !el;
        const bool r = box_exact(right ? R : L, q);
        if (right) cr = r ? BOX_HIT : BOX_MISS;
        else cl = r ? BOX_HIT : BOX_MISS;
    }
    *hl = cl == BOX_HIT;
    *hr = cr == BOX_HIT;
}

// KDTree::intersect(ray, tri) geometric part (kdtree.cpp:279-301); returns
// the distance or -1.  The edge-mask rejection is taken before the plane
// distance (same result, less work).
__device__ __forceinline__ float tri_test(f3 v0, f3 v1, f3 v2, const RayQ& q, float* dd_out = nullptr) {
    const f3 l0 = sub3_x(v1, v0), l1 = sub3_x(v2, v1), l2 = sub3_x(v0, v2);
    const f3 r0 = sub3_x(v0, q.o), r1 = sub3_x(v1, q.o), r2 = sub3_x(v2, q.o);
    const float s0 = dot_x(q.d, cross_x(l0, r0));
    const float s1 = dot_x(q.d, cross_x(l1, r1));
    const float s2 = dot_x(q.d, cross_x(l2, r2));
    const bool pos = s0 >= 0.f && s1 >= 0.f && s2 >= 0.f;
    const bool neg = s0 <= 0.f && s1 <= 0.f && s2 <= 0.f;
    if (!pos && !neg) return -1.f;
    const f3 n = normalize_x(cross_x(l0, l1));
    const float od = dot_x(n, r2);
    const float dd = dot_x(n, q.d);
    if (dd_out) *dd_out = dd;
    if (dd == 0.f) return -1.f;
    const float t = div_x(od, dd);
    if (t < 0.f) return -1.f;
    return t;
}

// pruning stays on only while the closest hit is not a near-grazing one
__device__ __forceinline__ void graze_check(RayQ& q, float dd) {
    if (fabsf(dd) < GRAZE_COS * length(q.d)) q.pf = __int_as_float(0x7f800000);
}

// Mesh::getWorldNormal without vertex normals (mesh.h:47-56)
__device__ __forceinline__ f3 face_normal(f3 v0, f3 v1, f3 v2) {
    return normalize_x(cross_x(sub3_x(v1, v0), sub3_x(v2, v0)));
}

// NoSelfCondition::legal (noself.cpp:13-20); object ids, -1 = none
__device__ __forceinline__ bool noself_legal(int inside, int contact, int hit_obj, f3 dir, f3 fn) {
    const float d = dot_x(dir, fn);
    const bool in = d <= 0.f, out = d >= 0.f;
    if (inside == contact) return !(in && contact == hit_obj);
    return !(out && inside != hit_obj);
}

__device__ __forceinline__ Box root_box(const DevTree& T) {
    return Box{T.root_lo[0], T.root_lo[1], T.root_lo[2], T.root_hi[0], T.root_hi[1], T.root_hi[2]};
}

struct Hit {
    float t;    // +inf when no hit
    int slot;   // -1 when no hit
};

__device__ __forceinline__ float4 ldg4(const float4* p) { return __ldg(p); }
__device__ __forceinline__ uint4 ldg4u(const uint4* p) { return __ldg(p); }

template <bool FILTERED, bool PRUNE>
__device__ __forceinline__ void leaf_test(const DevTree& T, uint32_t first, uint32_t count, RayQ& q, int inside,
                                          int contact, Hit& h) {
    for (uint32_t k = 0; k < count; k++) {
        const int slot = (int)(first + k);
        const TriRec* tr = T.tris + slot;
        const float4 a = ldg4(&tr->v0), b = ldg4(&tr->v1), c = ldg4(&tr->v2);
        const f3 v0 = xyz(a), v1 = xyz(b), v2 = xyz(c);
        float dd;
        const float t = tri_test(v0, v1, v2, q, &dd);
        if (t >= 0.f && (t < h.t || (t == h.t && slot > h.slot))) {
            if (FILTERED) {
                if (!noself_legal(inside, contact, (int)__float_as_uint(b.w), q.d, face_normal(v0, v1, v2))) continue;
            }
            h.t = t;
            h.slot = slot;
            if (PRUNE) graze_check(q, dd);
        }
    }
}

// The same with the filter chosen per ray (eye rays are traced without one)
template <bool PRUNE>
__device__ __forceinline__ void leaf_test_dyn(const TriRec* tris, uint32_t first, uint32_t count, RayQ& q, bool filt,
                                              int inside, int contact, Hit& h) {
    for (uint32_t k = 0; k < count; k++) {
        const int slot = (int)(first + k);
        const TriRec* tr = tris + slot;
        const float4 a = ldg4(&tr->v0), b = ldg4(&tr->v1), c = ldg4(&tr->v2);
        const f3 v0 = xyz(a), v1 = xyz(b), v2 = xyz(c);
        float dd;
        const float t = tri_test(v0, v1, v2, q, &dd);
        if (t >= 0.f && (t < h.t || (t == h.t && slot > h.slot))) {
            if (filt && !noself_legal(inside, contact, (int)__float_as_uint(b.w), q.d, face_normal(v0, v1, v2)))
                continue;
            h.t = t;
            h.slot = slot;
            if (PRUNE) graze_check(q, dd);
        }
    }
}

// Closest hit.  `stack` is this thread's stack: entries at stack[k * stride],
// at most `cap` of them (cap >= tree depth + 2 always suffices; a traversal
// that would exceed it stops and sets bit 0 of *err instead of writing past).
template <bool FILTERED, bool PRUNE>
__device__ __forceinline__ Hit trace_closest(const DevTree& T, const RayQ& q0, int inside, int contact,
                                             uint32_t* stack, int stride, int cap, unsigned int* err) {
    RayQ q = q0;
    Hit h;
    h.t = __int_as_float(0x7f800000);
    h.slot = -1;
    float tn;
    if (!box_pred(root_box(T), q, &tn)) return h;
    if (T.root_w1 & LEAF_FLAG) {
        leaf_test<FILTERED, PRUNE>(T, T.root_w0, T.root_w1 & ~LEAF_FLAG, q, inside, contact, h);
        return h;
    }
    int sp = 0;
    stack[0] = T.root_w0;
    sp = 1;
    while (sp > 0) {
        const uint32_t pi = stack[(--sp) * stride];
        const NodePair* P = T.pairs + pi;
        const float4 A = ldg4(&P->a), B = ldg4(&P->b), C = ldg4(&P->c);
        const uint4 W = ldg4u(&P->t);
        float tl, tr;
        bool hl, hr;
        pair_pred(Box{A.x, A.y, A.z, A.w, B.x, B.y}, Box{B.z, B.w, C.x, C.y, C.z, C.w}, q, &hl, &hr, &tl, &tr);
        if (PRUNE) {
            const float lim = h.t * q.pf + q.M;
            hl = hl && !(tl > lim);
            hr = hr && !(tr > lim);
        }
        // leaves first (they can tighten the bound), both through one code
        // path; then push internal children far-first so the near one is
        // popped next
        const bool ll = hl && (W.y & LEAF_FLAG), lr = hr && (W.w & LEAF_FLAG);
        for (int k = 0, nk = (int)ll + (int)lr; k < nk; k++) {
            const bool right = k == 1 || !ll;
            leaf_test<FILTERED, PRUNE>(T, right ? W.z : W.x, (right ? W.w : W.y) & ~LEAF_FLAG, q, inside, contact, h);
        }
        hl = hl && !ll;
        hr = hr && !lr;
        if (sp + 2 > cap) {
            atomicOr(err, 1u);
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
    return h;
}

// barycentric weights of v1, v2 at the hit point (mesh.h:67-73)
__device__ __forceinline__ void hit_barycentrics(const DevTree& T, int slot, const RayQ& q, float t, float* u1,
                                                 float* u2, uint32_t* gid) {
    const TriRec* tr = T.tris + slot;
    const float4 a = ldg4(&tr->v0), b = ldg4(&tr->v1), c = ldg4(&tr->v2);
    const f3 v0 = xyz(a), b1 = xyz(b) - v0, b2 = xyz(c) - v0;
    const f3 v = (q.o + q.d * t) - v0;
    const float d12 = dot(b1, b2), l1 = length(b1), l2 = length(b2);
    const float vb1 = dot(v, b1), vb2 = dot(v, b2);
    const float w2 = (vb1 * d12 - vb2 * l1 * l1) / (d12 * d12 - l1 * l1 * l2 * l2);
    *u1 = (vb1 - w2 * d12) / (l1 * l1);
    *u2 = w2;
    *gid = __float_as_uint(a.w);
}

}  // namespace wr
