// bpt.cu — WR_MODE_BIDIRECTIONAL: WalkRay's bidirectional path tracer
// (BidirectionalPathTracer, bidirPathTracer.cpp:10-313) on the GPU.
//
// One render call runs in batches of samples-per-pixel; a batch of B samples
// of every pixel is five kernels:
//
//   k_bpt_subpaths  persistent: the eye sub-paths (Camera::generateRay +
//                   MCRenderer::samplePath) and the light sub-paths
//                   (Scene::genLightSample + samplePath), one record per lane
//                   and turn, a lane taking a new sub-path as soon as its own
//                   ends; every ray record written to HBM (64 B per vertex,
//                   vertex-major so that stores of vertex k of consecutive
//                   samples are contiguous);
//   k_bpt_enum      one thread per (pixel, sample): the (light length, eye
//                   length) pairs that pass throughputByConnecting's path-shape
//                   tests, appended to a candidate list in runs of one pair;
//   k_bpt_visible   persistent, one candidate per thread and step: connectEdge
//                   and the visibility ray (MCRenderer::visibilityTest); the
//                   visible ones are appended to the contributing list;
//   k_bpt_connect   persistent, one contributing connection per thread and
//                   step: connectEdge again, connectingColorProb
//                   and the balance-heuristic weight of connectingMisWeight
//                   (FP64 products, as the reference) — adding to the sample's
//                   image: its own pixel, or, for one-vertex eye sub-paths, the
//                   pixel the light vertex projects to (light tracing);
//   k_bpt_resolve   per pixel: each sample's image through isLegalColor and
//                   fixVignetting into the caller's sum (and sum of squares).
//
// The connection step never builds the connected path: vertex i of it is
// light vertex i (i < l) or eye vertex l + e - 1 - i, read from HBM, except
// the two connection vertices, which connectEdge changes and which live in
// registers.  Draws: the eye sub-path takes the Philox stream of (pixel,
// sample) from draw 0, the light sub-path the same stream from draw 2^30;
// the connections draw nothing.  Homogeneous media take part (their
// free-flight densities are origin densities of the MIS weights);
// heterogeneous ones do not (their densities need an integration along every
// link) and scenes with one are refused by the caller.
#include <algorithm>
#include <memory>

#include "render_launch.h"
#include "wr_context.h"
#include "wr_shade.cuh"

namespace wr {

constexpr uint32_t BPT_LIGHT_DIM0 = 0x40000000u;
constexpr int BPT_MAX_RECORDS = 32;  // records per sub-path: max_path_len + 2
constexpr double INV_PI_D = 0.31830988618379067153776752674503;
constexpr double PI_D = 3.1415926535897932384626433832795;
constexpr double EPS_D = 1e-5;

// ---------------------------------------------------------------------------
// vertex records: {o, oP}, {d, dP}, {rad, inside},
// {contact normal, contact + 2 | photon type << 28 | delta << 31}
// ---------------------------------------------------------------------------
struct VtxStore {
    float4* base;
    uint32_t nsamp;  // samples in the batch (the stride between vertex k and k + 1)
    __device__ __forceinline__ float4* at(uint32_t sid, int k) const {
        return base + 4 * ((size_t)k * nsamp + sid);
    }
    __device__ __forceinline__ void put(uint32_t sid, int k, const PRay& r) const {
        float4* v = at(sid, k);
        v[0] = make_float4(r.o.x, r.o.y, r.o.z, r.oP);
        v[1] = make_float4(r.d.x, r.d.y, r.d.z, r.dP);
        v[2] = make_float4(r.rad.x, r.rad.y, r.rad.z, __int_as_float(r.inside));
        v[3] = make_float4(r.cnorm.x, r.cnorm.y, r.cnorm.z,
                           __uint_as_float((uint32_t)(r.contact + 2) | ((uint32_t)r.ptype << 28) |
                                           (r.delta ? 0x80000000u : 0u)));
    }
    __device__ __forceinline__ PRay get(uint32_t sid, int k) const {
        const float4* v = at(sid, k);
        const float4 a = __ldg(v), b = __ldg(v + 1), c = __ldg(v + 2), n = __ldg(v + 3);
        PRay r = ray_default();
        r.o = mk(a.x, a.y, a.z);
        r.oP = a.w;
        r.d = mk(b.x, b.y, b.z);
        r.dP = b.w;
        r.rad = mk(c.x, c.y, c.z);
        r.inside = __float_as_int(c.w);
        r.cnorm = mk(n.x, n.y, n.z);
        const uint32_t w = __float_as_uint(n.w);
        r.contact = (int)(w & 0x0fffffffu) - 2;
        r.ptype = (uint8_t)((w >> 28) & 3u);
        r.delta = (w >> 31) != 0;
        return r;
    }
};

// The weight's technique set: BidirectionalPathTracer's connections only, or
// VCMTracer's connections and merges (vcmTracer.cpp:225-330) with merge
// radius `radius` and nVM = pixel count; `merge`: the path was made by a merge.
struct MisKind {
    bool vcm, merge;
    float radius;
    double nvm;
};

struct BptParams {
    uint64_t seed;
    uint32_t s0;          // first sample index of the batch
    uint32_t nsamp;       // batch samples: npix * spp_in_batch
    uint32_t npix;
    uint32_t max_path_len;
    float pf;             // traversal prune factor
    int stack_cap;
    VtxStore eye, light;
    uint32_t* counts;     // per sample: eye records | light records << 8 (bytes 0 and 1, little-endian)
    float* film;          // per sample slot of the batch: npix * 3 floats
    uint2* cand;          // connection candidates with a light sub-path (l >= 1): {sample, l | e << 8}
    uint2* vis;           // connections that contribute: visible candidates and whole eye paths
    unsigned long long* ncand;  // [0]: entries of cand, [1]: entries of vis, [2]: light points, [3]: merges,
                                // [4]: sub-paths handed out
    // vertex merging (WR_MODE_VCM); per sample slot s of the batch, the hash grid of hashgrid.hxx
    bool vcm;
    const float* radii;   // merge radius of each slot's iteration
    uint2* pts;           // light points {sample, record}
    int* bbox;            // per slot: ordered-int keys of min x, y, z, max x, y, z
    int* head;            // per slot: npix buckets, first point or -1
    int* next;            // per point: next point of its bucket or -1
    uint4* merges;        // merges found by the grid queries: {sample, eye record, point}
    unsigned long long merge_cap;
    // progressive photon mapping (WR_MODE_PHOTON_MAP): light sub-paths only,
    // each photon's throughput
    bool light_only;
    float4* tput;
    // with participating media the INVOL photons have their own grid: grid
    // nslots + slot of the same arrays; their point entries carry bit 31
    bool vol_grid;
    uint32_t nslots;      // slots (iterations) of the batch
    unsigned int* err;    // error bits of the traversals inside the weights (heterogeneous media)
};

// the weight's technique set for a sample of this batch
__device__ __forceinline__ MisKind mis_kind(const BptParams& P, uint32_t sid, bool merge) {
    MisKind K;
    K.vcm = P.vcm;
    K.merge = merge;
    K.radius = P.vcm ? __ldg(&P.radii[sid / P.npix]) : 0.f;
    K.nvm = (double)P.npix;
    return K;
}

// appends `item` for the lanes with `ok` at consecutive places of list[*count++]
// (one atomic per warp); every lane of the warp must call it
__device__ __forceinline__ void warp_append(bool ok, uint2 item, uint2* list, unsigned long long* count) {
    constexpr unsigned FULL = 0xffffffffu;
    const unsigned lane = threadIdx.x & 31u;
    const unsigned want = __ballot_sync(FULL, ok);
    if (!want) return;
    const int leader = __ffs(want) - 1;
    unsigned long long base = 0;
    if ((int)lane == leader) base = atomicAdd(count, (unsigned long long)__popc(want));
    base = __shfl_sync(FULL, base, leader);
    if (ok) list[base + __popc(want & ((1u << lane) - 1u))] = item;
}

// Persistent: each lane takes sub-paths from a counter (eye sub-paths of
// samples 0..nsamp-1, then their light sub-paths; light only for photon
// mapping) and advances its sub-path one record per turn, so that a lane
// whose path ends takes the next one instead of waiting for the warp's
// longest path.  A turn: the lane stores its current record and scatters
// (MCRenderer::samplePath, mcRenderer.cpp:16-57), then every lane with a ray
// traces it at one call site (the first ray of a sub-path too: the camera
// ray unfiltered (camera.cpp:52), which a filter with no inside and no
// contact object is, the emitted ray with NoSelfCondition).
template <bool HM>
__global__ void __launch_bounds__(128) k_bpt_subpaths(RenderScene S, BptParams P, unsigned int* __restrict__ err) {
    constexpr unsigned FULL = 0xffffffffu;
    extern __shared__ uint32_t s_stack[];
    uint32_t* stack = s_stack + threadIdx.x;
    const int stride = blockDim.x;
    const unsigned lane = threadIdx.x & 31u;
    const unsigned long long total = (P.light_only ? 1ull : 2ull) * P.nsamp;
    unsigned long long* counter = P.ncand + 4;
    bool active = false, exhausted = false, light = false;
    uint32_t sid = 0, depth = 0;
    int n = 0;
    PRay prev = ray_default(), ray = ray_default();
    InsideStack st;
    st.reset(-1);
    PathRng g;
    g.init(0, 0, 0, 0);
    for (;;) {
        // refill idle lanes
        const bool want = !active && !exhausted;
        const unsigned need = __ballot_sync(FULL, want);
        bool fresh = false, has_ray = false;
        if (need) {
            const int leader = __ffs(need) - 1;
            unsigned long long base = 0;
            if ((int)lane == leader) base = atomicAdd(counter, (unsigned long long)__popc(need));
            base = __shfl_sync(FULL, base, leader);
            if (want) {
                const unsigned long long w = base + __popc(need & ((1u << lane) - 1u));
                if (w >= total) {
                    exhausted = true;
                } else {
                    light = P.light_only || w >= P.nsamp;
                    sid = (uint32_t)(light && !P.light_only ? w - P.nsamp : w);
                    const uint32_t pixel = sid % P.npix, sample = P.s0 + sid / P.npix;
                    n = 0;
                    depth = 0;
                    active = true;
                    fresh = true;
                    if (!light) {
                        g.init(P.seed, pixel, sample, 0);
                        ray = camera_ray(S.cam, pixel, g);
                        has_ray = true;
                    } else if (S.nlights == 0) {  // no emitter: an empty light sub-path
                        reinterpret_cast<uint8_t*>(P.counts + sid)[1] = 0;
                        active = false;
                        fresh = false;
                    } else {
                        // Scene::genLightSample -> AbstractObject::genSurfaceSample (abstractObj.cpp:18-52)
                        g.init(P.seed, pixel, sample, BPT_LIGHT_DIM0);
                        ray = light_sample(S, g);
                        ray.iobj = -1;
                        if (ray.contact >= 0) {
                            ray.inside = __ldg(&S.light_inside[ray.contact]);
                            has_ray = true;
                        }
                    }
                }
            }
        }
        if (__ballot_sync(FULL, active) == 0) {
            if (__ballot_sync(FULL, !exhausted) == 0) break;
            continue;
        }
        // one record of a running sub-path (the samplePath step up to its next ray)
        PRay next = ray_default();
        if (active && !fresh) {
            const VtxStore& out = light ? P.light : P.eye;
            out.put(sid, n++, prev);
            PRay term = ray_default();
            term.o = prev.o;
            term.rad = mk(0, 0, 0);
            term.delta = true;
            const int self = prev.inside >= 0 ? prev.inside : prev.iobj;
            bool done = false;
            if (self < 0) {
                out.put(sid, n++, term);
                done = true;
            } else {
                next = scatter<HM>(S, self, prev, g, st);
                if (length(next.d) < 0.5f) {
                    out.put(sid, n++, next);
                    done = true;
                } else if (depth + 1 > P.max_path_len) {
                    out.put(sid, n++, term);
                    done = true;
                } else {
                    st.set_top(next.inside);
                    ray = next;
                    has_ray = true;
                }
            }
            if (done) {
                reinterpret_cast<uint8_t*>(P.counts + sid)[light ? 1 : 0] = (uint8_t)n;
                active = false;
            }
        }
        // every ray of the turn at one call site
        Hit h;
        h.t = __int_as_float(0x7f800000);
        h.slot = -1;
        if (has_ray) {
            RayQ q = make_rayq(ray.o, ray.d, S.tree.scene_mag);
            q.pf = P.pf;
            const bool filt = !(fresh && !light);
            h = trace_closest<true, true>(S.tree, q, filt ? ray.inside : -1, filt ? ray.contact : -1, stack, stride,
                                          P.stack_cap, err);
        }
        if (active && fresh) {  // the sub-path's first record, its hit set
            if (light) {
                if (has_ray && h.slot >= 0 && h.t > 0.f) set_hit(S, ray, h);  // `if(dist > 0)`
                else ray.iobj = -1;
            } else {
                set_hit(S, ray, h);
            }
            prev = ray;
            st.reset(prev.inside);
        } else if (active && has_ray) {
            if (h.slot < 0) {  // a scattered ray that escapes: it and the terminating record end the path
                const VtxStore& out = light ? P.light : P.eye;
                PRay term = ray_default();
                term.o = prev.o;
                term.rad = mk(0, 0, 0);
                term.delta = true;
                out.put(sid, n++, ray);
                out.put(sid, n++, term);
                reinterpret_cast<uint8_t*>(P.counts + sid)[light ? 1 : 0] = (uint8_t)n;
                active = false;
            } else {
                set_hit(S, ray, h);
                prev = ray;
                depth++;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// the connection step
// ---------------------------------------------------------------------------
// Camera::getPixelSolidAngle (camera.cpp:125-131)
__device__ __forceinline__ float pixel_solid_angle(const CamParams& C, uint32_t pid) {
    const uint32_t x = pid % C.width, y = pid / C.width;
    const float xc = (float)((double)x + 0.5 - (C.width / 2.0)), yc = (float)((C.height / 2.0) - 0.5 - (double)y);
    const float dist = sqrtf(xc * xc + yc * yc + C.ipd * C.ipd);
    return C.ipd / powf(dist, 3.f);
}

// Ray::evalDirectionProbability (ray.cpp:32-38) with the objects' overrides;
// `same` is the reference's `&inRay == &outRay` (an emitted ray)
__device__ float bpt_dir_prob(const RenderScene& S, f3 in_d, const PRay& out, bool same, uint32_t cam_pixel) {
    if (out.contact == CAMERA_OBJ) return (float)(1.0 / (double)pixel_solid_angle(S.cam, cam_pixel));
    const int o = out.contact >= 0 ? out.contact : out.inside;
    if (o < 0) return 0.f;
    const wr_object_desc* m = &S.objs[o];
    const uint32_t t = __ldg(&m->type);
    if (t == WR_MAT_DIFFUSE || t == WR_MAT_GLOSSY) {  // diffuseObj.h:22-27, glossyObj.h:25-31
        if (out.contact < 0) return 0.f;
        const f3 al = ld3(m->albedo);
        float p = al.x;
        if (al.y > p) p = al.y;
        if (al.z > p) p = al.z;
        const float dn = dot(out.cnorm, out.d);
        if (t == WR_MAT_DIFFUSE) return p * (dn > 0.f ? (float)((double)dn * INV_PI_D) : 0.f);
        const float ct = (double)dn > EPS_D ? dn : (float)EPS_D;
        const float power = __ldg(&m->power);
        return p * (float)(((double)power + 1.0) * (double)powf(ct, power) * (INV_PI_D * 0.5));
    }
    if (t == WR_MAT_ANISO) {  // anisotropicGlossyObj.h:47-52, anisotropicPhong.h:19-33
        if (out.contact < 0) return 0.f;
        const f3 N = out.cnorm;
        if (!(dot(in_d, N) <= 0.f && dot(out.d, N) >= 0.f)) return 0.f;
        const f3 h = normalize(out.d - in_d);
        float pdf = aniso_half_pdf(__ldg(&m->nu), __ldg(&m->nv), N, h);
        pdf /= 4.f * fabsf(dot(in_d, h));
        return pdf;
    }
    if (t == WR_MAT_HOMOGENEOUS || t == WR_MAT_HETEROGENEOUS) {
        // homogeneousVolume.cpp:216-223, HeterogeneousVolume.cpp:430-437 (a boundary record is delta)
        if (out.delta) return 0.f;
        const f3 ss = ld3(m->sigma_s), st = ss + ld3(m->sigma_a);
        return luminance(ss) / luminance(st) * hg_value(__ldg(&m->g), in_d, out.d);
    }
    if (t == WR_MAT_REFLECTIVE) {  // reflectiveObj.h:44-46 with the unparenthesised MAX_VEC_COMP
        const f3 c = ld3(m->albedo);
        return c.x > c.y ? c.x : (c.y > c.z ? c.y : c.z);
    }
    // AbstractObject::evalDirectionProbability (abstractObj.cpp:61-68)
    return same ? (float)(INV_PI_D * 0.25f) * 2.f : 0.f;
}

// Ray::evalBSDF (ray.cpp:15-22); the camera's evaluateBSDF is AbstractObject's (1, 1, 1)
__device__ __forceinline__ f3 bpt_eval_bsdf(const RenderScene& S, f3 in_d, const PRay& out) {
    if (out.contact == CAMERA_OBJ) return mk(1, 1, 1);
    return eval_bsdf(S, in_d, out);
}

// Ray::evalOriginProbability (ray.cpp:24-30) of the link from a record at
// `in_o` whose inside object is `in_inside` to a record at `out_o`: 1 but in
// a homogeneous medium, whose surface / medium free-flight density over the
// distance (homogeneousVolume.cpp:209-214, homogeneousVolume.h:40-53) it is
// ---- heterogeneous media in the weights: the reference's ray-marched
// integrals (HeterogeneousVolume.cpp:171-248) -------------------------------
constexpr int HV_STACK = 96;  // traversal stack of these helpers (thread-local memory)

struct HvCtx {  // what their own traversal needs
    float pf;
    int cap;
    unsigned int* err;
};
__device__ __forceinline__ HvCtx hv_ctx(const BptParams& P) {
    return HvCtx{P.pf, P.stack_cap < HV_STACK ? P.stack_cap : HV_STACK, P.err};
}

// HeterogeneousVolume::check (:171-185) of a record inside the medium (its
// origin is inside the mesh by the record's inside object): the first hit of
// the record's ray under its NoSelfCondition
__device__ __forceinline__ bool hv_first_hit(const RenderScene& S, const PRay& r, const HvCtx& hc, float& idist) {
    uint32_t stack[HV_STACK];
    RayQ q = make_rayq(r.o, r.d, S.tree.scene_mag);
    q.pf = hc.pf;
    const Hit h = trace_closest<true, true>(S.tree, q, r.inside, r.contact, stack, 1, hc.cap, hc.err);
    if (h.slot < 0 || !(h.t > 0.f)) return false;
    idist = h.t;
    return true;
}

// integrateDensity (:187-210): Simpson's rule over the density alone (no
// sigma_t) along the record's ray up to min(dist, first hit), accumulated in
// double into a float
__device__ __noinline__ float hv_integrate(const RenderScene& S, const PRay& r, float dist, const HvCtx& hc) {
    const wr_object_desc* m = &S.objs[r.inside];
    float idist, acc = 0.f;
    if (!hv_first_hit(S, r, hc, idist)) return acc;
    dist = dist < idist ? dist : idist;
    f3 p = r.o;
    const unsigned n = (unsigned)ceilf(dist / (2.f * __ldg(&m->step_size)));
    const double ss = (double)(dist / (float)n), mult = (1.0 / 6.0) * ss;
    const f3 full = r.d * (float)ss, half = full * 0.5f;
    float n1 = hv_density_ref(S, r.inside, p);
    for (unsigned i = 0; i < n; i++) {
        const float n2 = hv_density_ref(S, r.inside, p + half), n3 = hv_density_ref(S, r.inside, p + full);
        acc = (float)((double)acc + mult * (double)(n1 + n2 * 4.f + n3));
        n1 = n3;
        p = p + full;
    }
    return acc;
}

// randianceDecay (:439-445): exp(-tau) of tau (:212-235), the Simpson
// integral of sigma_t * density in float vec3 steps
__device__ __noinline__ f3 hv_transmittance(const RenderScene& S, const PRay& r, float dist, const HvCtx& hc) {
    const wr_object_desc* m = &S.objs[r.inside];
    f3 acc = mk(0, 0, 0);
    float idist;
    if (hv_first_hit(S, r, hc, idist)) {
        dist = dist < idist ? dist : idist;
        const f3 sgt = ld3(m->sigma_s) + ld3(m->sigma_a);
        f3 p = r.o;
        const unsigned n = (unsigned)ceilf(dist / (2.f * __ldg(&m->step_size)));
        const double ss = (double)(dist / (float)n), mult = (1.0 / 6.0) * ss;
        const f3 full = r.d * (float)ss, half = full * 0.5f;
        f3 n1 = sgt * hv_density_ref(S, r.inside, p);
        for (unsigned i = 0; i < n; i++) {
            const f3 n2 = sgt * hv_density_ref(S, r.inside, p + half), n3 = sgt * hv_density_ref(S, r.inside, p + full);
            acc = acc + ((n1 + n2 * 4.f) + n3) * (float)mult;
            n1 = n3;
            p = p + full;
        }
    }
    return mk(expf(-acc.x), expf(-acc.y), expf(-acc.z));
}

// HeterogeneousVolume::evalOriginProbability (:422-428): PSurface = exp(-I)
// towards a record with a contact, else pMedium = Luminance(sigma_t *
// density(end)) * exp(-I), I the density integral over the distance
__device__ __noinline__ float hv_origin_prob(const RenderScene& S, const PRay& in, f3 out_o, int out_contact,
                                            const HvCtx& hc) {
    const wr_object_desc* m = &S.objs[in.inside];
    const float d0 = length(in.o - out_o);
    const float dist = (double)d0 > EPS_D ? d0 : (float)EPS_D;
    const float tau = hv_integrate(S, in, dist, hc);
    if (out_contact != -1) return expf(-tau);
    const f3 st = ld3(m->sigma_s) + ld3(m->sigma_a);
    const float dens = hv_density_ref(S, in.inside, in.o + in.d * dist);
    return luminance(st * dens) * expf(-tau);
}

// Ray::evalOriginProbability (ray.cpp:24-30) of the linked record `in`
// towards a record at out_o: 1 outside media, else the medium's surface or
// free-flight density over their distance (homogeneousVolume.cpp:209-214,
// PSurface / pMedium of homogeneousVolume.h:40-53; heterogeneous above)
template <bool HM>
__device__ __forceinline__ float bpt_origin_prob(const RenderScene& S, const PRay& in, f3 out_o, int out_contact,
                                                 const HvCtx& hc) {
    if (in.inside < 0) return 1.f;
    const uint32_t t = obj_type(S, in.inside);
    if constexpr (HM) {
        if (t == WR_MAT_HETEROGENEOUS) return hv_origin_prob(S, in, out_o, out_contact, hc);
    }
    if (t != WR_MAT_HOMOGENEOUS) return 1.f;
    const wr_object_desc* m = &S.objs[in.inside];
    const f3 st = ld3(m->sigma_s) + ld3(m->sigma_a);
    const float d0 = length(in.o - out_o);
    const float dist = (double)d0 > 1e-5 ? d0 : (float)1e-5;
    const f3 e = mk(expf(-st.x * dist), expf(-st.y * dist), expf(-st.z * dist));
    return out_contact != -1 ? luminance(e) : luminance(vmul(st, e));
}

// Ray::radianceDecay (ray.cpp:46-50) with the heterogeneous medium's marched tau
template <bool HM>
__device__ __forceinline__ f3 bpt_decay(const RenderScene& S, const PRay& r, float dist, const HvCtx& hc) {
    if constexpr (HM) {
        if (r.inside >= 0 && obj_type(S, r.inside) == WR_MAT_HETEROGENEOUS) return hv_transmittance(S, r, dist, hc);
    }
    return radiance_decay(S, r, dist);
}

__device__ __forceinline__ bool emissive(const RenderScene& S, int o) {
    return o >= 0 && obj_type(S, o) == WR_MAT_EMISSIVE;
}

__device__ __forceinline__ float max_eps(float a) { return (double)a > EPS_D ? a : (float)EPS_D; }

// PdfWtoA (util.h:100-106) with aPdfW = 1
__device__ __forceinline__ float pdf_w_to_a(float dist, float cos_there) { return fabsf(cos_there) / (dist * dist); }

// the connected path y0..y(l-1) x(e-1)..x0 of one (l, e) pair
struct Conn {
    VtxStore eye, light;
    uint32_t sid, lsid;  // samples of the eye and of the light sub-path (different for a merge)
    int l, e, n, c;
    bool mod;
    PRay lc, ec;  // the connection vertices after connectEdge (when mod)
    __device__ __forceinline__ PRay v(int i) const {
        if (mod && i == c) return lc;
        if (mod && i == c + 1) return ec;
        return i < l ? light.get(lsid, i) : eye.get(sid, e - 1 - (i - l));
    }
};



// BidirectionalPathTracer::linkVertex (bidirPathTracer.cpp:226-243) for
// start in [0, n): the record, pointed at its neighbour on the connecting side
__device__ __forceinline__ PRay link(const Conn& C, int start, bool reverse, const PRay& vs, const PRay& ve) {
    PRay r = vs;
    if ((reverse && start > C.c) || (!reverse && start <= C.c)) return r;
    r.d = normalize(ve.o - vs.o);
    r.inside = ve.inside;
    return r;
}

// BidirectionalPathTracer::connectingMisWeight (bidirPathTracer.cpp:142-220),
// expTerm = 1; the origin densities of surface vertices are 1
// (AbstractObject::evalOriginProbability, abstractObj.cpp:54-59)
template <bool HM>
__device__ float bpt_mis_weight(const RenderScene& S, const Conn& C, uint32_t pixel, double* rev, const MisKind& K,
                               const HvCtx& hc) {
    const int n = C.n, c = C.c;
    // reverse densities, eye end first (each record read once: a window
    // v2 = v(i + 2), v1 = v(i + 1), vi = v(i) slides towards the light)
    PRay v1 = C.v(n - 1), v2 = v1;
    rev[n - 1] = v1.oP;
    for (int i = n - 2; i >= 0; i--) {
        const PRay vi = C.v(i);
        const float dist = max_eps(length(v1.o - vi.o));
        const PRay lr = link(C, i, false, vi, v1);
        rev[i] = rev[i + 1] * (double)pdf_w_to_a(dist, cos_term(S, lr));
        if (!v1.delta) {
            float dirp;
            const PRay b = link(C, i + 1, true, v1, vi);
            if (i < n - 2) {
                const PRay a = link(C, i + 2, true, v2, v1);
                dirp = bpt_dir_prob(S, a.d, b, false, pixel);
            } else {
                dirp = bpt_dir_prob(S, v1.d, v1, true, pixel);  // vertex n-1 is the camera, never re-pointed
            }
            // link(i+1, reverse).evalOriginProbability(link(i, reverse))
            const float ori = bpt_origin_prob<HM>(S, b, vi.o, vi.contact, hc);
            rev[i] *= (double)(dirp * ori);
        }
        v2 = v1;
        v1 = vi;
    }
    // direct densities, light end first, with the sum over techniques in the
    // reference's order: connection of (i, i+1), then merge at i+1
    // (window pm2 = v(i - 2), pm1 = v(i - 1), vi = v(i), vn = v(i + 1))
    PRay pm1 = v1, pm2 = v1, vi = C.v(1);
    double dir = pm1.oP, all = 0.0, self = c == -1 ? rev[0] : 0.0;
    bool can_connect = false;
    if (!pm1.delta && !vi.delta) {
        all += dir * rev[1];
        can_connect = true;
    }
    if (c == 0) self = dir * rev[1];
    for (int i = 1; i < n; i++) {
        const float dist = max_eps(length(vi.o - pm1.o));
        const PRay lr = link(C, i, true, vi, pm1);
        const float g = pdf_w_to_a(dist, cos_term(S, lr));
        const double dir_prev = dir;
        dir = dir * (double)g;
        float dirp = 1.f, ori = 1.f;
        if (!pm1.delta) {
            const PRay b = link(C, i - 1, false, pm1, vi);
            if (i > 1) {
                const PRay a = link(C, i - 2, false, pm2, pm1);
                dirp = bpt_dir_prob(S, a.d, b, false, pixel);
            } else {
                dirp = bpt_dir_prob(S, b.d, b, true, pixel);
            }
            // link(i-1).evalOriginProbability(link(i))
            ori = bpt_origin_prob<HM>(S, b, vi.o, vi.contact, hc);
            dir *= (double)(dirp * ori);
        }
        if (K.vcm && i - 1 < n - 2 && !vi.delta) {  // merging at vertex i (vcmTracer.cpp:298-318)
            double p = dir_prev * rev[i];
            if (!pm1.delta) p *= (double)dirp;
            p *= (double)(pm1.delta ? bpt_origin_prob<HM>(S, link(C, i - 1, false, pm1, vi), vi.o, vi.contact, hc)
                                    : ori);  // link(i-1).evalOriginProbability(link(i))
            p *= (double)g;
            p *= PI_D * K.radius * K.radius;
            if (vi.inside >= 0 && vi.contact == -1) p *= 4.0 / 3 * K.radius;
            if (K.merge && i - 1 == c) self = p;
            all += p * K.nvm;
        }
        PRay vn = vi;
        if (i < n - 1) {
            vn = C.v(i + 1);
            if (!vi.delta && !vn.delta) {
                all += dir * rev[i + 1];
                can_connect = true;
            }
            if (i == c) self = dir * rev[i + 1];
        }
        pm2 = pm1;
        pm1 = vi;
        vi = vn;
    }
    if (!can_connect) all += rev[0];
    if (K.merge) self *= K.nvm;
    const double w = self / all;
    return (float)(w > 0.0 ? w : 0.0);  // also VCMTracer's `!(w >= 0) -> 0`
}

// BidirectionalPathTracer::connectingColorProb (bidirPathTracer.cpp:267-290),
// each record read once (prev = v(i - 1), cur = v(i), nx = v(i + 1))
// For a merge (VCMTracer::connectingColorProb, vcmTracer.cpp:357-366) the
// light vertex's density of landing within `radius` is multiplied in.
template <bool HM>
__device__ void bpt_color_prob(const RenderScene& S, const Conn& C, const HvCtx& hc, f3& color, float& prob,
                               bool merge = false, float radius = 0.f) {
    const int n = C.n, c = C.c;
    f3 col = mk(1, 1, 1);
    float pr = 1.f;
    PRay cur = C.v(0), prev = cur;
    for (int i = 0; i < n; i++) {
        const PRay nx = i + 1 < n ? C.v(i + 1) : cur;
        col = vmul(col, cur.rad);
        float dist = 0.f;
        if (i <= c) {
            dist = max_eps(length(cur.o - nx.o));
            col = vmul(col, bpt_decay<HM>(S, cur, dist, hc));
            if (i == c) col = col * (cos_term(S, cur) * cos_term(S, nx) / (dist * dist));
        } else if (i > c + 1) {
            dist = max_eps(length(prev.o - cur.o));
            col = vmul(col, bpt_decay<HM>(S, cur, dist, hc));
        }
        if (i != c && i != c + 1) col = col * cos_term(S, cur);
        pr *= cur.dP * cur.oP;
        if (merge && i == c) {
            pr = (float)((double)pr * (PI_D * radius * radius));
            pr *= pdf_w_to_a(dist, cos_term(S, nx));  // link(c + 1, reverse): the eye vertex as connected
            pr *= bpt_origin_prob<HM>(S, cur, nx.o, nx.contact, hc);  // link(c).evalOriginProbability(link(c+1))
            if (nx.inside >= 0 && nx.contact == -1) pr = (float)((double)pr * (4.0 / 3 * radius));
        }
        prev = cur;
        cur = nx;
    }
    color = col;
    prob = pr;
}

// Camera::convToRaster / convToRaster2 and checkPixelBound (camera.cpp:148-180);
// a non-finite coordinate (a point in the camera's plane) counts as outside
__device__ bool bpt_raster(const CamParams& C, f3 p, f3 lens_o, uint32_t* pid) {
    if (C.lens_radius > 0.f) {
        const f3 dir = normalize(p - lens_o);
        const float ft = C.focal_dist / fabsf(dot(C.front, dir));
        p = lens_o + dir * ft;
    }
    const f3 v = p - C.pos;
    const float scale = C.ipd / dot(v, C.front);
    const float rx = (float)(C.width / 2.0 + (double)(dot(v, C.right) * scale));
    const float ry = (float)(C.height / 2.0 - (double)(dot(v, C.top) * scale));
    if (!(fabsf(rx) < 2.0e9f) || !(fabsf(ry) < 2.0e9f)) return false;
    const int px = (int)rx, py = (int)ry;
    if (px < 0 || py < 0 || px >= (int)C.width || py >= (int)C.height) return false;
    *pid = (uint32_t)py * C.width + (uint32_t)px;
    return true;
}

__device__ __forceinline__ void film_add(float* f, uint32_t pid, f3 c) {
    atomicAdd(f + 3 * (size_t)pid, c.x);
    atomicAdd(f + 3 * (size_t)pid + 1, c.y);
    atomicAdd(f + 3 * (size_t)pid + 2, c.z);
}

// The path-shape tests of throughputByConnecting (bidirPathTracer.cpp:74-103)
// for every (light length l, eye length e) pair of a sample, from one word
// per record: the connected path must start at an emitter; a whole eye path
// (l = 0) counts only if no two neighbours are both non-delta; no emitter
// may sit at a connection vertex; connectEdge needs both connection vertices
// non-delta.  Passing pairs with a light sub-path go to the candidate list
// (their visibility is tested next), whole eye paths straight to the list of
// contributing connections; e outer and l inner with the same loop bounds in
// every lane, so that each warp appends runs of one (l, e) pair and the later
// kernels' warps get uniform work.
__global__ void __launch_bounds__(128) k_bpt_enum(RenderScene S, BptParams P) {
    constexpr unsigned FULL = 0xffffffffu;
    const uint32_t sid = blockIdx.x * blockDim.x + threadIdx.x;
    int ne = 0, nl = 0;
    uint32_t emE = 0, dE = 0, emL = 0, dL = 0;  // bit k: record k is an emitter / delta
    if (sid < P.nsamp) {
        const uint32_t cnt = __ldg(&P.counts[sid]);
        ne = (int)(cnt & 0xffu);
        nl = (int)((cnt >> 8) & 0xffu);
        for (int k = 0; k < ne; k++) {
            const uint32_t w = __float_as_uint(__ldg(&P.eye.at(sid, k)[3].w));
            emE |= (uint32_t)emissive(S, (int)(w & 0x0fffffffu) - 2) << k;
            dE |= (w >> 31) << k;
        }
        for (int k = 0; k < nl; k++) {
            const uint32_t w = __float_as_uint(__ldg(&P.light.at(sid, k)[3].w));
            emL |= (uint32_t)emissive(S, (int)(w & 0x0fffffffu) - 2) << k;
            dL |= (w >> 31) << k;
        }
    }
    const int nrec = (int)P.max_path_len + 2;
    for (int e = 1; e <= nrec; e++) {
        for (int l = 0; l <= nrec; l++) {
            bool ok = e <= ne && l <= nl && l + e >= 2;
            if (ok) {
                if (l == 0) {
                    const uint32_t m = ~dE & (e < 32 ? (1u << e) - 1u : FULL);
                    ok = ((emE >> (e - 1)) & 1u) && (m & (m >> 1)) == 0;
                } else {
                    ok = (emL & 1u) && !(l > 1 && ((emL >> (l - 1)) & 1u)) && !((emE >> (e - 1)) & 1u) &&
                         !((dL >> (l - 1)) & 1u) && !((dE >> (e - 1)) & 1u);
                }
            }
            const uint2 item = make_uint2(sid, (uint32_t)l | ((uint32_t)e << 8));
            if (l == 0) warp_append(ok, item, P.vis, P.ncand + 1);
            else warp_append(ok, item, P.cand, P.ncand);
        }
    }
}

// connectEdge (bidirPathTracer.cpp:293-312): the connection vertices of the
// (l >= 1, e) connection, pointed at each other, with their new radiance,
// direction probability and inside objects
__device__ __forceinline__ void bpt_connect_edge(const RenderScene& S, const BptParams& P, uint32_t sid, int l, int e,
                                                 PRay& lc, PRay& ec) {
    lc = P.light.get(sid, l - 1);
    ec = P.eye.get(sid, e - 1);
    const PRay pl = l - 1 > 0 ? P.light.get(sid, l - 2) : lc;
    const PRay pe = e >= 2 ? P.eye.get(sid, e - 2) : ec;
    lc.d = normalize(ec.o - lc.o);
    ec.d = -lc.d;
    lc.dP = 1.f;
    lc.delta = false;
    lc.rad = bpt_eval_bsdf(S, l - 1 > 0 ? pl.d : lc.d, lc);
    if (lc.contact != -1 && l - 1 > 0) lc.inside = dot(lc.cnorm, lc.d) > 0.f ? pl.inside : lc.contact;
    ec.dP = 1.f;
    ec.delta = false;
    ec.rad = bpt_eval_bsdf(S, e >= 2 ? pe.d : ec.d, ec);
    if (ec.contact != -1 && e >= 2) ec.inside = dot(ec.cnorm, ec.d) > 0.f ? pe.inside : ec.contact;
}

// MCRenderer::visibilityTest (mcRenderer.cpp:59-65) of every candidate, from
// the eye vertex towards the light vertex; the visible ones join the list of
// contributing connections.  Persistent: the grid strides over the list.
__global__ void __launch_bounds__(128) k_bpt_visible(RenderScene S, BptParams P, unsigned int* __restrict__ err) {
    extern __shared__ uint32_t s_stack[];
    uint32_t* stack = s_stack + threadIdx.x;
    const int stride = blockDim.x;
    const unsigned long long total = P.ncand[0];
    const unsigned long long step = (unsigned long long)gridDim.x * blockDim.x;
    // every lane runs the same number of turns (warp_append needs the whole warp)
    const unsigned long long turns = (total + step - 1) / step;
    for (unsigned long long t = 0; t < turns; t++) {
        const unsigned long long i = t * step + (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
        bool ok = false;
        uint2 c = make_uint2(0, 0);
        if (i < total) {
            c = P.cand[i];
            PRay lc, ec;
            bpt_connect_edge(S, P, c.x, (int)(c.y & 0xffu), (int)(c.y >> 8), lc, ec);
            RayQ q = make_rayq(ec.o, ec.d, S.tree.scene_mag);
            q.pf = P.pf;
            const Hit h = trace_closest<true, true>(S.tree, q, ec.inside, ec.contact, stack, stride, P.stack_cap, err);
            ok = h.slot < 0 || (double)(h.t - length(ec.o - lc.o)) >= -EPS_D;
        }
        warp_append(ok, c, P.vis, P.ncand + 1);
    }
}

// One contributing connection (sample sid, light length l, eye length e) of
// throughputByConnecting: connectEdge, the colour / probability product and
// the MIS weight, added to the sample's image.
template <bool HM>
__device__ void bpt_connect_one(const RenderScene& S, const BptParams& P, uint32_t sid, int l, int e) {
    const int W = l + e;
    const uint32_t pixel = sid % P.npix;
    float* film = P.film + 3 * (size_t)P.npix * (sid / P.npix);
    Conn C;
    C.eye = P.eye;
    C.light = P.light;
    C.sid = sid;
    C.lsid = sid;
    C.l = l;
    C.e = e;
    C.n = W;
    C.c = l - 1;
    C.mod = false;
    if (l > 0) {
        bpt_connect_edge(S, P, sid, l, e, C.lc, C.ec);
        C.mod = true;
    }
    f3 col;
    float prob;
    const HvCtx hc = hv_ctx(P);
    bpt_color_prob<HM>(S, C, hc, col, prob);
    if (prob == 0.f) return;
    if (length(col) == 0.f) return;
    double rev[2 * BPT_MAX_RECORDS];
    const float w = bpt_mis_weight<HM>(S, C, pixel, rev, mis_kind(P, sid, false), hc);
    f3 contrib = divs(col, prob) * w;
    if (contrib.x == 0.f && contrib.y == 0.f && contrib.z == 0.f) return;
    if (e > 1) {
        film_add(film, pixel, contrib);
        return;
    }
    // the light vertex seen by the camera: splat where it projects
    const PRay cr = C.v(W - 1), lv = C.v(W - 2);
    uint32_t pid;
    if (!bpt_raster(S.cam, lv.o, cr.o, &pid)) return;
    float sa;
    if (S.cam.lens_radius > 0.f) {  // Camera::computeSolidAngle (camera.cpp:133-142)
        const float ct = dot(normalize(lv.o - cr.o), S.cam.front);
        sa = S.cam.ipd / powf(S.cam.ipd / ct, 3.f);
    } else {
        sa = pixel_solid_angle(S.cam, pid);
    }
    const float f = (float)(1.0 / (double)sa);
    contrib = contrib * (f / (float)P.npix);
    film_add(film, pid, contrib);
}

// persistent: the grid strides over the contributing connections, 32
// consecutive ones (mostly one (l, e) pair) per warp
// MINB: resident blocks per SM the registers are fitted to (5 for the
// bidirectional weights: 96 registers, +5 % over 4 blocks; VCM's weights
// spill at that size and take 4; the marching instantiation 1)
template <bool HM, int MINB>
__global__ void __launch_bounds__(128, MINB) k_bpt_connect(RenderScene S, BptParams P) {
    const unsigned long long total = P.ncand[1];
    for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        const uint2 c = P.vis[i];
        bpt_connect_one<HM>(S, P, c.x, (int)(c.y & 0xffu), (int)(c.y >> 8));
    }
}

// ---------------------------------------------------------------------------
// vertex merging (VCMTracer::throughputByMerging, vcmTracer.cpp:175-223) and
// the reference's hash grid (hashgrid.hxx): npix buckets per iteration, cell
// size 2 r, the spatial hash of GetCellIndex, the 8 cells nearest a query and
// a bounding box over every particle — including the npix placeholder points
// at the origin that VCMTracer's point vector starts with (they never
// contribute, so only their place in the box is kept: the box starts at the
// origin).  The buckets are linked lists; a bucket reached through two of the
// 8 cells is walked twice, as in the reference.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int fkey(float f) {
    const int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7fffffff;
}
__device__ __forceinline__ float fkey_inv(int k) { return __int_as_float(k >= 0 ? k : k ^ 0x7fffffff); }

struct GridView {
    f3 bmin, bmax;
    float radius, inv_cell;
    const int* head;  // this slot's buckets
    uint32_t nb;
};

__device__ __forceinline__ GridView grid_view(const BptParams& P, uint32_t slot) {
    GridView G;
    const int* k = P.bbox + 6 * slot;
    G.bmin = mk(fkey_inv(k[0]), fkey_inv(k[1]), fkey_inv(k[2]));
    G.bmax = mk(fkey_inv(k[3]), fkey_inv(k[4]), fkey_inv(k[5]));
    G.radius = __ldg(&P.radii[slot]);
    G.inv_cell = 1.f / (G.radius * 2.f);
    G.head = P.head + (size_t)slot * P.npix;
    G.nb = P.npix;
    return G;
}

// HashGrid::GetCellIndex (hashgrid.hxx:185-202)
__device__ __forceinline__ uint32_t grid_bucket(const GridView& G, int cx, int cy, int cz) {
    const uint32_t x = (uint32_t)cx, y = (uint32_t)cy, z = (uint32_t)cz;
    return ((x * 73856093u) ^ (y * 19349663u) ^ (z * 83492791u)) % G.nb;
}
__device__ __forceinline__ uint32_t grid_bucket(const GridView& G, f3 p) {
    const f3 d = p - G.bmin;
    return grid_bucket(G, (int)floorf(G.inv_cell * d.x), (int)floorf(G.inv_cell * d.y), (int)floorf(G.inv_cell * d.z));
}

// The light points of each sample (vcmTracer.cpp:40-54): light records 1..
// before the first emitter, delta records skipped; their bounding box per slot.
__global__ void __launch_bounds__(128) k_vcm_points(RenderScene S, BptParams P) {
    const uint32_t sid = blockIdx.x * blockDim.x + threadIdx.x;
    int nl = 0;
    if (sid < P.nsamp) nl = (int)((__ldg(&P.counts[sid]) >> 8) & 0xffu);
    const int nrec = (int)P.max_path_len + 2;
    f3 lo = mk(0, 0, 0), hi = mk(0, 0, 0), vlo = lo, vhi = hi;
    bool any = false, vany = false, alive = true;
    for (int i = 1; i < nrec; i++) {  // equal loop bounds in every lane: warp_append needs the whole warp
        bool ok = false;
        uint2 item = make_uint2(sid, (uint32_t)i);
        if (alive && i < nl) {
            const PRay r = P.light.get(sid, i);
            if (emissive(S, r.contact)) alive = false;
            else if (!r.delta) {
                // photon mapping keeps OUTVOL records as surface photons and
                // INVOL records as volume photons (photonMap.cpp:74-85)
                const bool vol = P.light_only && r.ptype == PT_INVOL;
                ok = !P.light_only || r.ptype == PT_OUTVOL || vol;
                if (ok && vol) {
                    item.y |= 0x80000000u;
                    vlo = mk(fminf(vlo.x, r.o.x), fminf(vlo.y, r.o.y), fminf(vlo.z, r.o.z));
                    vhi = mk(fmaxf(vhi.x, r.o.x), fmaxf(vhi.y, r.o.y), fmaxf(vhi.z, r.o.z));
                    vany = true;
                } else if (ok) {
                    lo = mk(fminf(lo.x, r.o.x), fminf(lo.y, r.o.y), fminf(lo.z, r.o.z));
                    hi = mk(fmaxf(hi.x, r.o.x), fmaxf(hi.y, r.o.y), fmaxf(hi.z, r.o.z));
                    any = true;
                }
            }
        }
        warp_append(ok, item, P.pts, P.ncand + 2);
    }
    // the box: every lane's box includes the origin, so a lane without points
    // is neutral; a warp within one slot reduces first and adds once
    constexpr unsigned FULL = 0xffffffffu;
    const uint32_t slot = sid / P.npix;
    const bool uniform = __all_sync(FULL, __shfl_sync(FULL, slot, 0) == slot && sid < P.nsamp);
    if (uniform) {
        const int k0 = __reduce_min_sync(FULL, fkey(lo.x)), k1 = __reduce_min_sync(FULL, fkey(lo.y)),
                  k2 = __reduce_min_sync(FULL, fkey(lo.z)), k3 = __reduce_max_sync(FULL, fkey(hi.x)),
                  k4 = __reduce_max_sync(FULL, fkey(hi.y)), k5 = __reduce_max_sync(FULL, fkey(hi.z));
        if (__ballot_sync(FULL, any) && (threadIdx.x & 31u) == 0) {
            int* k = P.bbox + 6 * slot;
            atomicMin(k + 0, k0);
            atomicMin(k + 1, k1);
            atomicMin(k + 2, k2);
            atomicMax(k + 3, k3);
            atomicMax(k + 4, k4);
            atomicMax(k + 5, k5);
        }
    } else if (any) {
        int* k = P.bbox + 6 * slot;
        atomicMin(k + 0, fkey(lo.x));
        atomicMin(k + 1, fkey(lo.y));
        atomicMin(k + 2, fkey(lo.z));
        atomicMax(k + 3, fkey(hi.x));
        atomicMax(k + 4, fkey(hi.y));
        atomicMax(k + 5, fkey(hi.z));
    }
    if (vany) {  // volume photons: the slot's volume grid (its box also includes the origin)
        int* k = P.bbox + 6 * (P.nslots + slot);
        atomicMin(k + 0, fkey(vlo.x));
        atomicMin(k + 1, fkey(vlo.y));
        atomicMin(k + 2, fkey(vlo.z));
        atomicMax(k + 3, fkey(vhi.x));
        atomicMax(k + 4, fkey(vhi.y));
        atomicMax(k + 5, fkey(vhi.z));
    }
}

// HashGrid::Build: every point into its bucket's list
__global__ void __launch_bounds__(256) k_vcm_link(BptParams P) {
    const unsigned long long total = P.ncand[2];
    for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        const uint2 pt = P.pts[i];
        const uint32_t gi = pt.x / P.npix + ((pt.y >> 31) ? P.nslots : 0u);
        const GridView G = grid_view(P, gi);
        const f3 pos = xyz(__ldg(P.light.at(pt.x, (int)(pt.y & 0xffu))));
        const uint32_t b = grid_bucket(G, pos);
        P.next[i] = atomicExch(P.head + (size_t)gi * P.npix + b, (int)i);
    }
}

// One merge: light records [0, idx) of sample lsid, then eye records i..0 of
// sample sid (Query::Process, vcmTracer.cpp:188-201).  Adds w * colour / prob.
template <bool HM>
__device__ void vcm_merge_one(const RenderScene& S, const BptParams& P, uint32_t sid, int i, uint32_t lsid, int idx,
                              double* rev, f3& contrib) {
    Conn C;
    C.eye = P.eye;
    C.light = P.light;
    C.sid = sid;
    C.lsid = lsid;
    C.l = idx;
    C.e = i + 1;
    C.n = idx + i + 1;
    C.c = idx - 1;
    // connectEdge for a merge (vcmTracer.cpp:375-409): the light record is only
    // re-pointed, the eye vertex evaluated towards it
    PRay lc = P.light.get(lsid, idx - 1), ec = P.eye.get(sid, i);
    const PRay pe = P.eye.get(sid, i - 1);
    lc.d = normalize(ec.o - lc.o);
    ec.d = -lc.d;
    ec.dP = 1.f;
    ec.delta = false;
    ec.rad = bpt_eval_bsdf(S, pe.d, ec);
    if (ec.contact != -1) ec.inside = dot(ec.cnorm, ec.d) > 0.f ? pe.inside : ec.contact;
    C.lc = lc;
    C.ec = ec;
    C.mod = true;
    const MisKind K = mis_kind(P, sid, true);
    f3 col;
    float prob;
    const HvCtx hc = hv_ctx(P);
    bpt_color_prob<HM>(S, C, hc, col, prob, true, K.radius);
    if (length(col) == 0.f || prob == 0.f) return;
    const float w = bpt_mis_weight<HM>(S, C, sid % P.npix, rev, K, hc);
    contrib = contrib + divs(col * w, prob);
}

// One thread per (sample, eye vertex): every non-delta eye vertex before the
// sample's first emitter is a query of the hash grid (HashGrid::Process,
// hashgrid.hxx:97-161); neighbouring lanes take neighbouring samples at the
// same depth.  Each light point within the radius is a merge, appended to
// the merge list for k_vcm_eval; when the list is full the merge is
// evaluated here.  Each merge's contribution / nVM goes to the sample's pixel
// (the reference adds a query's sum / nVM: the same up to the order of the
// additions).
template <bool HM>
__global__ void __launch_bounds__(128) k_vcm_merge(RenderScene S, BptParams P) {
    const int nrec = (int)P.max_path_len + 2;
    const unsigned long long t = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (unsigned long long)P.nsamp * (unsigned long long)(nrec - 1)) return;
    const uint32_t sid = (uint32_t)(t % P.nsamp);
    const int i = 1 + (int)(t / P.nsamp);
    const int ne = (int)(__ldg(&P.counts[sid]) & 0xffu);
    if (i >= ne) return;
    // the sample's loop over its eye records stops at the first emitter (vcmTracer.cpp:213-215)
    for (int j = 1; j <= i; j++) {
        const uint32_t w = __float_as_uint(__ldg(P.eye.at(sid, j) + 3).w);
        if (emissive(S, (int)(w & 0x0fffffffu) - 2)) return;
    }
    const PRay q = P.eye.get(sid, i);
    if (q.delta) return;
    const uint32_t slot = sid / P.npix;
    const GridView G = grid_view(P, slot);
    const float rr = G.radius * G.radius;
    const unsigned long long npts = P.ncand[2];
    double rev[2 * BPT_MAX_RECORDS];
    f3 contrib = mk(0, 0, 0);
    const f3 dmin = q.o - G.bmin, dmax = G.bmax - q.o;
    if (!(dmin.x < 0.f || dmin.y < 0.f || dmin.z < 0.f || dmax.x < 0.f || dmax.y < 0.f || dmax.z < 0.f)) {
        const f3 cp = mk(G.inv_cell * dmin.x, G.inv_cell * dmin.y, G.inv_cell * dmin.z);
        const f3 cf = mk(floorf(cp.x), floorf(cp.y), floorf(cp.z));
        const int px = (int)cf.x, py = (int)cf.y, pz = (int)cf.z;
        const f3 fr = cp - cf;
        const int pxo = px + (fr.x < 0.5f ? -1 : 1), pyo = py + (fr.y < 0.5f ? -1 : 1),
                  pzo = pz + (fr.z < 0.5f ? -1 : 1);
        for (int jc = 0; jc < 8; jc++) {
            const int cx = (jc & 4) ? pxo : px, cy = (jc & 2) ? pyo : py, cz = (jc & 1) ? pzo : pz;
            // a list is at most every point of the batch long (bounded walk)
            unsigned long long guard = 0;
            for (int k = __ldg(&G.head[grid_bucket(G, cx, cy, cz)]); k >= 0 && guard++ < npts;
                 k = __ldg(&P.next[k])) {
                const uint2 pt = P.pts[k];
                const f3 pos = xyz(__ldg(P.light.at(pt.x, (int)pt.y)));
                const float dist = length(q.o - pos);
                if (!(dist * dist <= rr)) continue;
                const unsigned long long m = atomicAdd(P.ncand + 3, 1ull);
                if (m < P.merge_cap) P.merges[m] = make_uint4(sid, (uint32_t)i, (uint32_t)k, 0u);
                else vcm_merge_one<HM>(S, P, sid, i, pt.x, (int)pt.y, rev, contrib);
            }
        }
    }
    const f3 own = divs(contrib, (float)P.npix);
    if (own.x != 0.f || own.y != 0.f || own.z != 0.f)
        film_add(P.film + 3 * (size_t)P.npix * slot, sid % P.npix, own);
}

// the listed merges, one per thread and step (persistent)
template <bool HM>
__global__ void __launch_bounds__(128) k_vcm_eval(RenderScene S, BptParams P) {
    const unsigned long long n = P.ncand[3], total = n < P.merge_cap ? n : P.merge_cap;
    double rev[2 * BPT_MAX_RECORDS];
    for (unsigned long long t = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (unsigned long long)gridDim.x * blockDim.x) {
        const uint4 m = P.merges[t];
        const uint2 pt = P.pts[m.z];
        f3 contrib = mk(0, 0, 0);
        vcm_merge_one<HM>(S, P, m.x, (int)m.y, pt.x, (int)pt.y, rev, contrib);
        if (contrib.x != 0.f || contrib.y != 0.f || contrib.z != 0.f)
            film_add(P.film + 3 * (size_t)P.npix * (m.x / P.npix), m.x % P.npix, divs(contrib, (float)P.npix));
    }
}

// ---------------------------------------------------------------------------
// progressive photon mapping (PhotonMap::renderPixels, photonMap.cpp:20-148,
// as built: PPM on, no ray marching, ANI_PM off): the light points of VCM are
// the photons, in the same hash grid
// ---------------------------------------------------------------------------
constexpr uint32_t PPM_MERGE_LEN = 10;  // photonMap.cpp:9

// each photon's throughput up to its record (photonMap.cpp:228-236)
template <bool HM>
__global__ void __launch_bounds__(256) k_ppm_tput(RenderScene S, BptParams P) {
    const unsigned long long total = P.ncand[2];
    const HvCtx hc = hv_ctx(P);
    for (unsigned long long k = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; k < total;
         k += (unsigned long long)gridDim.x * blockDim.x) {
        const uint2 pt = P.pts[k];
        const int idx = (int)(pt.y & 0xffu);
        f3 t = mk(1, 1, 1);
        PRay cur = P.light.get(pt.x, 0);
        for (int i = 0; i < idx; i++) {
            const PRay nx = P.light.get(pt.x, i + 1);
            t = vmul(t, divs(divs(cur.rad, cur.dP), cur.oP));
            t = t * cos_term(S, cur);
            t = vmul(t, bpt_decay<HM>(S, cur, length(cur.o - nx.o), hc));
            cur = nx;
        }
        t = divs(t, cur.oP);
        P.tput[k] = make_float4(t.x, t.y, t.z, 0.f);
    }
}

// Query::Process (photonMap.cpp:219-246): one photon's density estimate at
// the eye record `out` (direction towards the camera side); a volume photon's
// kernel is over N r^3
__device__ __forceinline__ f3 ppm_photon(const RenderScene& S, const BptParams& P, uint32_t k, const PRay& out,
                                         float radius, bool volume = false) {
    const uint2 pt = P.pts[k];
    const int idx = (int)(pt.y & 0xffu);
    const float4 tp = __ldg(&P.tput[k]);
    const PRay prevl = P.light.get(pt.x, idx - 1);
    const f3 pos = xyz(__ldg(P.light.at(pt.x, idx)));
    const f3 color = vmul(mk(tp.x, tp.y, tp.z), eval_bsdf(S, prevl.d, out));
    const float dist_sqr = powf(length(out.o - pos), 2.f);
    if (!legal(color)) return mk(0, 0, 0);
    const float x = 1.f - dist_sqr / (radius * radius);
    const float sk = 0.f > x ? 0.f : x;
    const float kernel = (float)((double)(3.f * sk * sk) / PI_D);
    return color * (volume ? kernel / ((float)P.npix * radius * radius * radius)
                           : kernel / ((float)P.npix * radius * radius));
}

// ---- the anisotropic (elliptic) photon query, photonMap.cpp:384-652 --------
// Eigen-decomposition of the symmetric [[a, b], [b, c]] by LAPACK's published
// DLAEV2 algorithm: rt1 the eigenvalue of larger magnitude, rt2 the other,
// (cs1, sn1) the unit eigenvector of rt1.
__device__ void eig2_sym(double a, double b, double c, double& rt1, double& rt2, double& cs1, double& sn1) {
    const double sm = a + c, df = a - c, adf = fabs(df), tb = b + b, ab = fabs(tb);
    const double acmx = fabs(a) > fabs(c) ? a : c, acmn = fabs(a) > fabs(c) ? c : a;
    double rt;
    if (adf > ab) {
        const double q = ab / adf;
        rt = adf * sqrt(q * q + 1.);
    } else if (adf < ab) {
        const double q = adf / ab;
        rt = ab * sqrt(q * q + 1.);
    } else {
        rt = ab * sqrt(2.);
    }
    int sgn1;
    if (sm < 0.) {
        rt1 = (sm - rt) * .5;
        sgn1 = -1;
        rt2 = acmx / rt1 * acmn - b / rt1 * b;
    } else if (sm > 0.) {
        rt1 = (sm + rt) * .5;
        sgn1 = 1;
        rt2 = acmx / rt1 * acmn - b / rt1 * b;
    } else {
        rt1 = rt * .5;
        rt2 = rt * -.5;
        sgn1 = 1;
    }
    const int sgn2 = df >= 0. ? 1 : -1;
    const double cs = df >= 0. ? df + rt : df - rt;
    if (fabs(cs) > ab) {
        const double ct = -tb / cs;
        sn1 = 1. / sqrt(ct * ct + 1.);
        cs1 = ct * sn1;
    } else if (ab == 0.) {
        cs1 = 1.;
        sn1 = 0.;
    } else {
        const double tn = -cs / tb;
        cs1 = 1. / sqrt(tn * tn + 1.);
        sn1 = tn * cs1;
    }
    if (sgn1 == sgn2) {
        const double tn = cs1;
        cs1 = -sn1;
        sn1 = tn;
    }
}

// derivatives of the anisotropic spherical Gaussian
// cos(theta) exp(-sin^2(theta) (L cos^2(phi) + M sin^2(phi))) in theta and phi
// (PhotonMap::ASG_dF_dTheta / ASG_dF_dPhi, photonMap.cpp:681-691)
__device__ double asg_dtheta(double th, double ph, double L, double M) {
    const double k = L * cos(ph) * cos(ph) + M * sin(ph) * sin(ph), st = sin(th);
    return exp(-st * st * k) * st * (2 * cos(th) * cos(th) * (-k) - 1);
}
__device__ double asg_dphi(double th, double ph, double L, double M) {
    const double k = L * cos(ph) * cos(ph) + M * sin(ph) * sin(ph), st = sin(th);
    return exp(-st * st * k) * 2 * st * st * cos(th) * sin(ph) * cos(ph) * (L - M);
}

// The ellipse of the photon query at a diffuse point of normal hn reached
// along sp from an anisotropic surface of normal N (exponents nu, nv) entered
// along in_d (photonMap.cpp:384-613): the lobe's Hessian in the half-vector
// frame and its eigenvectors (the warped frame), the fastest and slowest
// directions of the warped Gaussian at sp with their steps for an error bound
// of 0.002, projected along sp onto the hit plane.  0 with the long axis ex,
// ey = hn x ex and the axis ratio; 1 (eigenvectors within |cs| or |sn| > 0.99)
// or 2 (degenerate projection, Xi_s / Xi_f <= 1) where the reference falls
// back to the round kernel.  Mixed float / double exactly as the reference's
// vec3f and double expressions; out of line, so that its FP64 registers stay
// out of the common path of k_ppm_eye.
__device__ __noinline__ int ellipse_frame(f3 in_d, f3 N, f3 sp, f3 hn, float nu, float nv, f3& ex, f3& ey,
                                          float& ratio) {
    const double lam = (double)(nu / 2.f), miu = (double)(nv / 2.f);
    const f3 O = -in_d;
    const float on = dot(O, N);
    const f3 I = normalize(N * (2.f * on) - O);
    f3 BX, BY, BZ;
    frame_from_n(N, BX, BY, BZ);
    const f3 Xh = normalize(cross(O, N)), Yi = cross(I, Xh);
    const double dxx = (double)dot(BZ, Xh), dyx = (double)dot(BX, Xh);
    double HA = lam * (dxx * dxx) + miu * (dyx * dyx);
    HA /= 4 * ((double)on * (double)on);
    double HB = (miu - lam) * (dxx * dyx);
    HB /= (double)(4.f * on);
    double HD = miu * (dxx * dxx) + lam * (dyx * dyx);
    HD /= 4;
    double L1, M1, cs, sn;
    eig2_sym(HA, HB, HD, L1, M1, cs, sn);
    L1 = fabs(L1);
    M1 = fabs(M1);
    if (fabs(cs) > 0.99 || fabs(sn) > 0.99) return 1;
    const f3 IX = Xh * (float)cs + Yi * (float)sn;
    const f3 IY = Xh * (float)-sn + Yi * (float)cs;
    const float a0 = dot(sp, IX), b0 = dot(sp, IY);
    const float c2 = 1.f - a0 * a0 - b0 * b0;
    const float c0 = sqrtf(c2 < 0.f ? 0.f : c2 > 1.f ? 1.f : c2);
    // acos of a float argument is the C++ float overload (acosf)
    const double theta = (double)acosf(c0 < -1.f ? -1.f : c0 > 1.f ? 1.f : c0), st = sin(theta);
    const double ca = (double)a0 / st;
    const double aphi = acos(ca < -1 ? -1.0 : ca > 1 ? 1.0 : ca);
    const double phi = b0 > 0.f ? aphi : 2 * PI_D - aphi;
    const f3 SY = normalize(cross(I, sp)), SX = cross(SY, sp);
    const double dl = 0.0001;
    const double fT = asg_dtheta(theta, phi, L1, M1), fP = asg_dphi(theta, phi, L1, M1);
    const double fTT = (asg_dtheta(theta + dl, phi, L1, M1) - asg_dtheta(theta - dl, phi, L1, M1)) / (2 * dl);
    const double fPP = (asg_dphi(theta, phi + dl, L1, M1) - asg_dphi(theta, phi - dl, L1, M1)) / (2 * dl);
    const double fTP = (asg_dtheta(theta, phi + dl, L1, M1) - asg_dtheta(theta, phi - dl, L1, M1)) / (2 * dl);
    const f3 fastest = normalize(SX * (float)fT + SY * (float)(fP / st));
    const f3 slowest = cross(sp, fastest);
    const f3 ltp = normalize(mk((float)fT, (float)(fP / st), 0.f));
    const double al1 = (double)acosf(fabsf(ltp.x)), al2 = PI_D / 2 - al1;
    const double eb = 0.002;
    const double lower = cos(theta) * exp(-st * st * (L1 * cos(phi) * cos(phi) + M1 * sin(phi) * sin(phi)));
    const double xf = fabs(eb * lower / (fT * cos(al1) + fP * sin(al1) / st));
    const double xs = sqrt(fabs(2 * eb * lower /
                                (fTT * cos(al2) * cos(al2) + 2 * fTP * sin(al2) * cos(al2) / st +
                                 fPP * sin(al2) * sin(al2) / (st * st))));
    f3 HX, HY, HZ;
    frame_from_n(hn, HX, HY, HZ);
    if (fabs((double)dot(sp, I)) < EPS_D || fabs((double)dot(sp, hn)) < EPS_D || fabs(xs / xf) <= 1.0) return 2;
    // A = [Zh; Xh] (I - D Np^T / D.Np) [fastest slowest]
    const double dn = (double)dot(sp, HY);
    const float D[3] = {sp.x, sp.y, sp.z}, Np[3] = {HY.x, HY.y, HY.z};
    const double Jp[2][3] = {{HZ.x, HZ.y, HZ.z}, {HX.x, HX.y, HX.z}};
    const double Je[3][2] = {{fastest.x, slowest.x}, {fastest.y, slowest.y}, {fastest.z, slowest.z}};
    double mid[3][3], pj[2][3] = {{0, 0, 0}, {0, 0, 0}}, A[2][2] = {{0, 0}, {0, 0}};
#pragma unroll
    for (int r = 0; r < 3; r++)
#pragma unroll
        for (int c = 0; c < 3; c++) mid[r][c] = (double)(r == c) - (double)(D[r] * Np[c]) / dn;
#pragma unroll
    for (int r = 0; r < 2; r++)
#pragma unroll
        for (int c = 0; c < 3; c++)
#pragma unroll
            for (int k = 0; k < 3; k++) pj[r][c] += Jp[r][k] * mid[k][c];
#pragma unroll
    for (int r = 0; r < 2; r++)
#pragma unroll
        for (int c = 0; c < 2; c++)
#pragma unroll
            for (int k = 0; k < 3; k++) A[r][c] += pj[r][k] * Je[k][c];
    const f3 fast = (HZ * (float)A[0][0] + HX * (float)A[1][0]) * (float)xf;
    const f3 slow = (HZ * (float)A[0][1] + HX * (float)A[1][1]) * (float)xs;
    const float lr = length(slow) / length(fast);
    ratio = (float)((double)lr > 1.0 ? (double)lr : 1.0);
    ex = normalize(slow);
    ey = cross(hn, ex);
    return 0;
}

// Query::EllipseProcess (photonMap.cpp:262-298): one photon's Gaussian-kernel
// estimate in the ellipse frame (axes radius * ratio and radius), its weight
// summed into sumw and counted
__device__ __forceinline__ f3 ppm_photon_ellipse(const RenderScene& S, const BptParams& P, uint32_t k, const PRay& out,
                                                 float radius, f3 ex, f3 ey, float ratio, double& sumw, int& count) {
    const uint2 pt = P.pts[k];
    const float4 tp = __ldg(&P.tput[k]);
    const PRay prevl = P.light.get(pt.x, (int)(pt.y & 0xffu) - 1);
    const f3 pos = xyz(__ldg(P.light.at(pt.x, (int)(pt.y & 0xffu))));
    const f3 color = vmul(mk(tp.x, tp.y, tp.z), eval_bsdf(S, prevl.d, out));
    if (!legal(color)) return mk(0, 0, 0);
    const f3 hp = pos - out.o;
    const float X = dot(hp, ex), Y = dot(hp, ey);
    const float A = radius * ratio, B = radius;
    const float md = X * X / (A * A) + Y * Y / (B * B);
    const float w = (float)(exp(-(double)md / 2) / (2 * PI_D));
    sumw += w;
    count++;
    const float conv = (float)(1.0 / ((double)P.npix * PI_D * radius * radius));
    return (color * w) * conv;
}

// the 8 cells of HashGrid::Process (hashgrid.hxx:96-165) around q: every
// photon within the radius through `visit(k)`
template <typename F>
__device__ __forceinline__ void ppm_grid_walk(const BptParams& P, const GridView& G, f3 q, F&& visit) {
    const f3 dmin = q - G.bmin, dmax = G.bmax - q;
    if (dmin.x < 0.f || dmin.y < 0.f || dmin.z < 0.f || dmax.x < 0.f || dmax.y < 0.f || dmax.z < 0.f) return;
    const f3 cp = mk(G.inv_cell * dmin.x, G.inv_cell * dmin.y, G.inv_cell * dmin.z);
    const f3 cf = mk(floorf(cp.x), floorf(cp.y), floorf(cp.z));
    const int px = (int)cf.x, py = (int)cf.y, pz = (int)cf.z;
    const f3 fr = cp - cf;
    const int pxo = px + (fr.x < 0.5f ? -1 : 1), pyo = py + (fr.y < 0.5f ? -1 : 1), pzo = pz + (fr.z < 0.5f ? -1 : 1);
    const float rr = G.radius * G.radius;
    const unsigned long long npts = P.ncand[2];
    for (int j = 0; j < 8; j++) {
        const int cx = (j & 4) ? pxo : px, cy = (j & 2) ? pyo : py, cz = (j & 1) ? pzo : pz;
        unsigned long long guard = 0;  // a list is at most every point of the batch long
        for (int k = __ldg(&G.head[grid_bucket(G, cx, cy, cz)]); k >= 0 && guard++ < npts; k = __ldg(&P.next[k])) {
            const uint2 pt = P.pts[k];
            const float dist = length(q - xyz(__ldg(P.light.at(pt.x, (int)(pt.y & 0xffu)))));
            if (!(dist * dist <= rr)) continue;
            visit((uint32_t)k);
        }
    }
}

// an eye segment inside a medium before the estimate's record, marched after
// the whole eye path (its draws come after the path's)
struct PpmSeg {
    f3 o, d;
    float dist;
    int inside, contact;
};

// One thread per sample: the eye path of PhotonMap::sampleMergePath (at most
// 10 bounces) up to its first emitter (its radiance) or diffuse record (the
// photon density there, throughputByDensityEstimation), times the camera
// record's factors, into the sample's image.  Without media the records after
// that one are never read, so the path is not continued.  MEDIA: the merge
// path's dispatch (a record inside a medium goes on with the object its ray
// hits; a boundary record whose ray hits a medium jumps to that hit), the
// whole path sampled (the march offsets are drawn after it), and each segment
// inside a medium before the estimate ray-marched against the volume photons
// (photonMap.cpp:306-367): color = Tr * surface + volume.
template <bool MEDIA, bool HM>
__global__ void __launch_bounds__(128) k_ppm_eye(RenderScene S, BptParams P, unsigned int* __restrict__ err) {
    extern __shared__ uint32_t s_stack[];
    uint32_t* stack = s_stack + threadIdx.x;
    const int stride = blockDim.x;
    const uint32_t sid = blockIdx.x * blockDim.x + threadIdx.x;
    if (sid >= P.nsamp) return;
    const uint32_t pixel = sid % P.npix, slot = sid / P.npix, sample = P.s0 + slot;
    PathRng g;
    g.init(P.seed, pixel, sample, 0);
    const PRay cam = camera_ray(S.cam, pixel, g);
    PRay prev = cam;
    {
        RayQ q = make_rayq(cam.o, cam.d, S.tree.scene_mag);
        q.pf = P.pf;
        const Hit h = trace_closest<false, true>(S.tree, q, -1, -1, stack, stride, P.stack_cap, err);
        set_hit(S, prev, h);
    }
    InsideStack st;
    st.reset(prev.inside);
    f3 surf = mk(0, 0, 0);
    f3 pdir = mk(0, 0, 0);  // direction of the record before `prev` (eyeMergePath[i-2])
    const GridView G = grid_view(P, slot);
    constexpr int NSEG = MEDIA ? (int)PPM_MERGE_LEN + 2 : 1;
    PpmSeg seg[NSEG];
    int nseg = 0;
    bool merged = false;  // the estimate's record is found; later records only advance the draws
    for (uint32_t depth = 0;; depth++) {
        int self;
        if constexpr (MEDIA) self = prev.inside >= 0 && !is_volume(S, prev.inside) ? prev.inside : prev.iobj;
        else self = prev.inside >= 0 ? prev.inside : prev.iobj;
        if (self < 0) break;  // the terminate record: nothing to estimate
        PRay next;
        if constexpr (MEDIA) {
            PRay cur = prev;
            const bool jump = self == prev.iobj && is_volume(S, self) && prev.contact >= 0 && is_volume(S, prev.contact);
            if (jump) {  // photonMap.cpp:165-168
                cur.o = cur.o + cur.d * cur.idist;
                cur.idist = 0.f;
            }
            if (jump && obj_type(S, self) == WR_MAT_HETEROGENEOUS && cur.inside == self) {
                // the medium's check() from the moved origin: inside its mesh
                // (or on it as the record's contact), then the first hit
                float chk = 0.f;
                if (cur.contact == self || inside_mesh(S, self, cur.o)) {
                    RayQ q = make_rayq(cur.o, cur.d, S.tree.scene_mag);
                    q.pf = P.pf;
                    const Hit h =
                        trace_closest<true, true>(S.tree, q, cur.inside, cur.contact, stack, stride, P.stack_cap, err);
                    if (h.slot >= 0 && h.t > 0.f) chk = h.t;
                }
                bool del = false;
                float ps = 1.f;
                next = scatter_heterogeneous_ref(S, self, cur, g, st, &del, &ps, chk);
            } else {
                next = scatter<HM>(S, self, cur, g, st);
            }
        } else {
            next = scatter(S, self, prev, g, st);
        }
        const bool ended = length(next.d) < 0.5f;
        if (!ended && depth + 1 > PPM_MERGE_LEN) break;  // cut: `next` is not a record
        if (!merged) {
            if constexpr (MEDIA) {
                if (prev.inside >= 0 && is_volume(S, prev.inside) && nseg < NSEG)
                    seg[nseg++] = PpmSeg{prev.o, prev.d, max_eps(length(prev.o - next.o)), prev.inside, prev.contact};
            }
            if (emissive(S, next.contact)) {
                surf = next.rad;
                merged = true;
            } else if (next.contact >= 0 && obj_type(S, next.contact) == WR_MAT_DIFFUSE) {  // nonSpecular()
                PRay out = next;
                out.d = -prev.d;
                // reached through an anisotropic record: the elliptic estimate
                f3 ex = mk(0, 0, 0), ey = mk(0, 0, 0);
                float ratio = 1.f;
                const bool ell = prev.contact >= 0 && obj_type(S, prev.contact) == WR_MAT_ANISO &&
                                 ellipse_frame(pdir, prev.cnorm, prev.d, next.cnorm, __ldg(&S.objs[prev.contact].nu),
                                               __ldg(&S.objs[prev.contact].nv), ex, ey, ratio) == 0;
                double sumw = 0.0;
                int count = 0;
                ppm_grid_walk(P, G, next.o, [&](uint32_t k) {
                    surf = surf + (ell ? ppm_photon_ellipse(S, P, k, out, G.radius, ex, ey, ratio, sumw, count)
                                       : ppm_photon(S, P, k, out, G.radius));
                });
                if (ell) {  // Query::weightScale (photonMap.cpp:300-302): vec3f /= float
                    const float d = (float)(sumw / count);
                    if (d != 0.f) surf = mk(surf.x / d, surf.y / d, surf.z / d);
                }
                merged = true;
            }
            if (merged && nseg == 0) break;  // no march: nothing left to draw for
        }
        if (ended) break;
        st.set_top(next.inside);
        RayQ q = make_rayq(next.o, next.d, S.tree.scene_mag);
        q.pf = P.pf;
        const Hit h = trace_closest<true, true>(S.tree, q, next.inside, next.contact, stack, stride, P.stack_cap, err);
        if (h.slot < 0) break;  // `next` was the last record and is checked above
        pdir = prev.d;
        prev = next;
        set_hit(S, prev, h);
    }
    f3 Tr = mk(1, 1, 1), vol = mk(0, 0, 0);
    if constexpr (MEDIA) {
        const HvCtx hc = hv_ctx(P);
        const GridView V = grid_view(P, P.nslots + slot);
        for (int k = 0; k < nseg; k++) {
            PRay vr = ray_default();
            vr.o = seg[k].o;
            vr.d = seg[k].d;
            vr.inside = seg[k].inside;
            vr.contact = seg[k].contact;
            // N = dist / stepSize steps (at least 1; bounded), from a random offset
            const float nf = seg[k].dist / __ldg(&S.objs[vr.inside].step_size);
            int N = nf < (float)(1 << 24) ? (int)nf : (1 << 24);
            if (N == 0) N++;
            const float step = seg[k].dist / (float)N;
            const float offset = step * g.next();
            float t = offset;
            Tr = vmul(Tr, bpt_decay<HM>(S, vr, offset, hc));
            for (int j = 0; j < N; j++, t += step) {
                PRay out = vr;
                out.d = -vr.d;
                out.o = vr.o + vr.d * t;
                out.contact = -1;
                f3 c = mk(0, 0, 0);
                ppm_grid_walk(P, V, out.o, [&](uint32_t kk) { c = c + ppm_photon(S, P, kk, out, V.radius, true); });
                Tr = vmul(Tr, bpt_decay<HM>(S, out, step, hc));
                vol = vol + vmul(c, Tr) * step;
            }
        }
    }
    // color = Tr * SurfaceColor + VolumeColor, times eyeMergePath[0]'s factors (photonMap.cpp:614-623)
    const f3 f = divs(divs(cam.rad * cos_term(S, cam), cam.dP), cam.oP);
    const f3 c = vmul(vmul(Tr, surf) + vol, f);
    float* fl = P.film + 3 * ((size_t)slot * P.npix + pixel);
    fl[0] += c.x;
    fl[1] += c.y;
    fl[2] += c.z;
}

// each sample's image: isLegalColor, fixVignetting, into the caller's film
__global__ void k_bpt_resolve(CamParams cam, float* __restrict__ film, uint32_t npix, uint32_t slots,
                              float* __restrict__ sum, float* __restrict__ sumsq) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npix) return;
    f3 acc = mk(0, 0, 0), acc2 = mk(0, 0, 0);
    for (uint32_t b = 0; b < slots; b++) {
        float* f = film + 3 * ((size_t)b * npix + p);
        f3 c = mk(f[0], f[1], f[2]);
        f[0] = f[1] = f[2] = 0.f;
        if (!legal(c)) c = mk(0, 0, 0);
        c = fix_vignetting(cam, c, p);
        acc = acc + c;
        acc2 = acc2 + vmul(c, c);
    }
    float* s = sum + 3 * (size_t)p;
    s[0] += acc.x;
    s[1] += acc.y;
    s[2] += acc.z;
    if (sumsq) {
        float* s2 = sumsq + 3 * (size_t)p;
        s2[0] += acc2.x;
        s2[1] += acc2.y;
        s2[2] += acc2.z;
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
struct BptState {
    DeviceBuffer eye, light, counts, film, cand, vis;
    DeviceBuffer pts, next, head, bbox, radii, merges;  // vertex merging
    DeviceBuffer tput;                                  // photon mapping
    std::vector<float> h_radii;
};

// VCMTracer's merge radius of iteration s (vcmTracer.cpp:27), alpha = 2/3,
// computed on the host with the C library's powf and sqrtf
float vcm_radius(float base, uint32_t s) {
    const float alpha = (float)(2.0 / 3);
    const float r = base * sqrtf(powf((float)(s + 1), alpha - 1.f));
    return (double)r > EPS_D ? r : (float)EPS_D;
}

int render_bidirectional(wr_ctx* ctx, const RenderScene& S, const RenderParams& RP, uint32_t spp_offset,
                         uint32_t spp, float* d_sum, float* d_sumsq, unsigned int* err, cudaStream_t stream,
                         int kind, float base_radius, bool hetero, bool media) {
    if (RP.max_path_len + 2 > (uint32_t)BPT_MAX_RECORDS)
        return set_error(ctx, WR_ERR_INVALID_ARGUMENT, "bidirectional mode: max_path_len is limited to 30");
    const bool vcm = kind == BIDIR_VCM, ppm = kind == BIDIR_PHOTON_MAP, grid_on = vcm || ppm;
    if (!ctx->bidir) ctx->bidir = std::make_shared<BptState>();
    BptState& st = *static_cast<BptState*>(ctx->bidir.get());
    const uint32_t npix = S.cam.width * S.cam.height;
    const uint32_t nrec = RP.max_path_len + 2;
    // a batch of whole samples-per-pixel: vertex records of both sub-paths
    // (64 B each), the counts, the lists and the batch's images in about 1 GiB
    const bool vol_grid = ppm && media;  // photon mapping's second grid, for the volume photons
    const uint32_t ngrid = vol_grid ? 2u : 1u;
    const size_t per_sample = (ppm ? 1ull : 2ull) * nrec * 64 + 4 + 12 + (ppm ? 0 : 16ull * nrec * (nrec + 1)) +
                              (grid_on ? 12ull * nrec + 4ull * ngrid : 0) + (vcm ? 128 : 0) + (ppm ? 16ull * nrec : 0);
    const uint64_t max_samples = std::max<uint64_t>(npix, (1ull << 30) / per_sample);
    const uint32_t per_batch = (uint32_t)std::min<uint64_t>(spp, std::max<uint64_t>(1, max_samples / npix));
    const uint64_t nsamp = (uint64_t)npix * per_batch;
    if (nsamp > 0xffffffffull) return set_error(ctx, WR_ERR_INVALID_ARGUMENT, "image too large");
    // a batch is at least one sample of every pixel (an iteration of the
    // reference's loop); it must fit in the context's device-memory budget
    if ((uint64_t)per_sample * nsamp > ctx->memory_budget)
        return set_error(ctx, WR_ERR_OUT_OF_MEMORY,
                         "bidirectional / VCM / photon-mapping scratch for one sample of every pixel (" +
                             std::to_string((uint64_t)per_sample * nsamp) + " bytes) exceeds the device-memory budget");
    if (!ppm) WR_CUDA(ctx, st.eye.reserve(64ull * nrec * nsamp));
    WR_CUDA(ctx, st.light.reserve(64ull * nrec * nsamp));
    WR_CUDA(ctx, st.counts.reserve(4ull * nsamp + 48));
    if (!ppm) {
        WR_CUDA(ctx, st.cand.reserve(8ull * nrec * (nrec + 1) * nsamp));
        WR_CUDA(ctx, st.vis.reserve(8ull * nrec * (nrec + 1) * nsamp));
    }
    const size_t film_bytes = 12ull * nsamp;
    if (st.film.bytes < film_bytes) {
        WR_CUDA(ctx, st.film.reserve(film_bytes));
        WR_CUDA(ctx, cudaMemsetAsync(st.film.p, 0, st.film.bytes, stream));
    }
    BptParams P{};
    P.seed = RP.seed;
    P.npix = npix;
    P.max_path_len = RP.max_path_len;
    P.pf = prune_factor(RP.flags);
    P.stack_cap = RP.stack_cap;
    P.err = err;
    P.eye.base = st.eye.as<float4>();
    P.light.base = st.light.as<float4>();
    P.counts = st.counts.as<uint32_t>();
    P.film = st.film.as<float>();
    P.cand = st.cand.as<uint2>();
    P.vis = st.vis.as<uint2>();
    P.vcm = vcm;
    P.light_only = ppm;
    P.vol_grid = vol_grid;
    P.nslots = 1;
    if (grid_on) {
        WR_CUDA(ctx, st.pts.reserve(8ull * nrec * nsamp));
        WR_CUDA(ctx, st.next.reserve(4ull * nrec * nsamp));
        WR_CUDA(ctx, st.head.reserve(4ull * ngrid * nsamp));
        WR_CUDA(ctx, st.bbox.reserve(24ull * ngrid * per_batch));
        WR_CUDA(ctx, st.radii.reserve(4ull * ngrid * per_batch));
        P.pts = st.pts.as<uint2>();
        P.next = st.next.as<int>();
        P.head = st.head.as<int>();
        P.bbox = st.bbox.as<int>();
        P.radii = st.radii.as<float>();
    }
    if (vcm) {
        // the merge list: 8 merges per sample of the batch (more are evaluated where found)
        P.merge_cap = 8ull * nsamp;
        WR_CUDA(ctx, st.merges.reserve(16ull * P.merge_cap));
        P.merges = st.merges.as<uint4>();
    }
    if (ppm) {
        WR_CUDA(ctx, st.tput.reserve(16ull * nrec * nsamp));
        P.tput = st.tput.as<float4>();
    }
    // the five counters live after the per-sample counts (8-byte aligned)
    P.ncand = reinterpret_cast<unsigned long long*>(st.counts.as<char>() + ((4ull * nsamp + 7) & ~7ull));
    // scenes with a heterogeneous medium take the kernels that march its
    // integrals in the weights; the others compile without those calls
    const auto k_subpaths = hetero ? k_bpt_subpaths<true> : k_bpt_subpaths<false>;
    const auto k_connect = hetero ? k_bpt_connect<true, 1> : vcm ? k_bpt_connect<false, 4> : k_bpt_connect<false, 5>;
    const auto k_merge = hetero ? k_vcm_merge<true> : k_vcm_merge<false>;
    const auto k_eval = hetero ? k_vcm_eval<true> : k_vcm_eval<false>;
    const auto k_tput = hetero ? k_ppm_tput<true> : k_ppm_tput<false>;
    const auto k_eye = !media ? k_ppm_eye<false, false> : hetero ? k_ppm_eye<true, true> : k_ppm_eye<true, false>;
    const int block = 128;
    const size_t smem = (size_t)RP.stack_cap * block * sizeof(uint32_t);
    if (smem > 48 * 1024) {
        WR_CUDA(ctx, cudaFuncSetAttribute(k_subpaths, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        WR_CUDA(ctx, cudaFuncSetAttribute(k_bpt_visible, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        WR_CUDA(ctx, cudaFuncSetAttribute(k_eye, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    }
    int per_sm = 0, per_sm_v = 0;
    WR_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_connect, block, 0));
    WR_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_v, k_bpt_visible, block, smem));
    const int connect_grid = std::max(1, per_sm) * std::max(1, ctx->num_sms);
    const int visible_grid = std::max(1, per_sm_v) * std::max(1, ctx->num_sms);
    const int stride_grid = std::max(1, ctx->num_sms) * 8;
    int per_sm_s = 0;
    WR_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_s, k_subpaths, block, smem));
    const int subpath_grid = std::max(1, per_sm_s) * std::max(1, ctx->num_sms);
    for (uint32_t done = 0; done < spp; done += per_batch) {
        const uint32_t b = std::min(per_batch, spp - done);
        P.s0 = spp_offset + done;
        P.nsamp = npix * b;
        P.eye.nsamp = P.light.nsamp = P.nsamp;
        const int grid = (int)((P.nsamp + block - 1) / block);
        WR_CUDA(ctx, cudaMemsetAsync(P.ncand, 0, 5 * sizeof(unsigned long long), stream));
        k_subpaths<<<subpath_grid, block, smem, stream>>>(S, P, err);
        WR_CUDA(ctx, cudaGetLastError());
        if (grid_on) {  // the batch's hash grids: one per slot (iteration), a second one for volume photons
            P.nslots = b;
            st.h_radii.resize((size_t)ngrid * b);
            for (uint32_t k = 0; k < ngrid * b; k++) st.h_radii[k] = vcm_radius(base_radius, P.s0 + k % b);
            WR_CUDA(ctx, cudaMemcpyAsync(st.radii.p, st.h_radii.data(), 4ull * ngrid * b, cudaMemcpyHostToDevice,
                                         stream));
            WR_CUDA(ctx, cudaMemsetAsync(P.bbox, 0, 24ull * ngrid * b, stream));
            WR_CUDA(ctx, cudaMemsetAsync(P.head, 0xff, 4ull * ngrid * P.nsamp, stream));
            k_vcm_points<<<grid, block, 0, stream>>>(S, P);
            WR_CUDA(ctx, cudaGetLastError());
            k_vcm_link<<<stride_grid, 256, 0, stream>>>(P);
            WR_CUDA(ctx, cudaGetLastError());
            ctx->kernel_launches += 2;
        }
        if (ppm) {
            k_tput<<<stride_grid, 256, 0, stream>>>(S, P);
            WR_CUDA(ctx, cudaGetLastError());
            k_eye<<<grid, block, smem, stream>>>(S, P, err);
            WR_CUDA(ctx, cudaGetLastError());
            ctx->kernel_launches += 2;
        } else {
            k_bpt_enum<<<grid, block, 0, stream>>>(S, P);
            WR_CUDA(ctx, cudaGetLastError());
            k_bpt_visible<<<visible_grid, block, smem, stream>>>(S, P, err);
            WR_CUDA(ctx, cudaGetLastError());
            k_connect<<<connect_grid, block, 0, stream>>>(S, P);
            WR_CUDA(ctx, cudaGetLastError());
            ctx->kernel_launches += 3;
        }
        if (vcm) {
            k_merge<<<(unsigned)((P.nsamp * (unsigned long long)(nrec - 1) + block - 1) / block), block, 0, stream>>>(S, P);
            WR_CUDA(ctx, cudaGetLastError());
            k_eval<<<connect_grid, block, 0, stream>>>(S, P);
            WR_CUDA(ctx, cudaGetLastError());
            ctx->kernel_launches += 2;
        }
        k_bpt_resolve<<<(npix + 255) / 256, 256, 0, stream>>>(S.cam, P.film, npix, b, d_sum, d_sumsq);
        WR_CUDA(ctx, cudaGetLastError());
        ctx->kernel_launches += 2;
    }
    return WR_OK;
}

}  // namespace wr
