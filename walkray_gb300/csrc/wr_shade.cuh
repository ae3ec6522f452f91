// wr_shade.cuh — per-path shading on sm_103a: camera rays, the material
// scatter() functions, media, and the reference's throughput product.
//
// Semantics follow WalkRay's PathTracer (pathTracer.cpp:21-68) and
// MCRenderer::samplePath (mcRenderer.cpp:16-57): the same path-vertex records,
// the same draw order per material (so draw d of a path is the same Philox
// number on the GPU and in the oracle), and the throughput factors applied in
// the reference's order:  for every vertex i but the last
//     color *= cos_i;  color *= decay_i(|o_{i+1} - o_i|);  color *= rad_i / oP_i / dP_i
// and for the last one only the last factor.  Differences from the reference,
// all statistical (no change of expectation):
//  * shading arithmetic is FP32 with CUDA's math library where the reference
//    mixes in double temporaries and glibc;
//  * findInsideObject on a refraction/medium exit is replaced by a per-path
//    stack of enclosing objects (equal for closed, properly nested meshes);
//  * heterogeneous media use delta tracking on the same trilinear density
//    instead of Simpson quadrature + Newton inversion (the reference's
//    estimator has quadrature bias; delta tracking has none).
#pragma once

#include "../../include/walkray.h"
#include "wr_traverse.cuh"

namespace wr {

constexpr int CAMERA_OBJ = -2;
constexpr int INSIDE_STACK = 4;
constexpr float PI_F = 3.14159265358979323846f;
constexpr float INV_PI_F = 0.31830988618379067154f;
constexpr float EPS_F = 1e-5f;

struct GridDev {
    uint32_t nx, ny, nz;
    float p0[3], p1[3];
    float majorant;  // max of the raw density (times density_scale and sigma_t in use)
    const float* data;
};

// camera of one render (Camera::setup / generateRay, camera.cpp:6-60); the
// image plane distance is in pixels, so it scales with the resolution
struct CamParams {
    f3 pos, focus, front, right, top;
    uint32_t width, height;
    float ipd, lens_radius, focal_dist;
    int inside;  // inside object of camera rays
};

struct RenderScene {
    DevTree tree;
    const wr_object_desc* objs;
    uint32_t num_objs;
    const uint32_t* tri_slot;  // global triangle id -> slot
    CamParams cam;             // the scene's own camera
    // lights (SurfaceSampler, surfaceSampler.cpp:7-23)
    uint32_t nlights;
    const int* light_obj;
    const float* light_thresh;
    float light_area;
    const float* obj_area;
    const float* pick_prob;
    const float* tri_thresh;  // cumulative triangle areas, indexed by global triangle id
    const GridDev* grids;
    const int* light_inside;  // per object: the object enclosing an emitter (-1 none; lights only)
};

// ---------------------------------------------------------------------------
// scene access
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t obj_type(const RenderScene& S, int o) { return __ldg(&S.objs[o].type); }
__device__ __forceinline__ bool is_volume(const RenderScene& S, int o) {
    uint32_t t = obj_type(S, o);
    return t == WR_MAT_HOMOGENEOUS || t == WR_MAT_HETEROGENEOUS;
}
__device__ __forceinline__ float obj_ior(const RenderScene& S, int o) {
    uint32_t t = obj_type(S, o);
    return (t == WR_MAT_REFRACTIVE || t == WR_MAT_HOMOGENEOUS || t == WR_MAT_HETEROGENEOUS) ? __ldg(&S.objs[o].ior)
                                                                                            : 1.0f;
}
__device__ __forceinline__ f3 ld3(const float* p) { return mk(__ldg(p), __ldg(p + 1), __ldg(p + 2)); }

// face normal of object o's local triangle t (Mesh::getWorldNormal, mesh.h:47-56)
__device__ __forceinline__ f3 obj_normal(const RenderScene& S, int o, uint32_t t) {
    uint32_t tb = __ldg(&S.objs[o].tri_begin), tc = __ldg(&S.objs[o].tri_count);
    if (t >= tc) t = tc ? tc - 1 : 0;  // the reference indexes out of range here; clamp
    const TriRec* r = S.tree.tris + __ldg(&S.tri_slot[tb + t]);
    return face_normal(xyz(__ldg(&r->v0)), xyz(__ldg(&r->v1)), xyz(__ldg(&r->v2)));
}

// ---------------------------------------------------------------------------
// path vertex (the reference Ray, ray.h:10-31)
// ---------------------------------------------------------------------------
struct PRay {
    f3 o, d, rad;
    float oP, dP;
    int iobj;       // hit object or -1
    float idist;
    uint32_t itri;  // hit triangle, object-local
    f3 inorm;       // face normal of the hit triangle
    int inside;
    int contact;    // object, CAMERA_OBJ or -1
    f3 cnorm;       // contact normal (valid when contact != -1)
    bool delta;     // isDeltaDirection (read by the bidirectional renderer only)
    uint8_t ptype;  // Ray::photonType (ray.h:12; read by photon mapping only)
};
// Ray::PhotonType
constexpr uint8_t PT_INVOL = 0, PT_OUTVOL = 1, PT_NOUSE = 2, PT_HITVOL = 3;

__device__ __forceinline__ PRay ray_default() {
    PRay r;
    r.o = mk(0, 0, 0);
    r.d = mk(0, 0, 0);
    r.rad = mk(1, 1, 1);
    r.oP = r.dP = 1.f;
    r.iobj = -1;
    r.idist = 0.f;
    r.itri = 0;
    r.inorm = mk(0, 0, 0);
    r.inside = -1;
    r.contact = -1;
    r.cnorm = mk(0, 0, 0);
    r.delta = false;
    r.ptype = PT_OUTVOL;
    return r;
}

// per-path stack of enclosing objects; top == current inside object
// Four named registers rather than an array: a runtime index into an array
// would put the stack (and the path state around it) in local memory.
struct InsideStack {
    int v0, v1, v2, v3;
    int n;
    __device__ __forceinline__ int get(int k) const { return k == 0 ? v0 : (k == 1 ? v1 : (k == 2 ? v2 : v3)); }
    __device__ __forceinline__ void put(int k, int x) {
        v0 = k == 0 ? x : v0;
        v1 = k == 1 ? x : v1;
        v2 = k == 2 ? x : v2;
        v3 = k == 3 ? x : v3;
    }
    __device__ __forceinline__ void reset(int top) {
        n = 0;
        v0 = v1 = v2 = v3 = -1;
        if (top >= 0) put(n++, top);
    }
    __device__ __forceinline__ int top() const { return n > 0 ? get(n - 1) : -1; }
    // object enclosing the exit point of `self` (what findInsideObject(outRay, self) finds for nested meshes)
    __device__ __forceinline__ int below(int self) const {
#pragma unroll
        for (int k = INSIDE_STACK - 1; k >= 0; k--)
            if (k < n && get(k) == self) return k > 0 ? get(k - 1) : -1;
        return n > 0 && get(n - 1) != self ? get(n - 1) : -1;
    }
    __device__ __forceinline__ void set_top(int obj) {
        // a ray's inside object changed: entering pushes, leaving pops
        if (obj == top()) return;
#pragma unroll
        for (int k = INSIDE_STACK - 1; k >= 0; k--)
            if (k < n && get(k) == obj) {
                n = k + 1;
                return;
            }
        if (obj < 0) {
            n = 0;
            return;
        }
        if (n < INSIDE_STACK) put(n++, obj);
        else put(n - 1, obj);
    }
};

// Ray::cosineTerm (ray.cpp:52-58)
__device__ __forceinline__ float cos_term(const RenderScene& S, const PRay& r) {
    float c = 1.f;
    bool has_cos = r.contact == CAMERA_OBJ || (r.contact >= 0 && !is_volume(S, r.contact));
    if (r.contact != -1 && has_cos && length(r.d) > 0.5f) c = fabsf(dot(r.cnorm, r.d));
    return c > EPS_F ? c : EPS_F;
}

// ---------------------------------------------------------------------------
// samplers
// ---------------------------------------------------------------------------
// Frame::setFromN (frame.h:30-49)
__device__ __forceinline__ void frame_from_n(f3 w, f3& X, f3& Y, f3& Z) {
    Y = w;
    if (fabsf(w.x) > EPS_F) {
        X = normalize(cross(mk(0, 1, 0), w));
        Z = cross(X, Y);
    } else {
        Z = normalize(cross(mk(1, 0, 0), w));
        X = cross(Y, Z);
    }
}
__device__ __forceinline__ f3 to_world(f3 X, f3 Y, f3 Z, f3 l) { return (X * l.x + Y * l.y) + Z * l.z; }
__device__ __forceinline__ f3 mirror_dir(f3 N, f3 d) { return normalize((N * (-dot(N, d))) * 2.f + d); }

// RotateMatrix(axis, angle) * vec4(v, 0) (util.h:40-54)
__device__ __forceinline__ f3 rotate_about(f3 a, float angle, f3 v) {
    float s, c;
    sincosf(angle, &s, &c);
    const float _c = 1.f - c;
    const float m00 = c + _c * a.x * a.x, m01 = _c * a.x * a.y - s * a.z, m02 = _c * a.x * a.z + s * a.y;
    const float m10 = _c * a.x * a.y + s * a.z, m11 = c + _c * a.y * a.y, m12 = _c * a.y * a.z - s * a.x;
    const float m20 = _c * a.x * a.z - s * a.y, m21 = _c * a.y * a.z + s * a.x, m22 = c + _c * a.z * a.z;
    return mk((v.x * m00 + v.y * m01) + v.z * m02, (v.x * m10 + v.y * m11) + v.z * m12,
              (v.x * m20 + v.y * m21) + v.z * m22);
}

// DiffuseBSDF::sampleBSDF (diffuseBsdf.h:21-30) + CosHemiSphereSampler
__device__ __forceinline__ f3 diffuse_sample(f3 albedo, f3 N, PathRng& g, f3& out, float& pdf) {
    f3 X, Y, Z;
    frame_from_n(N, X, Y, Z);
    const float a = g.next(), b = g.next();
    const float t2 = sqrtf(1.f - b);
    float s, c;
    sincosf(2.f * PI_F * a, &s, &c);
    out = to_world(X, Y, Z, mk(s * t2, sqrtf(b), c * t2));
    const float dn = dot(N, out);
    pdf = dn > 0.f ? dn * INV_PI_F : 0.f;
    return albedo * INV_PI_F;
}

// IsotropicPhong::sampleBSDF (isotropicPhong.h:20-38) + PowerCosHemiSphereSampler
__device__ __forceinline__ f3 phong_sample(f3 albedo, float power, f3 in, f3 N, PathRng& g, f3& out, float& pdf) {
    f3 X, Y, Z;
    frame_from_n(N, X, Y, Z);
    const float a = g.next(), b = g.next();
    const float t2 = powf(b, 1.f / (power + 1.f));
    const float t3 = sqrtf(fmaxf(0.f, 1.f - t2 * t2));
    float s, c;
    sincosf(2.f * PI_F * a, &s, &c);
    out = to_world(X, Y, Z, mk(s * t3, t2, c * t3));
    const float dn = dot(N, out);
    pdf = dn > 0.f ? (power + 1.f) * powf(dn, power) * (INV_PI_F * 0.5f) : 0.f;
    const f3 R = mirror_dir(N, in);
    const f3 rho = albedo * ((power + 2.f) * 0.5f * INV_PI_F);
    const float dRW = dot(R, out);
    if (dot(out, N) < 0.f) {
        out = mk(0, 0, 0);
        return mk(EPS_F, EPS_F, EPS_F);
    }
    return rho * powf(dRW > 0.f ? dRW : 0.f, power);
}

// IsotropicPhong's BRDF with directions sampled about the mirror direction R
// (WR_RENDER_PHONG_MIRROR): density (n+1)/(2 pi) (R.w)^n over the sphere, the
// lobe's own shape, so f cos / pdf = albedo (n+2)/(n+1) cos stays bounded.
// The BRDF is zero where R.w <= 0, and the density covers every direction
// where it is not, so the expectation is the reference's; a sample below the
// surface ends the path with zero radiance.  Same draws as phong_sample.
__device__ __forceinline__ f3 phong_sample_mirror(f3 albedo, float power, f3 in, f3 N, PathRng& g, f3& out,
                                                  float& pdf) {
    const f3 R = mirror_dir(N, in);
    f3 X, Y, Z;
    frame_from_n(R, X, Y, Z);
    const float a = g.next(), b = g.next();
    const float t2 = powf(b, 1.f / (power + 1.f));
    const float t3 = sqrtf(fmaxf(0.f, 1.f - t2 * t2));
    float s, c;
    sincosf(2.f * PI_F * a, &s, &c);
    out = normalize(to_world(X, Y, Z, mk(s * t3, t2, c * t3)));
    const float dR = fmaxf(dot(R, out), 0.f);
    const float lobe = powf(dR, power);
    pdf = (power + 1.f) * lobe * (INV_PI_F * 0.5f);
    if (!(dot(out, N) > 0.f)) {
        out = mk(0, 0, 0);
        return mk(0, 0, 0);
    }
    return albedo * ((power + 2.f) * 0.5f * INV_PI_F * lobe);
}

// AnisotropicPhong::evalBSDF (anisotropicPhong.h:62-101), including the
// reference's unparenthesised MAX in the specular denominator
__device__ __forceinline__ f3 aniso_eval(const wr_object_desc* m, f3 in, f3 out, f3 N) {
    if (!(dot(in, N) <= 0.f && dot(out, N) >= 0.f)) return mk(0, 0, 0);
    const f3 Rs = ld3(m->rs), Rd = ld3(m->rd);
    const float nu = __ldg(&m->nu), nv = __ldg(&m->nv);
    const f3 h = normalize(out - in);
    f3 X, Y, Z;
    frame_from_n(N, X, Y, Z);
    const float ndh = dot(N, h), kdh = fabsf(dot(in, h));
    const f3 F = Rs + (mk(1, 1, 1) - Rs) * powf(1.f - kdh, 5.f);
    const float hu = dot(h, Z), hv = dot(h, X);
    const float expo = fabsf(ndh) < EPS_F ? 1.f : (nu * hu * hu + nv * hv * hv) / (1.f - ndh * ndh);
    const float a = fabsf(dot(N, in)), b = fabsf(dot(N, out));
    const float den = (kdh * a > b) ? a : b;
    const float k = sqrtf((nu + 1.f) * (nv + 1.f)) / (8.f * PI_F);
    const f3 spec = divs((F * k) * powf(ndh, expo), den);
    const float t1 = 1.f - (-dot(in, N) / 2.f), t2 = 1.f - dot(out, N) / 2.f;
    const f3 diff = vmul(Rd * (28.f / (23.f * PI_F)), mk(1, 1, 1) - Rs) * (1.f - powf(t1, 5.f)) * (1.f - powf(t2, 5.f));
    return spec + diff;
}

// half-vector sampler pdf (anisotropicPhongHalfVecSampler.h:39-56)
__device__ __forceinline__ float aniso_half_pdf(float nu, float nv, f3 N, f3 h) {
    f3 X, Y, Z;
    frame_from_n(N, X, Y, Z);
    const float ct = dot(h, Y), st = sqrtf(fmaxf(0.f, 1.f - ct * ct));
    if (st < EPS_F) return 0.f;
    const float cp = dot(h, Z) / st, sp = dot(h, X) / st;
    return sqrtf((nu + 1.f) * (nv + 1.f)) / (2.f * PI_F) * powf(dot(N, h), nu * cp * cp + nv * sp * sp);
}

// AnisotropicPhong::sampleBSDF (anisotropicPhong.h:42-59), 3 draws
__device__ __forceinline__ f3 aniso_sample(const wr_object_desc* m, f3 in, f3 N, PathRng& g, f3& out, float& pdf) {
    const float nu = __ldg(&m->nu), nv = __ldg(&m->nv);
    f3 X, Y, Z;
    frame_from_n(N, X, Y, Z);
    const float sx = g.next(), sy = g.next();
    float phi = atanf(sqrtf((nu + 1.f) / (nv + 1.f)) * tanf(PI_F / 2.f * sx));
    const float choose = g.next();
    if (choose < 0.25f) {
    } else if (choose < 0.5f) phi = PI_F - phi;
    else if (choose < 0.75f) phi += PI_F;
    else phi = 2.f * PI_F - phi;
    float sp, cp;
    sincosf(phi, &sp, &cp);
    const float cosT = powf(1.f - sy, 1.f / (1.f + nu * cp * cp + nv * sp * sp));
    const float sinT = sqrtf(fmaxf(0.f, 1.f - cosT * cosT));
    const f3 h = to_world(X, Y, Z, mk(sinT * sp, cosT, sinT * cp));
    out = in + (h * 2.f) * (-dot(in, h));
    pdf = dot(N, out) > 0.f ? aniso_half_pdf(nu, nv, N, h) : 0.f;
    pdf /= 4.f * fabsf(dot(in, h));
    if (dot(out, N) < 0.f) {
        out = mk(0, 0, 0);
        return mk(0, 0, 0);
    }
    return aniso_eval(m, in, out, N);
}

// HGPhaseSampler (hgPhaseSampler.h:9-59): value/pdf and sampling, 2 draws
__device__ __forceinline__ float hg_value(float g, f3 a, f3 b) {
    const float ct = dot(a, b);
    const float temp = 1.f + g * g - 2.f * g * ct;
    return (1.f / (4.f * PI_F)) * (1.f - g * g) / (temp * sqrtf(temp));
}
__device__ __forceinline__ void ortho_basis(f3 w, f3& u, f3& v) {
    f3 co;
    if (fabsf(w.x) <= fabsf(w.y)) co = fabsf(w.x) <= fabsf(w.z) ? mk(0, -w.z, w.y) : mk(-w.y, w.x, 0);
    else co = fabsf(w.y) <= fabsf(w.z) ? mk(-w.z, 0, w.x) : mk(-w.y, w.x, 0);
    co = normalize(co);
    u = cross(w, co);
    v = cross(w, u);
}
__device__ __forceinline__ f3 hg_sample(float g, f3 in, PathRng& gen, f3& out, float& pdf) {
    const f3 rd = normalize(in);
    const float e1 = gen.next(), e2 = gen.next();
    float ct;
    if (fabsf(g) < EPS_F) ct = 1.f - 2.f * e1;
    else {
        const float sq = (1.f - g * g) / (1.f - g + 2.f * g * e1);
        ct = (1.f + g * g - sq * sq) / (2.f * g);
    }
    const float st = sqrtf(fmaxf(0.f, 1.f - ct * ct));
    float sp, cp;
    sincosf(2.f * PI_F * e2, &sp, &cp);
    f3 u, v;
    ortho_basis(rd, u, v);
    out = (u * (st * cp) + v * (st * sp)) + rd * ct;
    pdf = hg_value(g, rd, out);
    const float val = hg_value(g, in, out);
    return mk(val, val, val);
}

// trilinear density (HeterogeneousVolume.cpp:71-116), identity transform;
// the inside-mesh test is implied by the path's inside object
__device__ __forceinline__ float grid_D(const GridDev& G, int x, int y, int z) {
    x = min(max(x, 0), (int)G.nx - 1);
    y = min(max(y, 0), (int)G.ny - 1);
    z = min(max(z, 0), (int)G.nz - 1);
    return __ldg(&G.data[((size_t)z * G.ny + y) * G.nx + x]);
}
__device__ __forceinline__ float lerpf(float t, float a, float b) { return (1.f - t) * a + t * b; }
__device__ __forceinline__ float grid_density(const GridDev& G, f3 p, float scale) {
    if (p.x > G.p1[0] || p.x < G.p0[0] || p.y > G.p1[1] || p.y < G.p0[1] || p.z > G.p1[2] || p.z < G.p0[2])
        return 0.f;
    const float fx = (float)G.nx * (p.x - G.p0[0]) / (G.p1[0] - G.p0[0]);
    const float fy = (float)G.ny * (p.y - G.p0[1]) / (G.p1[1] - G.p0[1]);
    const float fz = (float)G.nz * (p.z - G.p0[2]) / (G.p1[2] - G.p0[2]);
    const int ix = (int)floorf(fx), iy = (int)floorf(fy), iz = (int)floorf(fz);
    if (ix < 0 || ix >= (int)G.nx || iy < 0 || iy >= (int)G.ny || iz < 0 || iz >= (int)G.nz) return 0.f;
    const float dx = fx - ix, dy = fy - iy, dz = fz - iz;
    const float s00 = lerpf(dx, grid_D(G, ix, iy, iz), grid_D(G, ix + 1, iy, iz));
    const float s10 = lerpf(dx, grid_D(G, ix, iy + 1, iz), grid_D(G, ix + 1, iy + 1, iz));
    const float s01 = lerpf(dx, grid_D(G, ix, iy, iz + 1), grid_D(G, ix + 1, iy, iz + 1));
    const float s11 = lerpf(dx, grid_D(G, ix, iy + 1, iz + 1), grid_D(G, ix + 1, iy + 1, iz + 1));
    return lerpf(dz, lerpf(dy, s00, s10), lerpf(dy, s01, s11)) * scale;
}

__device__ __forceinline__ float luminance(f3 c) { return 0.212671f * c.x + 0.715160f * c.y + 0.072169f * c.z; }

// ---------------------------------------------------------------------------
// scatter (the material's Ray scatter(Ray&)); `st` tracks enclosing objects
// ---------------------------------------------------------------------------
struct Fresnel {
    bool tir;
    f3 refl, refr;
    float er;
};
// shared dielectric boundary step (refractiveObj.h:37-82)
__device__ __forceinline__ Fresnel fresnel_split(f3 N, f3 d, float cn, float nn) {
    Fresnel f;
    f.refl = mirror_dir(N, d);
    f.refr = mk(0, 0, 0);
    f.er = 0.f;
    const float theta = acosf(fminf(1.f, fmaxf(-1.f, dot(d, N))));
    const float sin_phi = cn / nn * sinf(theta);
    f.tir = sin_phi > 1.f;
    if (f.tir) return f;
    float phi = asinf(sin_phi);
    if (theta > PI_F / 2.f) phi = PI_F - phi;
    const f3 axis = normalize(cross(N, d));
    f.refr = normalize(rotate_about(axis, phi, N));
    const float ct = fabsf(cosf(theta)), cp = fabsf(cosf(phi));
    const float a1 = fabsf(cn * ct - nn * cp) / (cn * ct + nn * cp);
    const float a2 = fabsf(nn * ct - cn * cp) / (nn * ct + cn * cp);
    f.er = (a1 * a1 + a2 * a2) / 2.f;
    return f;
}

__device__ __forceinline__ void set_contact(const RenderScene& S, PRay& out, int obj, uint32_t tri, f3 n) {
    out.contact = obj;
    out.cnorm = n;
    (void)S;
    (void)tri;
}

// Diffuse / Glossy / AnisotropicGlossy (diffuseObj.h:34-57, glossyObj.h:39-62, anisotropicGlossyObj.h:54-68)
__device__ __forceinline__ PRay scatter_surface(const RenderScene& S, int self, const PRay& in, PathRng& g,
                                                bool mirror = false) {
    const wr_object_desc* m = &S.objs[self];
    PRay out = ray_default();
    out.o = in.o + in.d * in.idist;
    const f3 N = in.inorm;
    out.inside = in.inside;
    // contactTriangleID = inRay.intersectTriangleID, normal looked up on `self`
    out.contact = self;
    out.cnorm = self == in.iobj ? N : obj_normal(S, self, in.itri);
    const uint32_t type = __ldg(&m->type);
    if (type == WR_MAT_ANISO) {
        out.rad = aniso_sample(m, in.d, N, g, out.d, out.dP);
        return out;
    }
    const f3 albedo = ld3(m->albedo);
    float p = albedo.x;
    if (albedo.y > p) p = albedo.y;
    if (albedo.z > p) p = albedo.z;
    if (g.next() < p) {
        if (type == WR_MAT_DIFFUSE) out.rad = diffuse_sample(albedo, N, g, out.d, out.dP);
        else if (mirror) out.rad = phong_sample_mirror(albedo, __ldg(&m->power), in.d, N, g, out.d, out.dP);
        else out.rad = phong_sample(albedo, __ldg(&m->power), in.d, N, g, out.d, out.dP);
        out.dP *= p;
    } else {
        out.d = mk(0, 0, 0);
        out.rad = mk(0, 0, 0);
        out.dP = 1.f - p;
    }
    return out;
}

// EmissiveObject::scatter (emissiveObj.h:15-28)
__device__ __forceinline__ PRay scatter_emissive(const RenderScene& S, int self, const PRay& in) {
    PRay out = ray_default();
    out.o = in.o + in.d * in.idist;
    out.d = mk(0, 0, 0);
    out.inside = -1;
    out.contact = self;
    out.cnorm = self == in.iobj ? in.inorm : obj_normal(S, self, in.itri);
    out.rad = dot(in.d, in.inorm) <= 0.f ? ld3(S.objs[self].emission) : mk(0, 0, 0);
    return out;
}

// ReflectiveObject::scatter (reflectiveObj.h:17-43): mirror direction about
// the hit face's normal; Russian roulette with p = MAX_VEC_COMP(color); on
// survival radiance color / cosineTerm, pdf p (a delta direction).  The
// reference's MAX macro (macros.h:13) has no parentheses, so MAX_VEC_COMP
// evaluates to x > y ? x : max(y, z), reproduced here.
__device__ __forceinline__ PRay scatter_reflective(const RenderScene& S, int self, const PRay& in, PathRng& g) {
    PRay out = ray_default();
    const f3 N = in.inorm;
    out.o = in.o + in.d * in.idist;
    out.inside = in.inside;
    out.d = mirror_dir(N, in.d);
    const f3 c = ld3(S.objs[self].albedo);
    const float p = c.x > c.y ? c.x : (c.y > c.z ? c.y : c.z);
    if (g.next() < p) {
        out.contact = self;
        out.cnorm = self == in.iobj ? N : obj_normal(S, self, in.itri);
        out.rad = divs(c, cos_term(S, out));
        out.dP = p;
        out.delta = true;
    } else {
        out.rad = mk(0, 0, 0);
        out.d = mk(0, 0, 0);
        out.dP = 1.f - p;
    }
    return out;
}

// RefractiveObject::scatter (refractiveObj.h:27-88)
__device__ __forceinline__ PRay scatter_refractive(const RenderScene& S, int self, const PRay& in, PathRng& g,
                                                   InsideStack& st, bool* delegate) {
    *delegate = in.iobj != self && in.inside == self;
    PRay out = ray_default();
    if (*delegate) return out;
    const f3 N = in.inorm;
    out.o = in.o + in.d * in.idist;
    out.d = in.d;
    const int curIn = in.inside;
    const int curOut = in.inside == self ? st.below(self) : self;
    const float cn = curIn >= 0 ? obj_ior(S, curIn) : 1.f, nn = curOut >= 0 ? obj_ior(S, curOut) : 1.f;
    out.contact = self;
    out.cnorm = self == in.iobj ? N : obj_normal(S, self, in.itri);
    const Fresnel f = fresnel_split(N, in.d, cn, nn);
    if (f.tir) {
        out.d = f.refl;
        out.inside = in.inside;
    } else {
        out.d = f.refr;
        if (g.next() < f.er) {
            out.d = f.refl;
            out.rad = out.rad * (f.er / cos_term(S, out));
            out.dP = f.er;
            out.inside = in.inside;
        } else {
            out.rad = out.rad * ((1.f - f.er) / cos_term(S, out));
            out.dP = 1.f - f.er;
            out.inside = curOut;
        }
    }
    out.d = normalize(out.d);
    out.delta = true;
    return out;
}

// entering a medium (homogeneousVolume.cpp:16-67 / HeterogeneousVolume.cpp:456-507)
__device__ __forceinline__ PRay medium_enter(const RenderScene& S, int self, const PRay& in, PathRng& g) {
    PRay out = ray_default();
    const f3 N = in.inorm;
    out.o = in.o + in.d * in.idist;
    out.d = in.d;
    const float cn = in.inside >= 0 ? obj_ior(S, in.inside) : 1.f, nn = obj_ior(S, self);
    out.contact = self;
    out.cnorm = N;
    out.delta = true;  // every boundary outcome is a delta direction (homogeneousVolume.cpp:45-80)
    const Fresnel f = fresnel_split(N, in.d, cn, nn);
    out.ptype = PT_NOUSE;
    if (f.tir) {
        out.d = f.refl;
        out.inside = in.inside;
        return out;
    }
    out.d = f.refr;
    if (g.next() < f.er) {
        out.d = f.refl;
        out.rad = out.rad * (f.er / cos_term(S, out));
        out.dP = f.er;
        out.inside = in.inside;
    } else {
        out.rad = out.rad * ((1.f - f.er) / cos_term(S, out));
        out.dP = 1.f - f.er;
        out.inside = self;
        out.ptype = PT_HITVOL;
    }
    out.d = normalize(out.d);
    return out;
}

// leaving a medium at its own boundary (Fresnel) or handing over to the surface hit inside it
// (homogeneousVolume.cpp:101-180 / HeterogeneousVolume.cpp:561-637); `delegate` asks the caller
// to run the hit object's scatter on the returned record and multiply its oP by P_surface
__device__ __forceinline__ PRay medium_exit(const RenderScene& S, int self, const PRay& in, float P_surface,
                                            PathRng& g, InsideStack& st, bool* delegate) {
    PRay out = in;
    out.o = in.o + in.d * in.idist;
    out.contact = in.iobj;
    out.cnorm = in.inorm;
    out.inside = self;
    out.dP = 1.f;
    out.rad = mk(1, 1, 1);
    *delegate = in.iobj != self;
    if (*delegate) {
        out.contact = -1;
        out.idist = 0.f;
        return out;
    }
    const f3 N = in.inorm;
    const int curOut = st.below(self);
    const float cn = obj_ior(S, self), nn = curOut >= 0 ? obj_ior(S, curOut) : 1.f;
    out.iobj = -1;
    out.delta = true;  // every boundary outcome is a delta direction (homogeneousVolume.cpp:141-186)
    out.ptype = PT_NOUSE;
    const Fresnel f = fresnel_split(N, in.d, cn, nn);
    if (f.tir) {
        out.d = f.refl;
        out.inside = in.inside;
        out.contact = self;
        out.oP = P_surface;
        return out;
    }
    out.d = f.refr;
    if (g.next() < f.er) {
        out.d = f.refl;
        out.rad = out.rad * (f.er / cos_term(S, out));
        out.dP = f.er;
        out.oP = P_surface;
        out.inside = in.inside;
    } else {
        out.rad = out.rad * ((1.f - f.er) / cos_term(S, out));
        out.dP = 1.f - f.er;
        out.oP = P_surface;
        out.inside = curOut;
    }
    out.d = normalize(out.d);
    return out;
}

// HomogeneousVolume::scatter (homogeneousVolume.cpp:7-199): analytic free flight on Luminance(sigma_t)
__device__ __forceinline__ PRay scatter_homogeneous(const RenderScene& S, int self, const PRay& in, PathRng& g,
                                                    InsideStack& st, bool* delegate, float* psurf) {
    const wr_object_desc* m = &S.objs[self];
    const f3 ss = ld3(m->sigma_s), st_ = ss + ld3(m->sigma_a);
    const float lt = luminance(st_);
    const float sampDist = -logf(1.f - g.next()) / lt;
    *delegate = false;
    const bool go_in = in.iobj == self && in.inside != self;
    const bool be_in = in.inside == self;
    if (go_in) return medium_enter(S, self, in, g);
    if (be_in && sampDist < in.idist) {
        PRay out = ray_default();
        out.o = in.o + in.d * sampDist;
        out.rad = hg_sample(__ldg(&m->g), in.d, g, out.d, out.dP);
        out.inside = self;
        out.ptype = PT_INVOL;
        const float albedo = luminance(ss) / lt;
        const f3 pm = mk(st_.x * expf(-st_.x * sampDist), st_.y * expf(-st_.y * sampDist), st_.z * expf(-st_.z * sampDist));
        if (g.next() < albedo) {
            out.contact = -1;
            out.dP *= albedo;
            out.oP = luminance(pm);
            out.rad = vmul(out.rad, ss);
        } else {
            out.d = mk(0, 0, 0);
            out.rad = mk(0, 0, 0);
            out.dP = 1.f;
            out.oP = luminance(pm);
            out.inside = -1;
            out.contact = -1;
        }
        return out;
    }
    if (be_in) {
        const float d = in.idist;
        *psurf = luminance(mk(expf(-st_.x * d), expf(-st_.y * d), expf(-st_.z * d)));
        return medium_exit(S, self, in, *psurf, g, st, delegate);
    }
    return ray_default();
}

// HeterogeneousVolume::scatter (HeterogeneousVolume.cpp:449-641) with delta
// tracking (Woodcock) against the grid's majorant in place of Simpson +
// Newton inversion.  For a grey sigma_t the reference's throughput weights
// reduce to 1 per free flight; this keeps the same product with
// oP = sigma_t * density at a collision and 1 on passing.
__device__ __forceinline__ PRay scatter_heterogeneous(const RenderScene& S, int self, const PRay& in, PathRng& g,
                                                      InsideStack& st, bool* delegate, float* psurf) {
    const wr_object_desc* m = &S.objs[self];
    *delegate = false;
    const bool go_in = in.iobj == self && in.inside != self;
    const bool be_in = in.inside == self;
    if (go_in) return medium_enter(S, self, in, g);
    const f3 ss = ld3(m->sigma_s), st_ = ss + ld3(m->sigma_a);
    const float sgt = st_.x;  // grey extinction (checked at upload)
    const GridDev G = S.grids[__ldg(&m->grid_index)];
    const float scale = __ldg(&m->density_scale);
    const float mu = G.majorant * scale * sgt;
    float t = 0.f;
    bool collided = false;
    float dens = 0.f;
    if (mu > 0.f) {
        for (int it = 0; it < 1 << 16; it++) {  // bounded: the expected count is mu * distance
            t += -logf(1.f - g.next()) / mu;
            if (t >= in.idist) break;
            dens = grid_density(G, in.o + in.d * t, scale);
            if (g.next() * mu < sgt * dens) {
                collided = true;
                break;
            }
        }
    }
    if (be_in && collided) {
        PRay out = ray_default();
        out.o = in.o + in.d * t;
        out.rad = hg_sample(__ldg(&m->g), in.d, g, out.d, out.dP);
        out.inside = self;
        out.ptype = PT_INVOL;
        const float albedo = luminance(ss) / luminance(st_);
        if (g.next() < albedo) {
            out.contact = -1;
            out.dP *= albedo;
            out.oP = sgt * dens;
            out.rad = vmul(out.rad, ss * dens);
        } else {
            out.d = mk(0, 0, 0);
            out.rad = mk(0, 0, 0);
            out.dP = 1.f;
            out.oP = sgt * dens;
            out.inside = -1;
            out.contact = -1;
        }
        return out;
    }
    if (be_in) {
        *psurf = 1.f;
        return medium_exit(S, self, in, 1.f, g, st, delegate);
    }
    return ray_default();
}

// lookUpDensity (HeterogeneousVolume.cpp:71-116) in the reference's order of
// operations (densityScale on each corner before the trilinear blend); the
// inside-mesh test is implied by the record's inside object
__device__ __forceinline__ float grid_density_ref(const GridDev& G, f3 p, float scale) {
    if (p.x > G.p1[0] || p.x < G.p0[0] || p.y > G.p1[1] || p.y < G.p0[1] || p.z > G.p1[2] || p.z < G.p0[2])
        return 0.f;
    const float bx = G.p1[0] - G.p0[0], by = G.p1[1] - G.p0[1], bz = G.p1[2] - G.p0[2];
    const float tx = p.x - G.p0[0], ty = p.y - G.p0[1], tz = p.z - G.p0[2];
    const int ix = (int)floorf((float)G.nx * tx / bx), iy = (int)floorf((float)G.ny * ty / by),
              iz = (int)floorf((float)G.nz * tz / bz);
    if (ix < 0 || ix >= (int)G.nx || iy < 0 || iy >= (int)G.ny || iz < 0 || iz >= (int)G.nz) return 0.f;
    const float dx = (float)G.nx * tx / bx - (float)ix, dy = (float)G.ny * ty / by - (float)iy,
                dz = (float)G.nz * tz / bz - (float)iz;
    const float s00 = lerpf(dx, grid_D(G, ix, iy, iz) * scale, grid_D(G, ix + 1, iy, iz) * scale);
    const float s10 = lerpf(dx, grid_D(G, ix, iy + 1, iz) * scale, grid_D(G, ix + 1, iy + 1, iz) * scale);
    const float s01 = lerpf(dx, grid_D(G, ix, iy, iz + 1) * scale, grid_D(G, ix + 1, iy, iz + 1) * scale);
    const float s11 = lerpf(dx, grid_D(G, ix, iy + 1, iz + 1) * scale, grid_D(G, ix + 1, iy + 1, iz + 1) * scale);
    return lerpf(dz, lerpf(dy, s00, s10), lerpf(dy, s01, s11));
}

// Scene::findInsideObjectWithID (scene.cpp:146-178) as lookUpDensity's
// checkIn (HeterogeneousVolume.cpp:164-169) asks it: the closest hits of the
// rays from p along -y and +y among object o's own triangles must both leave
// the mesh (a point on a face, whose ray meets that face at t = 0 against
// its normal, is outside).  Brute force over the mesh: a medium's boundary is
// a handful of triangles.
static __device__ __noinline__ bool inside_mesh(const RenderScene& S, int o, f3 p) {
    const uint32_t tb = __ldg(&S.objs[o].tri_begin), tc = __ldg(&S.objs[o].tri_count);
    for (int k = 0; k < 2; k++) {
        const f3 d = mk(0.f, k == 0 ? -1.f : 1.f, 0.f);
        const RayQ q = make_rayq(p, d, S.tree.scene_mag);
        float best = __int_as_float(0x7f800000);
        f3 bn = mk(0, 0, 0);
        for (uint32_t t = 0; t < tc; t++) {
            const TriRec* r = S.tree.tris + __ldg(&S.tri_slot[tb + t]);
            const f3 v0 = xyz(__ldg(&r->v0)), v1 = xyz(__ldg(&r->v1)), v2 = xyz(__ldg(&r->v2));
            const float h = tri_test(v0, v1, v2, q);
            if (h >= 0.f && h < best) {
                best = h;
                bn = face_normal(v0, v1, v2);
            }
        }
        if (!(best < __int_as_float(0x7f800000)) || dot(bn, d) < 0.f) return false;
    }
    return true;
}

// lookUpDensity of object `self` with its checkIn
__device__ __forceinline__ float hv_density_ref(const RenderScene& S, int self, f3 p) {
    if (!inside_mesh(S, self, p)) return 0.f;
    const wr_object_desc* m = &S.objs[self];
    return grid_density_ref(S.grids[__ldg(&m->grid_index)], p, __ldg(&m->density_scale));
}

// density of the quadratic through one Simpson step at offset x
// (HeterogeneousVolume.cpp:285-287, 299-301): temp * (float - double + float) in double
__device__ __forceinline__ float hv_dens_poly(float temp, float n1, float n2, float n3, float sss, double ss, float x) {
    return (float)((double)temp * ((double)(n1 * sss) - (double)(3.f * n1 - 4.f * n2 + n3) * ss * (double)x +
                                   (double)(2.f * (n1 - 2.f * n2 + n3) * x * x)));
}

// findDesiredIntegralDensity (HeterogeneousVolume.cpp:258-344) along the ray
// of `in`, a record inside the medium: Simpson steps of at most 2 stepSize up
// to its hit (the reference's check() traces the same ray under the same
// NoSelfCondition, so its first hit is in.idist; chk >= 0 gives check()'s
// distance where it differs, 0 for a failed check), then Newton-bisection on
// the step's quadratic.  0 found, 2 Newton stopped after 30 iterations (both
// with t, the integral and the density at t), 1 no hit, 3 no progress, 4 not
// reached.
static __device__ __noinline__ int hv_find_ref(const RenderScene& S, int self, const PRay& in, float desired,
                                               float& t, float& integ, float& dAtT, float chk) {
    if (chk >= 0.f ? !(chk > 0.f) : !(in.iobj >= 0 && in.idist > 0.f)) return 1;
    const float dist = chk >= 0.f ? chk : in.idist;
    integ = 0.f;
    f3 p = in.o;
    const unsigned n = (unsigned)ceilf(dist / (2.f * __ldg(&S.objs[self].step_size)));
    const double ss = (double)(dist / (float)n), mult = (1.0 / 6.0) * ss;
    const f3 full = in.d * (float)ss, half = full * 0.5f;
    float node1 = hv_density_ref(S, self, p);
    for (unsigned i = 0; i < n; i++) {
        const float node2 = hv_density_ref(S, self, p + half), node3 = hv_density_ref(S, self, p + full);
        const float nd = (float)((double)integ + mult * (double)(node1 + node2 * 4.f + node3));
        if (nd >= desired) {
            float a = 0.f, b = (float)ss, x = a, fx = integ - desired;
            const float sss = (float)(ss * ss), temp = (float)(1.0 / (double)sss);
            for (int it = 1;; it++) {
                const float dfx = hv_dens_poly(temp, node1, node2, node3, sss, ss, x);
                x -= fx / dfx;
                if (x <= a || x >= b || dfx == 0.f) x = (float)(0.5 * (double)(b + a));
                const float intval =
                    (float)((double)integ +
                            (double)temp * (1.0 / 6.0) *
                                ((double)x * ((double)(6.f * node1 * sss) -
                                              (double)(3.f * (3.f * node1 - 4.f * node2 + node3)) * ss * (double)x +
                                              (double)(4.f * (node1 - 2.f * node2 + node3) * x * x))));
                fx = intval - desired;
                const float dnow = hv_dens_poly(temp, node1, node2, node3, sss, ss, x);
                if (fabs((double)fx) < 1e-4 || it + 1 > 30) {
                    t = (float)((double)x + ss * i);
                    integ = intval;
                    dAtT = dnow;
                    return fabs((double)fx) < 1e-4 ? 0 : 2;
                }
                if (fx > 0.f) b = x;
                else a = x;
            }
        }
        const f3 nxt = p + full;
        if (nxt.x == p.x && nxt.y == p.y && nxt.z == p.z) return 3;
        integ = nd;
        node1 = node3;
        p = nxt;
    }
    return 4;
}

// HeterogeneousVolume::scatter (HeterogeneousVolume.cpp:449-641) as the
// reference samples it: sampleDistance (:354-404) inverts the Simpson-
// integrated density at -log(1-u) / Luminance(sigma_t); a collision keeps
// oP = exp(-integral) * density(t), passing the medium oP = exp(-integral).
// Used by the bidirectional renderers, whose weights evaluate the same
// densities (the unidirectional kernels use delta tracking).
static __device__ __noinline__ PRay scatter_heterogeneous_ref(const RenderScene& S, int self, const PRay& in,
                                                              PathRng& g, InsideStack& st, bool* delegate,
                                                              float* psurf, float chk = -1.f) {
    const wr_object_desc* m = &S.objs[self];
    *delegate = false;
    const bool go_in = in.iobj == self && in.inside != self;
    const bool be_in = in.inside == self;
    if (go_in) return medium_enter(S, self, in, g);
    const f3 ss = ld3(m->sigma_s), st_ = ss + ld3(m->sigma_a);
    const float desired = (float)(-log(1.0 - (double)g.next()) / (double)luminance(st_));
    float t = 0.f, integ = 0.f, dAtT = 0.f;
    const int flag = be_in ? hv_find_ref(S, self, in, desired, t, integ, dAtT, chk) : 1;
    const float expVal = expf(-integ);
    const bool ok = flag == 0 || flag == 2;
    if (be_in && ok) {
        PRay out = ray_default();
        out.o = in.o + in.d * t;
        out.rad = hg_sample(__ldg(&m->g), in.d, g, out.d, out.dP);
        out.inside = self;
        out.ptype = PT_INVOL;
        const float albedo = luminance(ss) / luminance(st_);
        if (g.next() < albedo) {
            out.contact = -1;
            out.dP *= albedo;
            out.oP = expVal * dAtT;
            out.rad = vmul(out.rad, ss * hv_density_ref(S, self, out.o));
        } else {
            out.d = mk(0, 0, 0);
            out.rad = mk(0, 0, 0);
            out.dP = 1.f;
            out.oP = expVal * dAtT;
            out.inside = -1;
            out.contact = -1;
        }
        return out;
    }
    if (be_in) {
        *psurf = expVal;
        return medium_exit(S, self, in, expVal, g, st, delegate);
    }
    return ray_default();
}

// one scatter() call, following delegations (RefractiveObject handing a hit
// inside it to the hit object; media handing over to the surface hit).
// RefMedia: heterogeneous media by the reference's own sampler.
template <bool RefMedia = false>
static __device__ __forceinline__ PRay scatter(const RenderScene& S, int self, const PRay& in, PathRng& g,
                                            InsideStack& st, bool mirror = false) {
    PRay cur = in;
    float oP_scale = 1.f;
    int medium_hit = -1;  // the object a medium handed over to (photonType, homogeneousVolume.cpp:192-194)
    for (int hop = 0; hop < 4; hop++) {
        const uint32_t type = obj_type(S, self);
        bool del = false;
        float ps = 1.f;
        PRay out;
        switch (type) {
            case WR_MAT_DIFFUSE:
            case WR_MAT_GLOSSY:
            case WR_MAT_ANISO: out = scatter_surface(S, self, cur, g, mirror); break;
            case WR_MAT_EMISSIVE: out = scatter_emissive(S, self, cur); break;
            case WR_MAT_REFLECTIVE: out = scatter_reflective(S, self, cur, g); break;
            case WR_MAT_REFRACTIVE:
                out = scatter_refractive(S, self, cur, g, st, &del);
                if (del) {  // `return inRay.intersectObj->scatter(inRay)`
                    self = cur.iobj;
                    continue;
                }
                break;
            case WR_MAT_HOMOGENEOUS: out = scatter_homogeneous(S, self, cur, g, st, &del, &ps); break;
            default:
                if constexpr (RefMedia) out = scatter_heterogeneous_ref(S, self, cur, g, st, &del, &ps);
                else out = scatter_heterogeneous(S, self, cur, g, st, &del, &ps);
                break;
        }
        if (del) {  // medium hands over to the surface it hit: scatter there, oP *= P_surface
            oP_scale *= ps;
            self = cur.iobj;
            medium_hit = self;
            cur = out;
            continue;
        }
        out.oP *= oP_scale;
        if (medium_hit >= 0) out.ptype = is_volume(S, medium_hit) ? PT_NOUSE : PT_OUTVOL;
        return out;
    }
    PRay dead = ray_default();
    dead.rad = mk(0, 0, 0);
    return dead;
}

// Ray::radianceDecay (ray.cpp:46-50): refractive decay^dist, homogeneous
// exp(-sigma_t dist); heterogeneous media are already weighted by tracking
__device__ __forceinline__ f3 radiance_decay(const RenderScene& S, const PRay& r, float dist) {
    if (r.inside < 0) return mk(1, 1, 1);
    const wr_object_desc* m = &S.objs[r.inside];
    const uint32_t t = __ldg(&m->type);
    if (t == WR_MAT_REFRACTIVE) {
        const f3 dc = ld3(m->decay);
        return mk(powf(dc.x, dist), powf(dc.y, dist), powf(dc.z, dist));
    }
    if (t == WR_MAT_HOMOGENEOUS) {
        const f3 s = ld3(m->sigma_s) + ld3(m->sigma_a);
        return mk(expf(-s.x * dist), expf(-s.y * dist), expf(-s.z * dist));
    }
    return mk(1, 1, 1);
}

// color *= rad / oP / dP with vec3/scalar's zero rule
__device__ __forceinline__ f3 weight(const PRay& r) { return divs(divs(r.rad, r.oP), r.dP); }

// Camera::generateRay (camera.cpp:6-60), draws 0 and 1 (+2, 3 for the lens)
__device__ __forceinline__ PRay camera_ray(const CamParams& S, uint32_t pixel, PathRng& g) {
    PRay r = ray_default();
    const uint32_t x = pixel % S.width, y = pixel / S.width;
    const float u = g.next(), v = g.next();
    r.d = normalize((S.front * S.ipd + S.right * (((float)x + u) - ((float)S.width / 2.f))) +
                    S.top * ((((float)S.height / 2.f) - (float)y) - v));
    r.o = S.pos;
    if (S.lens_radius > 0.f) {  // thin lens (camera.cpp:30-47, concentricSampleDisk :207-249)
        const float a = g.next(), b = g.next();
        const float sx = 2.f * a - 1.f, sy = 2.f * b - 1.f;
        float lu = 0.f, lv = 0.f;
        if (!(sx == 0.f && sy == 0.f)) {
            float rr, th;
            if (sx >= -sy) {
                if (sx > sy) {
                    rr = sx;
                    th = sy > 0.f ? sy / rr : 8.f + sy / rr;
                } else {
                    rr = sy;
                    th = 2.f - sx / rr;
                }
            } else {
                if (sx <= sy) {
                    rr = -sx;
                    th = 4.f - sy / rr;
                } else {
                    rr = -sy;
                    th = 6.f + sx / rr;
                }
            }
            th *= PI_F / 4.f;
            lu = rr * cosf(th);
            lv = rr * sinf(th);
        }
        lu *= S.lens_radius;
        lv *= S.lens_radius;
        const float ft = S.focal_dist / fabsf(dot(S.front, r.d));
        const f3 pf = r.o + r.d * ft;
        r.o = (S.pos + S.right * lu) + S.top * lv;
        r.d = normalize(pf - r.o);
    }
    r.contact = CAMERA_OBJ;
    r.cnorm = normalize(S.focus - r.o);
    r.inside = S.inside;
    return r;
}

// Camera::fixVignetting (camera.cpp:90-123) + isLegalColor (util.h:8-18)
__device__ __forceinline__ bool legal(f3 c) {
    return isfinite(c.x) && isfinite(c.y) && isfinite(c.z) && c.x >= 0.f && c.y >= 0.f && c.z >= 0.f;
}
__device__ __forceinline__ f3 fix_vignetting(const CamParams& S, f3 color, uint32_t pixel) {
    const uint32_t x = pixel % S.width, y = pixel / S.width;
    const f3 dir = normalize((S.front * S.ipd + S.right * ((float)x + 0.5f - S.width / 2.f)) +
                             S.top * (S.height / 2.f - 0.5f - (float)y));
    const float c = dot(dir, S.front);
    if (c == 0.f) return mk(0, 0, 0);
    const f3 r = divs(color, fabsf(c));
    return legal(r) ? r : mk(0, 0, 0);
}

// ---------------------------------------------------------------------------
// next-event estimation (PathTracer::renderPixels NEE branch, pathTracer.cpp:39-66)
// ---------------------------------------------------------------------------
struct ShadowReq {
    f3 o, d;        // from the path vertex towards the light sample
    float dist;     // |light.o - o| (visibility: hit beyond dist - EPSILON)
    f3 contrib;     // colour the path adds if the light is visible
    int inside, contact;
};

__device__ __forceinline__ uint32_t lower_bound_dev(const float* a, uint32_t lo, uint32_t n, float x) {
    uint32_t l = 0, h = n;
    while (l < h) {
        const uint32_t m = (l + h) >> 1;
        if (__ldg(&a[lo + m]) < x) l = m + 1;
        else h = m;
    }
    return l;
}

// SurfaceSampler::genSample -> AbstractObject::genSurfaceSample
// (surfaceSampler.cpp:17-23, abstractObj.cpp:18-52): 6 draws.  The reference
// also traces the light sample's own ray; its result is unused by the path
// tracer, so it is not traced here.
__device__ __forceinline__ PRay light_sample(const RenderScene& S, PathRng& g) {
    PRay r = ray_default();
    const float chosen = g.next() * S.light_area;
    uint32_t li = lower_bound_dev(S.light_thresh, 0, S.nlights, chosen);
    if (li == S.nlights) li--;
    const int o = __ldg(&S.light_obj[li]);
    const uint32_t tb = __ldg(&S.objs[o].tri_begin), tc = __ldg(&S.objs[o].tri_count);
    if (tc == 0) {  // an emitter without triangles: a dead sample (abstractObj.cpp:20-24)
        r.d = mk(0, 0, 0);
        r.rad = mk(0, 0, 0);
        return r;
    }
    const float ra = g.next() * __ldg(&S.obj_area[o]);
    uint32_t ti = lower_bound_dev(S.tri_thresh, tb, tc, ra);
    if (ti == tc) ti--;
    const TriRec* tr = S.tree.tris + __ldg(&S.tri_slot[tb + ti]);
    const f3 v0 = xyz(__ldg(&tr->v0)), v1 = xyz(__ldg(&tr->v1)), v2 = xyz(__ldg(&tr->v2));
    float u1 = g.next(), u2 = g.next();
    if (u1 + u2 > 1.f) {
        u1 = 1.f - u1;
        u2 = 1.f - u2;
    }
    r.o = (v0 + (v1 - v0) * u1) + (v2 - v0) * u2;
    const f3 N = face_normal(v0, v1, v2);
    const float sx = g.next(), sy = g.next();
    float s, c;
    sincosf(2.f * PI_F * sx, &s, &c);
    const float t2 = 2.f * sqrtf(fmaxf(0.f, sy - sy * sy));
    r.d = mk(c * t2, 1.f - 2.f * sy, s * t2);
    if (dot(r.d, N) < 0.f) r.d = -r.d;
    r.dP = INV_PI_F * 0.25f * 2.f;
    r.rad = ld3(S.objs[o].emission);
    r.contact = o;
    r.cnorm = N;
    r.oP = 1.f / __ldg(&S.obj_area[o]) * __ldg(&S.pick_prob[o]);
    return r;
}

// evaluateBSDF of the object at the connection vertex (Ray::evalBSDF, ray.cpp:15-22)
__device__ __forceinline__ f3 eval_bsdf(const RenderScene& S, f3 in_d, const PRay& out) {
    const int o = out.contact >= 0 ? out.contact : out.inside;
    if (o < 0) return mk(0, 0, 0);
    const wr_object_desc* m = &S.objs[o];
    const uint32_t t = __ldg(&m->type);
    switch (t) {
        case WR_MAT_DIFFUSE:  // diffuseBsdf.h:31-33
            if (out.contact < 0) return mk(0, 0, 0);
            if (dot(in_d, out.cnorm) <= 0.f && dot(out.d, out.cnorm) >= 0.f) return ld3(m->albedo) * INV_PI_F;
            return mk(0, 0, 0);
        case WR_MAT_GLOSSY: {  // isotropicPhong.h:41-49
            if (out.contact < 0) return mk(0, 0, 0);
            const f3 N = out.cnorm;
            if (!(dot(in_d, N) <= 0.f && dot(out.d, N) >= 0.f)) return mk(0, 0, 0);
            const float power = __ldg(&m->power);
            const f3 rho = ld3(m->albedo) * ((power + 2.f) * 0.5f * INV_PI_F);
            const float dRW = dot(mirror_dir(N, in_d), out.d);
            return rho * powf(dRW > 0.f ? dRW : 0.f, power);
        }
        case WR_MAT_ANISO:
            if (out.contact < 0) return mk(0, 0, 0);
            return aniso_eval(m, in_d, out.d, out.cnorm);
        case WR_MAT_EMISSIVE: return ld3(m->emission);
        case WR_MAT_HOMOGENEOUS:
        case WR_MAT_HETEROGENEOUS:
            if (out.contact < 0) {
                f3 r = ld3(m->sigma_s) * hg_value(__ldg(&m->g), in_d, out.d);
                if (t == WR_MAT_HETEROGENEOUS)
                    r = r * grid_density(S.grids[__ldg(&m->grid_index)], out.o, __ldg(&m->density_scale));
                return r;
            }
            if (out.contact != o) return mk(0, 0, 0);
            return mk(0, 0, 0);
    }
    return mk(0, 0, 0);
}

// transmittance along a connection inside a heterogeneous medium: ratio
// tracking against the majorant (unbiased; the reference integrates with
// Simpson steps)
__device__ __forceinline__ float ratio_tracking(const RenderScene& S, int obj, f3 o, f3 d, float dist, PathRng& g) {
    const wr_object_desc* m = &S.objs[obj];
    const GridDev G = S.grids[__ldg(&m->grid_index)];
    const float scale = __ldg(&m->density_scale);
    const float sgt = __ldg(&m->sigma_s[0]) + __ldg(&m->sigma_a[0]);
    const float mu = G.majorant * scale * sgt;
    if (!(mu > 0.f)) return 1.f;
    float T = 1.f, t = 0.f;
    for (int it = 0; it < 1 << 16; it++) {
        t += -logf(1.f - g.next()) / mu;
        if (t >= dist) break;
        T *= 1.f - sgt * grid_density(G, o + d * t, scale) / mu;
    }
    return T;
}

// Builds the shadow connection of a path whose ray `end` closes it (the
// reference's endRay) with `prev_d` the direction of the ray before it and
// `color` the product of the earlier vertices' factors.  Returns false when
// the reference adds nothing.
__device__ __forceinline__ bool nee_prepare(const RenderScene& S, const PRay& end, f3 prev_d, f3 color, PathRng& g,
                                            ShadowReq& sr) {
    if (S.nlights == 0) return false;
    PRay light = light_sample(S, g);
    if (end.contact >= 0) {
        const uint32_t t = obj_type(S, end.contact);
        if (t == WR_MAT_EMISSIVE) return false;  // isEmissive()
        if (t == WR_MAT_GLOSSY || t == WR_MAT_ANISO || t == WR_MAT_REFRACTIVE || t == WR_MAT_REFLECTIVE)
            return false;  // !nonSpecular()
    }
    PRay e = end;
    e.d = normalize(light.o - e.o);
    light.d = -e.d;
    const float cd0 = length(light.o - e.o);
    const float cd = cd0 > EPS_F ? cd0 : EPS_F;
    if (dot(e.d, light.cnorm) >= 0.f) return false;
    f3 decay = radiance_decay(S, e, cd);
    if (e.inside >= 0 && obj_type(S, e.inside) == WR_MAT_HETEROGENEOUS) {
        const float T = ratio_tracking(S, e.inside, e.o, e.d, cd, g);
        decay = mk(T, T, T);
    }
    f3 t = vmul(vmul(eval_bsdf(S, prev_d, e), light.rad), decay);
    t = t * cos_term(S, light) * cos_term(S, e);
    t = divs(t, cd * cd);
    sr.contrib = divs(vmul(color, t), e.oP * light.oP);
    sr.o = e.o;
    sr.d = e.d;
    sr.dist = length(e.o - light.o);
    sr.inside = e.inside;
    sr.contact = e.contact;
    return true;
}

// MCRenderer::visibilityTest (mcRenderer.cpp:59-65) on a closest hit
__device__ __forceinline__ bool nee_visible(const Hit& h, float dist) {
    return h.slot < 0 || h.t - dist >= -EPS_F;
}

// ---------------------------------------------------------------------------
// next-event estimation with multiple importance sampling (WR_RENDER_NEE_MIS)
// ---------------------------------------------------------------------------
// The surface materials whose scatter has a density to weigh against light
// sampling: diffuse, isotropic and anisotropic Phong.
__device__ __forceinline__ bool mis_material(uint32_t t) {
    return t == WR_MAT_DIFFUSE || t == WR_MAT_GLOSSY || t == WR_MAT_ANISO;
}

// Solid-angle density with which scatter_surface of object `o` samples `out`
// for the incoming direction `in` at normal N, Russian roulette left out
// (diffuseBsdf.h:21-30, isotropicPhong.h:20-38 or the mirror lobe,
// anisotropicPhongHalfVecSampler.h:39-56).  Used by both strategies' weights.
__device__ __forceinline__ float bsdf_pdf(const RenderScene& S, int o, f3 in, f3 N, f3 out, bool mirror) {
    const wr_object_desc* m = &S.objs[o];
    const uint32_t t = __ldg(&m->type);
    const float dn = dot(N, out);
    if (!(dn > 0.f)) return 0.f;
    if (t == WR_MAT_DIFFUSE) return dn * INV_PI_F;
    if (t == WR_MAT_GLOSSY) {
        const float power = __ldg(&m->power);
        const float c = mirror ? dot(mirror_dir(N, in), out) : dn;
        return c > 0.f ? (power + 1.f) * powf(c, power) * (INV_PI_F * 0.5f) : 0.f;
    }
    if (t == WR_MAT_ANISO) {
        const f3 h = normalize(out - in);
        const float ih = fabsf(dot(in, h));
        return ih > 0.f ? aniso_half_pdf(__ldg(&m->nu), __ldg(&m->nv), N, h) / (4.f * ih) : 0.f;
    }
    return 0.f;
}

// Solid-angle density with which the light sampler picks the emitter point
// a ray from a surface reaches at distance `dist` with cosine `cl` (the
// sampler is uniform in area over all emitters: SurfaceSampler's
// area-proportional object pick times the object's own uniform point).
__device__ __forceinline__ float light_pdf(const RenderScene& S, int emitter, float dist, float cl) {
    const float pa = __ldg(&S.pick_prob[emitter]) / __ldg(&S.obj_area[emitter]);
    return pa > 0.f && cl != 0.f ? pa * dist * dist / fabsf(cl) : 0.f;
}

// A light-sample connection: traced from o along d; it counts when the
// closest hit is the sampled emitter at (about) `dist`.
struct LightReq {
    f3 o, d;
    float dist;
    f3 contrib;  // the path's colour added when it counts (MIS-weighted)
    int light, inside, contact;
};

__device__ __forceinline__ bool light_req_visible(const RenderScene& S, const Hit& h, const LightReq& lr) {
    if (h.slot < 0) return false;
    const int obj = (int)__float_as_uint(__ldg(&S.tree.tris[h.slot].v1.w));
    return obj == lr.light && h.t >= lr.dist - fmaxf(EPS_F, 1e-4f * lr.dist);
}

// The light strategy at the surface vertex `cur` hits (object `self`, outside
// media), whose arriving throughput is T: one light sample (6 draws), the
// BSDF towards it, the geometry term and the power-heuristic weight against
// the density with which the scatter could have sampled the same direction.
__device__ __forceinline__ bool mis_light_request(const RenderScene& S, int self, const PRay& cur, f3 T, PathRng& g,
                                                  bool mirror, LightReq& lr) {
    if (S.nlights == 0) return false;
    const PRay L = light_sample(S, g);
    if (length(L.d) < 0.5f) return false;  // an emitter without triangles
    const f3 x = cur.o + cur.d * cur.idist;
    const f3 N = cur.inorm;
    const f3 v = L.o - x;
    const float dist = length(v);
    if (!(dist > EPS_F)) return false;
    const f3 wi = v * (1.f / dist);
    const float cl = dot(wi, L.cnorm);
    if (!(cl < 0.f)) return false;  // EmissiveObject emits against its normal only
    PRay e = ray_default();
    e.o = x;
    e.d = wi;
    e.contact = self;
    e.cnorm = N;
    e.inside = cur.inside;
    const f3 f = eval_bsdf(S, cur.d, e);
    if (f.x == 0.f && f.y == 0.f && f.z == 0.f) return false;
    const float pl = L.oP * dist * dist / -cl;
    const float pb = bsdf_pdf(S, self, cur.d, N, wi, mirror);
    const float w = pl * pl / (pl * pl + pb * pb);
    lr.contrib = vmul(vmul(T, f), L.rad) * (cos_term(S, e) * w / pl);
    lr.o = x;
    lr.d = wi;
    lr.dist = dist;
    lr.light = L.contact;
    lr.inside = cur.inside;
    lr.contact = self;
    return legal(lr.contrib);
}

// One bounce of MCRenderer::samplePath (mcRenderer.cpp:25-56) for a path
// whose current ray `cur` has its hit set: scatter, then either finish
// (returns true, `result` = the path's colour before isLegalColor) or apply
// cur's throughput factors (pathTracer.cpp:29-38) and make the scattered ray
// current (returns false; it must be traced next, a miss ends with 0).
//
// With NEE (WR_RENDER_NEE in `flags`), a path that ends with zero radiance
// and no contact or inside object on its last ray (it escaped, or was cut at
// the maximum length, or was absorbed in a medium) is connected to a light
// from the origin of the ray that closes it (the reference's endIndex rule,
// pathTracer.cpp:40-41): `nee_here` is set, `cur` is that ray, `prev_d` the
// direction before it and `color` the product of the earlier factors.  A
// scattered ray that misses is the caller's case: the same connection from it.
//
// With WR_RENDER_NEE_MIS, a vertex on a diffuse / Phong surface outside media
// whose scattered ray may still be traced (depth + 1 <= max_path_len) also
// asks for a light connection (`has_lr`, `lr`: the caller traces it and adds
// lr.contrib when light_req_visible), and an emitter reached straight from
// such a vertex is weighted against the light strategy; `mis_pdf` carries
// the scatter's density of the current ray (0: nothing to weigh).
// MIS_CODE: compiled with the WR_RENDER_NEE_MIS code (kernels that never see
// the flag leave it out, which keeps their register count down).
template <bool MIS_CODE>
__device__ __forceinline__ bool path_advance(const RenderScene& S, PRay& cur, f3& color, f3& prev_d,
                                             uint32_t& depth, InsideStack& st, PathRng& g, uint32_t max_path_len,
                                             uint32_t flags, f3& result, bool& nee_here, float& mis_pdf,
                                             LightReq& lr, bool& has_lr) {
    nee_here = false;
    has_lr = false;
    const bool nee = (flags & WR_RENDER_NEE) != 0;
    const bool mis = MIS_CODE && (flags & WR_RENDER_NEE_MIS) != 0;
    const bool mirror = (flags & WR_RENDER_PHONG_MIRROR) != 0;
    const int self = cur.inside >= 0 ? cur.inside : cur.iobj;
    if (self < 0) {  // escaped eye ray: terminateRay carries zero radiance, endIndex 0 connects nothing
        result = mk(0, 0, 0);
        return true;
    }
    const uint32_t stype = obj_type(S, self);
    // a light connection from this vertex is a path one segment longer, which
    // the reference only has while its scattered ray may still be traced
    const bool mis_vertex = mis && cur.inside < 0 && mis_material(stype) && depth + 1 <= max_path_len;
    if (mis_vertex) {
        const f3 T = vmul(color * cos_term(S, cur), weight(cur));
        has_lr = mis_light_request(S, self, cur, T, g, mirror, lr);
    }
    PRay next = scatter(S, self, cur, g, st, mirror);
    if (length(next.d) < 0.5f) {
        const bool zero = next.rad.x == 0.f && next.rad.y == 0.f && next.rad.z == 0.f;
        if (nee && zero) {
            result = mk(0, 0, 0);
            nee_here = next.contact == -1 && next.inside == -1 && depth >= 1;
            return true;
        }
        color = color * cos_term(S, cur);
        color = vmul(color, radiance_decay(S, cur, length(next.o - cur.o)));
        color = vmul(color, weight(cur));
        result = vmul(color, weight(next));
        if (mis && mis_pdf > 0.f && stype == WR_MAT_EMISSIVE && cur.inside < 0 && !zero) {
            // the emitter reached by the previous vertex's scatter: weigh against the light strategy
            const float pl = light_pdf(S, self, cur.idist * length(cur.d), dot(cur.d, cur.inorm));
            result = result * (mis_pdf * mis_pdf / (mis_pdf * mis_pdf + pl * pl));
        }
        return true;
    }
    if (depth + 1 > max_path_len) {
        result = mk(0, 0, 0);
        nee_here = nee && depth >= 1;
        return true;
    }
    mis_pdf = mis_vertex ? bsdf_pdf(S, self, cur.d, cur.inorm, next.d, mirror) : 0.f;
    st.set_top(next.inside);
    color = color * cos_term(S, cur);
    color = vmul(color, radiance_decay(S, cur, length(next.o - cur.o)));
    color = vmul(color, weight(cur));
    prev_d = cur.d;
    cur = next;
    depth++;
    return false;
}

// fill the hit fields of `r` from a closest-hit result
__device__ __forceinline__ void set_hit(const RenderScene& S, PRay& r, const Hit& h) {
    if (h.slot < 0) {
        r.iobj = -1;
        r.idist = -1.f;
        return;
    }
    const TriRec* tr = S.tree.tris + h.slot;
    const float4 a = __ldg(&tr->v0), b = __ldg(&tr->v1), c = __ldg(&tr->v2);
    r.iobj = (int)__float_as_uint(b.w);
    r.itri = __float_as_uint(c.w);
    r.idist = h.t;
    r.inorm = face_normal(xyz(a), xyz(b), xyz(c));
}

}  // namespace wr
