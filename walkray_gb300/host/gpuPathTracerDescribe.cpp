// gpuPathTracerDescribe.cpp — wrDefaultDescribe (gpuPathTracer.h): WalkRay's
// material classes read through their public methods.  Compiled inside a
// WalkRay tree, beside gpuPathTracer.cpp.
#include "gpuPathTracer.h"

#include <cmath>
#include <cstring>

// scene.h before the media headers (their inline constructors use Scene)
#include "scene.h"

#include "HeterogeneousVolume.h"
#include "abstractObj.h"
#include "anisotropicGlossyObj.h"
#include "diffuseObj.h"
#include "emissiveObj.h"
#include "glossyObj.h"
#include "homogeneousVolume.h"
#include "reflectiveObj.h"
#include "refractiveObj.h"

namespace LFJ {

namespace {

void put3(float* d, const vec3f& v) {
    d[0] = v.x;
    d[1] = v.y;
    d[2] = v.z;
}

// a probe ray pair at triangle 0 of `o`: incoming along -N, outgoing `out_dir`
vec3f probe(const AbstractObject* o, const vec3f& out_dir, vec3f* normal) {
    Ray in, out;
    vec3f p = o->getWorldVertexPosition(o->getVertexIndices(0)[0]);
    vec3f n = o->getWorldNormal(0, p);
    if (normal) *normal = n;
    in.direction = -n;
    out.origin = p;
    out.direction = out_dir.length() > 0 ? out_dir : n;
    out.contactObj = const_cast<AbstractObject*>(o);
    out.contactTriangleID = 0;
    return o->evaluateBSDF(in, out);
}

}  // namespace

// WalkRay's material classes, read through their public methods
bool wrDefaultDescribe(const AbstractObject* o, wr_object_desc* d) {
    if (o->getTriangleNum() == 0) return false;
    if (auto* e = dynamic_cast<const EmissiveObject*>(o)) {
        d->type = WR_MAT_EMISSIVE;
        put3(d->emission, e->getColor());
        return true;
    }
    if (dynamic_cast<const DiffuseObject*>(o)) {  // evaluateBSDF = albedo / pi (diffuseBsdf.h:31-33)
        d->type = WR_MAT_DIFFUSE;
        put3(d->albedo, probe(o, vec3f(0, 0, 0), nullptr) * (float)PI);
        return true;
    }
    if (dynamic_cast<const GlossyObject*>(o)) {  // rho (n+2)/(2 pi) cos^n(angle to mirror) (isotropicPhong.h:41-49)
        d->type = WR_MAT_GLOSSY;
        vec3f n;
        vec3f f0 = probe(o, vec3f(0, 0, 0), &n);
        Frame fr;
        fr.setFromN(n);
        // cos 0.99 off the mirror direction: cos^n stays representable up to n ~ 8000
        const double ct = 0.99;
        vec3f tilted = fr.toWorldFrame(vec3f((float)std::sqrt(1.0 - ct * ct), (float)ct, 0.f));
        vec3f ft = probe(o, tilted, nullptr);
        const double c0 = std::max(std::max(f0.x, f0.y), f0.z), c1 = std::max(std::max(ft.x, ft.y), ft.z);
        const double cos_real = (double)tilted.dot(n);  // the angle the probe actually used
        d->power = (c0 > 0 && c1 > 0) ? (float)(std::log(c0 / c1) / -std::log(cos_real)) : 1.f;
        put3(d->albedo, f0 * (2.f * (float)PI / (d->power + 2.f)));
        return true;
    }
    if (auto* a = dynamic_cast<const AnisotropicGlossyObject*>(o)) {
        d->type = WR_MAT_ANISO;
        const AnisotropicPhong* b = static_cast<const AnisotropicPhong*>(a->refBSDF());
        put3(d->rs, b->Rs);
        put3(d->rd, b->Rd);
        d->nu = b->n_u;
        d->nv = b->n_v;
        return true;
    }
    if (auto* r = dynamic_cast<const RefractiveObject*>(o)) {
        d->type = WR_MAT_REFRACTIVE;
        d->ior = r->getIOR();
        Ray ray;
        put3(d->decay, r->randianceDecay(ray, 1.f));  // decayColor^1
        return true;
    }
    if (dynamic_cast<const ReflectiveObject*>(o)) {
        // the colour is private: scatter a ray that arrives along -N (it leaves
        // along N, so cosineTerm is 1) with a local Rng until the roulette keeps
        // it; radiance * cosineTerm is then the colour (reflectiveObj.h:29-35)
        d->type = WR_MAT_REFLECTIVE;
        AbstractObject* m = const_cast<AbstractObject*>(o);
        Rng local(7), *saved = m->rng;
        m->rng = &local;
        Ray in;
        vec3f p = o->getWorldVertexPosition(o->getVertexIndices(0)[0]);
        vec3f n = o->getWorldNormal(0, p);
        in.origin = p + n;
        in.direction = -n;
        in.intersectObj = m;
        in.intersectTriangleID = 0;
        in.intersectDist = 1.f;
        vec3f c(0, 0, 0);
        for (int k = 0; k < 256; k++) {
            Ray out = o->scatter(in);
            if (out.direction.length() > 0.5f) {
                c = out.radiance * out.cosineTerm();
                break;
            }
        }
        m->rng = saved;
        put3(d->albedo, c);
        return true;
    }
    // media keep their coefficients and grids private; describe them through a
    // Describe callback (or accessors added to the media classes)
    return false;
}

}  // namespace LFJ
