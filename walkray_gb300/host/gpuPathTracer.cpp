// gpuPathTracer.cpp — see gpuPathTracer.h.  Compiled inside a WalkRay tree.
#include "gpuPathTracer.h"

#include <cmath>
#include <cstring>
#include <iostream>

#include "HeterogeneousVolume.h"
#include "abstractObj.h"
#include "anisotropicGlossyObj.h"
#include "diffuseObj.h"
#include "emissiveObj.h"
#include "glossyObj.h"
#include "homogeneousVolume.h"
#include "reflectiveObj.h"
#include "refractiveObj.h"
#include "renderEngine.h"
#include "scene.h"

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

GpuPathTracer::GpuPathTracer(RenderEngine* engine, uint spp, uint maxLen, uint32_t mode, Describe describe)
    : MCRenderer(engine, spp, maxLen), mode(mode), describe(describe ? describe : Describe(wrDefaultDescribe)) {
    name = "GpuPathTracer";
    wr_ctx_desc cd;
    std::memset(&cd, 0, sizeof cd);
    if (wr_ctx_create(&cd, &ctx) != WR_OK) {
        std::cerr << "GpuPathTracer: no usable CUDA device" << std::endl;
        ctx = nullptr;
    }
}

GpuPathTracer::~GpuPathTracer() {
    if (ctx) wr_ctx_destroy(ctx);
}

bool GpuPathTracer::uploadSceneFile() {
    wr_scene_file* f = nullptr;
    char err[512] = {0};
    if (wr_scene_file_load(sceneFile.c_str(), &f, err, sizeof err) != WR_OK) {
        std::cerr << "GpuPathTracer: " << err << std::endl;
        return false;
    }
    wr_scene_desc desc;
    wr_scene_file_settings settings;
    bool ok = wr_scene_file_get(f, &desc, &settings) == WR_OK;
    if (ok && desc.num_objects != engine->scene.objects.size()) {
        std::cerr << "GpuPathTracer: the scene file has " << desc.num_objects << " objects, the scene "
                  << engine->scene.objects.size() << std::endl;
        ok = false;
    }
    if (ok && wr_scene_upload(ctx, &desc, &sceneId) != WR_OK) {
        std::cerr << "GpuPathTracer: " << wr_last_error(ctx) << std::endl;
        ok = false;
    }
    wr_scene_file_free(f);
    uploaded = ok;
    return ok;
}

bool GpuPathTracer::uploadScene() {
    if (uploaded) return true;
    if (!sceneFile.empty()) return uploadSceneFile();
    Scene& sc = engine->scene;
    std::vector<wr_object_desc> objs(sc.objects.size());
    std::vector<float> verts;
    std::vector<uint32_t> tris;
    uint32_t vb = 0, tb = 0;
    for (size_t i = 0; i < sc.objects.size(); i++) {
        AbstractObject* o = sc.objects[i];
        wr_object_desc& d = objs[i];
        std::memset(&d, 0, sizeof d);
        d.ior = 1.5f;
        d.decay[0] = d.decay[1] = d.decay[2] = 1.f;
        d.density_scale = 100.f;
        d.step_size = 0.002f;
        d.grid_index = 0xffffffffu;
        if (!describe(o, &d)) {
            std::cerr << "GpuPathTracer: cannot describe scene object " << i << std::endl;
            return false;
        }
        d.vert_begin = vb;
        d.vert_count = o->getVertexNum();
        d.tri_begin = tb;
        d.tri_count = o->getTriangleNum();
        for (uint v = 0; v < o->getVertexNum(); v++) {
            vec3f p = o->getWorldVertexPosition(v);  // Scene::buildKDTree uses world positions (scene.cpp:29-31)
            verts.push_back(p.x);
            verts.push_back(p.y);
            verts.push_back(p.z);
        }
        for (uint t = 0; t < o->getTriangleNum(); t++) {
            vec3ui f = o->getVertexIndices(t);
            tris.push_back(f.x);
            tris.push_back(f.y);
            tris.push_back(f.z);
        }
        vb += d.vert_count;
        tb += d.tri_count;
    }
    wr_scene_desc desc;
    std::memset(&desc, 0, sizeof desc);
    desc.num_objects = (uint32_t)objs.size();
    desc.num_vertices = vb;
    desc.num_triangles = tb;
    desc.objects = objs.data();
    desc.vertices = verts.data();
    desc.triangles = tris.data();
    Camera& c = sc.mCamera;
    put3(desc.camera.position, c.mPosition);
    put3(desc.camera.focus, c.mFocus);
    put3(desc.camera.up, c.mUp);
    desc.camera.width = (uint32_t)c.mResolution.x;
    desc.camera.height = (uint32_t)c.mResolution.y;
    desc.camera.image_plane_dist = c.mImagePlaneDist;
    desc.camera.lens_radius = lens[0];
    desc.camera.focal_dist = lens[1];
    if (wr_scene_upload(ctx, &desc, &sceneId) != WR_OK) {
        std::cerr << "GpuPathTracer: " << wr_last_error(ctx) << std::endl;
        return false;
    }
    uploaded = true;
    return true;
}

namespace {

struct ProgressCtx {
    GpuPathTracer::Progress* hook;
    Camera* camera;
    std::string pfm;
    std::vector<vec3f>* img;
};

// after every chunk: the film and its PFM as the reference updates them
// after every iteration (pathTracer.cpp:67-70), then the caller's hook
int on_chunk(void* user, const float*, uint32_t done) {
    ProgressCtx* p = static_cast<ProgressCtx*>(user);
    p->camera->mFilm.setBuffer(*p->img);
    p->camera->mFilm.savePFM(p->pfm);
    return (*p->hook && (*p->hook)(*p->img, done)) ? 1 : 0;
}

}  // namespace

std::vector<vec3f> GpuPathTracer::renderPixels() {
    if (!ctx || !uploadScene()) return std::vector<vec3f>();
    Camera& c = engine->scene.mCamera;
    const size_t n = (size_t)c.mResolution.x * (size_t)c.mResolution.y;
    std::vector<vec3f> img(n);
    wr_render_desc d;
    std::memset(&d, 0, sizeof d);
    d.spp = spp;
    d.max_path_len = maxPathLen;
    d.seed = seed;
    d.mode = mode;
    d.radius = mergeRadius;
    d.flags = (useNextEventEstimation ? WR_RENDER_NEE : 0u) | extraFlags;
    static_assert(sizeof(vec3f) == 3 * sizeof(float), "vec3f must be three packed floats");
    ProgressCtx pc{&progress, &c, name + engine->scene.name + ".pfm", &img};
    uint32_t done = 0;
    if (wr_render_progressive(ctx, sceneId, &d, 0, &img[0].x, on_chunk, &pc, &done) != WR_OK) {
        std::cerr << "GpuPathTracer: " << wr_last_error(ctx) << std::endl;
        return std::vector<vec3f>();
    }
    return img;
}

}  // namespace LFJ
