// gpuPathTracer.cpp — see gpuPathTracer.h.  Compiled inside a WalkRay tree.
#include "gpuPathTracer.h"

#include <cmath>
#include <cstring>
#include <iostream>

#include "abstractObj.h"
#include "renderEngine.h"
#include "scene.h"

namespace LFJ {

namespace {

void put3(float* d, const vec3f& v) {
    d[0] = v.x;
    d[1] = v.y;
    d[2] = v.z;
}

}  // namespace

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
