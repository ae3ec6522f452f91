// run_dropin.cpp — runs the drop-in renderer (GpuPathTracer::renderPixels) on
// a scene read from a .wrs file, through the stand-in interfaces of this
// folder, and writes the image.  Test infrastructure (tests/test_dropin_gpu.py).
//
//   run_dropin scene.wrs spp max_path_len seed out.bin [stop_after_chunks]
//
// Prints one line: chunks=<progress calls> spp_done=<last> film_sets=<n> pfm_saves=<n>
#include <cstdio>
#include <cstdlib>
#include <memory>
#include <vector>

#include "gpuPathTracer.h"
#include "renderEngine.h"
#include "wrs_io.h"

using namespace LFJ;

// WalkRay's material classes are not here (gpuPathTracerDescribe.cpp reads
// them in a WalkRay tree); this run describes every object through its own
// callback instead.
bool LFJ::wrDefaultDescribe(const AbstractObject*, wr_object_desc*) { return false; }

int main(int argc, char** argv) {
    if (argc < 6) {
        std::fprintf(stderr, "usage: run_dropin scene.wrs spp max_path_len seed out.bin [stop_after_chunks]\n");
        return 2;
    }
    wrs_scene s;
    if (wrs_load(argv[1], &s) != 0) {
        std::fprintf(stderr, "cannot read %s\n", argv[1]);
        return 2;
    }
    const uint spp = (uint)std::strtoul(argv[2], nullptr, 10);
    const uint depth = (uint)std::strtoul(argv[3], nullptr, 10);
    const uint64_t seed = std::strtoull(argv[4], nullptr, 10);
    const int stop = argc > 6 ? std::atoi(argv[6]) : 0;

    RenderEngine engine;
    std::vector<std::unique_ptr<AbstractObject>> owned;
    for (uint32_t i = 0; i < s.num_objects; i++) {
        const wr_object_desc& d = s.objects[i];
        auto o = std::make_unique<AbstractObject>();
        for (uint32_t v = 0; v < d.vert_count; v++) {
            const float* p = s.vertices + 3 * ((size_t)d.vert_begin + v);
            o->positions.push_back(vec3f(p[0], p[1], p[2]));
        }
        for (uint32_t t = 0; t < d.tri_count; t++) {
            const uint32_t* f = s.triangles + 3 * ((size_t)d.tri_begin + t);
            vec3ui tri;
            tri.x = f[0];
            tri.y = f[1];
            tri.z = f[2];
            o->triangles.push_back(tri);
        }
        o->desc = d;
        engine.scene.objects.push_back(o.get());
        owned.push_back(std::move(o));
    }
    Camera& c = engine.scene.mCamera;
    c.mPosition = vec3f(s.camera.position[0], s.camera.position[1], s.camera.position[2]);
    c.mFocus = vec3f(s.camera.focus[0], s.camera.focus[1], s.camera.focus[2]);
    c.mUp = vec3f(s.camera.up[0], s.camera.up[1], s.camera.up[2]);
    c.mResolution.x = (int)s.camera.width;
    c.mResolution.y = (int)s.camera.height;
    c.mImagePlaneDist = s.camera.image_plane_dist;
    engine.scene.name = "dropin_test";

    GpuPathTracer gpt(&engine, spp, depth, WR_MODE_WAVEFRONT, [](const AbstractObject* o, wr_object_desc* d) {
        *d = o->desc;  // the material as the scene file gives it
        return true;
    });
    gpt.setSeed(seed);
    gpt.setDepthOfField(s.camera.lens_radius, s.camera.focal_dist);
    int chunks = 0;
    uint done = 0;
    gpt.setProgress([&](const std::vector<vec3f>&, uint spp_done) {
        chunks++;
        done = spp_done;
        return stop > 0 && chunks >= stop;
    });
    const std::vector<vec3f> img = gpt.renderPixels();
    if (img.empty()) {
        std::fprintf(stderr, "renderPixels failed: %s\n", gpt.lastError());
        return 1;
    }
    FILE* f = std::fopen(argv[5], "wb");
    if (!f || std::fwrite(img.data(), sizeof(vec3f), img.size(), f) != img.size()) {
        std::fprintf(stderr, "cannot write %s\n", argv[5]);
        return 1;
    }
    std::fclose(f);
    std::printf("chunks=%d spp_done=%u film_sets=%d pfm_saves=%d\n", chunks, done, c.mFilm.sets, c.mFilm.saves);
    wrs_free(&s);
    return 0;
}
