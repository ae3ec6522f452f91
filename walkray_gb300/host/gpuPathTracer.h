// gpuPathTracer.h — GpuPathTracer, a renderer that drops in beside WalkRay's
// PathTracer (pathTracer.h): same base class (MCRenderer, mcRenderer.h:14-36),
// same constructor arguments, same renderPixels() contract (a W*H linear-RGB
// FP32 image, p = y*W + x, row 0 at the top), selected by name in
// Config::load like "PathTracer" (config.cpp:528-539).  The path tracing runs
// on the GPU through the C ABI of libwalkray_gpu.so (include/walkray.h).
//
// This file is compiled inside a WalkRay source tree (it includes WalkRay's
// headers); registering it takes one include and one name branch in
// Config::load (config.cpp:528-573).
#pragma once

#include <functional>
#include <string>
#include <vector>

#include "mcRenderer.h"
#include "walkray.h"

namespace LFJ {

class AbstractObject;

// Fills the material part of `d` for WalkRay's surface material classes
// (diffuse, glossy, anisotropic glossy, refractive, emissive) from their
// public methods; false for anything else (media keep their parameters
// private).
bool wrDefaultDescribe(const AbstractObject* o, wr_object_desc* d);

class GpuPathTracer : public MCRenderer {
public:
    // How the material of one scene object is described to the library.  The
    // default (gpuPathTracer.cpp) recognises WalkRay's material classes by
    // dynamic_cast and reads their parameters through their public methods.
    using Describe = std::function<bool(const AbstractObject*, wr_object_desc*)>;

    GpuPathTracer(RenderEngine* engine, uint spp, uint maxLen, uint32_t mode = WR_MODE_WAVEFRONT,
                  Describe describe = Describe());
    ~GpuPathTracer();

    // PathTracer::renderPixels (pathTracer.cpp:7-76) on the GPU; an empty
    // vector (and a message on std::cerr, as the reference reports errors) on
    // failure.
    std::vector<vec3f> renderPixels();

    void setNextEventEstimation(bool on) { useNextEventEstimation = on; }
    void setSeed(uint64_t s) { seed = s; }
    // WR_MODE_VCM: VCMTracer::setRadius (vcmTracer.h:40); 0 = the reference's default 0.01
    void setMergeRadius(float r) { mergeRadius = r; }
    const char* lastError() const { return ctx ? wr_last_error(ctx) : "no GPU context"; }

private:
    bool uploadScene();  // engine->scene -> wr_scene_desc -> wr_scene_upload (once per scene)

    wr_ctx* ctx = nullptr;
    wr_scene_id sceneId = 0;
    bool uploaded = false;
    bool useNextEventEstimation = false;
    uint32_t mode;
    uint64_t seed = 1;
    float mergeRadius = 0.f;
    Describe describe;
};

}  // namespace LFJ
