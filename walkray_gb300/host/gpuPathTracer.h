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
    // failure.  Progressive like the reference: the samples are rendered in
    // chunks (about 16M paths each), and after each the running mean goes to
    // the camera's film and its PFM file (Film::setBuffer / savePFM, as
    // pathTracer.cpp:67-70 does after every iteration) and to the progress
    // hook, which may stop the render.  Config::load gives INT_MAX spp when
    // the configuration has no <iter> (config.cpp:534): such a render goes on
    // until the hook stops it, as the reference's does until it is killed.
    std::vector<vec3f> renderPixels();

    // Called after every chunk with the running mean and the samples per
    // pixel so far; return true to stop.
    using Progress = std::function<bool(const std::vector<vec3f>&, uint)>;
    void setProgress(Progress p) { progress = p; }
    void setNextEventEstimation(bool on) { useNextEventEstimation = on; }
    // WR_RENDER_NEE_MIS | WR_RENDER_PHONG_MIRROR and the like, on top of the reference's estimator
    void setRenderFlags(uint32_t f) { extraFlags = f; }
    void setSeed(uint64_t s) { seed = s; }
    // WR_MODE_VCM: VCMTracer::setRadius (vcmTracer.h:40); 0 = the reference's default 0.01
    void setMergeRadius(float r) { mergeRadius = r; }
    // The camera's thin lens (Camera::setDOFParameters, camera.cpp:207-249):
    // its radius and focal distance are private to Camera, so the code that
    // configures the camera (Config::load's <lensRadius> / <focalDist>)
    // passes them here too.
    void setDepthOfField(float lensRadius, float focalDist) {
        lens[0] = lensRadius;
        lens[1] = focalDist;
    }
    // Describes the scene from WalkRay's configuration file instead of the
    // loaded objects: the library's reader of the same XML and meshes
    // (wr_scene_file_load) gives every object's material, media and density
    // grids included (whose parameters the media classes keep private), and
    // the camera with its lens.  The object count must match engine->scene.
    void setSceneFile(const std::string& configPath) { sceneFile = configPath; }
    const char* lastError() const { return ctx ? wr_last_error(ctx) : "no GPU context"; }

private:
    bool uploadScene();  // engine->scene (or the scene file) -> wr_scene_desc -> wr_scene_upload, once
    bool uploadSceneFile();

    wr_ctx* ctx = nullptr;
    wr_scene_id sceneId = 0;
    bool uploaded = false;
    bool useNextEventEstimation = false;
    uint32_t mode;
    uint64_t seed = 1;
    float mergeRadius = 0.f;
    uint32_t extraFlags = 0;
    float lens[2] = {0.f, 3.402823466e38f};  // radius, focal distance (Camera's defaults)
    std::string sceneFile;
    Progress progress;
    Describe describe;
};

}  // namespace LFJ
