// scene.h (stand-in, test infrastructure; see wr_stub_types.h): the scene,
// camera and film members the drop-in reads and writes.  The film counts
// the updates it receives.
#pragma once

#include <string>
#include <vector>

#include "abstractObj.h"
#include "wr_stub_types.h"

namespace LFJ {

class Film {
public:
    void setBuffer(const std::vector<vec3f>& img) {
        buffer = img;
        sets++;
    }
    void savePFM(const std::string& path) {
        lastPath = path;
        saves++;
    }
    std::vector<vec3f> buffer;
    std::string lastPath;
    int sets = 0, saves = 0;
};

class Camera {
public:
    vec3f mPosition, mFocus, mUp;
    vec2i mResolution;
    float mImagePlaneDist = 1.f;
    Film mFilm;
};

class Scene {
public:
    std::vector<AbstractObject*> objects;
    Camera mCamera;
    std::string name;
};

}  // namespace LFJ
