// wr_stub_types.h — the vector types of the stand-in WalkRay interfaces in
// this folder.  Test infrastructure: these headers let the drop-in renderer
// (walkray_gb300/host/gpuPathTracer.cpp) be compiled and run where no WalkRay
// source tree is present.  They declare only what the drop-in uses, with
// WalkRay's names and meanings; they are not WalkRay's headers.
#pragma once

#include <cstdint>

typedef unsigned int uint;

struct vec3f {
    float x = 0, y = 0, z = 0;
    vec3f() = default;
    vec3f(float a, float b, float c) : x(a), y(b), z(c) {}
};

struct vec3ui {
    uint x = 0, y = 0, z = 0;
    uint operator[](int k) const { return k == 0 ? x : (k == 1 ? y : z); }
};

struct vec2i {
    int x = 0, y = 0;
};
