/* Extra forced include for pathTracer.cpp and bidirPathTracer.cpp only.
 * pathTracer.cpp:23 and bidirPathTracer.cpp:32 pass the temporary returned by
 * Camera::generateRay to MCRenderer::samplePath, which takes Ray& — MSVC
 * binds it, g++ does not.  The macro routes that one
 * call through an identity function that yields an lvalue; the reference
 * source file itself is compiled as it lies. */
#pragma once
#include "wr_ref_prelude.h"
#include "mcRenderer.h"
namespace wr_shim {
template <class T> T& as_lvalue(T&& t) { return t; }
}
#define samplePath(path, ray) samplePath(path, ::wr_shim::as_lvalue(ray))
