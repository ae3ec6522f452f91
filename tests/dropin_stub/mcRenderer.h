// mcRenderer.h (stand-in, test infrastructure; see wr_stub_types.h): the
// renderer base class the drop-in derives from — constructor (engine, spp,
// maximum path length) and renderPixels(), as WalkRay's MCRenderer.
#pragma once

#include <string>
#include <vector>

#include "wr_stub_types.h"

namespace LFJ {

class RenderEngine;

class MCRenderer {
public:
    MCRenderer(RenderEngine* engine, uint spp, uint maxLen) : engine(engine), spp(spp), maxPathLen(maxLen) {}
    virtual ~MCRenderer() = default;
    virtual std::vector<vec3f> renderPixels() = 0;

protected:
    RenderEngine* engine;
    uint spp;
    uint maxPathLen;
    std::string name;
};

}  // namespace LFJ
