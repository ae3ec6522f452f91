// renderEngine.h (stand-in, test infrastructure; see wr_stub_types.h): the
// engine that owns the scene the drop-in renders.
#pragma once

#include "scene.h"

namespace LFJ {

class RenderEngine {
public:
    Scene scene;
};

}  // namespace LFJ
