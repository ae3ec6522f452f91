// abstractObj.h (stand-in, test infrastructure; see wr_stub_types.h): a scene
// object as the drop-in reads it — world vertex positions and object-local
// triangles — plus the library descriptor the test's Describe callback hands
// over for its material.
#pragma once

#include <vector>

#include "walkray.h"
#include "wr_stub_types.h"

namespace LFJ {

class AbstractObject {
public:
    uint getVertexNum() const { return (uint)positions.size(); }
    vec3f getWorldVertexPosition(uint v) const { return positions[v]; }
    uint getTriangleNum() const { return (uint)triangles.size(); }
    vec3ui getVertexIndices(uint t) const { return triangles[t]; }

    std::vector<vec3f> positions;
    std::vector<vec3ui> triangles;
    wr_object_desc desc{};
};

}  // namespace LFJ
