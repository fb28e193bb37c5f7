// pt_mikktspace.h - MikkTSpace tangent frames for meshes without usable
// tangents (host side, world builder).
#pragma once

#include <stddef.h>

namespace ptw {

// `triangles` triangles given per corner (3 corners each): positions
// (3 floats), unit normals (3) and texture coordinates (2).  Writes the
// corner's unit tangent and handedness (+1 orientation-preserving, -1
// otherwise) as 4 floats per corner.
void mikktspace_tangents(size_t triangles, const float* pos, const float* nor, const float* uv, float* out);

}  // namespace ptw
