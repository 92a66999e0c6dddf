// Shim for the missing LiteScene mesh header (HydraCore3): the SimpleMesh
// container as the reference's renderer and builders use it (vertex
// attributes as float4 / float2 arrays, triangle indices, per-triangle
// material ids).  For compiling the reference in place (oracle pinning only);
// no mesh is ever loaded through it.
#pragma once
#include <cstdint>
#include <vector>
#include "LiteMath.h"

namespace cmesh4 {
struct SimpleMesh {
  std::vector<LiteMath::float4> vPos4f;
  std::vector<LiteMath::float4> vNorm4f;
  std::vector<LiteMath::float4> vTang4f;
  std::vector<LiteMath::float2> vTexCoord2f;
  std::vector<unsigned int> indices;
  std::vector<unsigned int> matIndices;
  size_t VerticesNum() const { return vPos4f.size(); }
  size_t IndicesNum() const { return indices.size(); }
  size_t TrianglesNum() const { return indices.size() / 3; }
};
}  // namespace cmesh4
