// bvh_build.h — binned-SAH BVH builder for bottom-level (triangles) and
// top-level (instances) acceleration structures.  Replaces the driver's
// BLAS/TLAS builds of PipelineRaytrace::createBottomLevelAS/TopLevelAS
// (src/pipeline/pipeline_raytrace.cpp:107-147).
#pragma once
#include <cstdint>
#include <vector>

#include "dev_types.h"

namespace asuna {

struct Aabb {
  float lo[3], hi[3];
};

struct BvhBuildOut {
  std::vector<BvhNode> nodes;   // node 0 is the root (always an inner node)
  std::vector<uint32_t> order;  // leaf order -> primitive id
  uint32_t maxDepth = 0;        // deepest leaf (root = 1)
};

// Builds a BVH over primitive boxes.  Leaf refs encode (first, count) over
// `order` with offset `firstBase` added; maxLeaf <= kMaxLeafTris.
// Returns false if the tree cannot be encoded (too many primitives).
bool buildBvh(const std::vector<Aabb>& boxes, const std::vector<float>& centroids, int maxLeaf, uint32_t firstBase,
              BvhBuildOut& out);


}  // namespace asuna
