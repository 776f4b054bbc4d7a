// bvh_device.h — bottom-level BVHs of every mesh built on the GPU with the
// host builder's binned-SAH algorithm (bvh_device.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "dev_types.h"

namespace asuna {

struct DeviceBlas {
  BvhNode* nodes = nullptr;        // device; BLAS nodes first, room for `extraNodes` more after them
  TriDev* tris = nullptr;          // device; leaf order, triBase[m] + i for mesh m
  uint32_t nodeCount = 0;          // BLAS node slots used (unused chunk tails included)
  uint32_t nodeCapacity = 0;
  uint32_t maxDepth = 0;           // deepest task (root = 1)
  std::vector<int32_t> roots;      // per mesh: root node (-1: no triangles)
  std::vector<BvhNode> rootNodes;  // host copies of the root nodes, in root order
};

// Builds every mesh's BLAS on `stream` from the uploaded shading vertices
// (positions in VtxDev.pu) and index triples.  triBase / vtxBase: first
// triangle / vertex of each mesh (triBase has one more entry, the total).
// out.nodes / out.tris are device allocations the caller owns, also on failure.
int buildBlasDevice(const VtxDev* vtx, const uint4* idx, const std::vector<uint32_t>& triBase,
                    const std::vector<uint32_t>& vtxBase, uint32_t extraNodes, cudaStream_t stream, DeviceBlas& out);

}  // namespace asuna
