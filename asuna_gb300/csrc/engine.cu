// engine.cu — contexts, scene upload + acceleration-structure build, films,
// and the wavefront render driver behind the C ABI.
//
// The render driver replaces the offline frame loop of Tracer::runOffline
// (src/tracer/tracer.cpp:204-258), which submits one 1-spp vkCmdTraceRaysKHR
// per frame and waits: here the (shot, frame, pixel) samples of many frames
// and shots are packed into one wavefront of up to `capacity` paths, run as
// raygen -> (extend -> shade -> connect) x depth -> accumulate on one stream
// with no host synchronisation, and accumulated in frame order so the film
// equals the frame-by-frame result.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <memory>
#include <chrono>
#include <cmath>
#include <cstddef>
#include <cstring>
#include <new>
#include <thread>
#include <vector>

#include "bvh_build.h"
#include "bvh_device.h"
#include "common.h"
#include "host_scene.h"
#include "kernels.h"

using namespace asuna;

#include "handles.h"

namespace {

constexpr uint64_t kBytesPerPath = 2 * 32 + 16 + 4 + 48 + 48 + 16 + 4 * kNumShadeClasses;

template <class T>
int devUpload(asuna_scene* s, const T* host, size_t n, const T** out) {
  void* p = nullptr;
  size_t bytes = std::max<size_t>(n * sizeof(T), 16);
  ASUNA_CUDA_TRY(cudaMalloc(&p, bytes));
  s->allocs.push_back(p);
  if (n) ASUNA_CUDA_TRY(cudaMemcpy(p, host, n * sizeof(T), cudaMemcpyHostToDevice));
  s->stats.device_bytes += bytes;
  *out = static_cast<const T*>(p);
  return ASUNA_OK;
}

void dropGraphs(asuna_ctx* c);

int ensureWave(asuna_ctx* c, uint64_t paths) {
  if (c->wave.capacity >= paths) return ASUNA_OK;
  dropGraphs(c);
  if (c->wave.base) {
    cudaStreamSynchronize(c->stream);
    cudaFree(c->wave.base);
    c->wave = WaveAlloc{};
  }
  const uint64_t align = 256;
  auto pad = [&](uint64_t b) { return (b + align - 1) / align * align; };
  uint64_t off = 0;
  uint64_t o_rayO0 = off; off += pad(paths * 16);
  uint64_t o_rayO1 = off; off += pad(paths * 16);
  uint64_t o_rayD0 = off; off += pad(paths * 16);
  uint64_t o_rayD1 = off; off += pad(paths * 16);
  uint64_t o_hit = off; off += pad(paths * 16);
  uint64_t o_hinst = off; off += pad(paths * 4);
  uint64_t o_shO = off; off += pad(paths * 16);
  uint64_t o_shD = off; off += pad(paths * 16);
  uint64_t o_shC = off; off += pad(paths * 16);
  uint64_t o_path = off; off += pad(paths * sizeof(PathDev));
  uint64_t o_rad = off; off += pad(paths * 16);
  uint64_t o_rec = off; off += pad(paths * 16);
  uint64_t o_cls[kNumShadeClasses];
  for (int k = 0; k < kNumShadeClasses; ++k) {
    o_cls[k] = off;
    off += pad(paths * 4);
  }
  void* base = nullptr;
  const cudaError_t me = cudaMalloc(&base, off);
  if (me == cudaErrorMemoryAllocation) {
    cudaGetLastError();  // not sticky: a smaller path budget can still render
    return fail(ASUNA_ERR_OOM, "wavefront buffers of %llu bytes (%llu path slots) do not fit in device memory",
                (unsigned long long)off, (unsigned long long)paths);
  }
  ASUNA_CUDA_TRY(me);
  char* b = static_cast<char*>(base);
  WaveDev& v = c->wave.view;
  v.rayO[0] = reinterpret_cast<float4*>(b + o_rayO0);
  v.rayO[1] = reinterpret_cast<float4*>(b + o_rayO1);
  v.rayD[0] = reinterpret_cast<float4*>(b + o_rayD0);
  v.rayD[1] = reinterpret_cast<float4*>(b + o_rayD1);
  v.hit = reinterpret_cast<float4*>(b + o_hit);
  v.hitInst = reinterpret_cast<uint32_t*>(b + o_hinst);
  v.shO = reinterpret_cast<float4*>(b + o_shO);
  v.shD = reinterpret_cast<float4*>(b + o_shD);
  v.shC = reinterpret_cast<float4*>(b + o_shC);
  v.path = reinterpret_cast<PathDev*>(b + o_path);
  v.rad = reinterpret_cast<float4*>(b + o_rad);
  v.rec = reinterpret_cast<uint4*>(b + o_rec);
  for (int k = 0; k < kNumShadeClasses; ++k) v.cls[k] = reinterpret_cast<uint32_t*>(b + o_cls[k]);
  v.cnt = c->cnt;
  c->wave.base = base;
  c->wave.capacity = paths;
  return ASUNA_OK;
}

template <class T>
int ensureDevArray(asuna_ctx* c, T** ptr, size_t* cap, size_t n) {
  if (*cap >= n) return ASUNA_OK;
  ASUNA_CUDA_TRY(cudaStreamSynchronize(c->stream));
  if (*ptr) cudaFree(*ptr);
  *ptr = nullptr;
  *cap = 0;
  size_t want = std::max<size_t>(n, 64);
  ASUNA_CUDA_TRY(cudaMalloc(reinterpret_cast<void**>(ptr), want * sizeof(T)));
  *cap = want;
  return ASUNA_OK;
}

void dropGraphs(asuna_ctx* c) {
  for (auto& g : c->gcache) cudaGraphExecDestroy(g.exec);
  c->gcache.clear();
}

// Reports the traversals cut short on the device since the last report, once
// the copy of the count queued after the latest render has landed (waits for
// it: call only where the stream is waited for anyway).
int reportTraversal(asuna_ctx* c) {
  if (!c->errPending) return ASUNA_OK;
  ASUNA_CUDA_TRY(cudaEventSynchronize(c->errEvent));
  c->errPending = false;
  const unsigned long long now = *c->hostErr;
  if (now <= c->errSeen) return ASUNA_OK;
  const unsigned long long d = now - c->errSeen;
  c->errSeen = now;
  return fail(ASUNA_ERR_TRAVERSAL,
              "traversal cut short (stack of %d entries full, or a loop bound reached) in %llu warps or rays: "
              "the image is wrong",
              c->stackLimit > 0 ? c->stackLimit : kStackDepth, d);
}

struct Batch {
  uint32_t rangeBegin, rangeEnd;
  uint32_t paths;
  uint32_t maxPix;
  int maxDepth;
  uint64_t pathOffset;  // global index of the batch's first path (records)
};

}  // namespace

// ============================================================================
extern "C" {

int asuna_ctx_create(int device_ordinal, asuna_ctx** out) {
  clearError();
  if (!out) return fail(ASUNA_ERR_INVALID, "asuna_ctx_create: out is NULL");
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0)
    return fail(ASUNA_ERR_NO_DEVICE, "no CUDA device available (%s)", cudaGetErrorString(e));
  if (device_ordinal < 0 || device_ordinal >= n)
    return fail(ASUNA_ERR_INVALID, "device ordinal %d out of range [0, %d)", device_ordinal, n);
  ASUNA_CUDA_TRY(cudaSetDevice(device_ordinal));
  asuna_ctx* c = new (std::nothrow) asuna_ctx;
  if (!c) return fail(ASUNA_ERR_OOM, "host allocation failed");
  c->device = device_ordinal;
  cudaDeviceProp prop;
  ASUNA_CUDA_TRY(cudaGetDeviceProperties(&prop, device_ordinal));
  c->numSMs = prop.multiProcessorCount;
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    return fail(ASUNA_ERR_CUDA, "cudaStreamCreate failed");
  }
  if (cudaMalloc(&c->cnt, sizeof(DevCounters)) != cudaSuccess ||
      cudaMallocHost(&c->hostCnt, sizeof(DevCounters)) != cudaSuccess ||
      cudaMallocHost(&c->hostErr, sizeof(unsigned long long)) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->errEvent, cudaEventDisableTiming) != cudaSuccess) {
    cudaFree(c->cnt);
    cudaFreeHost(c->hostCnt);
    cudaFreeHost(c->hostErr);
    if (c->errEvent) cudaEventDestroy(c->errEvent);
    cudaStreamDestroy(c->stream);
    delete c;
    return fail(ASUNA_ERR_OOM, "counter allocation failed");
  }
  *c->hostErr = 0;
  cudaMemset(c->cnt, 0, sizeof(DevCounters));
  c->traceGrid = c->traceGridShadow = c->numSMs * traceBlocksPerSm();
  c->shadeGrid = c->numSMs * shadeBlocksPerSm();
  c->raygenGrid = c->numSMs * 16;
  *out = c;
  return ASUNA_OK;
}

int asuna_ctx_destroy(asuna_ctx* c) {
  if (!c) return ASUNA_OK;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  for (auto ev : c->events) cudaEventDestroy(ev);
  for (auto& g : c->gcache) cudaGraphExecDestroy(g.exec);
  if (c->dShots) cudaFree(c->dShots);
  if (c->dRanges) cudaFree(c->dRanges);
  if (c->wave.base) cudaFree(c->wave.base);
  if (c->cnt) cudaFree(c->cnt);
  if (c->hostCnt) cudaFreeHost(c->hostCnt);
  if (c->hostErr) cudaFreeHost(c->hostErr);
  if (c->errEvent) cudaEventDestroy(c->errEvent);
  cudaStreamDestroy(c->stream);
  delete c;
  return ASUNA_OK;
}

int asuna_ctx_sync(asuna_ctx* c) {
  clearError();
  if (!c) return fail(ASUNA_ERR_INVALID, "null context");
  ASUNA_CUDA_TRY(cudaStreamSynchronize(c->stream));
  return reportTraversal(c);
}

void* asuna_ctx_stream(asuna_ctx* c) { return c ? static_cast<void*>(c->stream) : nullptr; }

int asuna_ctx_set_counters(asuna_ctx* c, int enable) {
  if (!c) return fail(ASUNA_ERR_INVALID, "null context");
  c->counters = enable ? 1 : 0;
  return ASUNA_OK;
}

int asuna_ctx_set_ray_sort(asuna_ctx* c, int enable) {
  clearError();
  if (!c) return fail(ASUNA_ERR_INVALID, "null context");
  if (enable < 0 || enable > 3) return fail(ASUNA_ERR_INVALID, "ray sort %d not in {0, 1, 2, 3}", enable);
  c->raySort = enable;
  return ASUNA_OK;
}

namespace {
// Persistent traversal grids of the two passes: every resident block of the
// pass's kernel variant, capped by asuna_ctx_set_launch's blocks per SM.
void updateTraceGrids(asuna_ctx* c) {
  auto grid = [&](int occ) {
    const int m = traceBlocksPerSm(occ, c->traceThreads, c->sharedStack);
    return c->numSMs * (c->traceBlocksCap > 0 ? std::min(c->traceBlocksCap, m) : m);
  };
  c->traceGrid = grid(c->occupancy);
  c->traceGridShadow = grid(c->occupancyShadow);
}
bool validOccupancy(int b) { return b == 0 || b == 8 || b == 10 || b == 12; }
}  // namespace

int asuna_ctx_set_traversal(asuna_ctx* c, int refillExtend, int refillShadow, int specExtend, int specShadow,
                            int blocksPerSm) {
  clearError();
  if (!c) return fail(ASUNA_ERR_INVALID, "null context");
  if (!validOccupancy(blocksPerSm))
    return fail(ASUNA_ERR_INVALID, "traversal blocks per SM %d not in {0, 8, 10, 12}", blocksPerSm);
  c->occupancy = c->occupancyShadow = blocksPerSm == 0 ? kTraceMinBlocks : blocksPerSm;
  updateTraceGrids(c);
  const int r[2] = {refillExtend, refillShadow}, sp[2] = {specExtend, specShadow};
  for (int k = 0; k < 2; ++k) {
    if (r[k] < 0 || r[k] > 32) return fail(ASUNA_ERR_INVALID, "refill lanes %d not in [0, 32]", r[k]);
    if (sp[k] < -1 || sp[k] > 1) return fail(ASUNA_ERR_INVALID, "speculate %d not in {-1, 0, 1}", sp[k]);
    c->refill[k] = r[k] == 0 ? uint32_t(kRefillLanes) : uint32_t(r[k]);
    c->speculate[k] = sp[k] < 0 ? 1 : sp[k];
  }
  return ASUNA_OK;
}

int asuna_ctx_set_traversal_occupancy(asuna_ctx* c, int extendBlocksPerSm, int shadowBlocksPerSm) {
  clearError();
  if (!c) return fail(ASUNA_ERR_INVALID, "null context");
  if (!validOccupancy(extendBlocksPerSm) || !validOccupancy(shadowBlocksPerSm))
    return fail(ASUNA_ERR_INVALID, "traversal blocks per SM %d / %d not in {0, 8, 10, 12}", extendBlocksPerSm,
                shadowBlocksPerSm);
  c->occupancy = extendBlocksPerSm == 0 ? kTraceMinBlocks : extendBlocksPerSm;
  c->occupancyShadow = shadowBlocksPerSm == 0 ? kTraceMinBlocks : shadowBlocksPerSm;
  updateTraceGrids(c);
  return ASUNA_OK;
}

int asuna_ctx_set_bvh_build(asuna_ctx* c, int mode) {
  clearError();
  if (!c) return fail(ASUNA_ERR_INVALID, "null context");
  if (mode != 0 && mode != 1) return fail(ASUNA_ERR_INVALID, "BVH build mode %d not in {0, 1}", mode);
  c->bvhBuild = mode;
  return ASUNA_OK;
}

int asuna_ctx_set_traversal_stack(asuna_ctx* c, int entries) {
  clearError();
  if (!c) return fail(ASUNA_ERR_INVALID, "null context");
  if (entries < 0 || entries > kStackDepth)
    return fail(ASUNA_ERR_INVALID, "traversal stack of %d entries not in [0, %d]", entries, kStackDepth);
  c->stackLimit = entries == kStackDepth ? 0 : entries;
  return ASUNA_OK;
}

int asuna_ctx_set_traversal_shape(asuna_ctx* c, int threadsPerBlock, int sharedStack) {
  clearError();
  if (!c) return fail(ASUNA_ERR_INVALID, "null context");
  if (threadsPerBlock != 0 && threadsPerBlock != 64 && threadsPerBlock != 128 && threadsPerBlock != 256)
    return fail(ASUNA_ERR_INVALID, "traversal block of %d threads not in {0, 64, 128, 256}", threadsPerBlock);
  if (sharedStack != 0 && sharedStack != 16 && sharedStack != 24 && sharedStack != 32)
    return fail(ASUNA_ERR_INVALID, "shared stack of %d entries not in {0, 16, 24, 32}", sharedStack);
  c->traceThreads = threadsPerBlock ? threadsPerBlock : kTraceThreads;
  c->sharedStack = sharedStack ? sharedStack : kSharedStack;
  updateTraceGrids(c);
  return ASUNA_OK;
}

int asuna_ctx_set_launch(asuna_ctx* c, int traceBlocks, int shadeBlocks) {
  if (!c) return fail(ASUNA_ERR_INVALID, "null context");
  const int smax = shadeBlocksPerSm();
  const int sh = shadeBlocks <= 0 ? smax : std::min(shadeBlocks, smax);
  c->traceBlocksCap = traceBlocks > 0 ? traceBlocks : 0;
  updateTraceGrids(c);
  c->shadeGrid = c->numSMs * sh;
  return ASUNA_OK;
}

int asuna_ctx_set_graphs(asuna_ctx* c, int enable) {
  if (!c) return fail(ASUNA_ERR_INVALID, "null context");
  c->graphs = enable ? 1 : 0;
  return ASUNA_OK;
}

int asuna_ctx_set_path_budget(asuna_ctx* c, uint64_t bytes) {
  if (!c) return fail(ASUNA_ERR_INVALID, "null context");
  c->pathBudget = bytes ? bytes : (4ull << 30);
  return ASUNA_OK;
}

// ---------------------------------------------------------------------------
int asuna_scene_create(asuna_ctx* c, const asuna_scene_desc* d, asuna_scene** out) {
  clearError();
  if (!c || !d || !out) return fail(ASUNA_ERR_INVALID, "asuna_scene_create: null argument");
  int rc = validateSceneDesc(d);
  if (rc) return rc;
  ASUNA_CUDA_TRY(cudaSetDevice(c->device));
  auto t0 = std::chrono::steady_clock::now();
  asuna_scene* s = new (std::nothrow) asuna_scene;
  if (!s) return fail(ASUNA_ERR_OOM, "host allocation failed");
  s->device = c->device;
  std::unique_ptr<asuna_scene, int (*)(asuna_scene*)> guard(s, asuna_scene_destroy);

  // ---- bottom level: one BVH per mesh, built on host threads ----
  const uint32_t nm = d->num_meshes;
  std::vector<uint32_t> triBase(nm + 1, 0), vtxBase(nm + 1, 0);
  for (uint32_t m = 0; m < nm; ++m) {
    triBase[m + 1] = triBase[m] + d->meshes[m].num_triangles;
    vtxBase[m + 1] = vtxBase[m] + d->meshes[m].num_vertices;
  }
  if (triBase[nm] > kMaxLeafFirst) return fail(ASUNA_ERR_UNSUPPORTED, "scene has more than 2^28 triangles");
  // shading data first: the device build reads positions and indices from them
  SceneDev& v = s->view;
  {
    std::vector<VtxDev> vtx(vtxBase[nm]);
    std::vector<uint4> idx(triBase[nm]);
    for (uint32_t m = 0; m < nm; ++m) {
      const asuna_mesh_desc& md = d->meshes[m];
      for (uint32_t k = 0; k < md.num_vertices; ++k) {
        const asuna_vertex& gv = md.vertices[k];
        vtx[vtxBase[m] + k].pu = make_float4(gv.pos[0], gv.pos[1], gv.pos[2], gv.uv[0]);
        vtx[vtxBase[m] + k].nv = make_float4(gv.normal[0], gv.normal[1], gv.normal[2], gv.uv[1]);
      }
      for (uint32_t t = 0; t < md.num_triangles; ++t)
        idx[triBase[m] + t] = make_uint4(md.indices[3 * t], md.indices[3 * t + 1], md.indices[3 * t + 2], 0u);
    }
    if ((rc = devUpload(s, vtx.data(), vtx.size(), &v.vtx)) || (rc = devUpload(s, idx.data(), idx.size(), &v.idx)))
      return rc;
  }
  // ---- bottom level: one BVH per mesh, on the device (default) or host threads ----
  const bool onDevice = c->bvhBuild == 0;
  std::vector<BvhBuildOut> blas(onDevice ? 0 : nm);
  DeviceBlas dblas;
  std::vector<BvhNode> nodes;
  std::vector<TriDev> tris;
  std::vector<int32_t> rootIndex(nm, -1);
  std::vector<BvhNode> rootNode(nm);
  uint32_t blasNodes = 0, blasDepth = 0;
  const uint32_t extraNodes = 2 * d->num_instances + 4;
  if (onDevice) {
    rc = buildBlasDevice(v.vtx, v.idx, triBase, vtxBase, extraNodes, c->stream, dblas);
    if (dblas.nodes) {
      s->allocs.push_back(dblas.nodes);
      s->stats.device_bytes += uint64_t(dblas.nodeCapacity) * sizeof(BvhNode);
    }
    if (dblas.tris) {
      s->allocs.push_back(dblas.tris);
      s->stats.device_bytes += uint64_t(std::max<uint32_t>(triBase[nm], 1)) * sizeof(TriDev);
    }
    if (rc) return rc;
    blasNodes = dblas.nodeCount;
    blasDepth = dblas.maxDepth;
    for (uint32_t m = 0; m < nm; ++m)
      if (dblas.roots[m] >= 0) {
        rootIndex[m] = dblas.roots[m];
        rootNode[m] = dblas.rootNodes[size_t(dblas.roots[m])];
      }
  } else {
    std::vector<int> okMesh(nm, 1);
    {
      std::atomic<uint32_t> next{0};
      unsigned nt = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
      std::vector<std::thread> th;
      for (unsigned t = 0; t < nt; ++t)
        th.emplace_back([&] {
          for (uint32_t m; (m = next++) < nm;) {
            const asuna_mesh_desc& md = d->meshes[m];
            std::vector<Aabb> boxes(md.num_triangles);
            std::vector<float> cen(size_t(md.num_triangles) * 3);
            for (uint32_t i = 0; i < md.num_triangles; ++i) {
              const float* p0 = md.vertices[md.indices[3 * i]].pos;
              const float* p1 = md.vertices[md.indices[3 * i + 1]].pos;
              const float* p2 = md.vertices[md.indices[3 * i + 2]].pos;
              for (int k = 0; k < 3; ++k) {
                boxes[i].lo[k] = std::min(p0[k], std::min(p1[k], p2[k]));
                boxes[i].hi[k] = std::max(p0[k], std::max(p1[k], p2[k]));
                cen[3 * i + k] = 0.5f * (boxes[i].lo[k] + boxes[i].hi[k]);
              }
            }
            okMesh[m] = buildBvh(boxes, cen, 4, triBase[m], blas[m]) ? 1 : 0;
          }
        });
      for (auto& t : th) t.join();
    }
    for (uint32_t m = 0; m < nm; ++m)
      if (!okMesh[m]) return fail(ASUNA_ERR_UNSUPPORTED, "mesh %u: BVH cannot be encoded", m);
    std::vector<uint32_t> nodeBase(nm + 1, 0);
    for (uint32_t m = 0; m < nm; ++m) {
      nodeBase[m + 1] = nodeBase[m] + uint32_t(blas[m].nodes.size());
      blasDepth = std::max(blasDepth, blas[m].maxDepth);
      if (d->meshes[m].num_triangles) {
        rootIndex[m] = int32_t(nodeBase[m]);
        rootNode[m] = blas[m].nodes[0];
      }
    }
    blasNodes = nodeBase[nm];
    nodes.reserve(nodeBase[nm] + extraNodes);
    tris.resize(triBase[nm]);
    for (uint32_t m = 0; m < nm; ++m) {
      const asuna_mesh_desc& md = d->meshes[m];
      for (BvhNode n : blas[m].nodes) {
        if (n.ref.x >= 0) n.ref.x += int32_t(nodeBase[m]);
        if (n.ref.y >= 0) n.ref.y += int32_t(nodeBase[m]);
        nodes.push_back(n);
      }
      for (uint32_t i = 0; i < md.num_triangles; ++i) {
        const uint32_t prim = blas[m].order[i];
        const float* p0 = md.vertices[md.indices[3 * prim]].pos;
        const float* p1 = md.vertices[md.indices[3 * prim + 1]].pos;
        const float* p2 = md.vertices[md.indices[3 * prim + 2]].pos;
        TriDev& t = tris[triBase[m] + i];
        uint32_t pb = prim;
        float pf;
        std::memcpy(&pf, &pb, 4);
        t.v0 = make_float4(p0[0], p0[1], p0[2], pf);
        t.v1 = make_float4(p1[0], p1[1], p1[2], 0.0f);
        t.v2 = make_float4(p2[0], p2[1], p2[2], 0.0f);
      }
    }
  }
  // ---- instances + top level ----
  const uint32_t ni = d->num_instances;
  std::vector<InstDev> inst(ni);
  std::vector<Aabb> iboxes;
  std::vector<float> icen;
  std::vector<uint32_t> ids;
  for (uint32_t i = 0; i < ni; ++i) {
    const asuna_instance_desc& id = d->instances[i];
    InstDev& I = inst[i];
    std::memset(&I, 0, sizeof(I));
    float w2o[12];
    invert3x4(id.transform, w2o);
    for (int r = 0; r < 3; ++r) {
      I.w2o[r] = make_float4(w2o[r * 4], w2o[r * 4 + 1], w2o[r * 4 + 2], w2o[r * 4 + 3]);
      I.o2w[r] = make_float4(id.transform[r * 4], id.transform[r * 4 + 1], id.transform[r * 4 + 2],
                             id.transform[r * 4 + 3]);
    }
    const uint32_t m = id.mesh_id;
    const bool empty = d->meshes[m].num_triangles == 0;
    I.blasRoot = empty ? -1 : rootIndex[m];
    I.vtxBase = vtxBase[m];
    I.idxBase = triBase[m];
    I.matId = id.light_id >= 0 ? -1 : id.material_id;
    I.lightId = id.light_id;
    I.matType = id.light_id >= 0 ? 0u : d->materials[id.material_id].type;
    s->view.classMask |= 1u << (id.light_id >= 0 ? int(kClsTerminal) : shadeClassOf(I.matType));
    if (empty) continue;
    // world box of the BLAS root's children
    const BvhNode& r = rootNode[m];
    float lo[3], hi[3];
    nodeGetBox(r, 0, lo, hi);
    if (r.ref.y != kStackSentinel) {
      float lo1[3], hi1[3];
      nodeGetBox(r, 1, lo1, hi1);
      for (int k = 0; k < 3; ++k) {
        lo[k] = std::min(lo[k], lo1[k]);
        hi[k] = std::max(hi[k], hi1[k]);
      }
    }
    Aabb wb;
    for (int k = 0; k < 3; ++k) {
      wb.lo[k] = INFINITY;
      wb.hi[k] = -INFINITY;
    }
    for (int cidx = 0; cidx < 8; ++cidx) {
      double p[3] = {(cidx & 1) ? hi[0] : lo[0], (cidx & 2) ? hi[1] : lo[1], (cidx & 4) ? hi[2] : lo[2]};
      for (int k = 0; k < 3; ++k) {
        double v = double(id.transform[k * 4]) * p[0] + double(id.transform[k * 4 + 1]) * p[1] +
                   double(id.transform[k * 4 + 2]) * p[2] + double(id.transform[k * 4 + 3]);
        wb.lo[k] = std::min(wb.lo[k], std::nextafter(float(v), -INFINITY));
        wb.hi[k] = std::max(wb.hi[k], std::nextafter(float(v), INFINITY));
      }
    }
    iboxes.push_back(wb);
    for (int k = 0; k < 3; ++k) icen.push_back(0.5f * (wb.lo[k] + wb.hi[k]));
    ids.push_back(i);
  }
  {
    // world bounds for the ray-sort origin cells
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (const Aabb& b : iboxes)
      for (int k = 0; k < 3; ++k) {
        lo[k] = std::min(lo[k], b.lo[k]);
        hi[k] = std::max(hi[k], b.hi[k]);
      }
    float sc[3];
    for (int k = 0; k < 3; ++k) {
      if (!(lo[k] <= hi[k])) lo[k] = hi[k] = 0.0f;
      sc[k] = hi[k] > lo[k] ? 4.0f / (hi[k] - lo[k]) : 0.0f;
    }
    s->view.boundLo = make_float4(lo[0], lo[1], lo[2], 0.0f);
    s->view.cellScale = make_float4(sc[0], sc[1], sc[2], 0.0f);
  }
  BvhBuildOut tlas;
  if (!buildBvh(iboxes, icen, 1, 0, tlas)) return fail(ASUNA_ERR_UNSUPPORTED, "TLAS cannot be encoded");
  const uint32_t tlasBase = blasNodes;
  std::vector<BvhNode> tlasNodes;
  for (BvhNode n : tlas.nodes) {
    for (int side = 0; side < 2; ++side) {
      int32_t& ref = side == 0 ? n.ref.x : n.ref.y;
      if (ref == kStackSentinel) continue;
      if (ref >= 0)
        ref += int32_t(tlasBase);
      else
        ref = encodeLeaf(ids[tlas.order[leafFirst(ref)]], 1);
    }
    tlasNodes.push_back(n);
  }
  if (tlasNodes.size() > extraNodes) return fail(ASUNA_ERR_INVALID, "TLAS larger than reserved");
  if (tlas.maxDepth + blasDepth + 1 > uint32_t(kStackDepth))
    return fail(ASUNA_ERR_UNSUPPORTED, "BVH too deep for the traversal stack (TLAS %u + BLAS %u levels, limit %d)",
                tlas.maxDepth, blasDepth, kStackDepth - 1);
  // ---- materials, lights, textures, environment ----
  std::vector<MatDev> mats(d->num_materials);
  for (uint32_t i = 0; i < d->num_materials; ++i) {
    const asuna_material& m = d->materials[i];
    float tb;
    std::memcpy(&tb, &m.type, 4);
    // emissive materials carry their radiance where the others carry the albedo
    const float* rgb = m.type == ASUNA_MAT_EMISSIVE ? m.radiance : m.diffuse;
    mats[i].a = make_float4(rgb[0], rgb[1], rgb[2], tb);
    // Disney: (anisotropic, opacity, ior, -); others: (alpha x, alpha y, ior, fdrInt)
    mats[i].b = m.type == ASUNA_MAT_DISNEY ? make_float4(m.anisotropic, m.rho_spec[0], m.ior, 0.0f)
                                           : make_float4(m.aniso_alpha[0], m.aniso_alpha[1], m.ior, m.radiance[0]);
    // Phong: specular reflectance (rhoSpec) and exponent; kang18: rhoSpec and
    // opacity (metalness); PBR:
    // roughness, metalness, opacity (specular); Disney: metalness, roughness,
    // subsurface, specular tint; others: radiance
    mats[i].c = m.type == ASUNA_MAT_PHONG    ? make_float4(m.rho_spec[0], m.rho_spec[1], m.rho_spec[2], m.specular)
                : m.type == ASUNA_MAT_KANG18 ? make_float4(m.rho_spec[0], m.rho_spec[1], m.rho_spec[2], m.metalness)
                : m.type == ASUNA_MAT_PBR_METALNESS_ROUGHNESS
                    ? make_float4(m.roughness, m.metalness, m.specular, 0.0f)
                : m.type == ASUNA_MAT_DISNEY ? make_float4(m.metalness, m.roughness, m.subsurface, m.specular_tint)
                                             : make_float4(m.radiance[0], m.radiance[1], m.radiance[2], 0.0f);
    // Disney: sheen, sheen tint, clearcoat, clearcoat gloss; others: radiance factor
    // brdf_pbr_metalness_roughness.rchit:152-160, brdf_disney.rchit:409-417,
    // brdf_kang18.rchit:150-187: opacity in specular / rho_spec[0] / metalness
    if (m.opacity_texture_id >= 0 || (m.type == ASUNA_MAT_PBR_METALNESS_ROUGHNESS && m.specular != 0.0f) ||
        (m.type == ASUNA_MAT_DISNEY && m.rho_spec[0] != 0.0f) || (m.type == ASUNA_MAT_KANG18 && m.metalness != 0.0f))
      if (m.type == ASUNA_MAT_PBR_METALNESS_ROUGHNESS || m.type == ASUNA_MAT_DISNEY || m.type == ASUNA_MAT_KANG18)
        s->view.passThrough = 1;
    mats[i].t0 = make_int4(m.diffuse_texture_id, m.normal_texture_id, m.roughness_texture_id, m.metalness_texture_id);
    mats[i].t1 = make_int4(m.radiance_texture_id, m.tangent_texture_id, m.opacity_texture_id, -1);
    mats[i].d = m.type == ASUNA_MAT_DISNEY
                    ? make_float4(m.sheen, m.sheen_tint, m.clearcoat, m.clearcoat_gloss)
                    : make_float4(m.radiance_factor[0], m.radiance_factor[1], m.radiance_factor[2], 0.0f);
  }
  std::vector<LightDev> lights(std::max(1u, d->num_lights));
  for (uint32_t i = 0; i < d->num_lights; ++i) {
    const asuna_light& l = d->lights[i];
    float tb, db;
    std::memcpy(&tb, &l.type, 4);
    std::memcpy(&db, &l.double_side, 4);
    lights[i].pos = make_float4(l.position[0], l.position[1], l.position[2], tb);
    lights[i].dir = make_float4(l.direction[0], l.direction[1], l.direction[2], l.radius);
    lights[i].rad = make_float4(l.radiance[0], l.radiance[1], l.radiance[2], 0.0f);
    lights[i].u = make_float4(l.u[0], l.u[1], l.u[2], l.area);
    lights[i].v = make_float4(l.v[0], l.v[1], l.v[2], db);
  }
  uint32_t ew = 1, eh = 1;
  // material textures: one texel pool and a (first, w, h) table
  std::vector<int4> texInfo(std::max(1u, d->num_textures), make_int4(0, 1, 1, 0));
  uint64_t nTexels = 0;
  for (uint32_t i = 0; i < d->num_textures; ++i) nTexels += uint64_t(d->textures[i].width) * d->textures[i].height;
  std::vector<float4> texels(std::max<uint64_t>(nTexels, 1), make_float4(0, 0, 0, 0));
  {
    uint64_t off = 0;
    for (uint32_t i = 0; i < d->num_textures; ++i) {
      const asuna_texture_desc& t = d->textures[i];
      const uint64_t n = uint64_t(t.width) * t.height;
      texInfo[i] = make_int4(int32_t(uint32_t(off)), int32_t(t.width), int32_t(t.height), 0);
      std::memcpy(&texels[off], t.rgba, n * sizeof(float4));
      off += n;
    }
  }
  std::vector<float4> env(1, make_float4(0, 0, 0, 0));
  std::vector<float2> marg(1, make_float2(0, 0)), cond(1, make_float2(0, 0));
  if (d->envmap.rgba && d->envmap.width && d->envmap.height) {
    ew = d->envmap.width;
    eh = d->envmap.height;
    const size_t np = size_t(ew) * eh;
    env.resize(np);
    std::memcpy(env.data(), d->envmap.rgba, np * 16);
    marg.resize(np);
    cond.resize(np);
    asuna_envmap_tables(ew, eh, d->envmap.rgba, reinterpret_cast<float*>(marg.data()),
                        reinterpret_cast<float*>(cond.data()));
  }
  if (onDevice) {
    // the top level goes after the device-built bottom levels
    v.nodes = dblas.nodes;
    v.tris = dblas.tris;
    if (!tlasNodes.empty())
      ASUNA_CUDA_TRY(cudaMemcpy(dblas.nodes + tlasBase, tlasNodes.data(), tlasNodes.size() * sizeof(BvhNode),
                                cudaMemcpyHostToDevice));
  } else {
    nodes.insert(nodes.end(), tlasNodes.begin(), tlasNodes.end());
    if ((rc = devUpload(s, nodes.data(), nodes.size(), &v.nodes)) || (rc = devUpload(s, tris.data(), tris.size(), &v.tris)))
      return rc;
  }
  if ((rc = devUpload(s, inst.data(), inst.size(), &v.inst)) ||
      (rc = devUpload(s, mats.data(), mats.size(), &v.mats)) ||
      (rc = devUpload(s, lights.data(), lights.size(), &v.lights)) ||
      (rc = devUpload(s, env.data(), env.size(), &v.env)) || (rc = devUpload(s, marg.data(), marg.size(), &v.marg)) ||
      (rc = devUpload(s, cond.data(), cond.size(), &v.cond)) ||
      (rc = devUpload(s, texels.data(), texels.size(), &v.texels)) ||
      (rc = devUpload(s, texInfo.data(), texInfo.size(), &v.texInfo)))
    return rc;
  v.tlasRoot = int32_t(tlasBase);
  std::memset(&v.sky, 0, sizeof(v.sky));
  if (d->sun_and_sky && d->sun_and_sky->in_use == 1) v.sky = *d->sun_and_sky;
  v.envW = int32_t(ew);
  v.envH = int32_t(eh);
  v.numInst = int32_t(ni);
  s->stats.triangles = triBase[nm];
  s->stats.instances = ni;
  s->stats.blas_nodes = blasNodes;
  s->stats.tlas_nodes = tlas.nodes.size();
  s->stats.build_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  *out = guard.release();
  return ASUNA_OK;
}

int asuna_scene_destroy(asuna_scene* s) {
  if (!s) return ASUNA_OK;
  cudaSetDevice(s->device);
  for (void* p : s->allocs) cudaFree(p);
  delete s;
  return ASUNA_OK;
}

int asuna_scene_get_stats(const asuna_scene* s, asuna_scene_stats* out) {
  if (!s || !out) return fail(ASUNA_ERR_INVALID, "null argument");
  *out = s->stats;
  return ASUNA_OK;
}

// ---------------------------------------------------------------------------
int asuna_film_create(asuna_ctx* c, uint32_t w, uint32_t h, asuna_film** out) {
  clearError();
  if (!c || !out || !w || !h) return fail(ASUNA_ERR_INVALID, "asuna_film_create: bad argument");
  if (uint64_t(w) * h > (1ull << 28)) return fail(ASUNA_ERR_INVALID, "film %ux%u too large", w, h);
  ASUNA_CUDA_TRY(cudaSetDevice(c->device));
  asuna_film* f = new (std::nothrow) asuna_film;
  if (!f) return fail(ASUNA_ERR_OOM, "host allocation failed");
  f->device = c->device;
  f->width = w;
  f->height = h;
  const size_t np = size_t(w) * h;
  if (cudaMalloc(&f->rad, np * 16) != cudaSuccess || cudaMalloc(&f->w, np * 16) != cudaSuccess ||
      cudaMalloc(&f->ch, np * 16 * ASUNA_MAX_CHANNELS) != cudaSuccess) {
    cudaFree(f->rad);
    cudaFree(f->w);
    cudaFree(f->ch);
    delete f;
    return fail(ASUNA_ERR_OOM, "film allocation failed (%ux%u)", w, h);
  }
  *out = f;
  return asuna_film_clear(c, f);
}

int asuna_film_destroy(asuna_film* f) {
  if (!f) return ASUNA_OK;
  cudaSetDevice(f->device);
  cudaFree(f->rad);
  cudaFree(f->w);
  cudaFree(f->ch);
  delete f;
  return ASUNA_OK;
}

int asuna_film_clear(asuna_ctx* c, asuna_film* f) {
  if (!c || !f) return fail(ASUNA_ERR_INVALID, "null argument");
  const size_t np = size_t(f->width) * f->height;
  ASUNA_CUDA_TRY(cudaMemsetAsync(f->rad, 0, np * 16, c->stream));
  ASUNA_CUDA_TRY(cudaMemsetAsync(f->w, 0, np * 16, c->stream));
  ASUNA_CUDA_TRY(cudaMemsetAsync(f->ch, 0, np * 16 * ASUNA_MAX_CHANNELS, c->stream));
  return ASUNA_OK;
}

int asuna_film_read(asuna_ctx* c, asuna_film* f, int image, float* host) {
  if (!c || !f || !host) return fail(ASUNA_ERR_INVALID, "null argument");
  if (image < 0 || image >= ASUNA_NUM_OUTPUT_IMAGES) return fail(ASUNA_ERR_INVALID, "image %d out of range", image);
  const size_t np = size_t(f->width) * f->height;
  const float4* src = image == 0 ? f->rad : (image == 8 ? f->w : f->ch + size_t(image - 1) * np);
  ASUNA_CUDA_TRY(cudaMemcpyAsync(host, src, np * 16, cudaMemcpyDeviceToHost, c->stream));
  ASUNA_CUDA_TRY(cudaStreamSynchronize(c->stream));
  return reportTraversal(c);
}

int asuna_film_image(asuna_film* f, int image, float** out) {
  if (!f || !out) return fail(ASUNA_ERR_INVALID, "null argument");
  if (image < 0 || image >= ASUNA_NUM_OUTPUT_IMAGES) return fail(ASUNA_ERR_INVALID, "image %d out of range", image);
  const size_t np = size_t(f->width) * f->height;
  float4* p = image == 0 ? f->rad : (image == 8 ? f->w : f->ch + size_t(image - 1) * np);
  *out = reinterpret_cast<float*>(p);
  return ASUNA_OK;
}

// ---------------------------------------------------------------------------
static int renderImpl(asuna_ctx* c, const asuna_scene* s, const asuna_shot* shots, asuna_film* const* films,
                      uint32_t n, asuna_render_stats* stats, asuna_path_record* hostRecords) {
  clearError();
  if (!c || !s || !shots || !films || n == 0) return fail(ASUNA_ERR_INVALID, "render: null or empty argument");
  if (s->device != c->device) return fail(ASUNA_ERR_INVALID, "scene and context are on different devices");
  ASUNA_CUDA_TRY(cudaSetDevice(c->device));
  cudaGetLastError();  // a non-sticky error left by the caller's own CUDA calls is not this call's failure
  std::vector<ShotDev> sd(n);
  uint64_t maxPix = 0;
  for (uint32_t i = 0; i < n; ++i) {
    const asuna_shot& sh = shots[i];
    const asuna_film* f = films[i];
    if (!f) return fail(ASUNA_ERR_INVALID, "shot %u: null film", i);
    if (f->device != c->device) return fail(ASUNA_ERR_INVALID, "shot %u: film on another device", i);
    if (sh.width != f->width || sh.height != f->height)
      return fail(ASUNA_ERR_INVALID, "shot %u: %ux%u does not match film %ux%u", i, sh.width, sh.height, f->width,
                  f->height);
    if (sh.state.max_path_depth < 1 || sh.state.max_path_depth > 32)
      return fail(ASUNA_ERR_INVALID, "shot %u: max_path_depth %d outside [1, 32]", i, sh.state.max_path_depth);
    if (sh.state.n_multi_channel > ASUNA_MAX_CHANNELS)
      return fail(ASUNA_ERR_INVALID, "shot %u: %u channels exceed %d", i, sh.state.n_multi_channel,
                  ASUNA_MAX_CHANNELS);
    if (sh.camera.type != ASUNA_CAMERA_PERSPECTIVE && sh.camera.type != ASUNA_CAMERA_OPENCV)
      return fail(ASUNA_ERR_UNSUPPORTED, "shot %u: camera type %u", i, sh.camera.type);
    ShotDev& d = sd[i];
    std::memset(&d, 0, sizeof(d));
    d.cam = sh.camera;
    d.state = sh.state;
    d.width = sh.width;
    d.height = sh.height;
    d.seed = sh.seed;
    d.flags = sh.flags;
    d.rrDepth = sh.rr_depth;
    d.depthSlot = sh.depth_out_channel;
    d.filmRad = films[i]->rad;
    d.filmW = films[i]->w;
    d.filmCh = films[i]->ch;
    maxPix = std::max<uint64_t>(maxPix, uint64_t(sh.width) * sh.height);
  }
  // capacity: at least one frame of the largest shot, else the memory budget
  uint64_t cap = std::max<uint64_t>(maxPix, c->pathBudget / kBytesPerPath);
  cap = std::min<uint64_t>(cap, 1ull << 30);
  if (hostRecords) {
    uint64_t total = uint64_t(shots[0].width) * shots[0].height * shots[0].frames;
    cap = std::max<uint64_t>(std::min<uint64_t>(cap, total), maxPix);
  }
  int rc = ensureWave(c, cap);
  if (rc) return rc;
  cap = c->wave.capacity;
  // pack (shot, frames) into batches of at most `cap` paths
  std::vector<RangeDev> ranges;
  std::vector<Batch> batches;
  {
    Batch b{0, 0, 0, 0, 0, 0};
    uint64_t global = 0;
    for (uint32_t i = 0; i < n; ++i) {
      const uint32_t npix = shots[i].width * shots[i].height;
      uint32_t f = 0;
      while (f < shots[i].frames) {
        uint64_t room = (cap - b.paths) / npix;
        if (room == 0) {
          b.rangeEnd = uint32_t(ranges.size());
          batches.push_back(b);
          global += b.paths;
          b = Batch{uint32_t(ranges.size()), 0, 0, 0, 0, global};
          continue;
        }
        uint32_t k = uint32_t(std::min<uint64_t>(room, shots[i].frames - f));
        RangeDev r{};
        r.pathBegin = b.paths;
        r.shot = i;
        r.frameBegin = shots[i].frame0 + f;
        r.nframes = k;
        r.npix = npix;
        ranges.push_back(r);
        b.paths += k * npix;
        b.maxPix = std::max(b.maxPix, npix);
        b.maxDepth = std::max(b.maxDepth, shots[i].state.max_path_depth);
        f += k;
      }
    }
    if (b.paths) {
      b.rangeEnd = uint32_t(ranges.size());
      batches.push_back(b);
    }
  }
  if (batches.empty()) return ASUNA_OK;
  asuna_path_record* dRec = nullptr;
  {
    const void* oldS = c->dShots;
    const void* oldR = c->dRanges;
    if ((rc = ensureDevArray(c, &c->dShots, &c->shotsCap, sd.size())) ||
        (rc = ensureDevArray(c, &c->dRanges, &c->rangesCap, ranges.size())))
      return rc;
    if (oldS != c->dShots || oldR != c->dRanges) dropGraphs(c);
  }
  ShotDev* dShots = c->dShots;
  RangeDev* dRanges = c->dRanges;
  ASUNA_CUDA_TRY(cudaMemcpyAsync(dShots, sd.data(), sd.size() * sizeof(ShotDev), cudaMemcpyHostToDevice, c->stream));
  ASUNA_CUDA_TRY(
      cudaMemcpyAsync(dRanges, ranges.data(), ranges.size() * sizeof(RangeDev), cudaMemcpyHostToDevice, c->stream));
  uint64_t totalPaths = 0;
  for (auto& b : batches) totalPaths += b.paths;
  if (hostRecords) ASUNA_CUDA_TRY(cudaMallocAsync(&dRec, totalPaths * sizeof(asuna_path_record), c->stream));
  // the statistics start at zero; the cut-short count (last) is cumulative
  if (stats) ASUNA_CUDA_TRY(cudaMemsetAsync(c->cnt, 0, offsetof(DevCounters, stackOverflow), c->stream));
  // timing events: [begin, end] + one pair per extend / shade / connect launch
  size_t evNeed = 2;
  for (auto& b : batches) evNeed += size_t(wavefrontPasses(b.maxDepth, s->view)) * 8;
  if (stats) {
    while (c->events.size() < evNeed) {
      cudaEvent_t ev;
      ASUNA_CUDA_TRY(cudaEventCreate(&ev));
      c->events.push_back(ev);
    }
    ASUNA_CUDA_TRY(cudaEventRecord(c->events[0], c->stream));
  }
  size_t evi = 2;
  std::vector<std::pair<int, size_t>> timed;  // (kind, first event index)
  // CUDA graph of the whole launch sequence, reused while the key matches
  const bool useGraph = c->graphs && !hostRecords;
  GraphEntry* hitEntry = nullptr;
  std::vector<uint64_t> key;
  if (useGraph) {
    key.resize((sizeof(SceneDev) + 7) / 8, 0);
    std::memcpy(key.data(), &s->view, sizeof(SceneDev));  // every scene pointer and size
    key.insert(key.end(), {uint64_t(uintptr_t(c->wave.base)), c->wave.capacity,
           uint64_t(uintptr_t(dShots)), uint64_t(uintptr_t(dRanges)), uint64_t(c->traceGrid), uint64_t(c->shadeGrid),
           uint64_t(c->raygenGrid), uint64_t(c->counters), uint64_t(stats ? 1 : 0), uint64_t(c->refill[0]),
           uint64_t(c->refill[1]), uint64_t(c->speculate[0]), uint64_t(c->speculate[1]), uint64_t(c->occupancy),
           uint64_t(c->raySort), uint64_t(c->stackLimit), uint64_t(c->traceThreads), uint64_t(c->sharedStack),
           uint64_t(c->occupancyShadow), uint64_t(c->traceGridShadow)});
    for (const Batch& b : batches)
      key.insert(key.end(), {b.rangeBegin, b.rangeEnd, b.paths, b.maxPix, uint64_t(b.maxDepth)});
    for (auto& g : c->gcache)
      if (g.key == key) hitEntry = &g;
  }
  if (hitEntry) {
    hitEntry->lastUse = ++c->useClock;
    ASUNA_CUDA_TRY(cudaGraphLaunch(hitEntry->exec, c->stream));
    timed = hitEntry->timed;
  } else {
  if (useGraph) ASUNA_CUDA_TRY(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  bool evFail = false;
  KParams P{};
  P.S = s->view;
  P.W = c->wave.view;
  P.W.shots = dShots;
  P.records = hostRecords ? 1 : 0;
  P.counters = c->counters;
  P.stackLimit = c->stackLimit > 0 && c->stackLimit < kStackDepth ? c->stackLimit : kStackDepth;
  for (const Batch& b : batches) {
    P.W.ranges = dRanges + b.rangeBegin;
    P.W.numRanges = b.rangeEnd - b.rangeBegin;
    P.W.numPaths = b.paths;
    P.depth = 0;
    P.cur = 0;
    int rg = int(std::min<uint64_t>((b.paths + 255) / 256, uint64_t(c->raygenGrid)));
    launchRaygen(P, std::max(rg, 1), c->stream);
    const int passes = wavefrontPasses(b.maxDepth, s->view);
    for (int depth = 1; depth <= passes; ++depth) {
      P.depth = uint32_t(depth);
      // inside a capture the events become event-record nodes of the graph,
      // so every replay records them again
      auto record = [&](cudaEvent_t ev) {
        return useGraph ? cudaEventRecordWithFlags(ev, c->stream, cudaEventRecordExternal)
                        : cudaEventRecord(ev, c->stream);
      };
      auto timedLaunch = [&](int kind, auto&& fn) {
        if (stats && record(c->events[evi]) != cudaSuccess) evFail = true;
        fn();
        if (stats) {
          if (record(c->events[evi + 1]) != cudaSuccess) evFail = true;
          timed.push_back({kind, evi});
          evi += 2;
        }
      };
      if (c->raySort && depth >= 2) {
        // sorted into the idle queue, which this pass then runs on
        timedLaunch(3, [&] { launchSortQueue(P, c->raySort, c->raygenGrid, c->stream); });
        P.cur ^= 1;
      }
      P.occupancy = c->occupancy;
      P.blockThreads = c->traceThreads;
      P.sharedStack = c->sharedStack;
      P.refillLanes = c->refill[0];
      P.speculate = c->speculate[0];
      timedLaunch(0, [&] { launchExtend(P, c->traceGrid, c->stream); });
      timedLaunch(1, [&] { launchShade(P, c->shadeGrid, c->stream); });
      P.refillLanes = c->refill[1];
      P.speculate = c->speculate[1];
      P.occupancy = c->occupancyShadow;
      timedLaunch(2, [&] { launchConnect(P, c->traceGridShadow, c->stream); });
      P.cur ^= 1;
    }
    launchAccumulate(P, b.maxPix, P.W.numRanges, c->stream);
    if (hostRecords) launchRecords(P, dRec + b.pathOffset, c->raygenGrid, c->stream);
  }
  if (useGraph) {
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamEndCapture(c->stream, &graph);
    if (e != cudaSuccess) return fail(ASUNA_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(e));
    if (evFail) {
      cudaGraphDestroy(graph);
      return fail(ASUNA_ERR_CUDA, "recording the timing events failed");
    }
    GraphEntry g;
    e = cudaGraphInstantiate(&g.exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return fail(ASUNA_ERR_CUDA, "graph instantiation failed: %s", cudaGetErrorString(e));
    g.key = key;
    g.timed = timed;
    g.lastUse = ++c->useClock;
    if (c->gcache.size() >= 8) {
      auto lru = std::min_element(c->gcache.begin(), c->gcache.end(),
                                  [](const GraphEntry& a, const GraphEntry& b) { return a.lastUse < b.lastUse; });
      cudaGraphExecDestroy(lru->exec);
      c->gcache.erase(lru);
    }
    c->gcache.push_back(g);
    ASUNA_CUDA_TRY(cudaGraphLaunch(g.exec, c->stream));
  }
    if (evFail) return fail(ASUNA_ERR_CUDA, "recording the timing events failed");
  }
  ASUNA_CUDA_TRY(cudaGetLastError());
  if (stats) ASUNA_CUDA_TRY(cudaEventRecord(c->events[1], c->stream));
  // every render queues the copy of the cut-short count (8 bytes, pinned)
  ASUNA_CUDA_TRY(cudaMemcpyAsync(c->hostErr, &c->cnt->stackOverflow, sizeof(unsigned long long),
                                 cudaMemcpyDeviceToHost, c->stream));
  ASUNA_CUDA_TRY(cudaEventRecord(c->errEvent, c->stream));
  c->errPending = true;
  if (hostRecords) {
    ASUNA_CUDA_TRY(cudaMemcpyAsync(hostRecords, dRec, totalPaths * sizeof(asuna_path_record), cudaMemcpyDeviceToHost,
                                   c->stream));
    ASUNA_CUDA_TRY(cudaFreeAsync(dRec, c->stream));
    ASUNA_CUDA_TRY(cudaStreamSynchronize(c->stream));
    if ((rc = reportTraversal(c))) return rc;
  }
  if (stats) {
    ASUNA_CUDA_TRY(cudaMemcpyAsync(c->hostCnt, c->cnt, sizeof(DevCounters), cudaMemcpyDeviceToHost, c->stream));
    ASUNA_CUDA_TRY(cudaStreamSynchronize(c->stream));
    std::memset(stats, 0, sizeof(*stats));
    stats->paths = c->hostCnt->paths;
    stats->extend_rays = c->hostCnt->extendRays;
    stats->shadow_rays = c->hostCnt->shadowRays;
    stats->nodes_visited = c->hostCnt->nodes;
    stats->tris_tested = c->hostCnt->tris;
    stats->shadow_nodes_visited = c->hostCnt->shNodes;
    stats->shadow_tris_tested = c->hostCnt->shTris;
    // raygen + accumulate (+ records) per wave; extend, shading, connect per depth
    for (const Batch& b : batches)
      stats->kernel_launches += 2 + (hostRecords ? 1 : 0) +
                                uint64_t(wavefrontPasses(b.maxDepth, s->view)) * (2 + shadeLaunches(s->view.classMask)) +
                                (c->raySort ? 3 * uint64_t(wavefrontPasses(b.maxDepth, s->view) - 1) : 0);
    float ms = 0;
    ASUNA_CUDA_TRY(cudaEventElapsedTime(&ms, c->events[0], c->events[1]));
    stats->ms_total = ms;
    for (auto& t : timed) {
      float m = 0;
      ASUNA_CUDA_TRY(cudaEventElapsedTime(&m, c->events[t.second], c->events[t.second + 1]));
      if (t.first == 0) {
        stats->ms_extend += m;
        stats->extend_launches++;
      } else if (t.first == 1) {
        stats->ms_shade += m;
      } else if (t.first == 3) {
        stats->ms_sort += m;
      } else {
        stats->ms_connect += m;
        stats->connect_launches++;
      }
    }
    if ((rc = reportTraversal(c))) return rc;
  }
  return ASUNA_OK;
}

int asuna_render(asuna_ctx* c, const asuna_scene* s, const asuna_shot* shot, asuna_film* film,
                 asuna_render_stats* stats) {
  return renderImpl(c, s, shot, &film, 1, stats, nullptr);
}

int asuna_render_batch(asuna_ctx* c, const asuna_scene* s, const asuna_shot* shots, asuna_film* const* films,
                       uint32_t n, asuna_render_stats* stats) {
  return renderImpl(c, s, shots, films, n, stats, nullptr);
}

int asuna_render_paths(asuna_ctx* c, const asuna_scene* s, const asuna_shot* shot, asuna_film* film,
                       asuna_path_record* host_records) {
  if (!host_records) return fail(ASUNA_ERR_INVALID, "null records");
  return renderImpl(c, s, shot, &film, 1, nullptr, host_records);
}

int asuna_scene_trace(asuna_ctx* c, const asuna_scene* s, const float* rays, uint32_t n, int any_hit, float* hits,
                      uint32_t* inst) {
  clearError();
  if (!c || !s || !rays || !hits || !inst) return fail(ASUNA_ERR_INVALID, "null argument");
  if (n == 0) return ASUNA_OK;
  ASUNA_CUDA_TRY(cudaSetDevice(c->device));
  float4 *dO = nullptr, *dD = nullptr, *dH = nullptr;
  uint32_t* dI = nullptr;
  std::vector<float4> ho(n), hd(n);
  for (uint32_t i = 0; i < n; ++i) {
    ho[i] = make_float4(rays[8 * i], rays[8 * i + 1], rays[8 * i + 2], rays[8 * i + 3]);
    hd[i] = make_float4(rays[8 * i + 4], rays[8 * i + 5], rays[8 * i + 6], rays[8 * i + 7]);
  }
  ASUNA_CUDA_TRY(cudaMallocAsync(&dO, n * 16, c->stream));
  ASUNA_CUDA_TRY(cudaMallocAsync(&dD, n * 16, c->stream));
  ASUNA_CUDA_TRY(cudaMallocAsync(&dH, n * 16, c->stream));
  ASUNA_CUDA_TRY(cudaMallocAsync(&dI, n * 4, c->stream));
  ASUNA_CUDA_TRY(cudaMemcpyAsync(dO, ho.data(), n * 16, cudaMemcpyHostToDevice, c->stream));
  ASUNA_CUDA_TRY(cudaMemcpyAsync(dD, hd.data(), n * 16, cudaMemcpyHostToDevice, c->stream));
  launchTraceQuery(s->view, dO, dD, n, any_hit, dH, dI, c->stream);
  ASUNA_CUDA_TRY(cudaGetLastError());
  ASUNA_CUDA_TRY(cudaMemcpyAsync(hits, dH, n * 16, cudaMemcpyDeviceToHost, c->stream));
  ASUNA_CUDA_TRY(cudaMemcpyAsync(inst, dI, n * 4, cudaMemcpyDeviceToHost, c->stream));
  cudaFreeAsync(dO, c->stream);
  cudaFreeAsync(dD, c->stream);
  cudaFreeAsync(dH, c->stream);
  cudaFreeAsync(dI, c->stream);
  ASUNA_CUDA_TRY(cudaStreamSynchronize(c->stream));
  return ASUNA_OK;
}

}  // extern "C"
