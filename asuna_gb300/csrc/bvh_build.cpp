// bvh_build.cpp — binned-SAH BVH builder (host).
//
// Top-down, 32 bins per axis, surface-area heuristic with unit traversal and
// intersection costs; leaves hold at most `maxLeaf` primitives.  Past depth
// 40 it falls back to object-median splits so the tree depth stays bounded
// by the traversal stack.  Child boxes are widened by a relative 2^-20 so the
// fused multiply-add slab test on the GPU never rejects a box that holds a
// hit of the watertight triangle test.
#include "bvh_build.h"

#include <algorithm>
#include <cfloat>
#include <cmath>

namespace asuna {
namespace {

constexpr int kBins = 32;
constexpr uint32_t kMedianDepth = 40;

struct Bin {
  Aabb box;
  uint32_t n;
};

inline void boxEmpty(Aabb& b) {
  for (int k = 0; k < 3; ++k) {
    b.lo[k] = FLT_MAX;
    b.hi[k] = -FLT_MAX;
  }
}
inline void boxGrow(Aabb& b, const Aabb& o) {
  for (int k = 0; k < 3; ++k) {
    b.lo[k] = std::min(b.lo[k], o.lo[k]);
    b.hi[k] = std::max(b.hi[k], o.hi[k]);
  }
}
inline float boxArea(const Aabb& b) {
  float dx = b.hi[0] - b.lo[0], dy = b.hi[1] - b.lo[1], dz = b.hi[2] - b.lo[2];
  if (dx < 0 || dy < 0 || dz < 0) return 0.0f;
  return 2.0f * (dx * dy + dy * dz + dz * dx);
}

struct Task {
  uint32_t node;  // index into out.nodes of the parent, or UINT32_MAX for root
  int side;       // which child slot of the parent
  uint32_t begin, end;
  uint32_t depth;
};

struct Builder {
  const std::vector<Aabb>& boxes;
  const std::vector<float>& cen;
  int maxLeaf;
  uint32_t firstBase;
  BvhBuildOut& out;

  Aabb rangeBox(uint32_t b, uint32_t e, Aabb* cbox) const {
    Aabb bb, cb;
    boxEmpty(bb);
    boxEmpty(cb);
    for (uint32_t i = b; i < e; ++i) {
      uint32_t p = out.order[i];
      boxGrow(bb, boxes[p]);
      for (int k = 0; k < 3; ++k) {
        cb.lo[k] = std::min(cb.lo[k], cen[3 * p + k]);
        cb.hi[k] = std::max(cb.hi[k], cen[3 * p + k]);
      }
    }
    if (cbox) *cbox = cb;
    return bb;
  }

  // Returns split position (begin < mid < end) or 0 for "make a leaf".
  uint32_t split(uint32_t b, uint32_t e, uint32_t depth, const Aabb& bb, const Aabb& cb) {
    const uint32_t n = e - b;
    int axis = 0;
    float ext = cb.hi[0] - cb.lo[0];
    for (int k = 1; k < 3; ++k)
      if (cb.hi[k] - cb.lo[k] > ext) {
        ext = cb.hi[k] - cb.lo[k];
        axis = k;
      }
    auto median = [&](int ax) {
      uint32_t mid = b + n / 2;
      std::nth_element(out.order.begin() + b, out.order.begin() + mid, out.order.begin() + e,
                       [&](uint32_t x, uint32_t y) {
                         float cx = cen[3 * x + ax], cy = cen[3 * y + ax];
                         return cx < cy || (cx == cy && x < y);
                       });
      return mid;
    };
    if (ext <= 0.0f) {
      // all centroids coincide: split by index if the leaf would be too big
      return n > uint32_t(maxLeaf) ? b + n / 2 : 0;
    }
    if (depth >= kMedianDepth) return median(axis);
    // binned SAH over the three axes
    float bestCost = FLT_MAX;
    int bestAxis = -1, bestBin = -1;
    const float parentArea = boxArea(bb);
    for (int ax = 0; ax < 3; ++ax) {
      float lo = cb.lo[ax], hi = cb.hi[ax];
      if (hi - lo <= 0.0f) continue;
      float scale = float(kBins) / (hi - lo);
      Bin bins[kBins];
      for (auto& bi : bins) {
        boxEmpty(bi.box);
        bi.n = 0;
      }
      for (uint32_t i = b; i < e; ++i) {
        uint32_t p = out.order[i];
        int k = int((cen[3 * p + ax] - lo) * scale);
        k = std::min(std::max(k, 0), kBins - 1);
        bins[k].n++;
        boxGrow(bins[k].box, boxes[p]);
      }
      float rightArea[kBins];
      uint32_t rightN[kBins];
      Aabb acc;
      boxEmpty(acc);
      uint32_t accN = 0;
      for (int k = kBins - 1; k > 0; --k) {
        boxGrow(acc, bins[k].box);
        accN += bins[k].n;
        rightArea[k] = boxArea(acc);
        rightN[k] = accN;
      }
      boxEmpty(acc);
      accN = 0;
      for (int k = 0; k < kBins - 1; ++k) {
        boxGrow(acc, bins[k].box);
        accN += bins[k].n;
        if (accN == 0 || rightN[k + 1] == 0) continue;
        float cost = 1.0f + (boxArea(acc) * float(accN) + rightArea[k + 1] * float(rightN[k + 1])) /
                                std::max(parentArea, 1e-30f);
        if (cost < bestCost) {
          bestCost = cost;
          bestAxis = ax;
          bestBin = k;
        }
      }
    }
    if (bestAxis < 0) return n > uint32_t(maxLeaf) ? median(axis) : 0;
    if (n <= uint32_t(maxLeaf) && bestCost >= float(n)) return 0;
    float lo = cb.lo[bestAxis], scale = float(kBins) / (cb.hi[bestAxis] - lo);
    auto mid = std::partition(out.order.begin() + b, out.order.begin() + e, [&](uint32_t p) {
      int k = int((cen[3 * p + bestAxis] - lo) * scale);
      k = std::min(std::max(k, 0), kBins - 1);
      return k <= bestBin;
    });
    uint32_t m = uint32_t(mid - out.order.begin());
    if (m == b || m == e) return median(axis);
    return m;
  }
};

inline void widen(Aabb& b) {
  for (int k = 0; k < 3; ++k) {
    float e = std::max(std::fabs(b.lo[k]), std::fabs(b.hi[k])) * 9.5367431640625e-07f + 1e-30f;
    b.lo[k] -= e;
    b.hi[k] += e;
  }
}

void setChild(BvhNode& n, int side, const Aabb& b, int32_t ref) {
  nodeSetBox(n, side, b.lo, b.hi);
  (side == 0 ? n.ref.x : n.ref.y) = ref;
}

}  // namespace

bool buildBvh(const std::vector<Aabb>& boxes, const std::vector<float>& centroids, int maxLeaf, uint32_t firstBase,
              BvhBuildOut& out) {
  const uint32_t n = uint32_t(boxes.size());
  out.nodes.clear();
  out.order.resize(n);
  out.maxDepth = 1;
  for (uint32_t i = 0; i < n; ++i) out.order[i] = i;
  if (maxLeaf > kMaxLeafTris) maxLeaf = kMaxLeafTris;
  if (uint64_t(firstBase) + n > kMaxLeafFirst) return false;
  Builder B{boxes, centroids, maxLeaf, firstBase, out};
  // Root is always an inner node; an unused child slot holds a degenerate box
  // far outside any scene (a point at 1e30), which no ray with tmax <= 1e10
  // can reach, whatever the signs of its direction.
  BvhNode root{};
  Aabb empty;
  for (int k = 0; k < 3; ++k) empty.lo[k] = empty.hi[k] = 1e30f;
  setChild(root, 0, empty, kStackSentinel);
  setChild(root, 1, empty, kStackSentinel);
  out.nodes.push_back(root);
  if (n == 0) return true;
  std::vector<Task> stack;
  Aabb cb;
  Aabb bb = B.rangeBox(0, n, &cb);
  uint32_t rootMid = (n > 1) ? B.split(0, n, 1, bb, cb) : 0;
  if (rootMid == 0) {
    Aabb w = bb;
    widen(w);
    setChild(out.nodes[0], 0, w, encodeLeaf(firstBase, n));
    out.maxDepth = 2;
    if (n > uint32_t(maxLeaf)) return false;
    return true;
  }
  stack.push_back({0, 1, rootMid, n, 2});
  stack.push_back({0, 0, 0, rootMid, 2});
  while (!stack.empty()) {
    Task t = stack.back();
    stack.pop_back();
    Aabb cbox;
    Aabb box = B.rangeBox(t.begin, t.end, &cbox);
    Aabb w = box;
    widen(w);
    out.maxDepth = std::max(out.maxDepth, t.depth);
    uint32_t m = (t.end - t.begin > 1) ? B.split(t.begin, t.end, t.depth, box, cbox) : 0;
    if (m == 0) {
      setChild(out.nodes[t.node], t.side, w, encodeLeaf(firstBase + t.begin, t.end - t.begin));
      continue;
    }
    uint32_t idx = uint32_t(out.nodes.size());
    BvhNode nn{};
    out.nodes.push_back(nn);
    setChild(out.nodes[t.node], t.side, w, int32_t(idx));
    stack.push_back({idx, 1, m, t.end, t.depth + 1});
    stack.push_back({idx, 0, t.begin, m, t.depth + 1});
  }
  return true;
}

}  // namespace asuna
