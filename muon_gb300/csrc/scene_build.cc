// Scene flattening and BVH construction on the host.
//
// The reference keeps primitives in object space and transforms every ray into
// object space per primitive test (muon/objects.cc:29-46). Here triangles are
// pre-transformed to world space once (the idea noted at muon/objects.h:65-66)
// and the reference's parallel-ray rejection |d.n| < 1e-4, which the reference
// applies to the object-space unnormalised normal and re-normalised direction
// (muon/objects.cc:104-108), is carried over as a per-triangle world-space
// threshold eps = 1e-4 * |n_world| / |n_object|. A triangle whose object-space
// |n| is below 1e-4 can never pass that test in the reference, so it is left
// out of the BVH (its primitive id stays reserved). Spheres keep their
// transforms and are intersected in object space like the reference.
//
// The BVH replaces the reference's 12-bucket widest-axis SAH build
// (muon/acceleration.cc:241-458): binned SAH over all three axes with a
// bounded leaf size. Closest hits do not depend on the tree shape.
#include "scene_build.h"
#include "tri_records.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <limits>
#include <thread>

namespace muon_gpu {

namespace {

constexpr int kBins = 32;

// Runs f(begin, end) over [0, n) in contiguous chunks on the host's threads
// (on the calling thread alone below `grain` items per chunk). Every use
// writes disjoint outputs or merges exact min / max / integer partials, so the
// result does not depend on the number of threads.
template <class F>
void ParallelFor(int64_t n, int64_t grain, F f) {
  const int64_t hw = std::max(1u, std::thread::hardware_concurrency());
  const int64_t parts = std::max<int64_t>(1, std::min(hw, n / std::max<int64_t>(grain, 1)));
  if (parts <= 1) {
    f(int64_t(0), n);
    return;
  }
  std::vector<std::thread> pool;
  for (int64_t k = 1; k < parts; ++k) pool.emplace_back(f, n * k / parts, n * (k + 1) / parts);
  f(int64_t(0), n / parts);
  for (std::thread &t : pool) t.join();
}
constexpr float kTraversalCost = 1.0f;
constexpr float kIntersectCost = 1.0f;

// A primitive reference: its box inline (sequential access while binning)
// and its index in the input.
struct Ref {
  Aabb box;
  int32_t idx;
  float C(int k) const { return 0.5f * (box.lo[k] + box.hi[k]); }
};

struct BuildNode {
  Aabb box;
  int32_t left = -1, right = -1;  // children in the build array
  int32_t start = 0, count = 0;   // leaf range in the ref array
};

Aabb EmptyBox() {
  Aabb b;
  for (int k = 0; k < 3; ++k) {
    b.lo[k] = std::numeric_limits<float>::infinity();
    b.hi[k] = -std::numeric_limits<float>::infinity();
  }
  return b;
}
void Grow(Aabb &b, const Aabb &o) {
  for (int k = 0; k < 3; ++k) {
    b.lo[k] = std::min(b.lo[k], o.lo[k]);
    b.hi[k] = std::max(b.hi[k], o.hi[k]);
  }
}
float Area(const Aabb &b) {
  float dx = b.hi[0] - b.lo[0], dy = b.hi[1] - b.lo[1], dz = b.hi[2] - b.lo[2];
  if (!(dx >= 0.0f) || !(dy >= 0.0f) || !(dz >= 0.0f)) return 0.0f;
  return 2.0f * (dx * dy + dx * dz + dy * dz);
}

// Nodes of one subtree, in depth-first order with the subtree root first.
struct Subtree {
  std::vector<BuildNode> nodes;
  int max_depth = 0;
  int64_t leaves = 0;
  int max_leaf = 0;
};

// Top-down binned builder. A subtree of at least kParallelRefs references
// below a split is built on its own thread while the caller builds its
// sibling; spliced back in the serial order, so the tree does not depend on
// the number of threads.
class Builder {
 public:
  static constexpr int32_t kParallelRefs = 1 << 15;
  // Nodes with at least this many references split their bounding and
  // binning passes across the host's threads.
  static constexpr int32_t kParallelPass = 1 << 15;

  Builder(const std::vector<Aabb> &boxes, int strategy, int max_leaf)
      : strategy_(strategy), max_leaf_(std::max(1, max_leaf)) {
    refs_.resize(boxes.size());
    for (size_t i = 0; i < boxes.size(); ++i) refs_[i] = Ref{boxes[i], static_cast<int32_t>(i)};
    unsigned hw = std::thread::hardware_concurrency();
    threads_left_ = static_cast<int>(hw > 1 ? hw - 1 : 0);
  }

  // A subtree left for the thread pool: refs_[start, end) at `depth`, whose
  // root goes to out.nodes[node].
  struct Task {
    int32_t node, start, end, depth;
  };

  // Builds refs_[start, end) into `out`; returns the subtree root's index.
  // With `tasks`, ranges below task_refs_ become placeholder nodes and tasks
  // (built afterwards by BuildTasks) instead of being built here.
  int32_t Build(Subtree &out, int32_t start, int32_t end, int depth, std::vector<Task> *tasks = nullptr) {
    if (tasks && end - start < task_refs_ && end - start > max_leaf_) {
      const int32_t id = static_cast<int32_t>(out.nodes.size());
      out.nodes.push_back(BuildNode{});
      tasks->push_back(Task{id, start, end, depth});
      return id;
    }
    BuildNode node;
    node.box = EmptyBox();
    Aabb cbox = EmptyBox();
    auto bounds = [&](int32_t a, int32_t b, Aabb &box, Aabb &cb) {
      for (int32_t i = a; i < b; ++i) {
        Grow(box, refs_[i].box);
        for (int k = 0; k < 3; ++k) {
          float c = refs_[i].C(k);
          cb.lo[k] = std::min(cb.lo[k], c);
          cb.hi[k] = std::max(cb.hi[k], c);
        }
      }
    };
    if (end - start >= kParallelPass) {
      // the top of the tree, before subtrees run on threads of their own
      const int parts = static_cast<int>(std::max(1u, std::thread::hardware_concurrency()));
      std::vector<Aabb> pb(parts, EmptyBox()), pc(parts, EmptyBox());
      std::vector<std::thread> pool;
      for (int k = 0; k < parts; ++k) {
        const int32_t a = start + static_cast<int32_t>(int64_t(end - start) * k / parts);
        const int32_t b = start + static_cast<int32_t>(int64_t(end - start) * (k + 1) / parts);
        pool.emplace_back([&, a, b, k] { bounds(a, b, pb[k], pc[k]); });
      }
      for (std::thread &t : pool) t.join();
      for (int k = 0; k < parts; ++k) Grow(node.box, pb[k]), Grow(cbox, pc[k]);
    } else {
      bounds(start, end, node.box, cbox);
    }
    out.max_depth = std::max(out.max_depth, depth);
    int32_t n = end - start;
    int32_t id = static_cast<int32_t>(out.nodes.size());
    out.nodes.push_back(node);
    if (n <= 1) return MakeLeaf(out, id, start, n);

    int32_t mid = -1;
    if (strategy_ == MUON_PARTITION_SAH) {
      mid = SplitSah(start, end, node.box, cbox);
    } else if (strategy_ == MUON_PARTITION_MIDPOINT) {
      int axis = WidestAxis(cbox);
      float m = 0.5f * (cbox.lo[axis] + cbox.hi[axis]);
      Ref *p = std::partition(&refs_[start], &refs_[0] + end, [&](const Ref &r) { return r.C(axis) < m; });
      mid = static_cast<int32_t>(p - &refs_[0]);
      if (mid == start || mid == end) mid = -2;
      if (n <= max_leaf_ && mid == -2) return MakeLeaf(out, id, start, n);
    } else {
      mid = -2;
    }
    if (mid == -1) return MakeLeaf(out, id, start, n);  // SAH chose a leaf
    if (mid == -2) {
      // Median split on the widest centroid axis (also the fallback when
      // every centroid coincides).
      int axis = WidestAxis(cbox);
      mid = start + n / 2;
      std::nth_element(&refs_[start], &refs_[mid], &refs_[0] + end,
                       [&](const Ref &a, const Ref &b) { return a.C(axis) < b.C(axis); });
    }
    int32_t l, r;
    if (!tasks && end - mid >= kParallelRefs && TakeThread()) {
      Subtree right;
      std::thread t([&] { Build(right, mid, end, depth + 1); });
      l = Build(out, start, mid, depth + 1);
      t.join();
      threads_left_.fetch_add(1);
      r = Splice(out, right);
    } else {
      l = Build(out, start, mid, depth + 1, tasks);
      r = Build(out, mid, end, depth + 1, tasks);
    }
    out.nodes[id].left = l;
    out.nodes[id].right = r;
    return id;
  }

  // Builds the tasks on all host threads (largest first), each into its own
  // subtree, then splices them into `out` in task order and moves each
  // subtree's root into its placeholder. The tree is the same whatever the
  // number of threads.
  void BuildTasks(Subtree &out, std::vector<Task> &tasks) {
    std::vector<Subtree> subs(tasks.size());
    std::vector<size_t> by_size(tasks.size());
    for (size_t i = 0; i < tasks.size(); ++i) by_size[i] = i;
    std::sort(by_size.begin(), by_size.end(), [&](size_t a, size_t b) {
      return tasks[a].end - tasks[a].start > tasks[b].end - tasks[b].start;
    });
    const int saved = threads_left_.exchange(0);  // no nested spawning
    std::atomic<size_t> next{0};
    auto worker = [&] {
      for (size_t k; (k = next.fetch_add(1)) < by_size.size();) {
        const Task &t = tasks[by_size[k]];
        Build(subs[by_size[k]], t.start, t.end, t.depth);
      }
    };
    const int hw = static_cast<int>(std::max(1u, std::thread::hardware_concurrency()));
    std::vector<std::thread> pool;
    for (int i = 1; i < hw && i < static_cast<int>(tasks.size()); ++i) pool.emplace_back(worker);
    worker();
    for (std::thread &th : pool) th.join();
    threads_left_ = saved;
    for (size_t i = 0; i < tasks.size(); ++i) {
      const int32_t off = Splice(out, subs[i]);
      out.nodes[tasks[i].node] = out.nodes[off];  // the copy at `off` is no longer referenced
    }
  }

  int32_t task_refs_ = 0;
  std::vector<Ref> refs_;

 private:
  static int WidestAxis(const Aabb &b) {
    float d[3] = {b.hi[0] - b.lo[0], b.hi[1] - b.lo[1], b.hi[2] - b.lo[2]};
    return d[0] > d[1] && d[0] > d[2] ? 0 : (d[1] > d[2] ? 1 : 2);
  }

  bool TakeThread() {
    int v = threads_left_.load();
    while (v > 0) {
      if (threads_left_.compare_exchange_weak(v, v - 1)) return true;
    }
    return false;
  }

  // Appends `sub` to `out`, shifting its child indices; returns its root.
  static int32_t Splice(Subtree &out, const Subtree &sub) {
    int32_t off = static_cast<int32_t>(out.nodes.size());
    for (BuildNode x : sub.nodes) {
      if (x.left >= 0) x.left += off, x.right += off;
      out.nodes.push_back(x);
    }
    out.max_depth = std::max(out.max_depth, sub.max_depth);
    out.leaves += sub.leaves;
    out.max_leaf = std::max(out.max_leaf, sub.max_leaf);
    return off;
  }

  static int32_t MakeLeaf(Subtree &out, int32_t id, int32_t start, int32_t n) {
    out.nodes[id].start = start;
    out.nodes[id].count = n;
    ++out.leaves;
    out.max_leaf = std::max(out.max_leaf, n);
    return id;
  }

  // Returns the split position, -1 for "make a leaf", -2 for "median split".
  int32_t SplitSah(int32_t start, int32_t end, const Aabb &box, const Aabb &cbox) {
    int32_t n = end - start;
    float best_cost = std::numeric_limits<float>::infinity();
    int best_axis = -1, best_bin = -1;
    float parent_area = Area(box);
    Aabb bin_box[3][kBins];
    int32_t bin_n[3][kBins] = {};
    float scale[3];
    for (int axis = 0; axis < 3; ++axis) {
      float extent = cbox.hi[axis] - cbox.lo[axis];
      scale[axis] = extent > 0.0f ? kBins / extent : 0.0f;
      for (int b = 0; b < kBins; ++b) bin_box[axis][b] = EmptyBox();
    }
    struct Bins {
      Aabb box[3][kBins];
      int32_t n[3][kBins];
    };
    auto bin = [&](int32_t a, int32_t b, Bins &out) {
      for (int32_t i = a; i < b; ++i) {
        const Aabb &bx = refs_[i].box;
        for (int axis = 0; axis < 3; ++axis) {
          int k = std::min(kBins - 1, static_cast<int>((refs_[i].C(axis) - cbox.lo[axis]) * scale[axis]));
          k = std::max(0, k);
          ++out.n[axis][k];
          Grow(out.box[axis][k], bx);
        }
      }
    };
    const int parts = n >= kParallelPass ? static_cast<int>(std::max(1u, std::thread::hardware_concurrency())) : 1;
    std::vector<Bins> part(parts);
    for (Bins &pb : part)
      for (int axis = 0; axis < 3; ++axis)
        for (int b = 0; b < kBins; ++b) pb.box[axis][b] = EmptyBox(), pb.n[axis][b] = 0;
    if (parts == 1) {
      bin(start, end, part[0]);
    } else {
      std::vector<std::thread> pool;
      for (int k = 0; k < parts; ++k) {
        const int32_t a = start + static_cast<int32_t>(int64_t(n) * k / parts);
        const int32_t b = start + static_cast<int32_t>(int64_t(n) * (k + 1) / parts);
        pool.emplace_back([&, a, b, k] { bin(a, b, part[k]); });
      }
      for (std::thread &t : pool) t.join();
    }
    for (const Bins &pb : part)
      for (int axis = 0; axis < 3; ++axis)
        for (int b = 0; b < kBins; ++b) bin_n[axis][b] += pb.n[axis][b], Grow(bin_box[axis][b], pb.box[axis][b]);
    for (int axis = 0; axis < 3; ++axis) {
      if (!(cbox.hi[axis] - cbox.lo[axis] > 0.0f)) continue;
      float right_area[kBins];
      int32_t right_n[kBins];
      Aabb acc = EmptyBox();
      int32_t cnt = 0;
      for (int b = kBins - 1; b > 0; --b) {
        Grow(acc, bin_box[axis][b]);
        cnt += bin_n[axis][b];
        right_area[b] = Area(acc);
        right_n[b] = cnt;
      }
      acc = EmptyBox();
      cnt = 0;
      for (int b = 0; b < kBins - 1; ++b) {
        Grow(acc, bin_box[axis][b]);
        cnt += bin_n[axis][b];
        if (cnt == 0 || right_n[b + 1] == 0) continue;
        float cost = Area(acc) * cnt + right_area[b + 1] * right_n[b + 1];
        if (cost < best_cost) {
          best_cost = cost;
          best_axis = axis;
          best_bin = b;
        }
      }
    }
    if (best_axis < 0) return n <= max_leaf_ ? -1 : -2;
    float split_cost = kTraversalCost + kIntersectCost * best_cost / std::max(parent_area, 1e-30f);
    float leaf_cost = kIntersectCost * n;
    if (n <= max_leaf_ && leaf_cost <= split_cost) return -1;
    float sc = scale[best_axis];
    float lo = cbox.lo[best_axis];
    Ref *p = std::partition(&refs_[start], &refs_[0] + end, [&](const Ref &r) {
      int b = std::min(kBins - 1, static_cast<int>((r.C(best_axis) - lo) * sc));
      return std::max(0, b) <= best_bin;
    });
    int32_t mid = static_cast<int32_t>(p - &refs_[0]);
    if (mid == start || mid == end) return -2;
    return mid;
  }

  int strategy_;
  int max_leaf_;
  std::atomic<int> threads_left_{0};
};

// Pads a box outwards by a few ulps so that rounding in the slab test cannot
// cull a primitive whose own test reports a hit on the box surface.
Aabb Pad(const Aabb &b) {
  Aabb o = b;
  for (int k = 0; k < 3; ++k) {
    if (!(b.lo[k] <= b.hi[k])) continue;
    float m = std::max(std::fabs(b.lo[k]), std::fabs(b.hi[k])) + (b.hi[k] - b.lo[k]);
    float e = m * 4e-7f + 1e-30f;
    o.lo[k] = b.lo[k] - e;
    o.hi[k] = b.hi[k] + e;
  }
  return o;
}

void SetChild(BvhNode &n, int slot, const Aabb &b0, int32_t link) {
  Aabb b = Pad(b0);
  if (slot == 0) {
    n.a.x = b.lo[0], n.a.y = b.hi[0], n.a.z = b.lo[1], n.a.w = b.hi[1];
    n.c.x = b.lo[2], n.c.y = b.hi[2];
    n.d.x = link;
  } else {
    n.b.x = b.lo[0], n.b.y = b.hi[0], n.b.z = b.lo[1], n.b.w = b.hi[1];
    n.c.z = b.lo[2], n.c.w = b.hi[2];
    n.d.y = link;
  }
}

}  // namespace

void BuildBvh(const std::vector<Aabb> &boxes, int accel, int strategy, int max_leaf,
              std::vector<BvhNode> *nodes, std::vector<int32_t> *order, std::vector<uint8_t> *last,
              BvhBuildStats *stats) {
  nodes->clear();
  order->clear();
  last->clear();
  *stats = BvhBuildStats();
  if (boxes.empty()) return;
  Builder b(boxes, strategy, accel == MUON_ACCEL_LINEAR ? static_cast<int>(boxes.size()) : max_leaf);
  Subtree tree;
  int32_t root;
  if (accel == MUON_ACCEL_LINEAR) {
    BuildNode leaf;
    leaf.box = EmptyBox();
    for (const Aabb &x : boxes) Grow(leaf.box, x);
    leaf.start = 0;
    leaf.count = static_cast<int32_t>(boxes.size());
    tree.nodes.push_back(leaf);
    tree.leaves = 1;
    tree.max_leaf = leaf.count;
    root = 0;
  } else {
    // The top of the tree on this thread (large nodes bin on all threads),
    // subtrees of about n / (2 threads) references on a thread pool.
    const int64_t hw = std::max(1u, std::thread::hardware_concurrency());
    b.task_refs_ = static_cast<int32_t>(std::max<int64_t>(4096, static_cast<int64_t>(boxes.size()) / (2 * hw)));
    std::vector<Builder::Task> tasks;
    root = b.Build(tree, 0, static_cast<int32_t>(boxes.size()), 0, &tasks);
    b.BuildTasks(tree, tasks);
  }
  order->resize(boxes.size());
  last->assign(boxes.size(), 0);
  for (size_t i = 0; i < boxes.size(); ++i) (*order)[i] = b.refs_[i].idx;
  const std::vector<BuildNode> &bn = tree.nodes;
  for (const BuildNode &x : bn) {
    if (x.left < 0 && x.count > 0) (*last)[x.start + x.count - 1] = 1;
  }

  // Depth-first flattening: each interior build node becomes one 64-byte
  // node holding its two children's boxes.
  nodes->reserve(bn.size() / 2 + 1);
  double sah = 0.0;
  float root_area = std::max(Area(bn[root].box), 1e-30f);
  if (bn[root].left < 0) {
    // The root is a leaf: both child slots refer to it. (An inverted box in
    // the second slot would pass the slab test, and an empty link ends the
    // traversal.) Testing the leaf twice cannot change a closest hit.
    BvhNode n{};
    SetChild(n, 0, bn[root].box, ~bn[root].start);
    SetChild(n, 1, bn[root].box, ~bn[root].start);
    nodes->push_back(n);
  } else {
    // Explicit stack of (build node, output slot).
    struct Item {
      int32_t build;
      int32_t out;
    };
    std::vector<Item> stack;
    nodes->push_back(BvhNode{});
    stack.push_back({root, 0});
    while (!stack.empty()) {
      Item it = stack.back();
      stack.pop_back();
      const BuildNode &x = bn[it.build];
      sah += kTraversalCost * Area(x.box) / root_area;
      int32_t kids[2] = {x.left, x.right};
      for (int s = 0; s < 2; ++s) {
        const BuildNode &k = bn[kids[s]];
        int32_t link;
        if (k.left < 0) {
          link = ~k.start;
          sah += kIntersectCost * k.count * Area(k.box) / root_area;
        } else {
          link = static_cast<int32_t>(nodes->size());
          nodes->push_back(BvhNode{});
          stack.push_back({kids[s], link});
        }
        SetChild((*nodes)[it.out], s, k.box, link);
      }
    }
  }
  stats->nodes = static_cast<int64_t>(nodes->size());
  stats->leaves = tree.leaves;
  stats->max_depth = tree.max_depth;
  stats->max_leaf = tree.max_leaf;
  stats->sah_cost = sah;
}

namespace {

mm::m4 ToM4(const float *m) {
  mm::m4 r;
  std::memcpy(&r, m, sizeof(float) * 16);
  return r;
}
void PackRows(const mm::m4 &m, float *out) {
  for (int c = 0; c < 4; ++c) {
    out[3 * c + 0] = m.c[c].x;
    out[3 * c + 1] = m.c[c].y;
    out[3 * c + 2] = m.c[c].z;
  }
}
F4 MakeF4(float x, float y, float z, float w) { return F4{x, y, z, w}; }
float IntBits(int32_t v) {
  float f;
  std::memcpy(&f, &v, 4);
  return f;
}
mm::v3 V3(const float *p) { return mm::make3(p[0], p[1], p[2]); }

// Lobe-selection probability of the reference BRDFs (Phong::reflectiveness,
// muon/materials.cc:113-123; GGX::reflectiveness, muon/materials.cc:270-293).
float Reflectiveness(const MuonMaterialDesc &m) {
  float specular = (m.specular[0] + m.specular[1] + m.specular[2]) / 3.0f;
  float diffuse = (m.diffuse[0] + m.diffuse[1] + m.diffuse[2]) / 3.0f;
  float denom = diffuse + specular;
  if (m.brdf == MUON_BRDF_GGX) {
    if (denom == 0.0f) return 1.0f;
    return mm::fmax_ref(specular / denom, 0.25f);
  }
  return denom > 0.0f ? specular / denom : 0.0f;
}

}  // namespace

bool BuildSceneImage(const MuonSceneDesc &desc, SceneImage *img, std::string *error, bool defer_bvh,
                     bool device_records) {
  defer_bvh = defer_bvh || device_records;
  if (desc.num_triangles < 0 || desc.num_spheres < 0 || desc.num_materials < 0 ||
      desc.num_lights < 0 || desc.num_transforms < 0) {
    *error = "negative array size in scene description";
    return false;
  }
  if ((desc.num_triangles > 0 && !desc.triangles) || (desc.num_spheres > 0 && !desc.spheres) ||
      (desc.num_materials > 0 && !desc.materials) || (desc.num_lights > 0 && !desc.lights) ||
      (desc.num_transforms > 0 && !desc.transforms)) {
    *error = "null array in scene description";
    return false;
  }
  if (desc.width <= 0 || desc.height <= 0 || desc.camera.width <= 0 || desc.camera.height <= 0) {
    *error = "film and camera sizes must be positive";
    return false;
  }
  const int64_t ntri = desc.num_triangles, nsph = desc.num_spheres;
  img->num_prims = ntri + nsph;
  img->camera = desc.camera;
  img->width = desc.width;
  img->height = desc.height;

  // Transforms.
  img->transforms.resize(desc.num_transforms);
  for (int32_t i = 0; i < desc.num_transforms; ++i) {
    DevTransform &t = img->transforms[i];
    std::memset(&t, 0, sizeof(t));
    PackRows(ToM4(desc.transforms[i].object_to_world), t.o2w);
    PackRows(ToM4(desc.transforms[i].world_to_object), t.w2o);
    PackRows(ToM4(desc.transforms[i].normal_to_world), t.n2w);
  }
  // Materials.
  img->materials.resize(desc.num_materials);
  for (int32_t i = 0; i < desc.num_materials; ++i) {
    const MuonMaterialDesc &m = desc.materials[i];
    if (m.brdf < MUON_BRDF_LAMBERTIAN || m.brdf > MUON_BRDF_GGX) {
      *error = "material has an unknown brdf";
      return false;
    }
    DevMaterial &d = img->materials[i];
    // Phong with a zero specular colour is the Lambertian BRDF: its lobe
    // probability is 0 and its specular term and density vanish
    // (muon/materials.cc:85-123), so the kernels take the shorter path.
    int32_t brdf = m.brdf;
    if (brdf == MUON_BRDF_PHONG && m.specular[0] == 0.0f && m.specular[1] == 0.0f && m.specular[2] == 0.0f)
      brdf = MUON_BRDF_LAMBERTIAN;
    d.diffuse = MakeF4(m.diffuse[0], m.diffuse[1], m.diffuse[2], m.shininess);
    d.specular = MakeF4(m.specular[0], m.specular[1], m.specular[2], m.roughness);
    d.emission = MakeF4(m.emission[0], m.emission[1], m.emission[2], IntBits(brdf));
    d.ambient = MakeF4(m.ambient[0], m.ambient[1], m.ambient[2], Reflectiveness(m));
  }
  // Lights: quad lights feed NEE/MIS; the others only the ray tracer.
  std::vector<int32_t> quad_index(desc.num_lights, -1);
  for (int32_t i = 0; i < desc.num_lights; ++i) {
    const MuonLightDesc &l = desc.lights[i];
    DevLight d{};
    d.corner = MakeF4(l.p0[0], l.p0[1], l.p0[2], IntBits(l.type));
    mm::v3 e0 = V3(l.p1), e1 = V3(l.p2);
    d.edge0 = MakeF4(e0.x, e0.y, e0.z, mm::length(e0));
    d.edge1 = MakeF4(e1.x, e1.y, e1.z, mm::length(e1));
    mm::v3 c01 = mm::cross(e0, e1);
    d.color = MakeF4(l.color[0], l.color[1], l.color[2], mm::length(c01));
    mm::v3 rn = mm::normalize(c01);
    d.rev_normal = MakeF4(rn.x, rn.y, rn.z, 0.0f);
    mm::v3 qn = mm::normalize(mm::cross(e1, e0));
    d.quad_normal = MakeF4(qn.x, qn.y, qn.z, 0.0f);
    if (l.type == MUON_LIGHT_QUAD) {
      quad_index[i] = static_cast<int32_t>(img->lights.size());
      img->lights.push_back(d);
      img->all_lights.push_back(d);
    } else if (l.type == MUON_LIGHT_POINT || l.type == MUON_LIGHT_DIRECTIONAL) {
      d.edge0 = MakeF4(l.p1[0], l.p1[1], l.p1[2], 0.0f);  // attenuation for point lights
      img->other_lights.push_back(d);
      img->all_lights.push_back(d);
    } else {
      *error = "light has an unknown type";
      return false;
    }
  }

  auto check_index = [&](int32_t v, int32_t n, const char *what) {
    if (v < -1 || v >= n) {
      *error = std::string("primitive refers to a missing ") + what;
      return false;
    }
    return true;
  };

  // World-space primitive data and bounds.
  std::vector<Aabb> boxes;
  std::vector<int64_t> source;  // box -> primitive (tri i, or ntri + sphere j)
  boxes.reserve(ntri + nsph);
  source.reserve(ntri + nsph);
  // triangles whose records this builds (none when the device builds them)
  const int64_t ntri_host = device_records ? 0 : ntri;
  std::vector<PrimRecord> tri_rec(ntri_host), tri_obj(ntri_host);
  std::vector<ShadeRecord> tri_shade(ntri_host);
  std::vector<F4> tri_normals, tri_normals_obj;
  // One pass over the triangles on all host threads: whether any is smooth,
  // and the first one with an index out of range (reported as the serial
  // check would report it).
  auto triangle_ok = [&](const MuonTriangleDesc &t) {
    return t.transform >= -1 && t.transform < desc.num_transforms && t.material >= 0 &&
           t.material < desc.num_materials && t.light >= -1 && t.light < desc.num_lights && t.prim_id >= 0 &&
           t.prim_id < img->num_prims;
  };
  std::atomic<int64_t> first_bad{ntri};
  std::atomic<bool> any_smooth{false};
  ParallelFor(ntri, 1 << 16, [&](int64_t i0, int64_t i1) {
    bool smooth = false;
    for (int64_t i = i0; i < i1; ++i) {
      const MuonTriangleDesc &t = desc.triangles[i];
      smooth |= t.smooth != 0;
      if (!triangle_ok(t)) {
        int64_t cur = first_bad.load();
        while (i < cur && !first_bad.compare_exchange_weak(cur, i)) {
        }
        break;
      }
    }
    if (smooth) any_smooth = true;
  });
  if (first_bad.load() < ntri) {
    const MuonTriangleDesc &t = desc.triangles[first_bad.load()];
    if (!check_index(t.transform, desc.num_transforms, "transform") ||
        !check_index(t.material, desc.num_materials, "material") || t.material < 0 ||
        !check_index(t.light, desc.num_lights, "light")) {
      if (t.material < 0) *error = "primitive refers to a missing material";
      return false;
    }
    *error = "primitive id out of range";
    return false;
  }
  img->any_smooth = any_smooth.load();
  if (img->any_smooth) tri_normals.resize(3 * ntri_host), tri_normals_obj.resize(3 * ntri_host);
  img->leaf_of_prim_id.assign(img->num_prims, -1);
  // Per-triangle records, on all host threads (each triangle writes its own
  // slots), then the boxes of the triangles that can be hit in input order.
  std::vector<Aabb> tri_box(ntri_host);
  std::vector<uint8_t> tri_keep(ntri_host, 0);
  ParallelFor(ntri_host, 1 << 14, [&](int64_t i0, int64_t i1) {
    for (int64_t i = i0; i < i1; ++i) {
      TriangleOut o;
      const bool keep = TriangleRecords(desc.triangles[i], desc.transforms, img->materials.data(), quad_index.data(), &o);
      tri_rec[i] = o.world;
      tri_obj[i] = o.object;
      tri_shade[i] = o.shade;
      if (desc.triangles[i].smooth) {
        for (int k = 0; k < 3; ++k) tri_normals[3 * i + k] = o.normals[k], tri_normals_obj[3 * i + k] = o.normals_obj[k];
      }
      if (!keep) continue;
      for (int k = 0; k < 3; ++k) tri_box[i].lo[k] = o.lo[k], tri_box[i].hi[k] = o.hi[k];
      tri_keep[i] = 1;
    }
  });
  img->quad_index = quad_index;
  for (int64_t i = 0; i < ntri_host; ++i) {
    if (!tri_keep[i]) continue;
    boxes.push_back(tri_box[i]);
    source.push_back(i);
  }
  std::vector<PrimRecord> sph_rec(nsph);
  std::vector<ShadeRecord> sph_shade(nsph);
  for (int64_t j = 0; j < nsph; ++j) {
    const MuonSphereDesc &s = desc.spheres[j];
    if (!check_index(s.transform, desc.num_transforms, "transform") ||
        !check_index(s.material, desc.num_materials, "material") || s.material < 0) {
      return false;
    }
    if (s.prim_id < 0 || s.prim_id >= img->num_prims) {
      *error = "primitive id out of range";
      return false;
    }
    PrimRecord &r = sph_rec[j];
    uint32_t flags = kPrimSphere;
    r.p0 = MakeF4(s.center[0], s.center[1], s.center[2], s.radius);
    r.p1 = MakeF4(0.0f, IntBits(s.transform), 0.0f, 0.0f);
    r.p2 = MakeF4(0, 0, 0, 0);
    r.p3 = MakeF4(0, 0, 0, 0);
    ShadeRecord &sh = sph_shade[j];
    sh.s0 = MakeF4(0, 0, 0, IntBits(s.material));
    int32_t sph_brdf;
    std::memcpy(&sph_brdf, &img->materials[s.material].emission.w, 4);
    const uint32_t sph_flags = flags | (static_cast<uint32_t>(3 + sph_brdf) << kClassShift);
    sh.s1 = I4{-1, s.prim_id, s.transform, static_cast<int32_t>(sph_flags)};
    std::memcpy(&r.p3.w, &sph_flags, 4);
    // World bounds: the object box's 8 corners transformed (Bounds::Transform,
    // muon/bounds.cc:52-69).
    mm::v3 c = V3(s.center);
    mm::v3 lo = c - mm::splat3(s.radius), hi = c + mm::splat3(s.radius);
    Aabb b;
    if (s.transform < 0) {
      for (int k = 0; k < 3; ++k) b.lo[k] = mm::comp(lo, k), b.hi[k] = mm::comp(hi, k);
    } else {
      mm::m4 m = ToM4(desc.transforms[s.transform].object_to_world);
      b = EmptyBox();
      for (int corner = 0; corner < 8; ++corner) {
        mm::v3 p = mm::make3(corner & 1 ? hi.x : lo.x, corner & 2 ? hi.y : lo.y, corner & 4 ? hi.z : lo.z);
        mm::v3 w = mm::xform_point(m, p);
        Aabb pb;
        for (int k = 0; k < 3; ++k) pb.lo[k] = pb.hi[k] = mm::comp(w, k);
        Grow(b, pb);
      }
    }
    boxes.push_back(b);
    source.push_back(ntri + j);
  }

  std::vector<int32_t> order;
  std::vector<uint8_t> last;
  int max_leaf = desc.max_leaf_size > 0 ? desc.max_leaf_size : 4;
  if (defer_bvh) {
    order.resize(boxes.size());
    for (size_t i = 0; i < order.size(); ++i) order[i] = static_cast<int32_t>(i);
    last.assign(boxes.size(), 1);
    img->nodes.clear();
    img->boxes.resize(6 * boxes.size());
    for (size_t i = 0; i < boxes.size(); ++i)
      for (int k = 0; k < 3; ++k) img->boxes[6 * i + k] = boxes[i].lo[k], img->boxes[6 * i + 3 + k] = boxes[i].hi[k];
  } else {
    BuildBvh(boxes, desc.acceleration, desc.partition_strategy, max_leaf, &img->nodes, &order, &last, &img->bvh);
  }
  img->prims.resize(order.size());
  img->prims_obj.resize(order.size());
  img->shade.resize(order.size());
  if (img->any_smooth) img->smooth_normals.resize(3 * order.size()), img->smooth_normals_obj.resize(3 * order.size());
  // Records into leaf order, on all host threads (each slot is written once).
  ParallelFor(static_cast<int64_t>(order.size()), 1 << 14, [&](int64_t s0, int64_t s1) {
  for (size_t slot = static_cast<size_t>(s0); slot < static_cast<size_t>(s1); ++slot) {
    int64_t src = source[order[slot]];
    PrimRecord r = src < ntri ? tri_rec[src] : sph_rec[src - ntri];
    PrimRecord ro = src < ntri ? tri_obj[src] : sph_rec[src - ntri];
    ShadeRecord s = src < ntri ? tri_shade[src] : sph_shade[src - ntri];
    uint32_t flags;
    std::memcpy(&flags, &r.p3.w, 4);
    if (last[slot]) flags |= kPrimLast;
    std::memcpy(&r.p3.w, &flags, 4);
    std::memcpy(&ro.p3.w, &flags, 4);
    img->prims[slot] = r;
    img->prims_obj[slot] = ro;
    img->shade[slot] = s;
    img->leaf_of_prim_id[s.s1.y] = static_cast<int32_t>(slot);
    if (img->any_smooth && src < ntri) {
      for (int k = 0; k < 3; ++k) {
        img->smooth_normals[3 * slot + k] = tri_normals[3 * src + k];
        img->smooth_normals_obj[3 * slot + k] = tri_normals_obj[3 * src + k];
      }
    }
  }
  });
  return true;
}

}  // namespace muon_gpu
