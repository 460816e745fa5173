// scene.cpp - flattens a scene description into the device layout of
// layout.h and builds the 4-wide BVH.
//
// The reference builds a binary BVH with a midpoint split and leaves of up to
// 8 shapes (pkg/geometry/bvh.go:26-160), nested per triangle mesh
// (pkg/geometry/triangle_mesh.go:123).  This builder flattens every shape to
// primitives (box -> 6 quads as in pkg/geometry/box.go:41-122, mesh ->
// triangles) and builds ONE tree with a binned surface-area heuristic, then
// collapses it to 4-wide nodes for 128-byte node fetches.  Leaves hold one
// primitive type, so each leaf is a contiguous run of one type array.
// The world center/radius the infinite lights need (pkg/geometry/bvh.go:39-48)
// are computed exactly as the reference does, in float64, from the
// reference's own shape bounding boxes.
#include "scene.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <future>
#include <memory>
#include <mutex>
#include <thread>

namespace gprt {
namespace {

struct D3 {
  double x = 0, y = 0, z = 0;
  D3() = default;
  D3(double a, double b, double c) : x(a), y(b), z(c) {}
  explicit D3(const double* p) : x(p[0]), y(p[1]), z(p[2]) {}
  D3 operator+(const D3& o) const { return {x + o.x, y + o.y, z + o.z}; }
  D3 operator-(const D3& o) const { return {x - o.x, y - o.y, z - o.z}; }
  D3 operator*(double s) const { return {x * s, y * s, z * s}; }
  double dot(const D3& o) const { return x * o.x + y * o.y + z * o.z; }
  D3 cross(const D3& o) const { return {y * o.z - z * o.y, z * o.x - x * o.z, x * o.y - y * o.x}; }
  double len() const { return std::sqrt(dot(*this)); }
  D3 norm() const {
    double l = len();
    return l == 0 ? D3() : D3(x / l, y / l, z / l);
  }
  double at(int a) const { return a == 0 ? x : a == 1 ? y : z; }
  // Vec3.Rotate X -> Y -> Z (pkg/core/vec3.go:162-198)
  D3 rotate(const D3& r) const {
    if (r.x == 0 && r.y == 0 && r.z == 0) return *this;
    D3 v = *this;
    if (r.x != 0) {
      double c = std::cos(r.x), s = std::sin(r.x);
      v = D3(v.x, v.y * c - v.z * s, v.y * s + v.z * c);
    }
    if (r.y != 0) {
      double c = std::cos(r.y), s = std::sin(r.y);
      v = D3(v.x * c + v.z * s, v.y, -v.x * s + v.z * c);
    }
    if (r.z != 0) {
      double c = std::cos(r.z), s = std::sin(r.z);
      v = D3(v.x * c - v.y * s, v.x * s + v.y * c, v.z);
    }
    return v;
  }
};

struct DBox {  // reference AABB semantics (pkg/geometry/aabb.go)
  D3 mn, mx;
  DBox unite(const DBox& o) const {
    return {{std::min(mn.x, o.mn.x), std::min(mn.y, o.mn.y), std::min(mn.z, o.mn.z)},
            {std::max(mx.x, o.mx.x), std::max(mx.y, o.mx.y), std::max(mx.z, o.mx.z)}};
  }
};
DBox box_of(const D3* p, int n) {
  DBox b{p[0], p[0]};
  for (int i = 1; i < n; i++) b = b.unite(DBox{p[i], p[i]});
  return b;
}
// Quad.BoundingBox with the thin box for axis-aligned quads (quad.go:183-210)
DBox quad_ref_box(const D3& c, const D3& u, const D3& v) {
  D3 n = u.cross(v).norm();
  D3 cs[4] = {c, c + u, c + v, c + u + v};
  const double th = 0.9999, tol = 0.0001, eps = 0.001;
  int al = 0;
  if (std::fabs(n.x) > th && std::fabs(n.y) < tol && std::fabs(n.z) < tol) al = 1;
  else if (std::fabs(n.y) > th && std::fabs(n.x) < tol && std::fabs(n.z) < tol) al = 2;
  else if (std::fabs(n.z) > th && std::fabs(n.x) < tol && std::fabs(n.y) < tol) al = 3;
  DBox b = box_of(cs, 4);
  if (al == 1) { b.mn.x = cs[0].x - eps; b.mx.x = cs[0].x + eps; }
  if (al == 2) { b.mn.y = cs[0].y - eps; b.mx.y = cs[0].y + eps; }
  if (al == 3) { b.mn.z = cs[0].z - eps; b.mx.z = cs[0].z + eps; }
  return b;
}

// generateFaces (pkg/geometry/box.go:41-122): corner, u, v of the 6 faces
void box_faces(const D3& center, const D3& size, const D3& rot, D3 corner[6], D3 u[6], D3 v[6], DBox& bbox) {
  D3 cs[8] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1}, {-1, -1, 1}, {1, -1, 1}, {1, 1, 1}, {-1, 1, 1}};
  for (auto& p : cs) p = D3(p.x * size.x, p.y * size.y, p.z * size.z).rotate(rot) + center;
  const int f[6][3] = {{4, 5, 7}, {1, 0, 2}, {5, 1, 6}, {0, 4, 3}, {3, 7, 2}, {4, 0, 5}};
  for (int i = 0; i < 6; i++) {
    corner[i] = cs[f[i][0]];
    u[i] = cs[f[i][1]] - cs[f[i][0]];
    v[i] = cs[f[i][2]] - cs[f[i][0]];
  }
  bbox = box_of(cs, 8);
}

// Runs f(begin, end) over [0, n) in contiguous chunks on the host's cores
// (one chunk when n is small).
template <class F>
void parallel_for(size_t n, F f) {
  unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  unsigned T = (unsigned)std::min<size_t>(hw, n / 32768 + 1);
  if (T <= 1) {
    f((size_t)0, n);
    return;
  }
  std::vector<std::thread> th;
  for (unsigned t = 0; t < T; t++) th.emplace_back([=]() { f(n * t / T, n * (t + 1) / T); });
  for (auto& x : th) x.join();
}

float4 mk4(const D3& a, float w) { return make_float4((float)a.x, (float)a.y, (float)a.z, w); }
float i2f(uint32_t i) {
  float f;
  std::memcpy(&f, &i, 4);
  return f;
}

// ---------------------------------------------------------------- primitives
struct Prim {
  int type;
  uint32_t shape, sub, material;
  D3 a, b, c;  // tri: v0,v1,v2 ; quad: corner,u,v ; sphere: center,(r,_,_) ;
               // quadric: disc centre,normal,(r,_,_) / cylinder base,top,(r,_,capped) /
               // cone base,top,(r0,r1,capped)
  int qkind;   // kQuadric* of a quadric
};

// The reference BoundingBox of a disc, cylinder or cone (disc.go:95-118,
// cylinder.go:42-94, cone.go:79-126): conservative, flat along an axis the
// cylinder or cone is parallel to.
float3 to_f3(const double* v) { return make_float3((float)v[0], (float)v[1], (float)v[2]); }

// The in-plane basis of a disc (NewDisc, disc.go:21-43)
void disc_basis(const D3& n, D3& right, D3& up) {
  right = (std::fabs(n.x) > 0.1 ? D3(0, 1, 0) : D3(1, 0, 0)).cross(n).norm();
  up = n.cross(right).norm();
}

DBox quadric_box(const Prim& p) {
  if (p.qkind == kQuadricDisc) {
    D3 n = p.b.norm(), right, up;
    disc_basis(n, right, up);
    D3 re = right * p.c.x, ue = up * p.c.x;
    D3 cs[4] = {p.a + re + ue, p.a + re - ue, p.a - re + ue, p.a - re - ue};
    return box_of(cs, 4);
  }
  D3 axis = (p.b - p.a).norm();
  double r = p.c.x;
  double e[3];
  for (int k = 0; k < 3; k++) e[k] = std::fabs(axis.at(k)) > 0.9999 ? 0.0 : r;
  return DBox{{std::min(p.a.x, p.b.x) - e[0], std::min(p.a.y, p.b.y) - e[1], std::min(p.a.z, p.b.z) - e[2]},
              {std::max(p.a.x, p.b.x) + e[0], std::max(p.a.y, p.b.y) + e[1], std::max(p.a.z, p.b.z) + e[2]}};
}

// The device record of a quadric (layout.h), precomputed in float64.
void quadric_record(const Prim& p, int group, float4 out[5]) {
  float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
  out[0] = out[1] = out[2] = out[3] = z;
  out[4] = make_float4(i2f((uint32_t)p.qkind), i2f(p.material), p.qkind == kQuadricDisc ? 0.f : (float)p.c.z,
                       i2f((uint32_t)group));
  if (p.qkind == kQuadricDisc) {
    D3 n = p.b.norm(), right, up;
    disc_basis(n, right, up);
    out[0] = mk4(p.a, (float)p.c.x);
    out[1] = mk4(n, 0.f);
    out[2] = mk4(right, 0.f);
    out[3] = mk4(up, 0.f);
    return;
  }
  D3 av = p.b - p.a;
  double height = av.len();
  D3 axis = av.norm();
  double r0 = p.c.x, r1 = p.qkind == kQuadricCylinder ? p.c.x : p.c.y;
  out[0] = mk4(p.a, (float)r0);
  out[1] = mk4(axis, (float)height);
  out[2] = mk4(p.b, (float)r1);
  if (p.qkind == kQuadricCone) {
    D3 apex = r1 == 0 ? p.b : p.b + axis * (r1 * height / (r0 - r1));
    double tan_a = (r0 - r1) / height;
    out[3] = mk4(apex, (float)(tan_a * tan_a));
  }
}

// Primitive storage that grows without initialising: the slots of a mesh are
// filled in parallel, so the pages are first touched by the filling threads.
struct PrimArray {
  std::unique_ptr<Prim[]> p;
  size_t n = 0, cap = 0;
  void reserve(size_t c) {
    if (c <= cap) return;
    std::unique_ptr<Prim[]> q(static_cast<Prim*>(::operator new[](c * sizeof(Prim))));
    if (n) std::memcpy(static_cast<void*>(q.get()), p.get(), n * sizeof(Prim));
    p.reset(q.release());
    cap = c;
  }
  void push_back(const Prim& x) {
    if (n == cap) reserve(std::max<size_t>(16, cap * 2));
    p[n++] = x;
  }
  void grow_uninit(size_t k) {
    reserve(n + k);
    n += k;
  }
  size_t size() const { return n; }
  Prim& operator[](size_t i) { return p[i]; }
  const Prim& operator[](size_t i) const { return p[i]; }
};

struct Ref {
  float lo[3], hi[3], ct[3];
  uint32_t prim;
};

// ---------------------------------------------------------------- SAH BVH2
struct BNode {
  float lo[3], hi[3];
  std::unique_ptr<BNode> l, r;
  uint32_t begin = 0, count = 0;
  int type = 0;
  bool leaf = false;
  double area() const {
    double dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
    if (dx < 0 || dy < 0 || dz < 0) return 0;
    return 2 * (dx * dy + dy * dz + dz * dx);
  }
};

// Scenes of at most kFlatScenePrims primitives, of which at most
// kFlatSceneSpheres spheres, get one leaf per primitive type under the root:
// every ray then tests the same primitives in the same order, so the lanes
// of a warp stay converged, where a tree walk would split them over a few
// nodes each.  Sphere tests are the costlier part of a flat leaf: the
// batched sphere scenes (14-32 spheres at the small end) measured slower flat.
constexpr size_t kFlatScenePrims = 32, kFlatSceneSpheres = 8;

struct Builder {
  std::vector<Ref>& refs;
  const PrimArray& prims;
  bool flat = false;  // one leaf per type (kFlatScenePrims)
  explicit Builder(std::vector<Ref>& r, const PrimArray& p) : refs(r), prims(p) {}

  static int max_leaf(int type) { return type == kPrimQuad || type == kPrimQuadric ? 2 : 4; }

  std::unique_ptr<BNode> build(uint32_t b, uint32_t e, int depth) {
    auto n = std::make_unique<BNode>();
    for (int k = 0; k < 3; k++) {
      n->lo[k] = INFINITY;
      n->hi[k] = -INFINITY;
    }
    float clo[3] = {INFINITY, INFINITY, INFINITY}, chi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (uint32_t i = b; i < e; i++) {
      const Ref& r = refs[i];
      for (int k = 0; k < 3; k++) {
        n->lo[k] = std::min(n->lo[k], r.lo[k]);
        n->hi[k] = std::max(n->hi[k], r.hi[k]);
        clo[k] = std::min(clo[k], r.ct[k]);
        chi[k] = std::max(chi[k], r.ct[k]);
      }
    }
    uint32_t cnt = e - b;
    int type = prims[refs[b].prim].type;
    n->type = type;
    auto make_leaf = [&]() {
      n->leaf = true;
      n->begin = b;
      n->count = cnt;
      return std::move(n);
    };
    if (cnt <= 1 || flat) return make_leaf();
    // binned SAH over the three axes (16 bins)
    const int B = 16;
    double best_cost = INFINITY;
    int best_axis = -1, best_bin = -1;
    double parent = n->area();
    for (int ax = 0; ax < 3; ax++) {
      float ext = chi[ax] - clo[ax];
      if (!(ext > 0)) continue;
      float lo[B][3], hi[B][3];
      uint32_t nb[B] = {0};
      for (int k = 0; k < B; k++)
        for (int j = 0; j < 3; j++) {
          lo[k][j] = INFINITY;
          hi[k][j] = -INFINITY;
        }
      float scale = B / ext;
      for (uint32_t i = b; i < e; i++) {
        const Ref& r = refs[i];
        int k = std::min(B - 1, (int)((r.ct[ax] - clo[ax]) * scale));
        nb[k]++;
        for (int j = 0; j < 3; j++) {
          lo[k][j] = std::min(lo[k][j], r.lo[j]);
          hi[k][j] = std::max(hi[k][j], r.hi[j]);
        }
      }
      double rarea[B];
      uint32_t rcount[B];
      float rl[3] = {INFINITY, INFINITY, INFINITY}, rh[3] = {-INFINITY, -INFINITY, -INFINITY};
      uint32_t rc = 0;
      for (int k = B - 1; k > 0; k--) {
        rc += nb[k];
        for (int j = 0; j < 3; j++) {
          rl[j] = std::min(rl[j], lo[k][j]);
          rh[j] = std::max(rh[j], hi[k][j]);
        }
        double dx = rh[0] - rl[0], dy = rh[1] - rl[1], dz = rh[2] - rl[2];
        rarea[k] = rc ? 2 * (dx * dy + dy * dz + dz * dx) : 0;
        rcount[k] = rc;
      }
      float ll[3] = {INFINITY, INFINITY, INFINITY}, lh[3] = {-INFINITY, -INFINITY, -INFINITY};
      uint32_t lc = 0;
      for (int k = 0; k < B - 1; k++) {
        lc += nb[k];
        for (int j = 0; j < 3; j++) {
          ll[j] = std::min(ll[j], lo[k][j]);
          lh[j] = std::max(lh[j], hi[k][j]);
        }
        if (lc == 0 || rcount[k + 1] == 0) continue;
        double dx = lh[0] - ll[0], dy = lh[1] - ll[1], dz = lh[2] - ll[2];
        double la = 2 * (dx * dy + dy * dz + dz * dx);
        double cost = la * lc + rarea[k + 1] * rcount[k + 1];
        if (cost < best_cost) {
          best_cost = cost;
          best_axis = ax;
          best_bin = k;
        }
      }
    }
    uint32_t mid;
    if (best_axis < 0) {
      // all centroids coincide: split by index
      if (cnt <= (uint32_t)max_leaf(type)) return make_leaf();
      mid = b + cnt / 2;
    } else {
      double split_cost = 1.0 + best_cost / std::max(parent, 1e-30);
      if (cnt <= (uint32_t)max_leaf(type) && (double)cnt <= split_cost) return make_leaf();
      float ext = chi[best_axis] - clo[best_axis];
      float scale = B / ext;
      auto it = std::partition(refs.begin() + b, refs.begin() + e, [&](const Ref& r) {
        int k = std::min(B - 1, (int)((r.ct[best_axis] - clo[best_axis]) * scale));
        return k <= best_bin;
      });
      mid = (uint32_t)(it - refs.begin());
      if (mid == b || mid == e) mid = b + cnt / 2;
    }
    if (cnt > 200000 && depth < 10) {
      auto fl = std::async(std::launch::async, [&, b, mid, depth]() { return build(b, mid, depth + 1); });
      n->r = build(mid, e, depth + 1);
      n->l = fl.get();
    } else {
      n->l = build(b, mid, depth + 1);
      n->r = build(mid, e, depth + 1);
    }
    return n;
  }
};

std::unique_ptr<BNode> join(std::unique_ptr<BNode> a, std::unique_ptr<BNode> b) {
  if (!a) return b;
  if (!b) return a;
  auto n = std::make_unique<BNode>();
  for (int k = 0; k < 3; k++) {
    n->lo[k] = std::min(a->lo[k], b->lo[k]);
    n->hi[k] = std::max(a->hi[k], b->hi[k]);
  }
  n->l = std::move(a);
  n->r = std::move(b);
  return n;
}

// ---------------------------------------------------------------- BVH4 emission
// The shading group (layout.h) of a primitive with material index `mat`.
int material_group(const HostScene& h, int64_t mat) {
  return mat >= 0 && mat < (int64_t)h.materials.size() ? shade_group(h.materials[(size_t)mat].kind) : 0;
}

struct Emitter {
  HostScene& out;
  const std::vector<Ref>& refs;
  const PrimArray& prims;
  std::vector<uint32_t>& final_index;  // prim -> index in its type array
  int max_depth = 0;

  void emit_prims(const BNode* leaf, int& first) {
    for (uint32_t i = 0; i < leaf->count; i++) {
      uint32_t pid = refs[leaf->begin + i].prim;
      const Prim& p = prims[pid];
      const float grp = i2f((uint32_t)material_group(out, p.material));
      if (p.type == kPrimTriangle) {
        uint32_t idx = (uint32_t)(out.tris.size() / 3);
        if (i == 0) first = (int)idx;
        final_index[pid] = idx;
        D3 e1 = p.b - p.a, e2 = p.c - p.a;
        out.tris.push_back(mk4(p.a, i2f(p.material)));
        out.tris.push_back(mk4(e1, grp));
        out.tris.push_back(mk4(e2, 0.f));
        out.tri_normals.push_back(mk4(e1.cross(e2).norm(), 0.f));  // computeNormal (triangle.go:92-99)
      } else if (p.type == kPrimQuad) {
        uint32_t idx = (uint32_t)(out.quads.size() / 5);
        if (i == 0) first = (int)idx;
        final_index[pid] = idx;
        // NewQuad (quad.go:109-130)
        D3 n = p.b.cross(p.c).norm();
        double d = n.dot(p.a);
        D3 w = n * (1.0 / n.dot(p.b.cross(p.c)));
        out.quads.push_back(mk4(p.a, (float)d));
        out.quads.push_back(mk4(p.b, i2f(p.material)));
        out.quads.push_back(mk4(p.c, grp));
        out.quads.push_back(mk4(n, 0.f));
        out.quads.push_back(mk4(w, 0.f));
      } else if (p.type == kPrimSphere) {
        uint32_t idx = (uint32_t)(out.spheres.size() / 2);
        if (i == 0) first = (int)idx;
        final_index[pid] = idx;
        out.spheres.push_back(mk4(p.a, (float)p.b.x));
        out.spheres.push_back(make_float4(i2f(p.material), grp, 0.f, 0.f));
      } else {
        uint32_t idx = (uint32_t)(out.quadrics.size() / 5);
        if (i == 0) first = (int)idx;
        final_index[pid] = idx;
        float4 rec[5];
        quadric_record(p, material_group(out, p.material), rec);
        out.quadrics.insert(out.quadrics.end(), rec, rec + 5);
      }
    }
  }

  int emit(const BNode* n, int depth) {
    max_depth = std::max(max_depth, depth);
    int idx = (int)(out.nodes.size() / 8);
    out.nodes.resize(out.nodes.size() + 8);
    // gather up to 4 children, opening the largest internal child first
    std::vector<const BNode*> slots;
    if (n->leaf) {
      slots.push_back(n);
    } else {
      slots.push_back(n->l.get());
      slots.push_back(n->r.get());
      while (slots.size() < 4) {
        int pick = -1;
        double best = -1;
        for (size_t i = 0; i < slots.size(); i++)
          if (!slots[i]->leaf && slots[i]->area() > best) {
            best = slots[i]->area();
            pick = (int)i;
          }
        if (pick < 0) break;
        const BNode* o = slots[pick];
        slots[pick] = o->l.get();
        slots.push_back(o->r.get());
      }
    }
    float lo[3][4], hi[3][4];
    int child[4], meta[4];
    for (int i = 0; i < 4; i++) {
      for (int k = 0; k < 3; k++) {
        lo[k][i] = 1e30f;  // empty slot: inverted box, also flagged kEmptyChild
        hi[k][i] = -1e30f;
      }
      child[i] = kEmptyChild;
      meta[i] = 0;
    }
    for (size_t i = 0; i < slots.size(); i++) {
      const BNode* s = slots[i];
      for (int k = 0; k < 3; k++) {
        lo[k][i] = s->lo[k];
        hi[k][i] = s->hi[k];
      }
      if (s->leaf) {
        int first = 0;
        emit_prims(s, first);
        child[i] = first;
        meta[i] = (int)s->count | (s->type << kLeafTypeShift);
      } else {
        child[i] = emit(s, depth + 1);
        meta[i] = 0;
      }
    }
    float4* N = &out.nodes[(size_t)idx * 8];
    for (int i = 0; i < 4; i++) {  // child i: (lo, ref) (hi, meta)
      N[2 * i] = make_float4(lo[0][i], lo[1][i], lo[2][i], i2f((uint32_t)child[i]));
      N[2 * i + 1] = make_float4(hi[0][i], hi[1][i], hi[2][i], i2f((uint32_t)meta[i]));
    }
    return idx;
  }
};

// conservative float box of a primitive: rounded outward by a few ulps
void pad_box(float lo[3], float hi[3], float extent) {
  for (int k = 0; k < 3; k++) {
    float pl = 4e-7f * std::fabs(lo[k]) + 1e-7f * extent;
    float ph = 4e-7f * std::fabs(hi[k]) + 1e-7f * extent;
    lo[k] -= pl;
    hi[k] += ph;
  }
}

}  // namespace

bool build_scene(const gprt_scene_desc* d, HostScene& out, std::string& err, bool device_bvh) {
  auto t0 = std::chrono::steady_clock::now();
  if (!d) {
    err = "null scene description";
    return false;
  }
  if (d->n_shapes && !d->shapes) {
    err = "shapes pointer is null";
    return false;
  }
  if (d->n_materials && !d->materials) {
    err = "materials pointer is null";
    return false;
  }
  // textures (NewImageTexture, image_texture.go:17-23)
  out.tex_info.clear();
  out.texels.clear();
  if (d->n_textures && !d->textures) {
    err = "textures missing";
    return false;
  }
  for (uint32_t i = 0; i < d->n_textures; i++) {
    const gprt_texture_desc& t = d->textures[i];
    if (t.width == 0 || t.height == 0 || !t.pixels || (uint64_t)t.width * t.height > (1ull << 28) ||
        out.texels.size() + (uint64_t)t.width * t.height > 0xFFFFFFFFull) {
      err = "texture needs a size (at most 2^28 texels) and pixels";
      return false;
    }
    out.tex_info.push_back(make_uint4((uint32_t)out.texels.size(), t.width, t.height, 0));
    size_t n = (size_t)t.width * t.height;
    for (size_t k = 0; k < n; k++)
      out.texels.push_back(make_float4((float)t.pixels[3 * k], (float)t.pixels[3 * k + 1], (float)t.pixels[3 * k + 2], 0.f));
  }
  // materials (NewMetal clamps fuzz, metal.go:18-30)
  out.materials.resize(d->n_materials);
  for (uint32_t i = 0; i < d->n_materials; i++) {
    const gprt_material_desc& m = d->materials[i];
    DevMaterial dm{};
    dm.kind = (int)m.kind;
    dm.tex = -1;
    if (m.kind == GPRT_MAT_LAMBERTIAN || m.kind == GPRT_MAT_METAL) {
      if (m.texture > d->n_textures) {
        err = "material texture index out of range";
        return false;
      }
      dm.tex = (int)m.texture - 1;
    }
    if (m.kind > GPRT_MAT_MIX) {
      err = "unknown material kind";
      return false;
    }
    dm.albedo = make_float3((float)m.albedo[0], (float)m.albedo[1], (float)m.albedo[2]);
    if (m.kind == GPRT_MAT_SPOT_EMISSIVE) {  // albedo = the unit spot direction
      D3 sd(m.albedo);
      if (!(sd.len() > 0)) {
        err = "spot emitter direction must be non-zero";
        return false;
      }
      sd = sd.norm();
      dm.albedo = make_float3((float)sd.x, (float)sd.y, (float)sd.z);
    }
    dm.fuzz = (float)std::min(1.0, std::max(0.0, m.fuzz));
    dm.ior = (float)m.ior;
    dm.emission = make_float3((float)m.emission[0], (float)m.emission[1], (float)m.emission[2]);
    if (m.kind == GPRT_MAT_LAYERED) {
      if (m.outer >= d->n_materials || m.inner >= d->n_materials ||
          d->materials[m.outer].kind == GPRT_MAT_LAYERED || d->materials[m.inner].kind == GPRT_MAT_LAYERED ||
          d->materials[m.outer].kind == GPRT_MAT_MIX || d->materials[m.inner].kind == GPRT_MAT_MIX) {
        err = "layered material must reference two non-layered, non-mix materials";
        return false;
      }
      dm.outer = (int)m.outer;
      dm.inner = (int)m.inner;
    }
    if (m.kind == GPRT_MAT_MIX) {  // NewMix clamps the ratio (mix.go:17-27)
      auto basic = [&](uint32_t k) {
        return k < d->n_materials && d->materials[k].kind != GPRT_MAT_LAYERED && d->materials[k].kind != GPRT_MAT_MIX;
      };
      if (!basic(m.outer) || !basic(m.inner)) {
        err = "mix material must reference two non-layered, non-mix materials";
        return false;
      }
      dm.outer = (int)m.outer;
      dm.inner = (int)m.inner;
      dm.fuzz = (float)std::min(1.0, std::max(0.0, m.fuzz));
    }
    out.materials[i] = dm;
  }
  auto check_mat = [&](uint32_t m) {
    if (m >= d->n_materials) {
      err = "material index out of range";
      return false;
    }
    return true;
  };
  // primitives and the reference's world box
  PrimArray prims;
  {
    size_t total = 0;
    for (uint32_t i = 0; i < d->n_shapes; i++) {
      const gprt_shape_desc& s = d->shapes[i];
      if (s.kind == GPRT_SHAPE_MESH && d->meshes && s.mesh < d->n_meshes) total += d->meshes[s.mesh].n_triangles;
      else total += s.kind == GPRT_SHAPE_BOX ? 6 : 1;
    }
    prims.reserve(total);
  }
  std::vector<int> shape_quad_prim(d->n_shapes, -1), shape_sphere_prim(d->n_shapes, -1),
      shape_disc_prim(d->n_shapes, -1);
  DBox world{};
  bool have_world = false;
  auto add_world = [&](const DBox& b) {
    world = have_world ? world.unite(b) : b;
    have_world = true;
  };
  for (uint32_t i = 0; i < d->n_shapes; i++) {
    const gprt_shape_desc& s = d->shapes[i];
    const double* p = s.p;
    switch (s.kind) {
      case GPRT_SHAPE_SPHERE: {
        if (!check_mat(s.material)) return false;
        D3 c(p);
        double r = p[3];
        shape_sphere_prim[i] = (int)prims.size();
        prims.push_back({kPrimSphere, i, 0, s.material, c, D3(r, 0, 0), D3()});
        add_world(DBox{c - D3(r, r, r), c + D3(r, r, r)});  // Sphere.BoundingBox (sphere.go:84-90)
        break;
      }
      case GPRT_SHAPE_QUAD: {
        if (!check_mat(s.material)) return false;
        D3 c(p), u(p + 3), v(p + 6);
        if (u.cross(v).len() == 0) {
          err = "degenerate quad";
          return false;
        }
        shape_quad_prim[i] = (int)prims.size();
        prims.push_back({kPrimQuad, i, 0, s.material, c, u, v});
        add_world(quad_ref_box(c, u, v));
        break;
      }
      case GPRT_SHAPE_BOX: {
        if (!check_mat(s.material)) return false;
        D3 corner[6], u[6], v[6];
        DBox bb;
        box_faces(D3(p), D3(p + 3), D3(p + 6), corner, u, v, bb);
        for (int f = 0; f < 6; f++) prims.push_back({kPrimQuad, i, (uint32_t)f, s.material, corner[f], u[f], v[f]});
        add_world(bb);
        break;
      }
      case GPRT_SHAPE_DISC:
      case GPRT_SHAPE_CYLINDER:
      case GPRT_SHAPE_CONE: {
        if (!check_mat(s.material)) return false;
        Prim q{kPrimQuadric, i, 0, s.material, D3(p), D3(p + 3), D3(p[6], p[7], p[8]), 0};
        if (s.kind == GPRT_SHAPE_DISC) {
          shape_disc_prim[i] = (int)prims.size();
          q.qkind = kQuadricDisc;
          q.c = D3(p[6], 0, 0);
          if (q.b.len() == 0) {
            err = "disc normal must be non-zero";
            return false;
          }
        } else if (s.kind == GPRT_SHAPE_CYLINDER) {
          q.qkind = kQuadricCylinder;
          q.c = D3(p[6], 0, p[7] != 0 ? 1 : 0);
          if ((q.b - q.a).len() == 0) {
            err = "cylinder base and top must differ";
            return false;
          }
        } else {
          q.qkind = kQuadricCone;
          q.c = D3(p[6], p[7], p[8] != 0 ? 1 : 0);
          // NewCone's checks (cone.go:28-50)
          if (!(p[6] > 0) || p[7] < 0 || p[6] <= p[7] || !((q.b - q.a).len() > 0)) {
            err = "invalid cone: need base radius > top radius >= 0 and distinct centres";
            return false;
          }
        }
        prims.push_back(q);
        add_world(quadric_box(q));
        break;
      }
      case GPRT_SHAPE_TRIANGLE: {
        if (!check_mat(s.material)) return false;
        D3 a(p), b(p + 3), c(p + 6);
        prims.push_back({kPrimTriangle, i, 0, s.material, a, b, c});
        D3 v3[3] = {a, b, c};
        add_world(box_of(v3, 3));
        break;
      }
      case GPRT_SHAPE_MESH: {
        if (s.mesh >= d->n_meshes || !d->meshes) {
          err = "mesh index out of range";
          return false;
        }
        const gprt_mesh_desc& m = d->meshes[s.mesh];
        if (m.n_triangles == 0) {
          err = "empty triangle mesh";
          return false;
        }
        if (!m.vertices || !m.indices) {
          err = "mesh arrays are null";
          return false;
        }
        // the triangles on all host cores; a bad face index (NewTriangleMesh
        // panics, triangle_mesh.go:73-76) or material is reported after
        size_t first = prims.size();
        prims.grow_uninit(m.n_triangles);
        std::vector<DBox> part(std::max(1u, std::thread::hardware_concurrency()));
        std::vector<uint8_t> used(part.size(), 0);
        std::atomic<unsigned> slot{0};
        std::atomic<int> bad{0};  // 1: face index, 2: material
        parallel_for(m.n_triangles, [&](size_t b0, size_t b1) {
          if (b0 == b1) return;
          unsigned me = slot++;
          DBox mb{};
          for (size_t t = b0; t < b1; t++) {
            uint32_t ia = m.indices[3 * t], ib = m.indices[3 * t + 1], ic = m.indices[3 * t + 2];
            uint32_t mat = m.tri_materials ? m.tri_materials[t] : s.material;
            if (ia >= m.n_vertices || ib >= m.n_vertices || ic >= m.n_vertices) {
              bad |= 1;
              ia = ib = ic = 0;
            }
            if (mat >= d->n_materials) bad |= 2;
            D3 a(m.vertices + 3 * ia), b(m.vertices + 3 * ib), c(m.vertices + 3 * ic);
            prims[first + t] = {kPrimTriangle, i, (uint32_t)t, mat, a, b, c};
            D3 v3[3] = {a, b, c};
            DBox tb = box_of(v3, 3);
            mb = t == b0 ? tb : mb.unite(tb);
          }
          part[me] = mb;
          used[me] = 1;
        });
        if (bad & 1) {
          err = "Face index out of bounds";
          return false;
        }
        if (bad & 2) {
          err = "material index out of range";
          return false;
        }
        DBox mb{};
        bool have = false;
        for (size_t k = 0; k < part.size(); k++)
          if (used[k]) {
            mb = have ? mb.unite(part[k]) : part[k];
            have = true;
          }
        add_world(mb);
        break;
      }
      default:
        err = "unknown shape kind";
        return false;
    }
  }
  if (have_world) {  // NewBVH (bvh.go:39-48)
    D3 c = (world.mn + world.mx) * 0.5;
    out.world_center[0] = c.x;
    out.world_center[1] = c.y;
    out.world_center[2] = c.z;
    out.world_radius = (world.mx - c).len();
  }
  // scene extent for box padding
  double ext = 0;
  if (have_world) ext = std::max({std::fabs(world.mx.x - world.mn.x), std::fabs(world.mx.y - world.mn.y),
                                  std::fabs(world.mx.z - world.mn.z)});
  float fext = (float)std::min(ext, 1e30);
  // references per type (rank of each primitive within its type, then the
  // boxes on all host cores)
  std::vector<Ref> refs[4];
  std::vector<uint32_t> rank(prims.size());
  {
    uint32_t cnt[4] = {0, 0, 0, 0};
    for (size_t k = 0; k < prims.size(); k++) rank[k] = cnt[prims[k].type]++;
    for (int t = 0; t < 4; t++) refs[t].resize(cnt[t]);
  }
  parallel_for(prims.size(), [&](size_t b0, size_t b1) {
   for (size_t kk = b0; kk < b1; kk++) {
    uint32_t k = (uint32_t)kk;
    const Prim& p = prims[k];
    Ref r;
    r.prim = k;
    D3 pts[4];
    int np;
    if (p.type == kPrimTriangle) {
      pts[0] = p.a, pts[1] = p.b, pts[2] = p.c;
      np = 3;
    } else if (p.type == kPrimQuad) {
      pts[0] = p.a, pts[1] = p.a + p.b, pts[2] = p.a + p.c, pts[3] = p.a + p.b + p.c;
      np = 4;
    } else if (p.type == kPrimSphere) {
      double ar = std::fabs(p.b.x);
      pts[0] = p.a - D3(ar, ar, ar);
      pts[1] = p.a + D3(ar, ar, ar);
      np = 2;
    } else {
      DBox qb = quadric_box(p);
      pts[0] = qb.mn;
      pts[1] = qb.mx;
      np = 2;
    }
    DBox b = box_of(pts, np);
    r.lo[0] = (float)b.mn.x, r.lo[1] = (float)b.mn.y, r.lo[2] = (float)b.mn.z;
    r.hi[0] = (float)b.mx.x, r.hi[1] = (float)b.mx.y, r.hi[2] = (float)b.mx.z;
    pad_box(r.lo, r.hi, fext);
    for (int j = 0; j < 3; j++) r.ct[j] = 0.5f * (r.lo[j] + r.hi[j]);
    refs[p.type][rank[k]] = r;
   }
  });
  out.n_tris = (uint32_t)refs[kPrimTriangle].size();
  out.n_quads = (uint32_t)refs[kPrimQuad].size();
  out.n_spheres = (uint32_t)refs[kPrimSphere].size();
  out.n_quadrics = (uint32_t)refs[kPrimQuadric].size();
  std::vector<uint32_t> final_index(prims.size(), 0);
  out.device_bvh = device_bvh && prims.size() >= 8;
  if (out.device_bvh) {
    // the device builder takes the primitives in flattened order
    BuildPrims& bp = out.pending;
    size_t np = prims.size();
    bp.box.resize(2 * np);
    bp.geo.resize(9 * np);
    bp.shape.resize(np);
    bp.sub.resize(np);
    for (int k = 0; k < 3; k++) {
      bp.clo[k] = INFINITY;
      bp.chi[k] = -INFINITY;
    }
    std::mutex mu;
    parallel_for(np, [&](size_t b0, size_t b1) {
      float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
      for (size_t k = b0; k < b1; k++) {
        const Prim& p = prims[k];
        const Ref& r = refs[p.type][rank[k]];
        uint32_t tw = (uint32_t)p.type | (p.type == kPrimQuadric ? (uint32_t)p.qkind << 4 : 0u);
        bp.box[2 * k] = make_float4(r.lo[0], r.lo[1], r.lo[2], i2f(tw));
        bp.box[2 * k + 1] = make_float4(r.hi[0], r.hi[1], r.hi[2], i2f(p.material));
        const D3* v[3] = {&p.a, &p.b, &p.c};
        for (int q = 0; q < 3; q++) {
          bp.geo[9 * k + 3 * q] = v[q]->x;
          bp.geo[9 * k + 3 * q + 1] = v[q]->y;
          bp.geo[9 * k + 3 * q + 2] = v[q]->z;
        }
        bp.shape[k] = p.shape;
        bp.sub[k] = p.sub;
        for (int j = 0; j < 3; j++) {
          lo[j] = std::min(lo[j], r.ct[j]);
          hi[j] = std::max(hi[j], r.ct[j]);
        }
        final_index[k] = (uint32_t)k;  // flattened order until the build
      }
      std::lock_guard<std::mutex> g(mu);
      for (int j = 0; j < 3; j++) {
        bp.clo[j] = std::min(bp.clo[j], lo[j]);
        bp.chi[j] = std::max(bp.chi[j], hi[j]);
      }
    });
  }
  auto t_flat = std::chrono::steady_clock::now();
  out.flatten_ms = std::chrono::duration<double, std::milli>(t_flat - t0).count();
  std::vector<Ref> all;
  all.reserve(prims.size());
  uint32_t off[4];
  for (int t = 0; t < 4; t++) {
    off[t] = (uint32_t)all.size();
    all.insert(all.end(), refs[t].begin(), refs[t].end());
  }
  if (!out.device_bvh) {
    Builder bld(all, prims);
    bld.flat = all.size() <= kFlatScenePrims && refs[kPrimSphere].size() <= kFlatSceneSpheres;
    std::unique_ptr<BNode> roots[4];
    for (int t = 0; t < 4; t++)
      if (!refs[t].empty()) roots[t] = bld.build(off[t], off[t] + (uint32_t)refs[t].size(), 0);
    std::unique_ptr<BNode> root =
        join(std::move(roots[0]), join(std::move(roots[1]), join(std::move(roots[2]), std::move(roots[3]))));
    if (root) {
      Emitter em{out, all, prims, final_index};
      em.emit(root.get(), 0);
      out.bvh_depth = em.max_depth;
    }
    out.bvh_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_flat).count();
    // primitive id maps
    out.prim_shape.assign(prims.size(), 0);
    out.prim_sub.assign(prims.size(), 0);
    uint32_t base[4] = {0, out.n_tris, out.n_tris + out.n_quads, out.n_tris + out.n_quads + out.n_spheres};
    for (uint32_t k = 0; k < prims.size(); k++) {
      uint32_t gid = base[prims[k].type] + final_index[k];
      out.prim_shape[gid] = prims[k].shape;
      out.prim_sub[gid] = prims[k].sub;
    }
    apply_mesh_options(d, out);
  }
  // lights (pkg/scene/scene.go:102-141) and the light sampler
  // (weighted_light_sampler.go:22-78)
  double wsum = 0;
  for (uint32_t i = 0; i < d->n_lights; i++) {
    if (d->weighted_sampler && d->lights[i].weight < 0) {
      err = "weights must be non-negative";
      return false;
    }
    wsum += d->lights[i].weight;
  }
  out.has_infinite = 0;
  for (uint32_t i = 0; i < d->n_lights; i++) {
    const gprt_light_desc& l = d->lights[i];
    DevLight L{};
    L.kind = (int)l.kind;
    L.prob = (float)(d->weighted_sampler ? (wsum == 0 ? 1.0 / d->n_lights : l.weight / wsum) : 1.0 / d->n_lights);
    auto emission_of = [&](uint32_t mat) {
      const gprt_material_desc& m = d->materials[mat];
      return m.kind == GPRT_MAT_EMISSIVE ? make_float3((float)m.emission[0], (float)m.emission[1], (float)m.emission[2])
                                         : make_float3(0.f, 0.f, 0.f);
    };
    switch (l.kind) {
      case GPRT_LIGHT_QUAD: {
        if (l.shape >= d->n_shapes || shape_quad_prim[l.shape] < 0) {
          err = "quad light must reference a quad shape";
          return false;
        }
        int pid = shape_quad_prim[l.shape];
        L.prim = (int)final_index[pid];
        L.area = (float)prims[pid].b.cross(prims[pid].c).len();
        L.a = emission_of(prims[pid].material);
        break;
      }
      case GPRT_LIGHT_SPHERE: {
        if (l.shape == GPRT_NO_SHAPE) {  // a sphere light that is not a scene shape (the PBRT point light)
          if (!(l.radius > 0)) {
            err = "a sphere light without a shape needs a positive radius";
            return false;
          }
          L.prim = -1;
          L.pos = to_f3(l.from);
          L.radius = (float)l.radius;
          L.a = to_f3(l.color_a);
          break;
        }
        if (l.shape >= d->n_shapes || shape_sphere_prim[l.shape] < 0) {
          err = "sphere light must reference a sphere shape";
          return false;
        }
        int pid = shape_sphere_prim[l.shape];
        L.prim = (int)final_index[pid];
        L.pos = make_float3((float)prims[pid].a.x, (float)prims[pid].a.y, (float)prims[pid].a.z);
        L.radius = (float)prims[pid].b.x;
        L.a = emission_of(prims[pid].material);
        break;
      }
      case GPRT_LIGHT_DISC:
      case GPRT_LIGHT_DISC_SPOT: {
        if (l.shape >= d->n_shapes || shape_disc_prim[l.shape] < 0) {
          err = "disc lights must reference a disc shape";
          return false;
        }
        int pid = shape_disc_prim[l.shape];
        uint32_t mk = d->materials[prims[pid].material].kind;
        if ((l.kind == GPRT_LIGHT_DISC) == (mk == GPRT_MAT_SPOT_EMISSIVE)) {
          err = "a disc spot light's disc (and only it) carries the spot emitter material";
          return false;
        }
        L.prim = (int)final_index[pid];
        L.area = (float)(M_PI * prims[pid].c.x * prims[pid].c.x);  // pi r^2 (disc_light.go:52)
        L.a = l.kind == GPRT_LIGHT_DISC ? emission_of(prims[pid].material) : to_f3(l.color_a);
        if (l.kind == GPRT_LIGHT_DISC) break;
      }
      // fall through: the spot parameters of the disc spot light
      case GPRT_LIGHT_POINT_SPOT: {
        // NewPointSpotLight / NewDiscSpotLight (point_spot_light.go:25-40, disc_spot_light.go:80-108)
        D3 from(l.from), to(l.to);
        if (!((to - from).len() > 0)) {
          err = "spot light position and target must differ";
          return false;
        }
        D3 dir = (to - from).norm();
        L.b = make_float3((float)dir.x, (float)dir.y, (float)dir.z);
        L.cos_total = (float)std::cos(l.cone_deg * M_PI / 180.0);
        L.cos_falloff = (float)std::cos((l.cone_deg - l.cone_delta_deg) * M_PI / 180.0);
        if (l.kind == GPRT_LIGHT_POINT_SPOT) {
          L.a = to_f3(l.color_a);
          L.pos = make_float3((float)from.x, (float)from.y, (float)from.z);
        }
        break;
      }
      case GPRT_LIGHT_UNIFORM_INFINITE:
        L.a = make_float3((float)l.color_a[0], (float)l.color_a[1], (float)l.color_a[2]);
        out.has_infinite = 1;
        break;
      case GPRT_LIGHT_GRADIENT_INFINITE:
        L.a = make_float3((float)l.color_a[0], (float)l.color_a[1], (float)l.color_a[2]);
        L.b = make_float3((float)l.color_b[0], (float)l.color_b[1], (float)l.color_b[2]);
        out.has_infinite = 1;
        break;
      default:
        err = "unknown light kind";
        return false;
    }
    out.lights.push_back(L);
    if (out.device_bvh)  // remapped to leaf order by the device builder
      out.pending.light_prim.push_back(l.kind == GPRT_LIGHT_QUAD     ? shape_quad_prim[l.shape]
                                       : l.kind == GPRT_LIGHT_SPHERE
                                           ? (l.shape == GPRT_NO_SHAPE ? -1 : shape_sphere_prim[l.shape])
                                       : (l.kind == GPRT_LIGHT_DISC || l.kind == GPRT_LIGHT_DISC_SPOT)
                                           ? shape_disc_prim[l.shape]
                                           : -1);
  }
  // camera (NewCamera, pkg/geometry/camera.go:70-170) in float64
  const gprt_camera_desc& c = d->camera;
  if (c.width == 0 || !(c.aspect_ratio > 0)) {
    err = "camera width and aspect ratio must be positive";
    return false;
  }
  D3 center(c.center), look(c.look_at), up(c.up);
  D3 w = (center - look).norm();
  D3 u = w.cross(up).norm();
  D3 v = w.cross(u);
  double fd = c.focus_distance > 0 ? c.focus_distance : (center - look).len();
  double lens_radius = c.aperture / 2;
  double lens_area = c.aperture == 0 ? 1.0 : M_PI * lens_radius * lens_radius;
  int width = (int)c.width;
  int height = (int)((double)width / c.aspect_ratio);
  double theta = c.vfov_deg * M_PI / 180.0;
  double h = std::tan(theta / 2.0);
  double vh = 2.0 * h * fd, vw = vh * c.aspect_ratio;
  double vh1 = 2.0 * h, vw1 = vh1 * c.aspect_ratio;
  D3 vu = u * vw, vv = v * vh;
  D3 du = vu * (1.0 / width), dv = vv * (1.0 / height);
  D3 ul = center - w * fd - vu * 0.5 - vv * 0.5;
  D3 p00 = ul + (du + dv) * 0.5;
  D3 corner = D3(-vw / 2, -vh / 2, -fd).norm();
  auto f3d = [](const D3& a) { return make_float3((float)a.x, (float)a.y, (float)a.z); };
  DevCamera& cam = out.cam;
  cam.center = f3d(center);
  cam.pixel00 = f3d(p00);
  cam.du = f3d(du);
  cam.dv = f3d(dv);
  cam.disk_u = f3d(u * (c.aperture / 2));
  cam.disk_v = f3d(v * (c.aperture / 2));
  cam.u = f3d(u);
  cam.v = f3d(v);
  cam.w = f3d(w);
  cam.forward = f3d((look - center).norm());
  cam.focus_distance = (float)fd;
  cam.lens_radius = (float)lens_radius;
  cam.lens_area = (float)lens_area;
  cam.image_plane_area = (float)(vw1 * vh1);
  cam.viewport_width = (float)vw;
  cam.viewport_height = (float)vh;
  cam.cos_total_width = (float)corner.dot(D3(0, 0, -1));
  cam.width = width;
  cam.height = height;
  cam.has_lens = (u * (c.aperture / 2)).len() > 0 ? 1 : 0;
  out.sampling = d->sampling;
  if (out.sampling.width == 0) out.sampling.width = (uint32_t)width;
  if (out.sampling.height == 0) out.sampling.height = (uint32_t)height;
  if (out.sampling.width != (uint32_t)width || out.sampling.height != (uint32_t)height) {
    err = "sampling width/height must match the camera image size";
    return false;
  }
  if (height <= 0) {
    err = "image height must be positive";
    return false;
  }
  if (out.sampling.max_depth > 64) {
    err = "max_depth above 64 is not supported";
    return false;
  }
  auto t1 = std::chrono::steady_clock::now();
  out.build_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
  return true;
}

// ---------------------------------------------------------------- invariants
// Every node is checked independently (on all host cores): used child slots
// come first; an inner child has a larger index than its parent (both
// builders number children after their parent, so the tree is acyclic) and
// lies inside the parent's slot box; a leaf names a valid range of one
// primitive array whose primitives lie inside its box.  Then every node but
// the root must be referenced exactly once and every primitive exactly once.
void apply_mesh_options(const gprt_scene_desc* d, HostScene& h) {
  bool any_n = false, any_uv = false;
  for (uint32_t k = 0; k < d->n_meshes; k++) {
    any_n |= d->meshes[k].tri_normals != nullptr;
    any_uv |= d->meshes[k].vertex_uvs != nullptr;
  }
  h.custom_normals = any_n;
  h.tri_uvs.clear();
  if ((!any_n && !any_uv) || h.n_tris == 0) return;
  if (any_uv) h.tri_uvs.assign(2 * (size_t)h.n_tris, make_float4(0.f, 0.f, 0.f, 0.f));
  parallel_for(h.n_tris, [&](size_t b0, size_t b1) {
    for (size_t g = b0; g < b1; g++) {
      const gprt_shape_desc& sh = d->shapes[h.prim_shape[g]];
      if (sh.kind != GPRT_SHAPE_MESH) continue;
      const gprt_mesh_desc& m = d->meshes[sh.mesh];
      size_t t = h.prim_sub[g];
      if (m.tri_normals) {  // NewTriangleWithNormal (triangle.go:35-49): normalised
        D3 n = D3(m.tri_normals + 3 * t).norm();
        h.tri_normals[g] = make_float4((float)n.x, (float)n.y, (float)n.z, 0.f);
      }
      if (m.vertex_uvs) {
        const double* u0 = m.vertex_uvs + 2 * (size_t)m.indices[3 * t];
        const double* u1 = m.vertex_uvs + 2 * (size_t)m.indices[3 * t + 1];
        const double* u2 = m.vertex_uvs + 2 * (size_t)m.indices[3 * t + 2];
        h.tri_uvs[2 * g] = make_float4((float)u0[0], (float)u0[1], (float)u1[0], (float)u1[1]);
        h.tri_uvs[2 * g + 1] = make_float4((float)u2[0], (float)u2[1], 1.f, 0.f);
      }
    }
  });
}

std::string validate_layout(const HostScene& s) {
  size_t nn = s.nodes.size() / 8;
  if (nn == 0) return (s.n_tris + s.n_quads + s.n_spheres + s.n_quadrics) ? "primitives without a BVH" : "";
  size_t np[4] = {s.n_tris, s.n_quads, s.n_spheres, s.n_quadrics};
  std::unique_ptr<std::atomic<uint8_t>[]> pseen[4];
  for (int t = 0; t < 4; t++) {
    pseen[t].reset(new std::atomic<uint8_t>[np[t] ? np[t] : 1]);
    for (size_t k = 0; k < np[t]; k++) pseen[t][k].store(0, std::memory_order_relaxed);
  }
  std::unique_ptr<std::atomic<uint8_t>[]> nseen(new std::atomic<uint8_t>[nn]);
  for (size_t k = 0; k < nn; k++) nseen[k].store(0, std::memory_order_relaxed);
  std::mutex mu;
  std::string first_err;
  auto ri = [](float f) {
    int x;
    std::memcpy(&x, &f, 4);
    return x;
  };
  parallel_for(nn, [&](size_t b0, size_t b1) {
    auto bad = [&](const char* m) {
      std::lock_guard<std::mutex> g(mu);
      if (first_err.empty()) first_err = m;
    };
    for (size_t n = b0; n < b1; n++) {
      const float4* N = &s.nodes[n * 8];
      bool seen_empty = false;
      for (int i = 0; i < 4; i++) {
        const float4 &A = N[2 * i], &B = N[2 * i + 1];
        int ch = ri(A.w), mt = ri(B.w);
        if (ch == kEmptyChild) {
          seen_empty = true;
          continue;
        }
        if (seen_empty) return bad("used child slot after an empty one");
        float lo[3] = {A.x, A.y, A.z}, hi[3] = {B.x, B.y, B.z};
        auto inside = [&](float x, int k) { return x >= lo[k] && x <= hi[k]; };
        if (mt == 0) {
          if (ch <= (int)n || (size_t)ch >= nn) return bad("bad child node index");
          nseen[ch].fetch_add(1, std::memory_order_relaxed);
          const float4* C = &s.nodes[(size_t)ch * 8];
          for (int j = 0; j < 4; j++) {
            const float4 &CA = C[2 * j], &CB = C[2 * j + 1];
            if (ri(CA.w) == kEmptyChild) continue;
            if (!(CA.x >= lo[0] && CB.x <= hi[0] && CA.y >= lo[1] && CB.y <= hi[1] && CA.z >= lo[2] && CB.z <= hi[2]))
              return bad("child box not inside its parent slot");
          }
          continue;
        }
        int cnt = mt & kLeafCountMask, type = (mt >> kLeafTypeShift) & 3;
        if (cnt <= 0 || (mt & ~0x3FF)) return bad("bad leaf meta");
        if (ch < 0 || (size_t)ch + cnt > np[type]) return bad("leaf range out of bounds");
        for (int k = 0; k < cnt; k++) {
          size_t p = (size_t)ch + k;
          pseen[type][p].fetch_add(1, std::memory_order_relaxed);
          if (type == kPrimTriangle) {
            const float4* T = &s.tris[p * 3];
            float v[3][3] = {{T[0].x, T[0].y, T[0].z}, {T[0].x + T[1].x, T[0].y + T[1].y, T[0].z + T[1].z},
                             {T[0].x + T[2].x, T[0].y + T[2].y, T[0].z + T[2].z}};
            for (auto& q : v)
              for (int a = 0; a < 3; a++)
                if (!inside(q[a], a)) return bad("triangle outside its leaf box");
          } else if (type == kPrimSphere) {
            const float4& S = s.spheres[p * 2];
            float r = std::fabs(S.w), c[3] = {S.x, S.y, S.z};
            for (int a = 0; a < 3; a++)
              if (!inside(c[a] - r, a) || !inside(c[a] + r, a)) return bad("sphere outside its leaf box");
          } else if (type == kPrimQuadric) {
            const float4* Q = &s.quadrics[p * 5];
            int kind;
            std::memcpy(&kind, &Q[4].x, 4);
            if (kind < kQuadricDisc || kind > kQuadricCone) return bad("bad quadric kind");
            float c[3] = {Q[0].x, Q[0].y, Q[0].z};
            for (int a = 0; a < 3; a++)
              if (!inside(c[a], a)) return bad("quadric outside its leaf box");
          } else {
            const float4* Q = &s.quads[p * 5];
            float c[3] = {Q[0].x, Q[0].y, Q[0].z}, u[3] = {Q[1].x, Q[1].y, Q[1].z}, v[3] = {Q[2].x, Q[2].y, Q[2].z};
            for (int a = 0; a < 3; a++) {
              float xs[4] = {c[a], c[a] + u[a], c[a] + v[a], c[a] + u[a] + v[a]};
              for (float x : xs)
                if (!inside(x, a)) return bad("quad outside its leaf box");
            }
          }
        }
      }
    }
  });
  if (!first_err.empty()) return first_err;
  if (nseen[0].load()) return "the root is referenced as a child";
  for (size_t i = 1; i < nn; i++) {
    uint8_t c = nseen[i].load(std::memory_order_relaxed);
    if (c == 0) return "unreachable node";
    if (c > 1) return "node referenced twice";
  }
  for (int t = 0; t < 4; t++)
    for (size_t k = 0; k < np[t]; k++) {
      uint8_t c = pseen[t][k].load(std::memory_order_relaxed);
      if (c == 0) return "primitive missing from the BVH";
      if (c > 1) return "primitive referenced twice";
    }
  // area lights name a primitive of their kind (a disc for the disc lights)
  for (const DevLight& L : s.lights) {
    size_t n = L.kind == kLightQuad ? s.n_quads
             : L.kind == kLightSphere ? s.n_spheres
             : (L.kind == kLightDisc || L.kind == kLightDiscSpot) ? s.n_quadrics
                                                                  : SIZE_MAX;
    if (n == SIZE_MAX || (L.kind == kLightSphere && L.prim == -1)) continue;  // -1: a sphere light with no shape
    if (L.prim < 0 || (size_t)L.prim >= n) return "light primitive out of range";
    if (L.kind == kLightDisc || L.kind == kLightDiscSpot) {
      int kind;
      std::memcpy(&kind, &s.quadrics[(size_t)L.prim * 5 + 4].x, 4);
      if (kind != kQuadricDisc) return "disc light does not name a disc";
    }
  }
  return "";
}

// ---------------------------------------------------------------- CPU walk
namespace {
// Closest hit distance of a quadric record in float64 (counts only), -1 when
// missed: body, then the caps, as the device routine.
double quadric_t(const float4* Q, const float o3[3], const float d3[3], double tmin, double tmax) {
  D3 o(o3[0], o3[1], o3[2]), d(d3[0], d3[1], d3[2]);
  D3 p0(Q[0].x, Q[0].y, Q[0].z), axis(Q[1].x, Q[1].y, Q[1].z), p1(Q[2].x, Q[2].y, Q[2].z), apex(Q[3].x, Q[3].y, Q[3].z);
  int kind;
  std::memcpy(&kind, &Q[4].x, 4);
  double r0 = Q[0].w, r1 = Q[2].w, height = Q[1].w, best = tmax;
  bool any = false;
  auto cap = [&](const D3& c, const D3& nrm, double r, double eps) {
    double den = d.dot(nrm);
    if (std::fabs(den) < eps) return;
    double t = (c - o).dot(nrm) / den;
    if (t < tmin || t > best) return;
    D3 cp = o + d * t - c;
    if (cp.dot(cp) > r * r) return;
    best = t;
    any = true;
  };
  if (kind == kQuadricDisc) {
    cap(p0, axis, r0, 1e-6);
    return any ? best : -1;
  }
  auto height_ok = [&](double t, double eps) {
    double h = (o + d * t - p0).dot(axis);
    return h >= -eps && h <= height + eps;
  };
  if (kind == kQuadricCylinder) {
    D3 delta = o - p0;
    double DV = d.dot(axis), dV = delta.dot(axis);
    double a = d.dot(d) - DV * DV, b = 2 * (delta.dot(d) - dV * DV), c = delta.dot(delta) - dV * dV - r0 * r0;
    double disc = b * b - 4 * a * c;
    if (std::fabs(a) >= 1e-8 && disc >= 0) {
      double t1 = (-b - std::sqrt(disc)) / (2 * a), t2 = (-b + std::sqrt(disc)) / (2 * a);
      for (double t : {t1, t2})
        if (t >= tmin && t <= best && height_ok(t, 0)) {
          best = t;
          any = true;
          break;
        }
    }
  } else {
    D3 CO = o - apex;
    double k = 1.0 + Q[3].w;
    double DV = d.dot(axis), COV = CO.dot(axis);
    double a = d.dot(d) - k * DV * DV, b = 2 * (d.dot(CO) - k * DV * COV), c = CO.dot(CO) - k * COV * COV;
    double disc = b * b - 4 * a * c;
    if (std::fabs(a) >= 1e-8 && disc >= 0) {
      double ts[2] = {(-b - std::sqrt(disc)) / (2 * a), (-b + std::sqrt(disc)) / (2 * a)};
      for (double t : ts)
        if (t >= tmin && t <= best && height_ok(t, 1e-8) && (o + d * t - apex).dot(axis) <= 1e-8) {
          best = t;
          any = true;
          break;
        }
    }
  }
  if (Q[4].z != 0.f) {
    cap(p0, axis * -1.0, r0, 1e-8);
    if (r1 > 0) cap(p1, axis, r1, 1e-8);
  }
  return any ? best : -1;
}
}  // namespace

void count_traversal(const HostScene& s, const gprt_ray* rays, uint32_t n, bool any_hit, uint64_t& nodes,
                     uint64_t& boxes, uint64_t& prims) {
  nodes = boxes = prims = 0;
  if (s.nodes.empty()) return;
  auto rd = [](const float4& v, int i) { return i == 0 ? v.x : i == 1 ? v.y : i == 2 ? v.z : v.w; };
  auto ri = [&](const float4& v, int i) {
    float f = rd(v, i);
    int x;
    std::memcpy(&x, &f, 4);
    return x;
  };
  for (uint32_t r = 0; r < n; r++) {
    const gprt_ray& ray = rays[r];
    float o[3] = {ray.ox, ray.oy, ray.oz}, d[3] = {ray.dx, ray.dy, ray.dz};
    float inv[3], ood[3];
    for (int k = 0; k < 3; k++) {
      float dd = std::fabs(d[k]) > 1e-20f ? d[k] : std::copysign(1e-20f, d[k]);
      inv[k] = 1.0f / dd;
      ood[k] = o[k] * inv[k];
    }
    std::vector<int> stack;
    int node = 0;
    float best = ray.tmax;
    bool done = false;
    while (node >= 0 && !done) {
      const float4* N = &s.nodes[(size_t)node * 8];
      nodes++;
      int ich[4];
      float itn[4];
      int nint = 0;
      for (int i = 0; i < 4 && !done; i++) {
        int ch = ri(N[2 * i], 3), mt = ri(N[2 * i + 1], 3);
        if (ch == kEmptyChild) break;
        boxes++;
        float t0[3], t1[3];
        for (int k = 0; k < 3; k++) {
          float lo = rd(N[2 * i], k), hi = rd(N[2 * i + 1], k);
          bool neg = inv[k] < 0;
          t0[k] = std::fma(neg ? hi : lo, inv[k], -ood[k]);
          t1[k] = std::fma(neg ? lo : hi, inv[k], -ood[k]);
        }
        float tn = std::max(std::max(t0[0], t0[1]), std::max(t0[2], ray.tmin));
        float tf = std::min(std::min(t1[0], t1[1]), std::min(t1[2], best));
        if (tn > tf) continue;
        if (mt == 0) {
          int k = nint++;
          while (k > 0 && itn[k - 1] > tn) {
            itn[k] = itn[k - 1];
            ich[k] = ich[k - 1];
            k--;
          }
          itn[k] = tn;
          ich[k] = ch;
          continue;
        }
        int cnt = mt & kLeafCountMask, type = (mt >> kLeafTypeShift) & 3;
        for (int k = 0; k < cnt; k++) {
          prims++;
          int p = ch + k;
          // exact distance of the candidate in float64 (counts only)
          double t = -1;
          if (type == kPrimTriangle) {
            const float4* T = &s.tris[(size_t)p * 3];
            double e1[3] = {T[1].x, T[1].y, T[1].z}, e2[3] = {T[2].x, T[2].y, T[2].z};
            double sv[3] = {o[0] - T[0].x, o[1] - T[0].y, o[2] - T[0].z};
            double h[3] = {d[1] * e2[2] - d[2] * e2[1], d[2] * e2[0] - d[0] * e2[2], d[0] * e2[1] - d[1] * e2[0]};
            double a = e1[0] * h[0] + e1[1] * h[1] + e1[2] * h[2];
            if (std::fabs(a) < 1e-8) continue;
            double f = 1.0 / a, u = f * (sv[0] * h[0] + sv[1] * h[1] + sv[2] * h[2]);
            if (u < 0 || u > 1) continue;
            double q[3] = {sv[1] * e1[2] - sv[2] * e1[1], sv[2] * e1[0] - sv[0] * e1[2], sv[0] * e1[1] - sv[1] * e1[0]};
            double vv = f * (d[0] * q[0] + d[1] * q[1] + d[2] * q[2]);
            if (vv < 0 || u + vv > 1) continue;
            t = f * (e2[0] * q[0] + e2[1] * q[1] + e2[2] * q[2]);
          } else if (type == kPrimQuad) {
            const float4* Q = &s.quads[(size_t)p * 5];
            double nn[3] = {Q[3].x, Q[3].y, Q[3].z};
            double den = d[0] * nn[0] + d[1] * nn[1] + d[2] * nn[2];
            if (std::fabs(den) < 1e-8) continue;
            t = (Q[0].w - (o[0] * nn[0] + o[1] * nn[1] + o[2] * nn[2])) / den;
            double hp[3] = {o[0] + d[0] * t - Q[0].x, o[1] + d[1] * t - Q[0].y, o[2] + d[2] * t - Q[0].z};
            double U[3] = {Q[1].x, Q[1].y, Q[1].z}, V[3] = {Q[2].x, Q[2].y, Q[2].z}, W[3] = {Q[4].x, Q[4].y, Q[4].z};
            double hv[3] = {hp[1] * V[2] - hp[2] * V[1], hp[2] * V[0] - hp[0] * V[2], hp[0] * V[1] - hp[1] * V[0]};
            double uh[3] = {U[1] * hp[2] - U[2] * hp[1], U[2] * hp[0] - U[0] * hp[2], U[0] * hp[1] - U[1] * hp[0]};
            double al = W[0] * hv[0] + W[1] * hv[1] + W[2] * hv[2], be = W[0] * uh[0] + W[1] * uh[1] + W[2] * uh[2];
            if (al < 0 || al > 1 || be < 0 || be > 1) continue;
          } else if (type == kPrimSphere) {
            const float4& S = s.spheres[(size_t)p * 2];
            double f[3] = {o[0] - S.x, o[1] - S.y, o[2] - S.z};
            double a = (double)d[0] * d[0] + (double)d[1] * d[1] + (double)d[2] * d[2];
            double hb = f[0] * d[0] + f[1] * d[1] + f[2] * d[2];
            double c = f[0] * f[0] + f[1] * f[1] + f[2] * f[2] - (double)S.w * S.w;
            double disc = hb * hb - a * c;
            if (disc < 0) continue;
            t = (-hb - std::sqrt(disc)) / a;
            if (t < ray.tmin || t > best) t = (-hb + std::sqrt(disc)) / a;
          } else {
            t = quadric_t(&s.quadrics[(size_t)p * 5], o, d, ray.tmin, best);
          }
          if (t >= ray.tmin && t <= best) {
            best = (float)t;
            if (any_hit) {
              done = true;
              break;
            }
          }
        }
      }
      if (done) break;
      int keep = 0;
      for (int k = 0; k < nint; k++)
        if (itn[k] <= best) {
          itn[keep] = itn[k];
          ich[keep] = ich[k];
          keep++;
        }
      if (keep > 0) {
        for (int k = keep - 1; k >= 1; k--) stack.push_back(ich[k]);
        node = ich[0];
      } else if (!stack.empty()) {
        node = stack.back();
        stack.pop_back();
      } else {
        node = -1;
      }
    }
  }
}

}  // namespace gprt
