// scene.h - host representation of a flattened scene (built by scene.cpp)
#pragma once

#include <string>
#include <vector>

#include "../../include/gprt.h"
#include "layout.h"

namespace gprt {

// Input of the device BVH builder (bvh_build.cu): every primitive in
// flattened order.
struct BuildPrims {
  std::vector<float4> box;           // 2 per primitive: (lo.xyz, type | quadric kind << 4) (hi.xyz, material), padded
  std::vector<double> geo;           // 9 per primitive: tri v0 v1 v2 / quad corner u v / sphere centre (r,0,0) /
                                     // quadric p0 p1 (r0, r1, capped) -- disc: centre normal (r, 0, 0)
  std::vector<uint32_t> shape, sub;  // index in scene.Shapes, box face / mesh triangle
  std::vector<int> light_prim;       // per light: flattened index of its primitive, -1 for infinite lights
  float clo[3], chi[3];              // centroid bounds
};

struct HostScene {
  // device layout (host copies, uploaded by the C ABI layer)
  std::vector<float4> nodes, tris, tri_normals, quads, spheres, quadrics;
  std::vector<DevMaterial> materials;
  std::vector<DevLight> lights;
  std::vector<float4> tri_uvs;  // per triangle when a mesh has VertexUVs (layout.h), else empty
  bool custom_normals = false;  // a mesh gave TriangleMeshOptions.Normals (tri_normals patched)
  std::vector<uint4> tex_info;  // per texture: first texel, width, height
  std::vector<float4> texels;
  // primitive id -> (index in scene.Shapes, box face / mesh triangle)
  std::vector<uint32_t> prim_shape, prim_sub;
  uint32_t n_tris = 0, n_quads = 0, n_spheres = 0, n_quadrics = 0;
  int has_infinite = 0;
  double world_center[3] = {0, 0, 0};
  double world_radius = 0;
  DevCamera cam{};
  gprt_sampling_desc sampling{};
  int bvh_depth = 0;
  double build_ms = 0, flatten_ms = 0, bvh_ms = 0, check_ms = 0;
  bool device_bvh = false;  // the BVH and primitive arrays are built on the GPU from `pending`
  bool test_stack_cap = false;  // GPRT_BUILD_TEST_STACK_CAP: rays get kTestStackCap stack entries
  BuildPrims pending;
};

// Flattens `desc` into `out`.  Returns false with `err` set on invalid or
// unsupported content.  With device_bvh (and at least 8 primitives) the BVH
// and the primitive arrays are left to the device builder: `out.pending`
// holds the primitives, light indices refer to the flattened order, and the
// primitive maps are filled by the builder.
bool build_scene(const gprt_scene_desc* desc, HostScene& out, std::string& err, bool device_bvh = false);

// TriangleMeshOptions.Normals / VertexUVs of the mesh triangles, applied by
// final triangle id through the primitive maps (either builder): patches
// tri_normals and fills tri_uvs.
void apply_mesh_options(const gprt_scene_desc* desc, HostScene& h);

// Checks the layout invariants of a built scene; returns "" when valid.
std::string validate_layout(const HostScene& s);

// CPU walk of the device BVH layout with the traversal order of the kernels,
// counting node visits, child-box tests and primitive tests.
void count_traversal(const HostScene& s, const gprt_ray* rays, uint32_t n, bool any_hit, uint64_t& nodes,
                     uint64_t& boxes, uint64_t& prims);

}  // namespace gprt
