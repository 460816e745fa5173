// scene.h - host representation of a flattened scene (built by scene.cpp)
#pragma once

#include <string>
#include <vector>

#include "../../include/gprt.h"
#include "layout.h"

namespace gprt {

struct HostScene {
  // device layout (host copies, uploaded by the C ABI layer)
  std::vector<float4> nodes, tris, tri_normals, quads, spheres;
  std::vector<DevMaterial> materials;
  std::vector<DevLight> lights;
  // primitive id -> (index in scene.Shapes, box face / mesh triangle)
  std::vector<uint32_t> prim_shape, prim_sub;
  uint32_t n_tris = 0, n_quads = 0, n_spheres = 0;
  int has_infinite = 0;
  double world_center[3] = {0, 0, 0};
  double world_radius = 0;
  DevCamera cam{};
  gprt_sampling_desc sampling{};
  int bvh_depth = 0;
  double build_ms = 0;
};

// Flattens `desc` into `out`.  Returns false with `err` set on invalid or
// unsupported content.
bool build_scene(const gprt_scene_desc* desc, HostScene& out, std::string& err);

// Checks the layout invariants of a built scene; returns "" when valid.
std::string validate_layout(const HostScene& s);

// CPU walk of the device BVH layout with the traversal order of the kernels,
// counting node visits, child-box tests and primitive tests.
void count_traversal(const HostScene& s, const gprt_ray* rays, uint32_t n, bool any_hit, uint64_t& nodes,
                     uint64_t& boxes, uint64_t& prims);

}  // namespace gprt
