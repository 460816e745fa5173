// layout.h - device data layout of a flattened scene, shared by the host
// builder (scene.cpp) and the kernels (device.cuh).
//
// HBM layout (all arrays 16-byte aligned, read with 16-byte vector loads):
//   nodes      8 x float4 (128 B, one cache line) per 4-wide BVH node; child i
//              is the pair (lo.x, lo.y, lo.z, ref) (hi.x, hi.y, hi.z, meta):
//              ref = node index (meta == 0), first primitive of a leaf
//              (meta = count | type << 8), or kEmptyChild.  Used slots come
//              first, so a traversal stops at the first empty one.
//   tris       3 x float4 (48 B): (v0, material) (e1 = v1 - v0, group) (e2 = v2 - v0, -)
//   tri_normals 1 x float4 per triangle: normalize(e1 x e2) computed in float64,
//              or the mesh's custom normal (TriangleMeshOptions.Normals), normalised
//   tri_uvs    2 x float4 per triangle when a mesh has VertexUVs:
//              (uv0, uv1) (uv2, has, -), has = 0 for triangles without them
//   quads      5 x float4 (80 B): (corner, D) (u, material) (v, group) (normal, -) (W, -)
//   spheres    2 x float4 (32 B): (center, radius) (material, group, -, -)
//   quadrics   5 x float4 (80 B): discs, cylinders and cones
//              (p0, r0) (axis, height) (p1, r1) (apex, tan^2) (kind, material, capped, group)
//              disc: p0 = centre, axis = unit normal, r0 = radius, p1 = right,
//              apex = up (the in-plane basis of Disc.SampleUniform);
//              cylinder: p0 = base, p1 = top, r0 = r1 = radius;
//              cone: p0 = base (radius r0), p1 = top (radius r1), apex of the extended cone
//   textures   tex_info uint4 per texture (first texel, width, height, -);
//              texels float4 (r, g, b, -), row-major (ImageTexture.Pixels)
//   group (int bits): shade_group of the primitive's material kind, read by
//              the slot-order kernels without a material lookup
// Primitive ids: triangles [0, quad_base), quads [quad_base, sphere_base),
// spheres [sphere_base, quadric_base), quadrics [quadric_base, n_prims); each
// type array is in BVH leaf order.
#pragma once

#include <cstdint>
#include <vector_types.h>
#include <vector_functions.h>

namespace gprt {

constexpr uint32_t kNoHit = 0xFFFFFFFFu;
constexpr int kEmptyChild = -1;
constexpr int kLeafCountMask = 0xFF;
constexpr int kLeafTypeShift = 8;
constexpr int kPrimTriangle = 0, kPrimQuad = 1, kPrimSphere = 2, kPrimQuadric = 3;
constexpr int kQuadricDisc = 0, kQuadricCylinder = 1, kQuadricCone = 2;
constexpr int kTraceStack = 64;
// A BVH root with this bit set (test-only, GPRT_JOB_TEST_STACK_CAP) gives the
// rays of its job kTestStackCap traversal stack entries instead of
// kTraceStack.  Node indices stay below 2^30 (128 GB of nodes).
constexpr int kRootStackCap = 1 << 30;
constexpr int kTestStackCap = 1;
constexpr int kMaxNodes = 1 << 30;
// Primitive id of the marker hit a ray returns when its traversal stack
// overflowed (never a primitive: quadric ids stay below it).
constexpr uint32_t kOverflowHit = 0xFFFFFFFEu;

// device error bits (status word read by the host after each pass).  The
// path queues cannot overflow: a shading step appends at most one path and
// one shadow ray per slot of a queue of the same capacity.
constexpr int kErrStackOverflow = 1;

// kMatSpotEmissive: the disc spot light's directional emitter; albedo holds
// the unit spot direction
// kMatMix: outer / inner are materials 1 / 2, fuzz the ratio
enum : int { kMatLambertian = 0, kMatMetal = 1, kMatDielectric = 2, kMatEmissive = 3, kMatLayered = 4,
             kMatSpotEmissive = 5, kMatMix = 6 };
enum : int { kLightQuad = 0, kLightSphere = 1, kLightUniformInfinite = 2, kLightGradientInfinite = 3, kLightDisc = 4,
             kLightDiscSpot = 5, kLightPointSpot = 6 };

// The shading group of a hit on a material of this kind (the slot order
// of the shading kernels): 0 when its scatter has a pdf, so that shading
// runs next-event estimation; specular scatter (pdf 0, metal.go:60,
// dielectric.go:57) 1 for Metal and 2 for Dielectric; 3 for the emitters,
// which do not scatter (as for missed rays).
constexpr int kShadeGroups = 4;
__host__ __device__ constexpr int shade_group(int kind) {
  return kind == kMatMetal ? 1 : kind == kMatDielectric ? 2 : kind == kMatEmissive || kind == kMatSpotEmissive ? 3 : 0;
}

struct DevMaterial {
  int kind, outer, inner;
  int tex;  // Lambertian / Metal: texture index (albedo from the texture at the hit's UV), -1 for none
  float3 albedo;
  float fuzz;
  float3 emission;
  float ior;
};

struct DevLight {
  int kind;
  int prim;   // index in the quad, sphere or quadric (disc) array (area lights);
              // -1 for a sphere light that is not a scene shape
  float prob; // light-sampler selection probability
  float area; // quad area |u x v| (quad_light.go:19-27); disc area pi r^2
  float3 a;   // emission (area, uniform, spot) or top colour (gradient)
  float cos_total;    // spot lights: cosine of the total cone angle
  float3 b;   // bottom colour (gradient); unit spot direction (spot lights)
  float cos_falloff;  // spot lights: cosine of the falloff start angle
  float3 pos; // point spot light position; sphere light centre
  float radius;  // sphere light radius
};
static_assert(sizeof(DevLight) == 64, "DevLight is four 16-byte words");

// Camera (pkg/geometry/camera.go:35-67), derived in float64 on the host
struct DevCamera {
  float3 center, pixel00, du, dv, disk_u, disk_v;
  float3 u, v, w, forward;
  float focus_distance, lens_radius, lens_area, image_plane_area;
  float viewport_width, viewport_height, cos_total_width;
  int width, height, has_lens;
};

struct DevScene {
  const float4* nodes;
  const float4* tris;
  const float4* tri_normals;
  const float4* quads;
  const float4* spheres;
  const float4* quadrics;
  const DevMaterial* materials;
  const DevLight* lights;
  const float4* tri_uvs;  // per triangle (u0, v0, u1, v1) (u2, v2, has, -); null when no mesh has VertexUVs
  const uint4* tex_info;  // per texture: (first texel, width, height, -)
  const float4* texels;   // RGB (+ pad), row-major per texture
  int has_textures;       // surface UVs are computed only when set
  int n_nodes;
  int root;  // BVH root node of the scene (-1: empty)
  int n_lights;
  uint32_t quad_base, sphere_base, quadric_base, n_prims;
  int has_infinite;
  int has_specular;  // a Metal or Dielectric material: shading groups pay even without misses
  float3 world_center;
  float world_radius;
  DevCamera cam;
  int max_depth;
  int rr_min_bounces;
};

}  // namespace gprt
