// bvh_build.cu - BVH construction on the GPU (GPRT_BUILD_DEVICE).
//
// Replaces the role of geometry.NewBVH (pkg/geometry/bvh.go:26-160) for
// scenes that must become renderable quickly: a linear BVH after Karras,
// "Maximizing Parallelism in the Construction of BVHs, Octrees, and k-d
// Trees" (HPG 2012), collapsed to the 4-wide node layout of layout.h.
//   1. keys: primitive type (2 bits, so each type's primitives form one
//      contiguous range) above a 60-bit Morton code of the box centroid;
//   2. radix sort of (key, primitive) pairs;
//   3. one thread per internal node finds its key range and split (binary
//      radix tree; equal keys are told apart by their sorted position);
//   4. bounds bottom-up: each leaf climbs, the second arrival at a node
//      forms the union of its two children;
//   5. collapse to BVH4 top-down, one level per launch: a node takes its two
//      children and opens the child of largest surface area until it holds
//      four; a subtree of at most 4 primitives (2 quads) of one type becomes
//      a leaf over its contiguous range;
//   6. the primitive arrays are written in sorted order (the leaf order) with
//      the same precomputation as the host emitter (float64 edge vectors,
//      normals, quad plane constants).
// The boxes are the host's padded float boxes, so the world bounds and the
// intersection results do not depend on which builder ran.
#include <cub/device/device_radix_sort.cuh>

#include <algorithm>
#include <chrono>
#include <cstring>

#include "handles.h"

namespace gprt {
namespace {

constexpr uint32_t kLeafBit = 0x80000000u;

__device__ __forceinline__ uint64_t spread_bits(uint32_t x) {  // 20 bits -> every third bit
  uint64_t v = x & 0xFFFFFu;
  v = (v | (v << 32)) & 0x1F00000000FFFFull;
  v = (v | (v << 16)) & 0x1F0000FF0000FFull;
  v = (v | (v << 8)) & 0x100F00F00F00F00Full;
  v = (v | (v << 4)) & 0x10C30C30C30C30C3ull;
  v = (v | (v << 2)) & 0x1249249249249249ull;
  return v;
}

__global__ void k_keys(uint32_t n, const float4* box, float3 clo, float3 cinv, unsigned long long* keys,
                       uint32_t* idx) {
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    float4 lo = box[2 * k], hi = box[2 * k + 1];
    uint32_t type = __float_as_uint(lo.w) & 3u;
    float c[3] = {0.5f * (lo.x + hi.x), 0.5f * (lo.y + hi.y), 0.5f * (lo.z + hi.z)};
    float o[3] = {clo.x, clo.y, clo.z}, s[3] = {cinv.x, cinv.y, cinv.z};
    uint64_t m = 0;
    for (int a = 0; a < 3; a++) {
      float q = fminf(fmaxf((c[a] - o[a]) * s[a], 0.f), 1.f);
      m |= spread_bits((uint32_t)(q * 1048575.f)) << (2 - a);
    }
    keys[k] = ((unsigned long long)type << 62) | m;
    idx[k] = k;
  }
}

// Common-prefix length of sorted keys i and j (-1 outside the array); equal
// keys compare by position.
__device__ __forceinline__ int delta(const unsigned long long* K, int n, int i, int j) {
  if (j < 0 || j >= n) return -1;
  unsigned long long a = K[i], b = K[j];
  if (a == b) return 64 + __clz((uint32_t)(i ^ j));
  return __clzll((long long)(a ^ b));
}

// Binary radix tree: internal node i of n - 1 (root 0).  Children carry
// kLeafBit when they are leaves (sorted positions).
__global__ void k_radix_tree(int n, const unsigned long long* K, uint32_t* left, uint32_t* right, uint32_t* first,
                             uint32_t* last, int* parent_int, int* parent_leaf) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n - 1; i += gridDim.x * blockDim.x) {
    int d = (delta(K, n, i, i + 1) - delta(K, n, i, i - 1)) >= 0 ? 1 : -1;
    int dmin = delta(K, n, i, i - d);
    int lmax = 2;
    while (delta(K, n, i, i + lmax * d) > dmin) lmax *= 2;
    int l = 0;
    for (int t = lmax / 2; t >= 1; t /= 2)
      if (delta(K, n, i, i + (l + t) * d) > dmin) l += t;
    int j = i + l * d;
    int dnode = delta(K, n, i, j);
    int s = 0;
    for (int div = 2;; div *= 2) {
      int t = (l + div - 1) / div;
      if (delta(K, n, i, i + (s + t) * d) > dnode) s += t;
      if (t <= 1) break;
    }
    int g = i + s * d + min(d, 0);
    int lo = min(i, j), hi = max(i, j);
    uint32_t lc = lo == g ? ((uint32_t)g | kLeafBit) : (uint32_t)g;
    uint32_t rc = hi == g + 1 ? ((uint32_t)(g + 1) | kLeafBit) : (uint32_t)(g + 1);
    left[i] = lc;
    right[i] = rc;
    first[i] = (uint32_t)lo;
    last[i] = (uint32_t)hi;
    if (lc & kLeafBit) parent_leaf[g] = i;
    else parent_int[g] = i;
    if (rc & kLeafBit) parent_leaf[g + 1] = i;
    else parent_int[g + 1] = i;
  }
}

struct Box3 {
  float3 lo, hi;
};

__device__ __forceinline__ Box3 leaf_box(const float4* box, const uint32_t* idx, uint32_t j) {
  uint32_t k = idx[j];
  float4 a = box[2 * k], b = box[2 * k + 1];
  return Box3{make_float3(a.x, a.y, a.z), make_float3(b.x, b.y, b.z)};
}

__device__ __forceinline__ Box3 child_box(const float4* box, const uint32_t* idx, const float4* ibox, uint32_t c) {
  if (c & kLeafBit) return leaf_box(box, idx, c & ~kLeafBit);
  float4 a = __ldcg(ibox + 2 * c), b = __ldcg(ibox + 2 * c + 1);
  return Box3{make_float3(a.x, a.y, a.z), make_float3(b.x, b.y, b.z)};
}

// Bounds bottom-up: the second thread to reach a node has both children.
__global__ void k_bounds(int n, const float4* box, const uint32_t* idx, const uint32_t* left, const uint32_t* right,
                         const int* parent_int, const int* parent_leaf, float4* ibox, int* visits) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    int p = parent_leaf[j];
    while (p >= 0) {
      __threadfence();
      if (atomicAdd(&visits[p], 1) == 0) break;  // the sibling's box is not ready yet
      Box3 a = child_box(box, idx, ibox, left[p]), b = child_box(box, idx, ibox, right[p]);
      ibox[2 * p] = make_float4(fminf(a.lo.x, b.lo.x), fminf(a.lo.y, b.lo.y), fminf(a.lo.z, b.lo.z), 0.f);
      ibox[2 * p + 1] = make_float4(fmaxf(a.hi.x, b.hi.x), fmaxf(a.hi.y, b.hi.y), fmaxf(a.hi.z, b.hi.z), 0.f);
      p = p == 0 ? -1 : parent_int[p];
    }
  }
}

struct TreeView {
  const unsigned long long* K;
  const float4* box;
  const uint32_t* idx;
  const uint32_t *left, *right, *first, *last;
  const float4* ibox;
  uint32_t off[4];  // first sorted position of each primitive type
};

__device__ __forceinline__ void range_of(const TreeView& T, uint32_t c, uint32_t& f, uint32_t& l) {
  if (c & kLeafBit) {
    f = l = c & ~kLeafBit;
  } else {
    f = T.first[c];
    l = T.last[c];
  }
}

__device__ __forceinline__ bool leafable(const TreeView& T, uint32_t c) {
  if (c & kLeafBit) return true;
  uint32_t f = T.first[c], l = T.last[c];
  uint32_t tf = (uint32_t)(T.K[f] >> 62), tl = (uint32_t)(T.K[l] >> 62);
  if (tf != tl) return false;
  return l - f + 1 <= (tf == (uint32_t)kPrimQuad || tf == (uint32_t)kPrimQuadric ? 2u : 4u);
}

__device__ __forceinline__ float area(const Box3& b) {
  float dx = b.hi.x - b.lo.x, dy = b.hi.y - b.lo.y, dz = b.hi.z - b.lo.z;
  return dx * dy + dy * dz + dz * dx;
}

// One level of the collapse: item q holds (radix-tree node, BVH4 node index).
__global__ void k_collapse(TreeView T, const uint2* qin, const uint32_t* qin_n, uint2* qout, uint32_t* qout_n,
                           uint32_t* n4, float4* nodes, uint32_t cap4, int* err) {
  uint32_t nq = *qin_n;
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += gridDim.x * blockDim.x) {
    uint2 item = qin[q];
    uint32_t slot[4];
    int ns = 2;
    slot[0] = T.left[item.x];
    slot[1] = T.right[item.x];
    while (ns < 4) {
      int pick = -1;
      float best = -1.f;
      for (int i = 0; i < ns; i++) {
        if (leafable(T, slot[i])) continue;
        float a = area(child_box(T.box, T.idx, T.ibox, slot[i]));
        if (a > best) {
          best = a;
          pick = i;
        }
      }
      if (pick < 0) break;
      uint32_t c = slot[pick];
      slot[pick] = T.left[c];
      slot[ns++] = T.right[c];
    }
    float4* N = nodes + (size_t)item.y * 8;
    for (int i = 0; i < 4; i++) {
      if (i >= ns) {
        N[2 * i] = make_float4(1e30f, 1e30f, 1e30f, __int_as_float(kEmptyChild));
        N[2 * i + 1] = make_float4(-1e30f, -1e30f, -1e30f, __int_as_float(0));
        continue;
      }
      uint32_t c = slot[i];
      Box3 b = child_box(T.box, T.idx, T.ibox, c);
      int ref, meta;
      if (leafable(T, c)) {
        uint32_t f, l;
        range_of(T, c, f, l);
        uint32_t type = (uint32_t)(T.K[f] >> 62);
        ref = (int)(f - T.off[type]);
        meta = (int)(l - f + 1) | (int)(type << kLeafTypeShift);
      } else {
        uint32_t child = atomicAdd(n4, 1u);
        if (child >= cap4) {
          atomicOr(err, 1);
          child = 0;
        } else {
          qout[atomicAdd(qout_n, 1u)] = make_uint2(c, child);
        }
        ref = (int)child;
        meta = 0;
      }
      N[2 * i] = make_float4(b.lo.x, b.lo.y, b.lo.z, __int_as_float(ref));
      N[2 * i + 1] = make_float4(b.hi.x, b.hi.y, b.hi.z, __int_as_float(meta));
    }
  }
}

// The primitive arrays in sorted (leaf) order, precomputed as the host
// emitter does (NewQuad, quad.go:109-130; computeNormal, triangle.go:92-99);
// `group` holds the shading group of each of the n_mat materials.
__global__ void k_gather(uint32_t n, const float4* box, const double* geo, const uint32_t* idx, uint4 off,
                         float4* tris, float4* tri_normals, float4* quads, float4* spheres, float4* quadrics,
                         uint32_t* final_index, const int* group, int n_mat) {
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    uint32_t k = idx[j];
    uint32_t tw = __float_as_uint(box[2 * k].w), type = tw & 3u;
    float mat = box[2 * k + 1].w;  // material index as int bits
    int mi = __float_as_int(mat);
    float grp = __int_as_float(mi >= 0 && mi < n_mat ? group[mi] : 0);
    const double* g = geo + (size_t)9 * k;
    double ax = g[0], ay = g[1], az = g[2], bx = g[3], by = g[4], bz = g[5], cx = g[6], cy = g[7], cz = g[8];
    uint32_t local;
    if (type == (uint32_t)kPrimTriangle) {
      local = j - off.x;
      double e1x = bx - ax, e1y = by - ay, e1z = bz - az, e2x = cx - ax, e2y = cy - ay, e2z = cz - az;
      double nx = e1y * e2z - e1z * e2y, ny = e1z * e2x - e1x * e2z, nz = e1x * e2y - e1y * e2x;
      double inv = 1.0 / sqrt(nx * nx + ny * ny + nz * nz);
      float4* T = tris + (size_t)local * 3;
      T[0] = make_float4((float)ax, (float)ay, (float)az, mat);
      T[1] = make_float4((float)e1x, (float)e1y, (float)e1z, grp);
      T[2] = make_float4((float)e2x, (float)e2y, (float)e2z, 0.f);
      tri_normals[local] = make_float4((float)(nx * inv), (float)(ny * inv), (float)(nz * inv), 0.f);
    } else if (type == (uint32_t)kPrimQuad) {
      local = j - off.y;
      double crx = by * cz - bz * cy, cry = bz * cx - bx * cz, crz = bx * cy - by * cx;  // u x v
      double inv = 1.0 / sqrt(crx * crx + cry * cry + crz * crz);
      double nx = crx * inv, ny = cry * inv, nz = crz * inv;
      double dd = nx * ax + ny * ay + nz * az;
      double w = 1.0 / (nx * crx + ny * cry + nz * crz);
      float4* Q = quads + (size_t)local * 5;
      Q[0] = make_float4((float)ax, (float)ay, (float)az, (float)dd);
      Q[1] = make_float4((float)bx, (float)by, (float)bz, mat);
      Q[2] = make_float4((float)cx, (float)cy, (float)cz, grp);
      Q[3] = make_float4((float)nx, (float)ny, (float)nz, 0.f);
      Q[4] = make_float4((float)(nx * w), (float)(ny * w), (float)(nz * w), 0.f);
    } else if (type == (uint32_t)kPrimSphere) {
      local = j - off.z;
      spheres[(size_t)local * 2] = make_float4((float)ax, (float)ay, (float)az, (float)bx);
      spheres[(size_t)local * 2 + 1] = make_float4(mat, grp, 0.f, 0.f);
    } else {
      // disc / cylinder / cone record (layout.h), as the host's quadric_record
      local = j - off.w;
      int kind = (int)(tw >> 4);
      float4* R = quadrics + (size_t)local * 5;
      float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
      R[2] = R[3] = z;
      R[4] = make_float4(__int_as_float(kind), mat, kind == kQuadricDisc ? 0.f : (float)cz, grp);
      if (kind == kQuadricDisc) {
        double inv = 1.0 / sqrt(bx * bx + by * by + bz * bz);
        R[0] = make_float4((float)ax, (float)ay, (float)az, (float)cx);
        R[1] = make_float4((float)(bx * inv), (float)(by * inv), (float)(bz * inv), 0.f);
      } else {
        double vx = bx - ax, vy = by - ay, vz = bz - az;
        double hgt = sqrt(vx * vx + vy * vy + vz * vz), inv = 1.0 / hgt;
        double ux = vx * inv, uy = vy * inv, uz = vz * inv;
        double r0 = cx, r1 = kind == kQuadricCylinder ? cx : cy;
        R[0] = make_float4((float)ax, (float)ay, (float)az, (float)r0);
        R[1] = make_float4((float)ux, (float)uy, (float)uz, (float)hgt);
        R[2] = make_float4((float)bx, (float)by, (float)bz, (float)r1);
        if (kind == kQuadricCone) {
          double s = r1 == 0 ? 0.0 : r1 * hgt / (r0 - r1), ta = (r0 - r1) / hgt;
          R[3] = make_float4((float)(bx + ux * s), (float)(by + uy * s), (float)(bz + uz * s), (float)(ta * ta));
        }
      }
    }
    final_index[k] = local;
  }
}

template <class T>
int upload_vec(gprt_ctx* ctx, std::vector<void*>& tmp, const std::vector<T>& v, T** out, cudaStream_t st) {
  int rc = dev_alloc(ctx, tmp, out, v.size());
  if (rc) return rc;
  if (!v.empty()) CK(ctx, cudaMemcpyAsync(*out, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st));
  return GPRT_OK;
}

}  // namespace

int device_build_bvh(gprt_ctx* ctx, HostScene& h, DevScene& d, std::vector<void*>& bufs, size_t* bytes) {
  auto t0 = std::chrono::steady_clock::now();
  cudaStream_t st = ctx->stream;
  BuildPrims& bp = h.pending;
  const uint32_t n = (uint32_t)(bp.box.size() / 2);
  std::vector<void*> tmp;
  auto cleanup = [&](int rc) {
    cudaStreamSynchronize(st);
    free_all(tmp);
    return rc;
  };
  float4* box = nullptr;
  double* geo = nullptr;
  int rc = upload_vec(ctx, tmp, bp.box, &box, st);
  if (!rc) rc = upload_vec(ctx, tmp, bp.geo, &geo, st);
  unsigned long long *keys = nullptr, *keys2 = nullptr;
  uint32_t *idx = nullptr, *idx2 = nullptr, *left = nullptr, *right = nullptr, *first = nullptr, *last = nullptr;
  int *pint = nullptr, *pleaf = nullptr, *visits = nullptr, *err = nullptr;
  float4* ibox = nullptr;
  uint2 *qa = nullptr, *qb = nullptr;
  uint32_t *qn = nullptr, *final_index = nullptr;
  float4* nodes_tmp = nullptr;
  rc |= dev_alloc(ctx, tmp, &keys, n);
  rc |= dev_alloc(ctx, tmp, &keys2, n);
  rc |= dev_alloc(ctx, tmp, &idx, n);
  rc |= dev_alloc(ctx, tmp, &idx2, n);
  rc |= dev_alloc(ctx, tmp, &left, n);
  rc |= dev_alloc(ctx, tmp, &right, n);
  rc |= dev_alloc(ctx, tmp, &first, n);
  rc |= dev_alloc(ctx, tmp, &last, n);
  rc |= dev_alloc(ctx, tmp, &pint, n);
  rc |= dev_alloc(ctx, tmp, &pleaf, n);
  rc |= dev_alloc(ctx, tmp, &visits, n);
  rc |= dev_alloc(ctx, tmp, &ibox, 2 * (size_t)n);
  rc |= dev_alloc(ctx, tmp, &qa, n);
  rc |= dev_alloc(ctx, tmp, &qb, n);
  rc |= dev_alloc(ctx, tmp, &qn, 4);  // [0],[1] queue sizes, [2] BVH4 node count
  rc |= dev_alloc(ctx, tmp, &err, 1);
  rc |= dev_alloc(ctx, tmp, &final_index, n);
  rc |= dev_alloc(ctx, tmp, &nodes_tmp, (size_t)n * 8);  // at most n - 1 nodes
  if (rc) return cleanup(GPRT_E_OOM);
  // 1. keys
  float3 clo = make_float3(bp.clo[0], bp.clo[1], bp.clo[2]);
  float ext[3] = {bp.chi[0] - bp.clo[0], bp.chi[1] - bp.clo[1], bp.chi[2] - bp.clo[2]};
  float3 cinv = make_float3(ext[0] > 0 ? 1.f / ext[0] : 0.f, ext[1] > 0 ? 1.f / ext[1] : 0.f,
                            ext[2] > 0 ? 1.f / ext[2] : 0.f);
  int grid = launch_grid(n, 256, ctx->sm_count * 8);
  k_keys<<<grid, 256, 0, st>>>(n, box, clo, cinv, keys, idx);
  // 2. sort
  size_t sort_bytes = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, sort_bytes, keys, keys2, idx, idx2, (int)n, 0, 64, st);
  void* sort_tmp = nullptr;
  if (dev_alloc(ctx, tmp, reinterpret_cast<unsigned char**>(&sort_tmp), sort_bytes)) return cleanup(GPRT_E_OOM);
  cub::DeviceRadixSort::SortPairs(sort_tmp, sort_bytes, keys, keys2, idx, idx2, (int)n, 0, 64, st);
  // 3. radix tree, 4. bounds
  CK(ctx, cudaMemsetAsync(pint, 0xFF, (size_t)n * sizeof(int), st));
  CK(ctx, cudaMemsetAsync(visits, 0, (size_t)n * sizeof(int), st));
  CK(ctx, cudaMemsetAsync(qn, 0, 4 * sizeof(uint32_t), st));
  CK(ctx, cudaMemsetAsync(err, 0, sizeof(int), st));
  k_radix_tree<<<grid, 256, 0, st>>>((int)n, keys2, left, right, first, last, pint, pleaf);
  k_bounds<<<grid, 256, 0, st>>>((int)n, box, idx2, left, right, pint, pleaf, ibox, visits);
  // 5. collapse, level by level from the root (n >= 8: the root is not a leaf)
  TreeView T{keys2, box, idx2, left, right, first, last, ibox,
             {0, h.n_tris, h.n_tris + h.n_quads, h.n_tris + h.n_quads + h.n_spheres}};
  uint2 root = make_uint2(0, 0);
  uint32_t one[3] = {1, 0, 1};  // one queued item; the root occupies BVH4 node 0
  CK(ctx, cudaMemcpyAsync(qa, &root, sizeof(root), cudaMemcpyHostToDevice, st));
  CK(ctx, cudaMemcpyAsync(qn, one, sizeof(one), cudaMemcpyHostToDevice, st));
  uint2 *qin = qa, *qout = qb;
  int in_slot = 0, levels = 0;
  for (;;) {
    CK(ctx, cudaMemcpyAsync(ctx->h_words, qn + in_slot, 4, cudaMemcpyDeviceToHost, st));
    CK(ctx, cudaStreamSynchronize(st));
    uint32_t cnt = ctx->h_words[0];
    if (cnt == 0) break;
    levels++;
    CK(ctx, cudaMemsetAsync(qn + (in_slot ^ 1), 0, 4, st));
    k_collapse<<<launch_grid(cnt, 128, ctx->sm_count * 16), 128, 0, st>>>(T, qin, qn + in_slot, qout, qn + (in_slot ^ 1),
                                                                       qn + 2, nodes_tmp, n, err);
    std::swap(qin, qout);
    in_slot ^= 1;
  }
  CK(ctx, cudaMemcpyAsync(ctx->h_words, qn + 2, 4, cudaMemcpyDeviceToHost, st));
  CK(ctx, cudaMemcpyAsync(ctx->h_words + 1, err, 4, cudaMemcpyDeviceToHost, st));
  CK(ctx, cudaStreamSynchronize(st));
  uint32_t n4 = ctx->h_words[0];
  int e = (int)ctx->h_words[1];
  if (e) return cleanup(fail(ctx, GPRT_E_BOUND, "device BVH build exceeded its node capacity"));
  // 6. primitive arrays in leaf order, and the node array at its final size
  float4 *nodes = nullptr, *tris = nullptr, *normals = nullptr, *quads = nullptr, *spheres = nullptr,
         *quadrics = nullptr;
  rc = 0;
  rc |= dev_alloc(ctx, bufs, &nodes, (size_t)n4 * 8, bytes);
  rc |= dev_alloc(ctx, bufs, &tris, (size_t)h.n_tris * 3, bytes);
  rc |= dev_alloc(ctx, bufs, &normals, (size_t)h.n_tris, bytes);
  rc |= dev_alloc(ctx, bufs, &quads, (size_t)h.n_quads * 5, bytes);
  rc |= dev_alloc(ctx, bufs, &spheres, (size_t)h.n_spheres * 2, bytes);
  rc |= dev_alloc(ctx, bufs, &quadrics, (size_t)h.n_quadrics * 5, bytes);
  if (rc) return cleanup(GPRT_E_OOM);
  CK(ctx, cudaMemcpyAsync(nodes, nodes_tmp, (size_t)n4 * 128, cudaMemcpyDeviceToDevice, st));
  uint4 off = make_uint4(0, h.n_tris, h.n_tris + h.n_quads, h.n_tris + h.n_quads + h.n_spheres);
  std::vector<int> groups(std::max<size_t>(1, h.materials.size()), 0);
  for (size_t m = 0; m < h.materials.size(); m++) groups[m] = shade_group(h.materials[m].kind);
  int* d_groups = nullptr;
  if (dev_alloc(ctx, tmp, &d_groups, groups.size())) return cleanup(GPRT_E_OOM);
  CK(ctx, cudaMemcpyAsync(d_groups, groups.data(), groups.size() * sizeof(int), cudaMemcpyHostToDevice, st));
  k_gather<<<grid, 256, 0, st>>>(n, box, geo, idx2, off, tris, normals, quads, spheres, quadrics, final_index,
                                 d_groups, (int)h.materials.size());
  cudaError_t le = cudaGetLastError();
  if (le != cudaSuccess) return cleanup(cuda_fail(ctx, le, "device BVH build launch"));
  // host copies (layout checks, traversal counts) and the primitive maps
  std::vector<uint32_t> fi(n);
  h.nodes.resize((size_t)n4 * 8);
  h.tris.resize((size_t)h.n_tris * 3);
  h.tri_normals.resize(h.n_tris);
  h.quads.resize((size_t)h.n_quads * 5);
  h.spheres.resize((size_t)h.n_spheres * 2);
  h.quadrics.resize((size_t)h.n_quadrics * 5);
  CK(ctx, cudaMemcpyAsync(fi.data(), final_index, (size_t)n * 4, cudaMemcpyDeviceToHost, st));
  CK(ctx, cudaMemcpyAsync(h.nodes.data(), nodes, h.nodes.size() * 16, cudaMemcpyDeviceToHost, st));
  if (h.n_tris) {
    CK(ctx, cudaMemcpyAsync(h.tris.data(), tris, h.tris.size() * 16, cudaMemcpyDeviceToHost, st));
    CK(ctx, cudaMemcpyAsync(h.tri_normals.data(), normals, h.tri_normals.size() * 16, cudaMemcpyDeviceToHost, st));
  }
  if (h.n_quads) CK(ctx, cudaMemcpyAsync(h.quads.data(), quads, h.quads.size() * 16, cudaMemcpyDeviceToHost, st));
  if (h.n_spheres)
    CK(ctx, cudaMemcpyAsync(h.spheres.data(), spheres, h.spheres.size() * 16, cudaMemcpyDeviceToHost, st));
  if (h.n_quadrics)
    CK(ctx, cudaMemcpyAsync(h.quadrics.data(), quadrics, h.quadrics.size() * 16, cudaMemcpyDeviceToHost, st));
  CK(ctx, cudaStreamSynchronize(st));
  free_all(tmp);
  h.prim_shape.assign(n, 0);
  h.prim_sub.assign(n, 0);
  uint32_t base[4] = {0, h.n_tris, h.n_tris + h.n_quads, h.n_tris + h.n_quads + h.n_spheres};
  for (uint32_t k = 0; k < n; k++) {
    uint32_t type = 0;
    std::memcpy(&type, &bp.box[2 * k].w, 4);
    type &= 3u;
    uint32_t gid = base[type] + fi[k];
    h.prim_shape[gid] = bp.shape[k];
    h.prim_sub[gid] = bp.sub[k];
  }
  for (size_t i = 0; i < h.lights.size() && i < bp.light_prim.size(); i++)
    if (bp.light_prim[i] >= 0) h.lights[i].prim = (int)fi[bp.light_prim[i]];
  h.bvh_depth = levels;
  d.nodes = nodes;
  d.tris = tris;
  d.tri_normals = normals;
  d.quads = quads;
  d.spheres = spheres;
  d.quadrics = quadrics;
  h.pending = BuildPrims{};
  h.bvh_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  h.build_ms += h.bvh_ms;
  return GPRT_OK;
}

}  // namespace gprt
