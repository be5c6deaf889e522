// Host BVH construction and device-layout conversion.
#pragma once

#include <stdint.h>

#include <string>
#include <vector>

namespace ct {

// Reference-layout records (byte-compatible with BVHNode / MBVHNode).
struct BinNode {  // 32 B: {min.xyz, leftFirst, max.xyz, count}
  float bmin[3];
  int32_t leftFirst;
  float bmax[3];
  int32_t count;
};
struct QuadNode {  // 128 B
  float bminx[4], bmaxx[4], bminy[4], bmaxy[4], bminz[4], bmaxz[4];
  int32_t childs[4], counts[4];
};
static_assert(sizeof(BinNode) == 32, "BinNode");
static_assert(sizeof(QuadNode) == 128, "QuadNode");

struct HostBVH {
  std::vector<BinNode> bin;    // empty when imported as a quad tree
  std::vector<QuadNode> quad;
  std::vector<uint32_t> prims;
  double build_ms = 0.0, collapse_ms = 0.0;
};

// Reference SAH build (BVHNode::SubdivideMT/Partition semantics) over float3
// vertices and uint3 indices; O(n) binning per node instead of the reference's
// thirty O(n) scans, with identical split choices and primitive order.
void build_binary(const float* verts, const uint32_t* idx, uint32_t ntri, int nthreads, HostBVH& out);
// MBVHNode::MergeNodes collapse of out.bin into out.quad (deterministic numbering).
void collapse_quad(HostBVH& out);
// Quad tree built for traversal speed (bvh_fast.cpp): padded-relative triangle
// boxes, 16-bin SAH to single triangles, cost-optimal four-wide collapse with
// leaves of at most four triangles. Fills out.quad and out.prims; out.bin stays
// empty.
void build_fast_quad(const float* verts, const uint32_t* idx, uint32_t ntri, int nthreads, HostBVH& out);
// The power-of-two scale of that build's surface-area costs, from the root box
// (shared with the device build, bvh_gpu_fast.cu).
float fast_area_scale(const float mn[3], const float mx[3]);
// Structural validation of an imported tree; returns "" when valid.
std::string validate_quad(const std::vector<QuadNode>& q, uint32_t prim_count);
std::string validate_binary(const std::vector<BinNode>& b, uint32_t prim_count);

struct DeviceLayout {
  std::vector<uint8_t> nodes;  // QNodeDev records
  std::vector<float> tris;     // 12 floats per leaf slot
  uint32_t leaf_shift = 0, first_mask = 0, count_mask = 0;
  uint32_t depth = 0, max_leaf = 0;
  int32_t stack_entries = 0;
};
// Leaf reference encoding for np primitives: first in the low `shift` bits,
// count above, bit 31 set. Returns "" or why a leaf of max_leaf primitives
// cannot be encoded.
std::string leaf_encoding(uint32_t np, uint32_t max_leaf, uint32_t& shift, uint32_t& first_mask, uint32_t& count_mask);
// Convert to the device layout; returns "" or an error message.
std::string to_device_layout(const HostBVH& h, const float* verts, const uint32_t* idx, uint32_t ntri,
                             DeviceLayout& out);

}  // namespace ct
