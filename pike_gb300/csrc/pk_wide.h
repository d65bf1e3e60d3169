// pk_wide.h -- 8-wide compressed BVH collapsed from the binary SAH BVH.
//
// Node record: 96 bytes = 6 x float4
//   [0] p.x, p.y, p.z (FP32 frame origin), w = bytes {ex+127, ey+127, ez+127, valid mask}
//   [1] code[0..3]   [2] code[4..7]
//       code >= 0: index of an 8-wide child node
//       code <  0: 0x80000000 | size << 24 | base, a binary leaf's triangles
//                  (the same word the binary traversal uses)
//   [3] qlo.x[8] qlo.y[8]   [4] qlo.z[8] qhi.x[8]   [5] qhi.y[8] qhi.z[8]
// Child box k on axis a: [p.a + 2^e.a * qlo.a[k], p.a + 2^e.a * qhi.a[k]],
// evaluated as one FP32 multiply (exact) and one FP32 add.  Quantisation is
// rounded outward against that exact decode, around boxes that already
// enclose every triangle (v0, v0 + e1, v0 + e2 as the triangle test sees
// them) with a margin of 2^-18 (times max(1, |x|)), so no intersection the
// triangle test accepts lies outside its ancestors' boxes, even after the
// traversal folds the decode into its slab test (a few ulps of the frame's
// coordinates).
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace pk {

struct WideHost {
  std::vector<float> nodes;  // 24 floats per node
  uint32_t n_nodes = 0;
  uint32_t max_depth = 0;
};

// nodes5: binary BFS nodes (5 words each); tris: 12 floats per leaf triangle
// ({v0, e1, e2} as the traversal-format triangle records).  Returns 0 on
// success, non-zero with a reason otherwise.
int build_wide_bvh(const int32_t* nodes5, uint32_t n_nodes, const float* tris, uint32_t n_tris, WideHost& out,
                   std::string& why);

// The binary BVH's inner records (64-byte layout of the drop-in traversal:
// both children's boxes, then their child codes) with FP32 boxes rounded
// outward from the same triangle-record bounds and margin as the wide nodes,
// instead of the reference's inward-truncated snorm16 boxes.  Traversed with
// (t, slot) ties and slack in the box tests, closest hits equal brute force.
int build_exact_binary(const int32_t* nodes5, uint32_t n_nodes, const float* tris, uint32_t n_tris,
                       std::vector<float>& records, int32_t& root_code, std::string& why);

}  // namespace pk
