// pk_bvh.h -- GPU builder of the reference BVH (bvh.js sweep SAH + trace_pass.js packing).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <string>

#include "pk_util.h"

namespace pk {

struct BvhOut {
  DevBuf<int32_t> nodes5;   // BFS nodes, 5 words each (BVHNodeStruct)
  DevBuf<int4> tri4_leaf;   // leaf-ordered {i0, i1, i2, matId}
  DevBuf<float4> verts4;    // normalised positions (xyz, 0)
  DevBuf<double> node_box;  // exact double bounds per BFS node {min xyz, max xyz} (raycaster.js uses them)
  uint32_t n_nodes = 0, n_leaf_tris = 0, depth = 0, largest_leaf = 0;
  double norm[4] = {0, 0, 0, 0};  // centre xyz, scale = 2 / longest
};

// Level-synchronous rebuild of bvh.js:12-223 with identical topology and
// primitive order: per level, segmented prefix/suffix box scans give every
// sweep cost of #computeSplit, a segmented arg-min picks the first minimum in
// (axis, index) order, `cost > n` makes a leaf, and a stable partition of the
// other two axis orders forms the children.  Levels are emitted in BFS order,
// which is serializeTree's order.  Returns non-zero with a reason on failure.
int build_bvh_sweep(cudaStream_t s, const double* pos3, uint32_t n_verts, const int4* tri4, uint32_t n_tris,
                    BvhOut& out, std::string& why);

// Binned SAH (16 bins per axis, leaves of at most 8 triangles): a different,
// faster-to-build topology than bvh.js; same output layout.
int build_bvh_binned(cudaStream_t s, const double* pos3, uint32_t n_verts, const int4* tri4, uint32_t n_tris,
                     BvhOut& out, std::string& why);

}  // namespace pk
