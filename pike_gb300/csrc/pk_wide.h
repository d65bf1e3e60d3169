// pk_wide.h -- 8-wide compressed BVH (form (1)) collapsed from the binary SAH
// BVH, in the node format of Ylitie, Karras & Laine, "Efficient Incoherent
// Ray Traversal on GPUs Through Compressed Wide BVHs" (HPG 2017).
//
// Node record: 80 bytes = 5 x float4
//   [0] p.x, p.y, p.z (FP32 frame origin),
//       w = bytes {ex + 127, ey + 127, ez + 127, imask}
//   [1] x = child_base (index of the first internal child node),
//       y = tri_base (index of the first triangle record of the node's leaves),
//       z, w = meta[0..7], one byte per child slot:
//         internal child: 0b00100000 | slot  (imask bit set)
//         leaf child:     unary triangle count (0b001, 0b011, 0b111) << 5 | offset
//                         (its triangles are records tri_base + offset ...)
//         empty slot:     0
//   [2] qlo.x[8] qlo.y[8]   [3] qlo.z[8] qhi.x[8]   [4] qhi.y[8] qhi.z[8]
// Child box k on axis a: [p.a + 2^e.a * qlo.a[k], p.a + 2^e.a * qhi.a[k]].
// Internal children are stored contiguously from child_base in slot order, so
// the child in slot s is node child_base + popc(imask & ((1 << s) - 1)).
// Children sit in octant order: slot s holds the child that comes first for
// rays whose direction signs are the bits of s (bit 0: x < 0, 1: y, 2: z), so
// a ray of octant o visits its hit children in the order of (slot ^ o).
// Quantisation is rounded outward around boxes that enclose every triangle
// (its three vertices) with a margin of 2^-18 (times max(1, |x|)).
//
// Triangle records (both the wide BVH's own leaf order and the binary
// tree's), 48 bytes = 3 x float4: {v0.xyz, v1.x}, {v1.yz, v2.xy},
// {v2.z, slot bits, 0, 0}, where `slot` is the triangle's index in the binary
// BVH's leaf order (the index every hit record reports and ties break on).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "pk_util.h"

namespace pk {

constexpr int WIDE_NODE_FLOATS = 20;
constexpr int WIDE_TRI_FLOATS = 12;

// Built on the GPU (pk_wide.cu) from the breadth-first binary nodes (5 words
// each), the leaf-ordered {i0, i1, i2, matId} and the normalised vertices on
// the device.  Return 0 on success, non-zero with a reason otherwise.
//
// The compressed 8-wide BVH: nodes_out (5 float4 per node), tris_out (3
// float4 per triangle, in the wide BVH's own leaf order), the node count and
// the depth in wide levels.
int build_wide_bvh_gpu(cudaStream_t s, const int32_t* nodes5, uint32_t n_nodes, const int4* tri4, uint32_t n_tris,
                       const float4* verts4, uint32_t n_verts, DevBuf<float4>& nodes_out, DevBuf<float4>& tris_out,
                       uint32_t& n_wide, uint32_t& depth, std::string& why);

// The binary BVH's inner records (64-byte layout of the drop-in traversal:
// both children's boxes, then their child codes) with FP32 boxes rounded
// outward from the same vertex bounds and margin as the wide nodes, instead of
// the reference's inward-truncated snorm16 boxes, and the binary leaf order's
// triangle records in the format above.  Traversed with (t, slot) ties and
// slack in the box tests, closest hits equal brute force.
int build_exact_binary_gpu(cudaStream_t s, const int32_t* nodes5, uint32_t n_nodes, const int4* tri4,
                           uint32_t n_tris, const float4* verts4, uint32_t n_verts, DevBuf<float4>& records,
                           DevBuf<float4>& tris, int32_t& root_code, std::string& why);

}  // namespace pk
