// pk_util.h -- small host helpers: owned device buffers, device-wide scans and sorts.
#pragma once
#include <cuda_runtime.h>
#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

namespace pk {

struct CudaError : std::runtime_error {
  explicit CudaError(const std::string& s) : std::runtime_error(s) {}
};

inline void check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw CudaError(std::string(what) + ": " + cudaGetErrorString(e));
}

// Owned device allocation (cudaMalloc / cudaFree).
template <class T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  explicit DevBuf(size_t count) { alloc(count); }
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  DevBuf(DevBuf&& o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
  DevBuf& operator=(DevBuf&& o) noexcept {
    if (this != &o) { release(); p = o.p; n = o.n; o.p = nullptr; o.n = 0; }
    return *this;
  }
  ~DevBuf() { release(); }
  void alloc(size_t count) {
    release();
    n = count;
    if (count) check(cudaMalloc(&p, count * sizeof(T) > 0 ? count * sizeof(T) : 1), "cudaMalloc");
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  size_t bytes() const { return n * sizeof(T); }
};

// Exclusive prefix sum of n u32 values (in may alias out).  If total is not
// null it receives the sum (device pointer).  Counts must stay below 2^31.
void scan_exclusive_u32(cudaStream_t s, const uint32_t* in, uint32_t* out, uint32_t n, uint32_t* total);

// Exclusive prefix sum of n u64 values (in may alias out); returns after the
// stream has finished it.
void scan_exclusive_u64(cudaStream_t s, const unsigned long long* in, unsigned long long* out, size_t n);

// Stable LSD radix sort of (key, value) pairs by the low `bits` bits of the
// 64-bit keys, ascending.  Sorts in place using the given scratch buffers.
void radix_sort_pairs_u64(cudaStream_t s, uint64_t* keys, uint32_t* vals, uint64_t* keys_tmp, uint32_t* vals_tmp,
                          uint32_t n, int bits);

// The levels of a binary tree (nodes5: 5 words per node, word 0 the left
// child (the right child follows it), word 1 > -1 for a leaf; children after
// their parents): the nodes of depth d are order[level[d], level[d + 1]).
// Returns non-zero when the tree is malformed (a child not after its parent,
// or a node not reached exactly once).
int tree_levels(cudaStream_t s, const int32_t* nodes5, uint32_t n_nodes, DevBuf<uint32_t>& order,
                std::vector<uint32_t>& level);

// EnvironmentGenerator tables on the GPU (pk_env.cu).
int build_env_tables_gpu(cudaStream_t s, const uchar4* rgbe, uint32_t w, uint32_t h, DevBuf<int2>& bins_out,
                         uint32_t& nb_out, DevBuf<int2>& coords_out, DevBuf<float>& pdf_out, std::string& why);
// The same tables for an FP32 RGB map (w x h x 3): radiance = luma of the
// stored values in double (the differentiable renderer's sampling tables).
int build_env_tables_gpu_f32(cudaStream_t s, const float* rgb, uint32_t w, uint32_t h, DevBuf<int2>& bins_out,
                             uint32_t& nb_out, DevBuf<int2>& coords_out, DevBuf<float>& pdf_out, std::string& why);

// PK_ENV_ALIAS's alias table for a w x h RGBE image on the device (pk_env.cu):
// {keep threshold, alias} per texel and the pdf texture of the table's exact
// selection probabilities.  Returns non-zero with a reason on failure.
int build_env_alias_gpu(cudaStream_t s, const uchar4* rgbe, uint32_t w, uint32_t h, DevBuf<uint2>& table_out,
                        DevBuf<float>& pdf_out, std::string& why);

}  // namespace pk
