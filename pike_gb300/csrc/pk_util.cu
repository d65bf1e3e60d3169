// pk_util.cu -- device-wide exclusive scan (single pass, decoupled look-back)
// and a stable LSD radix sort of 64-bit keys, used by the BVH and env builders.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <utility>
#include <vector>

#include "pk_internal.cuh"
#include "pk_util.h"

namespace pk {

constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 8;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_u32(const uint32_t* in, uint32_t* out,
                                                          uint32_t n, uint32_t* __restrict__ total,
                                                          unsigned long long* __restrict__ tiles,
                                                          uint32_t* __restrict__ ticket, uint32_t* __restrict__ err) {
  __shared__ uint32_t s_tile;
  __shared__ uint32_t s_warp[SCAN_THREADS / 32 + 1][2];
  __shared__ unsigned long long s_excl;
  const uint32_t ntiles = (n + SCAN_TILE - 1) / SCAN_TILE;
  for (;;) {
    if (threadIdx.x == 0) s_tile = atomicAdd(ticket, 1u);
    __syncthreads();
    const uint32_t tile = s_tile;
    if (tile >= ntiles) break;
    const size_t base = (size_t)tile * SCAN_TILE + (size_t)threadIdx.x * SCAN_ITEMS;
    uint32_t v[SCAN_ITEMS];
    uint32_t sum = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
      v[k] = (base + k < n) ? in[base + k] : 0u;
      sum += v[k];
    }
    uint32_t ea, eb, ta, tb;
    block_scan2<SCAN_THREADS / 32>(sum, 0u, ea, eb, ta, tb, s_warp);
    if (threadIdx.x == 0) s_excl = lookback2(tiles, tile, pack2(ta, 0u), err);
    __syncthreads();
    uint32_t run = unpack_a(s_excl) + ea;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
      if (base + k < n) out[base + k] = run;
      run += v[k];
    }
    if (tile == ntiles - 1 && threadIdx.x == 0 && total) *total = unpack_a(s_excl) + ta;
    __syncthreads();
  }
}

void scan_exclusive_u32(cudaStream_t s, const uint32_t* in, uint32_t* out, uint32_t n, uint32_t* total) {
  if (n == 0) {
    if (total) check(cudaMemsetAsync(total, 0, 4, s), "memset");
    return;
  }
  const uint32_t ntiles = (n + SCAN_TILE - 1) / SCAN_TILE;
  DevBuf<unsigned long long> tiles(ntiles);
  DevBuf<uint32_t> aux(2);  // ticket, err
  check(cudaMemsetAsync(tiles.p, 0, tiles.bytes(), s), "memset");
  check(cudaMemsetAsync(aux.p, 0, aux.bytes(), s), "memset");
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  unsigned grid = (unsigned)std::min<uint32_t>(ntiles, (uint32_t)sms * 4u);
  k_scan_u32<<<grid, SCAN_THREADS, 0, s>>>(in, out, n, total, tiles.p, aux.p, aux.p + 1);
  check(cudaGetLastError(), "k_scan_u32");
  uint32_t err = 0;
  check(cudaMemcpyAsync(&err, aux.p + 1, 4, cudaMemcpyDeviceToHost, s), "memcpy");
  check(cudaStreamSynchronize(s), "scan sync");
  if (err) throw CudaError("scan_exclusive_u32: look-back timed out");
}

// ---------------- exclusive scan of u64 values (three phases) ---------------
// Tiles of SCAN_TILE values: each block scans its tile and writes the tile's
// sum; the tile sums are scanned recursively; a last pass adds each tile's
// offset.  Integer sums, so the result does not depend on the grouping.
__device__ __forceinline__ unsigned long long warp_scan_incl_u64(unsigned long long v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned long long x = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += x;
  }
  return v;
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_u64_tiles(const unsigned long long* in,
                                                                unsigned long long* out, size_t n,
                                                                unsigned long long* __restrict__ tile_sums) {
  __shared__ unsigned long long s_warp[SCAN_THREADS / 32];
  const size_t base = (size_t)blockIdx.x * SCAN_TILE + (size_t)threadIdx.x * SCAN_ITEMS;
  unsigned long long v[SCAN_ITEMS], sum = 0;
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; k++) {
    v[k] = base + k < n ? in[base + k] : 0ull;
    sum += v[k];
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned long long incl = warp_scan_incl_u64(sum);
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  unsigned long long woff = 0, tot = 0;
  for (int k = 0; k < SCAN_THREADS / 32; k++) {
    if (k < warp) woff += s_warp[k];
    tot += s_warp[k];
  }
  unsigned long long run = woff + incl - sum;
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; k++) {
    if (base + k < n) out[base + k] = run;
    run += v[k];
  }
  if (threadIdx.x == 0) tile_sums[blockIdx.x] = tot;
}

__global__ void k_scan_u64_add(unsigned long long* out, size_t n, const unsigned long long* __restrict__ tile_offs) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] += tile_offs[i / SCAN_TILE];
}

void scan_exclusive_u64(cudaStream_t s, const unsigned long long* in, unsigned long long* out, size_t n) {
  if (n == 0) return;
  const size_t ntiles = (n + SCAN_TILE - 1) / SCAN_TILE;
  DevBuf<unsigned long long> sums(ntiles);
  k_scan_u64_tiles<<<(unsigned)ntiles, SCAN_THREADS, 0, s>>>(in, out, n, sums.p);
  check(cudaGetLastError(), "k_scan_u64_tiles");
  if (ntiles > 1) {
    scan_exclusive_u64(s, sums.p, sums.p, ntiles);
    k_scan_u64_add<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(out, n, sums.p);
    check(cudaGetLastError(), "k_scan_u64_add");
  }
  check(cudaStreamSynchronize(s), "scan sync");  // the tile sums are freed on return
}

// ---------------- stable LSD radix sort -------------------------------------
constexpr int SORT_THREADS = 256;
constexpr int SORT_WARPS = SORT_THREADS / 32;
constexpr int SORT_ROUNDS = 16;                       // rounds of 32 keys per warp
constexpr int SORT_TILE = SORT_THREADS * SORT_ROUNDS; // 4096 keys per block
constexpr int RADIX = 256;

__global__ void __launch_bounds__(SORT_THREADS) k_sort_hist(const uint64_t* __restrict__ keys, uint32_t n, int shift,
                                                            uint32_t nblocks, uint32_t* __restrict__ hist) {
  __shared__ uint32_t h[RADIX];
  for (int i = threadIdx.x; i < RADIX; i += SORT_THREADS) h[i] = 0;
  __syncthreads();
  const size_t base = (size_t)blockIdx.x * SORT_TILE;
  for (int k = threadIdx.x; k < SORT_TILE; k += SORT_THREADS) {
    const size_t i = base + k;
    if (i < n) atomicAdd(&h[(uint32_t)(keys[i] >> shift) & 0xffu], 1u);
  }
  __syncthreads();
  for (int d = threadIdx.x; d < RADIX; d += SORT_THREADS) hist[(size_t)d * nblocks + blockIdx.x] = h[d];
}

__global__ void __launch_bounds__(SORT_THREADS) k_sort_scatter(const uint64_t* __restrict__ keys,
                                                               const uint32_t* __restrict__ vals, uint32_t n, int shift,
                                                               uint32_t nblocks, const uint32_t* __restrict__ offs,
                                                               uint64_t* __restrict__ keys_out,
                                                               uint32_t* __restrict__ vals_out) {
  __shared__ uint32_t wh[SORT_WARPS][RADIX];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int i = threadIdx.x; i < SORT_WARPS * RADIX; i += SORT_THREADS) (&wh[0][0])[i] = 0;
  __syncthreads();
  const size_t wbase = (size_t)blockIdx.x * SORT_TILE + (size_t)warp * (SORT_ROUNDS * 32);
  const uint32_t lt = (1u << lane) - 1u;
  uint32_t rank[SORT_ROUNDS];
  uint32_t dig[SORT_ROUNDS];
#pragma unroll
  for (int r = 0; r < SORT_ROUNDS; r++) {
    const size_t i = wbase + (size_t)r * 32 + lane;
    const uint32_t d = i < n ? ((uint32_t)(keys[i] >> shift) & 0xffu) : RADIX;
    const uint32_t peers = __match_any_sync(0xffffffffu, d);
    uint32_t pre = 0;
    if (d < RADIX) pre = wh[warp][d];
    __syncwarp();
    rank[r] = pre + (uint32_t)__popc(peers & lt);
    dig[r] = d;
    if (d < RADIX && (peers & lt) == 0) wh[warp][d] = pre + (uint32_t)__popc(peers);
    __syncwarp();
  }
  __syncthreads();
  // per digit: exclusive prefix over warps (in place)
  for (int d = threadIdx.x; d < RADIX; d += SORT_THREADS) {
    uint32_t run = 0;
    for (int w = 0; w < SORT_WARPS; w++) {
      const uint32_t c = wh[w][d];
      wh[w][d] = run;
      run += c;
    }
  }
  __syncthreads();
#pragma unroll
  for (int r = 0; r < SORT_ROUNDS; r++) {
    const size_t i = wbase + (size_t)r * 32 + lane;
    if (i >= n) continue;
    const uint32_t d = dig[r];
    const uint32_t pos = offs[(size_t)d * nblocks + blockIdx.x] + wh[warp][d] + rank[r];
    keys_out[pos] = keys[i];
    vals_out[pos] = vals[i];
  }
}

void radix_sort_pairs_u64(cudaStream_t s, uint64_t* keys, uint32_t* vals, uint64_t* keys_tmp, uint32_t* vals_tmp,
                          uint32_t n, int bits) {
  if (n <= 1) return;
  const uint32_t nblocks = (n + SORT_TILE - 1) / SORT_TILE;
  DevBuf<uint32_t> hist((size_t)RADIX * nblocks);
  uint64_t* kin = keys;
  uint32_t* vin = vals;
  uint64_t* kout = keys_tmp;
  uint32_t* vout = vals_tmp;
  const int passes = (bits + 7) / 8;
  for (int p = 0; p < passes; p++) {
    const int shift = 8 * p;
    k_sort_hist<<<nblocks, SORT_THREADS, 0, s>>>(kin, n, shift, nblocks, hist.p);
    scan_exclusive_u32(s, hist.p, hist.p, (uint32_t)hist.n, nullptr);
    k_sort_scatter<<<nblocks, SORT_THREADS, 0, s>>>(kin, vin, n, shift, nblocks, hist.p, kout, vout);
    check(cudaGetLastError(), "radix sort");
    std::swap(kin, kout);
    std::swap(vin, vout);
  }
  if (kin != keys) {
    check(cudaMemcpyAsync(keys, kin, (size_t)n * 8, cudaMemcpyDeviceToDevice, s), "memcpy");
    check(cudaMemcpyAsync(vals, vin, (size_t)n * 4, cudaMemcpyDeviceToDevice, s), "memcpy");
  }
}

// ---- levels of a binary tree ------------------------------------------------
// order[b, e) lists the nodes of one level (any order within it); the
// children of its inner nodes, in that order, form the next level.
__global__ void k_level_flags(const int32_t* __restrict__ nodes5, const uint32_t* __restrict__ order, uint32_t b,
                              uint32_t e, uint32_t* __restrict__ flag) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (b + k >= e) return;
  flag[k] = nodes5[5 * (size_t)order[b + k] + 1] <= -1 ? 1u : 0u;
}
__global__ void k_level_children(const int32_t* __restrict__ nodes5, uint32_t* __restrict__ order, uint32_t b,
                                 uint32_t e, const uint32_t* __restrict__ rank, uint32_t n_nodes, uint32_t* err) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (b + k >= e) return;
  const uint32_t node = order[b + k];
  const int32_t* nd = nodes5 + 5 * (size_t)node;
  if (nd[1] > -1) return;
  const int32_t l = nd[0];
  if (l <= (int32_t)node || (uint32_t)l + 1 >= n_nodes) {  // children must come after their parent
    atomicOr(err, 1u);
    return;
  }
  order[e + 2 * rank[k]] = (uint32_t)l;
  order[e + 2 * rank[k] + 1] = (uint32_t)l + 1;
}

int tree_levels(cudaStream_t s, const int32_t* nodes5, uint32_t n_nodes, DevBuf<uint32_t>& order,
                std::vector<uint32_t>& level) {
  order.alloc(std::max<uint32_t>(n_nodes, 1u));
  check(cudaMemsetAsync(order.p, 0, 4, s), "memset");  // the root
  DevBuf<uint32_t> flag(std::max<uint32_t>(n_nodes, 1u)), tot(1), err(1);
  check(cudaMemsetAsync(err.p, 0, 4, s), "memset");
  level.assign(1, 0u);
  uint32_t b = 0, e = n_nodes ? 1u : 0u;
  uint32_t c = 0;
  while (b < e) {
    level.push_back(e);
    const unsigned blocks = (e - b + 127) / 128;
    k_level_flags<<<blocks, 128, 0, s>>>(nodes5, order.p, b, e, flag.p);
    scan_exclusive_u32(s, flag.p, flag.p, e - b, tot.p);
    check(cudaMemcpyAsync(&c, tot.p, 4, cudaMemcpyDeviceToHost, s), "D2H");
    check(cudaStreamSynchronize(s), "sync");
    const uint64_t next_end = (uint64_t)e + 2ull * c;
    if (next_end > n_nodes) return 1;
    k_level_children<<<blocks, 128, 0, s>>>(nodes5, order.p, b, e, flag.p, n_nodes, err.p);
    b = e;
    e = (uint32_t)next_end;
  }
  uint32_t herr = 0;
  check(cudaMemcpyAsync(&herr, err.p, 4, cudaMemcpyDeviceToHost, s), "D2H");
  check(cudaStreamSynchronize(s), "sync");
  return (e != n_nodes || herr) ? 1 : 0;
}

}  // namespace pk
