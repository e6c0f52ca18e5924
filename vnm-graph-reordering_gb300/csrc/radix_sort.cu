// Stable LSD radix sort of 64-bit keys with a 32-bit payload.
//
// Used wherever the path needs an order the reference gets from std::sort or
// Python's sorted(): the (row, col) order of a COO (customSort,
// mtx/readMtx.hpp:56-82), the VNM row order (reordering.py:219) and the
// compressor's (block, segment) grouping.  Keys are unique or ties are
// broken by the payload's original position, so stability makes the result
// identical to the reference's.
//
// One pass per 8-bit digit: (1) per-tile digit histograms, (2) an exclusive
// scan over (digit, tile) in digit-major order, (3) a stable scatter in which
// every warp walks a contiguous chunk of its tile and ranks keys among equal
// digits with __match_any_sync.  Only the low `bits` bits of the keys are
// sorted on, so callers pack keys tightly to save passes.
#include "common.cuh"

namespace vnm {

constexpr int RS_NT = 256;           // threads per tile
constexpr int RS_PER = 8;            // keys per thread
constexpr int RS_TILE = RS_NT * RS_PER;
constexpr int RS_WARPS = RS_NT / 32;
constexpr int RS_CHUNK = RS_TILE / RS_WARPS;  // keys per warp, walked in order

__global__ void __launch_bounds__(RS_NT) k_rs_hist(const unsigned long long* keys, int n, int shift, int* hist,
                                                    int ntiles) {
  __shared__ int h[256];
  for (int i = threadIdx.x; i < 256; i += RS_NT) h[i] = 0;
  __syncthreads();
  const int base = blockIdx.x * RS_TILE;
  for (int q = threadIdx.x; q < RS_TILE; q += RS_NT) {
    const int i = base + q;
    if (i < n) atomicAdd(&h[(unsigned)(keys[i] >> shift) & 255u], 1);
  }
  __syncthreads();
  for (int d = threadIdx.x; d < 256; d += RS_NT) hist[d * ntiles + blockIdx.x] = h[d];
}

__global__ void __launch_bounds__(RS_NT) k_rs_scatter(const unsigned long long* keys, const int* vals, int n,
                                                       int shift, const int* offs, int ntiles,
                                                       unsigned long long* okeys, int* ovals) {
  __shared__ int wcount[RS_WARPS][256];  // per warp, per digit: keys of that digit in the warp's chunk
  __shared__ int tileoff[256];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int base = blockIdx.x * RS_TILE + w * RS_CHUNK;
  for (int d = lane; d < 256; d += 32) wcount[w][d] = 0;
  for (int d = threadIdx.x; d < 256; d += RS_NT) tileoff[d] = offs[d * ntiles + blockIdx.x];
  __syncwarp();
  // pass A: per-warp digit counts
  for (int q = 0; q < RS_CHUNK; q += 32) {
    const int i = base + q + lane;
    const bool ok = i < n;
    const unsigned d = ok ? (unsigned)(keys[i] >> shift) & 255u : 256u;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const int leader = __ffs(peers) - 1;
    if (ok && lane == leader) wcount[w][d] += __popc(peers);
    __syncwarp();
  }
  __syncthreads();
  // exclusive prefix over warps for each digit (warps before this one)
  for (int d = threadIdx.x; d < 256; d += RS_NT) {
    int run = 0;
    for (int k = 0; k < RS_WARPS; ++k) {
      const int c = wcount[k][d];
      wcount[k][d] = run;
      run += c;
    }
  }
  __syncthreads();
  // pass B: stable scatter
  for (int q = 0; q < RS_CHUNK; q += 32) {
    const int i = base + q + lane;
    const bool ok = i < n;
    const unsigned long long k = ok ? keys[i] : 0ull;
    const unsigned d = ok ? (unsigned)(k >> shift) & 255u : 256u;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const int rank = __popc(peers & ((1u << lane) - 1u));
    if (ok) {
      const int dst = tileoff[d] + wcount[w][d] + rank;
      okeys[dst] = k;
      ovals[dst] = vals ? vals[i] : i;
    }
    __syncwarp();
    const int leader = __ffs(peers) - 1;
    if (ok && lane == leader) wcount[w][d] += __popc(peers);
    __syncwarp();
  }
}

size_t radix_sort_scratch_bytes(int n) {
  const int ntiles = (n + RS_TILE - 1) / RS_TILE;
  size_t b = 2 * arena_bytes(n, sizeof(unsigned long long)) + 2 * arena_bytes(n, sizeof(int));
  b += 2 * arena_bytes((size_t)256 * ntiles, sizeof(int));
  b += scan_scratch_bytes(256 * ntiles);
  return b + 4096;
}

// Sort keys[0..n) ascending, carrying vals (nullptr = original positions).
// Results land in *out_keys / *out_vals (arena memory or the inputs).
// `bits` = number of low key bits that can be nonzero (<= 64).
vnm_status radix_sort_u64(vnm_ctx* ctx, const unsigned long long* keys, const int* vals, int n, int bits,
                          unsigned long long** out_keys, int** out_vals) {
  if (n <= 0) {
    *out_keys = const_cast<unsigned long long*>(keys);
    *out_vals = const_cast<int*>(vals);
    return VNM_OK;
  }
  const int ntiles = (n + RS_TILE - 1) / RS_TILE;
  unsigned long long* kb[2] = {arena_take<unsigned long long>(ctx, n), arena_take<unsigned long long>(ctx, n)};
  int* vb[2] = {arena_take<int>(ctx, n), arena_take<int>(ctx, n)};
  int* hist = arena_take<int>(ctx, (size_t)256 * ntiles);
  int* offs = arena_take<int>(ctx, (size_t)256 * ntiles);
  if (!kb[0] || !kb[1] || !vb[0] || !vb[1] || !hist || !offs) return VNM_ERR_NOMEM;
  const unsigned long long* ck = keys;
  const int* cv = vals;
  int cur = 0;
  for (int shift = 0; shift < bits; shift += 8) {
    VNM_LAUNCH(ctx, k_rs_hist, ntiles, RS_NT, 0, ck, n, shift, hist, ntiles);
    VNM_TRY(exclusive_scan(ctx, hist, offs, 256 * ntiles, nullptr));
    VNM_LAUNCH(ctx, k_rs_scatter, ntiles, RS_NT, 0, ck, cv, n, shift, offs, ntiles, kb[cur], vb[cur]);
    ck = kb[cur];
    cv = vb[cur];
    cur ^= 1;
  }
  *out_keys = const_cast<unsigned long long*>(ck);
  *out_vals = const_cast<int*>(cv);
  return VNM_OK;
}

}  // namespace vnm
