// Context, scratch arena, prefix sum and the small host helpers of the C ABI.
#include <cstdlib>
#include <cstring>

#include "common.cuh"
#include "swap_heap.h"

namespace vnm {

vnm_status arena_reserve(vnm_ctx* ctx, size_t total) {
  ctx->arena.used = 0;
  if (total <= ctx->arena.cap) return VNM_OK;
  if (ctx->arena.base) {
    VNM_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    VNM_CUDA_TRY(cudaFree(ctx->arena.base));
    ctx->arena.base = nullptr;
    ctx->arena.cap = 0;
  }
  size_t cap = total + total / 4 + (1u << 20);
  void* p = nullptr;
  VNM_CUDA_TRY(cudaMalloc(&p, cap));
  ctx->arena.base = static_cast<char*>(p);
  ctx->arena.cap = cap;
  return VNM_OK;
}

vnm_status pinned_reserve(vnm_ctx* ctx, size_t ints) {
  if (ints <= ctx->h_pinned_cap) return VNM_OK;
  if (ctx->h_pinned) cudaFreeHost(ctx->h_pinned);
  ctx->h_pinned = nullptr;
  ctx->h_pinned_cap = 0;
  VNM_CUDA_TRY(cudaMallocHost(&ctx->h_pinned, ints * sizeof(int)));
  ctx->h_pinned_cap = ints;
  return VNM_OK;
}

vnm_status begin_call(vnm_ctx* ctx) {
  VNM_CUDA_TRY(cudaSetDevice(ctx->device));
  ctx->launches = 0;
  ctx->last_ms = 0.f;
  ctx->main_ms = 0.f;
  VNM_CUDA_TRY(cudaEventRecord(ctx->ev_start, ctx->stream));
  return VNM_OK;
}

vnm_status end_call(vnm_ctx* ctx) {
  VNM_CUDA_TRY(cudaEventRecord(ctx->ev_stop, ctx->stream));
  VNM_CUDA_TRY(cudaEventSynchronize(ctx->ev_stop));
  float ms = 0.f;
  VNM_CUDA_TRY(cudaEventElapsedTime(&ms, ctx->ev_start, ctx->ev_stop));
  ctx->last_ms = ms;
  return VNM_OK;
}

// ---------------------------------------------------------------------------
// Exclusive prefix sum: block-local scans of 2048 elements (one launch when
// that is all), then each block adds the sum of the tiles before it, read
// straight from the tile totals (up to 2048 tiles: two launches); longer
// arrays scan the tile totals recursively first.
// ---------------------------------------------------------------------------
constexpr int SCAN_NT = 512;
constexpr int SCAN_PER = 4;
constexpr int SCAN_TILE = SCAN_NT * SCAN_PER;

__device__ __forceinline__ int warp_incl_scan(int v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int t = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += t;
  }
  return v;
}

__global__ void __launch_bounds__(SCAN_NT) k_scan_tiles(const int* in, int* out, int n, int* tile_sums) {
  __shared__ int warp_tot[SCAN_NT / 32];
  const int base = blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_PER;
  int v[SCAN_PER];
  int s = 0;
#pragma unroll
  for (int q = 0; q < SCAN_PER; ++q) {
    int i = base + q;
    v[q] = i < n ? in[i] : 0;
    s += v[q];
  }
  int incl = warp_incl_scan(s);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 31) warp_tot[w] = incl;
  __syncthreads();
  if (w == 0) {
    int t = lane < SCAN_NT / 32 ? warp_tot[lane] : 0;
    t = warp_incl_scan(t);
    if (lane < SCAN_NT / 32) warp_tot[lane] = t;
  }
  __syncthreads();
  int run = incl - s + (w > 0 ? warp_tot[w - 1] : 0);
#pragma unroll
  for (int q = 0; q < SCAN_PER; ++q) {
    int i = base + q;
    if (i < n) out[i] = run;
    run += v[q];
  }
  if (threadIdx.x == SCAN_NT - 1) tile_sums[blockIdx.x] = run;
}

// Block b: add tiles 0 .. b-1's totals to its tile; the last block also
// writes the grand total.
__global__ void __launch_bounds__(SCAN_NT) k_scan_fix(int* out, int n, const int* tile_sums, int tiles, int* total) {
  __shared__ int warp_tot[SCAN_NT / 32];
  const int b = blockIdx.x;
  int s = 0;
  for (int t = threadIdx.x; t < b; t += SCAN_NT) s += tile_sums[t];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) warp_tot[threadIdx.x >> 5] = s;
  __syncthreads();
  int off = 0;
#pragma unroll
  for (int w = 0; w < SCAN_NT / 32; ++w) off += warp_tot[w];
  if (b > 0) {
    const int i = b * SCAN_TILE + threadIdx.x;
#pragma unroll
    for (int q = 0; q < SCAN_PER; ++q) {
      const int k = i + q * SCAN_NT;
      if (k < n) out[k] += off;
    }
  }
  if (total && b == tiles - 1 && threadIdx.x == 0) *total = off + tile_sums[b];
}

__global__ void k_scan_add(int* out, int n, const int* tile_off) {
  const int i = blockIdx.x * SCAN_TILE + threadIdx.x;
  const int add = tile_off[blockIdx.x];
#pragma unroll
  for (int q = 0; q < SCAN_PER; ++q) {
    int k = i + q * SCAN_NT;
    if (k < n) out[k] += add;
  }
}

__global__ void k_scan_total(const int* in_last, const int* out_last, int* total) {
  *total = *in_last + *out_last;
}

vnm_status exclusive_scan(vnm_ctx* ctx, const int* d_in, int* d_out, int n, int* d_total) {
  if (n <= 0) {
    if (d_total) VNM_CUDA_TRY(cudaMemsetAsync(d_total, 0, sizeof(int), ctx->stream));
    return VNM_OK;
  }
  const int ntiles = (n + SCAN_TILE - 1) / SCAN_TILE;
  if (ntiles <= SCAN_TILE) {  // up to 4 M elements: the tile scans, then one fix-up launch
    int* sums = arena_take<int>(ctx, ntiles);
    if (!sums) return VNM_ERR_NOMEM;
    VNM_LAUNCH(ctx, k_scan_tiles, ntiles, SCAN_NT, 0, d_in, d_out, n, sums);
    if (ntiles > 1 || d_total) VNM_LAUNCH(ctx, k_scan_fix, ntiles, SCAN_NT, 0, d_out, n, sums, ntiles, d_total);
    return VNM_OK;
  }
  // the last input is read back for the total before d_out may overwrite it
  int* last_in = arena_take<int>(ctx, 1);
  if (!last_in) return VNM_ERR_NOMEM;
  VNM_CUDA_TRY(cudaMemcpyAsync(last_in, d_in + n - 1, sizeof(int), cudaMemcpyDeviceToDevice, ctx->stream));
  const int tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
  int* sums = arena_take<int>(ctx, tiles);
  if (!sums) return VNM_ERR_NOMEM;
  VNM_LAUNCH(ctx, k_scan_tiles, tiles, SCAN_NT, 0, d_in, d_out, n, sums);
  if (tiles > 1) {
    VNM_TRY(exclusive_scan(ctx, sums, sums, tiles, nullptr));
    VNM_LAUNCH(ctx, k_scan_add, tiles, SCAN_NT, 0, d_out, n, sums);
  }
  if (d_total) VNM_LAUNCH(ctx, k_scan_total, 1, 1, 0, last_in, d_out + n - 1, d_total);
  return VNM_OK;
}

// upper bound of the arena scratch exclusive_scan takes for n elements
size_t scan_scratch_bytes(int n) {
  size_t b = arena_bytes((n + SCAN_TILE - 1) / SCAN_TILE + 1, sizeof(int));
  while (true) {
    b += arena_bytes(1, sizeof(int));
    int tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
    b += arena_bytes(tiles, sizeof(int));
    if (tiles <= 1) break;
    n = tiles;
  }
  return b;
}

}  // namespace vnm

extern "C" {

const char* vnm_status_string(vnm_status s) {
  switch (s) {
    case VNM_OK: return "ok";
    case VNM_ERR_ARG: return "invalid argument";
    case VNM_ERR_CUDA: return "CUDA runtime error";
    case VNM_ERR_UNSORTED: return "COO not sorted by (row, col) or has repeated entries";
    case VNM_ERR_RANGE: return "index out of range";
    case VNM_ERR_NOMEM: return "device allocation failed";
    case VNM_ERR_INTERNAL: return "internal invariant broken";
    case VNM_ERR_IO: return "file could not be read or written";
    case VNM_ERR_FORMAT: return "unsupported Matrix Market file";
    case VNM_ERR_NO_DEVICE: return "no usable CUDA device";
    case VNM_ERR_LIMIT: return "size above the documented maximum";
    default: return "unknown status";
  }
}

const char* vnm_version(void) { return "0.1.0 sm_103a"; }

vnm_status vnm_create(vnm_ctx** out, int device) {
  if (!out) return VNM_ERR_ARG;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) {
    (void)cudaGetLastError();
    return VNM_ERR_NO_DEVICE;
  }
  if (device < 0 || device >= n) return VNM_ERR_ARG;
  VNM_CUDA_TRY(cudaSetDevice(device));
  vnm_ctx* c = new vnm_ctx();
  c->device = device;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) {
    delete c;
    return VNM_ERR_CUDA;
  }
  c->num_sms = prop.multiProcessorCount;
  c->spare = new vnm_spmm_spare();
  c->spare->device = device;
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&c->ev_start) != cudaSuccess || cudaEventCreate(&c->ev_stop) != cudaSuccess ||
      cudaEventCreate(&c->ev_main0) != cudaSuccess || cudaEventCreate(&c->ev_main1) != cudaSuccess) {
    delete c;
    return VNM_ERR_CUDA;
  }
  *out = c;
  return VNM_OK;
}

vnm_status vnm_destroy(vnm_ctx* c) {
  if (!c) return VNM_ERR_ARG;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  if (c->arena.base) cudaFree(c->arena.base);
  if (c->h_pinned) cudaFreeHost(c->h_pinned);
  if (c->ev_start) cudaEventDestroy(c->ev_start);
  if (c->ev_stop) cudaEventDestroy(c->ev_stop);
  if (c->ev_main0) cudaEventDestroy(c->ev_main0);
  if (c->ev_main1) cudaEventDestroy(c->ev_main1);
  if (c->stream) cudaStreamDestroy(c->stream);
  if (c->spare) {
    bool last;
    {
      std::lock_guard<std::mutex> g(c->spare->m);
      if (c->spare->ptr) cudaFree(c->spare->ptr);
      c->spare->ptr = nullptr;
      c->spare->bytes = 0;
      c->spare->ctx_alive = false;
      last = --c->spare->refs == 0;
    }
    if (last) delete c->spare;
  }
  delete c;
  return VNM_OK;
}

float vnm_last_kernel_ms(const vnm_ctx* c) { return c ? c->last_ms : 0.f; }
int vnm_last_launch_count(const vnm_ctx* c) { return c ? c->launches : 0; }

float vnm_last_main_kernel_ms(const vnm_ctx* c) { return c ? c->main_ms : 0.f; }

vnm_status vnm_last_stats(const vnm_ctx* c, long long* out, int n) {
  if (!c || !out || n < 0) return VNM_ERR_ARG;
  for (int i = 0; i < n && i < 28; ++i) out[i] = c->stats[i];
  return VNM_OK;
}

vnm_status vnm_swap_heap_order(int n, const int* lg, const int* rg, int* order) {
  if (n < 0 || n > 255 || (n && (!lg || !rg || !order))) return VNM_ERR_ARG;
  int64_t key[256];
  uint8_t heap[256], ord[256];
  for (int i = 0; i < n; ++i) key[i] = swap_key(lg[i], rg[i]);
  swap_heap_pop_order(n, key, heap, ord);
  for (int i = 0; i < n; ++i) order[i] = ord[i];
  return VNM_OK;
}

}  // extern "C"
