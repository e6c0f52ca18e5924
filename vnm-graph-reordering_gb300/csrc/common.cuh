// Shared definitions of libvnm_gb300: status handling, the context object,
// the device scratch arena and launch accounting.
#ifndef VNM_COMMON_CUH
#define VNM_COMMON_CUH

#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>
#include <vector>

#include "../../include/vnm_gb300.h"

#define VNM_CUDA_TRY(expr)                    \
  do {                                        \
    cudaError_t e_ = (expr);                  \
    if (e_ != cudaSuccess) {                  \
      (void)cudaGetLastError();               \
      return e_ == cudaErrorMemoryAllocation  \
                 ? VNM_ERR_NOMEM              \
                 : VNM_ERR_CUDA;              \
    }                                         \
  } while (0)

#define VNM_TRY(expr)          \
  do {                         \
    vnm_status s_ = (expr);    \
    if (s_ != VNM_OK) return s_; \
  } while (0)

// Launch with accounting; the kernel's launch error is checked right away.
#define VNM_LAUNCH(ctx, kernel, grid, block, smem, ...)                             \
  do {                                                                              \
    kernel<<<(grid), (block), (smem), (ctx)->stream>>>(__VA_ARGS__);                \
    (ctx)->launches++;                                                              \
    cudaError_t le_ = cudaGetLastError();                                           \
    if (le_ != cudaSuccess) return VNM_ERR_CUDA;                                    \
  } while (0)

// Grow-only device arena: one allocation reused by successive calls.
struct DeviceArena {
  char* base = nullptr;
  size_t cap = 0;
  size_t used = 0;
};

// Device storage of a freed SpMM operand, kept for the next compression on
// the same context (a compression then skips cudaMalloc, a free skips the
// device-wide synchronisation of cudaFree).  Shared by the context and every
// operand it compressed; whichever of them goes last frees it.
struct vnm_spmm_spare {
  std::mutex m;
  int device = 0;
  void* ptr = nullptr;
  size_t bytes = 0;
  int refs = 1;  // the context and its live operands
  bool ctx_alive = true;
};

struct vnm_ctx {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev_start = nullptr, ev_stop = nullptr;
  cudaEvent_t ev_main0 = nullptr, ev_main1 = nullptr;  // around the call's main kernel
  float last_ms = 0.f;
  float main_ms = 0.f;
  long long stats[28] = {0};  // work counters of the last call (vnm_last_stats)
  int last_clusters_fit = 0;  // clusters of the launched size the GPU can hold at once (occupancy query)
  int launches = 0;
  int last_cluster = 1;  // blocks per job of the last NM round launch
  // SpMM column-block widths measured fastest, by (rows, K-steps, B width)
  long long spmm_tune_key[8][3] = {};
  int spmm_tune_nt[8] = {};
  int spmm_tune_next = 0;
  DeviceArena arena;
  vnm_spmm_spare* spare = nullptr;
  // pinned staging for small results
  int* h_pinned = nullptr;
  size_t h_pinned_cap = 0;
  // swap trace of the last NM call (host copies)
  bool trace = false;
  bool phase_timing = false;  // the round kernel's per-phase timers (vnm_nm_set_phase_timing)
  std::vector<int> trace_pairs, trace_round_end;
};

namespace vnm {

// Reserve `bytes` (256-byte aligned) of the arena; valid until arena_reset.
vnm_status arena_reserve(vnm_ctx* ctx, size_t total_bytes);
template <class T>
inline T* arena_take(vnm_ctx* ctx, size_t count) {
  size_t bytes = (count * sizeof(T) + 255) & ~size_t(255);
  if (ctx->arena.used + bytes > ctx->arena.cap) return nullptr;
  T* p = reinterpret_cast<T*>(ctx->arena.base + ctx->arena.used);
  ctx->arena.used += bytes;
  return p;
}
inline size_t arena_bytes(size_t count, size_t elem) { return (count * elem + 255) & ~size_t(255); }

vnm_status begin_call(vnm_ctx* ctx);
vnm_status end_call(vnm_ctx* ctx);  // records the stop event and synchronises
vnm_status pinned_reserve(vnm_ctx* ctx, size_t ints);

// Copy a caller array to the device (or alias it when it already is there).
template <class T>
inline vnm_status stage_in(vnm_ctx* ctx, const T* src, size_t count, int mem, const T** dst) {
  if (mem == VNM_MEM_DEVICE) {
    *dst = src;
    return VNM_OK;
  }
  T* d = arena_take<T>(ctx, count);
  if (!d) return VNM_ERR_NOMEM;
  if (count) VNM_CUDA_TRY(cudaMemcpyAsync(d, src, count * sizeof(T), cudaMemcpyHostToDevice, ctx->stream));
  *dst = d;
  return VNM_OK;
}

// exclusive prefix sum of n ints (out may alias in); returns the total in
// *d_total (device).  Uses arena scratch.
vnm_status exclusive_scan(vnm_ctx* ctx, const int* d_in, int* d_out, int n, int* d_total);
size_t scan_scratch_bytes(int n);

// stable LSD radix sort of 64-bit keys (low `bits` bits) carrying int payloads
// (nullptr payload = original positions); see radix_sort.cu
vnm_status radix_sort_u64(vnm_ctx* ctx, const unsigned long long* keys, const int* vals, int n, int bits,
                          unsigned long long** out_keys, int** out_vals);
size_t radix_sort_scratch_bytes(int n);

// The nonzero-valued pattern of one square matrix on the device: entries
// with val != 0 in (row, col) order, the same entries by column (CSC), and
// the invalid / present row counts of each M-column segment.
struct Pattern {
  int R = 0, nseg = 0, np = 0;
  int* prow = nullptr;
  int* pcol = nullptr;
  int* cptr = nullptr;
  int* crow = nullptr;    // rows of each column, grouped by row group (nm_reorder.cu row_group)
  int* csplit = nullptr;  // [16 R + 1] start of each (column, row group) in crow
  int* inv0 = nullptr;
  int* pres0 = nullptr;
  int* d_err = nullptr;  // [2] on the device: the input check's flag (bit 1 unsorted, bit 2 out of range), np
};
size_t pattern_bytes(int R, int nnz);
// validates (row, col) order and range, then builds P in the arena;
// h_scratch: at least 2 pinned ints.  deferred: no host synchronisation;
// P.np is left -1, the check's flag and np stay in P.d_err[0..1] for the
// caller to read back, and the kernels skip their work on a flagged input.
vnm_status build_pattern(vnm_ctx* ctx, int R, int nnz, const int* d_row, const int* d_col, const float* d_val,
                         int N, int M, Pattern& P, int* h_scratch, bool deferred = false);

}  // namespace vnm

#endif
