// VNM stage on the GPU: the row sort of reordering.py, rebuilt.
//
// The reference runs this stage as a Python subprocess (main.cu:116-153) over
// strings: it builds an M-character bit string per (row, segment)
// (generate_segmat, reordering.py:113-119), hashes each to its index in the
// reflected Gray code, negated when it has more than two ones
// (construct_bitcode_hash_tab, :95-107), stable-sorts the rows by the tuple
// of their hashes (:219), maps row -> new_id[row] and col -> new_id[col]
// with new_id[i] = sorted[i] (:223-229, :171-177), recounts the V-blocks
// whose OR has more than four ones (and, strictly, blocks with a row of more
// than two ones) (:125-152), and stops when the count grows (:242-246).
//
// Here every round is a handful of kernels over the COO:
//   1. radix-sort the entries by (row, col)                       -> groups
//   2. group bits, Gray-code hash, one sortable token per group
//   3. V-block counts with a dense OR table (blocks x segments bytes)
//   4. the row order: rows compared as token strings, ties kept in index
//      order.  Done by refinement: sort rows by (group of the previous
//      pass, k-th token) with the stable radix sort until no group of equal
//      rows can still be split.
// Token order: comparing the dense hash tuples of two rows is the same as
// comparing their lists of (segment, hash) tokens, where token (s, h) ranks
// by  h > 0: +(nseg - s),  h < 0: -(nseg - s),  end of row: 0, then by h.
#include <cstring>
#include <vector>

#include "common.cuh"

namespace vnm {

constexpr int VS_NT = 256;

static inline int vs_grid(const vnm_ctx* ctx, long long n) {
  long long g = (n + VS_NT - 1) / VS_NT, cap = (long long)ctx->num_sms * 16;
  if (g > cap) g = cap;
  return g < 1 ? 1 : (int)g;
}

static inline int bits_for(long long v) {  // bits to hold 0..v
  int b = 1;
  while ((1ll << b) <= v) ++b;
  return b;
}

__global__ void k_vs_keys(const int* row, const int* col, int nnz, int colbits, unsigned long long* keys) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nnz; i += gridDim.x * blockDim.x)
    keys[i] = ((unsigned long long)(unsigned)row[i] << colbits) | (unsigned)col[i];
}

// group heads among (row, col)-sorted keys: a new (row, col / M) pair
__global__ void k_vs_heads(const unsigned long long* keys, int nnz, int colbits, int M, int* flag) {
  const unsigned long long cmask = (1ull << colbits) - 1;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nnz; i += gridDim.x * blockDim.x) {
    const unsigned long long k = keys[i];
    int f = 1;
    if (i > 0) {
      const unsigned long long p = keys[i - 1];
      f = ((p >> colbits) != (k >> colbits)) || ((int)(p & cmask) / M != (int)(k & cmask) / M);
    }
    flag[i] = f;
  }
}

__device__ __forceinline__ int gray_rank(unsigned code) {  // index of `code` in the reflected Gray code list
  unsigned idx = code;
  idx ^= idx >> 1;
  idx ^= idx >> 2;
  idx ^= idx >> 4;
  idx ^= idx >> 8;
  return (int)idx;
}

// One group per head: bits (offset k at bit M-1-k, as int(segmat, 2)),
// the token, and the row.  Also the V-block OR table and the strict flags.
__global__ void k_vs_groups(const unsigned long long* keys, const int* gpos, int nnz, int colbits, int M, int nseg,
                            int V, int* grow, int* gseg, unsigned* gtok, unsigned* ortab, unsigned* badtab) {
  const unsigned long long cmask = (1ull << colbits) - 1;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nnz; i += gridDim.x * blockDim.x) {
    const unsigned long long k = keys[i];
    const int r = (int)(k >> colbits), c = (int)(k & cmask), s = c / M;
    if (i > 0) {
      const unsigned long long p = keys[i - 1];
      if ((int)(p >> colbits) == r && (int)(p & cmask) / M == s) continue;  // not a head
    }
    unsigned bits = 0;
    for (int q = 0; q < M && i + q < nnz; ++q) {
      const unsigned long long kk = keys[i + q];
      if ((int)(kk >> colbits) != r || (int)(kk & cmask) / M != s) break;
      bits |= 1u << (M - 1 - (int)(kk & cmask) % M);
    }
    const int pc = __popc(bits);
    const int g = gpos[i];
    const int h = pc <= 2 ? gray_rank(bits) : -gray_rank(bits);
    const int rank = h > 0 ? (nseg - s) : -(nseg - s);
    grow[g] = r;
    gseg[g] = s;
    gtok[g] = ((unsigned)(rank + nseg) << 9) | (unsigned)(h + 256);
    const long long cell = (long long)(r / V) * nseg + s;
    atomicOr(&ortab[cell >> 2], bits << ((cell & 3) * 8));
    if (pc > 2) atomicOr(&badtab[cell >> 2], 1u << ((cell & 3) * 8));
  }
}

__global__ void k_vs_count(const unsigned* ortab, const unsigned* badtab, long long ncells, int* out2) {
  int inv = 0, strict = 0;
  for (long long w = blockIdx.x * (long long)blockDim.x + threadIdx.x; w < (ncells + 3) / 4;
       w += (long long)gridDim.x * blockDim.x) {
    const unsigned o = ortab[w], b = badtab[w];
    for (int q = 0; q < 4; ++q) {
      if (w * 4 + q >= ncells) break;
      const unsigned ob = (o >> (8 * q)) & 0xffu;
      const bool a = __popc(ob) > 4;
      inv += a;
      strict += a || ((b >> (8 * q)) & 0xffu);
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    inv += __shfl_xor_sync(0xffffffffu, inv, o);
    strict += __shfl_xor_sync(0xffffffffu, strict, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&out2[0], inv);
    atomicAdd(&out2[1], strict);
  }
}

// first group of each row (groups are sorted by row)
__global__ void k_vs_rowptr(const int* grow, int ng, int m, int* rowptr) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r <= m; r += gridDim.x * blockDim.x) {
    int lo = 0, hi = ng;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (grow[mid] < r) lo = mid + 1;
      else hi = mid;
    }
    rowptr[r] = lo;
  }
}

__global__ void k_vs_iota(int* a, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) a[i] = i;
}

// keys for refinement pass k over rows in the current order:
// (group start << tokbits) | token_k ; rows that are settled keep token 0
__global__ void k_vs_refine_keys(const int* order, const int* gstart, const unsigned char* settled,
                                 const int* rowptr, const unsigned* gtok, int m, int k, int nseg, int tokbits,
                                 unsigned long long* keys, int* active) {
  const unsigned endtok = ((unsigned)nseg << 9) | 256u;
  int act = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
    const int r = order[i];
    unsigned tok = 0;
    if (!settled[i]) {
      const int g = rowptr[r] + k;
      tok = g < rowptr[r + 1] ? gtok[g] : endtok;
      act = 1;
    }
    keys[i] = ((unsigned long long)(unsigned)gstart[i] << tokbits) | tok;
  }
  if (__syncthreads_or(act) && threadIdx.x == 0) atomicOr(active, 1);
}

// after sorting by (group start, token): new group starts and settled flags.
// A row is settled when it is alone in its new group, or its token was the
// end of its row (all rows of the group are then equal).
__global__ void k_vs_regroup(const unsigned long long* skeys, const int* spos, const int* old_order, int m,
                             int tokbits, int nseg, int* new_order, int* head) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
    new_order[i] = old_order[spos[i]];
    head[i] = (i == 0 || skeys[i] != skeys[i - 1]) ? i : 0;
  }
}

__global__ void k_vs_settle(const unsigned long long* skeys, const int* gstart_new, int m, int tokbits, int nseg,
                            unsigned char* settled) {
  const unsigned endtok = ((unsigned)nseg << 9) | 256u;
  const unsigned long long tmask = (1ull << tokbits) - 1;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
    const int g = gstart_new[i];
    const bool alone = (i == g) && (i + 1 == m || gstart_new[i + 1] != g);
    const unsigned tok = (unsigned)(skeys[i] & tmask);
    settled[i] = alone || tok == endtok || tok == 0u;
  }
}

// inclusive max-scan of head positions -> group start of every position
__global__ void k_vs_maxscan_block(int* a, int n, int* blockmax) {
  __shared__ int s[1024];
  const int i = blockIdx.x * 1024 + threadIdx.x;
  int v = i < n ? a[i] : 0;
  s[threadIdx.x] = v;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {
    int t = threadIdx.x >= o ? s[threadIdx.x - o] : 0;
    __syncthreads();
    if (t > s[threadIdx.x]) s[threadIdx.x] = t;
    __syncthreads();
  }
  if (i < n) a[i] = s[threadIdx.x];
  if (threadIdx.x == 1023) blockmax[blockIdx.x] = s[1023];
}

__global__ void k_vs_maxscan_fix(int* a, int n, const int* blockmax) {
  const int b = blockIdx.x;
  if (b == 0) return;
  int carry = 0;
  for (int q = 0; q < b; ++q) carry = max(carry, blockmax[q]);
  const int i = b * 1024 + threadIdx.x;
  if (i < n && a[i] < carry) a[i] = carry;
}

__global__ void k_vs_apply(int* row, int* col, int nnz, const int* new_id) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nnz; i += gridDim.x * blockDim.x) {
    row[i] = new_id[row[i]];
    col[i] = new_id[col[i]];
  }
}

__global__ void k_vs_compose(int* comp, int m, const int* new_id) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) comp[i] = new_id[comp[i]];
}

struct VnmWork {
  int m, nnz, M, V, nseg, nblk, colbits, tokbits;
  long long ncells;
  // arena buffers
  unsigned long long* keys;
  int* flag;
  int* grow;
  int* gseg;
  unsigned* gtok;
  int* rowptr;
  unsigned* ortab;
  unsigned* badtab;
  int* counts;   // [2]
  int* order;    // [m]
  int* order2;   // [m]
  int* gstart;   // [m]
  unsigned char* settled;
  unsigned long long* rkeys;
  int* active;
  int* blockmax;
  int ng;
};

// Groups, tokens and counts of the current matrix (row, col) -> W.counts.
static vnm_status vnm_analyse(vnm_ctx* ctx, const int* row, const int* col, VnmWork& W, int* h2) {
  const int nnz = W.nnz;
  const size_t mark = ctx->arena.used;  // sort buffers are released at the end
  VNM_CUDA_TRY(cudaMemsetAsync(W.counts, 0, 2 * sizeof(int), ctx->stream));
  VNM_CUDA_TRY(cudaMemsetAsync(W.ortab, 0, ((W.ncells + 3) / 4) * 4, ctx->stream));
  VNM_CUDA_TRY(cudaMemsetAsync(W.badtab, 0, ((W.ncells + 3) / 4) * 4, ctx->stream));
  W.ng = 0;
  if (nnz > 0) {
    VNM_LAUNCH(ctx, k_vs_keys, vs_grid(ctx, nnz), VS_NT, 0, row, col, nnz, W.colbits, W.keys);
    unsigned long long* sk;
    int* sv;
    VNM_TRY(radix_sort_u64(ctx, W.keys, nullptr, nnz, 2 * W.colbits, &sk, &sv));
    VNM_LAUNCH(ctx, k_vs_heads, vs_grid(ctx, nnz), VS_NT, 0, sk, nnz, W.colbits, W.M, W.flag);
    int* d_ng = arena_take<int>(ctx, 1);
    if (!d_ng) return VNM_ERR_NOMEM;
    VNM_TRY(exclusive_scan(ctx, W.flag, W.flag, nnz, d_ng));
    VNM_LAUNCH(ctx, k_vs_groups, vs_grid(ctx, nnz), VS_NT, 0, sk, W.flag, nnz, W.colbits, W.M, W.nseg, W.V, W.grow,
               W.gseg, W.gtok, W.ortab, W.badtab);
    VNM_CUDA_TRY(cudaMemcpyAsync(h2 + 2, d_ng, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  }
  VNM_LAUNCH(ctx, k_vs_count, vs_grid(ctx, (W.ncells + 3) / 4), VS_NT, 0, W.ortab, W.badtab, W.ncells, W.counts);
  VNM_CUDA_TRY(cudaMemcpyAsync(h2, W.counts, 2 * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  VNM_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  if (nnz > 0) W.ng = h2[2];
  ctx->arena.used = mark;
  return VNM_OK;
}

static vnm_status maxscan(vnm_ctx* ctx, int* a, int n, int* blockmax) {
  const int nb = (n + 1023) / 1024;
  VNM_LAUNCH(ctx, k_vs_maxscan_block, nb, 1024, 0, a, n, blockmax);
  if (nb > 1) VNM_LAUNCH(ctx, k_vs_maxscan_fix, nb, 1024, 0, a, n, blockmax);
  return VNM_OK;
}

// The stable row order of reordering.py:219 for the analysed matrix.
static vnm_status vnm_row_order(vnm_ctx* ctx, VnmWork& W, int* h) {
  const int m = W.m;
  VNM_LAUNCH(ctx, k_vs_rowptr, vs_grid(ctx, m + 1), VS_NT, 0, W.grow, W.ng, m, W.rowptr);
  VNM_LAUNCH(ctx, k_vs_iota, vs_grid(ctx, m), VS_NT, 0, W.order, m);
  VNM_CUDA_TRY(cudaMemsetAsync(W.gstart, 0, sizeof(int) * m, ctx->stream));
  VNM_CUDA_TRY(cudaMemsetAsync(W.settled, 0, m, ctx->stream));
  const int keybits = W.tokbits + bits_for(m);
  for (int k = 0; k <= m; ++k) {  // at most one pass per token of the longest row
    VNM_CUDA_TRY(cudaMemsetAsync(W.active, 0, sizeof(int), ctx->stream));
    VNM_LAUNCH(ctx, k_vs_refine_keys, vs_grid(ctx, m), VS_NT, 0, W.order, W.gstart, W.settled, W.rowptr, W.gtok, m,
               k, W.nseg, W.tokbits, W.rkeys, W.active);
    VNM_CUDA_TRY(cudaMemcpyAsync(h, W.active, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    VNM_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    if (!h[0]) break;
    const size_t mark = ctx->arena.used;
    unsigned long long* sk;
    int* sp;
    VNM_TRY(radix_sort_u64(ctx, W.rkeys, nullptr, m, keybits, &sk, &sp));
    VNM_LAUNCH(ctx, k_vs_regroup, vs_grid(ctx, m), VS_NT, 0, sk, sp, W.order, m, W.tokbits, W.nseg, W.order2,
               W.gstart);
    VNM_TRY(maxscan(ctx, W.gstart, m, W.blockmax));
    VNM_LAUNCH(ctx, k_vs_settle, vs_grid(ctx, m), VS_NT, 0, sk, W.gstart, m, W.tokbits, W.nseg, W.settled);
    std::swap(W.order, W.order2);
    VNM_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    ctx->arena.used = mark;  // the sort's buffers are free again
  }
  return VNM_OK;
}

static size_t vnm_bytes(int m, int nnz, long long ncells) {
  size_t b = arena_bytes(nnz, 8) + arena_bytes(nnz, 4) * 3 + arena_bytes(nnz, 4) + arena_bytes(m + 1, 4);
  b += 2 * arena_bytes((ncells + 3) / 4, 4) + arena_bytes(2, 4);
  b += 4 * arena_bytes(m, 4) + arena_bytes(m, 1) + arena_bytes(m, 8) + arena_bytes(1, 4) +
       arena_bytes(m / 1024 + 2, 4);
  b += radix_sort_scratch_bytes(nnz > m ? nnz : m) + scan_scratch_bytes(nnz > 0 ? nnz : 1) + 4096;
  // per-round copies of the matrix and the composed map
  b += 4 * arena_bytes(nnz, 4) + 3 * arena_bytes(m, 4);
  return b;
}

static vnm_status vnm_setup(vnm_ctx* ctx, int m0, int n0, int nnz, int M, int V, VnmWork& W) {
  const int m = (m0 + M - 1) / M * M, n = (n0 + M - 1) / M * M;  // reordering.py:50-51
  W.m = m;
  W.nnz = nnz;
  W.M = M;
  W.V = V;
  W.nseg = n / M;
  W.nblk = (m + V - 1) / V;
  W.ncells = (long long)W.nblk * W.nseg;
  W.colbits = bits_for(n > m ? n : m);
  W.tokbits = bits_for(2ll * W.nseg) + 9;
  const int nn = nnz > 0 ? nnz : 1;
  W.keys = arena_take<unsigned long long>(ctx, nn);
  W.flag = arena_take<int>(ctx, nn);
  W.grow = arena_take<int>(ctx, nn);
  W.gseg = arena_take<int>(ctx, nn);
  W.gtok = arena_take<unsigned>(ctx, nn);
  W.rowptr = arena_take<int>(ctx, m + 1);
  W.ortab = arena_take<unsigned>(ctx, (W.ncells + 3) / 4);
  W.badtab = arena_take<unsigned>(ctx, (W.ncells + 3) / 4);
  W.counts = arena_take<int>(ctx, 2);
  W.order = arena_take<int>(ctx, m);
  W.order2 = arena_take<int>(ctx, m);
  W.gstart = arena_take<int>(ctx, m);
  W.settled = arena_take<unsigned char>(ctx, m);
  W.rkeys = arena_take<unsigned long long>(ctx, m);
  W.active = arena_take<int>(ctx, 1);
  W.blockmax = arena_take<int>(ctx, m / 1024 + 2);
  if (!W.keys || !W.flag || !W.grow || !W.gseg || !W.gtok || !W.rowptr || !W.ortab || !W.badtab || !W.counts ||
      !W.order || !W.order2 || !W.gstart || !W.settled || !W.rkeys || !W.active || !W.blockmax)
    return VNM_ERR_NOMEM;
  return VNM_OK;
}

__global__ void k_vs_check(const int* row, const int* col, int nnz, int m, int n, int* err) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nnz; i += gridDim.x * blockDim.x)
    if (row[i] < 0 || row[i] >= m || col[i] < 0 || col[i] >= n) atomicOr(err, 1);
}

static vnm_status vnm_args(vnm_ctx* ctx, int m, int n, int nnz, const int* row, const int* col, int mem, int M,
                           int V) {
  if (!ctx || m < 0 || n < 0 || nnz < 0 || M < 2 || M > 8 || V < 1) return VNM_ERR_ARG;
  if (mem != VNM_MEM_HOST && mem != VNM_MEM_DEVICE) return VNM_ERR_ARG;
  if (nnz > 0 && (!row || !col)) return VNM_ERR_ARG;
  if (m > (1 << 24) || n > (1 << 24)) return VNM_ERR_LIMIT;
  return VNM_OK;
}

}  // namespace vnm

using namespace vnm;

extern "C" {

vnm_status vnm_vnm_eval(vnm_ctx* ctx, int m, int n, int nnz, const int* row, const int* col, int mem, int M, int V,
                        int* out2) {
  VNM_TRY(vnm_args(ctx, m, n, nnz, row, col, mem, M, V));
  if (!out2) return VNM_ERR_ARG;
  const int mp = (m + M - 1) / M * M, np = (n + M - 1) / M * M;
  const long long ncells = (long long)((mp + V - 1) / V) * (np / M);
  VNM_TRY(arena_reserve(ctx, vnm_bytes(mp, nnz, ncells) + 2 * arena_bytes(nnz, 4)));
  VNM_TRY(pinned_reserve(ctx, 64));
  VNM_TRY(begin_call(ctx));
  const int *d_row, *d_col;
  VNM_TRY(stage_in(ctx, row, nnz, mem, &d_row));
  VNM_TRY(stage_in(ctx, col, nnz, mem, &d_col));
  int* err = arena_take<int>(ctx, 1);
  if (!err) return VNM_ERR_NOMEM;
  VNM_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), ctx->stream));
  if (nnz) VNM_LAUNCH(ctx, k_vs_check, vs_grid(ctx, nnz), VS_NT, 0, d_row, d_col, nnz, mp, np, err);
  VNM_CUDA_TRY(cudaMemcpyAsync(ctx->h_pinned, err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  VNM_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  if (ctx->h_pinned[0]) return VNM_ERR_RANGE;
  VnmWork W;
  VNM_TRY(vnm_setup(ctx, m, n, nnz, M, V, W));
  VNM_TRY(vnm_analyse(ctx, d_row, d_col, W, ctx->h_pinned));
  out2[0] = ctx->h_pinned[0];
  out2[1] = ctx->h_pinned[1];
  return end_call(ctx);
}

vnm_status vnm_vnm_reorder(vnm_ctx* ctx, int m, int n, int nnz, int* row, int* col, int mem, int M, int V,
                           int maxiter, int* out5, int* newpos) {
  VNM_TRY(vnm_args(ctx, m, n, nnz, row, col, mem, M, V));
  if (!out5) return VNM_ERR_ARG;
  const int mp = (m + M - 1) / M * M, np = (n + M - 1) / M * M;
  const long long ncells = (long long)((mp + V - 1) / V) * (np / M);
  VNM_TRY(arena_reserve(ctx, vnm_bytes(mp, nnz, ncells)));
  VNM_TRY(pinned_reserve(ctx, 64));
  VNM_TRY(begin_call(ctx));
  int* h = ctx->h_pinned;
  // state: prev (accepted) and cur (candidate) COO + composed row maps
  int* prev_r = arena_take<int>(ctx, nnz > 0 ? nnz : 1);
  int* prev_c = arena_take<int>(ctx, nnz > 0 ? nnz : 1);
  int* cur_r = arena_take<int>(ctx, nnz > 0 ? nnz : 1);
  int* cur_c = arena_take<int>(ctx, nnz > 0 ? nnz : 1);
  int* prev_comp = arena_take<int>(ctx, mp);
  int* cur_comp = arena_take<int>(ctx, mp);
  int* err = arena_take<int>(ctx, 1);
  if (!prev_r || !prev_c || !cur_r || !cur_c || !prev_comp || !cur_comp || !err) return VNM_ERR_NOMEM;
  if (nnz) {
    const cudaMemcpyKind kind = mem == VNM_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
    VNM_CUDA_TRY(cudaMemcpyAsync(prev_r, row, sizeof(int) * nnz, kind, ctx->stream));
    VNM_CUDA_TRY(cudaMemcpyAsync(prev_c, col, sizeof(int) * nnz, kind, ctx->stream));
  }
  VNM_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), ctx->stream));
  // columns index new_id[] (m entries), as in reordering.py:175-176
  if (nnz) VNM_LAUNCH(ctx, k_vs_check, vs_grid(ctx, nnz), VS_NT, 0, prev_r, prev_c, nnz, mp, mp < np ? mp : np, err);
  VNM_CUDA_TRY(cudaMemcpyAsync(h, err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  VNM_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  if (h[0]) return VNM_ERR_RANGE;
  VNM_LAUNCH(ctx, k_vs_iota, vs_grid(ctx, mp), VS_NT, 0, prev_comp, mp);
  VnmWork W;
  VNM_TRY(vnm_setup(ctx, m, n, nnz, M, V, W));
  VNM_TRY(vnm_analyse(ctx, prev_r, prev_c, W, h));
  const int init_inv = h[0], init_strict = h[1];
  int inv = init_inv, prev_inv = init_inv, prev_strict = init_strict;
  int round = 1;
  const int MAXITER = init_inv > maxiter ? init_inv : maxiter;  // reordering.py:209-210
  bool early = false;
  while (inv > 0 && round <= MAXITER) {
    // W holds the analysis of prev: sort its rows
    VNM_TRY(vnm_row_order(ctx, W, h));
    const int* new_id = W.order;  // new_id[i] = sorted_data[i][0]
    if (nnz) {
      VNM_CUDA_TRY(cudaMemcpyAsync(cur_r, prev_r, sizeof(int) * nnz, cudaMemcpyDeviceToDevice, ctx->stream));
      VNM_CUDA_TRY(cudaMemcpyAsync(cur_c, prev_c, sizeof(int) * nnz, cudaMemcpyDeviceToDevice, ctx->stream));
      VNM_LAUNCH(ctx, k_vs_apply, vs_grid(ctx, nnz), VS_NT, 0, cur_r, cur_c, nnz, new_id);
    }
    VNM_CUDA_TRY(cudaMemcpyAsync(cur_comp, prev_comp, sizeof(int) * mp, cudaMemcpyDeviceToDevice, ctx->stream));
    VNM_LAUNCH(ctx, k_vs_compose, vs_grid(ctx, mp), VS_NT, 0, cur_comp, mp, new_id);
    VNM_TRY(vnm_analyse(ctx, cur_r, cur_c, W, h));
    inv = h[0];
    const int istrict = h[1];
    if (inv > prev_inv) {  // reordering.py:242-246: keep the previous state
      early = true;
      break;
    }
    prev_inv = inv;
    prev_strict = istrict;
    std::swap(prev_r, cur_r);
    std::swap(prev_c, cur_c);
    std::swap(prev_comp, cur_comp);
    round += 1;
  }
  out5[0] = init_inv;
  out5[1] = init_strict;
  out5[2] = prev_inv;
  out5[3] = prev_strict;
  out5[4] = early ? round : round - 1;
  if (nnz) {
    const cudaMemcpyKind kind = mem == VNM_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
    VNM_CUDA_TRY(cudaMemcpyAsync(row, prev_r, sizeof(int) * nnz, kind, ctx->stream));
    VNM_CUDA_TRY(cudaMemcpyAsync(col, prev_c, sizeof(int) * nnz, kind, ctx->stream));
  }
  if (newpos) VNM_CUDA_TRY(cudaMemcpyAsync(newpos, prev_comp, sizeof(int) * mp, cudaMemcpyDeviceToHost, ctx->stream));
  return end_call(ctx);
}

}  // extern "C"
