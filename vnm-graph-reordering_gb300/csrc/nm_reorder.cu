// NM reorder on the GPU: a bit-exact, GB300-native rebuild of the reference's
// greedy swap search (reorder/reorder.h:1805-2474, reorder/swappair.h).
//
// What the reference does per round: recount invalid groups for every
// (row, segment) with one thread each (LocateinvalidSegment), then for each
// (primary, target) segment pair it visits, launch GetSegSwapScore over all
// rows (with cudaMalloc / memset / memcpy / cudaFree around it), push the M*M
// gains into a std::priority_queue, commit the best unvisited swap, and at
// the end of the round apply all swaps to the COO, copy it to the host, sort
// it, copy it back and rebuild BSR with cuSPARSE (Mtx::reset).
//
// Facts this design is built on (each is a property of the reference code):
//   1. A symmetric swap moves a row's groups to another row without changing
//      them, so invalid counts depend only on which node sits at which column
//      position.  The state of a job is therefore `orig[pos]` (the original
//      node at each position) plus per-segment counts; rows keep their
//      original ids throughout.
//   2. All gains of a round are computed against the round-start matrix
//      (swaps are applied only in reorder()), and a primary segment can take
//      at most M targets before all of its nodes are visited.  After the
//      first primary, the list is a subset of its <= M targets.  So a round
//      touches at most M+1 segments -- the first M+1 of the list in the
//      traversal order of the schedule -- and needs the gains of the
//      C(M+1, 2) segment pairs among them, all of which are computed up
//      front, in parallel.
//   3. For rows that touch only one of the two segments of a pair, the gain
//      depends on that segment alone: the left gain of swap (i, j) over such
//      rows is S_p(i) = #rows with bit i set and popcount == N+1.  Only rows
//      that touch both segments need the per-(i, j) terms.
//   4. The pop order of the swap-pair heap is fixed once its gains are known;
//      the visited filter only skips ahead in it.  So each ordered pair's pop
//      order is computed once per round (exact libstdc++ sift steps, one
//      thread per heap) and the walk reads the first unvisited entry -- or,
//      since a heap pops in non-increasing key order, takes the qualifying
//      swap of largest key directly when no other qualifying swap shares it.
//
// One thread-block cluster (or one block) runs one job (a matrix and a
// schedule) for all of its rounds: no host round trips, no allocation.  Many
// jobs (four schedules, or a batch of matrices) run in one launch.

#include <cooperative_groups.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "swap_heap.h"

namespace cg = cooperative_groups;

namespace vnm {

size_t scan_scratch_bytes(int n);

constexpr int NM_THREADS = 1024;  // threads per job block
constexpr unsigned FULL = 0xffffffffu;

// status bits a job reports in res[5]
constexpr int JOB_OK = 0;
constexpr int JOB_EMPTY_HEAP = 1;   // reference would call top() on an empty queue
constexpr int JOB_WAIT_LIMIT = 4;   // the walk waited too long for a swap heap's pops
constexpr int JOB_TABLE_FULL = 8;   // a row found no free table slot (cannot happen: at most 3/4 are taken)

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Time (ns) inside phases, accumulated by single threads of a job's leader
// block: [0] the walk warp, [1] its waits for swap-heap pops, [2] warp 0's
// rows in the process phase, [3] warp 0's rows in the apply phase, [4] and
// [5] warp 0's per-segment masks and pair corrections in the process phase.
__shared__ unsigned long long s_tin[6];

// The part of a job's row work one thread block does: block `rank` of the
// `cs` blocks (a thread-block cluster, cs a power of two <= 16) that share
// the job.  Rows are dealt to blocks in 16 groups: block `rank` owns the
// rows whose group lies in [rank * 16 / cs, (rank + 1) * 16 / cs).
struct Slice {
  int rank, cs;
};
constexpr int ROW_GROUPS = 16;
constexpr int JOB_RES = 32;  // ints of a job's result record (NMJob::res)

// A row's group: row & 15 rotated by a hash of row >> 4.  Within every
// aligned run of 16 rows each group occurs once, so a window of n rows puts
// at most ceil(n / 16) + 1 in a group; and the rows that share their low
// bits land in different groups.  (row & 15 alone gave the block owning
// group 0 the R-MAT hubs, whose low bits are 0: find_best at R-MAT 16384
// 2:4 took 13.6 ms.)
__host__ __device__ __forceinline__ int row_group(int row) {
  return (int)(((unsigned)row + (((unsigned)row >> 4) * 2654435761u >> 28)) & (ROW_GROUPS - 1));
}

struct NMJob {
  int R;              // padded rows = columns
  int nseg;           // R / M
  int sched;          // 0..3
  int maxiter;        // reorderUtil MAXITER before it is raised to init_size
  const int* cptr;    // [R+1] column pointers of the nonzero pattern (original ids)
  const int* crow;    // rows of each column, grouped by row_group
  const int* csplit;  // [16 R + 1] start of each (column, row group) in crow
  int* orig;          // [R] original node at each position (identity on entry)
  int* cnt;           // [nseg] invalid rows per segment
  int* zc;            // [nseg] all-zero rows per segment
  uint4* rec;         // [R] per-row scratch, zero on entry and on exit
  int* touched;       // [R + 32] scratch: block `rank` lists its touched rows from
                      //   rank * (ceil(R / 16) + 1) * (16 / cs) on
  int* res;           // [JOB_RES]: init_size, final_size, init_cnt, final_cnt, rounds, status,
                      //       swaps, gathered entries (lo, hi), touched rows (lo, hi),
                      //       [11] block-rounds with the records in a shared-memory
                      //       table, [12] block-rounds with them in global memory,
                      //       [13], [14] the job's start and end on the global timer
                      //       (units of 1024 ns, low 31 bits),
                      //       [16..22] time per round phase, [23] from the kernel's
                      //       start to its end (leader, thread 0), in units of 1024 ns,
                      //       [24], [25] the leader's own work in the process and
                      //       apply phases (before their barriers), [26..29] the
                      //       times inside phases of s_tin, same units
  int* trace_pairs;   // optional: swaps in commit order (v1, v2)
  int* trace_rounds;  // optional: pairs committed by the end of each round
  int trace_cap_pairs;
  int trace_cap_rounds;
  int walk_wait_limit;  // polls before a wait of the walk gives up (WALK_WAIT_LIMIT)
  int hold_heaps;       // test only: the swap heaps publish no pop, so a walk that waits runs out
  const int* err;       // the input check's flag (k_validate): nonzero, the job does nothing; null, no check
  int timed;            // measure the round phases (the leader's thread 0 reads the global timer)
};

// ---------------------------------------------------------------------------
// Setup kernels
// ---------------------------------------------------------------------------

// Range and strict (row, col) order check of the caller's COO.
__global__ void k_validate(const int* row, const int* col, int nnz, int R, int* err) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nnz; i += gridDim.x * blockDim.x) {
    int r = row[i], c = col[i];
    if (r < 0 || r >= R || c < 0 || c >= R) {
      atomicOr(err, 2);
      continue;
    }
    if (i > 0) {
      int rp = row[i - 1], cp = col[i - 1];
      if (rp > r || (rp == r && cp >= c)) atomicOr(err, 1);
    }
  }
}

__global__ void k_nonzero_flags(const float* val, int nnz, int* flags) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nnz; i += gridDim.x * blockDim.x)
    flags[i] = val[i] != 0.0f;  // reorder/reorder.h:93: the bitmap bit is (val != 0)
}

// Keep the entries with nonzero value, in order; count entries per
// (column, row group).  This kernel and every later one that takes indices
// as addresses do nothing when k_validate flagged the input (*err != 0): the
// host reads the flag once, at the end of the call.
__global__ void k_compact(const int* row, const int* col, const float* val, const int* pos, int nnz, int* prow,
                          int* pcol, int* gdeg, const int* err) {
  if (*err) return;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nnz; i += gridDim.x * blockDim.x) {
    if (val[i] != 0.0f) {
      int p = pos[i];
      prow[p] = row[i];
      pcol[p] = col[i];
      atomicAdd(&gdeg[(size_t)ROW_GROUPS * col[i] + row_group(row[i])], 1);
    }
  }
}

// cptr[c] = the start of column c's first group (c = 0 .. R)
__global__ void k_cptr_from_split(const int* csplit, int R, int* cptr) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c <= R; c += gridDim.x * blockDim.x)
    cptr[c] = csplit[(size_t)ROW_GROUPS * c];
}

// Column lists of the pattern, each grouped by row_group (the order inside
// a group is whatever the atomics give; nothing depends on it).
__global__ void k_csc_scatter(const int* prow, const int* pcol, const int* d_np, const int* csplit, int* cfill,
                              int* crow, const int* err) {
  if (*err) return;
  const int np = *d_np;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < np; i += gridDim.x * blockDim.x) {
    const size_t g = (size_t)ROW_GROUPS * pcol[i] + row_group(prow[i]);
    const int slot = atomicAdd(&cfill[g], 1);
    crow[csplit[g] + slot] = prow[i];
  }
}

// Invalid and non-empty group counts per segment at the identity arrangement.
// The pattern is sorted by (row, col), so a row's groups are runs of entries
// with equal col / M; the last entry of each run does the counting.
template <int M>
__global__ void k_locate(const int* prow, const int* pcol, const int* d_np, int N, int* inv, int* pres,
                         const int* err) {
  if (*err) return;
  const int np = *d_np;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < np; i += gridDim.x * blockDim.x) {
    const int r = prow[i], s = pcol[i] / M;
    const bool last = (i + 1 == np) || prow[i + 1] != r || pcol[i + 1] / M != s;
    if (!last) continue;
    int len = 1;
#pragma unroll
    for (int b = 1; b < M; ++b) {
      int k = i - b;
      if (k >= 0 && prow[k] == r && pcol[k] / M == s) len++;
    }
    atomicAdd(&pres[s], 1);
    if (len > N) atomicAdd(&inv[s], 1);
  }
}

__global__ void k_init_job(int* orig, int* cnt, int* zc, const int* inv0, const int* pres0, int R, int nseg) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < R; i += gridDim.x * blockDim.x) {
    orig[i] = i;
    if (i < nseg) {
      cnt[i] = inv0[i];
      zc[i] = R - pres0[i];
    }
  }
}

// newpos[orig[p]] = p
__global__ void k_invert(const int* orig, int R, int* newpos) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < R; i += gridDim.x * blockDim.x) newpos[orig[i]] = i;
}

__global__ void k_permute(int* row, int* col, int nnz, const int* newpos) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nnz; i += gridDim.x * blockDim.x) {
    row[i] = newpos[row[i]];
    col[i] = newpos[col[i]];
  }
}

// ---------------------------------------------------------------------------
// The round kernel
// ---------------------------------------------------------------------------
template <int M>
struct RoundSmem {
  static constexpr int K = M + 1;           // segments a round can touch
  static constexpr int NPAIR = K * (K - 1) / 2;
  static constexpr int MM = M * M;
  static constexpr int NW = NM_THREADS / 32;
  int xseg[K];      // the segments of this round, xseg[0] first
  int xcnt[K];      // their counts at round start
  int K_;           // how many
  int mode;         // 0 = pair walk, 1 = single invalid segment + minseg, 2 = single, minseg is itself
  int lsize, ltotal;
  int minseg;
  int ntouched;
  int E;            // gathered entries
  uint4* table;     // shared-memory row records (x, y, z: bitmaps; w: row + 1), or null
  int ts_max;       // slots of `table` (a power of two) or 0
  int ts_shift;     // 32 - log2(ts_max)
  int use_table;    // this round's records are in `table` (else in J.rec)
  int* tlist;       // the slots of `table` claimed this round, densely (ts_max entries)
  int tcount;       // how many
  int toff;         // this block's part of J.touched
  unsigned long long acc[4];  // leader: the helpers' work counters, added at the end
  uint4* rcache;    // the process phase's first pass of touched rows, kept for the apply phase
  int* rcrow;       //   (NM_THREADS x 4 records and their rows), or null
  int status;
  int nswaps;
  int hprog[K * K];  // pops of each ordered pair's heap written to ord so far
  int hstop;         // the walk is done: the heaps may stop
  uint8_t hsmall[K * K];  // the heap's entries hold the gains themselves ((l + r, r) in 12 + 12 bits)
  int go;           // the leader's decision to run another round (copied to every block)
  int S[K][M];                 // S_x(k): rows with bit k set and popcount == N+1
  int CL[NPAIR][MM];           // per unordered pair (a < b): left-side corrections
  int CR[NPAIR][MM];           //                              right-side corrections
  static constexpr int HSTR = (K * K + 31) / 32 * 32;  // heaps, rounded up to whole warps
  // Scratch at the head of dynamic shared memory, used by three phases in
  // turn: the process phase's per-warp row masks (2 x K x M words a warp),
  // the heap phase's slots [MM][HSTR] and entries [MM][HSTR] (4 B each), and
  // the apply phase's bit-move table (K x ceil(M/4) x 16 x 16 B, less than
  // the row masks).
  static constexpr int PROC_BYTES = NW * 2 * K * M * 4;
  static constexpr int HEAP_BYTES = MM * HSTR * 8;
  static constexpr int SCR_U4 = ((PROC_BYTES > HEAP_BYTES ? PROC_BYTES : HEAP_BYTES) + 15) / 16;
  uint8_t ord[MM][HSTR];       // pop order: ord[k][a * K + b] is the k-th pop of ordered pair (a, b)
  int colstart[K * M];
  int colpre[K * M + 1];
  static constexpr int DEST_W = (K * M + 3) / 4;  // dest in 32-bit words
  union {
    uint8_t dest[K][M];        // bit moves of this round's swaps: (xi << 4) | k
    uint32_t dest_w[DEST_W];   // the same bytes as words, for copies to other blocks
  };
  int newinv[K], newpres[K];
  int swaps[2 * K * M];        // committed swaps (positions)
  unsigned long long wtop[2][NW][K];
  unsigned long long sel_top[15][2][K];  // leader: each helper's scan (top K both orders) ...
  int sel_ls[15][2];                     // ... and its list size and total, pushed by the helper
  unsigned long long top[2][K];  // [0] Ldesc order (cnt desc, seg asc), [1] reverse
  unsigned long long red64[NW];
  int red32[2][NW];
};

template <int M>
__device__ __forceinline__ int pair_id(int a, int b) {  // a < b < K
  constexpr int K = M + 1;
  return a * (2 * K - a - 1) / 2 + (b - a - 1);
}

// Gains of swap idx = i*M + j of ordered pair (a = primary side, b = target side).
template <int M>
__device__ __forceinline__ void pair_gains(const RoundSmem<M>& sm, int a, int b, int idx, int& l, int& r) {
  const int i = idx / M, j = idx % M;
  if (a == b) {  // single segment paired with itself: direct sums kept in CL/CR[0]
    l = sm.CL[0][idx];
    r = sm.CR[0][idx];
  } else if (a < b) {
    const int p = pair_id<M>(a, b);
    l = sm.S[a][i] - sm.CL[p][i * M + j];
    r = sm.S[b][j] - sm.CR[p][i * M + j];
  } else {
    const int p = pair_id<M>(b, a);
    l = sm.S[a][i] - sm.CR[p][j * M + i];
    r = sm.S[b][j] - sm.CL[p][j * M + i];
  }
}

// insert `key` into a register list sorted descending (0 = empty)
template <int K>
__device__ __forceinline__ void topk_insert(unsigned long long (&a)[K], unsigned long long key) {
  if (key <= a[K - 1]) return;
  a[K - 1] = key;
#pragma unroll
  for (int q = K - 1; q > 0; --q) {
    if (a[q] > a[q - 1]) {
      unsigned long long t = a[q];
      a[q] = a[q - 1];
      a[q - 1] = t;
    }
  }
}

// merge the sorted lists of lanes 0 .. W-1 (W a power of two; the other
// lanes hold their own); lane 0 gets their top K in out[]
template <int K, int W = 32>
__device__ __forceinline__ void topk_warp_merge(unsigned long long (&a)[K], unsigned long long* out) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int q = 0; q < K; ++q) {
    unsigned long long h = a[0], m = h;
#pragma unroll
    for (int o = W / 2; o > 0; o >>= 1) {
      unsigned long long t = __shfl_xor_sync(FULL, m, o);
      m = t > m ? t : m;
    }
    if (lane == 0) out[q] = m;
    if (h == m && m != 0) {
#pragma unroll
      for (int z = 0; z < K - 1; ++z) a[z] = a[z + 1];
      a[K - 1] = 0;
    }
  }
}

__device__ __forceinline__ unsigned long long desc_key(int c, int s) {  // cnt descending, segment ascending
  return ((unsigned long long)(unsigned)c << 32) | (unsigned)(0xffffffffu - (unsigned)s);
}
__device__ __forceinline__ unsigned long long rev_key(int c, int s) {  // cnt ascending, segment descending
  return ((unsigned long long)(unsigned)(0x7fffffff - c) << 32) | (unsigned)s;
}

// Scan the segment counts of segments [s_beg, s_end) except the nx listed
// in xs: list size, total, first K in both orders.
template <int M>
__device__ void select_range(RoundSmem<M>& sm, const int* cnt, int s_beg, int s_end, const int* xs, int nx) {
  constexpr int K = M + 1;
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  unsigned long long kd[K], kr[K];
#pragma unroll
  for (int q = 0; q < K; ++q) kd[q] = kr[q] = 0;
  int lsz = 0, tot = 0;
  for (int s = s_beg + tid; s < s_end; s += NM_THREADS) {
    bool skip = false;
    for (int t = 0; t < nx; ++t) skip |= (xs[t] == s);
    const int c = skip ? 0 : cnt[s];
    if (c > 0) {
      lsz++;
      tot += c;
      topk_insert<K>(kd, desc_key(c, s));
      topk_insert<K>(kr, rev_key(c, s));
    }
  }
  topk_warp_merge<K>(kd, sm.wtop[0][w]);
  topk_warp_merge<K>(kr, sm.wtop[1][w]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    lsz += __shfl_xor_sync(FULL, lsz, o);
    tot += __shfl_xor_sync(FULL, tot, o);
  }
  if (lane == 0) {
    sm.red32[0][w] = lsz;
    sm.red32[1][w] = tot;
  }
  __syncthreads();
  if (w < 2) {  // warp 0 merges the descending lists, warp 1 the reverse ones
    unsigned long long a[K];
#pragma unroll
    for (int q = 0; q < K; ++q) a[q] = lane < RoundSmem<M>::NW ? sm.wtop[w][lane][q] : 0ull;
    topk_warp_merge<K>(a, sm.top[w]);
  } else if (w == 2) {
    int v0 = lane < RoundSmem<M>::NW ? sm.red32[0][lane] : 0;
    int v1 = lane < RoundSmem<M>::NW ? sm.red32[1][lane] : 0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      v0 += __shfl_xor_sync(FULL, v0, o);
      v1 += __shfl_xor_sync(FULL, v1, o);
    }
    if (lane == 0) {
      sm.lsize = v0;
      sm.ltotal = v1;
    }
  }
  __syncthreads();
}

// Scan the segment counts: list size, total, first K in both orders.
template <int M>
__device__ void select_phase(RoundSmem<M>& sm, const NMJob& J, const int* cnt) {
  select_range<M>(sm, cnt, 0, J.nseg, nullptr, 0);
}

// The same result as select_phase after a round, from the other blocks'
// scans of all segments but this round's (made while the leader ran the
// heaps and the walk; those counts did not change; each helper pushed its
// result into sel_top / sel_ls) and this round's segments with their new
// counts (leader block of a cluster).  Lane l holds helper l + 1's list:
// at most 15 helpers and 9 round segments, so the lists sit in lanes 0-15.
template <int M>
__device__ void select_merge(RoundSmem<M>& sm, cg::cluster_group& cl, int cs, const int* cnt) {
  constexpr int K = M + 1;
  static_assert(K <= 16, "the round's segments fit lanes 0-15");
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  (void)cl;
  if (w < 2) {  // warp 0 the descending lists, warp 1 the reverse ones
    unsigned long long a[K];  // a helper's list is sorted already
#pragma unroll
    for (int q = 0; q < K; ++q) a[q] = lane + 1 < cs ? sm.sel_top[lane][w][q] : 0ull;
    if (lane < sm.K_) {
      const int sg = sm.xseg[lane], c = cnt[sg];
      if (c > 0) topk_insert<K>(a, w == 0 ? desc_key(c, sg) : rev_key(c, sg));
    }
    topk_warp_merge<K, 16>(a, sm.top[w]);
  } else if (w == 2) {
    int v0 = 0, v1 = 0;
    if (lane + 1 < cs) {
      v0 = sm.sel_ls[lane][0];
      v1 = sm.sel_ls[lane][1];
    }
    if (lane < sm.K_) {
      const int c = cnt[sm.xseg[lane]];
      if (c > 0) {
        v0 += 1;
        v1 += c;
      }
    }
#pragma unroll
    for (int o = 8; o > 0; o >>= 1) {  // lanes 0-15
      v0 += __shfl_xor_sync(FULL, v0, o);
      v1 += __shfl_xor_sync(FULL, v1, o);
    }
    if (lane == 0) {
      sm.lsize = v0;
      sm.ltotal = v1;
    }
  }
  __syncthreads();
}

// locate_min_outdeg_seg (reorder/reorder.h:767-797): most all-zero rows,
// ties to the largest segment id.
template <int M>
__device__ void minseg_phase(RoundSmem<M>& sm, const NMJob& J) {
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  unsigned long long best = 0;
  for (int s = tid; s < J.nseg; s += NM_THREADS) {
    unsigned long long k = ((unsigned long long)(unsigned)J.zc[s] << 32) | (unsigned)s;
    best = k > best ? k : best;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long t = __shfl_xor_sync(FULL, best, o);
    best = t > best ? t : best;
  }
  if (lane == 0) sm.red64[w] = best;
  __syncthreads();
  if (w == 0) {
    unsigned long long v = lane < RoundSmem<M>::NW ? sm.red64[lane] : 0ull;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      unsigned long long t = __shfl_xor_sync(FULL, v, o);
      v = t > v ? t : v;
    }
    if (lane == 0) sm.minseg = (int)(unsigned)(v & 0xffffffffu);
  }
  __syncthreads();
}

__device__ __forceinline__ int seg_of_desc(unsigned long long k) { return (int)(0xffffffffu - (unsigned)k); }
__device__ __forceinline__ int cnt_of_desc(unsigned long long k) { return (int)(k >> 32); }
__device__ __forceinline__ int seg_of_rev(unsigned long long k) { return (int)(unsigned)k; }
__device__ __forceinline__ int cnt_of_rev(unsigned long long k) { return 0x7fffffff - (int)(k >> 32); }

// cmp (reorder/reorder.h:422-427) as "a comes out of the max-heap before b"
__device__ __forceinline__ bool before_cmp(int sa, int ca, int sb, int cb) {
  return ca != cb ? ca > cb : sa < sb;
}
// cmp_reverse (reorder/reorder.h:429-434)
__device__ __forceinline__ bool before_rev(int sa, int ca, int sb, int cb) {
  return ca != cb ? ca < cb : sa > sb;
}

// Which segments this round can touch (fact 2 above).
template <int M>
__device__ void choose_segments(RoundSmem<M>& sm, int sched) {
  constexpr int K = M + 1;
  if (threadIdx.x >= 32) return;  // warp 0; lane q handles list entry q
  const int lane = threadIdx.x;
  const int L = sm.lsize;
  if (L == 1) {
    if (lane == 0) {
      int s0 = seg_of_desc(sm.top[0][0]);
      sm.xseg[0] = s0;
      sm.xcnt[0] = cnt_of_desc(sm.top[0][0]);
      if (sm.minseg == s0) {
        sm.mode = 2;
        sm.K_ = 1;
      } else {
        sm.mode = 1;
        sm.xseg[1] = sm.minseg;
        sm.xcnt[1] = 0;
        sm.K_ = 2;
      }
    }
    return;
  }
  const int lim = L < K ? L : K;
  if (sched == 0 || sched == 2) {  // primary and targets follow one order: the first lim entries
    const int o = sched == 0 ? 0 : 1;
    if (lane < lim) {
      const unsigned long long k = sm.top[o][lane];
      sm.xseg[lane] = o == 0 ? seg_of_desc(k) : seg_of_rev(k);
      sm.xcnt[lane] = o == 0 ? cnt_of_desc(k) : cnt_of_rev(k);
    }
    if (lane == 0) {
      sm.mode = 0;
      sm.K_ = lim;
    }
    return;
  }
  // primary from one end, targets from the other: the first lim - 1
  // entries of the other order that are not the primary
  const int po = sched == 1 ? 0 : 1, to = 1 - po;
  const unsigned long long pk = sm.top[po][0];
  const int ps = po == 0 ? seg_of_desc(pk) : seg_of_rev(pk);
  unsigned long long k = 0;
  int sg = 0;
  if (lane < K) {
    k = sm.top[to][lane];
    sg = to == 0 ? seg_of_desc(k) : seg_of_rev(k);
  }
  const unsigned keep = __ballot_sync(FULL, lane < K && sg != ps);
  const int at = 1 + __popc(keep & ((1u << lane) - 1u));
  if (((keep >> lane) & 1u) && at < lim) {
    sm.xseg[at] = sg;
    sm.xcnt[at] = to == 0 ? cnt_of_desc(k) : cnt_of_rev(k);
  }
  if (lane == 0) {
    sm.mode = 0;
    sm.xseg[0] = ps;
    sm.xcnt[0] = po == 0 ? cnt_of_desc(pk) : cnt_of_rev(pk);
    const int n = 1 + __popc(keep);
    sm.K_ = n < lim ? n : lim;
  }
}

template <int M>
__device__ void clear_round_smem(RoundSmem<M>& sm) {
  constexpr int K = M + 1;
  for (int i = threadIdx.x; i < K * M; i += NM_THREADS) (&sm.S[0][0])[i] = 0;
  for (int i = threadIdx.x; i < RoundSmem<M>::NPAIR * RoundSmem<M>::MM; i += NM_THREADS) {
    (&sm.CL[0][0])[i] = 0;
    (&sm.CR[0][0])[i] = 0;
  }
  if (threadIdx.x < K) {
    sm.newinv[threadIdx.x] = 0;
    sm.newpres[threadIdx.x] = 0;
  }
  if (threadIdx.x == 0) {
    sm.ntouched = 0;
    sm.nswaps = 0;
  }
}

// OR the bitmaps of the round's segments into the records of the rows this
// block owns.  Every column's rows are stored grouped by row_group (csplit),
// so the block's entries of a column are one contiguous run of it, and no
// other block touches these records: the process and apply phases that
// follow need no cluster barrier.  The records go to the block's
// shared-memory table when its entries fill at most 3/4 of it, else to
// J.rec in global memory.
template <int M>
__device__ void gather_phase(RoundSmem<M>& sm, const NMJob& J, Slice sl = Slice{0, 1}) {
  constexpr int K = M + 1;
  const int tid = threadIdx.x;
  const int KM = sm.K_ * M;
  const int g0 = sl.rank * (ROW_GROUPS / sl.cs), g1 = g0 + ROW_GROUPS / sl.cs;
  if (tid < 32) {  // this block's run of each column of the round and their prefix sums, on one warp
    constexpr int CPL = (K * M + 31) / 32;  // columns per lane
    int len[CPL], tot = 0;
#pragma unroll
    for (int q = 0; q < CPL; ++q) {
      const int col = tid * CPL + q;
      len[q] = 0;
      if (col < KM) {
        const int u = J.orig[sm.xseg[col / M] * M + col % M];
        const int b = J.csplit[(size_t)ROW_GROUPS * u + g0];
        sm.colstart[col] = b;
        len[q] = J.csplit[(size_t)ROW_GROUPS * u + g1] - b;
      }
      tot += len[q];
    }
    int incl = tot;  // inclusive scan of the lanes' totals
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(FULL, incl, o);
      if (tid >= o) incl += t;
    }
    int run = incl - tot;
#pragma unroll
    for (int q = 0; q < CPL; ++q) {
      const int col = tid * CPL + q;
      if (col < KM) sm.colpre[col] = run;
      run += len[q];
    }
    if (tid == 31) {
      sm.colpre[KM] = incl;
      sm.E = incl;
      sm.use_table = sm.ts_max > 0 && incl <= (sm.ts_max >> 2) * 3;
    }
  }
  __syncthreads();
  const int E = sm.E;
  if (sm.use_table) {
    // open addressing, linear probing; a slot is claimed by CAS on its row
    // key and appended to the list of claimed slots, which the process and
    // apply phases walk in full 32-row chunks.  At most 3/4 of the slots
    // are taken, so a free one is always found.
    const unsigned mask = (unsigned)sm.ts_max - 1u;
    unsigned* tw = reinterpret_cast<unsigned*>(sm.table);
    // TABLE_U entries per thread per step, their row loads in flight together
    constexpr int TABLE_U = 2;
    for (int base = tid; base < E; base += NM_THREADS * TABLE_U) {
      int rows[TABLE_U], qs[TABLE_U];
#pragma unroll
      for (int u = 0; u < TABLE_U; ++u) {
        const int e = base + u * NM_THREADS;
        rows[u] = -1;
        qs[u] = 0;
        if (e < E) {
          int lo = 0, hi = KM - 1;  // last q with colpre[q] <= e
          while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (sm.colpre[mid] <= e) lo = mid;
            else hi = mid - 1;
          }
          qs[u] = lo;
          rows[u] = J.crow[sm.colstart[lo] + (e - sm.colpre[lo])];
        }
      }
#pragma unroll
      for (int u = 0; u < TABLE_U; ++u) {
        if (rows[u] < 0) continue;
        const int xi = qs[u] / M, k = qs[u] % M;
        const unsigned key = (unsigned)rows[u] + 1u;
        unsigned h = (key * 2654435761u) >> sm.ts_shift;
        bool placed = false;
        for (int probe = 0; probe <= (int)mask; ++probe) {
          const unsigned cur = atomicCAS(&tw[4 * h + 3], 0u, key);
          if (cur == 0u || cur == key) {
            atomicOr(&tw[4 * h + (xi >> 2)], (1u << k) << ((xi & 3) * 8));
            if (cur == 0u) sm.tlist[atomicAdd(&sm.tcount, 1)] = (int)h;
            placed = true;
            break;
          }
          h = (h + 1u) & mask;
        }
        if (!placed)
          atomicOr(sl.cs > 1 ? cg::this_cluster().map_shared_rank(&sm.status, 0) : &sm.status, JOB_TABLE_FULL);
      }
    }
    __syncthreads();
    if (tid == 0) sm.ntouched = sm.tcount;
    __syncthreads();
    return;
  }
  unsigned* recw = reinterpret_cast<unsigned*>(J.rec);
  int* tl = J.touched + sm.toff;
  // GATHER_U entries per thread per step: their row loads, their bitmap ORs
  // (no result used, so they issue as reductions) and their first-touch
  // atomics are all in flight together instead of one chain at a time.
  constexpr int GATHER_U = 4;
  for (int base = tid; base < E; base += NM_THREADS * GATHER_U) {
    int rr[GATHER_U];
    unsigned word[GATHER_U], bit[GATHER_U];
#pragma unroll
    for (int u = 0; u < GATHER_U; ++u) {
      const int e = base + u * NM_THREADS;
      rr[u] = -1;
      word[u] = 0;
      bit[u] = 0;
      if (e < E) {
        int lo = 0, hi = KM - 1;  // last q with colpre[q] <= e
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (sm.colpre[mid] <= e) lo = mid;
          else hi = mid - 1;
        }
        const int q = lo, xi = q / M, k = q % M;
        rr[u] = J.crow[sm.colstart[q] + (e - sm.colpre[q])];
        word[u] = (unsigned)(xi >> 2);
        bit[u] = (1u << k) << ((xi & 3) * 8);
      }
    }
#pragma unroll
    for (int u = 0; u < GATHER_U; ++u)
      if (rr[u] >= 0) atomicOr(&recw[4 * rr[u] + word[u]], bit[u]);
    unsigned first[GATHER_U];
#pragma unroll
    for (int u = 0; u < GATHER_U; ++u) first[u] = rr[u] >= 0 ? atomicOr(&recw[4 * rr[u] + 3], 1u) : 1u;
#pragma unroll
    for (int u = 0; u < GATHER_U; ++u)
      if (first[u] == 0u) tl[atomicAdd(&sm.ntouched, 1)] = rr[u];
  }
  __syncthreads();
}

__device__ __forceinline__ unsigned rec_byte(const uint4& w, int xi) {
  const unsigned word = xi < 4 ? w.x : (xi < 8 ? w.y : w.z);
  return (word >> ((xi & 3) * 8)) & 0xffu;
}

// Run f(row, record, valid) over the touched rows, one row per lane, with
// every lane of a warp calling f the same number of times (lanes past the
// end get valid = false and a zero record) so f may use warp votes.  Each
// lane first loads the records of TOUCH_U rows so their L2 round trips
// overlap.
// CM = 1: keep the records of the first pass in shared memory (process
// phase); CM = 2: take them from there (apply phase), saving two dependent
// L2 loads.  Both phases deal the rows to threads the same way, and the
// touched rows and their records do not change in between.
constexpr int TOUCH_U = 4;
template <int M, int CM, class F>
__device__ __forceinline__ void for_touched_warp(const RoundSmem<M>& sm, const NMJob& J, F&& f) {
  constexpr int NW = NM_THREADS / 32;
  const int nt = sm.ntouched;
  const int* tl = J.touched + sm.toff;  // the rows this block owns and the round touched
  // 32-row chunks dealt round-robin over the block's warps
  constexpr int NWt = NW;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  bool first = true;
  for (int c0 = w; c0 * 32 < nt; c0 += NWt * TOUCH_U) {
    int rv[TOUCH_U];
    uint4 wv[TOUCH_U];
    if (CM == 2 && first && sm.rcache) {
#pragma unroll
      for (int u = 0; u < TOUCH_U; ++u) {
        rv[u] = sm.rcrow[u * NM_THREADS + threadIdx.x];
        wv[u] = sm.rcache[u * NM_THREADS + threadIdx.x];
      }
    } else {
#pragma unroll
      for (int u = 0; u < TOUCH_U; ++u) {
        const int t = (c0 + u * NWt) * 32 + lane;
        rv[u] = t < nt ? tl[t] : -1;
      }
#pragma unroll
      for (int u = 0; u < TOUCH_U; ++u) wv[u] = rv[u] >= 0 ? J.rec[rv[u]] : make_uint4(0u, 0u, 0u, 0u);
      if (CM == 1 && first && sm.rcache) {
#pragma unroll
        for (int u = 0; u < TOUCH_U; ++u) {
          sm.rcrow[u * NM_THREADS + threadIdx.x] = rv[u];
          sm.rcache[u * NM_THREADS + threadIdx.x] = wv[u];
        }
      }
    }
    first = false;
#pragma unroll 1
    for (int u = 0; u < TOUCH_U && (c0 + u * NWt) * 32 < nt; ++u) f(rv[u], wv[u], rv[u] >= 0, c0 + u * NWt);
  }
}

// Run f(index, record, valid) over this round's row records: the table
// slots (index = slot) when the records are in shared memory, else the
// touched rows (index = row).  Warp-uniform like for_touched_warp.
template <int M, int CM, class F>
__device__ __forceinline__ void for_rows_warp(const RoundSmem<M>& sm, const NMJob& J, F&& f) {
  if (sm.use_table) {  // the rows this block's table holds, from its list of claimed slots
    constexpr int NW = NM_THREADS / 32;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int n = sm.tcount;
    for (int base = w * 32; base < n; base += NW * 32) {
      const int i = base + lane;
      const int slot = i < n ? sm.tlist[i] : 0;
      const uint4 v = i < n ? sm.table[slot] : make_uint4(0u, 0u, 0u, 0u);
      f(slot, v, i < n, base >> 5);
    }
  } else {
    for_touched_warp<M, CM>(sm, J, f);
  }
}

// Solo terms and pair corrections (fact 3), accumulated with warp votes:
// for 32 rows at a time, a count over rows of a product of two per-row bit
// conditions is popc(ballot(first) & ballot(second)), and one lane adds it
// to shared memory.  For the pair (a, c) with L = bits in a, R = bits in c,
// over rows where both are non-empty:
//   CL(i, j) = sum  R_j * eL_i,   eL = L if pL == N+1, ~L if pL == N, else 0
//   CR(i, j) = sum  L_i * eR_j,   eR = R if pR == N+1, ~R if pR == N, else 0
//   S_a(k)   = sum over all rows of [L_k and pL == N+1]
template <int M>
__device__ void process_phase(RoundSmem<M>& sm, const NMJob& J, int N, Slice sl = Slice{0, 1}) {
  constexpr int K = M + 1;
  constexpr int MM = M * M;
  const int Kn = sm.K_;
  const bool self = sm.mode == 2;
  const int lane = threadIdx.x & 31;
  // this warp's row masks: VL[x][k] at vw[2x * M + k], VE[x][k] at vw[(2x + 1) * M + k]
  extern __shared__ uint4 smem_heap[];
  unsigned* vw_warp = reinterpret_cast<unsigned*>(smem_heap) + (threadIdx.x >> 5) * (2 * K * M);
  const bool tmain = threadIdx.x == 0 && sl.rank == 0 && J.timed;  // the leader's thread 0 times (when asked)
  const unsigned long long t_in = tmain ? global_ns() : 0ull;
  // When every 32-row chunk's masks fit the scratch, each chunk leaves them
  // there and the sums are made afterwards over all chunks (gathered),
  // instead of a shared atomic per chunk, pair and entry: those atomics, and
  // the mask loads queued behind them, were 90 % of the process phase at
  // R-MAT 16384 2:4.
  constexpr int NCH = RoundSmem<M>::SCR_U4 * 16 / (2 * K * M * 4);  // chunks whose masks fit the scratch
  static_assert(NCH >= NM_THREADS / 32, "one chunk a warp fits the scratch");
  const int nchunks = ((sm.use_table ? sm.tcount : sm.ntouched) + 31) / 32;
  const bool gathered = !self && nchunks <= NCH;
  for_rows_warp<M, 1>(sm, J, [&](int r, const uint4& w, bool valid, int chunk) {
    (void)r;
    // chunk c's masks at c * 2KM when they are summed afterwards, else this warp's
    unsigned* vw = gathered ? reinterpret_cast<unsigned*>(smem_heap) + chunk * (2 * K * M) : vw_warp;
    const unsigned long long t_a = tmain ? global_ns() : 0ull;
    unsigned b[K];
    int p[K];
#pragma unroll
    for (int xi = 0; xi < K; ++xi) {
      b[xi] = (valid && xi < Kn) ? rec_byte(w, xi) : 0u;
      p[xi] = __popc(b[xi]);
    }
    if (self) {
      // reference kernel lines 108-121 with lval == rval: direct per (i, j)
      const unsigned L = b[0];
      const int pl = p[0];
      if (L == 0) return;
      for (int i = 0; i < M; ++i) {
        const unsigned li = (L >> i) & 1u;
        for (int j = 0; j < M; ++j) {
          const unsigned lj = (L >> j) & 1u;
          int l = (li && !lj && pl == N + 1) - (!li && lj && pl == N);
          int rr = (lj && !li && pl == N + 1) - (!lj && li && pl == N);
          if (l) atomicAdd(&sm.CL[0][i * M + j], l);
          if (rr) atomicAdd(&sm.CR[0][i * M + j], rr);
        }
      }
      return;
    }
    // Per segment x of the round, over the chunk's rows: VL[x][k] = rows
    // with bit k, VE[x][k] = rows with bit k of eL, and the solo terms.
    // With P1 = rows of popcount N+1 and P0 = rows of popcount N,
    // VE[x][k] = (VL[x][k] & P1) | (~VL[x][k] & P0) and the solo rows of
    // bit k are VL[x][k] & P1.  Lane k < M keeps the masks of bit k in this
    // warp's scratch.
#pragma unroll
    for (int xi = 0; xi < K; ++xi) {
      if (xi >= Kn) break;
      const unsigned bx = valid ? rec_byte(w, xi) : 0u;
      if (__ballot_sync(FULL, bx != 0u) == 0u) {
        if (gathered && lane < M) vw[(2 * xi) * M + lane] = vw[(2 * xi + 1) * M + lane] = 0u;
        continue;
      }
      const int px = __popc(bx);
      const unsigned p1 = __ballot_sync(FULL, px == N + 1), p0 = __ballot_sync(FULL, px == N);
      unsigned vl = 0u;
#pragma unroll
      for (int k = 0; k < M; ++k) {
        const unsigned l = __ballot_sync(FULL, (bx >> k) & 1u);
        if (lane == k) vl = l;
      }
      if (lane < M) {
        const unsigned so = vl & p1;
        if (so && !gathered) atomicAdd(&sm.S[xi][lane], __popc(so));
        vw[(2 * xi) * M + lane] = vl;
        vw[(2 * xi + 1) * M + lane] = so | (~vl & p0);
      }
    }
    __syncwarp();
    // Pair corrections, over the segment pairs that some row of this chunk
    // holds both of.  For the pair (a, c) the masks restricted to rows with
    // both segments non-empty are VE[a][i] & NZ[c] and VL[c][j] & NZ[a];
    // VE[a][i] lies inside NZ[a] (eL is empty when L is) and VL[c][j] inside
    // NZ[c], so CL(i, j) = popc(VE[a][i] & VL[c][j]) and likewise
    // CR(i, j) = popc(VL[a][i] & VE[c][j]).
    const bool timed = tmain;
    const unsigned long long t_b = timed ? global_ns() : 0ull;
    if (timed) s_tin[4] += t_b - t_a;
    if (gathered) {  // the masks stay in this warp's scratch for the sums below
      __syncwarp();
      return;
    }
    unsigned segs = 0;
#pragma unroll
    for (int xi = 0; xi < K; ++xi) segs |= (b[xi] != 0u ? 1u : 0u) << xi;
    unsigned wsegs = __popc(segs) >= 2 ? segs : 0u;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) wsegs |= __shfl_xor_sync(FULL, wsegs, o);
    constexpr int U = (MM + 31) / 32;  // (i, j) entries per lane
#pragma unroll 1
    for (unsigned sa = wsegs; sa; sa &= sa - 1) {
      const int a = __ffs(sa) - 1;
      unsigned ea[U], la[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int i = (lane + 32 * u < MM ? lane + 32 * u : 0) / M;
        ea[u] = vw[(2 * a + 1) * M + i];
        la[u] = vw[(2 * a) * M + i];
      }
#pragma unroll 1
      for (unsigned sc = sa & (sa - 1); sc; sc &= sc - 1) {
        const int c = __ffs(sc) - 1;
        const int pid = pair_id<M>(a, c);
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int idx = lane + 32 * u;
          if (idx < MM) {
            const int j = idx % M;
            const int cl = __popc(ea[u] & vw[(2 * c) * M + j]);
            const int cr = __popc(la[u] & vw[(2 * c + 1) * M + j]);
            if (cl) atomicAdd(&sm.CL[pid][idx], cl);
            if (cr) atomicAdd(&sm.CR[pid][idx], cr);
          }
        }
      }
    }
    __syncwarp();  // the masks are read before the next chunk writes them
    if (timed) s_tin[5] += global_ns() - t_b;
  });
  __syncthreads();
  if (gathered) {
    // sums over the chunks' masks (chunk c's at c * 2KM)
    const unsigned long long t_g = tmain ? global_ns() : 0ull;
    const unsigned* vb = reinterpret_cast<const unsigned*>(smem_heap);
    constexpr int NP = RoundSmem<M>::NPAIR;
    if constexpr (M % 4 == 0 && M >= 8) {
      // thread (pair, i) makes CL(i, .) and CR(i, .) of its pair from
      // VE[a][i], VL[a][i] and the 16-byte rows VL[c][.], VE[c][.] of each
      // chunk; the K * M threads after them make S[x][k] = popc(VL & VE)
      const int t = threadIdx.x;
      if (t < NP * M) {
        const int pid = t / M, i = t % M;
        int a = 0, q = pid;  // pair (a, c), a < c, of pair_id
        while (q >= K - 1 - a) {
          q -= K - 1 - a;
          ++a;
        }
        const int c = a + 1 + q;
        if (c < Kn) {
          int cl[M], cr[M];
#pragma unroll
          for (int j = 0; j < M; ++j) cl[j] = cr[j] = 0;
          for (int w = 0; w < nchunks; ++w) {
            const unsigned* v = vb + w * (2 * K * M);
            const unsigned ea = v[(2 * a + 1) * M + i], la = v[(2 * a) * M + i];
#pragma unroll
            for (int h = 0; h < M / 4; ++h) {
              const uint4 x = reinterpret_cast<const uint4*>(v + (2 * c) * M)[h];
              const uint4 y = reinterpret_cast<const uint4*>(v + (2 * c + 1) * M)[h];
              cl[4 * h] += __popc(ea & x.x);  // VE[a][i] & VL[c][j]
              cl[4 * h + 1] += __popc(ea & x.y);
              cl[4 * h + 2] += __popc(ea & x.z);
              cl[4 * h + 3] += __popc(ea & x.w);
              cr[4 * h] += __popc(la & y.x);  // VL[a][i] & VE[c][j]
              cr[4 * h + 1] += __popc(la & y.y);
              cr[4 * h + 2] += __popc(la & y.z);
              cr[4 * h + 3] += __popc(la & y.w);
            }
          }
#pragma unroll
          for (int j = 0; j < M; ++j) {
            if (cl[j]) atomicAdd(&sm.CL[pid][i * M + j], cl[j]);
            if (cr[j]) atomicAdd(&sm.CR[pid][i * M + j], cr[j]);
          }
        }
      } else if (t < NP * M + K * M) {
        const int e = t - NP * M, xi = e / M, k = e % M;
        int sum = 0;
        if (xi < Kn)
          for (int w = 0; w < nchunks; ++w) {
            const unsigned* v = vb + w * (2 * K * M);
            sum += __popc(v[(2 * xi) * M + k] & v[(2 * xi + 1) * M + k]);
          }
        if (sum) atomicAdd(&sm.S[xi][k], sum);
      }
      static_assert(RoundSmem<M>::NPAIR * M + (M + 1) * M <= NM_THREADS, "a thread a (pair, i) and an S entry");
    } else {
      // one thread an entry of S, CL, CR (in that order, as laid out)
      constexpr int NSUM = K * M + 2 * NP * MM;
      for (int e = threadIdx.x; e < NSUM; e += NM_THREADS) {
        int sum = 0;
        if (e < K * M) {  // S[x][k] = rows with bit k and popcount N+1 = popc(VL & VE)
          const int xi = e / M, k = e % M;
          if (xi < Kn)
            for (int w = 0; w < nchunks; ++w) {
              const unsigned* v = vb + w * (2 * K * M);
              sum += __popc(v[(2 * xi) * M + k] & v[(2 * xi + 1) * M + k]);
            }
          if (sum) atomicAdd(&sm.S[xi][k], sum);
        } else {
          const int f = e - K * M, side = f / (NP * MM), rem = f % (NP * MM);
          const int pid = rem / MM, idx = rem % MM, i = idx / M, j = idx % M;
          int a = 0, q = pid;  // pair (a, c), a < c, of pair_id
          while (q >= K - 1 - a) {
            q -= K - 1 - a;
            ++a;
          }
          const int c = a + 1 + q;
          if (c < Kn)
            for (int w = 0; w < nchunks; ++w) {
              const unsigned* v = vb + w * (2 * K * M);
              sum += side == 0 ? __popc(v[(2 * a + 1) * M + i] & v[(2 * c) * M + j])   // CL: VE[a][i] & VL[c][j]
                               : __popc(v[(2 * a) * M + i] & v[(2 * c + 1) * M + j]);  // CR: VL[a][i] & VE[c][j]
            }
          if (sum) atomicAdd(side == 0 ? &sm.CL[pid][idx] : &sm.CR[pid][idx], sum);
        }
      }
    }
    if (tmain) s_tin[5] += global_ns() - t_g;
    __syncthreads();
  }
  if (tmain) s_tin[2] += global_ns() - t_in;
}

// Pop order of every ordered pair's swap heap (fact 4).  The sift steps are
// those of swap_heap_pop_order; what differs is how a heap is held:
//  - a comparison needs only the order of two keys, so a heap entry is one
//    word, key << 8 | swap index, where the key is (l + r, r) packed in
//    12 + 12 bits when every gain of the heap fits, else the 64-bit key's
//    rank among the heap's keys (how many are smaller; equal keys get equal
//    ranks), computed by one warp per heap;
//  - then one thread per heap runs the sift steps on slots kept in shared
//    memory as [slot][heap], a row being a multiple of 32 words, so every
//    lane reads and writes its own bank whatever slot it is at;
//  - the steps are latency chains of dependent loads, so a push loads the
//    whole ancestor path at once, and a pop walks down on children loaded a
//    level ahead and writes its path back once (heap_sift);
//  - the walk rarely needs more than the first few pops of a heap, so the
//    sift steps run alongside it and stop when it is done.
// This part makes the entries (all warps).
template <int M>
__device__ void rank_phase(RoundSmem<M>& sm) {
  constexpr int K = M + 1, MM = M * M, SL = (MM + 31) / 32;
  constexpr int HS = RoundSmem<M>::HSTR;
  constexpr int NW = NM_THREADS / 32;
  static_assert(MM <= 64, "swap index in 8 bits, rank in 8 bits");
  const int Kn = sm.K_, np = Kn * Kn;
  const int tid = threadIdx.x, lane = tid & 31;
  // the scratch heads the kernel's dynamic shared memory (declared here too so
  // that accesses compile as shared-memory ones)
  extern __shared__ uint4 smem_heap[];
  unsigned* slot = reinterpret_cast<unsigned*>(smem_heap);  // [MM][HS]
  unsigned* ent = slot + MM * HS;                           // [MM][HS]
  for (int pq = tid >> 5; pq < np; pq += NW) {  // entries, one warp per heap
    const int a = pq / Kn, b = pq % Kn;
    if (a == b && sm.mode != 2) continue;
    const int c = a * K + b;  // column of the ordered pair in ord, slots and entries
    long long key[SL];
    bool small = true;  // every gain of the heap within +-2047
    int lr[SL], rr[SL];
#pragma unroll
    for (int q = 0; q < SL; ++q) {
      const int idx = lane + 32 * q;
      key[q] = 0;
      lr[q] = 0;
      rr[q] = 0;
      if (idx < MM) {
        int l, r;
        pair_gains<M>(sm, a, b, idx, l, r);
        key[q] = swap_key(l, r);
        lr[q] = l + r;
        rr[q] = r;
        small = small && lr[q] >= -2047 && lr[q] <= 2047 && r >= -2047 && r <= 2047;
      }
    }
    const bool all_small = __all_sync(FULL, small);
    if (lane == 0) sm.hsmall[c] = all_small ? 1 : 0;
    if (all_small) {
      // the key itself, (l + r, r) in 12 + 12 bits, orders like swap_key
#pragma unroll
      for (int q = 0; q < SL; ++q)
        if (lane + 32 * q < MM)
          ent[(lane + 32 * q) * HS + c] =
              ((((unsigned)(lr[q] + 2048) << 12) | (unsigned)(rr[q] + 2048)) << 8) | (unsigned)(lane + 32 * q);
      continue;
    }
    unsigned rk[SL];
#pragma unroll
    for (int q = 0; q < SL; ++q) rk[q] = 0;
#pragma unroll 8
    for (int j = 0; j < MM; ++j) {
      long long kr = key[0];
#pragma unroll
      for (int q = 1; q < SL; ++q)
        if ((j >> 5) == q) kr = key[q];
      const long long kj = __shfl_sync(FULL, kr, j & 31);
#pragma unroll
      for (int q = 0; q < SL; ++q) rk[q] += kj < key[q] ? 1u : 0u;
    }
#pragma unroll
    for (int q = 0; q < SL; ++q)
      if (lane + 32 * q < MM) ent[(lane + 32 * q) * HS + c] = (rk[q] << 8) | (unsigned)(lane + 32 * q);
  }
  if (tid < K * K) sm.hprog[tid] = 0;
  if (tid == 0) sm.hstop = 0;
  __syncthreads();
}

// The sift steps of every heap, one thread each (threads 0 .. Kn*Kn - 1),
// running while the walk warp consumes the pops: after writing pop k of
// its pair to ord, a thread publishes k + 1 in hprog; it stops early once
// the walk has set hstop.
template <int M>
__device__ void heap_sift(RoundSmem<M>& sm) {
  constexpr int K = M + 1, MM = M * M;
  constexpr int HS = RoundSmem<M>::HSTR;
  constexpr int D = MM <= 4 ? 2 : MM <= 8 ? 3 : MM <= 16 ? 4 : MM <= 32 ? 5 : 6;  // ceil(log2(MM))
  const int Kn = sm.K_, np = Kn * Kn;
  const int tid = threadIdx.x;
  extern __shared__ uint4 smem_heap[];
  unsigned* slot = reinterpret_cast<unsigned*>(smem_heap);  // [MM][HS]
  const unsigned* ent = slot + MM * HS;                     // [MM][HS]
  volatile int* prog = sm.hprog;
  volatile int* stop = &sm.hstop;
  const int a = tid / Kn, b = tid % Kn, pq = a * K + b;
  if (tid < np && (a != b || sm.mode == 2)) {
    unsigned* hs = slot + pq;
    uint8_t* ord = &sm.ord[0][0] + pq;
    auto ld = [&](int i) { return hs[(i < MM ? i : MM - 1) * HS]; };
    // MM pushes: heap.push_back(v); __push_heap(first, len, 0, v).  The
    // ancestors of `len` are loaded together; keys do not decrease going up
    // a path, so the entry rises past exactly the ancestors with key <= its own.
    for (int len = 0; len < MM; ++len) {
      const unsigned kv = ent[len * HS + pq];
      int pn[D + 1];
      unsigned av[D];
      pn[0] = len;
#pragma unroll
      for (int t = 0; t < D; ++t) {
        pn[t + 1] = pn[t] > 0 ? (pn[t] - 1) >> 1 : 0;
        av[t] = hs[pn[t + 1] * HS];
      }
      int m = 0;
#pragma unroll
      for (int t = 0; t < D; ++t) m += (pn[t] > 0 && (av[t] >> 8) <= (kv >> 8)) ? 1 : 0;
      int pm = pn[0];
#pragma unroll
      for (int t = 0; t < D; ++t) {
        if (t < m) hs[pn[t] * HS] = av[t];
        if (t + 1 == m) pm = pn[t + 1];
      }
      hs[pm * HS] = kv;
    }
    // MM pops: pop_heap(first, last) then pop_back().  __adjust_heap's walk
    // down to a leaf reads only children of the path, so it runs on values
    // loaded one level ahead, keeps the path in registers, finishes the
    // __push_heap of the old last entry there, and writes the path once.
    for (int len = MM, k = 0; len > 0; --len, ++k) {
      if (*stop) break;
      ord[k * HS] = (uint8_t)(hs[0] & 255u);
      __threadfence_block();
      prog[pq] = k + 1;
      if (len == 1) break;
      const int last = len - 1, lim = (last - 1) / 2;
      const unsigned kv = hs[last * HS];
      unsigned c1 = ld(1), c2 = ld(2), g0 = ld(3), g1 = ld(4), g2 = ld(5), g3 = ld(6);
      unsigned pv[D + 2];  // values moved up along the path, root first
      unsigned right = 0;  // bit t: step t of the path went to the right child
      int d = 0, second = 0;
#pragma unroll
      for (int lv = 0; lv < D; ++lv) {
        if (second < lim) {  // c1, c2: children of `second`; g0..g3: their children
          const bool left = (c2 >> 8) <= (c1 >> 8);
          const int x = left ? 2 * second + 1 : 2 * second + 2;
          pv[lv] = left ? c1 : c2;
          right |= left ? 0u : 1u << lv;
          d = lv + 1;
          second = x;
          c1 = left ? g0 : g2;
          c2 = left ? g1 : g3;
          g0 = ld(4 * x + 3);
          g1 = ld(4 * x + 4);
          g2 = ld(4 * x + 5);
          g3 = ld(4 * x + 6);
        }
      }
      if ((last & 1) == 0 && second == (last - 2) / 2) {  // one child left: c1, a left step
#pragma unroll
        for (int t = 0; t <= D; ++t)
          if (t == d) pv[t] = c1;
        ++d;
      }
      int m = 0;
#pragma unroll
      for (int t = 0; t <= D; ++t) m += (t < d && (pv[t] >> 8) <= (kv >> 8)) ? 1 : 0;
      const int cut = d - m;  // kv lands at path position cut, the rest below it move down one
      int node = 0;
#pragma unroll
      for (int t = 0; t <= D + 1; ++t) {
        if (t <= d) hs[node * HS] = t < cut ? pv[t] : (t == cut ? kv : pv[t > 0 ? t - 1 : 0]);
        node = 2 * node + 1 + (int)((right >> t) & 1u);
      }
    }
  }
}

// The greedy walk of run_onepair* over this round's segments, on one warp.
// Lane q holds round segment q: its current count and visited bits.  The
// list is a set (the primary is the list's top and the targets follow in
// traversal order, both strict total orders on (count, segment)), kept as
// a lane mask; each step is a few warp votes and shuffles:
//   - primary: the largest list key among the list's lanes; its visited
//     bits then live in a register of every lane for the pass;
//   - targets: each lane's position in traversal order by comparing keys,
//     inverted once per pass into a list of the targets' lanes;
//   - the first unvisited swap of a pair's pop order: the unique largest
//     qualifying key read off the entries, else a ballot over the pops;
//   - each committed swap's bit moves go straight into dest.
__device__ __forceinline__ unsigned order_key_hi(int c, bool rev) {  // count, order-preserving
  const unsigned u = (unsigned)c ^ 0x80000000u;
  return rev ? ~u : u;
}
__device__ __forceinline__ unsigned order_key_lo(int s, bool rev) {  // segment: ascending first for cmp
  return rev ? (unsigned)s : ~(unsigned)s;
}

// Runs on the block's last warp while heap_sift fills ord: a pair's pops
// are read as far as its heap has published them, waiting (with a limit)
// only when the first unvisited swap lies beyond.
constexpr int WALK_WAIT_LIMIT = 1 << 20;

template <int M>
__device__ void walk_phase(RoundSmem<M>& sm, int sched, int wait_limit) {
  constexpr int K = M + 1, MM = M * M;
  constexpr int HS = RoundSmem<M>::HSTR;
  constexpr unsigned FULLM = (1u << M) - 1u;
  constexpr int U = (MM + 31) / 32;  // swaps per lane
  const int lane = threadIdx.x & 31;
  volatile int* prog = sm.hprog;
  extern __shared__ uint4 smem_heap[];
  const unsigned* ent = reinterpret_cast<const unsigned*>(smem_heap) + MM * HS;  // [MM][HS], as rank_phase wrote
  bool dead = false;  // a wait ran out: the job is failed, finish without reading ord
  // pops of pair column `col` published so far, once at least `need`; -1 at the limit
  unsigned long long waited = 0;  // ns spent waiting for pops (lane 0)
  auto wait_pops = [&](int col, int need) -> int {
    int avail = __shfl_sync(FULL, prog[col], 0);
    if (avail >= need) {
      __threadfence_block();
      return avail;
    }
    const unsigned long long t_w = global_ns();
    for (int spin = 0; avail < need; ++spin) {
      if (spin >= wait_limit) return -1;
      avail = __shfl_sync(FULL, prog[col], 0);
    }
    __threadfence_block();
    waited += global_ns() - t_w;
    return avail;
  };
  // bit moves of the swaps for the recount (identity elsewhere)
  for (int t = lane; t < K * M; t += 32) (&sm.dest[0][0])[t] = (uint8_t)(((t / M) << 4) | (t % M));
  __syncwarp();
  int nsw = 0;
  const uint8_t* ord0 = &sm.ord[0][0];
  auto commit = [&](int a, int b, int idx) {  // lane 0 writes; every lane counts
    const int i = idx / M, j = idx % M;
    if (lane == 0) {
      sm.swaps[2 * nsw] = sm.xseg[a] * M + i;
      sm.swaps[2 * nsw + 1] = sm.xseg[b] * M + j;
      sm.dest[a][i] = (uint8_t)((b << 4) | j);
      sm.dest[b][j] = (uint8_t)((a << 4) | i);
    }
    ++nsw;
  };
  if (sm.mode != 0) {
    // |L| == 1: best pair of (top, minseg) with no visited filter (:1837-1860)
    const int b = sm.mode == 2 ? 0 : 1;
    int pick = 0;
    if (wait_pops(0 * K + b, 1) < 0) dead = true;
    else pick = ord0[0 * K + b];
    commit(0, b, pick);
  } else {
    const bool rev_list = sched >= 2;                  // inv_seg_list / updatePQ comparator
    const bool trav_rev = (sched == 1 || sched == 2);  // traversal comparator is cmp_reverse
    const int Kn = sm.K_;
    const int seg = lane < Kn ? sm.xseg[lane] : 0;
    int cnt = lane < Kn ? sm.xcnt[lane] : 0;
    unsigned vis = 0;
    unsigned Wm = (1u << Kn) - 1u;
    while (__popc(Wm) >= 2) {
      const bool inW = (Wm >> lane) & 1u;
      // primary = top of the list (largest key; 0 marks lanes outside it)
      const unsigned lh = inW ? order_key_hi(cnt, rev_list) : 0u, ll = inW ? order_key_lo(seg, rev_list) : 0u;
      const unsigned mh = __reduce_max_sync(FULL, lh);
      const unsigned ml = __reduce_max_sync(FULL, lh == mh ? ll : 0u);
      const int pxi = __ffs(__ballot_sync(FULL, inW && lh == mh && ll == ml)) - 1;
      int pc = __shfl_sync(FULL, cnt, pxi);
      unsigned vp = __shfl_sync(FULL, vis, pxi);  // the primary's visited bits, on every lane
      const int sp = __shfl_sync(FULL, seg, pxi);
      // targets: the rest of the list, by position in traversal order
      const unsigned Tm = Wm & ~(1u << pxi);
      const bool isT = (Tm >> lane) & 1u;
      const unsigned th = isT ? order_key_hi(cnt, trav_rev) : 0u, tl = isT ? order_key_lo(seg, trav_rev) : 0u;
      int pos = 0;
#pragma unroll
      for (int q = 0; q < K; ++q) {
        const unsigned qh = __shfl_sync(FULL, th, q), ql = __shfl_sync(FULL, tl, q);
        pos += (((Tm >> q) & 1u) && (qh > th || (qh == th && ql > tl))) ? 1 : 0;
      }
      // lane x: the lane of the x-th target
      int tx = 0;
#pragma unroll
      for (int q = 0; q < K; ++q) {
        const int pq = __shfl_sync(FULL, pos, q);
        if (((Tm >> q) & 1u) && pq == lane) tx = q;
      }
      const int nT = __popc(Tm);
      unsigned Um = 0;
      for (int x = 0; x < nT; ++x) {
        if (pc <= 0 || vp == FULLM) break;
        const int txi = __shfl_sync(FULL, tx, x);
        const unsigned vt = __shfl_sync(FULL, vis, txi);
        int tc = __shfl_sync(FULL, cnt, txi);
        // First pop of the pair whose two nodes are both unvisited.  A heap
        // pops in non-increasing key order, so that is the qualifying swap of
        // largest key when only one has it (read off the entries); on a tie
        // it is the first of them in the pops published so far, waiting for
        // more while none qualifies.
        const int col = pxi * K + txi;
        const uint8_t* ord = ord0 + col;
        int pick = -1, seen = 0;
        unsigned pe = ~0u;  // the pick's entry word, when read off the entries
        {
          unsigned eo[U];  // this lane's entries: entry k holds swap k
          unsigned kq[U];  // key + 1 of this lane's qualifying swaps, else 0
          unsigned best = 0;
#pragma unroll
          for (int u = 0; u < U; ++u) {
            const int k = lane + 32 * u;
            const unsigned e = k < MM ? ent[k * HS + col] : 0u;
            eo[u] = e;
            const bool ok = k < MM && !((vp >> (k / M)) & 1u) && !((vt >> (k % M)) & 1u);
            kq[u] = ok ? (e >> 8) + 1u : 0u;
            best = max(best, __reduce_max_sync(FULL, kq[u]));
          }
          int nbest = 0, who = -1;
#pragma unroll
          for (int u = 0; u < U; ++u) {
            const unsigned bb = __ballot_sync(FULL, best != 0u && kq[u] == best);
            nbest += __popc(bb);
            if (bb && who < 0) who = 32 * u + __ffs(bb) - 1;
          }
          if (nbest == 1) {  // swap index == entry position
            pick = who;
            unsigned ep = eo[0];
#pragma unroll
            for (int u = 1; u < U; ++u)
              if ((pick >> 5) == u) ep = eo[u];
            pe = __shfl_sync(FULL, ep, pick & 31);
          }
        }
        while (pick < 0 && !dead) {
          if (seen >= MM) {  // unreachable: a scored target always has an unvisited node
            if (lane == 0) sm.status |= JOB_EMPTY_HEAP;
            pick = ord[(MM - 1) * HS];
            break;
          }
          const int avail = wait_pops(col, seen + 1);
          if (avail < 0) {
            dead = true;
            break;
          }
          for (int k0 = seen; k0 < avail && pick < 0; k0 += 32) {
            const int k = k0 + lane;
            const int e = k < avail ? ord[k * HS] : 0;
            const bool ok = k < avail && !((vp >> (e / M)) & 1u) && !((vt >> (e % M)) & 1u);
            const unsigned bal = __ballot_sync(FULL, ok);
            if (bal) pick = __shfl_sync(FULL, e, __ffs(bal) - 1);
          }
          seen = avail;
        }
        if (dead) pick = 0;
        int l, r;
        if (sm.hsmall[col]) {  // the gains are the pick's key: (l + r + 2048) << 12 | (r + 2048)
          if (pe == ~0u || dead) pe = ent[pick * HS + col];  // picked from the pops
          const unsigned key = pe >> 8;
          r = (int)(key & 4095u) - 2048;
          l = (int)(key >> 12) - 2048 - r;
        } else {
          pair_gains<M>(sm, pxi, txi, pick, l, r);
        }
        const int i = pick / M, j = pick % M;
        if (lane == 0) {
          sm.swaps[2 * nsw] = sp * M + i;
          sm.swaps[2 * nsw + 1] = sm.xseg[txi] * M + j;
          sm.dest[pxi][i] = (uint8_t)((txi << 4) | j);
          sm.dest[txi][j] = (uint8_t)((pxi << 4) | i);
        }
        ++nsw;
        vp |= 1u << i;
        if (lane == txi) vis |= 1u << j;
        pc -= l;
        tc -= r;
        if (lane == txi) cnt = tc;
        if (tc > 0) Um |= 1u << txi;
      }
      if (lane == pxi) vis = vp;
      Wm = Um;
    }
  }
  if (lane == 0) {
    sm.nswaps = nsw;
    if (dead) sm.status |= JOB_WAIT_LIMIT;
    *(volatile int*)&sm.hstop = 1;
    s_tin[1] += waited;
  }
}

// Apply the swaps to orig[] (the leader block) and recount this block's
// slice of the touched rows into newinv / newpres.
template <int M>
__device__ void apply_recount(RoundSmem<M>& sm, const NMJob& J, int N, Slice sl) {
  constexpr int K = M + 1;
  const int tid = threadIdx.x;
  // a round's swaps are disjoint transpositions (the walk never reuses a
  // visited position), so each thread applies one of them
  if (sl.rank == 0 && tid < sm.nswaps) {
    const int v1 = sm.swaps[2 * tid], v2 = sm.swaps[2 * tid + 1];
    const int o1 = J.orig[v1], o2 = J.orig[v2];
    J.orig[v1] = o2;
    J.orig[v2] = o1;
  }
  const int Kn = sm.K_;
  const int lane = tid & 31;
  // where the bits of each nibble of each segment's group go, packed like
  // the record (4 segments per word): one table entry per (segment, nibble
  // position, nibble value)
  constexpr int NH = (M + 3) / 4;
  extern __shared__ uint4 smem_heap[];
  uint4 (*bitmove)[NH][16] = reinterpret_cast<uint4 (*)[NH][16]>(smem_heap);  // [K][NH][16]
  static_assert((M + 1) * NH * 16 * 16 <= RoundSmem<M>::PROC_BYTES, "bit-move table fits the scratch");
  for (int t = tid; t < Kn * NH * 16; t += NM_THREADS) {
    const int xi = t / (NH * 16), h = (t / 16) % NH, v = t % 16;
    unsigned o[3] = {0u, 0u, 0u};
    for (int q = 0; q < 4; ++q) {
      const int k = 4 * h + q;
      if (k < M && ((v >> q) & 1)) {
        const int d = sm.dest[xi][k];
        const int dx = d >> 4, dk = d & 15;
        o[dx >> 2] |= (1u << dk) << ((dx & 3) * 8);
      }
    }
    bitmove[xi][h][v] = make_uint4(o[0], o[1], o[2], 0u);
  }
  __syncthreads();
  const bool tmain = threadIdx.x == 0 && sl.rank == 0 && J.timed;
  const unsigned long long t_in = tmain ? global_ns() : 0ull;
  for_rows_warp<M, 2>(sm, J, [&](int r, const uint4& w, bool valid, int chunk) {
    (void)chunk;
    // the row's groups after the swaps, packed like the record
    unsigned n0 = 0, n1 = 0, n2 = 0;
#pragma unroll
    for (int xi = 0; xi < K; ++xi) {
      const unsigned bb = (valid && xi < Kn) ? rec_byte(w, xi) : 0u;
#pragma unroll
      for (int h = 0; h < NH; ++h) {
        const unsigned nib = (bb >> (4 * h)) & 15u;
        if (nib) {
          const uint4 m = bitmove[xi][h][nib];
          n0 |= m.x;
          n1 |= m.y;
          n2 |= m.z;
        }
      }
    }
    // non-empty and invalid groups per segment, one shared add per warp
#pragma unroll
    for (int xi = 0; xi < K; ++xi) {
      if (xi >= Kn) break;
      const unsigned nb = ((xi < 4 ? n0 : (xi < 8 ? n1 : n2)) >> ((xi & 3) * 8)) & 0xffu;
      const unsigned pres = __ballot_sync(FULL, nb != 0u);
      const unsigned inv = __ballot_sync(FULL, __popc(nb) > N);
      if (lane == 0 && pres) atomicAdd(&sm.newpres[xi], __popc(pres));
      if (lane == 0 && inv) atomicAdd(&sm.newinv[xi], __popc(inv));
    }
    if (valid) {
      if (sm.use_table) sm.table[r] = make_uint4(0u, 0u, 0u, 0u);
      else J.rec[r] = make_uint4(0u, 0u, 0u, 0u);
    }
  });
  if (tmain) s_tin[3] += global_ns() - t_in;
  __syncthreads();
  if (threadIdx.x == 0) sm.tcount = 0;  // the table is empty again (before the next round's inserts)
}

// The new counts of the round's segments (leader block), and the leader's
// partial sums cleared for the next round: the walk read the scores last,
// and each thread clears the recount words it read (what clear_round_smem
// does, without a barrier of its own).
template <int M>
__device__ void apply_finish(RoundSmem<M>& sm, const NMJob& J, int* cnt) {
  constexpr int K = M + 1;
  const int tid = threadIdx.x;
  if (tid < K) {
    if (tid < sm.K_) {
      cnt[sm.xseg[tid]] = sm.newinv[tid];
      J.zc[sm.xseg[tid]] = J.R - sm.newpres[tid];
    }
    sm.newinv[tid] = 0;
    sm.newpres[tid] = 0;
  }
  for (int i = tid; i < K * M; i += NM_THREADS) (&sm.S[0][0])[i] = 0;
  for (int i = tid; i < RoundSmem<M>::NPAIR * RoundSmem<M>::MM; i += NM_THREADS) {
    (&sm.CL[0][0])[i] = 0;
    (&sm.CR[0][0])[i] = 0;
  }
  if (tid == 0) {
    sm.ntouched = 0;
    sm.nswaps = 0;
  }
  __syncthreads();
}

// Helper block: add its nonzero partial sums of n ints at `mine` into the
// leader's copy (remote atomics, complete at the next cluster barrier) and
// clear them for the next round (nothing reads them again this round).
__device__ void cluster_push(cg::cluster_group& cl, int* mine, int n) {
  int* lead_arr = cl.map_shared_rank(mine, 0);
  for (int i = threadIdx.x; i < n; i += NM_THREADS) {
    const int v = mine[i];
    if (v) {
      atomicAdd(lead_arr + i, v);
      mine[i] = 0;
    }
  }
}

// All rounds of a job.  With cs == 1 one thread block runs the job; with
// cs > 1 the job runs on a thread-block cluster of cs blocks: the leader
// (rank 0) runs the sequential parts (segment choice, heaps, walk, counts)
// and every block gathers, scores and recounts the rows it owns (row_group
// in its share of the 16 groups), the partial sums meeting in the leader's
// shared memory.  A round has four cluster barriers: after the round's
// segments reach every block, after the partial sums of the scores, after
// the swaps reach every block, and after the partial recounts.  Every
// block runs the same sequence of them: the leader's decision to run a
// round is copied to every block before the barrier that opens it.
template <int M>
__global__ void __launch_bounds__(NM_THREADS, 1) k_nm_rounds(const NMJob* __restrict__ jobs, int N,
                                                              int cnt_in_smem, int ts_max, int cs, int rcache_on) {
  constexpr int K = M + 1;
  __shared__ RoundSmem<M> sm;
  static_assert(offsetof(RoundSmem<M>, CL) == offsetof(RoundSmem<M>, S) + sizeof(int) * K * M, "S, CL adjacent");
  static_assert(offsetof(RoundSmem<M>, CR) == offsetof(RoundSmem<M>, CL) + sizeof(int) * RoundSmem<M>::NPAIR *
                                                                              RoundSmem<M>::MM, "CL, CR adjacent");
  static_assert(offsetof(RoundSmem<M>, newpres) == offsetof(RoundSmem<M>, newinv) + sizeof(int) * K,
                "newinv, newpres adjacent");
  constexpr int NSUM = K * M + 2 * RoundSmem<M>::NPAIR * RoundSmem<M>::MM;
  // dynamic shared memory: [heap scratch][row-record table: ts_max x 16 B]
  // [claimed-slot list: ts_max x 4 B][record cache: NM_THREADS x TOUCH_U x
  // (16 + 4) B, when on][segment counts]
  extern __shared__ uint4 smem_heap[];
  uint4* smem_dyn = smem_heap + RoundSmem<M>::SCR_U4;
  int* smem_list = reinterpret_cast<int*>(smem_dyn + ts_max);
  uint4* smem_rcache = reinterpret_cast<uint4*>(smem_list + ts_max);
  int* smem_rcrow = reinterpret_cast<int*>(smem_rcache + (rcache_on ? NM_THREADS * TOUCH_U : 0));
  int* smem_cnt = smem_rcrow + (rcache_on ? NM_THREADS * TOUCH_U : 0);
  cg::cluster_group cl = cg::this_cluster();
  const int rank = cs > 1 ? (int)cl.block_rank() : 0;
  const bool lead = rank == 0;
  const Slice sl{rank, cs};
  __shared__ unsigned long long g_start;  // the kernel's start (thread 0 of the leader), global timer
  if (threadIdx.x == 0) g_start = global_ns();
  const NMJob J = jobs[blockIdx.x / cs];
  if (J.err && *J.err) return;  // every block of the cluster reads the same flag, before any barrier
  const int tid = threadIdx.x;
  int* cnt = cnt_in_smem ? smem_cnt : J.cnt;
  if (lead && cnt_in_smem)
    for (int s = tid; s < J.nseg; s += NM_THREADS) smem_cnt[s] = J.cnt[s];
  for (int i = tid; i < ts_max; i += NM_THREADS) smem_dyn[i] = make_uint4(0u, 0u, 0u, 0u);
  if (tid == 0) {
    sm.status = JOB_OK;
    sm.table = ts_max > 0 ? smem_dyn : nullptr;
    sm.tlist = ts_max > 0 ? smem_list : nullptr;
    sm.rcache = rcache_on ? smem_rcache : nullptr;
    sm.rcrow = rcache_on ? smem_rcrow : nullptr;
    sm.tcount = 0;
    sm.toff = rank * ((J.R + ROW_GROUPS - 1) / ROW_GROUPS + 1) * (ROW_GROUPS / cs);
    for (int q = 0; q < 4; ++q) sm.acc[q] = 0ull;
    sm.ts_max = ts_max;
    sm.ts_shift = 32 - (31 - __clz(ts_max > 0 ? ts_max : 1));
    sm.use_table = 0;
    sm.go = 0;
  }
  clear_round_smem<M>(sm);
  __syncthreads();
  if (lead) select_phase<M>(sm, J, cnt);
  const int init_size = sm.lsize, init_cnt = sm.ltotal;
  const int MAXITER = J.maxiter > init_size ? J.maxiter : init_size;  // reorder.h:1819
  int round = 1;
  int committed = 0;
  // this block's work counters: gathered entries, touched rows, rounds with
  // the records in the shared-memory table, rounds with them in global
  // memory (thread 0; in shared memory, as registers are scarce)
  __shared__ unsigned long long wk[4];
  if (tid == 0)
    for (int q = 0; q < 4; ++q) wk[q] = 0ull;
  // time spent in each phase of a round (ns, global timer), measured by
  // thread 0 of the leader at the barriers that end the phases: select,
  // choose, gather, process, heap, walk, apply.  (The SM cycle counter
  // undercounted the waits at cluster barriers: its phase sums fell short of
  // the kernel's time by up to 40 %.)  In shared memory: only thread 0 uses
  // them, and registers are scarce.
  __shared__ unsigned long long tph[7];
  __shared__ unsigned long long tpo[2];  // the leader's own work in the process and apply phases
  __shared__ unsigned long long t0;
  // (global timer reads on the leader's critical path cost ~2.5 % of the
  // kernel's time, so they are made only when the caller asks: J.timed)
  const bool timed = J.timed != 0;
  if (tid == 0) {
    for (int q = 0; q < 7; ++q) tph[q] = 0;
    tpo[0] = tpo[1] = 0;
    for (int q = 0; q < 6; ++q) s_tin[q] = 0;
    t0 = timed ? global_ns() : 0ull;
  }
#define VNM_PHASE(i)                                     \
  if (tid == 0 && timed) {                               \
    const unsigned long long t1 = global_ns();           \
    tph[i] += t1 - t0;                                   \
    t0 = t1;                                             \
  }
  if (cs > 1) cl.sync();  // every block's shared memory is set up before any remote access
  for (;;) {
    if (lead) {
      if (tid == 0) sm.go = (round <= MAXITER && sm.lsize >= 1 && sm.status == JOB_OK) ? 1 : 0;
      __syncthreads();
      if (sm.go) {
        if (sm.lsize == 1) minseg_phase<M>(sm, J);
        VNM_PHASE(0);
        choose_segments<M>(sm, J.sched);
        __syncthreads();
        VNM_PHASE(1);
      }
      // the round's segments to every block, one remote store a thread (a
      // thread issuing them all in turn took ~4 K cycles a round)
      constexpr int F = K + 3;
      if (tid < (cs - 1) * F) {
        const int f = tid % F;
        RoundSmem<M>* rs = cl.map_shared_rank(&sm, 1 + tid / F);
        if (f < K) rs->xseg[f] = sm.xseg[f];
        else if (f == K) rs->go = sm.go;
        else if (f == K + 1) rs->K_ = sm.K_;
        else rs->mode = sm.mode;
      }
    }
    if (cs > 1) cl.sync();
    if (!sm.go) break;  // the same decision in every block of the job
    // (a helper cleared its partial sums as it pushed them last round, the
    // leader in apply_finish)
    // the block's own rows: no barrier between its gather and its process phase
    gather_phase<M>(sm, J, sl);
    if (tid == 0) {
      wk[0] += (unsigned)sm.E;
      wk[1] += (unsigned)sm.ntouched;
      wk[sm.use_table ? 2 : 3] += 1;
    }
    VNM_PHASE(2);
    process_phase<M>(sm, J, N, sl);
    if (tid == 0 && timed) tpo[0] += global_ns() - t0;  // the leader's own part of the process phase
    if (cs > 1) {
      // (the leader pulling the helpers' sums over DSMEM instead was slower:
      // 8.92 against 8.55 ms at R-MAT 16384 2:4, 200.5 against 197.2 ms at
      // R-MAT 65536 2:8)
      if (!lead) cluster_push(cl, &sm.S[0][0], NSUM);
      cl.sync();
      if (!lead) {  // while the leader runs the heaps and the walk: next round's scan
        const int nh = cs - 1, hr = rank - 1;
        const int sb = (int)((long long)J.nseg * hr / nh), se = (int)((long long)J.nseg * (hr + 1) / nh);
        select_range<M>(sm, cnt_in_smem ? cl.map_shared_rank(smem_cnt, 0) : J.cnt, sb, se, sm.xseg, sm.K_);
        // the scan's result into the leader's shared memory, read there
        // after the barrier that follows the walk
        RoundSmem<M>* ls = cl.map_shared_rank(&sm, 0);
        if (tid < 2 * K) ls->sel_top[hr][tid / K][tid % K] = sm.top[tid / K][tid % K];
        else if (tid < 2 * K + 2) ls->sel_ls[hr][tid - 2 * K] = tid == 2 * K ? sm.lsize : sm.ltotal;
      }
    }
    VNM_PHASE(3);
    if (lead) {
      rank_phase<M>(sm);
      VNM_PHASE(4);
      const unsigned long long t_in = (tid == NM_THREADS - 32 && timed) ? global_ns() : 0ull;
      if (tid >= NM_THREADS - 32) walk_phase<M>(sm, J.sched, J.walk_wait_limit);  // the last warp walks ...
      else if (!J.hold_heaps) heap_sift<M>(sm);                                   // ... while the heaps pop
      if (tid == NM_THREADS - 32 && timed) s_tin[0] += global_ns() - t_in;
      __syncthreads();
      VNM_PHASE(5);
      if (tid == 0 && J.trace_pairs) {
        for (int q = 0; q < sm.nswaps; ++q) {
          if (committed < J.trace_cap_pairs) {
            J.trace_pairs[2 * committed] = sm.swaps[2 * q];
            J.trace_pairs[2 * committed + 1] = sm.swaps[2 * q + 1];
          }
          ++committed;
        }
        if (round - 1 < J.trace_cap_rounds) J.trace_rounds[round - 1] = committed;
      }
      // where each bit of the round's segments goes, to every block (one
      // remote word store a thread)
      constexpr int DW = RoundSmem<M>::DEST_W;
      if (tid < (cs - 1) * DW) {
        RoundSmem<M>* rs = cl.map_shared_rank(&sm, 1 + tid / DW);
        rs->dest_w[tid % DW] = sm.dest_w[tid % DW];
      }
    }
    if (cs > 1) cl.sync();
    apply_recount<M>(sm, J, N, sl);
    if (tid == 0 && timed) tpo[1] += global_ns() - t0;  // the leader's own part of the apply phase
    if (cs > 1) {
      if (!lead) {
        cluster_push(cl, &sm.newinv[0], 2 * K);
        if (tid == 0) sm.ntouched = 0;  // (read last by the recount, before its closing __syncthreads)
      }
      cl.sync();
    }
    if (lead) {
      apply_finish<M>(sm, J, cnt);  // also clears the leader's sums for the next round
      VNM_PHASE(6);
      if (cs > 1) select_merge<M>(sm, cl, cs, cnt);
      else select_phase<M>(sm, J, cnt);
    }
    round += 1;
  }
#undef VNM_PHASE
  if (cs > 1) {  // the helpers' counters to the leader
    if (!lead && tid == 0) {
      unsigned long long* acc = cl.map_shared_rank(&sm.acc[0], 0);
      for (int q = 0; q < 4; ++q) atomicAdd(acc + q, wk[q]);
    }
    cl.sync();
  }
  if (!lead) return;
  if (tid == 0)
    for (int q = 0; q < 4; ++q) wk[q] += sm.acc[q];
  if (cnt_in_smem)
    for (int s = tid; s < J.nseg; s += NM_THREADS) J.cnt[s] = smem_cnt[s];
  if (tid == 0) {
    J.res[0] = init_size;
    J.res[1] = sm.lsize;
    J.res[2] = init_cnt;
    J.res[3] = sm.ltotal;
    J.res[4] = round - 1;
    J.res[5] = sm.status;
    J.res[6] = committed;
    J.res[7] = (int)(wk[0] & 0x7fffffffull);
    J.res[8] = (int)(wk[0] >> 31);
    J.res[9] = (int)(wk[1] & 0x7fffffffull);
    J.res[10] = (int)(wk[1] >> 31);
    J.res[11] = (int)wk[2];
    J.res[12] = (int)wk[3];
    for (int q = 0; q < 7; ++q) J.res[16 + q] = (int)(tph[q] >> 10);  // units of 1024 ns
    J.res[24] = (int)(tpo[0] >> 10);
    J.res[25] = (int)(tpo[1] >> 10);
    for (int q = 0; q < 6; ++q) J.res[26 + q] = (int)(s_tin[q] >> 10);
    const unsigned long long g_end = global_ns();
    J.res[23] = (int)((g_end - g_start) >> 10);
    J.res[13] = (int)((g_start >> 10) & 0x7fffffffull);  // start and end, in units of 1024 ns
    J.res[14] = (int)((g_end >> 10) & 0x7fffffffull);
  }
}

// One segment pair's full gain table (GetSegSwapScore) through the same
// phases the round kernel uses; orig is the identity here.
template <int M>
__global__ void __launch_bounds__(NM_THREADS) k_pair_score(NMJob J, int N, int s1, int s2, int* score) {
  __shared__ RoundSmem<M> sm;  // + RoundSmem<M>::SCR_U4 x 16 B of dynamic scratch
  clear_round_smem<M>(sm);
  if (threadIdx.x == 0) {
    sm.table = nullptr;
    sm.ts_max = 0;
    sm.use_table = 0;
    sm.toff = 0;
    sm.rcache = nullptr;
    sm.rcrow = nullptr;
    sm.xseg[0] = s1;
    sm.xcnt[0] = 0;
    if (s1 == s2) {
      sm.mode = 2;
      sm.K_ = 1;
    } else {
      sm.mode = 1;
      sm.xseg[1] = s2;
      sm.xcnt[1] = 0;
      sm.K_ = 2;
    }
  }
  __syncthreads();
  gather_phase<M>(sm, J);
  process_phase<M>(sm, J, N);
  const int b = s1 == s2 ? 0 : 1;
  for (int idx = threadIdx.x; idx < M * M; idx += NM_THREADS) {
    int l, r;
    pair_gains<M>(sm, 0, b, idx, l, r);
    score[2 * idx] = l;
    score[2 * idx + 1] = r;
  }
  __syncthreads();
  for (int t = threadIdx.x; t < sm.ntouched; t += NM_THREADS) J.rec[J.touched[t]] = make_uint4(0u, 0u, 0u, 0u);
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
static inline int grid_for(const vnm_ctx* ctx, long long n, int nt = 256) {
  long long g = (n + nt - 1) / nt;
  long long cap = (long long)ctx->num_sms * 8;
  if (g > cap) g = cap;
  return g < 1 ? 1 : (int)g;
}

size_t pattern_bytes(int R, int nnz) {
  size_t b = 0;
  b += arena_bytes(2, sizeof(int));              // the input check's flag and the entry count
  b += arena_bytes(nnz, sizeof(int));            // flags / positions
  b += 2 * arena_bytes(nnz, sizeof(int));        // prow, pcol
  const size_t ng = (size_t)ROW_GROUPS * R + 1;
  b += arena_bytes(R + 1, sizeof(int));          // cptr
  b += 2 * arena_bytes(ng, sizeof(int));         // group counts -> csplit, cfill
  b += arena_bytes(nnz, sizeof(int));            // crow
  b += 2 * arena_bytes(R / 2 + 1, sizeof(int));  // inv0, pres0 (nseg <= R/2)
  b += arena_bytes(1, sizeof(int)) * 2;          // totals
  b += scan_scratch_bytes((size_t)nnz > ng ? nnz : (int)ng) * 2;
  return b;
}

template <int M>
static vnm_status build_pattern_t(vnm_ctx* ctx, int R, int nnz, const int* d_row, const int* d_col,
                                  const float* d_val, int N, Pattern& P, int* h_scratch, bool deferred) {
  P.R = R;
  P.nseg = R / M;
  int* err = arena_take<int>(ctx, 2);  // [0] the input check's flag, [1] the pattern's entry count
  int* pos = arena_take<int>(ctx, nnz > 0 ? nnz : 1);
  P.prow = arena_take<int>(ctx, nnz > 0 ? nnz : 1);
  P.pcol = arena_take<int>(ctx, nnz > 0 ? nnz : 1);
  const size_t ng = (size_t)ROW_GROUPS * R + 1;
  P.cptr = arena_take<int>(ctx, R + 1);
  P.csplit = arena_take<int>(ctx, ng);
  int* cfill = arena_take<int>(ctx, ng);
  P.crow = arena_take<int>(ctx, nnz > 0 ? nnz : 1);
  P.inv0 = arena_take<int>(ctx, R / 2 + 1);
  P.pres0 = arena_take<int>(ctx, R / 2 + 1);
  int* d_tot = arena_take<int>(ctx, 1);
  if (!err || !pos || !P.prow || !P.pcol || !P.cptr || !P.csplit || !cfill || !P.crow || !P.inv0 || !P.pres0 ||
      !d_tot)
    return VNM_ERR_NOMEM;
  int* d_np = err + 1;
  P.d_err = err;
  VNM_CUDA_TRY(cudaMemsetAsync(err, 0, 2 * sizeof(int), ctx->stream));
  VNM_CUDA_TRY(cudaMemsetAsync(P.csplit, 0, sizeof(int) * ng, ctx->stream));
  VNM_CUDA_TRY(cudaMemsetAsync(cfill, 0, sizeof(int) * ng, ctx->stream));
  VNM_CUDA_TRY(cudaMemsetAsync(P.inv0, 0, sizeof(int) * (P.nseg + 1), ctx->stream));
  VNM_CUDA_TRY(cudaMemsetAsync(P.pres0, 0, sizeof(int) * (P.nseg + 1), ctx->stream));
  if (nnz > 0) {
    // indices are checked before any kernel uses them as addresses: here,
    // or (deferred) by the kernels themselves, which skip their work when
    // the flag is set
    VNM_LAUNCH(ctx, k_validate, grid_for(ctx, nnz), 256, 0, d_row, d_col, nnz, R, err);
    if (!deferred) {
      VNM_CUDA_TRY(cudaMemcpyAsync(h_scratch, err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
      VNM_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
      if (h_scratch[0] & 2) return VNM_ERR_RANGE;
      if (h_scratch[0] & 1) return VNM_ERR_UNSORTED;
    }
    VNM_LAUNCH(ctx, k_nonzero_flags, grid_for(ctx, nnz), 256, 0, d_val, nnz, pos);
    VNM_TRY(exclusive_scan(ctx, pos, pos, nnz, d_np));
    VNM_LAUNCH(ctx, k_compact, grid_for(ctx, nnz), 256, 0, d_row, d_col, d_val, pos, nnz, P.prow, P.pcol,
               P.csplit, err);
  }
  VNM_TRY(exclusive_scan(ctx, P.csplit, P.csplit, (int)ng, d_tot));
  VNM_LAUNCH(ctx, k_cptr_from_split, grid_for(ctx, (long long)R + 1), 256, 0, P.csplit, R, P.cptr);
  if (deferred) {
    // the entry count stays on the device (read back with the call's
    // results); the grids cover every stored entry
    P.np = -1;
    if (nnz > 0) {
      VNM_LAUNCH(ctx, k_csc_scatter, grid_for(ctx, nnz), 256, 0, P.prow, P.pcol, d_np, P.csplit, cfill, P.crow,
                 err);
      VNM_LAUNCH(ctx, k_locate<M>, grid_for(ctx, nnz), 256, 0, P.prow, P.pcol, d_np, N, P.inv0, P.pres0, err);
    }
    return VNM_OK;
  }
  VNM_CUDA_TRY(cudaMemcpyAsync(h_scratch + 1, d_np, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  VNM_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  P.np = h_scratch[1];
  if (P.np > 0) {
    VNM_LAUNCH(ctx, k_csc_scatter, grid_for(ctx, P.np), 256, 0, P.prow, P.pcol, d_np, P.csplit, cfill, P.crow,
               err);
    VNM_LAUNCH(ctx, k_locate<M>, grid_for(ctx, P.np), 256, 0, P.prow, P.pcol, d_np, N, P.inv0, P.pres0, err);
  }
  return VNM_OK;
}

vnm_status build_pattern(vnm_ctx* ctx, int R, int nnz, const int* d_row, const int* d_col, const float* d_val,
                         int N, int M, Pattern& P, int* h_scratch, bool deferred) {
  switch (M) {
    case 2: return build_pattern_t<2>(ctx, R, nnz, d_row, d_col, d_val, N, P, h_scratch, deferred);
    case 3: return build_pattern_t<3>(ctx, R, nnz, d_row, d_col, d_val, N, P, h_scratch, deferred);
    case 4: return build_pattern_t<4>(ctx, R, nnz, d_row, d_col, d_val, N, P, h_scratch, deferred);
    case 5: return build_pattern_t<5>(ctx, R, nnz, d_row, d_col, d_val, N, P, h_scratch, deferred);
    case 6: return build_pattern_t<6>(ctx, R, nnz, d_row, d_col, d_val, N, P, h_scratch, deferred);
    case 7: return build_pattern_t<7>(ctx, R, nnz, d_row, d_col, d_val, N, P, h_scratch, deferred);
    case 8: return build_pattern_t<8>(ctx, R, nnz, d_row, d_col, d_val, N, P, h_scratch, deferred);
  }
  return VNM_ERR_ARG;
}

size_t job_bytes(int R) {
  const int nseg = R / 2 + 1;
  return arena_bytes(R, sizeof(int)) + 2 * arena_bytes(nseg, sizeof(int)) + arena_bytes(R, sizeof(uint4)) +
         arena_bytes((size_t)R + 2 * ROW_GROUPS, sizeof(int)) + arena_bytes(JOB_RES, sizeof(int));
}

// Carve one job's state out of the arena and initialise it.
static vnm_status make_job(vnm_ctx* ctx, const Pattern& P, int sched, int maxiter, NMJob& J) {
  J.R = P.R;
  J.nseg = P.nseg;
  J.sched = sched;
  J.maxiter = maxiter;
  J.cptr = P.cptr;
  J.crow = P.crow;
  J.csplit = P.csplit;
  J.orig = arena_take<int>(ctx, P.R > 0 ? P.R : 1);
  J.cnt = arena_take<int>(ctx, P.nseg + 1);
  J.zc = arena_take<int>(ctx, P.nseg + 1);
  J.rec = arena_take<uint4>(ctx, P.R > 0 ? P.R : 1);
  J.touched = arena_take<int>(ctx, (size_t)P.R + 2 * ROW_GROUPS);
  J.res = arena_take<int>(ctx, JOB_RES);
  J.trace_pairs = nullptr;
  J.trace_rounds = nullptr;
  J.trace_cap_pairs = 0;
  J.trace_cap_rounds = 0;
  // Test hooks for the walk's bounded wait (a job whose wait runs out fails
  // with VNM_ERR_INTERNAL instead of hanging): VNM_NM_TEST_WAIT_LIMIT
  // lowers the poll limit, VNM_NM_TEST_HOLD_HEAPS=1 keeps the swap heaps
  // from publishing, so the first wait runs out.  Unset, they change nothing.
  J.walk_wait_limit = WALK_WAIT_LIMIT;
  J.hold_heaps = 0;
  J.err = nullptr;
  J.timed = ctx->phase_timing ? 1 : 0;
  if (const char* e = getenv("VNM_NM_TEST_WAIT_LIMIT")) {
    const int v = atoi(e);
    if (v > 0 && v < WALK_WAIT_LIMIT) J.walk_wait_limit = v;
  }
  if (const char* e = getenv("VNM_NM_TEST_HOLD_HEAPS")) J.hold_heaps = atoi(e) == 1 ? 1 : 0;
  if (!J.orig || !J.cnt || !J.zc || !J.rec || !J.touched || !J.res) return VNM_ERR_NOMEM;
  VNM_CUDA_TRY(cudaMemsetAsync(J.rec, 0, sizeof(uint4) * (P.R > 0 ? P.R : 1), ctx->stream));
  VNM_CUDA_TRY(cudaMemsetAsync(J.res, 0, sizeof(int) * JOB_RES, ctx->stream));
  if (P.R > 0)
    VNM_LAUNCH(ctx, k_init_job, grid_for(ctx, P.R), 256, 0, J.orig, J.cnt, J.zc, P.inv0, P.pres0, P.R, P.nseg);
  return VNM_OK;
}

// Shared memory beyond RoundSmem: the swap-heap scratch, the segment counts when
// they are small (<= 64 KB), and a row-record table of up to 8192 16-byte
// slots in what is left of a 150 KB budget (the rest of the SM's 256 KB is L1,
// which the gather phase's reads of the column pattern live on: 200 KB ran the
// 256-matrix 2:8 batch 4 % slower when it used one block per job).
constexpr size_t NM_SMEM_BUDGET = 150u << 10;

// k_nm_rounds<M>'s dynamic shared-memory ceiling depends on the call (the
// segment counts and the table size), and it is a property of the function
// shared by every host thread: one lock
// covers each setting of it together with the launch it is for, so that a
// call on another thread cannot lower it in between.
static std::mutex g_round_launch_mu;

template <int M>
static vnm_status launch_rounds_t(vnm_ctx* ctx, const NMJob* d_jobs, int njobs, int N, int max_nseg, int cs) {
  std::lock_guard<std::mutex> launch_lock(g_round_launch_mu);
  ctx->last_clusters_fit = 0;
  const size_t cbytes = (size_t)max_nseg * sizeof(int);
  const int in_smem = cbytes <= (64u << 10) ? 1 : 0;
  const size_t hbytes = (size_t)RoundSmem<M>::SCR_U4 * sizeof(uint4);
  const size_t fixed = sizeof(RoundSmem<M>) + hbytes + (in_smem ? cbytes : 0);
  constexpr size_t SLOT = sizeof(uint4) + sizeof(int);  // a table slot and its list entry
  int ts = 8192;
  while (ts >= 1024 && fixed + (size_t)ts * SLOT > NM_SMEM_BUDGET) ts >>= 1;
  if (ts < 1024) ts = 0;
  // Each block keeps the records of the rows it owns in its own table (a
  // round whose entries would fill more than 3/4 of it uses J.rec in global
  // memory instead).  VNM_NM_ROW_TABLE=0 keeps every round's records in
  // global memory, for measurement.
  if (const char* e = getenv("VNM_NM_ROW_TABLE"))
    if (atoi(e) == 0) ts = 0;

  // the record cache of the apply phase, when the budget allows it
  constexpr size_t RCACHE = (size_t)NM_THREADS * TOUCH_U * (sizeof(uint4) + sizeof(int));
  int rc = fixed + (size_t)ts * SLOT + RCACHE <= NM_SMEM_BUDGET ? 1 : 0;
  const size_t dyn = hbytes + (size_t)ts * SLOT + (rc ? RCACHE : 0) + (in_smem ? cbytes : 0);
  // static + dynamic shared memory may pass the 48 KB a launch gets without
  // opting in (RoundSmem<8> alone is ~30 KB)
  VNM_CUDA_TRY(cudaFuncSetAttribute(k_nm_rounds<M>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn));
  if (cs > 8)
    VNM_CUDA_TRY(cudaFuncSetAttribute(k_nm_rounds<M>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
  if (cs > 1) {
    // How many clusters of a size the GPU can hold at once depends on the
    // SMs of each of its GPCs; take the largest size (halving from cs) at
    // which every job of the call runs concurrently, else the largest that
    // fits at all.
    cudaLaunchConfig_t cfg = {};
    cfg.blockDim = dim3(NM_THREADS);
    cfg.dynamicSmemBytes = dyn;
    cfg.stream = ctx->stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int pick = 1, fallback = 1;
    for (int c = cs; c > 1; c >>= 1) {
      attr[0].val.clusterDim.x = (unsigned)c;
      cfg.gridDim = dim3((unsigned)(njobs * c));
      int nclusters = 0;
      if (cudaOccupancyMaxActiveClusters(&nclusters, k_nm_rounds<M>, &cfg) != cudaSuccess) {
        (void)cudaGetLastError();
        continue;
      }
      if (nclusters >= 1 && fallback == 1) {
        fallback = c;
        ctx->last_clusters_fit = nclusters;
      }
      if (nclusters >= njobs) {
        pick = c;
        ctx->last_clusters_fit = nclusters;
        break;
      }
    }
    if (pick == 1) pick = fallback;
    if (pick > 1) {
      attr[0].val.clusterDim.x = (unsigned)pick;
      cfg.gridDim = dim3((unsigned)(njobs * pick));
      VNM_CUDA_TRY(cudaLaunchKernelEx(&cfg, k_nm_rounds<M>, d_jobs, N, in_smem, ts, pick, rc));
      ctx->launches++;
      ctx->last_cluster = pick;
      return VNM_OK;
    }
    // no cluster fits: one block per job
    VNM_LAUNCH(ctx, k_nm_rounds<M>, njobs, NM_THREADS, dyn, d_jobs, N, in_smem, ts, 1, rc);
    ctx->last_cluster = 1;
    return VNM_OK;
  }
  VNM_LAUNCH(ctx, k_nm_rounds<M>, njobs, NM_THREADS, dyn, d_jobs, N, in_smem, ts, 1, rc);
  ctx->last_cluster = 1;
  return VNM_OK;
}

// Blocks per job for calls with few jobs (one matrix, or its four
// schedules); batches run clusters of 2 (run_batch).  Measured on GB300 (find_best,
// four jobs) with 4 / 8 / 16 blocks: R-MAT 2048 2:8 (26 K entries) 6.7 /
// 6.8 / 7.3 ms, R-MAT 16384 2:4 (228 K entries) 17.1 / 12.9 / 12.4 ms,
// R-MAT 65536 2:8 (1.8 M entries) 472 / 295 / 209 ms; so 16 (a non-portable
// cluster size) from 128 K pattern entries on, 8 below.  VNM_NM_CLUSTER
// (1..16) in the environment overrides the choice.
static int nm_cluster_size(long long np) {
  if (const char* e = getenv("VNM_NM_CLUSTER")) {  // rounded down to a power of two (rows are dealt in 16 groups)
    const int v = atoi(e);
    if (v >= 1 && v <= 16) return v >= 16 ? 16 : v >= 8 ? 8 : v >= 4 ? 4 : v >= 2 ? 2 : 1;
  }
  return np >= (1ll << 17) ? 16 : 8;
}

static vnm_status launch_rounds(vnm_ctx* ctx, const NMJob* d_jobs, int njobs, int N, int M, int max_nseg,
                                int cs = 1) {
  switch (M) {
    case 2: return launch_rounds_t<2>(ctx, d_jobs, njobs, N, max_nseg, cs);
    case 3: return launch_rounds_t<3>(ctx, d_jobs, njobs, N, max_nseg, cs);
    case 4: return launch_rounds_t<4>(ctx, d_jobs, njobs, N, max_nseg, cs);
    case 5: return launch_rounds_t<5>(ctx, d_jobs, njobs, N, max_nseg, cs);
    case 6: return launch_rounds_t<6>(ctx, d_jobs, njobs, N, max_nseg, cs);
    case 7: return launch_rounds_t<7>(ctx, d_jobs, njobs, N, max_nseg, cs);
    case 8: return launch_rounds_t<8>(ctx, d_jobs, njobs, N, max_nseg, cs);
  }
  return VNM_ERR_ARG;
}

static vnm_status check_nm_args(int nrows, int nnz, const int* row, const int* col, const float* val, int mem, int N,
                                int M) {
  if (M < 2 || M > 8 || N < 1 || N >= M) return VNM_ERR_ARG;
  if (nrows < 0 || nnz < 0 || (nrows % M) != 0) return VNM_ERR_ARG;
  if (mem != VNM_MEM_HOST && mem != VNM_MEM_DEVICE) return VNM_ERR_ARG;
  if (nnz > 0 && (!row || !col || !val)) return VNM_ERR_ARG;
  if (nrows >= (1 << 27)) return VNM_ERR_LIMIT;  // 16 nrows + 1 row groups fit an int
  return VNM_OK;
}

// find_best_2toX's choice (main.cu:80-113) from the four result vectors:
// largest improve rate, ties to the lower schedule id; 0 when the matrix is
// empty or has no invalid segment (main.cu:85).
__host__ __device__ static int pick_best(const int* res, int nsched, int nnz) {
  float max_imprv = 0.0f;
  int best = 0;
  for (int s = 0; s < nsched; ++s) {
    const int* r = res + 5 * s;
    if (nnz == 0 || r[0] == 0) return 0;
    const float imp = (r[2] != 0) ? ((r[2] - r[3]) * 1.0f / r[2]) : 0;
    if (imp > max_imprv) {
      max_imprv = imp;
      best = s;
    }
  }
  return best;
}

// newpos[orig[p]] = p for job `job`, or (job < 0) for the find_best_2toX
// winner of the jobs' results, chosen on the device as pick_best does on
// the host; the choice goes to *picked.
__global__ void k_pick_invert(const NMJob* jobs, int njobs, int nnz, int job, int R, int* newpos, int* picked) {
  __shared__ int s_job;
  if (threadIdx.x == 0) {
    if (job < 0) {
      int r5[20];
      for (int s = 0; s < njobs && s < 4; ++s)
        for (int q = 0; q < 5; ++q) r5[5 * s + q] = jobs[s].res[q];
      job = pick_best(r5, njobs < 4 ? njobs : 4, nnz);
    }
    s_job = job;
    if (blockIdx.x == 0) *picked = job;
  }
  __syncthreads();
  const int* orig = jobs[s_job].orig;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < R; i += gridDim.x * blockDim.x) newpos[orig[i]] = i;
}

// Pinned host words of run_matrix: the jobs' results, then the input
// check's flag, the pattern's entry count and the device's pick, then the
// job records on their way to the device.
constexpr int PIN_FLAGS = 4 * JOB_RES, PIN_JOBS = 256;
static_assert(4 * sizeof(NMJob) <= 256 * sizeof(int), "four job records fit the pinned words after PIN_JOBS");

// Run `nsched` jobs on one matrix (schedules sched0 .. sched0+nsched-1).
// newpos_job >= 0 selects the job whose permutation goes to newpos_out;
// -1 selects the find_best_2toX winner (reported in *picked).
static vnm_status run_matrix(vnm_ctx* ctx, int nrows, int nnz, const int* row, const int* col, const float* val,
                             int mem, int N, int M, int sched0, int nsched, int maxiter, int* res5_out,
                             int* newpos_out, int newpos_job, bool trace, int* picked = nullptr) {
  const int R = nrows;
  const int trace_pairs_cap = trace ? 2 * (M + 1) * M * 4096 : 0;
  const int trace_rounds_cap = trace ? 65536 : 0;
  size_t need = pattern_bytes(R, nnz) + (size_t)nsched * job_bytes(R) + arena_bytes(nsched, sizeof(NMJob)) +
                arena_bytes(R, sizeof(int)) + 3 * arena_bytes(nnz, sizeof(int)) +
                arena_bytes(trace_pairs_cap * 2, sizeof(int)) + arena_bytes(trace_rounds_cap, sizeof(int)) + 4096;
  VNM_TRY(arena_reserve(ctx, need));
  VNM_TRY(pinned_reserve(ctx, 512 + (size_t)trace_pairs_cap * 2 + trace_rounds_cap));
  if (nsched < 1 || nsched > 4) return VNM_ERR_ARG;
  VNM_TRY(begin_call(ctx));
  const int *d_row, *d_col;
  const float* d_val;
  VNM_TRY(stage_in(ctx, row, nnz, mem, &d_row));
  VNM_TRY(stage_in(ctx, col, nnz, mem, &d_col));
  VNM_TRY(stage_in(ctx, val, nnz, mem, &d_val));
  // No host synchronisation until the end of the call: the input check's
  // flag and the pattern's entry count come back with the results (a
  // flagged input makes every kernel after the check skip its work).
  Pattern P;
  VNM_TRY(build_pattern(ctx, R, nnz, d_row, d_col, d_val, N, M, P, ctx->h_pinned, true));
  NMJob hj[4];
  for (int s = 0; s < nsched; ++s) {
    VNM_TRY(make_job(ctx, P, sched0 + s, maxiter, hj[s]));
    hj[s].err = P.d_err;
  }
  int* d_tp = nullptr;
  int* d_tr = nullptr;
  if (trace) {
    d_tp = arena_take<int>(ctx, trace_pairs_cap * 2);
    d_tr = arena_take<int>(ctx, trace_rounds_cap);
    if (!d_tp || !d_tr) return VNM_ERR_NOMEM;
    hj[0].trace_pairs = d_tp;
    hj[0].trace_rounds = d_tr;
    hj[0].trace_cap_pairs = trace_pairs_cap;
    hj[0].trace_cap_rounds = trace_rounds_cap;
  }
  NMJob* d_jobs = arena_take<NMJob>(ctx, nsched);
  int* d_newpos = newpos_out && R > 0 ? arena_take<int>(ctx, R) : nullptr;
  if (!d_jobs || (newpos_out && R > 0 && !d_newpos)) return VNM_ERR_NOMEM;
  // the job records go through pinned memory, so that the copy is queued
  // behind the pattern build instead of waiting for it
  NMJob* pj = reinterpret_cast<NMJob*>(ctx->h_pinned + PIN_JOBS);
  memcpy(pj, hj, sizeof(NMJob) * nsched);
  VNM_CUDA_TRY(cudaMemcpyAsync(d_jobs, pj, sizeof(NMJob) * nsched, cudaMemcpyHostToDevice, ctx->stream));
  VNM_CUDA_TRY(cudaEventRecord(ctx->ev_main0, ctx->stream));
  // the stored entries stand in for the pattern's (nonzero-valued) entries
  // when sizing the clusters: their count is known without a readback
  VNM_TRY(launch_rounds(ctx, d_jobs, nsched, N, M, P.nseg, nm_cluster_size(nnz)));
  VNM_CUDA_TRY(cudaEventRecord(ctx->ev_main1, ctx->stream));
  int* hp = ctx->h_pinned;
  for (int s = 0; s < nsched; ++s)
    VNM_CUDA_TRY(cudaMemcpyAsync(hp + JOB_RES * s, hj[s].res, sizeof(int) * JOB_RES, cudaMemcpyDeviceToHost,
                                 ctx->stream));
  VNM_CUDA_TRY(cudaMemcpyAsync(hp + PIN_FLAGS, P.d_err, 2 * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  if (d_newpos) {
    VNM_LAUNCH(ctx, k_pick_invert, grid_for(ctx, R), 256, 0, d_jobs, nsched, nnz, newpos_job, R, d_newpos,
               P.d_err + 1);  // the entry count was read back above: its word now takes the pick
    VNM_CUDA_TRY(cudaMemcpyAsync(hp + PIN_FLAGS + 2, P.d_err + 1, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    VNM_CUDA_TRY(cudaMemcpyAsync(newpos_out, d_newpos, sizeof(int) * R, cudaMemcpyDeviceToHost, ctx->stream));
  }
  VNM_TRY(end_call(ctx));
  VNM_CUDA_TRY(cudaEventElapsedTime(&ctx->main_ms, ctx->ev_main0, ctx->ev_main1));
  const int flag = hp[PIN_FLAGS];
  if (flag & 2) return VNM_ERR_RANGE;
  if (flag & 1) return VNM_ERR_UNSORTED;
  P.np = nnz > 0 ? hp[PIN_FLAGS + 1] : 0;
  const int dev_pick = hp[PIN_FLAGS + 2];
  int hres_copy[4 * JOB_RES];
  memcpy(hres_copy, hp, sizeof(int) * JOB_RES * nsched);
  for (int q = 0; q < 28; ++q) ctx->stats[q] = 0;
  ctx->stats[3] = P.nseg;
  ctx->stats[4] = nsched;
  ctx->stats[5] = P.np;
  ctx->stats[6] = ctx->last_cluster;
  {  // when the jobs ran: spread of their starts and the span of all of them (us)
    int s0 = hres_copy[13], s1 = hres_copy[13], e1 = hres_copy[14];
    for (int s = 1; s < nsched; ++s) {
      const int* h = hres_copy + JOB_RES * s;
      if ((int)((unsigned)h[13] - (unsigned)s0) < 0) s0 = h[13];
      if ((int)((unsigned)h[13] - (unsigned)s1) > 0) s1 = h[13];
      if ((int)((unsigned)h[14] - (unsigned)e1) > 0) e1 = h[14];
    }
    ctx->stats[17] = (long long)(((unsigned)s1 - (unsigned)s0) & 0x7fffffffu) * 1024 / 1000;
    ctx->stats[18] = (long long)(((unsigned)e1 - (unsigned)s0) & 0x7fffffffu) * 1024 / 1000;
    ctx->stats[19] = ctx->last_clusters_fit;
  }
  for (int s = 0; s < nsched; ++s) {
    const int* h = hres_copy + JOB_RES * s;
    if (h[5] != 0) return VNM_ERR_INTERNAL;
    for (int q = 0; q < 5; ++q) res5_out[5 * s + q] = h[q];
    ctx->stats[0] += h[4];
    ctx->stats[1] += (long long)h[7] + ((long long)h[8] << 31);
    ctx->stats[2] += (long long)h[9] + ((long long)h[10] << 31);
    for (int q = 0; q < 7; ++q) ctx->stats[8 + q] += h[16 + q];
    ctx->stats[7] += h[11];
    ctx->stats[15] += h[12];
    ctx->stats[16] += h[23];
    ctx->stats[20] += h[24];
    ctx->stats[21] += h[25];
    for (int q = 0; q < 6; ++q) ctx->stats[22 + q] += h[26 + q];
  }
  const int pick = newpos_job >= 0 ? newpos_job : pick_best(res5_out, nsched, nnz);
  if (picked) *picked = pick;
  if (d_newpos && dev_pick != pick) {  // the device chose from the same integers with the same arithmetic
    VNM_LAUNCH(ctx, k_invert, grid_for(ctx, R), 256, 0, hj[pick].orig, R, d_newpos);
    VNM_CUDA_TRY(cudaMemcpyAsync(newpos_out, d_newpos, sizeof(int) * R, cudaMemcpyDeviceToHost, ctx->stream));
    VNM_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  }
  if (trace) {
    const int committed = hres_copy[6];
    const int rounds = hres_copy[4];
    const int np = committed < trace_pairs_cap ? committed : trace_pairs_cap;
    const int nr = rounds < trace_rounds_cap ? rounds : trace_rounds_cap;
    int* ht = ctx->h_pinned + 128;  // over the per-job results, which were copied out above
    if (np) VNM_CUDA_TRY(cudaMemcpyAsync(ht, d_tp, sizeof(int) * 2 * np, cudaMemcpyDeviceToHost, ctx->stream));
    if (nr)
      VNM_CUDA_TRY(cudaMemcpyAsync(ht + 2 * np, d_tr, sizeof(int) * nr, cudaMemcpyDeviceToHost, ctx->stream));
    VNM_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    ctx->trace_pairs.assign(ht, ht + 2 * np);
    ctx->trace_round_end.assign(ht + 2 * np, ht + 2 * np + nr);
  }
  return VNM_OK;
}


// ---------------------------------------------------------------------------
// Batches: many matrices as one block-diagonal matrix.  Matrix b's ids are
// shifted by its row offset, so one pattern build covers the whole batch;
// job b sees the columns of its own diagonal block and the rows it reaches
// are its own (global ids), so the jobs share the row-record array without
// overlapping.  All jobs run as the blocks of one persistent launch.
// ---------------------------------------------------------------------------
__global__ void k_batch_offset(const int* row, const int* col, const long long* nnz_off, const int* row_off,
                               const int* nrows, int nmat, long long nnz, int* grow, int* gcol, int* err) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nnz;
       i += (long long)gridDim.x * blockDim.x) {
    int lo = 0, hi = nmat - 1;  // last b with nnz_off[b] <= i
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (nnz_off[mid] <= i) lo = mid;
      else hi = mid - 1;
    }
    const int b = lo, R = nrows[b];
    const int r = row[i], c = col[i];
    if (r < 0 || r >= R || c < 0 || c >= R) {
      atomicOr(err, 2);
      grow[i] = gcol[i] = 0;
      continue;
    }
    if (i > nnz_off[b]) {
      const int rp = row[i - 1], cp = col[i - 1];
      if (rp > r || (rp == r && cp >= c)) atomicOr(err, 1);
    }
    grow[i] = r + row_off[b];
    gcol[i] = c + row_off[b];
  }
}

__global__ void k_batch_init(const NMJob* jobs, const int* inv0, const int* pres0, const int* seg_off) {
  const NMJob J = jobs[blockIdx.x];
  const int so = seg_off[blockIdx.x];
  for (int i = threadIdx.x; i < J.R; i += blockDim.x) {
    J.orig[i] = i;
    if (i < J.nseg) {
      J.cnt[i] = inv0[so + i];
      J.zc[i] = J.R - pres0[so + i];
    }
  }
}

__global__ void k_batch_invert(const NMJob* jobs, const int* row_off, int* newpos) {
  const NMJob J = jobs[blockIdx.x];
  int* out = newpos + row_off[blockIdx.x];
  for (int i = threadIdx.x; i < J.R; i += blockDim.x) out[J.orig[i]] = i;
}

static vnm_status run_batch(vnm_ctx* ctx, int nmat, const int* nrows, const int64_t* nnz_offset, const int* row,
                            const int* col, const float* val, int N, int M, int sched, int maxiter, int* res5,
                            int* newpos) {
  if (!ctx || nmat < 0 || !nrows || !nnz_offset || !res5) return VNM_ERR_ARG;
  if (M < 2 || M > 8 || N < 1 || N >= M || sched < 0 || sched > 3) return VNM_ERR_ARG;
  if (nmat == 0) return VNM_OK;
  std::vector<int> row_off(nmat + 1), seg_off(nmat);
  long long totR = 0;
  for (int b = 0; b < nmat; ++b) {
    if (nrows[b] < 0 || nrows[b] % M != 0 || nnz_offset[b + 1] < nnz_offset[b]) return VNM_ERR_ARG;
    row_off[b] = (int)totR;
    seg_off[b] = (int)(totR / M);
    totR += nrows[b];
  }
  row_off[nmat] = (int)totR;
  const long long nnz = nnz_offset[nmat] - nnz_offset[0];
  if (nnz_offset[0] != 0 || totR >= (1 << 27) || nnz > (1ll << 31) - 1) return VNM_ERR_LIMIT;
  if (nnz > 0 && (!row || !col || !val)) return VNM_ERR_ARG;
  const int R = (int)totR, n = (int)nnz;
  size_t need = pattern_bytes(R, n) + 5 * arena_bytes(n, sizeof(int)) + arena_bytes(nmat + 1, 8) +
                3 * arena_bytes(nmat + 1, sizeof(int)) + arena_bytes(nmat, sizeof(NMJob)) +
                arena_bytes(R, sizeof(int)) + arena_bytes((size_t)R + (size_t)2 * ROW_GROUPS * nmat, sizeof(int)) +
                arena_bytes(R, sizeof(uint4)) + 2 * arena_bytes(R / M + nmat, sizeof(int)) +
                arena_bytes((size_t)JOB_RES * nmat, sizeof(int)) + arena_bytes(R, sizeof(int)) + 8192;
  VNM_TRY(arena_reserve(ctx, need));
  VNM_TRY(pinned_reserve(ctx, 256 + (size_t)JOB_RES * nmat));
  VNM_TRY(begin_call(ctx));
  const int *d_row, *d_col;
  const float* d_val;
  VNM_TRY(stage_in(ctx, row, n, VNM_MEM_HOST, &d_row));
  VNM_TRY(stage_in(ctx, col, n, VNM_MEM_HOST, &d_col));
  VNM_TRY(stage_in(ctx, val, n, VNM_MEM_HOST, &d_val));
  long long* d_noff = arena_take<long long>(ctx, nmat + 1);
  int* d_roff = arena_take<int>(ctx, nmat + 1);
  int* d_soff = arena_take<int>(ctx, nmat + 1);
  int* d_nrows = arena_take<int>(ctx, nmat + 1);
  int* grow = arena_take<int>(ctx, n > 0 ? n : 1);
  int* gcol = arena_take<int>(ctx, n > 0 ? n : 1);
  int* err = arena_take<int>(ctx, 1);
  if (!d_noff || !d_roff || !d_soff || !d_nrows || !grow || !gcol || !err) return VNM_ERR_NOMEM;
  VNM_CUDA_TRY(cudaMemcpyAsync(d_noff, nnz_offset, sizeof(long long) * (nmat + 1), cudaMemcpyHostToDevice,
                               ctx->stream));
  VNM_CUDA_TRY(cudaMemcpyAsync(d_roff, row_off.data(), sizeof(int) * (nmat + 1), cudaMemcpyHostToDevice,
                               ctx->stream));
  VNM_CUDA_TRY(cudaMemcpyAsync(d_soff, seg_off.data(), sizeof(int) * nmat, cudaMemcpyHostToDevice, ctx->stream));
  VNM_CUDA_TRY(cudaMemcpyAsync(d_nrows, nrows, sizeof(int) * nmat, cudaMemcpyHostToDevice, ctx->stream));
  VNM_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), ctx->stream));
  if (n > 0)
    VNM_LAUNCH(ctx, k_batch_offset, grid_for(ctx, n), 256, 0, d_row, d_col, d_noff, d_roff, d_nrows, nmat,
               (long long)n, grow, gcol, err);
  VNM_CUDA_TRY(cudaMemcpyAsync(ctx->h_pinned, err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  VNM_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  if (ctx->h_pinned[0] & 2) return VNM_ERR_RANGE;
  if (ctx->h_pinned[0] & 1) return VNM_ERR_UNSORTED;
  Pattern P;
  VNM_TRY(build_pattern(ctx, R, n, grow, gcol, d_val, N, M, P, ctx->h_pinned));
  // per-job state, one allocation per field for the whole batch
  int* orig = arena_take<int>(ctx, R > 0 ? R : 1);
  int* touched = arena_take<int>(ctx, (size_t)R + (size_t)2 * ROW_GROUPS * nmat);  // 32 of slack per job
  uint4* rec = arena_take<uint4>(ctx, R > 0 ? R : 1);
  int* cnt = arena_take<int>(ctx, R / M + nmat);
  int* zc = arena_take<int>(ctx, R / M + nmat);
  int* res = arena_take<int>(ctx, (size_t)JOB_RES * nmat);
  NMJob* d_jobs = arena_take<NMJob>(ctx, nmat);
  if (!orig || !touched || !rec || !cnt || !zc || !res || !d_jobs) return VNM_ERR_NOMEM;
  VNM_CUDA_TRY(cudaMemsetAsync(rec, 0, sizeof(uint4) * (R > 0 ? R : 1), ctx->stream));
  VNM_CUDA_TRY(cudaMemsetAsync(res, 0, sizeof(int) * JOB_RES * nmat, ctx->stream));
  std::vector<NMJob> hj(nmat);
  int max_nseg = 0;
  for (int b = 0; b < nmat; ++b) {
    NMJob& J = hj[b];
    J.R = nrows[b];
    J.nseg = nrows[b] / M;
    J.sched = sched;
    J.maxiter = maxiter;
    J.cptr = P.cptr + row_off[b];
    J.crow = P.crow;
    J.csplit = P.csplit + (size_t)ROW_GROUPS * row_off[b];
    J.orig = orig + row_off[b];
    J.cnt = cnt + seg_off[b] + b;
    J.zc = zc + seg_off[b] + b;
    J.rec = rec;
    J.touched = touched + row_off[b] + 2 * ROW_GROUPS * b;
    J.res = res + JOB_RES * b;
    J.trace_pairs = nullptr;
    J.trace_rounds = nullptr;
    J.trace_cap_pairs = 0;
    J.trace_cap_rounds = 0;
    J.walk_wait_limit = WALK_WAIT_LIMIT;
    J.hold_heaps = 0;
    J.err = nullptr;
    J.timed = ctx->phase_timing ? 1 : 0;
    if (J.nseg > max_nseg) max_nseg = J.nseg;
  }
  VNM_CUDA_TRY(cudaMemcpyAsync(d_jobs, hj.data(), sizeof(NMJob) * nmat, cudaMemcpyHostToDevice, ctx->stream));
  VNM_LAUNCH(ctx, k_batch_init, nmat, 256, 0, d_jobs, P.inv0, P.pres0, d_soff);
  VNM_CUDA_TRY(cudaEventRecord(ctx->ev_main0, ctx->stream));
  // clusters of 2 blocks per job: the batch's time is its largest matrices'
  // jobs, and two SMs each shorten them more than the extra waves cost
  // (GB300, 256 R-MAT matrices 256-8192 rows at 2:8: 88 ms with one block
  // per job, 63 ms with 2, 69 ms with 4)
  VNM_TRY(launch_rounds(ctx, d_jobs, nmat, N, M, max_nseg, 2));
  VNM_CUDA_TRY(cudaEventRecord(ctx->ev_main1, ctx->stream));
  int* hres = ctx->h_pinned + 256;
  VNM_CUDA_TRY(cudaMemcpyAsync(hres, res, sizeof(int) * JOB_RES * nmat, cudaMemcpyDeviceToHost, ctx->stream));
  if (newpos && R > 0) {
    int* d_np = arena_take<int>(ctx, R);
    if (!d_np) return VNM_ERR_NOMEM;
    VNM_LAUNCH(ctx, k_batch_invert, nmat, 256, 0, d_jobs, d_roff, d_np);
    VNM_CUDA_TRY(cudaMemcpyAsync(newpos, d_np, sizeof(int) * R, cudaMemcpyDeviceToHost, ctx->stream));
  }
  VNM_TRY(end_call(ctx));
  VNM_CUDA_TRY(cudaEventElapsedTime(&ctx->main_ms, ctx->ev_main0, ctx->ev_main1));
  for (int q = 0; q < 28; ++q) ctx->stats[q] = 0;
  ctx->stats[3] = max_nseg;
  ctx->stats[4] = nmat;
  ctx->stats[5] = P.np;
  for (int b = 0; b < nmat; ++b) {
    const int* h = hres + JOB_RES * b;
    if (h[5] != 0) return VNM_ERR_INTERNAL;
    for (int q = 0; q < 5; ++q) res5[5 * b + q] = h[q];
    ctx->stats[0] += h[4];
    ctx->stats[1] += (long long)h[7] + ((long long)h[8] << 31);
    ctx->stats[2] += (long long)h[9] + ((long long)h[10] << 31);
    for (int q = 0; q < 7; ++q) ctx->stats[8 + q] += h[16 + q];
    ctx->stats[7] += h[11];
    ctx->stats[15] += h[12];
    ctx->stats[16] += h[23];
  }
  return VNM_OK;
}

}  // namespace vnm

using namespace vnm;

extern "C" {

vnm_status vnm_nm_reorder(vnm_ctx* ctx, int nrows, int nnz, const int* row, const int* col, const float* val,
                          int mem, int N, int M, int sched, int nm_maxiter, int* res5, int* newpos) {
  if (!ctx || !res5) return VNM_ERR_ARG;
  VNM_TRY(check_nm_args(nrows, nnz, row, col, val, mem, N, M));
  if (sched < 0 || sched > 3) return VNM_ERR_ARG;
  return run_matrix(ctx, nrows, nnz, row, col, val, mem, N, M, sched, 1, nm_maxiter, res5, newpos, 0, ctx->trace);
}

vnm_status vnm_nm_search(vnm_ctx* ctx, int nrows, int nnz, const int* row, const int* col, const float* val,
                         int mem, int N, int M, int nm_maxiter, int* best_sched, int* res5x4, int* newpos_best) {
  if (!ctx || !best_sched) return VNM_ERR_ARG;
  VNM_TRY(check_nm_args(nrows, nnz, row, col, val, mem, N, M));
  int res[20];
  // the four schedules run as four blocks of one launch; the winner's final
  // arrangement is already on the device, so its permutation is read back
  // without a second run
  VNM_TRY(run_matrix(ctx, nrows, nnz, row, col, val, mem, N, M, 0, 4, nm_maxiter, res, newpos_best, -1, false,
                     best_sched));
  if (res5x4) memcpy(res5x4, res, sizeof res);
  return VNM_OK;
}

vnm_status vnm_nm_set_trace(vnm_ctx* ctx, int enable) {
  if (!ctx) return VNM_ERR_ARG;
  ctx->trace = enable != 0;
  return VNM_OK;
}

vnm_status vnm_nm_set_phase_timing(vnm_ctx* ctx, int enable) {
  if (!ctx) return VNM_ERR_ARG;
  ctx->phase_timing = enable != 0;
  return VNM_OK;
}

vnm_status vnm_nm_get_trace(vnm_ctx* ctx, int* pairs, int cap_pairs, int* npairs, int* round_end, int cap_rounds,
                            int* nrounds) {
  if (!ctx || !npairs || !nrounds) return VNM_ERR_ARG;
  const int np = (int)ctx->trace_pairs.size() / 2, nr = (int)ctx->trace_round_end.size();
  *npairs = np;
  *nrounds = nr;
  if (pairs)
    for (int i = 0; i < 2 * np && i < 2 * cap_pairs; ++i) pairs[i] = ctx->trace_pairs[i];
  if (round_end)
    for (int i = 0; i < nr && i < cap_rounds; ++i) round_end[i] = ctx->trace_round_end[i];
  return VNM_OK;
}

vnm_status vnm_permute_coo(vnm_ctx* ctx, int nrows, int nnz, int* row, int* col, int mem, const int* newpos) {
  if (!ctx || nrows < 0 || nnz < 0 || !newpos || (nnz > 0 && (!row || !col))) return VNM_ERR_ARG;
  if (mem != VNM_MEM_HOST && mem != VNM_MEM_DEVICE) return VNM_ERR_ARG;
  VNM_TRY(arena_reserve(ctx, 3 * arena_bytes(nnz, sizeof(int)) + arena_bytes(nrows, sizeof(int)) + 1024));
  VNM_TRY(begin_call(ctx));
  int *d_row = row, *d_col = col;
  const int* d_np = newpos;
  if (mem == VNM_MEM_HOST) {
    d_row = arena_take<int>(ctx, nnz > 0 ? nnz : 1);
    d_col = arena_take<int>(ctx, nnz > 0 ? nnz : 1);
    int* t = arena_take<int>(ctx, nrows > 0 ? nrows : 1);
    if (!d_row || !d_col || !t) return VNM_ERR_NOMEM;
    if (nnz) {
      VNM_CUDA_TRY(cudaMemcpyAsync(d_row, row, sizeof(int) * nnz, cudaMemcpyHostToDevice, ctx->stream));
      VNM_CUDA_TRY(cudaMemcpyAsync(d_col, col, sizeof(int) * nnz, cudaMemcpyHostToDevice, ctx->stream));
    }
    if (nrows) VNM_CUDA_TRY(cudaMemcpyAsync(t, newpos, sizeof(int) * nrows, cudaMemcpyHostToDevice, ctx->stream));
    d_np = t;
  }
  if (nnz) VNM_LAUNCH(ctx, k_permute, grid_for(ctx, nnz), 256, 0, d_row, d_col, nnz, d_np);
  if (mem == VNM_MEM_HOST && nnz) {
    VNM_CUDA_TRY(cudaMemcpyAsync(row, d_row, sizeof(int) * nnz, cudaMemcpyDeviceToHost, ctx->stream));
    VNM_CUDA_TRY(cudaMemcpyAsync(col, d_col, sizeof(int) * nnz, cudaMemcpyDeviceToHost, ctx->stream));
  }
  return end_call(ctx);
}

vnm_status vnm_permute_coo_async(vnm_ctx* ctx, int nrows, int nnz, int* row, int* col, const int* newpos,
                                 void* stream) {
  if (!ctx || nrows < 0 || nnz < 0 || !newpos || (nnz > 0 && (!row || !col))) return VNM_ERR_ARG;
  VNM_CUDA_TRY(cudaSetDevice(ctx->device));
  ctx->launches = 0;
  ctx->last_ms = ctx->main_ms = 0.f;
  if (nnz == 0) return VNM_OK;
  const int grid = grid_for(ctx, nnz);
  k_permute<<<grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(row, col, nnz, newpos);
  ctx->launches = 1;
  return cudaGetLastError() == cudaSuccess ? VNM_OK : VNM_ERR_CUDA;
}

vnm_status vnm_nm_segment_counts(vnm_ctx* ctx, int nrows, int nnz, const int* row, const int* col,
                                 const float* val, int mem, int N, int M, int* invalid, int* allzero) {
  if (!ctx || !invalid || !allzero) return VNM_ERR_ARG;
  VNM_TRY(check_nm_args(nrows, nnz, row, col, val, mem, N, M));
  VNM_TRY(arena_reserve(ctx, pattern_bytes(nrows, nnz) + 3 * arena_bytes(nnz, sizeof(int)) + 4096));
  VNM_TRY(pinned_reserve(ctx, 64));
  VNM_TRY(begin_call(ctx));
  const int *d_row, *d_col;
  const float* d_val;
  VNM_TRY(stage_in(ctx, row, nnz, mem, &d_row));
  VNM_TRY(stage_in(ctx, col, nnz, mem, &d_col));
  VNM_TRY(stage_in(ctx, val, nnz, mem, &d_val));
  Pattern P;
  VNM_TRY(build_pattern(ctx, nrows, nnz, d_row, d_col, d_val, N, M, P, ctx->h_pinned));
  const int nseg = nrows / M;
  if (nseg) {
    VNM_CUDA_TRY(cudaMemcpyAsync(invalid, P.inv0, sizeof(int) * nseg, cudaMemcpyDeviceToHost, ctx->stream));
    VNM_CUDA_TRY(cudaMemcpyAsync(allzero, P.pres0, sizeof(int) * nseg, cudaMemcpyDeviceToHost, ctx->stream));
  }
  VNM_TRY(end_call(ctx));
  for (int s = 0; s < nseg; ++s) allzero[s] = nrows - allzero[s];
  return VNM_OK;
}

vnm_status vnm_nm_pair_score(vnm_ctx* ctx, int nrows, int nnz, const int* row, const int* col, const float* val,
                             int mem, int N, int M, int seg1, int seg2, int* score) {
  if (!ctx || !score) return VNM_ERR_ARG;
  VNM_TRY(check_nm_args(nrows, nnz, row, col, val, mem, N, M));
  const int nseg = nrows / M;
  if (seg1 < 0 || seg2 < 0 || seg1 >= nseg || seg2 >= nseg) return VNM_ERR_ARG;
  VNM_TRY(arena_reserve(ctx, pattern_bytes(nrows, nnz) + job_bytes(nrows) + 3 * arena_bytes(nnz, sizeof(int)) +
                                 arena_bytes(2 * M * M, sizeof(int)) + 4096));
  VNM_TRY(pinned_reserve(ctx, 64));
  VNM_TRY(begin_call(ctx));
  const int *d_row, *d_col;
  const float* d_val;
  VNM_TRY(stage_in(ctx, row, nnz, mem, &d_row));
  VNM_TRY(stage_in(ctx, col, nnz, mem, &d_col));
  VNM_TRY(stage_in(ctx, val, nnz, mem, &d_val));
  Pattern P;
  VNM_TRY(build_pattern(ctx, nrows, nnz, d_row, d_col, d_val, N, M, P, ctx->h_pinned));
  NMJob J;
  VNM_TRY(make_job(ctx, P, 0, 10, J));
  int* d_score = arena_take<int>(ctx, 2 * M * M);
  if (!d_score) return VNM_ERR_NOMEM;
  switch (M) {
#define VNM_PS(MM)                                                                          \
  case MM:                                                                                  \
    VNM_CUDA_TRY(cudaFuncSetAttribute(k_pair_score<MM>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                                      RoundSmem<MM>::SCR_U4 * 16));                                   \
    VNM_LAUNCH(ctx, k_pair_score<MM>, 1, NM_THREADS, RoundSmem<MM>::SCR_U4 * 16, J, N, seg1, seg2,   \
               d_score);                                                                              \
    break;
    VNM_PS(2) VNM_PS(3) VNM_PS(4) VNM_PS(5) VNM_PS(6) VNM_PS(7) VNM_PS(8)
#undef VNM_PS
  }
  VNM_CUDA_TRY(cudaMemcpyAsync(score, d_score, sizeof(int) * 2 * M * M, cudaMemcpyDeviceToHost, ctx->stream));
  return end_call(ctx);
}

vnm_status vnm_nm_reorder_batch(vnm_ctx* ctx, int nmat, const int* nrows, const int64_t* nnz_offset,
                                const int* row, const int* col, const float* val, int N, int M, int sched,
                                int nm_maxiter, int* res5, int* newpos) {
  return run_batch(ctx, nmat, nrows, nnz_offset, row, col, val, N, M, sched, nm_maxiter, res5, newpos);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// NM reorder without allocation
//
// Some callers cannot call cudaMalloc: services whose device memory is all
// handed out up front by their own allocator (a foreign allocation would
// break its accounting or fail), and latency-critical loops where an
// allocation -- which can synchronise the device -- is not allowed.  For
// them, vnm_nm_reorder_noalloc runs the same kernels as vnm_nm_reorder with
// its scratch taken from one fixed array in device memory instead of the
// context's allocator, and with no context at all.
//
// Limits: nrows <= VNM_NOALLOC_MAX_ROWS, nnz <= VNM_NOALLOC_MAX_NNZ; the
// array is VNM_NOALLOC_SCRATCH_BYTES and every GPU that loads this library
// keeps it until the process exits.  All calls share it: calls that overlap
// on the GPU (other streams, other host threads) race and must not be made.
// ---------------------------------------------------------------------------

namespace vnm {

constexpr int NOALLOC_MAX_ROWS = 32768;
constexpr int NOALLOC_MAX_NNZ = 1 << 19;
constexpr size_t NOALLOC_BYTES = size_t(16) << 20;  // 16 MiB

// The scratch itself.  Host code must not use this symbol as an address
// (in host code it names a host-side shadow); it asks the runtime for the
// device address instead (noalloc_scratch below).
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_BYTES];

// Device address of g_noalloc_scratch on the current device.  Looked up on
// every call (no stream work, no allocation): an address kept from an
// earlier call would be stale after a device reset, which reloads the module.
static vnm_status noalloc_scratch(unsigned char** out) {
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess || !p) {
    (void)cudaGetLastError();
    return VNM_ERR_CUDA;
  }
  *out = static_cast<unsigned char*>(p);
  return VNM_OK;
}

}  // namespace vnm

extern "C" vnm_status vnm_nm_reorder_noalloc(int nrows, int nnz, const int* row, const int* col, const float* val,
                                             int N, int M, int sched, int nm_maxiter, int* res5, int* newpos,
                                             void* stream) {
  using namespace vnm;
  VNM_TRY(check_nm_args(nrows, nnz, row, col, val, VNM_MEM_DEVICE, N, M));
  if (sched < 0 || sched > 3 || !res5 || !newpos) return VNM_ERR_ARG;
  if (nrows > NOALLOC_MAX_ROWS || nnz > NOALLOC_MAX_NNZ) return VNM_ERR_LIMIT;
  const size_t need = pattern_bytes(nrows, nnz) + job_bytes(nrows) + arena_bytes(1, sizeof(NMJob)) + 4096;
  if (need > NOALLOC_BYTES) return VNM_ERR_LIMIT;
  int device = 0;
  VNM_CUDA_TRY(cudaGetDevice(&device));
  unsigned char* scratch = nullptr;
  VNM_TRY(noalloc_scratch(&scratch));
  // a context on the stack: its "arena" is the fixed array, its stream the
  // caller's; no event, stream or memory is created
  vnm_ctx c;
  c.device = device;
  c.num_sms = 1;
  VNM_CUDA_TRY(cudaDeviceGetAttribute(&c.num_sms, cudaDevAttrMultiProcessorCount, device));
  c.stream = static_cast<cudaStream_t>(stream);
  c.arena.base = reinterpret_cast<char*>(scratch);
  c.arena.cap = NOALLOC_BYTES;
  c.arena.used = 0;
  int hs[16] = {0};  // host readback (pageable)
  Pattern P;
  VNM_TRY(build_pattern(&c, nrows, nnz, row, col, val, N, M, P, hs));
  NMJob hj;
  VNM_TRY(make_job(&c, P, sched, nm_maxiter, hj));  // clears the job's scratch
  NMJob* d_job = arena_take<NMJob>(&c, 1);
  if (!d_job) return VNM_ERR_LIMIT;
  VNM_CUDA_TRY(cudaMemcpyAsync(d_job, &hj, sizeof(NMJob), cudaMemcpyHostToDevice, c.stream));
  // the same launch shape as vnm_nm_reorder (a cluster of blocks per job);
  // the scratch it needs does not depend on the cluster size
  VNM_TRY(launch_rounds(&c, d_job, 1, N, M, P.nseg, nm_cluster_size(P.np)));
  VNM_CUDA_TRY(cudaMemcpyAsync(hs, hj.res, sizeof(int) * 16, cudaMemcpyDeviceToHost, c.stream));
  VNM_CUDA_TRY(cudaStreamSynchronize(c.stream));
  if (hs[5] != 0) return VNM_ERR_INTERNAL;
  VNM_CUDA_TRY(cudaMemcpyAsync(res5, hj.res, sizeof(int) * 5, cudaMemcpyDeviceToDevice, c.stream));
  if (nrows > 0) VNM_LAUNCH(&c, k_invert, grid_for(&c, nrows), 256, 0, hj.orig, nrows, newpos);
  VNM_CUDA_TRY(cudaStreamSynchronize(c.stream));
  return VNM_OK;
}
