/*
 * vnm_gb300 -- GB300-native V:N:M graph reordering and SpMM, C ABI.
 *
 * This header is the drop-in boundary of libvnm_gb300.so.  The reference
 * (PictureResearch/vnm-graph-reordering) ships no library API: its path is the
 * `spmm` command built from main.cu over header templates.  Each entry point
 * below names the reference function it replaces (file:line).  The `spmm`
 * drop-in command of this project is a thin C++ program over these calls.
 *
 * Conventions
 *   - Plain C types only.  Every call returns a vnm_status (0 = success); no
 *     call exits the process or throws across the ABI.
 *   - Matrices are COO, 0-based, int32 indices, float32 values, square with
 *     `nrows` already padded to a multiple of M (as Mtx::init_from_file does),
 *     sorted by (row, col) with no repeated (row, col) -- the state a matrix
 *     is in after the reference's reader (mtx/readMtx.hpp:354-425).  The NM
 *     calls take nrows < 2^27 (a batch: the sum of its nrows), else
 *     VNM_ERR_LIMIT.
 *   - `mem` says where the caller's arrays live: VNM_MEM_HOST (pageable or
 *     pinned host memory; the call copies them) or VNM_MEM_DEVICE (device
 *     memory of the context's GPU; nothing is copied).
 *   - A context owns one CUDA stream and its scratch memory; use one context
 *     per host thread.  Calls are synchronous with respect to the host unless
 *     stated otherwise; the *_async calls enqueue on a stream the caller
 *     passes and return without waiting.
 */
#ifndef VNM_GB300_H
#define VNM_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int vnm_status;
#define VNM_OK 0
#define VNM_ERR_ARG 1          /* invalid argument (sizes, N/M/V, schedule) */
#define VNM_ERR_CUDA 2         /* a CUDA runtime call failed */
#define VNM_ERR_UNSORTED 3     /* COO not sorted by (row, col) or has repeats */
#define VNM_ERR_RANGE 4        /* an index outside [0, nrows) */
#define VNM_ERR_NOMEM 5        /* device allocation failed */
#define VNM_ERR_INTERNAL 6     /* a kernel reported a broken invariant, or a bounded wait inside a
                                  kernel ran out (it returns instead of spinning on) */
#define VNM_ERR_IO 7           /* file could not be read or written */
#define VNM_ERR_FORMAT 8       /* Matrix Market banner/size/type not supported */
#define VNM_ERR_NO_DEVICE 9    /* no usable CUDA device */
#define VNM_ERR_LIMIT 10       /* a size above a documented maximum */

#define VNM_MEM_HOST 0
#define VNM_MEM_DEVICE 1

typedef struct vnm_ctx vnm_ctx;

/* Human-readable text of a status code (static storage). */
const char* vnm_status_string(vnm_status s);

/* Library version string, e.g. "0.1.0 sm_103a". */
const char* vnm_version(void);

/* Create a context on CUDA device `device` with its own non-blocking stream. */
vnm_status vnm_create(vnm_ctx** ctx, int device);
vnm_status vnm_destroy(vnm_ctx* ctx);

/* Milliseconds of device time spent in the kernels of the last call
 * (CUDA events on the context's stream, first launch to last). */
float vnm_last_kernel_ms(const vnm_ctx* ctx);
/* Number of kernels the last call launched. */
int vnm_last_launch_count(const vnm_ctx* ctx);

/* Milliseconds of the last call's main kernel alone (the persistent reorder
 * kernel for the NM calls), CUDA events on the context's stream. */
float vnm_last_main_kernel_ms(const vnm_ctx* ctx);

/* Work counters of the last NM call (for roofline accounting):
 * out[0] rounds summed over jobs, out[1] column entries gathered,
 * out[2] row records touched, out[3] segments per job, out[4] jobs,
 * out[5] nonzero-valued entries of the pattern, out[6] thread blocks per
 * job (the cluster size the launch used), out[7] block-rounds whose row
 * records were in the block's shared-memory table (a block keeps the
 * records of the rows it owns; summed over blocks and jobs), out[8..14]
 * time spent per round phase (select, choose, gather, process, heap
 * entries, swap heaps and walk overlapped, apply) in units of 1024 ns,
 * summed over jobs (with vnm_nm_set_phase_timing on, else 0),
 * out[15] block-rounds whose row records were in global memory (the
 * block's entries would have filled more than 3/4 of its table), out[16]
 * the time from the round kernel's start to its end in units of 1024 ns
 * summed over jobs (out[8..14] plus the set-up and the final write-back),
 * out[17] the
 * spread of the jobs' start times and out[18] the span from the first
 * start to the last end, in microseconds (jobs that run at once start
 * together), out[19] how many clusters of the launched size the GPU can
 * hold at once by the occupancy query (0 for single-block launches),
 * out[20], out[21] the leaders' own work in the process and apply phases
 * (before the barriers that close them), units of 1024 ns summed over
 * jobs, out[22..27] times inside phases in the same units (out[20..27]
 * other than out[23] with vnm_nm_set_phase_timing on, else 0): the walk warp,
 * its waits for swap-heap pops, warp 0 of the leader over its rows in
 * the process phase and in the apply phase, and that warp's per-segment
 * masks and pair corrections in the process phase.  n <= 28 values. */
vnm_status vnm_last_stats(const vnm_ctx* ctx, long long* out, int n);

/* ---------------------------------------------------------------------------
 * NM reorder
 * ------------------------------------------------------------------------- */

/* One reorder job: reorderUtil<float>(mat, nm_maxiter) followed by
 * run_onepair (sched 0), run_onepair_double (1), run_onepair_reverse (2) or
 * run_onepair_reverse_double (3).  Replaces reorder/reorder.h:1805-2474
 * together with LocateinvalidSegment, GetSegSwapScore, LocateAllZeroSegment,
 * Reorder and Mtx::reset (reorder/reorder.h:23-317, :392-418,
 * mtx/Mtx.h:437-478).
 *
 * Entries whose value is 0.0f are not part of the N:M bitmap, as in
 * reorder/reorder.h:93.  Requires 1 <= N < M <= 8.
 *
 * Outputs (host memory, caller-owned):
 *   res5[5]   = {init_size, final_size, init_cnt, final_cnt, rounds}, the
 *               vector run_onepair* returns (reorder/reorder.h:1966)
 *   newpos    = optional (NULL to skip), length nrows: final position of each
 *               node.  Apply it to a COO with vnm_permute_coo().
 */
vnm_status vnm_nm_reorder(vnm_ctx* ctx, int nrows, int nnz, const int* row, const int* col, const float* val,
                          int mem, int N, int M, int sched, int nm_maxiter, int* res5, int* newpos);

/* All four schedules of one matrix in a single persistent launch, one job
 * per schedule (each job on a thread-block cluster of 2-16 blocks, chosen
 * by matrix size and by what the GPU can co-schedule; vnm_last_stats out[6]
 * reports it); then the choice of find_best_2toX
 * (main.cu:72-114): the largest improve rate (init_cnt-final_cnt)/init_cnt,
 * ties to the lowest schedule id (the reference breaks ties by wall time).
 * Returns 0 as the best schedule when nnz == 0 or init_size == 0 (main.cu:85).
 *   res5x4[20]  = res5 of schedules 0..3
 *   newpos_best = optional, length nrows, the best schedule's permutation
 */
vnm_status vnm_nm_search(vnm_ctx* ctx, int nrows, int nnz, const int* row, const int* col, const float* val,
                         int mem, int N, int M, int nm_maxiter, int* best_sched, int* res5x4, int* newpos_best);

/* Many independent matrices, each with one schedule, reordered in one
 * persistent launch (a two-block cluster per matrix).  Matrix b occupies
 * row/col/val[nnz_offset[b] .. nnz_offset[b+1]) and has nrows[b] rows;
 * newpos (optional) is laid out at row_offset[b] = sum of nrows[0..b).
 * All arrays are host arrays.  res5 is [nmat][5]. */
vnm_status vnm_nm_reorder_batch(vnm_ctx* ctx, int nmat, const int* nrows, const int64_t* nnz_offset,
                                const int* row, const int* col, const float* val, int N, int M, int sched,
                                int nm_maxiter, int* res5, int* newpos);

/* Record of the swaps committed by one job (parity diagnostics): after a
 * vnm_nm_reorder call with tracing on, `pairs` receives up to `cap` (v1, v2)
 * position pairs in commit order and round_end[r] the number of pairs
 * committed by the end of round r.  Tracing is off unless enabled. */
vnm_status vnm_nm_set_trace(vnm_ctx* ctx, int enable);

/* Per-phase timers of the round kernel (vnm_last_stats out[8..14] and
 * out[20..27] other than out[23]).  Off by default: reading the global
 * timer at every phase boundary on the leader's critical path costs about
 * 2.5 % of the kernel's time, so those values read 0 unless this is
 * enabled.  No counterpart in the reference. */
vnm_status vnm_nm_set_phase_timing(vnm_ctx* ctx, int enable);
vnm_status vnm_nm_get_trace(vnm_ctx* ctx, int* pairs, int cap_pairs, int* npairs, int* round_end, int cap_rounds,
                            int* nrounds);

/* vnm_nm_reorder for callers that cannot allocate device memory.  No
 * counterpart in the reference.  Some callers cannot call cudaMalloc:
 * services whose device memory is all handed out up front by their own
 * allocator, and latency-critical loops where an allocation (which can
 * synchronise the device) is not allowed.  This entry point allocates
 * nothing and needs no context: its scratch is one fixed array in device
 * memory of VNM_NOALLOC_SCRATCH_BYTES, which every GPU that loads the
 * library keeps until the process exits.
 *   - row, col, val: device memory of the current device, sorted COO as for
 *     vnm_nm_reorder; res5 (5 ints) and newpos (nrows ints): device memory
 *     the caller owns; work is issued on `stream` (a cudaStream_t, NULL for
 *     the default stream).  The call reads a status back on the host and
 *     synchronises `stream` before it returns.
 *   - nrows <= VNM_NOALLOC_MAX_ROWS and nnz <= VNM_NOALLOC_MAX_NNZ, else
 *     VNM_ERR_LIMIT.
 *   - Each call looks up the array's device address on the current device
 *     (no stream work), so a device reset between calls does no harm.
 *   - Each job runs on a thread-block cluster sized as vnm_nm_reorder sizes
 *     it; results are identical to vnm_nm_reorder's.
 *   - All calls share the array.  Calls that overlap on the GPU (from other
 *     streams or host threads) race; serialise them. */
#define VNM_NOALLOC_MAX_ROWS 32768
#define VNM_NOALLOC_MAX_NNZ 524288
#define VNM_NOALLOC_SCRATCH_BYTES (16u << 20)
vnm_status vnm_nm_reorder_noalloc(int nrows, int nnz, const int* row, const int* col, const float* val, int N, int M,
                                  int sched, int nm_maxiter, int* res5, int* newpos, void* stream);

/* Apply a node permutation to a COO in place: row = newpos[row],
 * col = newpos[col] -- the Reorder kernel of reorder/reorder.h:23-35 with all
 * rounds composed.  The order of the entries does not change. */
vnm_status vnm_permute_coo(vnm_ctx* ctx, int nrows, int nnz, int* row, int* col, int mem, const int* newpos);

/* vnm_permute_coo for device arrays, enqueued on the caller's `stream` (a
 * cudaStream_t, NULL = the default stream) without waiting. */
vnm_status vnm_permute_coo_async(vnm_ctx* ctx, int nrows, int nnz, int* row, int* col, const int* newpos,
                                 void* stream);

/* Per-segment counts of the current matrix: invalid[s] = rows whose M-group
 * in segment s has more than N nonzeros (LocateinvalidSegment,
 * reorder/reorder.h:262-289); allzero[s] = rows whose group is empty
 * (LocateAllZeroSegment, :291-317).  Host outputs of length nrows/M. */
vnm_status vnm_nm_segment_counts(vnm_ctx* ctx, int nrows, int nnz, const int* row, const int* col,
                                 const float* val, int mem, int N, int M, int* invalid, int* allzero);

/* Swap gains of one segment pair (GetSegSwapScore, reorder/reorder.h:74-131):
 * score[(i*M+j)*2+0] = left gain, score[(i*M+j)*2+1] = right gain. */
vnm_status vnm_nm_pair_score(vnm_ctx* ctx, int nrows, int nnz, const int* row, const int* col, const float* val,
                             int mem, int N, int M, int seg1, int seg2, int* score);

/* ---------------------------------------------------------------------------
 * Learned-proposal reorder.  No counterpart in the reference: a parallel
 * search with the reference's objective (fewer invalid M-groups), or with
 * the retained-nonzero count of an N:M pruning, for matrices where the
 * sequential greedy of run_onepair is too slow.  Not bit-exact with
 * vnm_nm_reorder by design.
 *
 * Each round, every segment holding an invalid group proposes swaps of its
 * M nodes with the nodes of `targets` sampled segments (targets*M*M
 * candidates); the candidates are ranked (by the proposal network, at
 * random, or not at all), the best topk (or all, exhaustive mode) are scored
 * exactly by an integer kernel, each segment keeps its best improving swap,
 * and a claim-based matching accepts swaps that touch disjoint segments, so
 * every accepted gain is exact and they add up.  Rounds stop after
 * `max_rounds`, when no segment holds an invalid group, after `patience`
 * rounds in a row that accepted nothing, or once the gain reaches
 * `stop_gain` (time to a target quality).  The network proposes at most one
 * swap per target segment.
 * ------------------------------------------------------------------------- */

#define VNM_LEARNED_MLP 0        /* network ranks, the top topk scored exactly */
#define VNM_LEARNED_EXHAUSTIVE 1 /* every candidate scored exactly */
#define VNM_LEARNED_RANDOM 2     /* topk random candidates scored exactly */

#define VNM_MLP_FEATURES 32
#define VNM_MLP_HIDDEN 128

/* Proposal network: 32 features -> 128 -> 128 -> 1, ReLU, BF16 operands
 * and FP32 accumulation at inference (tcgen05), FP32 master weights and
 * Adam state on the device.  Parameter vector (vnm_mlp_param_count floats):
 * W1[128][32], b1[128], W2[128][128], b2[128], w3[128], b3. */
typedef struct vnm_mlp vnm_mlp;
int vnm_mlp_param_count(void);
vnm_status vnm_mlp_create(vnm_ctx* ctx, unsigned seed, vnm_mlp** net);
vnm_status vnm_mlp_free(vnm_mlp* net);
vnm_status vnm_mlp_get(const vnm_mlp* net, float* params);
vnm_status vnm_mlp_set(vnm_mlp* net, const float* params); /* also resets Adam */
/* Scores of n feature rows X[n][32] (host) into Y[n] (host), tensor cores. */
vnm_status vnm_mlp_forward(vnm_ctx* ctx, const vnm_mlp* net, const float* X, int n, float* Y);
/* Gradient of L = mean((f(x) - t)^2) / 2 over one batch of B rows (host
 * X[B][32], t[B]); the forward pass rounds layer inputs and weights to BF16
 * as the inference does.  grads: vnm_mlp_param_count floats (host). */
vnm_status vnm_mlp_grad(vnm_ctx* ctx, vnm_mlp* net, const float* X, const float* t, int B, float* grads,
                        float* loss);
/* Adam (beta 0.9 / 0.999) over n rows in mini-batches of B, `epochs` passes
 * in the given order; *final_loss = mean batch loss of the last pass. */
vnm_status vnm_mlp_train(vnm_ctx* ctx, vnm_mlp* net, const float* X, const float* t, int n, int B, int epochs,
                         float lr, float* final_loss);

typedef struct vnm_learned_params {
  int mode;            /* VNM_LEARNED_* */
  int objective;       /* 0 invalid groups, 1 retained nonzeros (sum of min(popcount, N)) */
  int targets;         /* target segments sampled per proposing segment and round; targets*M*M <= 2048 */
  int topk;            /* proposals per segment scored exactly (1..8; network and random modes) */
  int max_rounds;
  int patience;        /* >= 1 */
  unsigned seed;
  int dump_every;      /* > 0: keep 1 in dump_every exactly scored candidates as training pairs */
  int dump_cap;        /* capacity of the dump buffers (pairs) */
  float* dump_features; /* host [dump_cap][32] */
  float* dump_gains;    /* host [dump_cap], exact gain in objective units */
  long long stop_gain;  /* > 0: stop once the accepted gains add up to this much */
} vnm_learned_params;

typedef struct vnm_learned_result {
  long long init_invalid, final_invalid;   /* groups with popcount > N */
  long long init_retained, final_retained; /* sum over groups of min(popcount, N) */
  long long gain;                          /* sum of accepted exact gains */
  long long exact_scored;                  /* candidates scored exactly */
  int rounds, swaps, ndump, reserved;
} vnm_learned_result;

/* Same input contract as vnm_nm_reorder; newpos optional (nrows ints). */
vnm_status vnm_nm_learned(vnm_ctx* ctx, int nrows, int nnz, const int* row, const int* col, const float* val,
                          int mem, int N, int M, const vnm_mlp* net, const vnm_learned_params* params,
                          vnm_learned_result* result, int* newpos);

/* ---------------------------------------------------------------------------
 * VNM stage (the row sort of reordering.py)
 * ------------------------------------------------------------------------- */

/* `python3 reordering.py --evalonly --m M --v V` (reordering.py:187-198):
 * out2 = {V-blocks whose OR over V rows has more than 4 ones, the same
 * count also flagging blocks with a row of more than 2 ones}.  m, n are the
 * matrix shape (padded to multiples of M inside, reordering.py:50-51); the
 * pattern is every stored entry (values are not read).  COO in any order. */
vnm_status vnm_vnm_eval(vnm_ctx* ctx, int m, int n, int nnz, const int* row, const int* col, int mem, int M, int V,
                        int* out2);

/* `python3 reordering.py --m M --v V` (reordering.py:200-265): repeated
 * stable sorts of the rows by their Gray-code hashed segment strings, each
 * applied to rows and columns, stopping when the V-block count grows or
 * reaches 0 or after max(maxiter, initial count) rounds.  row/col are
 * replaced by the matrix the script writes back (entries keep their order).
 *   out5   = the five integers of output.txt:
 *            {init, init_strict, final, final_strict, rounds}
 *   newpos = optional, length m padded to M: final position of each row. */
vnm_status vnm_vnm_reorder(vnm_ctx* ctx, int m, int n, int nnz, int* row, int* col, int mem, int M, int V,
                           int maxiter, int* out5, int* newpos);

/* ---------------------------------------------------------------------------
 * V:N:M SpMM (replaces the BSR WMMA kernel of kernel/spmm.cu:44-161)
 * ------------------------------------------------------------------------- */

typedef struct vnm_spmm_matrix vnm_spmm_matrix;

/* Compress a (reordered) sparse matrix into the V:N:M layout the SpMM
 * kernels read: 128-row tiles; every V x M block with at least V nonzeros
 * (VNM_SPMM_DENSE_MIN in the environment sets another threshold, 0 = every
 * block) is cut into slices of 4 columns with at most 2 nonzeros per row
 * (one slice when the block satisfies V:N:M, more when it does not, so
 * nothing is dropped) for the tensor cores; their values are divided by
 * their V-block row's largest magnitude and stored as `dtype` (1 = BF16,
 * 0 = FP16).  The nonzeros of sparser blocks form a row-major residual
 * (FP32 values) that a CUDA-core kernel multiplies.  Requires 128 % V == 0,
 * 2 <= M <= 8.
 * COO in any order.  The result lives in device memory of the context's
 * GPU until vnm_spmm_free; its storage is taken from the last operand this
 * context's operands freed when that is large enough, else allocated. */
vnm_status vnm_spmm_compress(vnm_ctx* ctx, int nrows, int nnz, const int* row, const int* col, const float* val,
                             int mem, int M, int V, int dtype, vnm_spmm_matrix** out);

/* info[0..12] = {nnz, non-empty blocks, blocks that satisfy V:N:M, slices,
 * slices after padding tiles to K-steps of 4, K-steps, tiles, bytes of A
 * tiles, residual nonzeros, residual tasks, tiles with tensor-core work,
 * the block threshold used, partial rows of split residual rows}. */
vnm_status vnm_spmm_info(const vnm_spmm_matrix* A, long long* info, int n);

/* C (nrows x n, FP32, row-major) = A * B with B (nrows x n, row-major, the
 * compressed dtype).  n must be a multiple of 64.  mem = where B and C are
 * (device: 16-byte aligned).  The tensor-core kernel works on column blocks
 * of 256, 128 or 64; the first call of a context for an operand shape (rows, K-steps)
 * and n times each width that divides n once and keeps the fastest for
 * later calls (up to 8 shapes per context).  VNM_SPMM_WIDTH=64|128|256 in
 * the environment fixes the width where it divides n. */
vnm_status vnm_spmm_run(vnm_ctx* ctx, const vnm_spmm_matrix* A, const void* B, int n, float* C, int mem);

/* vnm_spmm_run on the caller's stream, for device buffers, without
 * waiting: the kernels are enqueued on `stream` (a cudaStream_t, NULL = the
 * default stream) after the work the caller enqueued there, and the call
 * returns at once.  B (nrows x n, the operand's 16-bit type) and C (nrows x
 * n, FP32) are device memory, 16-byte aligned, valid until the stream
 * reaches the product.  Exceptions to "without waiting": the first call for
 * an operand shape and n times the tensor-core column-block widths
 * (synchronising `stream` once), and the first call with a larger n than
 * before allocates the operand's scratch (cudaMalloc).  Calls on one operand
 * share that scratch, so they must run in order (one stream, or streams the
 * caller orders).  A bounded wait that ran out inside the tensor-core kernel
 * sets a flag on the operand; vnm_spmm_check reads it. */
vnm_status vnm_spmm_run_async(vnm_ctx* ctx, vnm_spmm_matrix* A, const void* B, int n, float* C, void* stream);

/* Waits for `stream`; *failed = 1 when a vnm_spmm_run_async of A failed
 * inside a kernel since the last check (the flag is cleared), else 0. */
vnm_status vnm_spmm_check(vnm_spmm_matrix* A, void* stream, int* failed);

/* Release an operand.  While its context lives, the context keeps the
 * largest freed operand's device storage for its next vnm_spmm_compress
 * (no cudaMalloc there, no device-wide synchronisation here) and releases
 * it in vnm_destroy; an operand may outlive its context. */
vnm_status vnm_spmm_free(vnm_spmm_matrix* A);

/* ---------------------------------------------------------------------------
 * Matrix Market files and the text round trips of the `spmm` pipeline
 * (host code)
 * ------------------------------------------------------------------------- */

/* readMtx + Mtx::init_from_file (mtx/readMtx.hpp:354-425, mtx/Mtx.h:98-112):
 * banner and size line, tuples, symmetric banners mirrored, repeated entries
 * removed, sorted by (row, col), rows and cols padded to a multiple of
 * `aligned`.  Arrays are malloc'ed; release them with vnm_host_free. */
vnm_status vnm_mtx_read(const char* path, int aligned, int* nrows, int* ncols, int* nnz, int** row, int** col,
                        float** val);
void vnm_host_free(void* p);

/* Mtx::write_to_file (mtx/Mtx.h:412-435): "real general" banner, size line,
 * "%d %d %.2f" entries in the given order, 1-based. */
vnm_status vnm_mtx_write(const char* path, int nrows, int ncols, int nnz, const int* row, const int* col,
                         const float* val);

/* Values as the VNM stage reads them from the NM stage's temp.mtx: the
 * float64 of each value's "%.2f" text (main.cu:246-247, reordering.py:41). */
vnm_status vnm_text_nm_values(int nnz, const float* val, double* out);

/* temp.mtx written by the VNM stage (scipy mmwrite, precision=1:
 * reordering.py:179-181) and read back by the NM stage (readMtx): "%.0e"
 * values; under 100 rows with symmetric values only the lower triangle,
 * mirrored back by the reader.  In: the VNM stage's n x n matrix in its
 * entry order.  Out: the reader's COO (malloc'ed). */
vnm_status vnm_text_vnm_roundtrip(int n, int nnz, const int* row, const int* col, const double* val, int aligned,
                                  int* out_nrows, int* out_nnz, int** out_row, int** out_col, float** out_val);

/* Host helper: the pop order of the SwapPair priority queue of
 * reorder/reorder.h:521-532 (Comparator, reorder/swappair.h:112-120) for n
 * pairs pushed in index order -- the exact emulation the kernels use. */
vnm_status vnm_swap_heap_order(int n, const int* lg, const int* rg, int* order);

#ifdef __cplusplus
}
#endif
#endif /* VNM_GB300_H */
