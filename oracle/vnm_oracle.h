/*
 * CPU oracle for the V:N:M graph-reordering path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: the parity tests,
 * the smoke check and the CPU-baseline leg of the benchmark call it.  The
 * product (the CUDA library and the `spmm` drop-in) never links or calls it.
 *
 * It restates, in plain C++17, the algorithms of PictureResearch/
 * vnm-graph-reordering for the path that the GPU library replaces:
 *   - Matrix Market input/output        mtx/readMtx.hpp, mtx/mmio.hpp, mtx/Mtx.h
 *   - NM reorder, schedules 0-3         reorder/reorder.h, reorder/swappair.h
 *   - VNM row sort (reordering.py)      reordering.py
 *   - schedule search + hybrid driver   main.cu
 * Each function cites the reference lines it follows.
 *
 * All entry points use plain C types so that Python (ctypes) can drive them.
 * Arrays returned through `T**` out-parameters are malloc'ed and must be
 * released with orc_free().
 */
#ifndef VNM_ORACLE_H
#define VNM_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define ORC_OK 0
#define ORC_ERR_IO 1          /* file not found / unwritable */
#define ORC_ERR_FORMAT 2      /* bad banner / size line / unsupported type */
#define ORC_ERR_ARG 3         /* bad N, M, V, schedule, sizes */
#define ORC_ERR_INTERNAL 4    /* an invariant of the reference algorithm broke */

void orc_free(void* p);

/* Number of OpenMP threads the oracle may use (1 = scalar port). */
void orc_set_threads(int nthreads);
int orc_get_max_threads(void);

/* readMtx + Mtx::init_from_file (mtx/readMtx.hpp:354-425, mtx/Mtx.h:98-112).
 * Returns COO sorted by (row, col), symmetric banners mirrored, duplicates
 * removed, rows (and cols) padded up to a multiple of `aligned`.
 * `is_symmetric_out` reports the banner's storage scheme ('S' only). */
int orc_mtx_read(const char* path, int aligned, int* nrows, int* ncols,
                 int* nnz, int** row, int** col, float** val);

/* Mtx::write_to_file (mtx/Mtx.h:412-435): banner, "R C nnz", "%d %d %.2f". */
int orc_mtx_write(const char* path, int nrows, int ncols, int nnz,
                  const int* row, const int* col, const float* val);

/* One NM reorder job: reorderUtil(mat, 10) + run_onepair* for `sched`
 * (reorder/reorder.h:322-335, :1805-2474).  The COO arrays are permuted in
 * place exactly as the Reorder kernel does (order of entries unchanged).
 * Entries with val == 0.0f are not part of the N:M bitmap (reorder.h:93).
 *   res5   = {init_size, final_size, init_cnt, final_cnt, rounds}
 *   newpos = (optional, length nrows) final position of each start position.
 * `nm_maxiter` is the MAXITER the reorderUtil is built with (10 in main.cu). */
int orc_nm_run(int nrows, int nnz, int* row, int* col, const float* val,
               int N, int M, int sched, int nm_maxiter, int* res5,
               int* newpos);

/* Per-round trace of orc_nm_run: for each round, the swaps committed, as
 * (v1, v2) position pairs, flattened; `round_ptr[r]..round_ptr[r+1]` index
 * into `pairs` (in units of pairs).  Used by the parity tests to localise a
 * divergence.  Caller frees *pairs and *round_ptr. */
int orc_nm_run_trace(int nrows, int nnz, int* row, int* col, const float* val,
                     int N, int M, int sched, int nm_maxiter, int* res5,
                     int** pairs, int** round_ptr, int* nrounds);

/* LocateinvalidSegment / LocateAllZeroSegment counts for the current COO
 * (reorder/reorder.h:262-317): per segment, #rows with popcount > N and
 * #rows with an all-zero group. */
int orc_nm_segment_counts(int nrows, int nnz, const int* row, const int* col,
                          const float* val, int N, int M, int* invalid,
                          int* allzero);

/* GetSegSwapScore (reorder/reorder.h:74-131) for one (seg1, seg2) pair:
 * score[(i*M+j)*2+0] = left gain, [..+1] = right gain. */
int orc_nm_pair_score(int nrows, int nnz, const int* row, const int* col,
                      const float* val, int N, int M, int seg1, int seg2,
                      int* score);

/* Pop order of the SwapPair priority queue (reorder/reorder.h:521-532 with
 * Comparator of reorder/swappair.h:112-120): `n` pairs with gains lg/rg are
 * pushed in index order, then popped until empty; order[k] = index popped
 * k-th.  Exercises libstdc++'s heap exactly as the reference does. */
void orc_swap_heap_order(int n, const int* lg, const int* rg, int* order);

/* reordering.py --evalonly (reordering.py:187-198): out2 = {invalid V-blocks,
 * strict invalid V-blocks}.  m, n are the file's shape (padded inside). */
int orc_vnm_eval(int m, int n, int nnz, const int* row, const int* col,
                 int M, int V, int* out2);

/* reordering.py main loop (reordering.py:200-265).  row/col are replaced by
 * the state the script writes back to temp.mtx.  out5 = the five integers
 * of output.txt.  newpos (optional, length padded m) = composed row map. */
int orc_vnm_run(int m, int n, int nnz, int* row, int* col, int M, int V,
                int maxiter, int* out5, int* newpos);

/* Value after the NM writer's "%.2f" text round trip (mtx/Mtx.h:431 then
 * fscanf "%f", mtx/readMtx.hpp:115). */
float orc_roundtrip_nm(float v);
/* Value after the VNM writer: scipy mmwrite(precision=1) prints "%.0e" of
 * the float64 it read; the NM reader parses it back with "%f"
 * (reordering.py:181, mtx/readMtx.hpp:115). */
float orc_roundtrip_vnm(float v);

/* find_best_2toX (main.cu:72-114) on an in-memory matrix.  Ties in improve
 * rate go to the lowest schedule id (the reference breaks them by measured
 * wall time, which is not reproducible).  out12x4 = graph_NM_reordering's
 * 12-float vectors (timing slot = 0), 4 rows.  Returns best schedule via
 * *best. */
int orc_find_best(int nrows, int nnz, const int* row, const int* col,
                  const float* val, int N, int M, int nscheds, int* best,
                  float* out12x4);

/* The whole `spmm` command (main.cu:339-352) with the file round trips of
 * main.cu:246-311 and reordering.py emulated in memory.  `init_mb_path`, if
 * non-NULL, is the stale temp.mtx that eval_venom reads before the first NM
 * pass (main.cu:207); NULL evaluates the input matrix instead.
 * csv16 = the 16 numbers printed at main.cu:331-335 (ms slot = 0).
 * The final matrix (the --outmtxfile contents) is returned in out_*. */
int orc_spmm_cli(const char* mtxfile, const char* init_mb_path, int N, int M,
                 int V, int maxiter, double* csv16, int* best_sched,
                 int* out_nrows, int* out_nnz, int** out_row, int** out_col,
                 float** out_val);

/* The same with the schedule fixed (force_sched 0..3; -1 = search).
 * find_best_2toX breaks ties on improve rate by measured wall time
 * (main.cu:90-99), so a recorded run of the reference command is
 * reproduced by giving the schedule it picked. */
int orc_spmm_cli_sched(const char* mtxfile, const char* init_mb_path, int N,
                       int M, int V, int maxiter, int force_sched,
                       double* csv16, int* best_sched, int* out_nrows,
                       int* out_nnz, int** out_row, int** out_col,
                       float** out_val);

/* Retained-nnz (project metric): N:M = sum over (row, seg) of min(popc, N);
 * V:N:M = per (V-block, seg) keep the 4 columns with most nonzeros (ties to
 * the lower offset), then sum over rows of min(popc(row & kept), N). */
int64_t orc_retained_nm(int nrows, int nnz, const int* row, const int* col,
                        const float* val, int N, int M);
int64_t orc_retained_vnm(int nrows, int nnz, const int* row, const int* col,
                         const float* val, int N, int M, int V);

/* FP64 reference SpMM: C[nrows x n] = A (COO) * B[ncolsA x n], row-major. */
void orc_spmm_f64(int nrows, int nnz, const int* row, const int* col,
                  const double* val, const double* B, int n, double* C);

#ifdef __cplusplus
}
#endif
#endif
