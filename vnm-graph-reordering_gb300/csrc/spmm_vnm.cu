// V:N:M SpMM: C = A * B with A sparse (the reordered matrix) and B dense,
// BF16 or FP16 operands, FP32 accumulation.  Dense V:N:M blocks run on the
// tcgen05 tensor cores; the blocks too sparse to pay for a tensor-core tile
// run on the CUDA cores.
//
// Replaces the reference's BSR WMMA kernel (kernel/spmm.cu:44-161), which
// runs one warp per 16x16 output tile with wmma m16n16k16 over 16x16 BSR
// blocks.  Here A is first compressed into its V:N:M layout and the dense
// products run as tcgen05.mma with the accumulator in tensor memory.
//
// Layout (the compressor below builds it on the device):
//   - rows are cut into tiles of 128 (the MMA's M); V must divide 128, so a
//     tile holds 128 / V block rows of V rows each.
//   - every non-empty (block row, segment) block -- V rows x M columns --
//     with at least `dense_min` nonzeros is cut into slices: 4 of its
//     columns, and per row at most 2 nonzeros among them (2:4 inside the
//     slice).  A block that satisfies V:N:M (at most 4 nonzero columns, at
//     most 2 nonzeros per row) is one slice; a block that does not spills
//     into more slices, so no nonzero is dropped and the product is exact up
//     to the operand rounding.
//   - 4 slices make one K-step of 16: the A operand of a K-step (128 rows x
//     16) is stored ready for the MMA (K-major, core matrices of 8 rows x 16
//     bytes), and the 16 B rows it multiplies are listed by index (-1 for a
//     column that only pads a slice: its B row is zero-filled, not read).
//   - values are stored divided by their block row's scale (max |a| of the
//     V rows), and the epilogue multiplies each output row back by it.
//   - the nonzeros of sparser blocks form the residual: a row-major CSR with
//     FP32 values, cut into tasks of at most 256 nonzeros of one row (a row
//     with more is split into chunks whose partial rows are added in a fixed
//     order afterwards, so the sums do not depend on timing).  No cap on the
//     chunks of a row: on a power-law graph (Chung-Lu 262144, max degree
//     72098, n=256) a cap of 32 left one warp walking 2254 entries while the
//     other SMs idled: 0.60 ms a product on GB300, 0.39 ms without the cap.
// On graph sparsity most blocks hold one or two nonzeros; a 128 x 16
// tensor-core tile for them would be >99 % padding, while a CUDA-core
// gather reads one B row per nonzero.  `dense_min` (VNM_SPMM_DENSE_MIN in the
// environment, else the default below) sets the split.
//
// Kernels of one product, in stream order:
//   k_spmm_res  CUDA cores: every residual task (and every row of a tile with
//               no tensor-core work) gathers its B rows with 16-byte loads and
//               writes its C row (or a partial row);
//   k_spmm_fin  adds the partial rows of the split rows, in chunk order;
//   k_spmm_vnm  tensor cores, one CTA per (tile with K-steps, column block of
//               C).  A producer warp streams each K-step's A tile (one bulk
//               copy) and copies its 16 B rows with 16-byte cp.async loads
//               into the 128-byte swizzled layout, with the row ids loaded
//               eight K-steps ahead; one thread issues the MMA per K-step;
//               eight stages keep copies in flight while the MMAs run.  Four
//               warps then read the FP32 accumulator out of tensor memory,
//               scale it and store it, or add it to what the residual wrote.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <cstdlib>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "sm100_ptx.cuh"

struct vnm_spmm_matrix {
  int device = 0;
  int R = 0, M = 0, V = 0, dtype = 1;  // dtype: 1 bf16, 0 f16
  int ntiles = 0, nsteps = 0;
  long long nnz = 0, groups = 0, slices = 0, slices_padded = 0, valid_blocks = 0;
  // tensor-core part
  int ntt = 0;                 // tiles with at least one K-step
  int* tile_step = nullptr;    // [ntiles + 1]
  int2* tlist = nullptr;       // [ntt] {tile, 1 when the residual kernel wrote the tile's rows first}
  int* cols = nullptr;         // [nsteps * 16], -1 = padding column
  unsigned char* a = nullptr;  // [nsteps * 4096]
  float* rscale = nullptr;     // [ntiles * 128]
  // CUDA-core part
  int dense_min = 0;           // blocks with fewer nonzeros went to the residual
  long long nres = 0;          // residual nonzeros
  int ntask = 0, nmulti = 0, nslots = 0;
  int2* rcv = nullptr;         // [nres], row-major: {column, value bits}
  int4* task = nullptr;        // [ntask] {row, begin, end, partial slot or -1}
  int4* multi = nullptr;       // [nmulti] {row, first slot, chunks, 0}
  void* base = nullptr;        // one allocation for all of the above
  size_t bytes = 0;            // its size
  vnm_spmm_spare* spare = nullptr;  // the compressing context's spare storage
  // state of the asynchronous entry point, allocated on its first call
  float* part = nullptr;       // partial rows of split rows, for the largest n seen
  size_t part_floats = 0;
  int* err = nullptr;          // sticky failure flag of the tensor-core kernel
};

namespace vnm {

constexpr int SP_TM = 128;        // rows per tile (MMA M)
constexpr int SP_KSTEP_BYTES = 4096;
constexpr int SP_THREADS = 128;
constexpr uint32_t SP_WAIT_LIMIT = 1u << 22;  // polls before a wait gives up
constexpr int RES_CHUNK = 256;    // residual nonzeros per task, at most
constexpr int RES_THREADS = 256;
constexpr int RES_U = 8;          // entries in flight per lane group (8 measured ahead of 4)
constexpr int RES_BLOCKS_PER_SM = 4;  // resident blocks of k_spmm_res an SM (64 registers a thread)
// A block runs on the tensor cores when it holds at least V nonzeros (one
// a row on average), else on the CUDA cores.  Measured on GB300 with the
// R-MAT 16384 (V=64, n=128) and Chung-Lu 262144 (V=128, n=256) operands,
// thresholds 2..64 against all-residual: every tensor-core share was slower
// (C2 0.037 ms all-residual vs 0.046-0.30 ms; C5 0.50 ms vs 0.67-4.9 ms):
// at one or two nonzeros per block a tile is >99 % padding and its fixed
// costs dominate.  A V:N:M operand whose blocks are full (2V nonzeros) goes
// to the tensor cores.  VNM_SPMM_DENSE_MIN overrides the threshold (0 =
// every block on the tensor cores).

static inline int sp_grid(const vnm_ctx* ctx, long long n, int nt = 256) {
  long long g = (n + nt - 1) / nt, cap = (long long)ctx->num_sms * 16;
  if (g > cap) g = cap;
  return g < 1 ? 1 : (int)g;
}

static inline int sp_bits(long long v) {
  int b = 1;
  while ((1ll << b) <= v) ++b;
  return b;
}

// ---------------------------------------------------------------------------
// Compressor
// ---------------------------------------------------------------------------
// An entry's sort key: its V x M block (block row, segment) in the high
// bits, then the row inside the block (bv = log2 V bits; V is a power of
// two) and the column inside the segment (bm = ceil(log2 M) bits), so that
// every field comes out with a shift and a mask.  Sorted, the keys order the
// entries by block, row, column.
__host__ __device__ inline int key_bits_m(int M) { return M <= 2 ? 1 : M <= 4 ? 2 : 3; }

__global__ void k_cmp_keys(const int* row, const int* col, int nnz, int M, int V, int nseg, int bm, int bv,
                           unsigned long long* keys) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nnz; i += gridDim.x * blockDim.x) {
    const int r = row[i], c = col[i];
    const unsigned long long blk = (unsigned long long)(r >> bv) * nseg + (unsigned)(c / M);
    keys[i] = (((blk << bv) | (unsigned)(r & (V - 1))) << bm) | (unsigned)(c % M);
  }
}

__global__ void k_cmp_heads(const unsigned long long* keys, int nnz, int sh, int* flag) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nnz; i += gridDim.x * blockDim.x)
    flag[i] = (i == 0) || ((keys[i] >> sh) != (keys[i - 1] >> sh));
}

__global__ void k_cmp_group_start(const int* flag_scan, const unsigned long long* keys, int nnz, int sh,
                                  int* gstart) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nnz; i += gridDim.x * blockDim.x)
    if (i == 0 || (keys[i] >> sh) != (keys[i - 1] >> sh)) gstart[flag_scan[i]] = i;
}

// max |a| per block row of V rows, over the entries in sorted order: a
// thread takes SCALE_RUN consecutive entries (nearly always of one block
// row) and issues one atomic per block row it saw, instead of one per entry
// all landing on a few hundred words.
constexpr int SCALE_RUN = 16;
__global__ void k_cmp_scale(const unsigned long long* skeys, const int* spos, const float* val, int nnz, int sh,
                            int nseg, unsigned* bmax) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t * SCALE_RUN < nnz;
       t += (long long)gridDim.x * blockDim.x) {
    const int b = (int)(t * SCALE_RUN), e = min(b + SCALE_RUN, nnz);
    long long cur = -1;
    unsigned long long lo = 1, hi = 0;  // the blocks of block row `cur`: [lo, hi)
    unsigned m = 0;
    for (int i = b; i < e; ++i) {
      const unsigned long long blk = skeys[i] >> sh;
      long long br = cur;
      if (blk < lo || blk >= hi) {  // a division only where the block row changes
        br = (long long)(blk / (unsigned long long)nseg);
        lo = (unsigned long long)br * (unsigned long long)nseg;
        hi = lo + (unsigned long long)nseg;
      }
      if (br != cur) {
        if (m) atomicMax(&bmax[cur], m);
        cur = br;
        m = 0;
      }
      m = max(m, __float_as_uint(fabsf(val[spos[i]])));  // non-negative floats order like their bits
    }
    if (m) atomicMax(&bmax[cur], m);
  }
}

// The slices of one block, formed greedily: take the (up to) 4 columns with
// the most remaining nonzeros (ties to the lower offset), give each row at
// most 2 of its remaining nonzeros among them (lowest offsets first), repeat
// until the block is empty.  `emit(sel, nsel, chosen)` is called once per
// slice with the chosen offsets and must remove what each row takes (the
// lowest two bits of mask & chosen).  Row masks: bit o = column offset o.
template <class Emit>
__device__ __forceinline__ int block_slices(unsigned char* mask, int nr, int M, Emit&& emit) {
  int ns = 0;
  for (int guard = 0; guard < 64; ++guard) {
    int cnt[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    bool any = false;
    for (int r = 0; r < nr; ++r)
      for (int o = 0; o < M; ++o)
        if ((mask[r] >> o) & 1u) {
          cnt[o]++;
          any = true;
        }
    if (!any) break;
    int sel[4], nsel = 0;
    unsigned chosen = 0;
    for (int pick = 0; pick < 4; ++pick) {
      int best = -1;
      for (int o = 0; o < M; ++o)
        if (!((chosen >> o) & 1u) && cnt[o] > 0 && (best < 0 || cnt[o] > cnt[best])) best = o;
      if (best < 0) break;
      chosen |= 1u << best;
    }
    for (int o = 0; o < M; ++o)
      if ((chosen >> o) & 1u) sel[nsel++] = o;
    emit(sel, nsel, chosen);
    ++ns;
  }
  return ns;
}

__device__ __forceinline__ unsigned low2(unsigned m) {  // the lowest two set bits of m
  const unsigned a = m & (0u - m);
  const unsigned rest = m & ~a;
  return a | (rest & (0u - rest));
}

// Count slices per block and per tile.  A block with fewer than dense_min
// nonzeros gets no slice: its entries are flagged for the residual (by
// original position), counted per row and per tile.
__global__ void k_cmp_count(const unsigned long long* skeys, const int* spos, const int* gstart, const int* d_ngroups,
                            int nnz, int M, int V, int nseg, int bm, int dense_min, int* gsl, int* tile_raw,
                            int* valid_blocks, int* resflag, int* rowlen, int* tile_res) {
  const int ngroups = *d_ngroups;
  const int sh = bm + __ffs(V) - 1;
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < ngroups; g += gridDim.x * blockDim.x) {
    const int b0 = gstart[g], b1 = g + 1 < ngroups ? gstart[g + 1] : nnz;
    const long long blk = (long long)(skeys[b0] >> sh);
    const int brow = (int)(blk / nseg);
    unsigned char mask[128];
    int nr = 0, lastr = -1;
    for (int i = b0; i < b1; ++i) {
      const unsigned long long k = skeys[i];
      const int rr = (int)(k >> bm) & (V - 1), o = (int)(k & ((1u << bm) - 1u));
      if (rr != lastr) {
        mask[nr++] = 0;
        lastr = rr;
      }
      mask[nr - 1] |= (unsigned char)(1u << o);
    }
    int valid = 1;
    unsigned orb = 0;
    for (int r = 0; r < nr; ++r) {
      orb |= mask[r];
      if (__popc(mask[r]) > 2) valid = 0;
    }
    if (__popc(orb) > 4) valid = 0;
    {  // one atomic per group of converged lanes: every block adds to this one word
      const unsigned am = __activemask();
      const unsigned vb = __ballot_sync(am, valid != 0);
      if ((int)(threadIdx.x & 31) == __ffs(am) - 1 && vb) atomicAdd(valid_blocks, __popc(vb));
    }
    if (b1 - b0 < dense_min) {
      for (int i = b0; i < b1; ++i) {
        resflag[spos[i]] = 1;
        atomicAdd(&rowlen[brow * V + ((int)(skeys[i] >> bm) & (V - 1))], 1);
      }
      atomicAdd(&tile_res[(brow * V) / SP_TM], b1 - b0);
      gsl[g] = 0;
      continue;
    }
    const int ns = block_slices(mask, nr, M, [&](const int*, int, unsigned chosen) {
      for (int r = 0; r < nr; ++r) mask[r] &= ~(unsigned char)low2(mask[r] & chosen);
    });
    gsl[g] = ns;
    atomicAdd(&tile_raw[(brow * V) / SP_TM], ns);
  }
}

__global__ void k_cmp_pad(const int* tile_raw, int ntiles, int* tile_pad, int* tile_has) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < ntiles; t += gridDim.x * blockDim.x) {
    tile_pad[t] = (tile_raw[t] + 3) & ~3;
    tile_has[t] = tile_raw[t] > 0 ? 1 : 0;
  }
}

// The residual entries in their original order, keyed by row for the
// stable sort that makes the CSR.
__global__ void k_res_compact(const int* resflag, const int* rpos, const int* row, int nnz, unsigned long long* rkey,
                              int* rsrc) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nnz; i += gridDim.x * blockDim.x)
    if (resflag[i]) {
      rkey[rpos[i]] = (unsigned long long)(unsigned)row[i];
      rsrc[rpos[i]] = i;
    }
}

__global__ void k_res_gather(const int* src, const int* col, const float* val, int nres, int2* rcv) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nres; i += gridDim.x * blockDim.x) {
    const int e = src[i];
    rcv[i] = make_int2(col[e], __float_as_int(val[e]));
  }
}

// Residual tasks of a row: none when its tile runs on the tensor cores and
// holds no residual entry (the tensor kernel then writes the rows), else one
// per chunk of at most RES_CHUNK entries (one task for an empty row, which
// writes zeros).
__device__ __forceinline__ int res_chunks(int len, bool needed) {
  if (!needed) return 0;
  return len <= RES_CHUNK ? 1 : (len + RES_CHUNK - 1) / RES_CHUNK;
}

__global__ void k_res_task_count(const int* rptr, int R, const int* tile_has, const int* tile_res, int* nmt, int* nst,
                                 int* nmr) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < R; r += gridDim.x * blockDim.x) {
    const int t = r / SP_TM;
    const int nch = res_chunks(rptr[r + 1] - rptr[r], !(tile_has[t] && tile_res[t] == 0));
    nmt[r] = nch > 1 ? nch : 0;
    nst[r] = nch == 1 ? 1 : 0;
    nmr[r] = nch > 1 ? 1 : 0;
  }
}

// Split rows' chunks first (they are the longest tasks), then the others.
__global__ void k_res_task_fill(const int* rptr, int R, const int* tile_has, const int* tile_res, const int* mt_off,
                                const int* st_off, const int* mr_off, int nmt_total, int4* task, int4* multi) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < R; r += gridDim.x * blockDim.x) {
    const int t = r / SP_TM;
    const int b = rptr[r], e = rptr[r + 1];
    const int nch = res_chunks(e - b, !(tile_has[t] && tile_res[t] == 0));
    if (nch == 1) {
      task[nmt_total + st_off[r]] = make_int4(r, b, e, -1);
    } else if (nch > 1) {
      const int base = mt_off[r], csz = (e - b + nch - 1) / nch;
      for (int j = 0; j < nch; ++j) {
        const int cb = min(b + j * csz, e), ce = min(cb + csz, e);
        task[base + j] = make_int4(r, cb, ce, base + j);
      }
      multi[mr_off[r]] = make_int4(r, base, nch, 0);
    }
  }
}

__global__ void k_tile_list(const int* tile_has, const int* tile_res, int ntiles, const int* tl_off, int2* tlist) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < ntiles; t += gridDim.x * blockDim.x)
    if (tile_has[t]) tlist[tl_off[t]] = make_int2(t, tile_res[t] > 0 ? 1 : 0);
}

template <class T>
__device__ __forceinline__ T to_t(float x);
template <>
__device__ __forceinline__ __nv_bfloat16 to_t<__nv_bfloat16>(float x) {
  return __float2bfloat16_rn(x);
}
template <>
__device__ __forceinline__ __half to_t<__half>(float x) {
  return __float2half_rn(x);
}

// Write every block's slices: B-row indices and A values in MMA layout.
template <class T>
__global__ void k_cmp_fill(const unsigned long long* skeys, const int* spos, const float* val, const int* gstart,
                           int ngroups, int nnz, int M, int V, int nseg, int bm, int dense_min, const int* gofs,
                           const int* tile_base, const int* tile_rawbase, const unsigned* bmax, int* cols,
                           unsigned char* a) {
  const int sh = bm + __ffs(V) - 1;
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < ngroups; g += gridDim.x * blockDim.x) {
    const int b0 = gstart[g], b1 = g + 1 < ngroups ? gstart[g + 1] : nnz;
    if (b1 - b0 < dense_min) continue;  // a residual block
    const long long blk = (long long)(skeys[b0] >> sh);
    const int brow = (int)(blk / nseg), seg = (int)(blk % nseg);
    const int t = (brow * V) / SP_TM;
    const float scale = bmax[brow] ? __uint_as_float(bmax[brow]) : 1.0f;
    const float inv = 1.0f / scale;
    unsigned char mask[128], orig[128];
    int rowin[128], first[128];
    int nr = 0, lastr = -1;
    for (int i = b0; i < b1; ++i) {
      const unsigned long long k = skeys[i];
      const int rr = (int)(k >> bm) & (V - 1), o = (int)(k & ((1u << bm) - 1u));
      if (rr != lastr) {
        rowin[nr] = rr;
        first[nr] = i;
        mask[nr] = 0;
        ++nr;
        lastr = rr;
      }
      mask[nr - 1] |= (unsigned char)(1u << o);
    }
    for (int r = 0; r < nr; ++r) orig[r] = mask[r];
    int si = tile_base[t] + (gofs[g] - tile_rawbase[t]);  // this block's first slice
    block_slices(mask, nr, M, [&](const int* sel, int nsel, unsigned chosen) {
      const int ks = si >> 2, j = si & 3;
      for (int q = 0; q < 4; ++q) cols[ks * 16 + 4 * j + q] = q < nsel ? seg * M + sel[q] : -1;
      unsigned char* tile = a + (size_t)ks * SP_KSTEP_BYTES;
      for (int r = 0; r < nr; ++r) {
        const unsigned take = low2(mask[r] & chosen);
        if (!take) continue;
        mask[r] &= ~(unsigned char)take;
        const int rt = (brow * V - t * SP_TM) + rowin[r];  // row inside the tile
        unsigned tt = take;
        while (tt) {
          const int o = __ffs(tt) - 1;
          tt &= tt - 1;
          int kk = 0;
          while (sel[kk] != o) ++kk;
          const int e = spos[first[r] + __popc(orig[r] & ((1u << o) - 1u))];
          const int k = 4 * j + kk;
          const int off = (rt >> 3) * 256 + (k >> 3) * 128 + (rt & 7) * 16 + (k & 7) * 2;
          *reinterpret_cast<T*>(tile + off) = to_t<T>(val[e] * inv);
        }
      }
      ++si;
    });
  }
}

__global__ void k_cmp_rscale(const unsigned* bmax, int ntiles, int R, int V, float* rscale, const int* tile_base,
                             int* tile_step) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ntiles * SP_TM; i += gridDim.x * blockDim.x) {
    const unsigned m = i < R ? bmax[i / V] : 0u;
    rscale[i] = m ? __uint_as_float(m) : 1.0f;
    if (i <= ntiles) tile_step[i] = tile_base[i] >> 2;
  }
}

// ---------------------------------------------------------------------------
// Residual kernels (CUDA cores)
// ---------------------------------------------------------------------------
// acc[0..3] (4 pairs of FP32 accumulators, packed two to a 64-bit register,
// element 0 in the low half) += w * the 8 16-bit values in b (element 0 in
// the low half of b.x), as four packed FP32 FMAs (fma.rn.f32x2: two
// round-to-nearest FP32 FMAs, the same results as eight scalar ones in half
// the instructions); ww is w in both halves.  The accumulators stay packed
// for a whole task.
template <bool BF16>
__device__ __forceinline__ void fma8(unsigned long long (&acc)[4], uint4 b, unsigned long long ww) {
  const uint32_t q[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    uint32_t lo, hi;
    if (BF16) {
      lo = q[i] << 16;
      hi = q[i] & 0xffff0000u;
    } else {
      const float2 f = __half22float2(*reinterpret_cast<const __half2*>(&q[i]));
      lo = __float_as_uint(f.x);
      hi = __float_as_uint(f.y);
    }
    unsigned long long xx;
    asm("mov.b64 %0, {%1, %2};" : "=l"(xx) : "r"(lo), "r"(hi));
    asm("fma.rn.f32x2 %0, %1, %2, %0;" : "+l"(acc[i]) : "l"(ww), "l"(xx));
  }
}

// Groups of LW lanes (32 / LW per warp) walk the task list with a stride
// of every group of the grid (one wave of resident blocks); each lane owns 8
// consecutive columns of the block's 8 * LW.  The records of a task are read
// LW at a time, lane l of the group holding record l, and handed to the
// lanes by shuffles; every lane gathers its 16 bytes of each B row, RES_U
// rows in flight.  The next batch of records, and the next task with its
// first batch, are loaded while the current ones are worked on, so a short
// task costs about one round trip for its B rows.  Loop trip counts are the
// warp's maximum; a group past its end reads a zero weight and a zero row,
// so the arithmetic needs no predicate.
template <int LW, bool BF16>
__global__ void __launch_bounds__(RES_THREADS, RES_BLOCKS_PER_SM)
    k_spmm_res(const int4* __restrict__ task, int ntask, const int2* __restrict__ rcv,
               const unsigned char* __restrict__ B, size_t ldb, float* __restrict__ C, int ldc,
               float* __restrict__ P, int ldp) {
  constexpr int G = 32 / LW;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, grp = lane / LW, lid = lane % LW;
  const int stride = gridDim.x * (RES_THREADS / 32) * G;
  int t = (blockIdx.x * (RES_THREADS / 32) + warp) * G + grp;
  const int cb = blockIdx.y * (8 * LW) + lid * 8;  // this lane's first column
  const unsigned char* bcol = B + (size_t)cb * 2;
  int4 tk = t < ntask ? task[t] : make_int4(0, 0, 0, -1);
  int2 rc = tk.y + lid < tk.z ? __ldg(rcv + tk.y + lid) : make_int2(0, 0);
  int4 tkn = t + stride < ntask ? task[t + stride] : make_int4(0, 0, 0, -1);
  while (__any_sync(0xffffffffu, t < ntask)) {
    const int len = tk.z - tk.y;  // 0 past the end
    const int maxlen = G == 1 ? len : __reduce_max_sync(0xffffffffu, len);
    // the next task's first records, and the task after it
    const int2 rc1 = tkn.y + lid < tkn.z ? __ldg(rcv + tkn.y + lid) : make_int2(0, 0);
    const int4 tk2 = t + 2 * stride < ntask ? task[t + 2 * stride] : make_int4(0, 0, 0, -1);
    unsigned long long acc[4] = {0ull, 0ull, 0ull, 0ull};  // FP32 pairs
    for (int k0 = 0; k0 < maxlen; k0 += LW) {
      const int kn = k0 + LW + lid;
      const int2 rcn = kn < len ? __ldg(rcv + tk.y + kn) : make_int2(0, 0);
#pragma unroll 1
      for (int u0 = 0; u0 < LW; u0 += RES_U) {
        if (k0 + u0 >= maxlen) break;
        uint4 b[RES_U];
#pragma unroll
        for (int u = 0; u < RES_U; ++u) {
          const int col = __shfl_sync(0xffffffffu, rc.x, grp * LW + u0 + u);
          b[u] = k0 + u0 + u < len ? __ldg(reinterpret_cast<const uint4*>(bcol + (size_t)col * ldb))
                                   : make_uint4(0, 0, 0, 0);
        }
        // the weights are fetched once the rows are in flight
#pragma unroll
        for (int u = 0; u < RES_U; ++u) {
          const int vbits = __shfl_sync(0xffffffffu, rc.y, grp * LW + u0 + u);
          const uint32_t w = k0 + u0 + u < len ? (uint32_t)vbits : 0u;
          unsigned long long ww;
          asm("mov.b64 %0, {%1, %1};" : "=l"(ww) : "r"(w));
          fma8<BF16>(acc, b[u], ww);
        }
      }
      rc = rcn;
    }
    if (t < ntask) {
      float* dst = tk.w < 0 ? C + (size_t)tk.x * ldc + cb : P + (size_t)tk.w * ldp + cb;
      float f[8];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        f[2 * i] = __uint_as_float((uint32_t)acc[i]);
        f[2 * i + 1] = __uint_as_float((uint32_t)(acc[i] >> 32));
      }
      reinterpret_cast<float4*>(dst)[0] = make_float4(f[0], f[1], f[2], f[3]);
      reinterpret_cast<float4*>(dst)[1] = make_float4(f[4], f[5], f[6], f[7]);
    }
    t += stride;
    tk = tkn;
    tkn = tk2;
    rc = rc1;
  }
}

// C row of a split row = the sum of its partial rows in a fixed order: the
// block's threads cover the row's float4 columns qpb at a time, and the
// ng = FIN_THREADS / qpb thread groups of a column sum every ng-th chunk
// (group g: chunks g, g + ng, ...) before the group sums are added in group
// order.  A row of a few hundred chunks (a hub of a power-law graph) is then
// not one thread's serial chain of loads.
constexpr int FIN_THREADS = 256;
__device__ __forceinline__ void add4(float4& s, const float4 x) {
  s.x += x.x;
  s.y += x.y;
  s.z += x.z;
  s.w += x.w;
}
__global__ void __launch_bounds__(FIN_THREADS)
    k_spmm_fin(const int4* __restrict__ multi, const float* __restrict__ P, int ldp, float* C, int ldc, int n) {
  __shared__ float4 red[FIN_THREADS];
  const int4 m = multi[blockIdx.x];
  const int nq = n / 4;
  const int qpb = nq < FIN_THREADS ? nq : FIN_THREADS;
  const int ng = FIN_THREADS / qpb;
  const int g = threadIdx.x / qpb, qi = threadIdx.x % qpb;
  for (int q0 = 0; q0 < nq; q0 += qpb) {
    const int q = q0 + qi;
    float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
    if (g < ng && q < nq) {
      const float4* src = reinterpret_cast<const float4*>(P + (size_t)m.y * ldp) + q;
      const size_t step = (size_t)ng * (ldp / 4);
      int j = g;
      for (; j + 3 * ng < m.z; j += 4 * ng) {  // four loads in flight, added in chunk order
        const float4 x0 = src[(size_t)j * (ldp / 4)], x1 = src[(size_t)j * (ldp / 4) + step],
                     x2 = src[(size_t)j * (ldp / 4) + 2 * step], x3 = src[(size_t)j * (ldp / 4) + 3 * step];
        add4(s, x0);
        add4(s, x1);
        add4(s, x2);
        add4(s, x3);
      }
      for (; j < m.z; j += ng) add4(s, src[(size_t)j * (ldp / 4)]);
    }
    red[threadIdx.x] = s;
    __syncthreads();
    if (g == 0 && q < nq) {
      float4 t = red[qi];
      for (int h = 1; h < ng; ++h) add4(t, red[h * qpb + qi]);
      reinterpret_cast<float4*>(C + (size_t)m.x * ldc)[q] = t;
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Tensor-core kernel
// ---------------------------------------------------------------------------
struct SpmmArgs {
  const int2* tlist;
  const int* tile_step;
  const int* cols;
  const unsigned char* a;
  const unsigned char* B;  // dense operand, row-major, 16-bit values
  size_t ldb;              // its row stride in bytes
  const float* rscale;
  float* C;
  int R, n, ldc;
  uint32_t idesc;
  int* err;
  uint32_t wait_limit;  // polls of a pipeline wait (copies <-> MMAs) before it gives up
};

// K-steps in flight per CTA (192 KB of stages at NT = 256).  On a full
// V:2:8 operand (19456 rows, n=256) with three producer warps: 8 stages
// 0.161 ms, 10 0.145, 12 0.143, 14 0.133, 16 0.128 (one producer warp had
// been faster with 8: 0.25 against 0.29 ms).
constexpr int SP_STAGES = 16;
constexpr int SP_PF = 8;      // pairs of K-steps whose column ids are loaded ahead (the ids come from DRAM)

template <int NT>
struct SpmmSmem {
  static constexpr int B_BYTES = 16 * NT * 2;  // K=16 rows x NT columns, 16-bit
  alignas(1024) unsigned char b[SP_STAGES][B_BYTES];
  alignas(1024) unsigned char a[SP_STAGES][SP_KSTEP_BYTES];
  alignas(8) uint64_t full[SP_STAGES];
  alignas(8) uint64_t empty[SP_STAGES];
  alignas(8) uint64_t done;
  int last_k[SP_STAGES];  // the last K-step whose copies were issued into each stage
  uint32_t tmem_base;
  int abort;
};

// Warps that issue the copies: every warp but warp 1, whose lane 0 issues
// the MMAs.  K-step i is copied by producer i % SP_PRODUCERS.  One producer
// warp left the tensor pipe idle ~80 % of the time on a full V:2:8 operand
// (16 B-row copies, their shuffles and addresses per K-step on one warp).
constexpr int SP_PRODUCERS = SP_THREADS / 32 - 1;

template <int NT>
__global__ void __launch_bounds__(SP_THREADS, 1)
    k_spmm_vnm(SpmmArgs p) {
  extern __shared__ unsigned char sp_raw[];
  SpmmSmem<NT>& sm = *reinterpret_cast<SpmmSmem<NT>*>(
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(sp_raw) + 1023) & ~uintptr_t(1023)));
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int2 tl = p.tlist[blockIdx.x];
  const int t = tl.x;
  const bool add = tl.y != 0;  // the residual kernel wrote these rows first
  const int n0 = blockIdx.y * NT;
  const int s0 = p.tile_step[t], nsteps = p.tile_step[t + 1] - s0;

  if (tid == 0) {
    for (int s = 0; s < SP_STAGES; ++s) {
      ptx::mbar_init(&sm.full[s], 1 + 32);  // the A copy's expect-tx arrival + one per producer lane
      ptx::mbar_init(&sm.empty[s], 1);
      sm.last_k[s] = -1;
    }
    ptx::mbar_init(&sm.done, 1);
    sm.abort = 0;
    ptx::fence_mbar_init();
  }
  if (warp == 0) {
    ptx::tmem_alloc(&sm.tmem_base, NT);
    ptx::tmem_relinquish();
  }
  ptx::tc_fence_before();
  __syncthreads();
  ptx::tc_fence_after();
  const uint32_t tmem = sm.tmem_base;

  if (nsteps > 0) {
    if (warp != 1) {
      // producer warps.  Producer pw copies K-steps pw, pw + P, pw + 2P, ...
      // (P = SP_PRODUCERS), two at a time.  Lane l holds column id (l & 15)
      // of the (l >> 4)-th K-step of each of the SP_PF pairs ahead
      // (coalesced 64-byte loads issued well before use); lane 0 issues the
      // A tile by bulk copy, and every lane copies its 16-byte pieces of the
      // 16 B rows.
      const int pw = warp == 0 ? 0 : warp - 1;
      constexpr int P = SP_PRODUCERS;
      const uint64_t pol_a = ptx::policy_evict_first(), pol_b = ptx::policy_evict_last();
      int pf[SP_PF];
#pragma unroll
      for (int q = 0; q < SP_PF; ++q) {
        const int st = pw + P * (2 * q + (lane >> 4));
        pf[q] = st < nsteps ? p.cols[(size_t)(s0 + st) * 16 + (lane & 15)] : 0;
      }
      bool stop = false;
      for (int j = 0; pw + P * j < nsteps && !stop; j += 2) {
        const int cur = pf[0];
#pragma unroll
        for (int q = 0; q + 1 < SP_PF; ++q) pf[q] = pf[q + 1];
        {
          const int st = pw + P * (j + 2 * SP_PF + (lane >> 4));
          pf[SP_PF - 1] = st < nsteps ? p.cols[(size_t)(s0 + st) * 16 + (lane & 15)] : 0;
        }
        for (int d = 0; d < 2; ++d) {
          const int ii = pw + P * (j + d), s = ii % SP_STAGES;
          if (ii >= nsteps) break;
          int ok = 1;
          if (lane == 0) {
            if (*reinterpret_cast<volatile int*>(&sm.abort)) ok = 0;
            else if (ii >= SP_STAGES)
              ok = ptx::mbar_wait(&sm.empty[s], ((ii / SP_STAGES) - 1) & 1, p.wait_limit) ? 1 : 0;
          }
          ok = __shfl_sync(0xffffffffu, ok, 0);
          if (!ok) {
            if (lane == 0) {
              atomicOr(p.err, 1);
              sm.abort = 1;
            }
            stop = true;
            break;
          }
          if (lane == 0) {
            sm.last_k[s] = ii;
            // A tiles are read once: evict-first, so that they do not push
            // the B rows (read by every tile) out of L2
            ptx::mbar_arrive_expect_tx(&sm.full[s], SP_KSTEP_BYTES);
            ptx::bulk_g2s_hint(sm.a[s], p.a + (size_t)(s0 + ii) * SP_KSTEP_BYTES, SP_KSTEP_BYTES, &sm.full[s],
                               pol_a);
          }
          // the 16 B rows: each lane copies 16-byte chunks into the
          // 128-byte-swizzled layout of the MMA's B operand (atoms of 8 k-rows
          // x 128 bytes, n-atoms 2048 bytes apart, k-atoms 1024 bytes apart,
          // chunk j of k-row r stored at chunk j ^ (r % 8))
          {
            constexpr int CPR = NT / 8;       // 16-byte chunks per row
            constexpr int RPI = 32 / CPR;     // rows per warp instruction
            const int c = lane % CPR, sub = lane / CPR;
            unsigned char* bs = sm.b[s];
#pragma unroll
            for (int kr0 = 0; kr0 < 16; kr0 += RPI) {
              const int kr = kr0 + sub;
              const int row = __shfl_sync(0xffffffffu, cur, d * 16 + kr);
              // a padding column (-1): its A column is zero; fill zeros, read nothing
              const unsigned char* src = p.B + (size_t)(row < 0 ? 0 : row) * p.ldb + (size_t)(n0 + 8 * c) * 2;
              unsigned char* dst = bs + (c >> 3) * 2048 + (kr >> 3) * 1024 + (kr & 7) * 128 + (((c & 7) ^ (kr & 7)) << 4);
              ptx::cp_async16_zfill_hint(dst, src, row < 0 ? 0u : 16u, pol_b);
            }
            ptx::cp_async_mbar_arrive(&sm.full[s]);
          }
          __syncwarp();
        }
      }
    } else if (tid == 32) {
      // MMA issuer
      for (int i = 0; i < nsteps; ++i) {
        const int s = i % SP_STAGES;
        if (!ptx::mbar_wait(&sm.full[s], (i / SP_STAGES) & 1, p.wait_limit)) {
          atomicOr(p.err, 2);
          sm.abort = 1;
          break;
        }
        // the B rows were written by the load/store path: order them before
        // the tensor core reads shared memory
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        ptx::tc_fence_after();
        const uint64_t adesc = ptx::smem_desc(ptx::smem_addr(sm.a[s]), 128, 256, 0);
        const uint64_t bdesc = ptx::smem_desc(ptx::smem_addr(sm.b[s]), 2048, 1024, 2);
        ptx::mma_f16(tmem, adesc, bdesc, p.idesc, i > 0 ? 1u : 0u);
        ptx::mma_commit(&sm.empty[s]);
      }
      ptx::mma_commit(&sm.done);
    }
    __syncwarp();
    // everybody waits for the last MMA
    bool ok = ptx::mbar_wait(&sm.done, 0, SP_WAIT_LIMIT);
    if (!ok && tid == 0) atomicOr(p.err, 4);
    __syncthreads();
    if (tid == 0 && (sm.abort || !ok)) {
      // a wait gave up: let every stage's last issued copies land before exit
      // (the last K-step of a stage is the only one whose phase can be open)
      for (int s = 0; s < SP_STAGES; ++s)
        if (sm.last_k[s] >= 0) ptx::mbar_wait(&sm.full[s], (sm.last_k[s] / SP_STAGES) & 1, SP_WAIT_LIMIT);
    }
    __syncthreads();
    ptx::tc_fence_after();
    if (ok && !sm.abort) {
      // warp w reads TMEM lanes 32 (w % 4) ..; the SP_THREADS / 128 warps of
      // a lane quarter split the columns
      constexpr int EG = SP_THREADS / 128, CW = NT / EG;
      const int row = t * SP_TM + (warp & 3) * 32 + lane;
      const float sc = row < p.R ? p.rscale[row] : 0.f;
#pragma unroll 1
      for (int c0 = (warp >> 2) * CW; c0 < (warp >> 2) * CW + CW; c0 += 32) {
        uint32_t v[32];
        ptx::tmem_ld_32x32b_x32(tmem + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)c0, v);
        ptx::tmem_ld_wait();
        if (row < p.R) {
          float4* dst = reinterpret_cast<float4*>(p.C + (size_t)row * p.ldc + n0 + c0);
#pragma unroll
          for (int q = 0; q < 8; ++q) {
            float4 o = make_float4(__uint_as_float(v[4 * q]) * sc, __uint_as_float(v[4 * q + 1]) * sc,
                                   __uint_as_float(v[4 * q + 2]) * sc, __uint_as_float(v[4 * q + 3]) * sc);
            if (add) {
              const float4 r = dst[q];
              o.x += r.x;
              o.y += r.y;
              o.z += r.z;
              o.w += r.w;
            }
            dst[q] = o;
          }
        }
      }
    }
  }
  ptx::tc_fence_before();
  __syncthreads();
  if (warp == 0) ptx::tmem_dealloc(tmem, NT);
}

// ---------------------------------------------------------------------------
// Host
// ---------------------------------------------------------------------------
static int spmm_dense_min(int V) {
  if (const char* e = getenv("VNM_SPMM_DENSE_MIN")) {
    const int v = atoi(e);
    if (v >= 0) return v;
  }
  return V;
}

// Poll limit of the tensor kernel's pipeline waits.  A test hook,
// VNM_SPMM_TEST_WAIT_LIMIT, sets a small one so that a wait runs out and the
// kernel takes its error path (stop issuing, let the copies in flight land,
// report); the wait for the last MMA and the drain keep the full limit.
static uint32_t spmm_wait_limit() {
  if (const char* e = getenv("VNM_SPMM_TEST_WAIT_LIMIT")) {
    const long v = atol(e);
    if (v > 0) return (uint32_t)v;
  }
  return SP_WAIT_LIMIT;
}

// Arena bytes compress_t takes for nnz entries and R rows.
static size_t compress_scratch_bytes(int R, int nnz) {
  const int ntiles = (R + SP_TM - 1) / SP_TM;
  const size_t n = nnz > 0 ? (size_t)nnz : 1;
  size_t b = arena_bytes(n, 8) + 6 * arena_bytes(n, 4);          // keys, flag, gstart, gsl, gofs, resflag, rpos
  b += arena_bytes(n, 8) + arena_bytes(n, 4);                    // residual keys and sources
  b += 2 * radix_sort_scratch_bytes(nnz);
  b += 7 * arena_bytes(ntiles + 1, 4);                           // tile_raw/pad/has/base/rawbase/res, tl_off
  b += 5 * arena_bytes((size_t)R + 1, 4);                        // rowlen, rptr, nmt, nst, nmr
  b += 3 * arena_bytes((size_t)R + 1, 4);                        // their scans
  b += arena_bytes((size_t)R + 2, 4);                            // bmax (R / V + 1 entries at most)
  b += 8 * scan_scratch_bytes((nnz > R ? nnz : R) + 1) + 16384;
  return b;
}

template <class T>
static vnm_status compress_t(vnm_ctx* ctx, int R, int nnz, const int* d_row, const int* d_col, const float* d_val,
                             int M, int V, vnm_spmm_matrix* out) {
  const int nseg = (R + M - 1) / M;
  const int nbrow = (R + V - 1) / V;
  const int ntiles = (R + SP_TM - 1) / SP_TM;
  const int dense_min = spmm_dense_min(V);
  const int bm = key_bits_m(M), bv = __builtin_ctz((unsigned)V), sh = bm + bv;  // V is a power of two (divides 128)
  int* h = ctx->h_pinned;
  const size_t n1 = nnz > 0 ? (size_t)nnz : 1;
  unsigned long long* keys = arena_take<unsigned long long>(ctx, n1);
  int* flag = arena_take<int>(ctx, n1);
  int* gstart = arena_take<int>(ctx, n1);
  int* gsl = arena_take<int>(ctx, n1);
  int* gofs = arena_take<int>(ctx, n1);
  int* resflag = arena_take<int>(ctx, n1);
  int* rpos = arena_take<int>(ctx, n1);
  int* tile_raw = arena_take<int>(ctx, ntiles + 1);
  int* tile_pad = arena_take<int>(ctx, ntiles + 1);
  int* tile_has = arena_take<int>(ctx, ntiles + 1);
  int* tile_res = arena_take<int>(ctx, ntiles + 1);
  int* tile_base = arena_take<int>(ctx, ntiles + 1);
  int* tile_rawbase = arena_take<int>(ctx, ntiles + 1);
  int* tl_off = arena_take<int>(ctx, ntiles + 1);
  int* rowlen = arena_take<int>(ctx, (size_t)R + 1);
  int* rptr = arena_take<int>(ctx, (size_t)R + 1);
  int* nmt = arena_take<int>(ctx, (size_t)R + 1);
  int* nst = arena_take<int>(ctx, (size_t)R + 1);
  int* nmr = arena_take<int>(ctx, (size_t)R + 1);
  int* mt_off = arena_take<int>(ctx, (size_t)R + 1);
  int* st_off = arena_take<int>(ctx, (size_t)R + 1);
  int* mr_off = arena_take<int>(ctx, (size_t)R + 1);
  unsigned* bmax = arena_take<unsigned>(ctx, nbrow + 1);
  int* counters = arena_take<int>(ctx, 16);
  if (!keys || !flag || !gstart || !gsl || !gofs || !resflag || !rpos || !tile_raw || !tile_pad || !tile_has ||
      !tile_res || !tile_base || !tile_rawbase || !tl_off || !rowlen || !rptr || !nmt || !nst || !nmr || !mt_off ||
      !st_off || !mr_off || !bmax || !counters)
    return VNM_ERR_NOMEM;
  cudaStream_t st = ctx->stream;
  VNM_CUDA_TRY(cudaMemsetAsync(tile_raw, 0, sizeof(int) * (ntiles + 1), st));
  VNM_CUDA_TRY(cudaMemsetAsync(tile_pad, 0, sizeof(int) * (ntiles + 1), st));
  VNM_CUDA_TRY(cudaMemsetAsync(tile_has, 0, sizeof(int) * (ntiles + 1), st));
  VNM_CUDA_TRY(cudaMemsetAsync(tile_res, 0, sizeof(int) * (ntiles + 1), st));
  VNM_CUDA_TRY(cudaMemsetAsync(rowlen, 0, sizeof(int) * ((size_t)R + 1), st));
  VNM_CUDA_TRY(cudaMemsetAsync(resflag, 0, sizeof(int) * n1, st));
  VNM_CUDA_TRY(cudaMemsetAsync(bmax, 0, sizeof(unsigned) * (nbrow + 1), st));
  VNM_CUDA_TRY(cudaMemsetAsync(counters, 0, sizeof(int) * 16, st));
  unsigned long long* skeys = keys;
  int* spos = nullptr;
  if (nnz > 0) {
    // the group count stays on the device until the storage is sized: the
    // counting grid covers every entry, and the scan of the slices per group
    // runs over nnz words, zero past the last group
    VNM_CUDA_TRY(cudaMemsetAsync(gsl, 0, sizeof(int) * n1, st));
    VNM_LAUNCH(ctx, k_cmp_keys, sp_grid(ctx, nnz), 256, 0, d_row, d_col, nnz, M, V, nseg, bm, bv, keys);
    const long long maxkey = ((long long)nbrow * nseg) << sh;
    VNM_TRY(radix_sort_u64(ctx, keys, nullptr, nnz, sp_bits(maxkey), &skeys, &spos));
    VNM_LAUNCH(ctx, k_cmp_heads, sp_grid(ctx, nnz), 256, 0, skeys, nnz, sh, flag);
    VNM_TRY(exclusive_scan(ctx, flag, flag, nnz, counters));
    VNM_LAUNCH(ctx, k_cmp_group_start, sp_grid(ctx, nnz), 256, 0, flag, skeys, nnz, sh, gstart);
    VNM_LAUNCH(ctx, k_cmp_scale, sp_grid(ctx, (nnz + SCALE_RUN - 1) / SCALE_RUN), 256, 0, skeys, spos, d_val, nnz,
               sh, nseg, bmax);
    VNM_LAUNCH(ctx, k_cmp_count, sp_grid(ctx, nnz, 128), 128, 0, skeys, spos, gstart, counters, nnz, M, V, nseg, bm,
               dense_min, gsl, tile_raw, counters + 1, resflag, rowlen, tile_res);
    VNM_TRY(exclusive_scan(ctx, gsl, gofs, nnz, counters + 2));
  }
  VNM_LAUNCH(ctx, k_cmp_pad, sp_grid(ctx, ntiles), 256, 0, tile_raw, ntiles, tile_pad, tile_has);
  VNM_TRY(exclusive_scan(ctx, tile_pad, tile_base, ntiles + 1, nullptr));
  VNM_TRY(exclusive_scan(ctx, tile_raw, tile_rawbase, ntiles + 1, nullptr));
  VNM_TRY(exclusive_scan(ctx, tile_has, tl_off, ntiles, counters + 3));
  VNM_TRY(exclusive_scan(ctx, resflag, rpos, nnz, counters + 4));
  VNM_TRY(exclusive_scan(ctx, rowlen, rptr, R + 1, nullptr));
  VNM_LAUNCH(ctx, k_res_task_count, sp_grid(ctx, R), 256, 0, rptr, R, tile_has, tile_res, nmt, nst, nmr);
  VNM_TRY(exclusive_scan(ctx, nmt, mt_off, R, counters + 5));
  VNM_TRY(exclusive_scan(ctx, nst, st_off, R, counters + 6));
  VNM_TRY(exclusive_scan(ctx, nmr, mr_off, R, counters + 7));
  VNM_CUDA_TRY(cudaMemcpyAsync(h, tile_base + ntiles, sizeof(int), cudaMemcpyDeviceToHost, st));
  VNM_CUDA_TRY(cudaMemcpyAsync(h + 1, counters, 8 * sizeof(int), cudaMemcpyDeviceToHost, st));
  VNM_CUDA_TRY(cudaStreamSynchronize(st));
  const int padded = h[0];
  const int ngroups = nnz > 0 ? h[1] : 0;
  out->valid_blocks = h[2];
  out->slices = ngroups > 0 ? h[3] : 0;
  out->ntt = h[4];
  out->nres = h[5];
  const int nmt_total = h[6], nst_total = h[7];
  out->nslots = nmt_total;
  out->ntask = nmt_total + nst_total;
  out->nmulti = h[8];
  out->dense_min = dense_min;
  out->slices_padded = padded;
  out->groups = ngroups;
  out->nsteps = padded / 4;
  out->ntiles = ntiles;
  // the matrix's own storage (kept across calls)
  const size_t b_step = arena_bytes(ntiles + 1, 4), b_tl = arena_bytes((size_t)out->ntt + 1, 8),
               b_cols = arena_bytes((size_t)out->nsteps * 16 + 1, 4),
               b_a = arena_bytes((size_t)out->nsteps * SP_KSTEP_BYTES + 16, 1),
               b_sc = arena_bytes((size_t)ntiles * SP_TM, 4), b_rc = arena_bytes((size_t)out->nres + 1, 8),
               b_tk = arena_bytes((size_t)out->ntask + 1, 16),
               b_mu = arena_bytes((size_t)out->nmulti + 1, 16);
  const size_t need = b_step + b_tl + b_cols + b_a + b_sc + b_rc + b_tk + b_mu;
  void* base = nullptr;
  size_t have = 0;
  if (ctx->spare) {  // a freed operand's storage, when large enough
    std::lock_guard<std::mutex> g(ctx->spare->m);
    if (ctx->spare->ptr && ctx->spare->bytes >= need) {
      base = ctx->spare->ptr;
      have = ctx->spare->bytes;
      ctx->spare->ptr = nullptr;
      ctx->spare->bytes = 0;
    }
  }
  if (!base) {
    VNM_CUDA_TRY(cudaMalloc(&base, need));
    have = need;
  }
  out->base = base;
  out->bytes = have;
  char* pb = static_cast<char*>(base);
  size_t o = 0;
  out->tile_step = reinterpret_cast<int*>(pb + o);
  o += b_step;
  out->tlist = reinterpret_cast<int2*>(pb + o);
  o += b_tl;
  out->cols = reinterpret_cast<int*>(pb + o);
  o += b_cols;
  out->a = reinterpret_cast<unsigned char*>(pb + o);
  o += b_a;
  out->rscale = reinterpret_cast<float*>(pb + o);
  o += b_sc;
  out->rcv = reinterpret_cast<int2*>(pb + o);
  o += b_rc;
  out->task = reinterpret_cast<int4*>(pb + o);
  o += b_tk;
  out->multi = reinterpret_cast<int4*>(pb + o);
  // residual CSR: the residual entries in their original order, stably
  // sorted by row
  if (out->nres > 0) {
    unsigned long long* rkey = arena_take<unsigned long long>(ctx, (size_t)out->nres);
    int* rsrc = arena_take<int>(ctx, (size_t)out->nres);
    if (!rkey || !rsrc) return VNM_ERR_NOMEM;
    VNM_LAUNCH(ctx, k_res_compact, sp_grid(ctx, nnz), 256, 0, resflag, rpos, d_row, nnz, rkey, rsrc);
    unsigned long long* sk = nullptr;
    int* ss = nullptr;
    VNM_TRY(radix_sort_u64(ctx, rkey, rsrc, (int)out->nres, sp_bits(R), &sk, &ss));
    VNM_LAUNCH(ctx, k_res_gather, sp_grid(ctx, out->nres), 256, 0, ss, d_col, d_val, (int)out->nres, out->rcv);
  }
  if (out->ntask > 0)
    VNM_LAUNCH(ctx, k_res_task_fill, sp_grid(ctx, R), 256, 0, rptr, R, tile_has, tile_res, mt_off, st_off, mr_off,
               nmt_total, out->task, out->multi);
  if (out->ntt > 0)
    VNM_LAUNCH(ctx, k_tile_list, sp_grid(ctx, ntiles), 256, 0, tile_has, tile_res, ntiles, tl_off, out->tlist);
  VNM_CUDA_TRY(cudaMemsetAsync(out->cols, 0xff, b_cols, st));  // -1: padding columns
  VNM_CUDA_TRY(cudaMemsetAsync(out->a, 0, b_a, st));
  if (ngroups > 0 && out->nsteps > 0)
    VNM_LAUNCH(ctx, k_cmp_fill<T>, sp_grid(ctx, ngroups, 128), 128, 0, skeys, spos, d_val, gstart, ngroups, nnz, M,
               V, nseg, bm, dense_min, gofs, tile_base, tile_rawbase, bmax, out->cols, out->a);
  VNM_LAUNCH(ctx, k_cmp_rscale, sp_grid(ctx, (long long)ntiles * SP_TM), 256, 0, bmax, ntiles, R, V, out->rscale,
             tile_base, out->tile_step);
  return VNM_OK;
}

template <int NT>
static vnm_status launch_spmm(vnm_ctx* ctx, const vnm_spmm_matrix* A, SpmmArgs& p) {
  // enough shared memory that at most 512 / NT CTAs share an SM: their NT
  // column accumulators then fit the SM's 512 tensor-memory columns, so an
  // allocation never waits for another CTA (228 KB of shared memory per SM)
  constexpr size_t floor_bytes = (228u << 10) / (512 / NT + 1) + 1024;
  size_t smem = sizeof(SpmmSmem<NT>) + 1024;
  if (smem < floor_bytes) smem = floor_bytes;
  dim3 grid(A->ntt, p.n / NT);
  VNM_CUDA_TRY(cudaFuncSetAttribute(k_spmm_vnm<NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  p.idesc = ptx::idesc_f16(A->dtype == 1 ? 1u : 0u, 0u, 1u, SP_TM, NT);
  VNM_LAUNCH(ctx, k_spmm_vnm<NT>, grid, SP_THREADS, smem, p);
  return VNM_OK;
}

}  // namespace vnm

using namespace vnm;

extern "C" {

vnm_status vnm_spmm_compress(vnm_ctx* ctx, int nrows, int nnz, const int* row, const int* col, const float* val,
                             int mem, int M, int V, int dtype, vnm_spmm_matrix** out) {
  if (!ctx || !out || nrows <= 0 || nnz < 0 || M < 2 || M > 8 || V < 1 || (SP_TM % V) != 0) return VNM_ERR_ARG;
  if (dtype != 0 && dtype != 1) return VNM_ERR_ARG;
  if (mem != VNM_MEM_HOST && mem != VNM_MEM_DEVICE) return VNM_ERR_ARG;
  if (nnz > 0 && (!row || !col || !val)) return VNM_ERR_ARG;
  *out = nullptr;
  const size_t need = 3 * arena_bytes(nnz, 4) + compress_scratch_bytes(nrows, nnz);
  VNM_TRY(arena_reserve(ctx, need));
  VNM_TRY(pinned_reserve(ctx, 64));
  VNM_TRY(begin_call(ctx));
  const int *d_row, *d_col;
  const float* d_val;
  VNM_TRY(stage_in(ctx, row, nnz, mem, &d_row));
  VNM_TRY(stage_in(ctx, col, nnz, mem, &d_col));
  VNM_TRY(stage_in(ctx, val, nnz, mem, &d_val));
  vnm_spmm_matrix* A = new vnm_spmm_matrix();
  A->device = ctx->device;
  A->R = nrows;
  A->M = M;
  A->V = V;
  A->dtype = dtype;
  A->nnz = nnz;
  vnm_status st = dtype == 1 ? compress_t<__nv_bfloat16>(ctx, nrows, nnz, d_row, d_col, d_val, M, V, A)
                             : compress_t<__half>(ctx, nrows, nnz, d_row, d_col, d_val, M, V, A);
  if (st == VNM_OK) st = end_call(ctx);
  if (st != VNM_OK) {
    if (A->base) cudaFree(A->base);
    delete A;
    return st;
  }
  if (ctx->spare) {
    std::lock_guard<std::mutex> g(ctx->spare->m);
    ctx->spare->refs++;
    A->spare = ctx->spare;
  }
  *out = A;
  return VNM_OK;
}

vnm_status vnm_spmm_info(const vnm_spmm_matrix* A, long long* info, int n) {
  if (!A || !info) return VNM_ERR_ARG;
  const long long v[13] = {A->nnz, A->groups, A->valid_blocks, A->slices, A->slices_padded, A->nsteps, A->ntiles,
                           (long long)A->nsteps * SP_KSTEP_BYTES, A->nres, A->ntask, A->ntt, A->dense_min,
                           A->nslots};
  for (int i = 0; i < n && i < 13; ++i) info[i] = v[i];
  return VNM_OK;
}

vnm_status vnm_spmm_free(vnm_spmm_matrix* A) {
  if (!A) return VNM_ERR_ARG;
  cudaSetDevice(A->device);
  if (A->part) cudaFree(A->part);
  if (A->err) cudaFree(A->err);
  bool last = false;
  if (A->spare) {
    // keep the storage for the context's next compression (the larger of
    // this block and the one kept, while the context lives)
    std::lock_guard<std::mutex> g(A->spare->m);
    if (A->base && A->spare->ctx_alive && A->bytes > A->spare->bytes) {
      if (A->spare->ptr) cudaFree(A->spare->ptr);
      A->spare->ptr = A->base;
      A->spare->bytes = A->bytes;
      A->base = nullptr;
    }
    last = --A->spare->refs == 0;
  }
  if (A->base) cudaFree(A->base);
  if (last) delete A->spare;
  delete A;
  return VNM_OK;
}

// Enqueue one product on ctx->stream: the residual kernels, then the tensor
// kernel at the column-block width the context measured fastest for this
// operand shape and n (timed here, which synchronises the stream, on the
// first call for a shape).  dB, dC, P and err are device memory.
static vnm_status spmm_enqueue(vnm_ctx* ctx, const vnm_spmm_matrix* A, const void* dB, int n, float* dC, float* P,
                               int* err, bool timed) {
  SpmmArgs p;
  p.tlist = A->tlist;
  p.tile_step = A->tile_step;
  p.cols = A->cols;
  p.a = A->a;
  p.B = static_cast<const unsigned char*>(dB);
  p.ldb = (size_t)n * 2;
  p.rscale = A->rscale;
  p.C = dC;
  p.R = A->R;
  p.n = n;
  p.ldc = n;
  p.err = err;
  p.wait_limit = spmm_wait_limit();
  // the CUDA-core part: lanes per task so that 8 columns a lane tile n
  auto launch_res = [&]() -> vnm_status {
    if (A->ntask > 0) {
      const int lw = (n % 256) == 0 ? 32 : (n % 128) == 0 ? 16 : 8;
      // one wave of resident blocks (the task list is walked with a stride)
      const int per_block = (RES_THREADS / 32) * (32 / lw);
      int bx = (A->ntask + per_block - 1) / per_block;
      if (bx > ctx->num_sms * RES_BLOCKS_PER_SM) bx = ctx->num_sms * RES_BLOCKS_PER_SM;
      dim3 grid((unsigned)bx, (unsigned)(n / (8 * lw)));
#define VNM_RES(LWV, BFV)                                                                                   \
  VNM_LAUNCH(ctx, (k_spmm_res<LWV, BFV>), grid, RES_THREADS, 0, A->task, A->ntask, A->rcv, p.B, p.ldb, dC, \
             n, P, n)
      if (A->dtype == 1) {
        if (lw == 32) VNM_RES(32, true);
        else if (lw == 16) VNM_RES(16, true);
        else VNM_RES(8, true);
      } else {
        if (lw == 32) VNM_RES(32, false);
        else if (lw == 16) VNM_RES(16, false);
        else VNM_RES(8, false);
      }
#undef VNM_RES
    }
    if (A->nmulti > 0) VNM_LAUNCH(ctx, k_spmm_fin, A->nmulti, FIN_THREADS, 0, A->multi, P, n, dC, n, n);
    return VNM_OK;
  };
  const long long key[3] = {A->R, A->nsteps, n};
  int nt = 0;
  if (const char* e = getenv("VNM_SPMM_WIDTH")) {  // a fixed width (64, 128 or 256) that divides n
    const int w = atoi(e);
    if ((w == 64 || w == 128 || w == 256) && n % w == 0) nt = w;
  }
  for (int q = 0; q < 8 && nt == 0; ++q)
    if (ctx->spmm_tune_nt[q] && ctx->spmm_tune_key[q][0] == key[0] && ctx->spmm_tune_key[q][1] == key[1] &&
        ctx->spmm_tune_key[q][2] == key[2])
      nt = ctx->spmm_tune_nt[q];
  auto launch_nt = [&](int w) -> vnm_status {
    if (A->ntt == 0) return VNM_OK;
    if (w == 256) return launch_spmm<256>(ctx, A, p);
    if (w == 128) return launch_spmm<128>(ctx, A, p);
    return launch_spmm<64>(ctx, A, p);
  };
  if (nt == 0 && A->ntt == 0) nt = 64;  // no tensor-core work: nothing to tune
  if (nt == 0) {
    // the tensor kernel adds into rows the residual kernel wrote: time each
    // width on that state (the final launches below write C afresh)
    VNM_TRY(launch_res());
    const int cand[3] = {256, 128, 64};
    float best = 0.f;
    for (int w : cand) {
      if (n % w) continue;
      VNM_CUDA_TRY(cudaEventRecord(ctx->ev_main0, ctx->stream));
      VNM_TRY(launch_nt(w));
      VNM_CUDA_TRY(cudaEventRecord(ctx->ev_main1, ctx->stream));
      VNM_CUDA_TRY(cudaEventSynchronize(ctx->ev_main1));
      float ms = 0.f;
      VNM_CUDA_TRY(cudaEventElapsedTime(&ms, ctx->ev_main0, ctx->ev_main1));
      if (nt == 0 || ms < best) {
        best = ms;
        nt = w;
      }
    }
    const int slot = ctx->spmm_tune_next;
    ctx->spmm_tune_next = (slot + 1) % 8;
    for (int k = 0; k < 3; ++k) ctx->spmm_tune_key[slot][k] = key[k];
    ctx->spmm_tune_nt[slot] = nt;
  }
  if (timed) VNM_CUDA_TRY(cudaEventRecord(ctx->ev_main0, ctx->stream));
  VNM_TRY(launch_res());
  VNM_TRY(launch_nt(nt));
  if (timed) VNM_CUDA_TRY(cudaEventRecord(ctx->ev_main1, ctx->stream));
  return VNM_OK;
}

vnm_status vnm_spmm_run(vnm_ctx* ctx, const vnm_spmm_matrix* A, const void* B, int n, float* C, int mem) {
  if (!ctx || !A || !B || !C || n <= 0 || (n % 64) != 0) return VNM_ERR_ARG;
  if (mem != VNM_MEM_HOST && mem != VNM_MEM_DEVICE) return VNM_ERR_ARG;
  if (A->device != ctx->device) return VNM_ERR_ARG;
  const size_t bbytes = (size_t)A->R * n * 2, cbytes = (size_t)A->R * n * sizeof(float);
  const size_t pbytes = arena_bytes((size_t)A->nslots * n + 1, sizeof(float));
  VNM_TRY(arena_reserve(ctx, (mem == VNM_MEM_HOST ? bbytes + cbytes + 512 : 0) + pbytes + 4096));
  VNM_TRY(pinned_reserve(ctx, 64));
  VNM_TRY(begin_call(ctx));
  const void* dB = B;
  float* dC = C;
  if (mem == VNM_MEM_HOST) {
    void* tb = arena_take<unsigned char>(ctx, bbytes);
    dC = arena_take<float>(ctx, (size_t)A->R * n);
    if (!tb || !dC) return VNM_ERR_NOMEM;
    VNM_CUDA_TRY(cudaMemcpyAsync(tb, B, bbytes, cudaMemcpyHostToDevice, ctx->stream));
    dB = tb;
  }
  if ((reinterpret_cast<uintptr_t>(dB) & 15) != 0 || (reinterpret_cast<uintptr_t>(dC) & 15) != 0)
    return VNM_ERR_ARG;
  float* P = arena_take<float>(ctx, (size_t)A->nslots * n + 1);
  int* err = arena_take<int>(ctx, 1);
  if (!err || !P) return VNM_ERR_NOMEM;
  VNM_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), ctx->stream));
  VNM_TRY(spmm_enqueue(ctx, A, dB, n, dC, P, err, true));
  VNM_CUDA_TRY(cudaMemcpyAsync(ctx->h_pinned, err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  if (mem == VNM_MEM_HOST)
    VNM_CUDA_TRY(cudaMemcpyAsync(C, dC, cbytes, cudaMemcpyDeviceToHost, ctx->stream));
  VNM_TRY(end_call(ctx));
  VNM_CUDA_TRY(cudaEventElapsedTime(&ctx->main_ms, ctx->ev_main0, ctx->ev_main1));
  if (ctx->h_pinned[0] != 0) return VNM_ERR_INTERNAL;
  return VNM_OK;
}

vnm_status vnm_spmm_run_async(vnm_ctx* ctx, vnm_spmm_matrix* A, const void* B, int n, float* C, void* stream) {
  if (!ctx || !A || !B || !C || n <= 0 || (n % 64) != 0) return VNM_ERR_ARG;
  if (A->device != ctx->device) return VNM_ERR_ARG;
  if ((reinterpret_cast<uintptr_t>(B) & 15) != 0 || (reinterpret_cast<uintptr_t>(C) & 15) != 0) return VNM_ERR_ARG;
  VNM_CUDA_TRY(cudaSetDevice(ctx->device));
  const size_t need = (size_t)A->nslots * n + 1;
  if (!A->err) {
    VNM_CUDA_TRY(cudaMalloc(&A->err, sizeof(int)));
    VNM_CUDA_TRY(cudaMemset(A->err, 0, sizeof(int)));
  }
  if (need > A->part_floats) {  // the first call for a larger n: make room (this waits for the device)
    if (A->part) VNM_CUDA_TRY(cudaFree(A->part));
    A->part = nullptr;
    A->part_floats = 0;
    VNM_CUDA_TRY(cudaMalloc(&A->part, need * sizeof(float)));
    A->part_floats = need;
  }
  ctx->launches = 0;
  ctx->last_ms = ctx->main_ms = 0.f;
  cudaStream_t own = ctx->stream;
  ctx->stream = static_cast<cudaStream_t>(stream);
  const vnm_status st = spmm_enqueue(ctx, A, B, n, C, A->part, A->err, false);
  ctx->stream = own;
  return st;
}

vnm_status vnm_spmm_check(vnm_spmm_matrix* A, void* stream, int* failed) {
  if (!A || !failed) return VNM_ERR_ARG;
  *failed = 0;
  if (!A->err) return VNM_OK;
  VNM_CUDA_TRY(cudaSetDevice(A->device));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int h = 0;
  VNM_CUDA_TRY(cudaMemcpyAsync(&h, A->err, sizeof(int), cudaMemcpyDeviceToHost, s));
  VNM_CUDA_TRY(cudaStreamSynchronize(s));
  VNM_CUDA_TRY(cudaMemsetAsync(A->err, 0, sizeof(int), s));
  *failed = h != 0;
  return VNM_OK;
}

}  // extern "C"
