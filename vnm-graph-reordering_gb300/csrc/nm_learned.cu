// Learned-proposal reorder: a parallel, conflict-free swap-matching search
// whose candidate swaps are ranked by a small MLP before exact scoring.
//
// The reference's greedy (reorder/reorder.h:1805-2474) visits at most M+1
// segments per round and scores every one of their M*M swaps exactly; it is
// sequential by construction.  This mode is a different search with the same
// objective (fewer invalid M-groups, i.e. more retained nonzeros) built for a
// GPU: every round, every invalid segment p proposes swaps with the nodes of
// KT sampled target segments, the MLP scores all of them, only the best 8 per
// segment are scored exactly (the integer kernel decides), and a claim-based
// matching accepts at most one improving swap per segment, so the accepted
// swaps touch disjoint segments and their exact gains add up.  An exhaustive
// mode scores every candidate exactly instead (the fallback and the baseline
// the network is measured against).
//
// State in HBM, all indexed by original ids (rows never move; only which node
// sits at which column position does):
//   G[r * nseg + s]  the M-bit group of row r in segment s (bit i = the column
//                    at position s*M+i), R * nseg bytes;
//   cnt[s]           rows whose group in s has more than N bits;
//   hist[s][k]       rows whose group in s has exactly k bits (k = 0..8);
//   colh[u][k]       rows of column u whose group (in u's segment) has k bits.
//
// MLP: 32 features -> 128 -> 128 -> 1 (ReLU), BF16 operands, FP32
// accumulation.  Inference runs on tcgen05: a CTA builds the features of
// 128 candidates into shared memory, two chained MMAs go through tensor
// memory, and the last layer is a dot product in registers.
#include <cuda_bf16.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "sm100_ptx.cuh"

namespace vnm {

constexpr int LF = 32;       // features
constexpr int LH = 128;      // hidden width
constexpr int LTOP = 8;      // proposals per segment that are scored exactly
constexpr int L_THREADS = 128;
constexpr uint32_t L_WAIT = 1u << 22;

struct LMat {  // one matrix's state
  int R, M, N, nseg;
  int obj;    // 0: invalid groups, 1: retained nonzeros
  const int* cptr;
  const int* crow;
  int* orig;  // position -> node
  int* pos;   // node -> position
  unsigned char* G;
  int* cnt;
  int* hist;  // [nseg * 9]
  int* colh;  // [R * 9]
};

// ---------------------------------------------------------------------------
// State build and maintenance
// ---------------------------------------------------------------------------
__global__ void k_l_build_G(const int* prow, const int* pcol, int np, int M, int nseg, unsigned* Gw) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < np; i += gridDim.x * blockDim.x) {
    const long long cell = (long long)prow[i] * nseg + pcol[i] / M;
    atomicOr(&Gw[cell >> 2], (1u << (pcol[i] % M)) << ((cell & 3) * 8));
  }
}

// hist / cnt from the sorted pattern (runs of equal (row, col/M) are groups)
__global__ void k_l_hist(const int* prow, const int* pcol, int np, int M, int N, int* hist, int* cnt) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < np; i += gridDim.x * blockDim.x) {
    const int r = prow[i], s = pcol[i] / M;
    if (i + 1 < np && prow[i + 1] == r && pcol[i + 1] / M == s) continue;
    int len = 1;
    for (int b = 1; b < M && i - b >= 0 && prow[i - b] == r && pcol[i - b] / M == s; ++b) len++;
    atomicAdd(&hist[s * 9 + len], 1);
    if (len > N) atomicAdd(&cnt[s], 1);
  }
}

__global__ void k_l_hist_zero(int* hist, int nseg, int R) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < nseg; s += gridDim.x * blockDim.x) {
    int t = 0;
    for (int k = 1; k <= 8; ++k) t += hist[s * 9 + k];
    hist[s * 9] = R - t;
  }
}

// colh of the columns at the given positions.  A column's rows are cut into
// chunks of L_CHUNK, one warp per chunk, so a hub column spreads over many
// warps: k_l_colh_prep zeroes each column's histogram and counts its
// chunks, an exclusive scan turns the counts into offsets, and
// k_l_colh_rows adds each chunk's histogram.
constexpr int L_CHUNK = 256;

__global__ void k_l_colh_prep(LMat L, const int* positions, const int* npos_p, int npos_fixed, int cap,
                              int* nchunk) {
  const int npos = npos_p ? *npos_p : npos_fixed;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < cap; q += gridDim.x * blockDim.x) {
    int c = 0;
    if (q < npos) {
      const int u = L.orig[positions ? positions[q] : q];
#pragma unroll
      for (int z = 0; z < 9; ++z) L.colh[u * 9 + z] = 0;
      c = (L.cptr[u + 1] - L.cptr[u] + L_CHUNK - 1) / L_CHUNK;
    }
    nchunk[q] = c;
  }
}

// the entry of a sorted offset table that holds `item`: last q with offs[q] <= item
__device__ __forceinline__ int chunk_owner(const int* offs, int n, int item) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (offs[mid] <= item) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

__global__ void k_l_colh_rows(LMat L, const int* positions, const int* npos_p, int npos_fixed, const int* offs,
                              const int* ntot) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  const int npos = npos_p ? *npos_p : npos_fixed, tot = *ntot;
  for (int item = warp; item < tot; item += nw) {
    const int q = chunk_owner(offs, npos, item);
    const int a = positions ? positions[q] : q;
    const int u = L.orig[a], s = a / L.M;
    const int beg = L.cptr[u] + (item - offs[q]) * L_CHUNK;
    const int end = min(beg + L_CHUNK, L.cptr[u + 1]);
    int h[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int e = beg + lane; e < end; e += 32) {
      const int r = L.crow[e];
      const int k = __popc(L.G[(long long)r * L.nseg + s]);
#pragma unroll
      for (int z = 0; z < 9; ++z) h[z] += (k == z);
    }
#pragma unroll
    for (int z = 0; z < 9; ++z) {
      const int v = __reduce_add_sync(0xffffffffu, h[z]);
      if (lane == z && v) atomicAdd(&L.colh[u * 9 + z], v);
    }
  }
}

__global__ void k_l_iota2(int* orig, int* pos, int R) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < R; i += gridDim.x * blockDim.x) orig[i] = pos[i] = i;
}

// ---------------------------------------------------------------------------
// Candidates and features
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned mix32(unsigned x) {
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}

// target segment q of segment p in round `round` (never p itself)
__device__ __forceinline__ int target_of(int p, int q, int round, int nseg, unsigned seed) {
  const unsigned h = mix32((unsigned)p * 0x9e3779b9u ^ mix32((unsigned)q + 0x632be5abu * (unsigned)round) ^ seed);
  int t = (int)(h % (unsigned)(nseg - 1));
  return t >= p ? t + 1 : t;
}

// candidate c of segment p: target slot q, offsets i (in p) and j (in t)
__device__ __forceinline__ void cand_of(int c, int M, int& q, int& i, int& j) {
  q = c / (M * M);
  i = (c / M) % M;
  j = c % M;
}

__device__ void features(const LMat& L, int p, int i, int t, int j, float* f) {
  const int u = L.orig[p * L.M + i], w = L.orig[t * L.M + j];
  const int du = L.cptr[u + 1] - L.cptr[u], dw = L.cptr[w + 1] - L.cptr[w];
  const float iu = 1.0f / (float)max(du, 1), iw = 1.0f / (float)max(dw, 1), iR = 1.0f / (float)L.R;
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    f[k] = (k + 1 <= L.M) ? L.colh[u * 9 + k + 1] * iu : 0.f;
    f[8 + k] = (k + 1 <= L.M) ? L.colh[w * 9 + k + 1] * iw : 0.f;
  }
#pragma unroll
  for (int k = 0; k < 9; ++k) f[16 + k] = L.hist[t * 9 + k] * iR;
  f[25] = log2f(1.0f + du) * (1.0f / 16);
  f[26] = log2f(1.0f + dw) * (1.0f / 16);
  f[27] = L.hist[p * 9 + L.N] * iR;
  f[28] = L.hist[p * 9 + L.N + 1] * iR;
  f[29] = L.colh[u * 9 + L.N + 1] * (1.0f / 16);
  f[30] = L.colh[w * 9 + L.N + 1] * (1.0f / 16);
  f[31] = 1.0f;
}

// Exact gain of exchanging the columns at positions p*M+i and t*M+j, from
// the group table.  A row holding exactly one of the two columns moves one
// bit between its groups in p and t; a row holding both (or neither) keeps
// its groups.  Objective 0 counts invalid groups (popcount > N) removed,
// objective 1 the nonzeros an N:M pruning keeps (sum of min(popcount, N)).
__device__ __forceinline__ int move_gain(int obj, int N, int from, int to) {  // popcounts before the move
  return obj == 0 ? (from == N + 1) - (to == N) : (to < N) - (from <= N);
}

__device__ int exact_gain_warp(const LMat& L, int p, int i, int t, int j) {
  constexpr int U = 4;  // rows per lane in flight: a hub column is a long chain of dependent loads
  const int lane = threadIdx.x & 31;
  const int u = L.orig[p * L.M + i], w = L.orig[t * L.M + j];
  const unsigned bi = 1u << i, bj = 1u << j;
  int g = 0;
  for (int side = 0; side < 2; ++side) {
    const int col = side == 0 ? u : w;
    const int end = L.cptr[col + 1];
    for (int e0 = L.cptr[col] + lane; e0 < end; e0 += 32 * U) {
      int r[U];
#pragma unroll
      for (int k = 0; k < U; ++k) r[k] = e0 + 32 * k < end ? L.crow[e0 + 32 * k] : -1;
      unsigned gp[U], gt[U];
#pragma unroll
      for (int k = 0; k < U; ++k) {
        gp[k] = r[k] >= 0 ? L.G[(long long)r[k] * L.nseg + p] : 0u;
        gt[k] = r[k] >= 0 ? L.G[(long long)r[k] * L.nseg + t] : 0u;
      }
#pragma unroll
      for (int k = 0; k < U; ++k) {
        if (r[k] < 0) continue;
        if (side == 0) {
          if (!(gt[k] & bj)) g += move_gain(L.obj, L.N, __popc(gp[k]), __popc(gt[k]));  // else w is here too
        } else {
          if (!(gp[k] & bi)) g += move_gain(L.obj, L.N, __popc(gt[k]), __popc(gp[k]));
        }
      }
    }
  }
  return __reduce_add_sync(0xffffffffu, g);
}

// ---------------------------------------------------------------------------
// MLP inference on tcgen05 (fused with feature construction and top-8)
// ---------------------------------------------------------------------------
struct MlpW {  // device weights
  const float* W1;  // [LH][LF]
  const float* b1;  // [LH]
  const float* W2;  // [LH][LH]
  const float* b2;
  const float* w3;  // [LH]
  const float* b3;  // [1]
};

// K-major canonical layout of a [rows x K] bf16 operand: core matrices of
// 8 rows x 16 bytes; k-chunks at 128 B, 8-row groups at K*16 B.
__device__ __forceinline__ int kmaj_off(int r, int k, int K) {
  return (r >> 3) * (K * 16) + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2;
}

struct MlpSmem {
  alignas(1024) unsigned char W1[LH * LF * 2];    // 8 KB
  alignas(1024) unsigned char W2[LH * LH * 2];    // 32 KB
  alignas(1024) unsigned char A1[128 * LF * 2];   // 8 KB
  alignas(1024) unsigned char A2[128 * LH * 2];   // 32 KB
  float b1[LH], b2[LH], w3[LH];
  float score[2048];
  alignas(8) uint64_t bar1, bar2;
  uint32_t tmem;
  int err;
};

__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// The MLP on tcgen05.  Candidate mode (kPlain = false): one CTA per active
// segment at a time scores all of its candidates and keeps the best LTOP ids
// in top[a], at most one per target segment (ties to the lower id), so the
// exactly scored proposals are not near-copies of one swap.  Plain mode: rows of X in tiles of 128,
// scores to Y (the inference path on given features, for tests and timing).
// Per tile of 128 candidates: features -> A1 (bf16, K-major), MMA 128x128x32
// into tensor-memory columns 0..127, bias + ReLU -> A2, MMA 128x128x128 into
// columns 128..255, bias + ReLU + dot with w3 in registers.  Thread t owns
// candidate t of the tile, which is TMEM lane t.
template <bool kPlain>
__global__ void __launch_bounds__(L_THREADS, 1)
    k_l_mlp(LMat L, MlpW W, const int* active, const int* nactive_p, int KT, int round, unsigned seed, int* top,
            const float* X, int nX, float* Y, int* err) {
  extern __shared__ unsigned char l_raw[];
  MlpSmem& sm = *reinterpret_cast<MlpSmem*>(
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(l_raw) + 1023) & ~uintptr_t(1023)));
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  // weights -> canonical layouts (B operands: rows = output features, K-major)
  for (int e = tid; e < LH * LF; e += L_THREADS) {
    const int n = e / LF, k = e % LF;
    *reinterpret_cast<__nv_bfloat16*>(sm.W1 + kmaj_off(n, k, LF)) = __float2bfloat16_rn(W.W1[e]);
  }
  for (int e = tid; e < LH * LH; e += L_THREADS) {
    const int n = e / LH, k = e % LH;
    *reinterpret_cast<__nv_bfloat16*>(sm.W2 + kmaj_off(n, k, LH)) = __float2bfloat16_rn(W.W2[e]);
  }
  for (int e = tid; e < LH; e += L_THREADS) {
    sm.b1[e] = W.b1[e];
    sm.b2[e] = W.b2[e];
    sm.w3[e] = W.w3[e];
  }
  if (tid == 0) {
    ptx::mbar_init(&sm.bar1, 1);
    ptx::mbar_init(&sm.bar2, 1);
    sm.err = 0;
    ptx::fence_mbar_init();
  }
  if (warp == 0) {
    ptx::tmem_alloc(&sm.tmem, 256);
    ptx::tmem_relinquish();
  }
  fence_async_smem();
  ptx::tc_fence_before();
  __syncthreads();
  ptx::tc_fence_after();
  const uint32_t tm = sm.tmem;
  const uint32_t idesc = ptx::idesc_f16(1u, 0u, 0u, 128, LH);
  const float b3 = W.b3[0];
  const int ncand = kPlain ? 0 : KT * L.M * L.M;
  const int nwork = kPlain ? (nX + 127) / 128 : *nactive_p;
  const int ntile = kPlain ? 1 : (ncand + 127) / 128;
  uint32_t phase = 0;
  // this thread's features of candidate `tid` of tile (a, tile); the next
  // tile's are computed while the tensor core runs the current one's first
  // layer, so their loads' latency is hidden behind it
  auto feats = [&](int a, int tile, float (&f)[LF]) {
    const int c = kPlain ? a * 128 + tid : tile * 128 + tid;
    const bool live = a < nwork && (kPlain ? c < nX : c < ncand);
    if (!live) {
#pragma unroll
      for (int k = 0; k < LF; ++k) f[k] = 0.f;
    } else if (kPlain) {
#pragma unroll
      for (int k = 0; k < LF; ++k) f[k] = X[(size_t)c * LF + k];
    } else {
      int q, i, j;
      cand_of(c, L.M, q, i, j);
      const int p = active[a];
      features(L, p, i, target_of(p, q, round, L.nseg, seed), j, f);
    }
  };
  float f[LF];
  feats(blockIdx.x, 0, f);
  for (int a = blockIdx.x; a < nwork; a += gridDim.x) {
    for (int tile = 0; tile < ntile; ++tile) {
      const int c = kPlain ? a * 128 + tid : tile * 128 + tid;
      const bool live = kPlain ? c < nX : c < ncand;
#pragma unroll
      for (int k = 0; k < LF; k += 2)
        *reinterpret_cast<__nv_bfloat162*>(sm.A1 + kmaj_off(tid, k, LF)) = __floats2bfloat162_rn(f[k], f[k + 1]);
      fence_async_smem();
      ptx::tc_fence_before();
      __syncthreads();
      ptx::tc_fence_after();
      if (tid == 0) {
        for (int kk = 0; kk < LF / 16; ++kk) {
          const uint64_t ad = ptx::smem_desc(ptx::smem_addr(sm.A1) + kk * 256, 128, LF * 16, 0);
          const uint64_t bd = ptx::smem_desc(ptx::smem_addr(sm.W1) + kk * 256, 128, LF * 16, 0);
          ptx::mma_f16(tm, ad, bd, idesc, kk > 0 ? 1u : 0u);
        }
        ptx::mma_commit(&sm.bar1);
      }
      // the next tile's features (A1 is rewritten only after this tile's
      // second barrier, by which time the first layer has read it)
      if (tile + 1 < ntile) feats(a, tile + 1, f);
      else feats(a + gridDim.x, 0, f);
      if (!ptx::mbar_wait(&sm.bar1, phase, L_WAIT)) sm.err = 1;
      ptx::tc_fence_after();
      // layer 1 epilogue: bias, ReLU, BF16 -> A2
#pragma unroll 1
      for (int c0 = 0; c0 < LH; c0 += 32) {
        uint32_t v[32];
        ptx::tmem_ld_32x32b_x32(tm + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
        ptx::tmem_ld_wait();
#pragma unroll
        for (int z = 0; z < 32; z += 2) {
          const float h0 = fmaxf(__uint_as_float(v[z]) + sm.b1[c0 + z], 0.f);
          const float h1 = fmaxf(__uint_as_float(v[z + 1]) + sm.b1[c0 + z + 1], 0.f);
          *reinterpret_cast<__nv_bfloat162*>(sm.A2 + kmaj_off(tid, c0 + z, LH)) = __floats2bfloat162_rn(h0, h1);
        }
      }
      fence_async_smem();
      ptx::tc_fence_before();
      __syncthreads();
      ptx::tc_fence_after();
      if (tid == 0) {
        for (int kk = 0; kk < LH / 16; ++kk) {
          const uint64_t ad = ptx::smem_desc(ptx::smem_addr(sm.A2) + kk * 256, 128, LH * 16, 0);
          const uint64_t bd = ptx::smem_desc(ptx::smem_addr(sm.W2) + kk * 256, 128, LH * 16, 0);
          ptx::mma_f16(tm + 128, ad, bd, idesc, kk > 0 ? 1u : 0u);
        }
        ptx::mma_commit(&sm.bar2);
      }
      if (!ptx::mbar_wait(&sm.bar2, phase, L_WAIT)) sm.err = 1;
      ptx::tc_fence_after();
      float y = b3;
#pragma unroll 1
      for (int c0 = 0; c0 < LH; c0 += 32) {
        uint32_t v[32];
        ptx::tmem_ld_32x32b_x32(tm + ((uint32_t)(warp * 32) << 16) + 128u + (uint32_t)c0, v);
        ptx::tmem_ld_wait();
#pragma unroll
        for (int z = 0; z < 32; ++z) {
          const float h = fmaxf(__uint_as_float(v[z]) + sm.b2[c0 + z], 0.f);
          y = fmaf(__bfloat162float(__float2bfloat16_rn(h)), sm.w3[c0 + z], y);
        }
      }
      if (kPlain) {
        if (live) Y[c] = y;
      } else if (live) {
        sm.score[c] = y;
      }
      phase ^= 1u;
      ptx::tc_fence_before();
      __syncthreads();
      ptx::tc_fence_after();
    }
    if (!kPlain) {
      // top LTOP of this segment (ties to the lower id); warp 0
      if (warp == 0) {
        for (int k = 0; k < LTOP; ++k) {
          float best = -INFINITY;
          int bid = 0x7fffffff;
          for (int c = lane; c < ncand; c += 32) {
            const float s = sm.score[c];
            if (s > best || (s == best && c < bid)) {
              best = s;
              bid = c;
            }
          }
          for (int o = 16; o > 0; o >>= 1) {
            const float ob = __shfl_xor_sync(0xffffffffu, best, o);
            const int oi = __shfl_xor_sync(0xffffffffu, bid, o);
            if (ob > best || (ob == best && oi < bid)) {
              best = ob;
              bid = oi;
            }
          }
          if (lane == 0) top[a * LTOP + k] = bid < ncand ? bid : -1;
          // one proposal per target segment: drop the rest of the winner's slot
          if (bid < ncand) {
            const int mm = L.M * L.M, q0 = bid / mm;
            for (int z = lane; z < mm; z += 32) sm.score[q0 * mm + z] = -INFINITY;
          }
          __syncwarp();
        }
      }
      __syncthreads();
    }
  }
  if (tid == 0 && sm.err) atomicOr(err, 8);
  ptx::tc_fence_before();
  __syncthreads();
  ptx::tc_fence_after();
  if (warp == 0) ptx::tmem_dealloc(tm, 256);
}

// ---------------------------------------------------------------------------
// Exact scoring, matching, apply
// ---------------------------------------------------------------------------
enum { L_MODE_MLP = 0, L_MODE_EXHAUSTIVE = 1, L_MODE_RANDOM = 2 };

// Exact gains of candidates: the first topk (<= LTOP) proposals of each
// active segment (network or random), or every candidate (exhaustive).  Each active
// segment's best strictly positive candidate goes to best[a] as
// (gain << 40 | (2^40 - 1 - candidate)), so larger is better and ties go to
// the lower candidate id; 0 when none improves.  A sample of the scored
// candidates (1 in dump_every) is written out as (features, gain) pairs.
__global__ void k_l_exact(LMat L, const int* active, const int* nactive_p, int KT, int round, unsigned seed,
                          const int* top, int mode, int topk, unsigned long long* best, float* dump_x, float* dump_y,
                          int dump_every, int* ndump, int dump_cap, unsigned long long* nscored) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  const int nactive = *nactive_p;
  const int ncand = KT * L.M * L.M;
  const int per = mode == L_MODE_EXHAUSTIVE ? ncand : topk;
  unsigned long long scored = 0;
  for (long long w = warp; w < (long long)nactive * per; w += nw) {
    const int a = (int)(w / per), k = (int)(w % per);
    int c;
    if (mode == L_MODE_EXHAUSTIVE) c = k;
    else if (mode == L_MODE_RANDOM) c = (int)(mix32((unsigned)w * 0x9e3779b9u ^ mix32((unsigned)round ^ seed)) % (unsigned)ncand);
    else c = top[a * LTOP + k];
    if (c < 0) continue;
    const int p = active[a];
    int q, i, j;
    cand_of(c, L.M, q, i, j);
    const int t = target_of(p, q, round, L.nseg, seed);
    const int g = exact_gain_warp(L, p, i, t, j);
    ++scored;
    if (lane == 0) {
      if (g > 0)
        atomicMax(&best[a], ((unsigned long long)g << 40) | ((1ull << 40) - 1 - (unsigned long long)c));
      if (dump_x && dump_every > 0 &&
          (mix32((unsigned)w * 2654435761u ^ seed ^ mix32((unsigned)round)) % (unsigned)dump_every) == 0) {
        const int slot = atomicAdd(ndump, 1);
        if (slot < dump_cap) {
          float f[LF];
          features(L, p, i, t, j, f);
          for (int z = 0; z < LF; ++z) dump_x[(size_t)slot * LF + z] = f[z];
          dump_y[slot] = (float)g;
        }
      }
    }
  }
  if (lane == 0 && scored) atomicAdd(nscored, scored);
}

// claim both segments of each segment's best swap; the highest claim wins
__global__ void k_l_claim(LMat L, const int* active, const int* nactive_p, int round, unsigned seed,
                          const unsigned long long* best, unsigned long long* claim) {
  const int nactive = *nactive_p;
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < nactive; a += gridDim.x * blockDim.x) {
    const unsigned long long b = best[a];
    if (!b) continue;
    const int c = (int)((1ull << 40) - 1 - (b & ((1ull << 40) - 1)));
    int q, i, j;
    cand_of(c, L.M, q, i, j);
    const int p = active[a], t = target_of(p, q, round, L.nseg, seed);
    const unsigned long long key = (b & ~((1ull << 40) - 1)) | (unsigned long long)(unsigned)a;
    atomicMax(&claim[p], key);
    atomicMax(&claim[t], key);
  }
}

// winners: swaps that hold the claim on both of their segments, so accepted
// swaps touch disjoint segments and their exact gains add up
__global__ void k_l_accept(LMat L, const int* active, const int* nactive_p, int round, unsigned seed,
                           const unsigned long long* best, const unsigned long long* claim, int4* acc, int* nacc,
                           unsigned long long* gain_sum) {
  const int nactive = *nactive_p;
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < nactive; a += gridDim.x * blockDim.x) {
    const unsigned long long b = best[a];
    if (!b) continue;
    const int c = (int)((1ull << 40) - 1 - (b & ((1ull << 40) - 1)));
    int q, i, j;
    cand_of(c, L.M, q, i, j);
    const int p = active[a], t = target_of(p, q, round, L.nseg, seed);
    const unsigned long long key = (b & ~((1ull << 40) - 1)) | (unsigned long long)(unsigned)a;
    if (claim[p] == key && claim[t] == key) {
      const int s = atomicAdd(nacc, 1);
      acc[s] = make_int4(p, i, t, j);
      atomicAdd(gain_sum, b >> 40);
    }
  }
}

// Apply accepted swaps: flip the two bits of every row that holds exactly one
// of the two columns, keep hist / cnt in step, and exchange the nodes.
// Accepted swaps touch disjoint segments, and a row holding both columns
// moves nothing, so the rows of the two columns are independent: they are
// cut into chunks of L_CHUNK, one warp per chunk.  k_l_apply_prep records
// each swap's two nodes, counts their chunks and exchanges the nodes;
// k_l_apply_rows moves the bits, summing a chunk's hist / cnt changes in
// registers and adding them once per warp.
__global__ void k_l_apply_prep(LMat L, const int4* acc, const int* nacc, int cap, int2* uw, int* nchunk) {
  const int n = *nacc;
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < cap; s += gridDim.x * blockDim.x) {
    int c = 0;
    if (s < n) {
      const int4 sw = acc[s];
      const int a = sw.x * L.M + sw.y, b = sw.z * L.M + sw.w;
      const int u = L.orig[a], w = L.orig[b];
      uw[s] = make_int2(u, w);
      c = (L.cptr[u + 1] - L.cptr[u] + L_CHUNK - 1) / L_CHUNK + (L.cptr[w + 1] - L.cptr[w] + L_CHUNK - 1) / L_CHUNK;
      L.orig[a] = w;
      L.orig[b] = u;
      L.pos[w] = a;
      L.pos[u] = b;
    }
    nchunk[s] = c;
  }
}

__global__ void k_l_apply_rows(LMat L, const int4* acc, const int* nacc, const int2* uw, const int* offs,
                               const int* ntot) {
  const int n = *nacc, tot = *ntot;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  unsigned* Gw = reinterpret_cast<unsigned*>(L.G);
  for (int item = warp; item < tot; item += nw) {
    const int s = chunk_owner(offs, n, item);
    const int4 sw = acc[s];
    const int p = sw.x, i = sw.y, t = sw.z, j = sw.w;
    const int u = uw[s].x, w = uw[s].y;
    const unsigned bi = 1u << i, bj = 1u << j;
    const int cu = (L.cptr[u + 1] - L.cptr[u] + L_CHUNK - 1) / L_CHUNK;
    int k = item - offs[s];
    const int col = k < cu ? u : w;
    if (k >= cu) k -= cu;
    const int beg = L.cptr[col] + k * L_CHUNK, end = min(beg + L_CHUNK, L.cptr[col + 1]);
    int dp[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, dt[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    int dcp = 0, dct = 0;
    for (int e = beg + lane; e < end; e += 32) {
      const int r = L.crow[e];
      const long long cp = (long long)r * L.nseg + p, ct = (long long)r * L.nseg + t;
      const unsigned gp = L.G[cp], gt = L.G[ct];
      const bool inU = gp & bi, inW = gt & bj;
      if (inU == inW) continue;  // both columns or neither: nothing moves
      const unsigned np_ = inW ? (gp | bi) : (gp & ~bi);
      const unsigned nt_ = inU ? (gt | bj) : (gt & ~bj);
      atomicXor(&Gw[cp >> 2], (gp ^ np_) << ((cp & 3) * 8));
      atomicXor(&Gw[ct >> 2], (gt ^ nt_) << ((ct & 3) * 8));
      const int a0 = __popc(gp), a1 = __popc(np_), c0 = __popc(gt), c1 = __popc(nt_);
#pragma unroll
      for (int z = 0; z < 9; ++z) {
        dp[z] += (z == a1) - (z == a0);
        dt[z] += (z == c1) - (z == c0);
      }
      dcp += (a1 > L.N) - (a0 > L.N);
      dct += (c1 > L.N) - (c0 > L.N);
    }
#pragma unroll
    for (int z = 0; z < 9; ++z) {
      const int vp = __reduce_add_sync(0xffffffffu, dp[z]), vt = __reduce_add_sync(0xffffffffu, dt[z]);
      if (lane == z && vp) atomicAdd(&L.hist[p * 9 + z], vp);
      if (lane == z && vt) atomicAdd(&L.hist[t * 9 + z], vt);
    }
    const int vcp = __reduce_add_sync(0xffffffffu, dcp), vct = __reduce_add_sync(0xffffffffu, dct);
    if (lane == 0 && vcp) atomicAdd(&L.cnt[p], vcp);
    if (lane == 0 && vct) atomicAdd(&L.cnt[t], vct);
  }
}

// positions of all columns of the segments touched by accepted swaps
__global__ void k_l_touched_cols(const int4* acc, const int* nacc, int M, int* cols, int* ncols) {
  const int n = *nacc;
  if (blockIdx.x == 0 && threadIdx.x == 0) *ncols = n * 2 * M;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n * 2 * M; e += gridDim.x * blockDim.x) {
    const int s = e / (2 * M), k = e % (2 * M);
    const int4 sw = acc[s];
    cols[e] = (k < M ? sw.x : sw.z) * M + (k % M);
  }
}

__global__ void k_l_flags(const int* cnt, int nseg, int* flags) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < nseg; s += gridDim.x * blockDim.x) flags[s] = cnt[s] > 0;
}

__global__ void k_l_scatter_active(const int* cnt, const int* idx, int nseg, int* active) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < nseg; s += gridDim.x * blockDim.x)
    if (cnt[s] > 0) active[idx[s]] = s;
}

// totals from the segment histograms: [0] invalid groups, [1] retained nonzeros
__global__ void k_l_totals(const int* hist, int nseg, int N, unsigned long long* out) {
  unsigned long long inv = 0, ret = 0;
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < nseg; s += gridDim.x * blockDim.x)
    for (int k = 1; k <= 8; ++k) {
      const unsigned long long h = (unsigned long long)hist[s * 9 + k];
      if (k > N) inv += h;
      ret += h * (unsigned long long)(k < N ? k : N);
    }
  for (int o = 16; o > 0; o >>= 1) {
    inv += __shfl_xor_sync(0xffffffffu, inv, o);
    ret += __shfl_xor_sync(0xffffffffu, ret, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&out[0], inv);
    atomicAdd(&out[1], ret);
  }
}

__global__ void k_l_invert(const int* orig, int R, int* newpos) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < R; i += gridDim.x * blockDim.x) newpos[orig[i]] = i;
}

}  // namespace vnm

// ---------------------------------------------------------------------------
// Training kernels (FP32 accumulation; operands rounded to BF16 exactly where
// the tensor-core inference rounds them: the layer inputs and the weights)
// ---------------------------------------------------------------------------
namespace vnm {

__device__ __forceinline__ float bf(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

// Y[b][o] = act(sum_i bf(X[b][i]) * bf(W[o][i]) + bias[o])
__global__ void k_t_fwd(const float* X, const float* W, const float* bias, int B, int I, int O, int relu, float* Y) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < (long long)B * O;
       e += (long long)gridDim.x * blockDim.x) {
    const int b = (int)(e / O), o = (int)(e % O);
    float s = 0.f;
    for (int i = 0; i < I; ++i) s += bf(X[(size_t)b * I + i]) * bf(W[(size_t)o * I + i]);
    s += bias[o];
    Y[e] = relu ? fmaxf(s, 0.f) : s;
  }
}

// last layer (fp32 dot, as the inference epilogue does) and dL/dy of
// L = mean((y - t)^2) / 2
__global__ void k_t_out(const float* H2, const float* w3, const float* b3, const float* t, int B, float* y,
                        float* dy, float* loss) {
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < B; b += gridDim.x * blockDim.x) {
    float s = b3[0];
    for (int o = 0; o < LH; ++o) s += bf(H2[(size_t)b * LH + o]) * w3[o];
    y[b] = s;
    const float d = s - t[b];
    dy[b] = d / B;
    atomicAdd(loss, 0.5f * d * d / B);
  }
}

// dW[o][i] = sum_b dZ[b][o] * bf(A[b][i]);  db[o] = sum_b dZ[b][o]
__global__ void k_t_wgrad(const float* dZ, const float* A, int B, int I, int O, float* dW, float* db) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < (long long)O * (I + 1);
       e += (long long)gridDim.x * blockDim.x) {
    const int o = (int)(e / (I + 1)), i = (int)(e % (I + 1));
    float s = 0.f;
    if (i < I) {
      for (int b = 0; b < B; ++b) s += dZ[(size_t)b * O + o] * bf(A[(size_t)b * I + i]);
      dW[(size_t)o * I + i] = s;
    } else {
      for (int b = 0; b < B; ++b) s += dZ[(size_t)b * O + o];
      db[o] = s;
    }
  }
}

// dA[b][i] = (sum_o dZ[b][o] * bf(W[o][i])) * [A[b][i] > 0]
__global__ void k_t_dgrad(const float* dZ, const float* W, const float* A, int B, int I, int O, float* dA) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < (long long)B * I;
       e += (long long)gridDim.x * blockDim.x) {
    const int b = (int)(e / I), i = (int)(e % I);
    float s = 0.f;
    for (int o = 0; o < O; ++o) s += dZ[(size_t)b * O + o] * bf(W[(size_t)o * I + i]);
    dA[e] = A[e] > 0.f ? s : 0.f;
  }
}

// gradient of the last layer: dw3[o] = sum_b dy[b] * bf(H2[b][o]), db3;
// dH2[b][o] = dy[b] * w3[o] * [H2 > 0]
__global__ void k_t_out_grad(const float* dy, const float* H2, const float* w3, int B, float* dw3, float* db3,
                             float* dH2) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < (long long)B * LH + LH + 1;
       e += (long long)gridDim.x * blockDim.x) {
    if (e < (long long)B * LH) {
      const int b = (int)(e / LH), o = (int)(e % LH);
      dH2[e] = H2[e] > 0.f ? dy[b] * w3[o] : 0.f;
    } else if (e < (long long)B * LH + LH) {
      const int o = (int)(e - (long long)B * LH);
      float s = 0.f;
      for (int b = 0; b < B; ++b) s += dy[b] * bf(H2[(size_t)b * LH + o]);
      dw3[o] = s;
    } else {
      float s = 0.f;
      for (int b = 0; b < B; ++b) s += dy[b];
      db3[0] = s;
    }
  }
}

__global__ void k_t_adam(float* p, const float* g, float* m, float* v, int n, float lr, float b1, float b2, float eps,
                         float c1, float c2) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float gi = g[i];
    m[i] = b1 * m[i] + (1.f - b1) * gi;
    v[i] = b2 * v[i] + (1.f - b2) * gi * gi;
    p[i] -= lr * (m[i] / c1) / (sqrtf(v[i] / c2) + eps);
  }
}

}  // namespace vnm

// ---------------------------------------------------------------------------
// Host
// ---------------------------------------------------------------------------
// parameter vector layout: W1 [LH][LF], b1 [LH], W2 [LH][LH], b2 [LH], w3 [LH], b3 [1]
constexpr int L_OFF_W1 = 0;
constexpr int L_OFF_B1 = L_OFF_W1 + vnm::LH * vnm::LF;
constexpr int L_OFF_W2 = L_OFF_B1 + vnm::LH;
constexpr int L_OFF_B2 = L_OFF_W2 + vnm::LH * vnm::LH;
constexpr int L_OFF_W3 = L_OFF_B2 + vnm::LH;
constexpr int L_OFF_B3 = L_OFF_W3 + vnm::LH;
constexpr int L_NPARAM = L_OFF_B3 + 1;

struct vnm_mlp {
  int device = 0;
  float* p = nullptr;  // [L_NPARAM] master weights
  float* g = nullptr;  // gradients
  float* m = nullptr;  // Adam moments
  float* v = nullptr;
  int steps = 0;
};

namespace vnm {

static MlpW mlp_view(const vnm_mlp* n) {
  MlpW w;
  w.W1 = n->p + L_OFF_W1;
  w.b1 = n->p + L_OFF_B1;
  w.W2 = n->p + L_OFF_W2;
  w.b2 = n->p + L_OFF_B2;
  w.w3 = n->p + L_OFF_W3;
  w.b3 = n->p + L_OFF_B3;
  return w;
}

static size_t mlp_smem() { return sizeof(MlpSmem) + 1024; }

// forward + backward of one batch (device X [B][LF], t [B]); gradients land in n->g
static vnm_status mlp_grad(vnm_ctx* ctx, vnm_mlp* n, const float* X, const float* t, int B, float* d_loss) {
  float* H1 = arena_take<float>(ctx, (size_t)B * LH);
  float* H2 = arena_take<float>(ctx, (size_t)B * LH);
  float* y = arena_take<float>(ctx, B);
  float* dy = arena_take<float>(ctx, B);
  float* dH2 = arena_take<float>(ctx, (size_t)B * LH);
  float* dH1 = arena_take<float>(ctx, (size_t)B * LH);
  if (!H1 || !H2 || !y || !dy || !dH2 || !dH1) return VNM_ERR_NOMEM;
  const int G = ctx->num_sms * 8;
  float* p = n->p;
  float* g = n->g;
  VNM_LAUNCH(ctx, k_t_fwd, G, 256, 0, X, p + L_OFF_W1, p + L_OFF_B1, B, LF, LH, 1, H1);
  VNM_LAUNCH(ctx, k_t_fwd, G, 256, 0, H1, p + L_OFF_W2, p + L_OFF_B2, B, LH, LH, 1, H2);
  VNM_CUDA_TRY(cudaMemsetAsync(d_loss, 0, sizeof(float), ctx->stream));
  VNM_LAUNCH(ctx, k_t_out, G, 256, 0, H2, p + L_OFF_W3, p + L_OFF_B3, t, B, y, dy, d_loss);
  VNM_LAUNCH(ctx, k_t_out_grad, G, 256, 0, dy, H2, p + L_OFF_W3, B, g + L_OFF_W3, g + L_OFF_B3, dH2);
  VNM_LAUNCH(ctx, k_t_wgrad, G, 256, 0, dH2, H1, B, LH, LH, g + L_OFF_W2, g + L_OFF_B2);
  VNM_LAUNCH(ctx, k_t_dgrad, G, 256, 0, dH2, p + L_OFF_W2, H1, B, LH, LH, dH1);
  VNM_LAUNCH(ctx, k_t_wgrad, G, 256, 0, dH1, X, B, LF, LH, g + L_OFF_W1, g + L_OFF_B1);
  return VNM_OK;
}

}  // namespace vnm

using namespace vnm;

extern "C" {

int vnm_mlp_param_count(void) { return L_NPARAM; }

vnm_status vnm_mlp_create(vnm_ctx* ctx, unsigned seed, vnm_mlp** out) {
  if (!ctx || !out) return VNM_ERR_ARG;
  *out = nullptr;
  VNM_CUDA_TRY(cudaSetDevice(ctx->device));
  std::vector<float> h(L_NPARAM, 0.f);
  unsigned s = seed * 747796405u + 2891336453u;
  auto rnd = [&]() {  // uniform (-1, 1), PCG-style hash
    s = s * 747796405u + 2891336453u;
    unsigned x = ((s >> ((s >> 28) + 4)) ^ s) * 277803737u;
    x = (x >> 22) ^ x;
    return (x >> 8) * (2.0f / 16777216.0f) - 1.0f;
  };
  const float a1 = sqrtf(6.0f / LF), a2 = sqrtf(6.0f / LH), a3 = sqrtf(3.0f / LH);
  for (int i = 0; i < LH * LF; ++i) h[L_OFF_W1 + i] = a1 * rnd();
  for (int i = 0; i < LH * LH; ++i) h[L_OFF_W2 + i] = a2 * rnd();
  for (int i = 0; i < LH; ++i) h[L_OFF_W3 + i] = a3 * rnd();
  vnm_mlp* n = new vnm_mlp();
  n->device = ctx->device;
  void* base = nullptr;
  if (cudaMalloc(&base, sizeof(float) * L_NPARAM * 4) != cudaSuccess) {
    delete n;
    return VNM_ERR_NOMEM;
  }
  n->p = static_cast<float*>(base);
  n->g = n->p + L_NPARAM;
  n->m = n->g + L_NPARAM;
  n->v = n->m + L_NPARAM;
  cudaMemset(base, 0, sizeof(float) * L_NPARAM * 4);
  cudaMemcpy(n->p, h.data(), sizeof(float) * L_NPARAM, cudaMemcpyHostToDevice);
  *out = n;
  return VNM_OK;
}

vnm_status vnm_mlp_free(vnm_mlp* n) {
  if (!n) return VNM_ERR_ARG;
  cudaSetDevice(n->device);
  cudaFree(n->p);
  delete n;
  return VNM_OK;
}

vnm_status vnm_mlp_get(const vnm_mlp* n, float* params) {
  if (!n || !params) return VNM_ERR_ARG;
  VNM_CUDA_TRY(cudaMemcpy(params, n->p, sizeof(float) * L_NPARAM, cudaMemcpyDeviceToHost));
  return VNM_OK;
}

vnm_status vnm_mlp_set(vnm_mlp* n, const float* params) {
  if (!n || !params) return VNM_ERR_ARG;
  VNM_CUDA_TRY(cudaMemcpy(n->p, params, sizeof(float) * L_NPARAM, cudaMemcpyHostToDevice));
  n->steps = 0;
  VNM_CUDA_TRY(cudaMemset(n->m, 0, sizeof(float) * L_NPARAM * 2));
  return VNM_OK;
}

vnm_status vnm_mlp_grad(vnm_ctx* ctx, vnm_mlp* n, const float* X, const float* t, int B, float* grads,
                        float* loss) {
  if (!ctx || !n || !X || !t || B <= 0 || !grads || !loss) return VNM_ERR_ARG;
  VNM_TRY(arena_reserve(ctx, arena_bytes((size_t)B * LF, 4) + arena_bytes(B, 4) * 3 +
                                 4 * arena_bytes((size_t)B * LH, 4) + 4096));
  VNM_TRY(pinned_reserve(ctx, 64));
  VNM_TRY(begin_call(ctx));
  const float *dX, *dt;
  VNM_TRY(stage_in(ctx, X, (size_t)B * LF, VNM_MEM_HOST, &dX));
  VNM_TRY(stage_in(ctx, t, (size_t)B, VNM_MEM_HOST, &dt));
  float* dl = arena_take<float>(ctx, 1);
  if (!dl) return VNM_ERR_NOMEM;
  VNM_TRY(mlp_grad(ctx, n, dX, dt, B, dl));
  VNM_CUDA_TRY(cudaMemcpyAsync(grads, n->g, sizeof(float) * L_NPARAM, cudaMemcpyDeviceToHost, ctx->stream));
  VNM_CUDA_TRY(cudaMemcpyAsync(loss, dl, sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
  return end_call(ctx);
}

// Adam steps over a dataset (host X [n][LF], t [n]): `epochs` passes in
// mini-batches of B (the data order is fixed; shuffle on the host).
vnm_status vnm_mlp_train(vnm_ctx* ctx, vnm_mlp* net, const float* X, const float* t, int n, int B, int epochs,
                         float lr, float* final_loss) {
  if (!ctx || !net || !X || !t || n <= 0 || B <= 0 || epochs <= 0) return VNM_ERR_ARG;
  const int nb = n / B;
  if (nb == 0) return VNM_ERR_ARG;
  VNM_TRY(arena_reserve(ctx, arena_bytes((size_t)n * LF, 4) + arena_bytes(n, 4) + arena_bytes(B, 4) * 3 +
                                 4 * arena_bytes((size_t)B * LH, 4) + arena_bytes(nb + 1, 4) + 8192));
  VNM_TRY(pinned_reserve(ctx, 64 + nb));
  VNM_TRY(begin_call(ctx));
  const float *dX, *dt;
  VNM_TRY(stage_in(ctx, X, (size_t)n * LF, VNM_MEM_HOST, &dX));
  VNM_TRY(stage_in(ctx, t, (size_t)n, VNM_MEM_HOST, &dt));
  float* losses = arena_take<float>(ctx, nb + 1);
  if (!losses) return VNM_ERR_NOMEM;
  const size_t mark = ctx->arena.used;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  for (int e = 0; e < epochs; ++e) {
    for (int k = 0; k < nb; ++k) {
      ctx->arena.used = mark;
      VNM_TRY(mlp_grad(ctx, net, dX + (size_t)k * B * LF, dt + (size_t)k * B, B, losses + k));
      net->steps++;
      const float c1 = 1.f - powf(b1, (float)net->steps), c2 = 1.f - powf(b2, (float)net->steps);
      VNM_LAUNCH(ctx, k_t_adam, 64, 256, 0, net->p, net->g, net->m, net->v, L_NPARAM, lr, b1, b2, eps, c1, c2);
    }
  }
  VNM_CUDA_TRY(cudaMemcpyAsync(ctx->h_pinned, losses, sizeof(float) * nb, cudaMemcpyDeviceToHost, ctx->stream));
  VNM_TRY(end_call(ctx));
  if (final_loss) {
    double s = 0;
    const float* l = reinterpret_cast<const float*>(ctx->h_pinned);
    for (int k = 0; k < nb; ++k) s += l[k];
    *final_loss = (float)(s / nb);
  }
  return VNM_OK;
}

}  // extern "C"

namespace vnm {

static int lgrid(const vnm_ctx* ctx, long long n, int nt = 256) {
  long long g = (n + nt - 1) / nt;
  const long long cap = (long long)ctx->num_sms * 8;
  if (g > cap) g = cap;
  return g < 1 ? 1 : (int)g;
}

static vnm_status mlp_launch_prep(size_t smem) {
  static bool done[2] = {false, false};
  if (!done[0]) {
    VNM_CUDA_TRY(cudaFuncSetAttribute(k_l_mlp<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    done[0] = true;
  }
  if (!done[1]) {
    VNM_CUDA_TRY(cudaFuncSetAttribute(k_l_mlp<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    done[1] = true;
  }
  return VNM_OK;
}

}  // namespace vnm

extern "C" {

vnm_status vnm_mlp_forward(vnm_ctx* ctx, const vnm_mlp* net, const float* X, int n, float* Y) {
  if (!ctx || !net || n < 0 || (n > 0 && (!X || !Y))) return VNM_ERR_ARG;
  if (n == 0) return VNM_OK;
  VNM_TRY(arena_reserve(ctx, arena_bytes((size_t)n * LF, 4) + arena_bytes(n, 4) + arena_bytes(1, 4) + 1024));
  VNM_TRY(pinned_reserve(ctx, 64));
  VNM_TRY(begin_call(ctx));
  const float* dX;
  VNM_TRY(stage_in(ctx, X, (size_t)n * LF, VNM_MEM_HOST, &dX));
  float* dY = arena_take<float>(ctx, n);
  int* err = arena_take<int>(ctx, 1);
  if (!dY || !err) return VNM_ERR_NOMEM;
  VNM_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), ctx->stream));
  const size_t smem = mlp_smem();
  VNM_TRY(mlp_launch_prep(smem));
  LMat L{};
  const int tiles = (n + 127) / 128;
  const int grid = tiles < 2 * ctx->num_sms ? tiles : 2 * ctx->num_sms;
  VNM_CUDA_TRY(cudaEventRecord(ctx->ev_main0, ctx->stream));
  VNM_LAUNCH(ctx, k_l_mlp<true>, grid, L_THREADS, smem, L, mlp_view(net), nullptr, nullptr, 0, 0, 0u, nullptr, dX,
             n, dY, err);
  VNM_CUDA_TRY(cudaEventRecord(ctx->ev_main1, ctx->stream));
  VNM_CUDA_TRY(cudaMemcpyAsync(Y, dY, sizeof(float) * n, cudaMemcpyDeviceToHost, ctx->stream));
  VNM_CUDA_TRY(cudaMemcpyAsync(ctx->h_pinned, err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  VNM_TRY(end_call(ctx));
  VNM_CUDA_TRY(cudaEventElapsedTime(&ctx->main_ms, ctx->ev_main0, ctx->ev_main1));
  return ctx->h_pinned[0] ? VNM_ERR_INTERNAL : VNM_OK;
}

vnm_status vnm_nm_learned(vnm_ctx* ctx, int nrows, int nnz, const int* row, const int* col, const float* val,
                          int mem, int N, int M, const vnm_mlp* net, const vnm_learned_params* prm,
                          vnm_learned_result* out, int* newpos) {
  if (!ctx || !prm || !out) return VNM_ERR_ARG;
  if (M < 2 || M > 8 || N < 1 || N >= M) return VNM_ERR_ARG;
  if (nrows < 0 || nnz < 0 || (nrows % M) != 0) return VNM_ERR_ARG;
  if (mem != VNM_MEM_HOST && mem != VNM_MEM_DEVICE) return VNM_ERR_ARG;
  if (nnz > 0 && (!row || !col || !val)) return VNM_ERR_ARG;
  if (nrows >= (1 << 27)) return VNM_ERR_LIMIT;  // 16 nrows + 1 row groups fit an int
  const int mode = prm->mode, KT = prm->targets;
  if (mode < VNM_LEARNED_MLP || mode > VNM_LEARNED_RANDOM) return VNM_ERR_ARG;
  if (mode == VNM_LEARNED_MLP && !net) return VNM_ERR_ARG;
  if (net && net->device != ctx->device) return VNM_ERR_ARG;
  if (prm->objective < 0 || prm->objective > 1 || prm->max_rounds < 0 || prm->patience < 1) return VNM_ERR_ARG;
  if (KT < 1 || KT * M * M > 2048) return VNM_ERR_ARG;
  if (mode != VNM_LEARNED_EXHAUSTIVE && (prm->topk < 1 || prm->topk > LTOP)) return VNM_ERR_ARG;
  if (prm->dump_cap < 0 || (prm->dump_cap > 0 && (!prm->dump_features || !prm->dump_gains))) return VNM_ERR_ARG;
  memset(out, 0, sizeof(*out));
  const int R = nrows, nseg = R / M;
  const long long gbytes = ((long long)R * nseg + 3) & ~3ll;
  const int dcap = prm->dump_every > 0 ? prm->dump_cap : 0;
  size_t need = pattern_bytes(R, nnz) + 3 * arena_bytes(nnz, 4) + arena_bytes(gbytes, 1) +
                arena_bytes((size_t)nseg * 9, 4) + arena_bytes(nseg, 4) + arena_bytes((size_t)R * 9, 4) +
                3 * arena_bytes(R, 4) + 3 * arena_bytes(nseg + 1, 4) + arena_bytes((size_t)nseg * LTOP, 4) +
                2 * arena_bytes(nseg, 8) + arena_bytes(nseg, 16) + arena_bytes(2 * (size_t)R, 4) +
                arena_bytes(16, 4) + arena_bytes(8, 8) + arena_bytes(R + 1, 4) + arena_bytes(nseg + 1, 8) +
                // scratch of the scans, given back every round: the active list, the applied
                // swaps and the column histograms (the first histograms' scan before the loop)
                scan_scratch_bytes(R + 1) + 2 * scan_scratch_bytes(nseg + 1) +
                arena_bytes((size_t)dcap * LF, 4) + arena_bytes(dcap, 4) + 8192;
  VNM_TRY(arena_reserve(ctx, need));
  VNM_TRY(pinned_reserve(ctx, 256));
  VNM_TRY(begin_call(ctx));
  const int *d_row, *d_col;
  const float* d_val;
  VNM_TRY(stage_in(ctx, row, nnz, mem, &d_row));
  VNM_TRY(stage_in(ctx, col, nnz, mem, &d_col));
  VNM_TRY(stage_in(ctx, val, nnz, mem, &d_val));
  Pattern P;
  VNM_TRY(build_pattern(ctx, R, nnz, d_row, d_col, d_val, N, M, P, ctx->h_pinned));
  LMat L;
  L.R = R;
  L.M = M;
  L.N = N;
  L.nseg = nseg;
  L.obj = prm->objective;
  L.cptr = P.cptr;
  L.crow = P.crow;
  L.G = arena_take<unsigned char>(ctx, gbytes > 0 ? gbytes : 4);
  L.hist = arena_take<int>(ctx, (size_t)nseg * 9 + 1);
  L.cnt = arena_take<int>(ctx, nseg + 1);
  L.colh = arena_take<int>(ctx, (size_t)R * 9 + 1);
  L.orig = arena_take<int>(ctx, R + 1);
  L.pos = arena_take<int>(ctx, R + 1);
  int* flags = arena_take<int>(ctx, nseg + 1);
  int* active = arena_take<int>(ctx, nseg + 1);
  int* top = arena_take<int>(ctx, (size_t)nseg * LTOP + 1);
  unsigned long long* best = arena_take<unsigned long long>(ctx, nseg + 1);
  unsigned long long* claim = arena_take<unsigned long long>(ctx, nseg + 1);
  int4* acc = arena_take<int4>(ctx, nseg + 1);
  int* cols = arena_take<int>(ctx, 2 * (size_t)R + 1);
  int* chunks = arena_take<int>(ctx, R + 1);     // per column (or swap) chunk counts, then their offsets
  int2* uw = arena_take<int2>(ctx, nseg + 1);    // the two nodes of each accepted swap
  int* ci = arena_take<int>(ctx, 16);  // [0] nactive [1] nacc [2] ncols [3] ndump [4] err [5..6] chunk totals
  unsigned long long* cu = arena_take<unsigned long long>(ctx, 8);  // [0] gain [1] scored [2..3] totals
  float* dx = dcap ? arena_take<float>(ctx, (size_t)dcap * LF) : nullptr;
  float* dy = dcap ? arena_take<float>(ctx, dcap) : nullptr;
  int* d_newpos = arena_take<int>(ctx, R + 1);
  if (!L.G || !L.hist || !L.cnt || !L.colh || !L.orig || !L.pos || !flags || !active || !top || !best || !claim ||
      !acc || !cols || !chunks || !uw || !ci || !cu || !d_newpos || (dcap && (!dx || !dy)))
    return VNM_ERR_NOMEM;
  cudaStream_t st = ctx->stream;
  VNM_CUDA_TRY(cudaMemsetAsync(L.G, 0, gbytes > 0 ? gbytes : 4, st));
  VNM_CUDA_TRY(cudaMemsetAsync(L.hist, 0, sizeof(int) * ((size_t)nseg * 9 + 1), st));
  VNM_CUDA_TRY(cudaMemsetAsync(L.cnt, 0, sizeof(int) * (nseg + 1), st));
  VNM_CUDA_TRY(cudaMemsetAsync(ci, 0, sizeof(int) * 16, st));
  VNM_CUDA_TRY(cudaMemsetAsync(cu, 0, sizeof(unsigned long long) * 8, st));
  if (R > 0) VNM_LAUNCH(ctx, k_l_iota2, lgrid(ctx, R), 256, 0, L.orig, L.pos, R);
  if (P.np > 0) {
    VNM_LAUNCH(ctx, k_l_build_G, lgrid(ctx, P.np), 256, 0, P.prow, P.pcol, P.np, M, nseg,
               reinterpret_cast<unsigned*>(L.G));
    VNM_LAUNCH(ctx, k_l_hist, lgrid(ctx, P.np), 256, 0, P.prow, P.pcol, P.np, M, N, L.hist, L.cnt);
  }
  if (nseg > 0) {
    VNM_LAUNCH(ctx, k_l_hist_zero, lgrid(ctx, nseg), 256, 0, L.hist, nseg, R);
    VNM_LAUNCH(ctx, k_l_totals, lgrid(ctx, nseg), 256, 0, L.hist, nseg, N, cu + 2);
  }
  const size_t round_mark = ctx->arena.used;  // scan scratch from here on is given back every round
  if (R > 0) {  // every column's histogram
    VNM_LAUNCH(ctx, k_l_colh_prep, lgrid(ctx, R), 256, 0, L, nullptr, nullptr, R, R, chunks);
    VNM_TRY(exclusive_scan(ctx, chunks, chunks, R, ci + 5));
    VNM_LAUNCH(ctx, k_l_colh_rows, lgrid(ctx, (long long)R * 32), 256, 0, L, nullptr, nullptr, R, chunks, ci + 5);
  }
  unsigned long long* hcu = reinterpret_cast<unsigned long long*>(ctx->h_pinned);  // 8 words
  int* hci = ctx->h_pinned + 32;                                                    // 16 ints
  VNM_CUDA_TRY(cudaMemcpyAsync(hcu, cu, sizeof(unsigned long long) * 4, cudaMemcpyDeviceToHost, st));
  VNM_CUDA_TRY(cudaStreamSynchronize(st));
  out->init_invalid = out->final_invalid = (long long)hcu[2];
  out->init_retained = out->final_retained = (long long)hcu[3];
  const size_t smem = mlp_smem();
  if (mode == VNM_LEARNED_MLP) VNM_TRY(mlp_launch_prep(smem));
  const MlpW W = net ? mlp_view(net) : MlpW{};
  const int pgrid = 2 * ctx->num_sms;
  const int egrid = ctx->num_sms * 8;
  int idle = 0, rounds = 0, swaps = 0;
  VNM_CUDA_TRY(cudaEventRecord(ctx->ev_main0, st));
  for (int round = 0; round < prm->max_rounds && nseg >= 2 && P.np > 0; ++round) {
    ctx->arena.used = round_mark;
    VNM_CUDA_TRY(cudaMemsetAsync(ci + 1, 0, sizeof(int) * 2, st));
    VNM_CUDA_TRY(cudaMemsetAsync(best, 0, sizeof(unsigned long long) * nseg, st));
    VNM_CUDA_TRY(cudaMemsetAsync(claim, 0, sizeof(unsigned long long) * nseg, st));
    VNM_LAUNCH(ctx, k_l_flags, lgrid(ctx, nseg), 256, 0, L.cnt, nseg, flags);
    VNM_TRY(exclusive_scan(ctx, flags, flags, nseg, ci));
    VNM_LAUNCH(ctx, k_l_scatter_active, lgrid(ctx, nseg), 256, 0, L.cnt, flags, nseg, active);
    if (mode == VNM_LEARNED_MLP)
      VNM_LAUNCH(ctx, k_l_mlp<false>, pgrid, L_THREADS, smem, L, W, active, ci, KT, round, prm->seed, top, nullptr,
                 0, nullptr, ci + 4);
    VNM_LAUNCH(ctx, k_l_exact, egrid, 256, 0, L, active, ci, KT, round, prm->seed, top, mode, prm->topk, best, dx, dy,
               prm->dump_every, ci + 3, dcap, cu + 1);
    VNM_LAUNCH(ctx, k_l_claim, lgrid(ctx, nseg), 256, 0, L, active, ci, round, prm->seed, best, claim);
    VNM_LAUNCH(ctx, k_l_accept, lgrid(ctx, nseg), 256, 0, L, active, ci, round, prm->seed, best, claim, acc, ci + 1,
               cu);
    VNM_LAUNCH(ctx, k_l_apply_prep, lgrid(ctx, nseg), 256, 0, L, acc, ci + 1, nseg, uw, chunks);
    VNM_TRY(exclusive_scan(ctx, chunks, chunks, nseg, ci + 6));
    VNM_LAUNCH(ctx, k_l_apply_rows, egrid, 256, 0, L, acc, ci + 1, uw, chunks, ci + 6);
    VNM_LAUNCH(ctx, k_l_touched_cols, lgrid(ctx, 2 * (long long)R), 256, 0, acc, ci + 1, M, cols, ci + 2);
    VNM_LAUNCH(ctx, k_l_colh_prep, lgrid(ctx, R), 256, 0, L, cols, ci + 2, 0, R, chunks);
    VNM_TRY(exclusive_scan(ctx, chunks, chunks, R, ci + 5));
    VNM_LAUNCH(ctx, k_l_colh_rows, egrid, 256, 0, L, cols, ci + 2, 0, chunks, ci + 5);
    VNM_CUDA_TRY(cudaMemcpyAsync(hci, ci, sizeof(int) * 8, cudaMemcpyDeviceToHost, st));
    VNM_CUDA_TRY(cudaMemcpyAsync(hcu, cu, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
    VNM_CUDA_TRY(cudaStreamSynchronize(st));
    if (hci[4]) return VNM_ERR_INTERNAL;
    rounds = round + 1;
    if (hci[0] == 0) break;  // no segment holds an invalid group
    swaps += hci[1];
    idle = hci[1] == 0 ? idle + 1 : 0;
    if (idle >= prm->patience) break;
    if (prm->stop_gain > 0 && (long long)hcu[0] >= prm->stop_gain) break;
  }
  VNM_CUDA_TRY(cudaEventRecord(ctx->ev_main1, st));
  VNM_CUDA_TRY(cudaMemsetAsync(cu + 2, 0, sizeof(unsigned long long) * 2, st));
  if (nseg > 0) VNM_LAUNCH(ctx, k_l_totals, lgrid(ctx, nseg), 256, 0, L.hist, nseg, N, cu + 2);
  VNM_CUDA_TRY(cudaMemcpyAsync(hcu, cu, sizeof(unsigned long long) * 4, cudaMemcpyDeviceToHost, st));
  VNM_CUDA_TRY(cudaMemcpyAsync(hci, ci, sizeof(int) * 8, cudaMemcpyDeviceToHost, st));
  VNM_CUDA_TRY(cudaStreamSynchronize(st));
  VNM_CUDA_TRY(cudaEventElapsedTime(&ctx->main_ms, ctx->ev_main0, ctx->ev_main1));
  out->final_invalid = (long long)hcu[2];
  out->final_retained = (long long)hcu[3];
  out->gain = (long long)hcu[0];
  out->exact_scored = (long long)hcu[1];
  out->rounds = rounds;
  out->swaps = swaps;
  out->ndump = hci[3] < dcap ? hci[3] : dcap;
  for (int q = 0; q < 28; ++q) ctx->stats[q] = 0;
  ctx->stats[0] = rounds;
  ctx->stats[1] = out->exact_scored;
  ctx->stats[2] = swaps;
  ctx->stats[3] = nseg;
  ctx->stats[5] = P.np;
  if (out->ndump) {
    VNM_CUDA_TRY(cudaMemcpyAsync(prm->dump_features, dx, sizeof(float) * LF * out->ndump, cudaMemcpyDeviceToHost, st));
    VNM_CUDA_TRY(cudaMemcpyAsync(prm->dump_gains, dy, sizeof(float) * out->ndump, cudaMemcpyDeviceToHost, st));
  }
  if (newpos && R > 0) {
    VNM_LAUNCH(ctx, k_l_invert, lgrid(ctx, R), 256, 0, L.orig, R, d_newpos);
    VNM_CUDA_TRY(cudaMemcpyAsync(newpos, d_newpos, sizeof(int) * R, cudaMemcpyDeviceToHost, st));
  }
  return end_call(ctx);
}

}  // extern "C"
