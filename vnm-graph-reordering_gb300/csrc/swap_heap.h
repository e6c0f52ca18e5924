// Pop order of the reference's swap-pair priority queue, emulated exactly.
//
// get_segment_swap_score (reorder/reorder.h:521-532) pushes the M*M swap
// pairs of one segment pair, in index order, into a
// std::priority_queue<SwapPair*, std::vector<SwapPair*>, Comparator>, and the
// greedy loop pops from it (reorder/reorder.h:1897-1908).  Comparator
// (reorder/swappair.h:112-120) is `<=` on full ties, so which of several
// equal pairs comes out first is decided by the heap's sift steps.  The
// routines below perform the same sift steps as GCC's libstdc++ push_heap /
// pop_heap (the sequence priority_queue::push and ::pop run), so the pop order
// matches the reference bit for bit.  Keys are precomputed so that the
// comparator is one 64-bit compare:
//   key = (left_gain + right_gain) << 32  |  (right_gain + 2^31)
//   Comparator(a, b)  <=>  key[a] <= key[b]
#ifndef VNM_SWAP_HEAP_H
#define VNM_SWAP_HEAP_H

#include <stdint.h>

#ifdef __CUDACC__
#define VNM_HD __host__ __device__ __forceinline__
#else
#define VNM_HD inline
#endif

VNM_HD int64_t swap_key(int lg, int rg) {
  return (int64_t)((uint64_t)(int64_t)(lg + rg) << 32) + (int64_t)((uint32_t)rg ^ 0x80000000u);
}

// `key[n]` holds the keys of pairs 0..n-1; `heap` is scratch of n entries;
// `order[k]` receives the index popped k-th.  n <= 255.
VNM_HD void swap_heap_pop_order(int n, const int64_t* key, uint8_t* heap, uint8_t* order) {
  // n pushes: heap.push_back(v); __push_heap(first, len, 0, v)
  for (int len = 0; len < n; ++len) {
    const int v = len;
    const int64_t kv = key[v];
    int hole = len;
    int parent = (hole - 1) / 2;
    while (hole > 0 && key[heap[parent]] <= kv) {
      heap[hole] = heap[parent];
      hole = parent;
      parent = (hole - 1) / 2;
    }
    heap[hole] = (uint8_t)v;
  }
  // n pops: pop_heap(first, last) then pop_back()
  for (int len = n, k = 0; len > 0; --len, ++k) {
    order[k] = heap[0];
    if (len > 1) {
      const int last = len - 1;  // element at `last` is re-inserted from the hole at the root
      const int v = heap[last];
      const int64_t kv = key[v];
      // __adjust_heap(first, 0, last, v)
      int hole = 0, second = 0;
      while (second < (last - 1) / 2) {
        second = 2 * (second + 1);
        if (key[heap[second]] <= key[heap[second - 1]]) second--;
        heap[hole] = heap[second];
        hole = second;
      }
      if ((last & 1) == 0 && second == (last - 2) / 2) {
        second = 2 * (second + 1);
        heap[hole] = heap[second - 1];
        hole = second - 1;
      }
      // __push_heap(first, hole, 0, v)
      int parent = (hole - 1) / 2;
      while (hole > 0 && key[heap[parent]] <= kv) {
        heap[hole] = heap[parent];
        hole = parent;
        parent = (hole - 1) / 2;
      }
      heap[hole] = (uint8_t)v;
    }
  }
}

#endif
