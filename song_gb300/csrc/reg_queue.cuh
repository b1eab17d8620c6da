// reg_queue.cuh -- a sorted array of (distance, id) keys held in the registers
// of one warp.  The search keeps its candidate queue (the reference's serial
// min-max heap, smmh2.h) and its top-pq list (the binary heap, bin_heap.h) in
// two of them.
//
// Layout: capacity C = 32*S positions, lane-blocked (lane l holds positions
// l*S .. l*S+S-1 in v[0..S-1]), ascending.  Both lists use the WINDOW form:
// positions C-pq .. C-1 always hold pq keys, the live keys first and then
// "infinite" keys (~0); every position left of the window holds 0, smaller
// than any real key (real keys carry order-preserving distance bits
// >= 0x007fffff in their high word).  Consequences:
//   * an insertion is always "insert and drop the window's maximum": keys not
//     below the new key move one place right and an infinite key (or, when
//     all pq are live, the real maximum) falls off -- one code path, per-slot
//     compares and selects, one shuffle at the lane boundary;
//   * the maximum is always at position C-1 (lane 31, v[S-1]): O(1);
//   * the minimum is at position C-pq; removing it shifts the window one
//     place left and appends an infinite key;
//   * reads at a run-time (warp-uniform) position are a binary tree of
//     selects on the slot bits; nothing is indexed at run time, so the array
//     never goes to local memory.
// (insert_grow, the right-aligned form without a window, serves the FP32
// re-rank of low-precision storage.)  All operations are warp-uniform.
#pragma once

#include <cstdint>

#include "device_common.cuh"

namespace song {

template <int S>
struct RegQueue {
  static constexpr int C = 32 * S;
  uint64_t v[S];

  __device__ __forceinline__ void clear() {
#pragma unroll
    for (int j = 0; j < S; ++j) v[j] = 0ull;
  }

  // Largest live key (0 when empty).
  __device__ __forceinline__ uint64_t max() const { return __shfl_sync(FULL, v[S - 1], 31); }

  // Key at the warp-uniform position pos (broadcast).  (Selections never
  // index v[] with a run-time value: the compiler would move the array to
  // local memory.)
  __device__ __forceinline__ uint64_t at(int pos, int lane) const {
    const int owner = pos / S;
    return __shfl_sync(FULL, slot(pos - owner * S), owner);
  }

  // Insert, n -> n + 1 (requires n < C): keys below `key` move one place left.
  __device__ __forceinline__ void insert_grow(uint64_t key, int lane) {
    uint64_t nxt = __shfl_down_sync(FULL, v[0], 1);
    if (lane == 31) nxt = ~0ull;
#pragma unroll
    for (int j = 0; j < S; ++j) {
      const uint64_t right = j + 1 < S ? v[j + 1] : nxt;
      v[j] = right < key ? right : (v[j] < key ? key : v[j]);
    }
  }

  // Insert and drop the maximum, n unchanged: keys not below `key` move one
  // place right and the old maximum falls off.  If key >= the maximum nothing
  // changes (the key itself is dropped).
  __device__ __forceinline__ void insert_evict(uint64_t key, int lane) {
    uint64_t prv = __shfl_up_sync(FULL, v[S - 1], 1);
    if (lane == 0) prv = 0ull;
#pragma unroll
    for (int j = S - 1; j >= 0; --j) {
      const uint64_t left = j > 0 ? v[j - 1] : prv;
      v[j] = v[j] < key ? v[j] : (left < key ? key : left);
    }
  }

  // v[r] for a warp-uniform slot r in [0, S): a binary tree of selects on
  // the bits of r (S - 1 selects, depth log2 S; a chain of S compares would
  // serialise S dependent selects).
  __device__ __forceinline__ uint64_t slot(int r) const {
    uint64_t t[S];
#pragma unroll
    for (int j = 0; j < S; ++j) t[j] = v[j];
#pragma unroll
    for (int w = 1; w < S; w <<= 1) {
      const bool b = (r & w) != 0;
#pragma unroll
      for (int j = 0; j + w < S; j += 2 * w) t[j] = b ? t[j + w] : t[j];
    }
    return t[0];
  }

  // Window form (positions start .. C-1 hold the keys, start warp-uniform):
  // returns the key at start and shifts the window one place left, position
  // C-1 receiving ~0; *next gets the new key at start.
  __device__ __forceinline__ uint64_t pop_window(int start, int lane, uint64_t *next) {
    const int owner = start / S, r = start - owner * S;
    const uint64_t m = __shfl_sync(FULL, slot(r), owner);
    uint64_t nxt = __shfl_down_sync(FULL, v[0], 1);
    if (lane == 31) nxt = ~0ull;
#pragma unroll
    for (int j = 0; j < S; ++j) {
      const uint64_t right = j + 1 < S ? v[j + 1] : nxt;
      v[j] = (lane * S + j) >= start ? right : v[j];
    }
    *next = __shfl_sync(FULL, slot(r), owner);
    return m;
  }

  // Key of rank i (0 = smallest) among n live keys, for the output: lane l's
  // slot j holds rank l*S + j - (C - n).
  __device__ __forceinline__ int rank_of(int j, int n, int lane) const { return lane * S + j - (C - n); }
};

}  // namespace song
