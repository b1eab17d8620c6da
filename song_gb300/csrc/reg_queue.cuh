// reg_queue.cuh -- a sorted array of (distance, id) keys held in the registers
// of one warp.  Replaces the reference's serial min-max heap (smmh2.h) and
// binary heap (bin_heap.h).
//
// Layout: capacity C = 32*S positions, lane-blocked (lane l holds positions
// l*S .. l*S+S-1 in v[0..S-1]), ascending, RIGHT-aligned: the n live keys sit
// at positions C-n .. C-1 and every position left of them holds 0, a key
// smaller than any real key (real keys carry order-preserving distance bits
// >= 0x007fffff in their high word).  Consequences:
//   * the maximum is always at position C-1 (lane 31, v[S-1]): O(1);
//   * inserting without eviction moves the smaller keys one place left,
//     inserting with eviction of the maximum moves the larger keys one place
//     right; neither needs the insertion position, only per-slot compares
//     against the new key and one shuffle for the lane boundary;
//   * removing the minimum (position C-n) is the only operation that touches
//     a dynamic position: one select pass over the S slots.
// All operations are warp-uniform.
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

  // Key at position pos (broadcast).
  // (Selections compare the full position, lane*S + j, rather than a slot
  // index: written as "slot == r" the compiler turns the loop into a dynamic
  // array index and moves the array to local memory.)
  __device__ __forceinline__ uint64_t at(int pos, int lane) const {
    uint64_t x = 0;
#pragma unroll
    for (int j = 0; j < S; ++j) x = (lane * S + j) == pos ? v[j] : x;
    return __shfl_sync(FULL, x, pos / S);
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

  // Remove the minimum of n >= 1 live keys; returns it, and the new minimum
  // in *next (~0 if none is left).
  __device__ __forceinline__ uint64_t pop_min(int n, int lane, uint64_t *next) {
    const int pos = C - n;
    uint64_t x = 0, y = ~0ull;
#pragma unroll
    for (int j = 0; j < S; ++j) {
      const int q = lane * S + j;
      x = q == pos ? v[j] : x;
      y = q == pos + 1 ? v[j] : y;
      v[j] = q == pos ? 0ull : v[j];
    }
    const uint64_t m = __shfl_sync(FULL, x, pos / S);
    *next = n > 1 ? __shfl_sync(FULL, y, (pos + 1) / S) : ~0ull;
    return m;
  }

  // Key of rank i (0 = smallest) among n live keys, for the output: lane l's
  // slot j holds rank l*S + j - (C - n).
  __device__ __forceinline__ int rank_of(int j, int n, int lane) const { return lane * S + j - (C - n); }
};

}  // namespace song
