// reg_queue.cuh -- a sorted array of (distance, id) keys held in the registers
// of one warp, lane-blocked: lane l holds elements l*S .. l*S+S-1.  Capacity
// 32*S.  Every operation is warp-uniform; dynamic positions are resolved with
// unrolled compare/select over the S slots, so the array never leaves the
// register file.  Replaces the reference's serial min-max heap (smmh2.h) and
// binary heap (bin_heap.h): insert, pop-min and drop-max cost O(S) register
// operations and one or two shuffles instead of O(log pq) dependent memory
// accesses by one thread.
#pragma once

#include <cstdint>

#include "device_common.cuh"

namespace song {

template <int S>
struct RegQueue {
  uint64_t v[S];

  __device__ __forceinline__ void clear() {
#pragma unroll
    for (int j = 0; j < S; ++j) v[j] = ~0ull;
  }

  // Element i (0 <= i < 32*S), broadcast to all lanes.
  __device__ __forceinline__ uint64_t get(int i) const {
    const int l = i / S, s = i - l * S;
    uint64_t x = v[0];
#pragma unroll
    for (int j = 1; j < S; ++j)
      if (j == s) x = v[j];
    return __shfl_sync(FULL, x, l);
  }

  // Number of the first n elements that are < key (= insertion position).
  __device__ __forceinline__ int lower_bound(uint64_t key, int n, int lane) const {
    int c = 0;
#pragma unroll
    for (int j = 0; j < S; ++j) c += (lane * S + j < n && v[j] < key) ? 1 : 0;
    return static_cast<int>(__reduce_add_sync(FULL, static_cast<unsigned>(c)));
  }

  // Insert key at position p; elements p.. move up one place (the last one of
  // a full array falls off).
  __device__ __forceinline__ void insert_at(int p, uint64_t key, int lane) {
    const uint64_t carry = __shfl_up_sync(FULL, v[S - 1], 1);
#pragma unroll
    for (int j = S - 1; j >= 0; --j) {
      const int i = lane * S + j;
      const uint64_t prev = j > 0 ? v[j - 1] : carry;
      v[j] = i < p ? v[j] : (i == p ? key : prev);
    }
  }

  __device__ __forceinline__ int insert(uint64_t key, int &n, int lane) {
    const int p = lower_bound(key, n, lane);
    insert_at(p, key, lane);
    ++n;
    return p;
  }

  // Remove element 0; everything moves down one place.
  __device__ __forceinline__ void pop_front(int lane) {
    const uint64_t nxt = __shfl_down_sync(FULL, v[0], 1);
#pragma unroll
    for (int j = 0; j < S - 1; ++j) v[j] = v[j + 1];
    v[S - 1] = lane == 31 ? ~0ull : nxt;
  }
};

}  // namespace song
