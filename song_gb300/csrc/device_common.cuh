// device_common.cuh -- warp-cooperative building blocks of the search kernel:
// bulk-copy / mbarrier wrappers (inline PTX, sm_90+ forms valid on sm_103a),
// the sort keys of the candidate / top-pq queues, and the visited hashes held
// in the shared memory slice of one warp.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace song {

constexpr unsigned FULL = 0xffffffffu;
constexpr int32_t FH_EMPTY = -1;     // fixhash.h:3 EMPTY
constexpr int32_t FH_DELETION = -2;  // fixhash.h:3 DELETION (never written with backward-shift delete)
// fixhash.h:9, the first multiplier / xor pair used by hash(0, x).
constexpr uint64_t FH_R0 = 0x4bcb391f924ed183ULL;
constexpr uint64_t FH_R1 = 0xa0ab69ccd854fc0aULL;

// Bounded waits: an mbarrier that does not complete within this many polls
// (each poll may itself suspend in hardware) sets the error flag and returns.
// The default of an index; song_debug_set_wait changes it per index.
constexpr uint32_t WAIT_LIMIT = 1u << 24;

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}

// 1-D bulk copy global -> shared, completion counted on `bar` in bytes.
// dst, src and bytes must be multiples of 16.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait for phase `parity` of `bar`; false on timeout.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, uint32_t limit) {
  for (uint32_t i = 0; i < limit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// Two FP32 lanes in one 64-bit register, for the paired FP32 instructions of
// sm_100-family GPUs (sub/fma .rn.f32x2: each half rounded to nearest even,
// exactly the scalar __fsub_rn / __fmaf_rn).
__device__ __forceinline__ uint64_t f2_pack(float lo, float hi) {
  uint64_t r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
  return r;
}
__device__ __forceinline__ void f2_unpack(uint64_t r, float &lo, float &hi) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(r));
}
__device__ __forceinline__ uint64_t f2_sub(uint64_t a, uint64_t b) {
  uint64_t r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ uint64_t f2_fma(uint64_t a, uint64_t b, uint64_t c) {
  uint64_t r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
  return r;
}
__device__ __forceinline__ uint64_t f2_add(uint64_t a, uint64_t b) {
  uint64_t r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}

// The xor butterfly 16, 8, 4, 2, 1 over the 32 lanes' partial sums of H rows
// at once.  At the first log2(H) levels each lane keeps half of its rows and
// sends its partner the other half, so one shuffle serves two rows; every
// row still meets its partials in the butterfly's pairs (each pair sum is
// the same two floats, and a + b == b + a), so the sums are bit for bit the
// per-row butterfly's.  Returns, in lane l, the sum of row l / (32 / H).
template <int H>
__device__ __forceinline__ float butterfly_rows(float (&v)[H], int lane) {
  static_assert(H >= 1 && H <= 32 && (H & (H - 1)) == 0, "H must be a power of two");
  int o = 16;
#pragma unroll
  for (int n = H; n > 1; n >>= 1, o >>= 1) {
    const bool hi = (lane & o) != 0;
#pragma unroll
    for (int i = 0; i < n / 2; ++i) {
      const float keep = hi ? v[i + n / 2] : v[i];
      const float send = hi ? v[i] : v[i + n / 2];
      v[i] = __fadd_rn(keep, __shfl_xor_sync(FULL, send, o));
    }
  }
#pragma unroll
  for (; o > 0; o >>= 1) v[0] = __fadd_rn(v[0], __shfl_xor_sync(FULL, v[0], o));
  return v[0];
}

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// ---------------------------------------------------------------------------
// Keys of the sorted queues: (distance, id) in one uint64 whose unsigned
// order is (distance ascending, id ascending).  The distance is mapped to an
// order-preserving uint32 after -0 is folded onto +0, so that the reference's
// float comparisons (which treat -0 == +0) and key comparisons agree.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t dist_bits(float d) {
  if (d == 0.0f) d = 0.0f;
  uint32_t u = __float_as_uint(d);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ uint64_t make_key(float d, uint32_t id) {
  return (static_cast<uint64_t>(dist_bits(d)) << 32) | id;
}
__device__ __forceinline__ uint32_t key_dist(uint64_t k) { return static_cast<uint32_t>(k >> 32); }
__device__ __forceinline__ uint32_t key_id(uint64_t k) { return static_cast<uint32_t>(k); }

// ---------------------------------------------------------------------------
// Visited hash: the reference's FixHash<int, 8*pq> (fixhash.h) in the warp's
// shared memory, with the same slot function, linear probing and
// backward-shift delete, so that membership answers (including the rare
// entries its delete loses) are the reference's.
// ---------------------------------------------------------------------------
struct VisitedHash {
  int32_t *tab;
  int cap;        // 8 * pq
  uint64_t magic; // floor((2^64 - 1) / cap): v % cap by one high multiply and one correction

  // hash(0, x) = (x ^ (x >> 16) * r0 ^ r1) % cap (fixhash.h:20-24).  x is the
  // stored int widened to 64 bits; ids are < 2^31 so that is the id itself.
  __device__ __forceinline__ int slot(uint32_t id) const {
    uint64_t x = id;
    uint64_t v = x ^ ((x >> 16) * FH_R0) ^ FH_R1;
    uint64_t q = __umul64hi(v, magic);
    uint64_t r = v - q * static_cast<uint64_t>(cap);
    if (r >= static_cast<uint64_t>(cap)) r -= static_cast<uint64_t>(cap);
    return static_cast<int>(r);
  }

  // s < cap + 32 <= 3 * cap (every caller adds at most 32 to a slot, and
  // cap = 8 * pq >= 16): two conditional subtractions, no branch
  __device__ __forceinline__ int wrap(int s) const {
    s = s >= cap ? s - cap : s;
    return s >= cap ? s - cap : s;
  }

  __device__ __forceinline__ void clear(int lane) {
    for (int i = lane; i < cap; i += 32) tab[i] = FH_EMPTY;
    __syncwarp();
  }

  // One lane, own key (fixhash.h:49-57).
  __device__ __forceinline__ bool test(uint32_t id) const {
    int c = slot(id);
    for (int i = 0; i < cap; ++i) {
      int32_t v = tab[c];
      if (v == FH_EMPTY) return false;
      if (v == static_cast<int32_t>(id)) return true;
      c = c + 1 == cap ? 0 : c + 1;
    }
    return false;
  }

  // Whole warp, one key (fixhash.h:38-47): first EMPTY/DELETION slot on the
  // probe sequence, found 32 slots at a time with a ballot.  `home` is
  // slot(id), computed by the caller (often in parallel, one lane per key).
  __device__ __forceinline__ void add_at(uint32_t id, int home, int lane) {
    int base = home;
    for (int w = 0; w * 32 < cap + 32; ++w) {
      int s = wrap(base + lane);
      int32_t v = tab[s];
      unsigned b = __ballot_sync(FULL, v == FH_EMPTY || v == FH_DELETION);
      if (b) {
        if (lane == __ffs(b) - 1) tab[s] = static_cast<int32_t>(id);
        break;
      }
      base = wrap(base + 32);
    }
    __syncwarp();
  }

  __device__ __forceinline__ void add(uint32_t id, int lane) { add_at(id, slot(id), lane); }

  // Whole warp, one key (fixhash.h:59-93), `home` = slot(id).  The run after
  // the removed entry is read 32 slots at a time; the reference's sequential
  // case analysis then runs uniformly over it, with each lane's slot value
  // and home slot fetched by shuffle.  Home slots of the run are computed
  // only when the slot after the removed entry is occupied.
  __device__ __forceinline__ void del_at(uint32_t id, int home, int lane) {
    const int32_t x = static_cast<int32_t>(id);
    int code = home;
    int r = -1;
    int base = code;
    for (int w = 0; w * 32 < cap + 32; ++w) {
      int s = wrap(base + lane);
      int32_t v = tab[s];
      unsigned be = __ballot_sync(FULL, v == FH_EMPTY);
      unsigned bm = __ballot_sync(FULL, v == x);
      unsigned before = be ? ((1u << (__ffs(be) - 1)) - 1u) : FULL;
      unsigned hit = bm & before;
      if (hit) {
        r = wrap(base + __ffs(hit) - 1);
        break;
      }
      if (be) return;  // not present
      base = wrap(base + 32);
    }
    if (r < 0) return;
    int nbase = wrap(r + 1);
    for (int w = 0; w * 32 < cap + 32; ++w) {
      int s = wrap(nbase + lane);
      int32_t v = tab[s];
      unsigned be = __ballot_sync(FULL, v == FH_EMPTY);
      int run = be ? __ffs(be) - 1 : 32;
      int hv = 0;
      if (run > 0) hv = v >= 0 ? slot(static_cast<uint32_t>(v)) : 0;  // warp-uniform branch
      for (int i = 0; i < run; ++i) {
        int nxt = wrap(nbase + i);
        int ncode = __shfl_sync(FULL, hv, i);
        int32_t val = __shfl_sync(FULL, v, i);
        bool cond1 = code <= r;
        bool cond2 = r < nxt;
        bool move;
        if (cond1 && cond2) move = ncode <= r;
        else if (cond1) move = nxt < ncode && ncode <= r;
        else move = nxt < ncode || ncode <= r;
        if (move) {
          if (lane == 0) tab[r] = val;
          r = nxt;
          code = ncode;
        }
      }
      __syncwarp();
      if (be) break;
      nbase = wrap(nbase + 32);
    }
    if (lane == 0) tab[r] = FH_EMPTY;
    __syncwarp();
  }

  __device__ __forceinline__ void del(uint32_t id, int lane) { del_at(id, slot(id), lane); }
};

// ---------------------------------------------------------------------------
// Exact visited set for the learned / low-precision path, which makes no
// bit-parity claim with the reference: power-of-two capacity (>= 4*pq), a
// multiplicative slot function, linear probing and the textbook
// backward-shift delete (an entry moves into the hole when its home slot is
// not cyclically inside (hole, position]), so no entry is ever lost.  Half the
// shared memory of VisitedHash at the same pq, and a two-instruction slot.
// ---------------------------------------------------------------------------
struct ExactVisited {
  int32_t *tab;
  int cap;       // power of two
  int log2cap;

  __device__ __forceinline__ int slot(uint32_t id) const {
    return static_cast<int>((id * 0x9E3779B1u) >> (32 - log2cap));  // cap >= 32
  }
  __device__ __forceinline__ int wrap(int s) const { return s & (cap - 1); }

  __device__ __forceinline__ void clear(int lane) {
    for (int i = lane; i < cap; i += 32) tab[i] = FH_EMPTY;
    __syncwarp();
  }

  __device__ __forceinline__ bool test(uint32_t id) const {
    int c = slot(id);
    for (int i = 0; i < cap; ++i) {
      const int32_t v = tab[c];
      if (v == FH_EMPTY) return false;
      if (v == static_cast<int32_t>(id)) return true;
      c = (c + 1) & (cap - 1);
    }
    return false;
  }

  __device__ __forceinline__ void add_at(uint32_t id, int home, int lane) {
    int base = home;
    for (int w = 0; w * 32 < cap + 32; ++w) {
      const int s = wrap(base + lane);
      const int32_t v = tab[s];
      const unsigned b = __ballot_sync(FULL, v == FH_EMPTY);
      if (b) {
        if (lane == __ffs(b) - 1) tab[s] = static_cast<int32_t>(id);
        break;
      }
      base = wrap(base + 32);
    }
    __syncwarp();
  }

  __device__ __forceinline__ void add(uint32_t id, int lane) { add_at(id, slot(id), lane); }

  __device__ __forceinline__ void del_at(uint32_t id, int home, int lane) {
    const int32_t x = static_cast<int32_t>(id);
    int base = home, h = -1;
    for (int w = 0; w * 32 < cap + 32; ++w) {
      const int s = wrap(base + lane);
      const int32_t v = tab[s];
      const unsigned be = __ballot_sync(FULL, v == FH_EMPTY);
      const unsigned bm = __ballot_sync(FULL, v == x);
      const unsigned before = be ? ((1u << (__ffs(be) - 1)) - 1u) : FULL;
      const unsigned hit = bm & before;
      if (hit) {
        h = wrap(base + __ffs(hit) - 1);
        break;
      }
      if (be) return;
      base = wrap(base + 32);
    }
    if (h < 0) return;
    int nbase = wrap(h + 1);
    for (int w = 0; w * 32 < cap + 32; ++w) {
      const int s = wrap(nbase + lane);
      const int32_t v = tab[s];
      const int home = v >= 0 ? slot(static_cast<uint32_t>(v)) : 0;
      const unsigned be = __ballot_sync(FULL, v == FH_EMPTY);
      const int run = be ? __ffs(be) - 1 : 32;
      for (int i = 0; i < run; ++i) {
        const int j = wrap(nbase + i);
        const int hm = __shfl_sync(FULL, home, i);
        const int32_t val = __shfl_sync(FULL, v, i);
        if (((j - hm) & (cap - 1)) >= ((j - h) & (cap - 1))) {
          if (lane == 0) tab[h] = val;
          h = j;
        }
      }
      __syncwarp();
      if (be) break;
      nbase = wrap(nbase + 32);
    }
    if (lane == 0) tab[h] = FH_EMPTY;
    __syncwarp();
  }

  __device__ __forceinline__ void del(uint32_t id, int lane) { del_at(id, slot(id), lane); }
};

}  // namespace song
