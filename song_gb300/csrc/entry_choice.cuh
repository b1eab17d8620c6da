// entry_choice.cuh -- the pieces of the entry-point choice shared by the
// pre-pass kernels (entries.cu) and the server's persistent warps (serve.cu):
// the search distance of one entry row computed by one thread, bit for bit
// as the search kernel computes it (32 lane-strided FMA partial sums in
// dimension order, added in the xor butterfly's pairs), and the per-lane
// sorted lists with their warp merge (ties to the smaller id).
#pragma once

#include <cstdint>

#include "song_gb300.h"

namespace song {

__device__ __forceinline__ bool closer(float d, uint32_t id, float bd, uint32_t bid) {
  return d < bd || (d == bd && id < bid);
}

// The search distance of one entry row (padded to d4 float4s) to one staged
// query, computed by one thread exactly as nearest_entry_kernel does.
template <int METRIC, bool GLOBAL>
__device__ __forceinline__ float entry_distance(const float4 *x4, const float4 *q4, int d4) {
  float t[32], l[32];
#pragma unroll
  for (int i = 0; i < 32; ++i) t[i] = l[i] = 0.0f;
  // Rows read from L2 are loaded one group of 32 dimensions ahead, so each
  // group's loads are in flight while the previous group is summed.
  float4 nxt[8];
  if (GLOBAL) {
#pragma unroll
    for (int i = 0; i < 8; ++i) nxt[i] = i < d4 ? __ldg(x4 + i) : make_float4(0.f, 0.f, 0.f, 0.f);
  }
  for (int c0 = 0; c0 < d4; c0 += 8) {
    float4 cur[8];
    if (GLOBAL) {
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        cur[i] = nxt[i];
        nxt[i] = c0 + 8 + i < d4 ? __ldg(x4 + c0 + 8 + i) : make_float4(0.f, 0.f, 0.f, 0.f);
      }
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      if (c0 + i < d4) {
        const float4 xv = GLOBAL ? cur[i] : x4[c0 + i];
        const float4 qv = q4[c0 + i];
        const float xs[4] = {xv.x, xv.y, xv.z, xv.w};
        const float qq[4] = {qv.x, qv.y, qv.z, qv.w};
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          if (METRIC == SONG_METRIC_L2) {
            const float d = __fsub_rn(qq[c], xs[c]);
            t[4 * i + c] = __fmaf_rn(d, d, t[4 * i + c]);
          } else {
            t[4 * i + c] = __fmaf_rn(qq[c], xs[c], t[4 * i + c]);
            if (METRIC == SONG_METRIC_COS) l[4 * i + c] = __fmaf_rn(xs[c], xs[c], l[4 * i + c]);
          }
        }
      }
    }
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
#pragma unroll
    for (int i = 0; i < off; ++i) {
      t[i] = __fadd_rn(t[i], t[i + off]);
      if (METRIC == SONG_METRIC_COS) l[i] = __fadd_rn(l[i], l[i + off]);
    }
  }
  if (METRIC == SONG_METRIC_L2) return t[0];
  if (METRIC == SONG_METRIC_IP) return -t[0];
  if (l[0] != 0.0f) {
    const float sign = t[0] < 0.0f ? 1.0f : -1.0f;
    return __fdiv_rn(__fmul_rn(__fmul_rn(sign, t[0]), t[0]), l[0]);
  }
  return 0.0f;
}

// Sorted insertion into a lane's NS best (distance, id); the last falls off.
template <int NS>
__device__ __forceinline__ void list_insert(float (&bd)[NS], uint32_t (&bi)[NS], float d, uint32_t id) {
#pragma unroll
  for (int m = NS - 1; m >= 0; --m) {
    const bool above = m > 0 && closer(d, id, bd[m > 0 ? m - 1 : 0], bi[m > 0 ? m - 1 : 0]);
    const bool here = closer(d, id, bd[m], bi[m]);
    if (above) {
      bd[m] = bd[m - (m > 0 ? 1 : 0)];
      bi[m] = bi[m - (m > 0 ? 1 : 0)];
    } else if (here) {
      bd[m] = d;
      bi[m] = id;
    }
  }
}

// One round of the warp merge: the nearest head over the lanes' lists (every
// lane gets it); the owning lane moves past it.
template <int NS>
__device__ __forceinline__ uint32_t list_take(const float (&bd)[NS], const uint32_t (&bi)[NS], int &h) {
  float d = __int_as_float(0x7f800000);
  uint32_t id = 0xffffffffu;
#pragma unroll
  for (int m = 0; m < NS; ++m)
    if (m == h) {
      d = bd[m];
      id = bi[m];
    }
  float wd = d;
  uint32_t wid = id;
  for (int o = 16; o > 0; o >>= 1) {
    const float od = __shfl_xor_sync(0xffffffffu, wd, o);
    const uint32_t oid = __shfl_xor_sync(0xffffffffu, wid, o);
    if (closer(od, oid, wd, wid)) {
      wd = od;
      wid = oid;
    }
  }
  if (id == wid && id != 0xffffffffu) ++h;
  return wid;
}

}  // namespace song
