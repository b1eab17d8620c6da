// entry_tiles.cuh -- exact search distances of a warp tile of 4 queries x 8
// rows (32 pairs), for the two-level entry choice (entries.cu).
//
// The search distance of a query q to a row x is fixed by the search kernel's
// arithmetic (warp_astar_accelerator.h:237-287 with nvcc's FMA contraction):
// partial l (l = 0..31) is the fused multiply-add chain over dimensions
// l, l+32, l+64, ... in that order, and the 32 partials meet in the xor
// butterfly 16, 8, 4, 2, 1.  Here, as in the search, lane l of a warp keeps
// partial l -- for all 32 pairs of the tile at once -- reading dimension j of
// every query and row from shared memory (consecutive lanes, consecutive
// words: no bank conflicts).  The 32 pairs' partials then meet in one
// transposed butterfly (butterfly_rows<32>): at each level a lane keeps half
// of its pairs and adds its partner's partials of that half, so every pair
// sum is the butterfly's own pair and lane l ends with pair l's distance, bit
// for bit the search kernel's.  Products are computed two rows at a time with
// the paired FP32 instructions.
#pragma once

#include <cstdint>

#include "device_common.cuh"
#include "song_gb300.h"

namespace song {

// Lane l returns the search distance of query l >> 3 (q + (l >> 3) * qs) to
// row l & 7 (x + (l & 7) * xs); dpad elements, zero-padded past the dimension.
template <int METRIC>
__device__ __forceinline__ float warp_tile_distance(const float *q, int qs, const float *x, int xs, int dpad,
                                                    int lane) {
  constexpr bool COS = METRIC == SONG_METRIC_COS;
  uint64_t acc[4][4];  // query a, rows (2p, 2p+1)
  uint64_t ln[4];      // rows (2p, 2p+1): squared norms (cosine)
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int p = 0; p < 4; ++p) acc[a][p] = 0ull;
#pragma unroll
  for (int p = 0; p < 4; ++p) ln[p] = 0ull;
#pragma unroll 2
  for (int j = lane; j < dpad; j += 32) {
    uint64_t xx[4];
#pragma unroll
    for (int p = 0; p < 4; ++p) xx[p] = f2_pack(x[(2 * p) * xs + j], x[(2 * p + 1) * xs + j]);
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      const float qv = q[a * qs + j];
      const uint64_t qq = f2_pack(qv, qv);
#pragma unroll
      for (int p = 0; p < 4; ++p) {
        if (METRIC == SONG_METRIC_L2) {
          const uint64_t df = f2_sub(qq, xx[p]);
          acc[a][p] = f2_fma(df, df, acc[a][p]);
        } else {
          acc[a][p] = f2_fma(qq, xx[p], acc[a][p]);
        }
      }
    }
    if (COS) {
#pragma unroll
      for (int p = 0; p < 4; ++p) ln[p] = f2_fma(xx[p], xx[p], ln[p]);
    }
  }
  float v[32];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int p = 0; p < 4; ++p) f2_unpack(acc[a][p], v[8 * a + 2 * p], v[8 * a + 2 * p + 1]);
  const float t = butterfly_rows<32>(v, lane);  // pair `lane`
  if (METRIC == SONG_METRIC_L2) return t;
  if (METRIC == SONG_METRIC_IP) return -t;
  float lv[8];
#pragma unroll
  for (int p = 0; p < 4; ++p) f2_unpack(ln[p], lv[2 * p], lv[2 * p + 1]);
  const float lsum = butterfly_rows<8>(lv, lane);                // row lane / 4
  const float len = __shfl_sync(0xffffffffu, lsum, 4 * (lane & 7));  // row lane & 7
  if (len != 0.0f) {
    const float sign = t < 0.0f ? 1.0f : -1.0f;
    return __fdiv_rn(__fmul_rn(__fmul_rn(sign, t), t), len);
  }
  return 0.0f;
}

// One round of a merge over the 8 lanes of a query's group (lanes 8a ..
// 8a+7), each holding a sorted list: every lane of the group gets the
// nearest head, and the owning lane moves past it (ids are distinct).
template <int NS>
__device__ __forceinline__ void group8_take(const float (&bd)[NS], const uint32_t (&bi)[NS], int &h, float &wd,
                                            uint32_t &wid) {
  float d = __int_as_float(0x7f800000);
  uint32_t id = 0xffffffffu;
#pragma unroll
  for (int m = 0; m < NS; ++m)
    if (m == h) {
      d = bd[m];
      id = bi[m];
    }
  wd = d;
  wid = id;
#pragma unroll
  for (int o = 4; o > 0; o >>= 1) {
    const float od = __shfl_xor_sync(0xffffffffu, wd, o);
    const uint32_t oid = __shfl_xor_sync(0xffffffffu, wid, o);
    if (od < wd || (od == wd && oid < wid)) {
      wd = od;
      wid = oid;
    }
  }
  if (id == wid && id != 0xffffffffu) ++h;
}

}  // namespace song
