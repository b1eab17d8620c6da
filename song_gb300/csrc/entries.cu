// entries.cu -- entry points: each query starts its search at the nearest of a
// set of entry vertices instead of vertex 0.
//
// The reference always starts at vertex 0 (warp_astar_accelerator.h:173, and
// graph.h:176 with its random start commented out); that stays the default.
// With entries set (song_index_set_entries), a pre-pass picks for every query
// the entry with the smallest search distance, ties to the smaller id, and
// the search starts there.  Nothing else in the search changes.
//
// The distance is the search kernel's, bit for bit, on the FP32 rows: lane l
// of the search sums dims l, l+32, ... with fused multiply-adds and the 32
// partial sums meet in an xor butterfly (16, 8, 4, 2, 1).  Here one thread
// computes a whole distance: it keeps the 32 partial sums, adds each element
// to the partial of its lane in dimension order, and then adds them in the
// butterfly's pairs, which gives every lane's (identical) result.  The entry
// rows are copied once into a contiguous block, which stays in L2.  The
// two-level choice instead spreads each row over a warp as the search does,
// 32 (query, row) pairs at a time, and adds the partials in a transposed
// butterfly (entry_tiles.cuh): the same sums.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <vector>

#include "entry_choice.cuh"
#include "entry_tiles.cuh"
#include "internal.h"
#include "song_gb300.h"

namespace song {
namespace {

// One warp serves QB queries; lane e takes entries e, e+32, ... and reads
// each entry row once, in 16-byte pieces, for all QB queries.  Rows and the
// staged queries are zero-padded to dpad (a multiple of 4) floats: a padded
// element adds fma(0, 0, t) = t, leaving every partial sum exactly as the
// search leaves it.  Each lane keeps its NS nearest entries per query in a
// sorted register list; the warp then merges the lists, ns rounds of an xor
// argmin, into starts[q*ns ..], ascending by (distance, id).
template <int METRIC, int QB, int NS>
__global__ void __launch_bounds__(256) nearest_entry_kernel(const float *queries, int nq, int qstride, int dim,
                                                            int dpad,
                                                            const float *entry_rows, const uint32_t *entry_ids,
                                                            int n_entries, int ns, uint32_t *starts) {
  extern __shared__ float4 qs4[];  // (blockDim / 32) * QB query rows of dpad floats
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int q0 = (blockIdx.x * (blockDim.x >> 5) + wib) * QB;
  if (q0 >= nq) return;  // whole warps leave together
  const int d4 = dpad >> 2;
  float *qw = reinterpret_cast<float *>(qs4) + static_cast<size_t>(wib) * QB * dpad;
  for (int b = 0; b < QB; ++b)
    for (int j = lane; j < dpad; j += 32)
      qw[b * dpad + j] = (q0 + b < nq && j < dim) ? queries[static_cast<size_t>(q0 + b) * qstride + j] : 0.0f;
  __syncwarp();
  const float4 *q4 = reinterpret_cast<const float4 *>(qw);
  float bd[QB][NS];
  uint32_t bi[QB][NS];
#pragma unroll
  for (int b = 0; b < QB; ++b)
#pragma unroll
    for (int m = 0; m < NS; ++m) {
      bd[b][m] = __int_as_float(0x7f800000);  // +inf
      bi[b][m] = 0xffffffffu;
    }
  for (int e = lane; e < n_entries; e += 32) {
    const float4 *x4 = reinterpret_cast<const float4 *>(entry_rows + static_cast<size_t>(e) * dpad);
    float t[QB][32], l[32];
#pragma unroll
    for (int i = 0; i < 32; ++i) {
      l[i] = 0.0f;
#pragma unroll
      for (int b = 0; b < QB; ++b) t[b][i] = 0.0f;
    }
    for (int c0 = 0; c0 < d4; c0 += 8) {  // 32 dimensions: partial 4i + c takes dimension 4 (c0 + i) + c
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        if (c0 + i < d4) {
          const float4 xv = __ldg(x4 + c0 + i);
          const float xs[4] = {xv.x, xv.y, xv.z, xv.w};
#pragma unroll
          for (int b = 0; b < QB; ++b) {
            const float4 qv = q4[b * d4 + c0 + i];
            const float qq[4] = {qv.x, qv.y, qv.z, qv.w};
#pragma unroll
            for (int c = 0; c < 4; ++c) {
              if (METRIC == SONG_METRIC_L2) {
                const float d = __fsub_rn(qq[c], xs[c]);
                t[b][4 * i + c] = __fmaf_rn(d, d, t[b][4 * i + c]);
              } else {
                t[b][4 * i + c] = __fmaf_rn(qq[c], xs[c], t[b][4 * i + c]);
              }
            }
          }
          if (METRIC == SONG_METRIC_COS) {
#pragma unroll
            for (int c = 0; c < 4; ++c) l[4 * i + c] = __fmaf_rn(xs[c], xs[c], l[4 * i + c]);
          }
        }
      }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
#pragma unroll
      for (int i = 0; i < off; ++i) {
#pragma unroll
        for (int b = 0; b < QB; ++b) t[b][i] = __fadd_rn(t[b][i], t[b][i + off]);
        if (METRIC == SONG_METRIC_COS) l[i] = __fadd_rn(l[i], l[i + off]);
      }
    }
    const uint32_t id = entry_ids[e];
#pragma unroll
    for (int b = 0; b < QB; ++b) {
      float d;
      if (METRIC == SONG_METRIC_L2) {
        d = t[b][0];
      } else if (METRIC == SONG_METRIC_IP) {
        d = -t[b][0];
      } else if (l[0] != 0.0f) {
        const float sign = t[b][0] < 0.0f ? 1.0f : -1.0f;
        d = __fdiv_rn(__fmul_rn(__fmul_rn(sign, t[b][0]), t[b][0]), l[0]);
      } else {
        d = 0.0f;
      }
      // sorted insertion, the last entry falls off (positions read before written)
#pragma unroll
      for (int m = NS - 1; m >= 0; --m) {
        const bool above = m > 0 && closer(d, id, bd[b][m > 0 ? m - 1 : 0], bi[b][m > 0 ? m - 1 : 0]);
        const bool here = closer(d, id, bd[b][m], bi[b][m]);
        if (above) {
          bd[b][m] = bd[b][m - (m > 0 ? 1 : 0)];
          bi[b][m] = bi[b][m - (m > 0 ? 1 : 0)];
        } else if (here) {
          bd[b][m] = d;
          bi[b][m] = id;
        }
      }
    }
  }
#pragma unroll
  for (int b = 0; b < QB; ++b) {
    int h = 0;  // this lane's next unused list position
    for (int r = 0; r < ns; ++r) {
      float d = __int_as_float(0x7f800000);
      uint32_t id = 0xffffffffu;
#pragma unroll
      for (int m = 0; m < NS; ++m)
        if (m == h) {
          d = bd[b][m];
          id = bi[b][m];
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
      if (id == wid && id != 0xffffffffu) ++h;  // entry ids are distinct: one lane owns the winner
      if (lane == 0 && q0 + b < nq) starts[static_cast<size_t>(q0 + b) * ns + r] = wid;
    }
  }
}

// The same choice with the entry rows staged through shared memory, for rows
// of up to 1 KB: the block loads 32 entry rows at a time with coalesced
// 16-byte loads into rows padded to an odd number of 16-byte units (so the
// lanes' 16-byte reads of 32 different rows hit distinct banks), and every
// warp of the block then scores them against its queries, lane e taking row
// e of the tile.  Partial sums, order and merge are those of
// nearest_entry_kernel.
template <int METRIC, int QB, int NS>
__global__ void __launch_bounds__(256) nearest_entry_tiled_kernel(const float *queries, int nq, int qstride, int dim,
                                                            int dpad,
                                                                  const float *entry_rows,
                                                                  const uint32_t *entry_ids, int n_entries, int ns,
                                                                  uint32_t *starts) {
  extern __shared__ float4 sm4[];
  constexpr int TILE = 32;
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const int q0 = (blockIdx.x * nwarps + wib) * QB;
  const bool active = q0 < nq;  // warp-uniform; idle warps still help load tiles
  const int d4 = dpad >> 2, rs4 = d4 + 1;
  float4 *tile = sm4;
  float *qw = reinterpret_cast<float *>(sm4 + TILE * rs4) + static_cast<size_t>(wib) * QB * dpad;
  for (int b = 0; b < QB; ++b)
    for (int j = lane; j < dpad; j += 32)
      qw[b * dpad + j] = (q0 + b < nq && j < dim) ? queries[static_cast<size_t>(q0 + b) * qstride + j] : 0.0f;
  const float4 *q4 = reinterpret_cast<const float4 *>(qw);
  float bd[QB][NS];
  uint32_t bi[QB][NS];
#pragma unroll
  for (int b = 0; b < QB; ++b)
#pragma unroll
    for (int m = 0; m < NS; ++m) {
      bd[b][m] = __int_as_float(0x7f800000);
      bi[b][m] = 0xffffffffu;
    }
  for (int t0 = 0; t0 < n_entries; t0 += TILE) {
    const int rows = min(TILE, n_entries - t0);
    __syncthreads();  // the previous tile is consumed (and, first time, the queries are staged)
    for (int i = threadIdx.x; i < rows * d4; i += blockDim.x) {
      const int r = i / d4, c = i - r * d4;
      tile[r * rs4 + c] = __ldg(reinterpret_cast<const float4 *>(entry_rows + static_cast<size_t>(t0 + r) * dpad) + c);
    }
    __syncthreads();
    if (!active || lane >= rows) continue;
    const float4 *x4 = tile + lane * rs4;
    float t[QB][32], l[32];
#pragma unroll
    for (int i = 0; i < 32; ++i) {
      l[i] = 0.0f;
#pragma unroll
      for (int b = 0; b < QB; ++b) t[b][i] = 0.0f;
    }
    for (int c0 = 0; c0 < d4; c0 += 8) {
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        if (c0 + i < d4) {
          const float4 xv = x4[c0 + i];
          const float xs[4] = {xv.x, xv.y, xv.z, xv.w};
#pragma unroll
          for (int b = 0; b < QB; ++b) {
            const float4 qv = q4[b * d4 + c0 + i];
            const float qq[4] = {qv.x, qv.y, qv.z, qv.w};
#pragma unroll
            for (int c = 0; c < 4; ++c) {
              if (METRIC == SONG_METRIC_L2) {
                const float d = __fsub_rn(qq[c], xs[c]);
                t[b][4 * i + c] = __fmaf_rn(d, d, t[b][4 * i + c]);
              } else {
                t[b][4 * i + c] = __fmaf_rn(qq[c], xs[c], t[b][4 * i + c]);
              }
            }
          }
          if (METRIC == SONG_METRIC_COS) {
#pragma unroll
            for (int c = 0; c < 4; ++c) l[4 * i + c] = __fmaf_rn(xs[c], xs[c], l[4 * i + c]);
          }
        }
      }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
#pragma unroll
      for (int i = 0; i < off; ++i) {
#pragma unroll
        for (int b = 0; b < QB; ++b) t[b][i] = __fadd_rn(t[b][i], t[b][i + off]);
        if (METRIC == SONG_METRIC_COS) l[i] = __fadd_rn(l[i], l[i + off]);
      }
    }
    const uint32_t id = entry_ids[t0 + lane];
#pragma unroll
    for (int b = 0; b < QB; ++b) {
      float d;
      if (METRIC == SONG_METRIC_L2) {
        d = t[b][0];
      } else if (METRIC == SONG_METRIC_IP) {
        d = -t[b][0];
      } else if (l[0] != 0.0f) {
        const float sign = t[b][0] < 0.0f ? 1.0f : -1.0f;
        d = __fdiv_rn(__fmul_rn(__fmul_rn(sign, t[b][0]), t[b][0]), l[0]);
      } else {
        d = 0.0f;
      }
#pragma unroll
      for (int m = NS - 1; m >= 0; --m) {
        const bool above = m > 0 && closer(d, id, bd[b][m > 0 ? m - 1 : 0], bi[b][m > 0 ? m - 1 : 0]);
        const bool here = closer(d, id, bd[b][m], bi[b][m]);
        if (above) {
          bd[b][m] = bd[b][m - (m > 0 ? 1 : 0)];
          bi[b][m] = bi[b][m - (m > 0 ? 1 : 0)];
        } else if (here) {
          bd[b][m] = d;
          bi[b][m] = id;
        }
      }
    }
  }
  if (!active) return;
#pragma unroll
  for (int b = 0; b < QB; ++b) {
    int h = 0;
    for (int r = 0; r < ns; ++r) {
      float d = __int_as_float(0x7f800000);
      uint32_t id = 0xffffffffu;
#pragma unroll
      for (int m = 0; m < NS; ++m)
        if (m == h) {
          d = bd[b][m];
          id = bi[b][m];
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
      if (lane == 0 && q0 + b < nq) starts[static_cast<size_t>(q0 + b) * ns + r] = wid;
    }
  }
}

// Gathers the FP32 rows of the entries into a contiguous block.
__global__ void gather_entry_rows_kernel(const float *rows, uint32_t row_floats, const uint32_t *ids, int n,
                                         int dpad, float *out) {
  const uint64_t total = static_cast<uint64_t>(n) * dpad;
  for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < total;
       i += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
    const uint64_t e = i / dpad;
    out[i] = rows[static_cast<uint64_t>(ids[e]) * row_floats + (i - e * dpad)];
  }
}

// The ns nearest of n entry rows (ids) for each of nq query rows (stride
// qstride floats), into out[q*ns ..].
cudaError_t launch_nearest(const float *queries, int nq, int qstride, int dim, int dpad, int metric,
                           const float *rows, const uint32_t *ids, int n, int ns, uint32_t *out, cudaStream_t s) {
  // warps per block: up to 8, within the default 48 KB of shared memory;
  // rows of up to 1 KB are staged through shared memory in 32-row tiles
  const int qb = metric == SONG_METRIC_COS ? 1 : 2;
  const int per_warp = static_cast<int>(sizeof(float)) * dpad * qb;
  const int tile_bytes = 32 * (dpad / 4 + 1) * 16;
  const bool tiled = dpad * 4 <= 1024 && tile_bytes + per_warp <= 48 * 1024;
  const int avail = 48 * 1024 - (tiled ? tile_bytes : 0);
  const int wpb = std::max(1, std::min(8, avail / per_warp));
  const size_t smem = static_cast<size_t>(per_warp) * wpb + (tiled ? tile_bytes : 0);
  const unsigned grid = static_cast<unsigned>((nq + wpb * qb - 1) / (wpb * qb));
  const int NSel = ns <= 1 ? 1 : (ns <= 2 ? 2 : (ns <= 4 ? 4 : 8));
#define SONG_ENTRY_LAUNCH(M, QB, NS)                                                                        \
  do {                                                                                                   \
    if (tiled)                                                                                           \
      nearest_entry_tiled_kernel<M, QB, NS><<<grid, 32 * wpb, smem, s>>>(queries, nq, qstride, dim, dpad,  \
                                                                         rows, ids, n, ns, out);         \
    else                                                                                                 \
      nearest_entry_kernel<M, QB, NS><<<grid, 32 * wpb, smem, s>>>(queries, nq, qstride, dim, dpad, rows, \
                                                                   ids, n, ns, out);                     \
  } while (0)
#define SONG_ENTRY_BY_NS(M, QB)                 \
  switch (NSel) {                               \
    case 1: SONG_ENTRY_LAUNCH(M, QB, 1); break; \
    case 2: SONG_ENTRY_LAUNCH(M, QB, 2); break; \
    case 4: SONG_ENTRY_LAUNCH(M, QB, 4); break; \
    default: SONG_ENTRY_LAUNCH(M, QB, 8); break; \
  }
  switch (metric) {
    case SONG_METRIC_L2: SONG_ENTRY_BY_NS(SONG_METRIC_L2, 2); break;
    case SONG_METRIC_IP: SONG_ENTRY_BY_NS(SONG_METRIC_IP, 2); break;
    default: SONG_ENTRY_BY_NS(SONG_METRIC_COS, 1); break;
  }
#undef SONG_ENTRY_BY_NS
#undef SONG_ENTRY_LAUNCH
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Two-level choice: the probes nearest coarse entries, then the ns nearest
// entries of their clusters.  Both phases score warp tiles of 4 queries x 8
// rows (entry_tiles.cuh: exact search distances) from shared memory.  The
// second phase runs cluster by cluster: the probe lists are inverted into one
// query list per cluster, and a block loads each cluster's rows once for all
// queries probing it.  Each query's per-cluster best lists are then merged.
// ---------------------------------------------------------------------------

// 16-byte global-to-shared copies that complete without holding registers
// (cp.async, waited for by group).
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
  const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// Block shape of the two kernels: `warps` warps (4 queries each), row tiles
// of `rows` rows (a multiple of 8), nbuf tiles in flight.  Wide rows get
// smaller blocks and tiles so that a block fits its shared memory.
struct TileShape {
  int warps, rows, nbuf;
  size_t smem(int dpad) const {
    return sizeof(float) * static_cast<size_t>(dpad) * (4 * warps + static_cast<size_t>(nbuf) * rows);
  }
};

TileShape tile_shape(int dpad) {
  TileShape t{8, 32, 2};
  const size_t budget = 100u * 1024u;
  while (t.smem(dpad) > budget) {
    if (t.nbuf == 2) t.nbuf = 1;
    else if (t.rows > 8) t.rows /= 2;
    else if (t.warps > 1) t.warps /= 2;
    else break;
  }
  return t;
}

// Streams rows [r0, r1) of the row-major block `rows` (dpad floats each)
// through nbuf shared-memory tiles of tile_rows rows (the next tile's copies in
// flight while the current one is scored) and calls score(first_row, n, tile)
// for each; every thread of the block takes part.  Only rows below r1 are
// copied.
template <class F>
__device__ __forceinline__ void stream_rows(const float *rows, int dpad, int r0, int r1, int tile_rows, int nbuf,
                                            float *xb, F &&score) {
  const size_t tile = static_cast<size_t>(dpad) * tile_rows;
  auto issue = [&](int first, float *buf) {
    const int n = min(tile_rows, r1 - first);
    const float4 *src = reinterpret_cast<const float4 *>(rows + static_cast<size_t>(first) * dpad);
    float4 *dst = reinterpret_cast<float4 *>(buf);
    const int n4 = n * (dpad / 4);
    for (int i = threadIdx.x; i < n4; i += blockDim.x) cp_async16(dst + i, src + i);
    cp_async_commit();
  };
  if (nbuf == 2 && r0 < r1) issue(r0, xb);
  for (int first = r0, k = 0; first < r1; first += tile_rows, ++k) {
    float *cur = xb + (nbuf == 2 ? static_cast<size_t>(k & 1) * tile : 0);
    if (nbuf == 2) {
      // the other buffer was last read before the previous iteration's closing barrier
      if (first + tile_rows < r1) {
        issue(first + tile_rows, xb + static_cast<size_t>((k + 1) & 1) * tile);
      } else {
        cp_async_commit();
      }
      cp_async_wait<1>();
    } else {
      issue(first, cur);
      cp_async_wait<0>();
    }
    __syncthreads();  // every thread's copies (and the staged queries) are visible
    score(first, min(tile_rows, r1 - first), cur);
    __syncthreads();
  }
}

// Two-level choice, first kernel: each query's `probes` nearest coarse
// entries (positions in the coarse list, which is sorted by id, so the
// position is the tie order), and the number of probes of each cluster.
// A block takes 4 queries per warp and streams all coarse rows; lane l of a
// warp scores its query l >> 3 against rows l & 7 of each group of 8.
template <int METRIC, int NP>
__global__ void __launch_bounds__(256) heads_tiled_kernel(const float *queries, int nq, int dim, int dpad,
                                                          const float *coarse_rows, int n_coarse, int probes,
                                                          int tile_rows, int nbuf, uint32_t *probe_out,
                                                          uint32_t *cl_count) {
  extern __shared__ __align__(16) float smt[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int bq = 4 * (blockDim.x >> 5);  // queries per block
  const int q0 = blockIdx.x * bq;
  float *qs = smt;
  float *xb = smt + static_cast<size_t>(dpad) * bq;
  for (int i = threadIdx.x; i < bq * dpad; i += blockDim.x) {
    const int r = i / dpad, j = i - r * dpad;
    qs[i] = (q0 + r < nq && j < dim) ? queries[static_cast<size_t>(q0 + r) * dim + j] : 0.0f;
  }
  float pd[NP];
  uint32_t pi[NP];
#pragma unroll
  for (int m = 0; m < NP; ++m) {
    pd[m] = __int_as_float(0x7f800000);
    pi[m] = 0xffffffffu;
  }
  const float *qw = qs + static_cast<size_t>(4 * warp) * dpad;
  stream_rows(coarse_rows, dpad, 0, n_coarse, tile_rows, nbuf, xb, [&](int first, int n, const float *cur) {
    for (int g = 0; g < n; g += 8) {
      const float d = warp_tile_distance<METRIC>(qw, dpad, cur + static_cast<size_t>(g) * dpad, dpad, dpad, lane);
      const int r = g + (lane & 7);
      if (r < n) list_insert<NP>(pd, pi, d, static_cast<uint32_t>(first + r));
    }
  });
  const int q = q0 + 4 * warp + (lane >> 3);
  int h = 0;
  for (int r = 0; r < probes; ++r) {
    float wd;
    uint32_t wid;
    group8_take<NP>(pd, pi, h, wd, wid);
    if (wid >= static_cast<uint32_t>(n_coarse)) wid = 0;  // no finite distance (a query that is not finite)
    if ((lane & 7) == 0 && q < nq) {
      probe_out[static_cast<size_t>(q) * probes + r] = wid;
      atomicAdd(cl_count + wid, 1u);
    }
  }
}

// Exclusive scan of the per-cluster probe counts (one block): offs[0..n],
// and a copy of offs[0..n-1] as the scatter cursors.
// Exclusive block scan of one value per thread (1024 threads); returns this
// thread's exclusive prefix, and the total in *total.
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t s, uint32_t *warp_sum, uint32_t *total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = s;  // inclusive scan within the warp
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  __syncthreads();  // warp_sum may still be read by a previous scan
  if (lane == 31) warp_sum[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = lane < static_cast<int>(blockDim.x >> 5) ? warp_sum[lane] : 0u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    warp_sum[lane] = w;
  }
  __syncthreads();
  *total = warp_sum[(blockDim.x >> 5) - 1];
  return x - s + (warp > 0 ? warp_sum[warp - 1] : 0u);
}

// Exclusive scans of the per-cluster probe counts (one block): offs[0..n],
// a copy of offs[0..n-1] as the scatter cursors, and task_offs[0..n] of the
// clusters' warp tasks (one per 4 of its queries), the clusters taken in the
// order `order` (task_offs[i] belongs to cluster order[i]).
__global__ void __launch_bounds__(1024) cluster_scan_kernel(const uint32_t *count, int n, const uint32_t *order,
                                                            uint32_t *offs, uint32_t *cursor, uint32_t *task_offs) {
  __shared__ uint32_t warp_sum[32];
  const int per = (n + blockDim.x - 1) / blockDim.x;
  const int b = threadIdx.x * per, e = min(n, b + per);
  uint32_t s = 0, st = 0;
  for (int i = b; i < e; ++i) {
    s += count[i];
    st += (count[order[i]] + 3u) / 4u;
  }
  uint32_t total, ttotal;
  uint32_t run = block_exclusive_scan(s, warp_sum, &total);
  uint32_t trun = block_exclusive_scan(st, warp_sum, &ttotal);
  for (int i = b; i < e; ++i) {
    offs[i] = run;
    cursor[i] = run;
    run += count[i];
    if (task_offs) task_offs[i] = trun;
    trun += (count[order[i]] + 3u) / 4u;
  }
  if (threadIdx.x == 0) {
    offs[n] = total;
    if (task_offs) task_offs[n] = ttotal;
  }
}

// Inverts the probe lists: list[cursor[c]++] = q * probes + r for every
// probe r of every query q that names cluster c.
__global__ void cluster_scatter_kernel(const uint32_t *probe, int total, uint32_t *cursor, uint32_t *list) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x)
    list[atomicAdd(cursor + probe[i], 1u)] = static_cast<uint32_t>(i);
}

// Two-level choice, second kernel: block c scores cluster c's entries
// (rows row_offs[c] .. row_offs[c+1] of the cluster-ordered block) against
// every query that probes it, 4 per warp at a time, and writes each
// (query, probe) pair's NS nearest entries, ascending, to part_*.
template <int METRIC, int NS>
__global__ void __launch_bounds__(256) clusters_tiled_kernel(const float *queries, int dim, int dpad,
                                                             const float *fine_rows, const uint32_t *fine_ids,
                                                             const uint32_t *row_offs, const uint32_t *q_offs,
                                                             const uint32_t *q_list, int probes, int tile_rows,
                                                             int nbuf, float *part_d, uint32_t *part_i) {
  extern __shared__ __align__(16) float smt[];
  const int c = blockIdx.x;
  const uint32_t a0 = q_offs[c], a1 = q_offs[c + 1];
  if (a0 == a1) return;  // no query probes this cluster (uniform over the block)
  const int r0 = static_cast<int>(row_offs[c]), r1 = static_cast<int>(row_offs[c + 1]);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int bq = 4 * (blockDim.x >> 5);  // queries per pass
  float *qs = smt;
  float *xb = smt + static_cast<size_t>(dpad) * bq;
  const float *qw = qs + static_cast<size_t>(4 * warp) * dpad;
  for (uint32_t qb = a0; qb < a1; qb += bq) {
    const int nqb = static_cast<int>(min(static_cast<uint32_t>(bq), a1 - qb));
    const bool busy = 4 * warp < nqb;  // warp-uniform
    __syncthreads();  // the previous query tile is no longer read
    for (int i = threadIdx.x; i < bq * dpad; i += blockDim.x) {
      const int r = i / dpad, j = i - r * dpad;
      float v = 0.0f;
      if (r < nqb && j < dim) v = queries[static_cast<size_t>(q_list[qb + r] / probes) * dim + j];
      qs[i] = v;
    }
    float bd[NS];
    uint32_t bi[NS];
#pragma unroll
    for (int m = 0; m < NS; ++m) {
      bd[m] = __int_as_float(0x7f800000);
      bi[m] = 0xffffffffu;
    }
    stream_rows(fine_rows, dpad, r0, r1, tile_rows, nbuf, xb, [&](int first, int n, const float *cur) {
      if (!busy) return;
      for (int g = 0; g < n; g += 8) {
        const float d = warp_tile_distance<METRIC>(qw, dpad, cur + static_cast<size_t>(g) * dpad, dpad, dpad, lane);
        const int r = g + (lane & 7);
        if (r < n) list_insert<NS>(bd, bi, d, fine_ids[first + r]);
      }
    });
    const int slot = 4 * warp + (lane >> 3);
    const uint32_t pair = slot < nqb ? q_list[qb + slot] : 0u;
    int h = 0;
#pragma unroll
    for (int r = 0; r < NS; ++r) {
      float wd;
      uint32_t wid;
      group8_take<NS>(bd, bi, h, wd, wid);
      if ((lane & 7) == 0 && slot < nqb) {
        part_d[static_cast<size_t>(pair) * NS + r] = wd;
        part_i[static_cast<size_t>(pair) * NS + r] = wid;
      }
    }
  }
}

// Two-level choice, second kernel for rows of up to WARP_TASK_DPAD floats:
// warp tasks of (cluster, 4 of the queries that probe it), taken by
// persistent warps (task_offs: the scan's per-cluster task offsets).  A warp
// stages its 4 queries and streams the cluster's rows 8 at a time through a
// double buffer of its own (cp.async; warp barriers only), scores them as a
// warp tile, and writes each (query, probe) pair's NS nearest entries.
constexpr int WARP_TASK_DPAD = 256;
constexpr int WT_WARPS = 4;  // warps per block

size_t warp_task_smem(int dpad) { return sizeof(float) * static_cast<size_t>(dpad) * (4 + 2 * 8) * WT_WARPS; }

template <int METRIC, int NS>
__global__ void __launch_bounds__(WT_WARPS * 32) clusters_warp_kernel(const float *queries, int dim, int dpad,
                                                                      const float *fine_rows,
                                                                      const uint32_t *fine_ids,
                                                                      const uint32_t *row_offs,
                                                                      const uint32_t *q_offs, const uint32_t *q_list,
                                                                      const uint32_t *task_offs,
                                                                      const uint32_t *cl_order, int n_clusters,
                                                                      int probes, float *part_d, uint32_t *part_i) {
  extern __shared__ __align__(16) float smt[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  float *qs = smt + static_cast<size_t>(wib) * dpad * (4 + 16);
  float *xb = qs + static_cast<size_t>(4) * dpad;  // two buffers of 8 rows
  const uint32_t total = task_offs[n_clusters];
  const uint32_t nwarps = gridDim.x * (blockDim.x >> 5);
  const int d4 = dpad / 4;
  for (uint32_t t = blockIdx.x * (blockDim.x >> 5) + wib; t < total; t += nwarps) {
    // the cluster of task t: the last position with task_offs <= t
    int lo = 0, hi = n_clusters - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (task_offs[mid] <= t) lo = mid;
      else hi = mid - 1;
    }
    const int at = lo;
    const int c = static_cast<int>(cl_order[at]);
    const uint32_t qb = q_offs[c] + 4u * (t - task_offs[at]);
    const int nqg = static_cast<int>(min(4u, q_offs[c + 1] - qb));
    const int r0 = static_cast<int>(row_offs[c]), r1 = static_cast<int>(row_offs[c + 1]);
    __syncwarp();  // the previous task's buffers are no longer read
    for (int i = lane; i < 4 * dpad; i += 32) {
      const int a = i / dpad, j = i - a * dpad;
      qs[i] = (a < nqg && j < dim) ? queries[static_cast<size_t>(q_list[qb + a] / probes) * dim + j] : 0.0f;
    }
    float bd[NS];
    uint32_t bi[NS];
#pragma unroll
    for (int m = 0; m < NS; ++m) {
      bd[m] = __int_as_float(0x7f800000);
      bi[m] = 0xffffffffu;
    }
    auto issue = [&](int first, float *buf) {
      const int n4 = min(8, r1 - first) * d4;
      const float4 *src = reinterpret_cast<const float4 *>(fine_rows + static_cast<size_t>(first) * dpad);
      float4 *dst = reinterpret_cast<float4 *>(buf);
      for (int i = lane; i < n4; i += 32) cp_async16(dst + i, src + i);
      cp_async_commit();
    };
    issue(r0, xb);
    for (int first = r0, k = 0; first < r1; first += 8, ++k) {
      float *cur = xb + static_cast<size_t>(k & 1) * 8 * dpad;
      if (first + 8 < r1) {
        issue(first + 8, xb + static_cast<size_t>((k + 1) & 1) * 8 * dpad);
      } else {
        cp_async_commit();
      }
      cp_async_wait<1>();
      __syncwarp();  // every lane's copies (and the staged queries) are visible
      const float d = warp_tile_distance<METRIC>(qs, dpad, cur, dpad, dpad, lane);
      const int r = first + (lane & 7);
      if (r < r1) list_insert<NS>(bd, bi, d, fine_ids[r]);
      __syncwarp();  // this buffer is refilled two rounds on
    }
    const int a = lane >> 3;
    const uint32_t pair = a < nqg ? q_list[qb + a] : 0u;
    int h = 0;
#pragma unroll
    for (int r = 0; r < NS; ++r) {
      float wd;
      uint32_t wid;
      group8_take<NS>(bd, bi, h, wd, wid);
      if ((lane & 7) == 0 && a < nqg) {
        part_d[static_cast<size_t>(pair) * NS + r] = wd;
        part_i[static_cast<size_t>(pair) * NS + r] = wid;
      }
    }
  }
}

// Each query's ns nearest over its probes' lists, ascending by (distance, id).
template <int NS>
__global__ void merge_starts_kernel(const float *part_d, const uint32_t *part_i, int nq, int probes, int ns,
                                    uint32_t *starts) {
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += gridDim.x * blockDim.x) {
    float bd[NS];
    uint32_t bi[NS];
#pragma unroll
    for (int m = 0; m < NS; ++m) {
      bd[m] = __int_as_float(0x7f800000);
      bi[m] = 0xffffffffu;
    }
    const size_t base = static_cast<size_t>(q) * probes * NS;
    for (int i = 0; i < probes * NS; ++i) list_insert<NS>(bd, bi, part_d[base + i], part_i[base + i]);
#pragma unroll
    for (int m = 0; m < NS; ++m)
      if (m < ns) starts[static_cast<size_t>(q) * ns + m] = bi[m];
  }
}

// Raises a kernel's dynamic shared-memory limit.
template <class K>
cudaError_t allow_smem(K kern, size_t bytes) {
  return cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(bytes));
}

// The two-level choice on stream s.  `out` holds nq * (ns + probes) words:
// the starts, then the probed clusters.
cudaError_t launch_2level(song_index *ix, const float *queries, int nq, uint32_t *out, cudaStream_t s) {
  const int dim = ix->dx.dim, dpad = static_cast<int>(ix->dx.f32_row_bytes / 4);
  const int ns = ix->n_starts, np = ix->n_probes, coarse = ix->n_coarse;
  const TileShape ts = tile_shape(dpad);
  const size_t smem = ts.smem(dpad);
  const int bq = 4 * ts.warps;
  const int NSel = ns <= 1 ? 1 : (ns <= 2 ? 2 : (ns <= 4 ? 4 : 8));
  const int NPsel = np <= 1 ? 1 : (np <= 2 ? 2 : (np <= 4 ? 4 : 8));
  uint32_t *probes = out + static_cast<size_t>(nq) * ns;
  // work area: cursors, offsets, inverted lists, per-(query, probe) lists
  const size_t pairs = static_cast<size_t>(nq) * np;
  const size_t need = static_cast<size_t>(coarse) * 3 + 2 + pairs + 2 * pairs * NSel;
  if (need > ix->cap_entry_work) {
    cudaFree(ix->d_entry_work);
    ix->d_entry_work = nullptr;
    ix->cap_entry_work = 0;
    cudaError_t e = song::dev_malloc(&ix->d_entry_work, sizeof(uint32_t) * need);
    if (e != cudaSuccess) return e;
    ix->cap_entry_work = need;
  }
  uint32_t *cursor = ix->d_entry_work;
  uint32_t *q_offs = cursor + coarse;
  uint32_t *q_list = q_offs + coarse + 1;
  float *part_d = reinterpret_cast<float *>(q_list + pairs);
  uint32_t *part_i = q_list + pairs + pairs * NSel;
  uint32_t *task_offs = part_i + pairs * NSel;  // coarse + 1
  cudaError_t e = cudaMemsetAsync(ix->d_cl_count, 0, sizeof(uint32_t) * coarse, s);
  if (e != cudaSuccess) return e;
  const unsigned grid_q = static_cast<unsigned>((nq + bq - 1) / bq);
#define SONG_HEADS(M, NP)                                                                                \
  do {                                                                                                   \
    auto k_ = heads_tiled_kernel<M, NP>;                                                                 \
    if ((e = allow_smem(k_, smem)) != cudaSuccess) return e;                                             \
    k_<<<grid_q, ts.warps * 32, smem, s>>>(queries, nq, dim, dpad, ix->d_coarse_rows, coarse, np, ts.rows, \
                                           ts.nbuf, probes, ix->d_cl_count);                             \
  } while (0)
#define SONG_CLUSTERS(M, NS)                                                                             \
  do {                                                                                                   \
    if (dpad <= WARP_TASK_DPAD) {                                                                        \
      auto w_ = clusters_warp_kernel<M, NS>;                                                             \
      const size_t wsm = warp_task_smem(dpad);                                                           \
      if ((e = allow_smem(w_, wsm)) != cudaSuccess) return e;                                            \
      int per_sm = 0, sms = 0, dev = 0;                                                                  \
      cudaGetDevice(&dev);                                                                               \
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);                                 \
      if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, w_, WT_WARPS * 32, wsm)) != cudaSuccess) \
        return e;                                                                                        \
      w_<<<std::max(1, per_sm) * sms, WT_WARPS * 32, wsm, s>>>(queries, dim, dpad, ix->d_entry_rows,    \
                                                             ix->d_entry_ids, ix->d_offsets, q_offs, q_list, \
                                                             task_offs, ix->d_cl_order, coarse, np, part_d,   \
                                                             part_i);                                   \
      merge_starts_kernel<NS><<<(nq + 255) / 256, 256, 0, s>>>(part_d, part_i, nq, np, ns, out);         \
      break;                                                                                             \
    }                                                                                                    \
    auto k_ = clusters_tiled_kernel<M, NS>;                                                              \
    if ((e = allow_smem(k_, smem)) != cudaSuccess) return e;                                             \
    k_<<<coarse, ts.warps * 32, smem, s>>>(queries, dim, dpad, ix->d_entry_rows, ix->d_entry_ids,         \
                                           ix->d_offsets, q_offs, q_list, np, ts.rows, ts.nbuf, part_d,  \
                                           part_i);                                                      \
    merge_starts_kernel<NS><<<(nq + 255) / 256, 256, 0, s>>>(part_d, part_i, nq, np, ns, out);           \
  } while (0)
#define SONG_HEADS_BY_NP(M)               \
  switch (NPsel) {                        \
    case 1: SONG_HEADS(M, 1); break;      \
    case 2: SONG_HEADS(M, 2); break;      \
    case 4: SONG_HEADS(M, 4); break;      \
    default: SONG_HEADS(M, 8); break;     \
  }
#define SONG_CLUSTERS_BY_NS(M)            \
  switch (NSel) {                         \
    case 1: SONG_CLUSTERS(M, 1); break;   \
    case 2: SONG_CLUSTERS(M, 2); break;   \
    case 4: SONG_CLUSTERS(M, 4); break;   \
    default: SONG_CLUSTERS(M, 8); break;  \
  }
  if (heads_mma_usable(ix, queries, np)) {  // tensor-core scores, exact re-scoring of a shortlist
    if ((e = launch_heads_mma(ix, queries, nq, np, probes, s)) != cudaSuccess) return e;
  } else {
    switch (ix->dx.metric) {
      case SONG_METRIC_L2: SONG_HEADS_BY_NP(SONG_METRIC_L2); break;
      case SONG_METRIC_IP: SONG_HEADS_BY_NP(SONG_METRIC_IP); break;
      default: SONG_HEADS_BY_NP(SONG_METRIC_COS); break;
    }
  }
  cluster_scan_kernel<<<1, 1024, 0, s>>>(ix->d_cl_count, coarse, ix->d_cl_order, q_offs, cursor, task_offs);
  cluster_scatter_kernel<<<static_cast<unsigned>(std::min<size_t>((pairs + 255) / 256, 4096)), 256, 0, s>>>(
      probes, static_cast<int>(pairs), cursor, q_list);
  switch (ix->dx.metric) {
    case SONG_METRIC_L2: SONG_CLUSTERS_BY_NS(SONG_METRIC_L2); break;
    case SONG_METRIC_IP: SONG_CLUSTERS_BY_NS(SONG_METRIC_IP); break;
    default: SONG_CLUSTERS_BY_NS(SONG_METRIC_COS); break;
  }
#undef SONG_CLUSTERS_BY_NS
#undef SONG_HEADS_BY_NP
#undef SONG_CLUSTERS
#undef SONG_HEADS
  return cudaGetLastError();
}

}  // namespace

void clear_entries(song_index *ix) {
  cudaFree(ix->d_entry_ids);
  cudaFree(ix->d_entry_rows);
  cudaFree(ix->d_coarse_rows);
  cudaFree(ix->d_offsets);
  cudaFree(ix->d_cl_count);
  cudaFree(ix->d_cl_order);
  cudaFree(ix->d_entry_work);
  cudaFree(ix->d_head_n2);
  cudaFree(ix->d_head_scores);
  ix->d_head_n2 = nullptr;
  ix->d_head_scores = nullptr;
  ix->cap_head_scores = 0;
  ix->heads_mma = false;
  ix->d_entry_ids = nullptr;
  ix->d_entry_rows = nullptr;
  ix->d_coarse_rows = nullptr;
  ix->d_offsets = nullptr;
  ix->d_cl_count = nullptr;
  ix->d_cl_order = nullptr;
  ix->d_entry_work = nullptr;
  ix->cap_entry_work = 0;
  ix->n_entries = 0;
  ix->n_coarse = 0;
  ix->n_probes = 0;
  ix->n_starts = 1;
}

int prepare_starts(song_index *ix, SearchCall &c, cudaStream_t s) {
  c.starts = nullptr;
  c.n_starts = 1;
  if (ix->n_entries <= 0 || c.nq <= 0) return SONG_OK;
  if (ix->n_starts > c.pq) return fail(SONG_ERR_ARG, "%d start vertices need pq >= %d", ix->n_starts, ix->n_starts);
  // the starts, then (two-level choice) each query's probed clusters
  const size_t need = static_cast<size_t>(c.nq) * (ix->n_starts + (ix->n_coarse > 0 ? ix->n_probes : 0));
  if (need > ix->cap_starts) {
    if (ix->d_starts) cudaFree(ix->d_starts);
    ix->d_starts = nullptr;
    ix->cap_starts = 0;
    cudaError_t e = song::dev_malloc(&ix->d_starts, sizeof(uint32_t) * need);
    if (e != cudaSuccess) return fail(SONG_ERR_OOM, "entry starts: %s", cudaGetErrorString(e));
    ix->cap_starts = need;
  }
  const int dim = ix->dx.dim, dpad = static_cast<int>(ix->dx.f32_row_bytes / 4);
  const cudaError_t le =
      ix->n_coarse > 0 ? launch_2level(ix, c.queries, c.nq, ix->d_starts, s)
                       : launch_nearest(c.queries, c.nq, dim, dim, dpad, ix->dx.metric, ix->d_entry_rows,
                                        ix->d_entry_ids, ix->n_entries, ix->n_starts, ix->d_starts, s);
  if (le != cudaSuccess) return fail(SONG_ERR_CUDA, "entry launch: %s", cudaGetErrorString(le));
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(SONG_ERR_CUDA, "entry launch: %s", cudaGetErrorString(e));
  c.starts = ix->d_starts;
  c.n_starts = ix->n_starts;
  return SONG_OK;
}

}  // namespace song

extern "C" int song_index_set_entries(song_index *ix, const uint64_t *ids, int count, int starts) {
  using namespace song;
  clear_error();
  if (!ix) return fail(SONG_ERR_ARG, "null index");
  if (count < 0 || count > SONG_MAX_ENTRIES) return fail(SONG_ERR_ARG, "entry count must be 0..%d", SONG_MAX_ENTRIES);
  if (count > 0 && (starts < 1 || starts > SONG_MAX_STARTS || starts > count))
    return fail(SONG_ERR_ARG, "starts must be 1..min(%d, entry count)", SONG_MAX_STARTS);
  if (count > 0 && !ids) return fail(SONG_ERR_ARG, "null entry ids");
  std::vector<uint32_t> h(static_cast<size_t>(count));
  for (int i = 0; i < count; ++i) {
    if (ids[i] >= ix->dx.n) return fail(SONG_ERR_ARG, "entry %d: id %llu >= n", i, (unsigned long long)ids[i]);
    h[i] = static_cast<uint32_t>(ids[i]);
  }
  {
    std::vector<uint32_t> u(h);
    std::sort(u.begin(), u.end());
    if (std::adjacent_find(u.begin(), u.end()) != u.end()) return fail(SONG_ERR_ARG, "entry ids must be distinct");
  }
  if (ix->servers > 0) return fail(SONG_ERR_ARG, "entries are in use by %d server(s)", ix->servers);
  DeviceGuard guard(ix->device);
  if (!guard.ok) return fail(SONG_ERR_CUDA, "cannot select device %d", ix->device);
  cudaError_t e = cudaSuccess;
  clear_entries(ix);
  if (count == 0) return SONG_OK;
  const int dpad = static_cast<int>(ix->dx.f32_row_bytes / 4);
  e = song::dev_malloc(&ix->d_entry_ids, sizeof(uint32_t) * count);
  if (e == cudaSuccess) e = song::dev_malloc(&ix->d_entry_rows, sizeof(float) * count * static_cast<size_t>(dpad));
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(ix->d_entry_ids, h.data(), sizeof(uint32_t) * count, cudaMemcpyHostToDevice, ix->stream);
  if (e == cudaSuccess) {
    gather_entry_rows_kernel<<<256, 256, 0, ix->stream>>>(ix->dx.rows_f32, static_cast<uint32_t>(dpad),
                                                          ix->d_entry_ids, count, dpad, ix->d_entry_rows);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(ix->stream);
  if (e != cudaSuccess) {
    cudaFree(ix->d_entry_ids);
    cudaFree(ix->d_entry_rows);
    ix->d_entry_ids = nullptr;
    ix->d_entry_rows = nullptr;
    return fail(e == cudaErrorMemoryAllocation ? SONG_ERR_OOM : SONG_ERR_CUDA, "entries: %s", cudaGetErrorString(e));
  }
  ix->n_entries = count;
  ix->n_starts = starts;
  return SONG_OK;
}

extern "C" int song_index_set_entries_2level(song_index *ix, const uint64_t *ids, int count, int coarse, int probes,
                                             int starts) {
  using namespace song;
  clear_error();
  if (!ix) return fail(SONG_ERR_ARG, "null index");
  if (count < 1 || count > SONG_MAX_ENTRIES_2LEVEL || !ids)
    return fail(SONG_ERR_ARG, "entry count must be 1..%d", SONG_MAX_ENTRIES_2LEVEL);
  if (coarse < 1 || coarse > count || coarse > SONG_MAX_COARSE)
    return fail(SONG_ERR_ARG, "coarse must be 1..min(count, %d)", SONG_MAX_COARSE);
  if (probes < 1 || probes > SONG_MAX_STARTS || probes > coarse)
    return fail(SONG_ERR_ARG, "probes must be 1..min(%d, coarse)", SONG_MAX_STARTS);
  if (starts < 1 || starts > probes) return fail(SONG_ERR_ARG, "starts must be 1..probes");
  const int dim = ix->dx.dim, dpad = static_cast<int>(ix->dx.f32_row_bytes / 4);
  // the smallest block shape (one warp, 4 queries, one tile of 8 rows) fits
  // a block's shared memory
  auto fits = [](int dp) { return TileShape{1, 8, 1}.smem(dp) <= 227u * 1024u; };
  if (!fits(dpad)) {
    int widest = 4;
    while (fits(widest + 4)) widest += 4;
    return fail(SONG_ERR_ARG, "two-level entries support rows of up to %d floats", widest);
  }
  std::vector<uint32_t> h(static_cast<size_t>(count));
  for (int i = 0; i < count; ++i) {
    if (ids[i] >= ix->dx.n) return fail(SONG_ERR_ARG, "entry %d: id %llu >= n", i, (unsigned long long)ids[i]);
    h[i] = static_cast<uint32_t>(ids[i]);
  }
  {
    std::vector<uint32_t> u(h);
    std::sort(u.begin(), u.end());
    if (std::adjacent_find(u.begin(), u.end()) != u.end()) return fail(SONG_ERR_ARG, "entry ids must be distinct");
  }
  if (ix->servers > 0) return fail(SONG_ERR_ARG, "entries are in use by %d server(s)", ix->servers);
  DeviceGuard guard(ix->device);
  if (!guard.ok) return fail(SONG_ERR_CUDA, "cannot select device %d", ix->device);
  cudaError_t e = cudaSuccess;
  clear_entries(ix);
  // 1. all entry rows in list order; the clusters of the non-coarse entries
  uint32_t *d_ids = nullptr, *d_assign = nullptr, *d_perm = nullptr;
  float *d_rows = nullptr;
  std::vector<uint32_t> assign(static_cast<size_t>(count - coarse));
  e = song::dev_malloc(&d_ids, sizeof(uint32_t) * count);
  if (e == cudaSuccess) e = song::dev_malloc(&d_rows, sizeof(float) * static_cast<size_t>(count) * dpad);
  if (e == cudaSuccess && count > coarse) e = song::dev_malloc(&d_assign, sizeof(uint32_t) * (count - coarse));
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_ids, h.data(), sizeof(uint32_t) * count, cudaMemcpyHostToDevice, ix->stream);
  if (e == cudaSuccess) {
    gather_entry_rows_kernel<<<256, 256, 0, ix->stream>>>(ix->dx.rows_f32, static_cast<uint32_t>(dpad), d_ids, count,
                                                          dpad, d_rows);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && count > coarse)
    e = launch_nearest(d_rows + static_cast<size_t>(coarse) * dpad, count - coarse, dpad, dim, dpad, ix->dx.metric,
                       d_rows, d_ids, coarse, 1, d_assign, ix->stream);
  if (e == cudaSuccess && count > coarse)
    e = cudaMemcpyAsync(assign.data(), d_assign, sizeof(uint32_t) * (count - coarse), cudaMemcpyDeviceToHost,
                        ix->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ix->stream);
  // 2. clusters numbered by coarse id; entries ordered by cluster
  std::vector<int> corder(static_cast<size_t>(coarse));
  for (int i = 0; i < coarse; ++i) corder[i] = i;
  std::sort(corder.begin(), corder.end(), [&](int a, int b) { return h[a] < h[b]; });
  std::vector<uint32_t> cl_of_id_sorted(static_cast<size_t>(coarse));  // sorted coarse ids
  std::vector<int> rank(static_cast<size_t>(coarse));
  for (int k = 0; k < coarse; ++k) {
    rank[corder[k]] = k;
    cl_of_id_sorted[k] = h[corder[k]];
  }
  std::vector<uint32_t> cluster(static_cast<size_t>(count));
  for (int f = 0; f < count && e == cudaSuccess; ++f) {
    if (f < coarse) {
      cluster[f] = static_cast<uint32_t>(rank[f]);
    } else {
      const auto it = std::lower_bound(cl_of_id_sorted.begin(), cl_of_id_sorted.end(), assign[f - coarse]);
      cluster[f] = static_cast<uint32_t>(it - cl_of_id_sorted.begin());
    }
  }
  std::vector<uint32_t> offsets(static_cast<size_t>(coarse) + 1, 0u), perm(static_cast<size_t>(count)),
      fine_ids(static_cast<size_t>(count)), cperm(static_cast<size_t>(coarse));
  for (int f = 0; f < count; ++f) ++offsets[cluster[f] + 1];
  for (int k = 0; k < coarse; ++k) offsets[k + 1] += offsets[k];
  {
    std::vector<uint32_t> fill(offsets.begin(), offsets.end() - 1);
    for (int f = 0; f < count; ++f) {
      const uint32_t pos = fill[cluster[f]]++;
      perm[pos] = static_cast<uint32_t>(f);  // row f of d_rows
      fine_ids[pos] = h[f];
    }
  }
  for (int k = 0; k < coarse; ++k) cperm[k] = static_cast<uint32_t>(corder[k]);
  // the clusters largest first: the cluster phase's warps take tasks in this
  // order, so that the long tasks start first and the last ones are short
  std::vector<uint32_t> by_size(static_cast<size_t>(coarse));
  for (int k = 0; k < coarse; ++k) by_size[k] = static_cast<uint32_t>(k);
  std::stable_sort(by_size.begin(), by_size.end(), [&](uint32_t a, uint32_t b) {
    return offsets[a + 1] - offsets[a] > offsets[b + 1] - offsets[b];
  });
  // 3. device copies: entries in cluster order, coarse rows by id, offsets
  uint32_t *d_cperm = nullptr;
  if (e == cudaSuccess) e = song::dev_malloc(&d_perm, sizeof(uint32_t) * count);
  if (e == cudaSuccess) e = song::dev_malloc(&d_cperm, sizeof(uint32_t) * coarse);
  if (e == cudaSuccess) e = song::dev_malloc(&ix->d_entry_rows, sizeof(float) * static_cast<size_t>(count) * dpad);
  if (e == cudaSuccess) e = song::dev_malloc(&ix->d_entry_ids, sizeof(uint32_t) * count);
  if (e == cudaSuccess) e = song::dev_malloc(&ix->d_coarse_rows, sizeof(float) * static_cast<size_t>(coarse) * dpad);
  if (e == cudaSuccess) e = song::dev_malloc(&ix->d_offsets, sizeof(uint32_t) * (coarse + 1));
  if (e == cudaSuccess) e = song::dev_malloc(&ix->d_cl_order, sizeof(uint32_t) * coarse);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(ix->d_cl_order, by_size.data(), sizeof(uint32_t) * coarse, cudaMemcpyHostToDevice, ix->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_perm, perm.data(), sizeof(uint32_t) * count, cudaMemcpyHostToDevice, ix->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_cperm, cperm.data(), sizeof(uint32_t) * coarse, cudaMemcpyHostToDevice, ix->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(ix->d_entry_ids, fine_ids.data(), sizeof(uint32_t) * count, cudaMemcpyHostToDevice, ix->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(ix->d_offsets, offsets.data(), sizeof(uint32_t) * (coarse + 1), cudaMemcpyHostToDevice,
                        ix->stream);
  if (e == cudaSuccess) {
    gather_entry_rows_kernel<<<256, 256, 0, ix->stream>>>(d_rows, static_cast<uint32_t>(dpad), d_perm, count, dpad,
                                                          ix->d_entry_rows);
    gather_entry_rows_kernel<<<64, 256, 0, ix->stream>>>(d_rows, static_cast<uint32_t>(dpad), d_cperm, coarse, dpad,
                                                         ix->d_coarse_rows);
    e = cudaGetLastError();
  }
  // 4. the per-cluster probe counters of the second kernel; the head rows'
  // tensor map and norms (the tensor-core head phase; without them the
  // CUDA-core kernel scores the heads)
  if (e == cudaSuccess) e = song::dev_malloc(&ix->d_cl_count, sizeof(uint32_t) * coarse);
  if (e == cudaSuccess) song::heads_mma_prepare(ix, coarse);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ix->stream);
  cudaFree(d_ids);
  cudaFree(d_rows);
  cudaFree(d_assign);
  cudaFree(d_perm);
  cudaFree(d_cperm);
  if (e != cudaSuccess) {
    clear_entries(ix);
    return fail(e == cudaErrorMemoryAllocation ? SONG_ERR_OOM : SONG_ERR_CUDA, "entries: %s", cudaGetErrorString(e));
  }
  ix->n_entries = count;
  ix->n_coarse = coarse;
  ix->n_probes = probes;
  ix->n_starts = starts;
  return SONG_OK;
}
