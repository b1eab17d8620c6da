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
// rows are copied once into a contiguous block, which stays in L2.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <vector>

#include "internal.h"
#include "song_gb300.h"

namespace song {
namespace {

__device__ __forceinline__ bool closer(float d, uint32_t id, float bd, uint32_t bid) {
  return d < bd || (d == bd && id < bid);
}

// One warp serves QB queries; lane e takes entries e, e+32, ... and reads
// each entry row once, in 16-byte pieces, for all QB queries.  Rows and the
// staged queries are zero-padded to dpad (a multiple of 4) floats: a padded
// element adds fma(0, 0, t) = t, leaving every partial sum exactly as the
// search leaves it.  Each lane keeps its NS nearest entries per query in a
// sorted register list; the warp then merges the lists, ns rounds of an xor
// argmin, into starts[q*ns ..], ascending by (distance, id).
template <int METRIC, int QB, int NS>
__global__ void __launch_bounds__(256) nearest_entry_kernel(const float *queries, int nq, int dim, int dpad,
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
      qw[b * dpad + j] = (q0 + b < nq && j < dim) ? queries[static_cast<size_t>(q0 + b) * dim + j] : 0.0f;
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
__global__ void __launch_bounds__(256) nearest_entry_tiled_kernel(const float *queries, int nq, int dim, int dpad,
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
      qw[b * dpad + j] = (q0 + b < nq && j < dim) ? queries[static_cast<size_t>(q0 + b) * dim + j] : 0.0f;
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

}  // namespace

int prepare_starts(song_index *ix, SearchCall &c, cudaStream_t s) {
  c.starts = nullptr;
  c.n_starts = 1;
  if (ix->n_entries <= 0 || c.nq <= 0) return SONG_OK;
  if (ix->n_starts > c.pq) return fail(SONG_ERR_ARG, "%d start vertices need pq >= %d", ix->n_starts, ix->n_starts);
  const size_t need = static_cast<size_t>(c.nq) * ix->n_starts;
  if (need > ix->cap_starts) {
    if (ix->d_starts) cudaFree(ix->d_starts);
    ix->d_starts = nullptr;
    ix->cap_starts = 0;
    cudaError_t e = cudaMalloc(&ix->d_starts, sizeof(uint32_t) * need);
    if (e != cudaSuccess) return fail(SONG_ERR_OOM, "entry starts: %s", cudaGetErrorString(e));
    ix->cap_starts = need;
  }
  const int dim = ix->dx.dim, dpad = static_cast<int>(ix->dx.f32_row_bytes / 4);
  // warps per block: up to 8, within the default 48 KB of shared memory;
  // rows of up to 1 KB are staged through shared memory in 32-row tiles
  const int qb = ix->dx.metric == SONG_METRIC_COS ? 1 : 2;
  const int per_warp = static_cast<int>(sizeof(float)) * dpad * qb;
  const int tile_bytes = 32 * (dpad / 4 + 1) * 16;
  const bool tiled = dpad * 4 <= 1024 && tile_bytes + per_warp <= 48 * 1024;
  const int avail = 48 * 1024 - (tiled ? tile_bytes : 0);
  const int wpb = std::max(1, std::min(8, avail / per_warp));
  const size_t smem = static_cast<size_t>(per_warp) * wpb + (tiled ? tile_bytes : 0);
  const unsigned grid = static_cast<unsigned>((c.nq + wpb * qb - 1) / (wpb * qb));
  const int ns = ix->n_starts;
  const int NSel = ns <= 1 ? 1 : (ns <= 2 ? 2 : (ns <= 4 ? 4 : 8));
#define SONG_ENTRY_LAUNCH(M, QB, NS)                                                                        \
  do {                                                                                                   \
    if (tiled)                                                                                           \
      nearest_entry_tiled_kernel<M, QB, NS><<<grid, 32 * wpb, smem, s>>>(                                \
          c.queries, c.nq, dim, dpad, ix->d_entry_rows, ix->d_entry_ids, ix->n_entries, ns, ix->d_starts); \
    else                                                                                                 \
      nearest_entry_kernel<M, QB, NS><<<grid, 32 * wpb, smem, s>>>(                                      \
          c.queries, c.nq, dim, dpad, ix->d_entry_rows, ix->d_entry_ids, ix->n_entries, ns, ix->d_starts); \
  } while (0)
#define SONG_ENTRY_BY_NS(M, QB)              \
  switch (NSel) {                            \
    case 1: SONG_ENTRY_LAUNCH(M, QB, 1); break; \
    case 2: SONG_ENTRY_LAUNCH(M, QB, 2); break; \
    case 4: SONG_ENTRY_LAUNCH(M, QB, 4); break; \
    default: SONG_ENTRY_LAUNCH(M, QB, 8); break; \
  }
  switch (ix->dx.metric) {
    case SONG_METRIC_L2: SONG_ENTRY_BY_NS(SONG_METRIC_L2, 2); break;
    case SONG_METRIC_IP: SONG_ENTRY_BY_NS(SONG_METRIC_IP, 2); break;
    default: SONG_ENTRY_BY_NS(SONG_METRIC_COS, 1); break;
  }
#undef SONG_ENTRY_BY_NS
#undef SONG_ENTRY_LAUNCH
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
  cudaError_t e = cudaSetDevice(ix->device);
  if (e != cudaSuccess) return fail(SONG_ERR_CUDA, "cannot select device %d", ix->device);
  cudaFree(ix->d_entry_ids);
  cudaFree(ix->d_entry_rows);
  ix->d_entry_ids = nullptr;
  ix->d_entry_rows = nullptr;
  ix->n_entries = 0;
  if (count == 0) return SONG_OK;
  const int dpad = static_cast<int>(ix->dx.f32_row_bytes / 4);
  e = cudaMalloc(&ix->d_entry_ids, sizeof(uint32_t) * count);
  if (e == cudaSuccess) e = cudaMalloc(&ix->d_entry_rows, sizeof(float) * count * static_cast<size_t>(dpad));
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
