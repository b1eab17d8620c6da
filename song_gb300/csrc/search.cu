// search.cu -- host side of the search kernel: shared-memory layout, launch
// shape, and dispatch to the per-storage translation units
// (search_f32.cu, search_bf16.cu, search_fp8.cu, search_learned.cu).  The
// kernel itself is in search_kernel.cuh.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <mutex>
#include <vector>

#include "search_kernel.cuh"

namespace song {

__global__ void debug_fixhash_kernel(const uint32_t *ids, int count, int cap, uint64_t magic,
                                     int32_t *out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  VisitedHash vh{nullptr, cap, magic};
  if (i < count) out[i] = vh.slot(ids[i]);
}

namespace {

uint32_t align_up(uint32_t x, uint32_t a) { return (x + a - 1) / a * a; }

// Rows staged per buffer half: a typical hop evaluates 2-5 neighbours.
// Rows per staging chunk (two chunks in flight).  Rows of up to 1 KB: 4 while
// pq is small (many new candidates per hop), 1 from pq 512 on, where a hop
// brings ~2 new candidates and the smaller staging ring leaves room for one
// more resident warp next to the 8*pq-slot visited hash (measured: 1M x 128,
// pq 800: 39.0 -> 35.7 ms; pq 200: 12.6 ms with 4 rows, 14.6 ms with 1).
int stage_rows(uint32_t row_bytes, int pq) { return row_bytes <= 1024 ? (pq >= 512 ? 1 : 4) : 2; }

// Register-queue segment: smallest power of two S with 32*S >= pq + 1.
int queue_segment(int pq) {
  int s = 1;
  while (32 * s < pq + 1) s <<= 1;
  return s;
}

struct Layout {
  uint32_t warp_bytes, off_mbar, off_cand, off_q, off_hash;
  int cap, H, S;
};

// FixHash capacity 8*pq (the reference's TOPK*4*2) for the plain kernel; the
// learned kernel's exact set: the power of two >= max(32, 4*pq).
int exact_cap(int pq) {
  int c = 32;
  while (c < 4 * pq) c <<= 1;
  return c;
}

Layout make_layout(const DeviceIndex &ix, int pq, bool learned, bool multi = false) {
  Layout L;
  L.H = stage_rows(ix.row_bytes, pq);
  L.S = queue_segment(pq);
  L.cap = learned ? exact_cap(pq) : 8 * pq;
  uint32_t off = 2u * L.H * ix.row_bytes;
  off = align_up(off, 16);
  L.off_mbar = off;
  off += 16;
  L.off_cand = off;
  off += (multi ? MAX_PROBES : 1) * 32 * 4;
  off = align_up(off, 16);
  L.off_q = off;
  off += align_up(static_cast<uint32_t>(ix.dim) * 4u, 16);
  L.off_hash = off;
  off += 4u * L.cap;
  L.warp_bytes = align_up(off, 128);
  return L;
}

struct Shape {
  const void *fn;
  int dev;
  uint32_t warp_bytes, extra;
  int wpb, blocks_per_sm, sms;
};

std::mutex g_shape_mu;
std::vector<Shape> g_shapes;

}  // namespace

int get_shape(const void *fn, uint32_t warp_bytes, uint32_t extra, int *wpb, int *grid_cap) {
  std::lock_guard<std::mutex> lk(g_shape_mu);
  int dev = 0;
  cudaGetDevice(&dev);
  for (const Shape &s : g_shapes)
    if (s.fn == fn && s.dev == dev && s.warp_bytes == warp_bytes && s.extra == extra) {
      *wpb = s.wpb;
      *grid_cap = s.blocks_per_sm * s.sms;
      return 0;
    }
  int sms = 0, optin = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  // One kernel serves indexes and pq values of different footprints, so its
  // dynamic shared-memory limit is raised once to the device maximum rather
  // than to the size of any one launch.
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
  if (e != cudaSuccess) return e;
  Shape best{fn, dev, warp_bytes, extra, 0, 0, sms};
  for (int w = MAX_WARPS_PER_BLOCK; w >= 1; w >>= 1) {
    const size_t smem = static_cast<size_t>(warp_bytes) * w + extra;
    if (smem > static_cast<size_t>(optin)) continue;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, w * 32, smem);
    if (e != cudaSuccess) return e;
    if (per_sm * w > best.blocks_per_sm * best.wpb) {
      best.wpb = w;
      best.blocks_per_sm = per_sm;
    }
  }
  if (best.wpb == 0) return -1;
  g_shapes.push_back(best);
  *wpb = best.wpb;
  *grid_cap = best.blocks_per_sm * best.sms;
  return 0;
}

uint32_t search_warp_bytes(const DeviceIndex &ix, int pq, bool multi) {
  return make_layout(ix, pq, false, multi).warp_bytes;
}

int launch_search(const DeviceIndex &ix, const SearchCall &c, cudaStream_t stream) {
  if (c.nq <= 0) return 0;
  const bool learned = c.mlp != nullptr || c.trace != nullptr || c.exit_max_hops > 0;
  const bool multi = c.probes > 1 || c.finish_cnt > 1 || c.double_check;
  if (multi && (learned || ix.storage != 0 || c.probes > MAX_PROBES || c.finish_cnt < 1)) return -1;
  const Layout L = make_layout(ix, c.pq, learned, multi);
  Params p;
  p.rows = static_cast<const uint8_t *>(ix.rows);
  p.row_bytes = ix.row_bytes;
  p.scale_off = ix.scale_off;
  p.rows_f32 = ix.rows_f32;
  p.f32_row_bytes = ix.f32_row_bytes;
  p.rerank = ix.storage == 0 ? 0 : c.rerank;
  p.adj = ix.adj;
  p.shift = ix.shift;
  p.dim = ix.dim;
  p.queries = c.queries;
  p.nq = c.nq;
  p.pq = c.pq;
  p.k = c.k;
  p.out = c.out;
  p.hops = c.hops;
  p.evals = c.evals;
  p.counter = c.counter;
  p.error = c.error;
  p.warp_bytes = L.warp_bytes;
  p.off_mbar = L.off_mbar;
  p.off_cand = L.off_cand;
  p.off_q = L.off_q;
  p.off_hash = L.off_hash;
  p.cap = L.cap;
  p.magic = ~0ull / static_cast<uint64_t>(L.cap);
  p.log2cap = 0;
  while ((1 << p.log2cap) < L.cap) ++p.log2cap;
  p.mlp = c.mlp;
  p.exit_threshold = c.exit_threshold;
  p.exit_min_hops = c.exit_min_hops;
  p.exit_every = c.exit_every > 0 ? c.exit_every : 1;
  p.exit_max_hops = c.exit_max_hops;
  p.trace = c.trace;
  p.trace_hops = c.trace_hops;
  p.trace_final = c.trace_final;
  p.starts = c.starts;
  p.n_starts = c.starts ? c.n_starts : 1;
  p.qcodes = c.qcodes;
  p.wait_limit = c.wait_limit;
  p.extra_tx = c.extra_tx;
  p.probes = c.probes;
  p.finish_cnt = c.finish_cnt;
  p.double_check = c.double_check;
  if (multi) return launch_multi(p, ix.metric, L.H, L.S, stream);
  if (learned) {
    if (ix.storage >= 2) return -1;
    return launch_learned(p, ix.storage, ix.metric, L.H, L.S, stream);
  }
  switch (ix.storage) {
    case 0: return launch_f32(p, ix.metric, L.H, L.S, stream);
    case 1: return launch_bf16(p, ix.metric, L.H, L.S, stream);
    case 2: return launch_fp8(p, ix.metric, L.H, L.S, stream);
    case 3: return c.qcodes ? launch_bits(p, ix.metric, L.S, stream) : -1;  // query codes come from the caller's path
    default: return -1;
  }
}

int launch_debug_fixhash(const uint32_t *ids, int count, int pq, int32_t *out, cudaStream_t s) {
  if (count <= 0) return 0;
  const int cap = 8 * pq;
  debug_fixhash_kernel<<<(count + 255) / 256, 256, 0, s>>>(ids, count, cap,
                                                           ~0ull / static_cast<uint64_t>(cap), out);
  return cudaGetLastError();
}

}  // namespace song
