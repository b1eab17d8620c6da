// search.cu -- the batched best-first graph search kernel for sm_103a.
//
// It computes what warp_independent_search_kernel computes
// (warp_astar_accelerator.h:41-341): for each query, a best-first walk from
// vertex 0 over the fixed-degree graph with a candidate queue bounded at pq,
// a top-pq list of expanded vertices, a visited hash over queue and list, the
// select-insert rule (skip a candidate when the queue is full and its maximum
// is closer) and the finish rule (stop when the list is full and its maximum
// is <= the vertex just popped).  Distances are FP32 with the reference's
// summation order: lane l sums dims l, l+32, ... with fused multiply-add and
// the 32 partial sums meet in the xor butterfly 16, 8, 4, 2, 1.
//
// What is different, for GB300:
//  * persistent warps: a grid sized to fill the 152 SMs pulls queries from a
//    work counter, one query per warp at a time; warps never synchronise with
//    one another;
//  * all per-query state lives in the warp's slice of shared memory instead
//    of device-heap allocations: query vector, candidate queue, top-pq list,
//    visited hash, staging ring;
//  * the neighbour rows of a hop are gathered with 1-D bulk async copies
//    (cp.async.bulk + mbarrier transaction counts) into a two-buffer ring,
//    so the rows of the next chunk are in flight while the current chunk's
//    distances are computed; the whole warp then reads them from shared
//    memory in the reference's lane order;
//  * the neighbour scan reads the adjacency row with one coalesced load and
//    tests all neighbours against the visited hash at once, one lane each;
//  * queue and list are sorted arrays of (distance, id) keys updated by the
//    whole warp (ballot search + shifted window), which replaces the serial
//    min-max heap (smmh2.h) and binary heap (bin_heap.h); equal distances
//    leave in id order, where the reference's heaps leave them in an order
//    that depends on their shape.  Nothing else differs, and the visited
//    hash sees the reference's exact sequence of add/delete operations.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <mutex>
#include <vector>

#include "device_common.cuh"
#include "internal.h"
#include "reg_queue.cuh"

namespace song {

constexpr int MAX_WARPS_PER_BLOCK = 4;

struct Params {
  const uint8_t *rows;
  uint32_t row_bytes;
  const float *row_scale;
  const uint32_t *adj;
  int shift;
  int dim;
  const float *queries;
  int nq, pq, k;
  uint64_t *out;
  int32_t *hops;
  int32_t *evals;
  uint32_t *counter;
  int32_t *error;
  uint32_t warp_bytes;
  uint32_t off_mbar, off_cand, off_q, off_hash;
  int cap;
  uint64_t magic;
};

template <int METRIC>
__device__ __forceinline__ float finish_distance(float t, float len) {
  if (METRIC == 0) return t;
  if (METRIC == 1) return -t;
  // warp_astar_accelerator.h:275-281: sign * tmp * tmp / len in float.
  if (len != 0.0f) {
    float sign = t < 0.0f ? 1.0f : -1.0f;
    return __fdiv_rn(__fmul_rn(__fmul_rn(sign, t), t), len);
  }
  return 0.0f;
}

// Distances of candidates 0..m-1 (candidate c's id in lane c); candidate c's
// distance is returned in lane c.  False if a bulk copy never completed.
template <int METRIC, int H>
__device__ __forceinline__ bool gather_distances(const Params &p, uint8_t *stage, uint64_t *mbar,
                                                 uint32_t &ph0, uint32_t &ph1, const float *qv,
                                                 int m, uint32_t cid, float &out, int lane) {
  const int nchunks = (m + H - 1) / H;
  const uint32_t rb = p.row_bytes;
  auto issue = [&](int c) {
    const int b = c & 1;
    const int first = c * H;
    const int cnt = min(H, m - first);
    // The buffer was last read through the generic proxy; order those reads
    // before the async-proxy writes of the copies issued below.
    fence_proxy_async();
    if (lane == 0) mbar_arrive_expect_tx(&mbar[b], static_cast<uint32_t>(cnt) * rb);
    __syncwarp();
    const uint32_t id = __shfl_sync(FULL, cid, (first + lane) & 31);
    if (lane < cnt)
      bulk_g2s(stage + static_cast<size_t>(b * H + lane) * rb,
               p.rows + static_cast<uint64_t>(id) * rb, rb, &mbar[b]);
  };
  if (nchunks > 0) issue(0);
  if (nchunks > 1) issue(1);
  out = 0.0f;
  for (int c = 0; c < nchunks; ++c) {
    const int b = c & 1;
    uint32_t &ph = b ? ph1 : ph0;
    if (!mbar_wait(&mbar[b], ph)) return false;
    ph ^= 1u;
    const int first = c * H;
    const int cnt = min(H, m - first);
    const uint8_t *buf = stage + static_cast<size_t>(b * H) * rb;
    float acc[H], len[H];
#pragma unroll
    for (int i = 0; i < H; ++i) {
      acc[i] = 0.0f;
      len[i] = 0.0f;
      if (i < cnt) {
        const float *x = reinterpret_cast<const float *>(buf + static_cast<size_t>(i) * rb);
        for (int j = lane; j < p.dim; j += 32) {
          const float qj = qv[j];
          const float xj = x[j];
          if (METRIC == 0) {
            const float d = __fsub_rn(qj, xj);
            acc[i] = __fmaf_rn(d, d, acc[i]);
          } else {
            acc[i] = __fmaf_rn(qj, xj, acc[i]);
            if (METRIC == 2) len[i] = __fmaf_rn(xj, xj, len[i]);
          }
        }
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
      for (int i = 0; i < H; ++i) {
        acc[i] = __fadd_rn(acc[i], __shfl_xor_sync(FULL, acc[i], o));
        if (METRIC == 2) len[i] = __fadd_rn(len[i], __shfl_xor_sync(FULL, len[i], o));
      }
    }
#pragma unroll
    for (int i = 0; i < H; ++i)
      if (i < cnt && lane == first + i) out = finish_distance<METRIC>(acc[i], len[i]);
    __syncwarp();
    if (c + 2 < nchunks) issue(c + 2);
  }
  return true;
}

__device__ __forceinline__ uint64_t warp_min_u64(uint64_t x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const uint64_t y = __shfl_xor_sync(FULL, x, o);
    x = y < x ? y : x;
  }
  return x;
}

template <int METRIC, int H, int S>
__global__ void __launch_bounds__(MAX_WARPS_PER_BLOCK * 32, 1)
    search_kernel(const Params p) {
  extern __shared__ __align__(128) uint8_t smem_raw[];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  uint8_t *ws = smem_raw + static_cast<size_t>(wib) * p.warp_bytes;
  uint8_t *stage = ws;
  uint64_t *mbar = reinterpret_cast<uint64_t *>(ws + p.off_mbar);
  uint32_t *cbuf = reinterpret_cast<uint32_t *>(ws + p.off_cand);
  float *qv = reinterpret_cast<float *>(ws + p.off_q);
  VisitedHash vh{reinterpret_cast<int32_t *>(ws + p.off_hash), p.cap, p.magic};
  RegQueue<S> Q, T;  // candidate queue and top-pq list, ascending (distance, id)

  if (lane == 0) {
    mbar_init(&mbar[0], 1);
    mbar_init(&mbar[1], 1);
    fence_mbar_init();
  }
  __syncwarp();
  uint32_t ph0 = 0, ph1 = 0;
  const int nslots = 1 << p.shift;

  for (;;) {
    uint32_t qid = 0;
    if (lane == 0) qid = atomicAdd(p.counter, 1u);
    qid = __shfl_sync(FULL, qid, 0);
    if (qid >= static_cast<uint32_t>(p.nq)) break;

    const float *qsrc = p.queries + static_cast<size_t>(qid) * p.dim;
    for (int j = lane; j < p.dim; j += 32) qv[j] = qsrc[j];
    vh.clear(lane);
    // Adjacency row of vertex 0, the first vertex popped.
    uint32_t next_id = 0;
    uint32_t a_next = lane < nslots ? __ldg(p.adj + lane) : 0u;

    // warp_astar_accelerator.h:115-176: distance to vertex 0, queue = {0}.
    float cd;
    if (!gather_distances<METRIC, H>(p, stage, mbar, ph0, ph1, qv, 1, 0u, cd, lane)) {
      if (lane == 0) atomicOr(p.error, 1);
      return;
    }
    int qn = 0, tn = 0;
    Q.clear();
    T.clear();
    Q.insert(make_key(__shfl_sync(FULL, cd, 0), 0u), qn, lane);
    vh.add(0u, lane);
    int hops = 0, evals = 1;

    while (qn > 0) {
      // :186-193 pop the minimum, drop it from the visited hash.
      const uint64_t now = Q.get(0);
      Q.pop_front(lane);
      --qn;
      const uint32_t now_id = key_id(now);
      uint32_t a = a_next;
      if (now_id != next_id)  // not taken: the prefetch predicts the pop exactly
        a = lane < nslots ? __ldg(p.adj + (static_cast<uint64_t>(now_id) << p.shift) + lane) : 0u;
      vh.del(now_id, lane);
      // :191 finish test (<=) against the list maximum.
      if (tn == p.pq && key_dist(T.get(tn - 1)) <= key_dist(now)) break;
      ++hops;
      // :198-210 move it to the top-pq list.
      T.insert(now, tn, lane);
      vh.add(now_id, lane);
      if (tn > p.pq) {
        const uint64_t ev = T.get(tn - 1);
        vh.del(key_id(ev), lane);
        --tn;
      }
      // :211-224 neighbours not in the visited hash, in row order.
      const int deg = static_cast<int>(__shfl_sync(FULL, a, 0));
      const bool isnb = lane >= 1 && lane <= deg;
      const bool fresh = isnb && !vh.test(a);
      const unsigned fm = __ballot_sync(FULL, fresh);
      const int m = __popc(fm);
      if (fresh) cbuf[__popc(fm & lanemask_lt())] = a;
      __syncwarp();
      const uint32_t cid = lane < m ? cbuf[lane] : 0u;
      // :237-287 distances.
      if (!gather_distances<METRIC, H>(p, stage, mbar, ph0, ph1, qv, m, cid, cd, lane)) {
        if (lane == 0) atomicOr(p.error, 1);
        return;
      }
      evals += m;
      // The next vertex popped is the smaller of the queue head and the best
      // candidate (the select-insert rule can only reject candidates above a
      // full queue's maximum); start loading its adjacency row now so that it
      // arrives while the candidates are inserted.
      const uint64_t ck = lane < m ? make_key(cd, cid) : ~0ull;
      const uint64_t cmin = warp_min_u64(ck);
      const uint64_t qh = qn > 0 ? Q.get(0) : ~0ull;
      const uint64_t nk = cmin < qh ? cmin : qh;
      if (nk != ~0ull) {
        next_id = key_id(nk);
        a_next = lane < nslots ? __ldg(p.adj + (static_cast<uint64_t>(next_id) << p.shift) + lane) : 0u;
      }
      // :297-322 select-insert in candidate order.
      for (int c = 0; c < m; ++c) {
        const float d = __shfl_sync(FULL, cd, c);
        const uint32_t id = __shfl_sync(FULL, cid, c);
        const uint64_t key = make_key(d, id);
        if (qn >= p.pq && key_dist(Q.get(qn - 1)) < key_dist(key)) continue;
        Q.insert(key, qn, lane);
        vh.add(id, lane);
        if (qn >= p.pq + 1) {
          const uint64_t ev = Q.get(qn - 1);
          vh.del(key_id(ev), lane);
          --qn;
        }
      }
    }
    // :331-335 ascending ids; slots past the list length get UINT64_MAX.
    uint64_t *o = p.out + static_cast<size_t>(qid) * p.k;
#pragma unroll
    for (int j = 0; j < S; ++j) {
      const int i = lane * S + j;
      if (i < p.k) o[i] = i < tn ? static_cast<uint64_t>(key_id(T.v[j])) : ~0ull;
    }
    if (lane == 0) {
      if (p.hops) p.hops[qid] = hops;
      if (p.evals) p.evals[qid] = evals;
    }
    __syncwarp();
  }
}

__global__ void debug_fixhash_kernel(const uint32_t *ids, int count, int cap, uint64_t magic,
                                     int32_t *out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  VisitedHash vh{nullptr, cap, magic};
  if (i < count) out[i] = vh.slot(ids[i]);
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
namespace {

uint32_t align_up(uint32_t x, uint32_t a) { return (x + a - 1) / a * a; }

// Rows staged per buffer half: a typical hop evaluates 2-5 neighbours.
int stage_rows(uint32_t row_bytes) { return row_bytes <= 1024 ? 4 : 2; }

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

Layout make_layout(const DeviceIndex &ix, int pq) {
  Layout L;
  L.H = stage_rows(ix.row_bytes);
  L.S = queue_segment(pq);
  L.cap = 8 * pq;
  uint32_t off = 2u * L.H * ix.row_bytes;
  off = align_up(off, 16);
  L.off_mbar = off;
  off += 16;
  L.off_cand = off;
  off += 32 * 4;
  off = align_up(off, 16);
  L.off_q = off;
  off += align_up(static_cast<uint32_t>(ix.dim) * 4u, 16);
  L.off_hash = off;
  off += 4u * L.cap;
  L.warp_bytes = align_up(off, 128);
  return L;
}

// Launch shape per (kernel, bytes per warp): the warps-per-block in {4, 2, 1}
// that keeps the most warps resident per SM.
struct Shape {
  const void *fn;
  uint32_t warp_bytes;
  int wpb, blocks_per_sm, sms;
};

std::mutex g_shape_mu;
std::vector<Shape> g_shapes;

int get_shape(const void *fn, uint32_t warp_bytes, Shape &out) {
  std::lock_guard<std::mutex> lk(g_shape_mu);
  int dev = 0;
  cudaGetDevice(&dev);
  for (const Shape &s : g_shapes)
    if (s.fn == fn && s.warp_bytes == warp_bytes) {
      out = s;
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
  Shape best{fn, warp_bytes, 0, 0, sms};
  for (int wpb = MAX_WARPS_PER_BLOCK; wpb >= 1; wpb >>= 1) {
    const size_t smem = static_cast<size_t>(warp_bytes) * wpb;
    if (smem > static_cast<size_t>(optin)) continue;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, wpb * 32, smem);
    if (e != cudaSuccess) return e;
    if (per_sm * wpb > best.blocks_per_sm * best.wpb) {
      best.wpb = wpb;
      best.blocks_per_sm = per_sm;
    }
  }
  if (best.wpb == 0) return -1;
  g_shapes.push_back(best);
  out = best;
  return 0;
}

template <int METRIC, int H, int S>
int launch_t(const DeviceIndex &ix, const SearchCall &c, const Layout &L, cudaStream_t stream) {
  Params p;
  p.rows = static_cast<const uint8_t *>(ix.rows);
  p.row_bytes = ix.row_bytes;
  p.row_scale = ix.row_scale;
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

  auto kern = search_kernel<METRIC, H, S>;
  Shape sh;
  int e = get_shape(reinterpret_cast<const void *>(kern), L.warp_bytes, sh);
  if (e != 0) return e;
  const int want = (c.nq + sh.wpb - 1) / sh.wpb;
  const int grid = std::max(1, std::min(want, sh.blocks_per_sm * sh.sms));
  cudaError_t ce = cudaMemsetAsync(c.counter, 0, sizeof(uint32_t), stream);
  if (ce != cudaSuccess) return ce;
  kern<<<grid, sh.wpb * 32, static_cast<size_t>(L.warp_bytes) * sh.wpb, stream>>>(p);
  return cudaGetLastError();
}

template <int METRIC, int H>
int launch_s(const DeviceIndex &ix, const SearchCall &c, const Layout &L, cudaStream_t s) {
  switch (L.S) {
    case 1: return launch_t<METRIC, H, 1>(ix, c, L, s);
    case 2: return launch_t<METRIC, H, 2>(ix, c, L, s);
    case 4: return launch_t<METRIC, H, 4>(ix, c, L, s);
    case 8: return launch_t<METRIC, H, 8>(ix, c, L, s);
    case 16: return launch_t<METRIC, H, 16>(ix, c, L, s);
    case 32: return launch_t<METRIC, H, 32>(ix, c, L, s);
    default: return -1;
  }
}

template <int METRIC>
int launch_m(const DeviceIndex &ix, const SearchCall &c, const Layout &L, cudaStream_t s) {
  return L.H == 4 ? launch_s<METRIC, 4>(ix, c, L, s) : launch_s<METRIC, 2>(ix, c, L, s);
}

}  // namespace

uint32_t search_warp_bytes(const DeviceIndex &ix, int pq) { return make_layout(ix, pq).warp_bytes; }

int launch_search(const DeviceIndex &ix, const SearchCall &c, cudaStream_t stream) {
  if (c.nq <= 0) return 0;
  const Layout L = make_layout(ix, c.pq);
  switch (ix.metric) {
    case 0: return launch_m<0>(ix, c, L, stream);
    case 1: return launch_m<1>(ix, c, L, stream);
    case 2: return launch_m<2>(ix, c, L, stream);
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
