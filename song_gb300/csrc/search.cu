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

#include "device_common.cuh"
#include "internal.h"

namespace song {

constexpr int WARPS_PER_BLOCK = 4;

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
  uint32_t off_mbar, off_cand, off_q, off_Q, off_T, off_hash;
  int qmask, tmask, cap;
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

template <int METRIC, int H>
__global__ void __launch_bounds__(WARPS_PER_BLOCK * 32)
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
  SortedRing Q{reinterpret_cast<uint64_t *>(ws + p.off_Q), p.qmask};
  SortedRing T{reinterpret_cast<uint64_t *>(ws + p.off_T), p.tmask};

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

    // warp_astar_accelerator.h:115-176: distance to vertex 0, queue = {0}.
    float cd;
    if (!gather_distances<METRIC, H>(p, stage, mbar, ph0, ph1, qv, 1, 0u, cd, lane)) {
      if (lane == 0) atomicOr(p.error, 1);
      return;
    }
    const float d0 = __shfl_sync(FULL, cd, 0);
    int qhead = 0, qn = 0, tn = 0;
    Q.insert(qhead, qn, make_key(d0, 0u), lane);
    vh.add(0u, lane);
    int hops = 0, evals = 1;

    while (qn > 0) {
      // :186-193 pop the minimum, drop it from the visited hash.
      const uint64_t now = Q.at(qhead, 0);
      qhead = (qhead + 1) & p.qmask;
      --qn;
      const uint32_t now_id = key_id(now);
      const uint32_t *arow = p.adj + (static_cast<uint64_t>(now_id) << p.shift);
      const uint32_t a = lane < nslots ? __ldg(arow + lane) : 0u;
      vh.del(now_id, lane);
      // :191 finish test (<=) against the list maximum.
      if (tn == p.pq && key_dist(T.at(0, tn - 1)) <= key_dist(now)) break;
      ++hops;
      // :198-210 move it to the top-pq list.
      T.insert(0, tn, now, lane);
      vh.add(now_id, lane);
      if (tn > p.pq) {
        const uint64_t ev = T.at(0, tn - 1);
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
      // :297-322 select-insert in candidate order.
      for (int c = 0; c < m; ++c) {
        const float d = __shfl_sync(FULL, cd, c);
        const uint32_t id = __shfl_sync(FULL, cid, c);
        const uint64_t key = make_key(d, id);
        if (qn >= p.pq && key_dist(Q.at(qhead, qn - 1)) < key_dist(key)) continue;
        Q.insert(qhead, qn, key, lane);
        vh.add(id, lane);
        if (qn >= p.pq + 1) {
          const uint64_t ev = Q.at(qhead, qn - 1);
          vh.del(key_id(ev), lane);
          --qn;
        }
      }
    }
    // :331-335 ascending ids; slots past the list length get UINT64_MAX.
    uint64_t *o = p.out + static_cast<size_t>(qid) * p.k;
    for (int i = lane; i < p.k; i += 32)
      o[i] = i < tn ? static_cast<uint64_t>(key_id(T.at(0, i))) : ~0ull;
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

int pow2_at_least(int x) {
  int p = 1;
  while (p < x) p <<= 1;
  return p;
}

// Rows staged per buffer: enough rows for a typical hop, a few KB per warp.
int stage_rows(uint32_t row_bytes) {
  if (row_bytes <= 256) return 8;
  if (row_bytes <= 1024) return 4;
  return 2;
}

struct Layout {
  uint32_t warp_bytes, off_mbar, off_cand, off_q, off_Q, off_T, off_hash;
  int qcap, tcap, cap, H;
};

Layout make_layout(const DeviceIndex &ix, int pq) {
  Layout L;
  L.H = stage_rows(ix.row_bytes);
  L.qcap = pow2_at_least(pq + 1);
  L.tcap = pow2_at_least(pq + 1);
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
  L.off_Q = off;
  off += 8u * L.qcap;
  L.off_T = off;
  off += 8u * L.tcap;
  L.off_hash = off;
  off += 4u * L.cap;
  L.warp_bytes = align_up(off, 128);
  return L;
}

template <int METRIC, int H>
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
  p.off_Q = L.off_Q;
  p.off_T = L.off_T;
  p.off_hash = L.off_hash;
  p.qmask = L.qcap - 1;
  p.tmask = L.tcap - 1;
  p.cap = L.cap;
  p.magic = ~0ull / static_cast<uint64_t>(L.cap);

  const size_t smem = static_cast<size_t>(L.warp_bytes) * WARPS_PER_BLOCK;
  auto kern = search_kernel<METRIC, H>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(smem));
  if (e != cudaSuccess) return e;
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, WARPS_PER_BLOCK * 32, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return -1;
  const int want = (c.nq + WARPS_PER_BLOCK - 1) / WARPS_PER_BLOCK;
  const int grid = std::max(1, std::min(want, per_sm * sms));
  e = cudaMemsetAsync(c.counter, 0, sizeof(uint32_t), stream);
  if (e != cudaSuccess) return e;
  kern<<<grid, WARPS_PER_BLOCK * 32, smem, stream>>>(p);
  return cudaGetLastError();
}

template <int METRIC>
int launch_m(const DeviceIndex &ix, const SearchCall &c, const Layout &L, cudaStream_t s) {
  switch (L.H) {
    case 8: return launch_t<METRIC, 8>(ix, c, L, s);
    case 4: return launch_t<METRIC, 4>(ix, c, L, s);
    default: return launch_t<METRIC, 2>(ix, c, L, s);
  }
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
