// search_kernel.cuh -- the batched best-first graph search kernel for sm_103a.
//
// It computes what warp_independent_search_kernel computes
// (warp_astar_accelerator.h:41-341): for each query, a best-first walk from
// vertex 0 over the fixed-degree graph with a candidate queue bounded at pq,
// a top-pq list of expanded vertices, a visited hash over queue and list, the
// select-insert rule (skip a candidate when the queue is full and its maximum
// is closer) and the finish rule (stop when the list is full and its maximum
// is <= the vertex just popped).  With FP32 storage the distances are the
// reference's bit for bit: lane l sums dims l, l+32, ... with fused
// multiply-add and the 32 partial sums meet in the xor butterfly 16,8,4,2,1.
//
// GB300 design:
//  * persistent warps pull queries from a work counter; warps never wait for
//    one another (the only block barrier is the model load at kernel start);
//  * per-query state: query vector, visited hash (the reference's FixHash,
//    8*pq slots) and a two-buffer staging ring in the warp's shared memory;
//    candidate queue and top-pq list in registers (reg_queue.cuh);
//  * each hop's unvisited neighbour rows are gathered with 1-D bulk async
//    copies (cp.async.bulk, mbarrier transaction counts) into the ring, two
//    chunks in flight, and read back in the reference's lane order;
//  * the next hop's adjacency row is loaded as soon as the next pop is known.
//
// Template parameters: METRIC (0 L2, 1 IP, 2 COS), STORAGE (0 F32, 1 BF16,
// 2 FP8-E4M3 with a per-row scale), H (rows per staging buffer), S (register
// queue segment, capacity 32*S >= pq+1), LEARNED (per-hop features: trace
// capture and/or the early-exit network).
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_fp8.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "device_common.cuh"
#include "internal.h"
#include "reg_queue.cuh"

namespace song {

constexpr int MAX_WARPS_PER_BLOCK = 4;
constexpr int MAX_PROBES = 4;  // candidate list of the MULTI kernel: MAX_PROBES * 32 ids
constexpr int MLP_IN = 5, MLP_H = 32;
// FP32 parameters of the early-exit network, in this order.
constexpr int MLP_W1 = 0;                        // [MLP_H][MLP_IN]
constexpr int MLP_B1 = MLP_W1 + MLP_H * MLP_IN;  // [MLP_H]
constexpr int MLP_W2 = MLP_B1 + MLP_H;           // [MLP_H][MLP_H]
constexpr int MLP_B2 = MLP_W2 + MLP_H * MLP_H;   // [MLP_H]
constexpr int MLP_W3 = MLP_B2 + MLP_H;           // [MLP_H]
constexpr int MLP_B3 = MLP_W3 + MLP_H;           // [1]
constexpr int MLP_NPARAM = MLP_B3 + 1;
constexpr int TRACE_FIELDS = 6;  // 5 features + top-k version

struct Params {
  const uint8_t *rows;
  uint32_t row_bytes;
  uint32_t scale_off;  // FP8: byte offset of the row's float scale
  const float *rows_f32;
  uint32_t f32_row_bytes;
  int rerank;  // final candidates re-ranked with FP32 distances (low-precision storage)
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
  uint64_t magic;  // VisitedHash (plain kernel)
  int log2cap;     // ExactVisited (learned kernel)
  uint32_t wait_limit;  // polls of a bounded mbarrier wait
  uint32_t extra_tx;    // test hook: bytes every copy batch expects beyond its rows (0 in use)
  // the reference's N_MULTIPROBE / FINISH_CNT knobs (MULTI kernel only)
  int probes;      // vertices popped per iteration, 1..MAX_PROBES
  int finish_cnt;  // finish tests that must hold before the search ends, >= 1
  int double_check;  // select-insert skips candidates already visited (__ENABLE_MULTIPROBE_DOUBLE_CHECK)
  // learned variant
  const __nv_bfloat16 *mlp;  // MLP_NPARAM weights (BF16), null = no early exit
  float exit_threshold;
  int exit_min_hops;
  int exit_every;
  int exit_max_hops;      // > 0: stop after this many hops (fixed-budget heuristic)
  float *trace;           // [nq][trace_hops][TRACE_FIELDS] or null
  int trace_hops;
  int32_t *trace_final;   // [nq]: final top-k version, hops traced
  const uint32_t *qcodes; // BITS storage: [nq][8] 256-bit codes of the queries
  const uint32_t *starts; // [nq][n_starts] start vertices of each query, or null: vertex 0
  int n_starts;
  // entry points chosen inside the server's persistent warps (entry_rows
  // null: vertex 0); the layout of song_index's entry fields
  const float *entry_rows;
  const uint32_t *entry_ids;
  int n_entries;
  const float *coarse_rows;
  int n_coarse;
  const uint32_t *entry_offsets;
  int n_probes;
  int entry_dpad;
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

// Element j of a staged row as float.  FP8 elements are decoded and scaled
// (x = e4m3(y) * scale, rounded to float), so a low-precision search equals
// an FP32 search over the dequantised vectors.
template <int STORAGE>
__device__ __forceinline__ float load_elem(const uint8_t *row, int j, float scale) {
  if (STORAGE == 0) return reinterpret_cast<const float *>(row)[j];
  if (STORAGE == 1) return __bfloat162float(reinterpret_cast<const __nv_bfloat16 *>(row)[j]);
  const __half_raw h = __nv_cvt_fp8_to_halfraw(static_cast<__nv_fp8_storage_t>(row[j]), __NV_E4M3);
  return __fmul_rn(__half2float(__half(h)), scale);
}

// The 256-bit code of a query (BITS storage), in every lane.
struct Code8 {
  uint32_t w[8];
};

// Distances of candidates 0..m-1 (candidate c's id in lane c); candidate c's
// distance is returned in lane c.  False if a bulk copy never completed.
// Rows are taken in pairs through the paired FP32 instructions (the same
// roundings, in the same order, as the scalar form: lane l sums dims l, l+32,
// ... of each row with fused multiply-add).
template <int METRIC, int STORAGE, int H>
__device__ __forceinline__ bool gather_distances(const Params &p, uint8_t *stage, uint64_t *mbar,
                                                 uint32_t &ph0, uint32_t &ph1, const float *qv,
                                                 int m, uint32_t cid, float &out, int lane,
                                                 const Code8 &qc) {
  if constexpr (STORAGE == 3) {
    // Hamming distance of 256-bit codes: lane c reads candidate c's 32-byte
    // code straight from global memory (two 16-byte loads) and sums the
    // popcounts of its xor with the query's code (an integer, exact as float)
    out = 0.0f;
    if (lane < m) {
      const uint4 *r = reinterpret_cast<const uint4 *>(p.rows + static_cast<uint64_t>(cid) * 32u);
      const uint4 a = __ldg(r), b = __ldg(r + 1);
      const int h = __popc(a.x ^ qc.w[0]) + __popc(a.y ^ qc.w[1]) + __popc(a.z ^ qc.w[2]) + __popc(a.w ^ qc.w[3]) +
                    __popc(b.x ^ qc.w[4]) + __popc(b.y ^ qc.w[5]) + __popc(b.z ^ qc.w[6]) + __popc(b.w ^ qc.w[7]);
      out = static_cast<float>(h);
    }
    return true;
  }
  const int nchunks = (m + H - 1) / H;
  const uint32_t rb = p.row_bytes;
  auto issue = [&](int c) {
    const int b = c & 1;
    const int first = c * H;
    const int cnt = min(H, m - first);
    // The buffer was last read through the generic proxy; order those reads
    // before the async-proxy writes of the copies issued below.
    fence_proxy_async();
    if (lane == 0) mbar_arrive_expect_tx(&mbar[b], static_cast<uint32_t>(cnt) * rb + p.extra_tx);
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
    if (!mbar_wait(&mbar[b], ph, p.wait_limit)) {
      // give up: wait (bounded again) for the other buffer's copies, still in
      // flight into this warp's shared memory, before the warp leaves
      if (c + 1 < nchunks) mbar_wait(&mbar[b ^ 1], b ? ph0 : ph1, p.wait_limit);
      return false;
    }
    ph ^= 1u;
    const int first = c * H;
    const int cnt = min(H, m - first);
    const uint8_t *buf = stage + static_cast<size_t>(b * H) * rb;
    float acc[H], len[H];
    if constexpr (H == 1) {
      float a = 0.0f, l2 = 0.0f;
      const float scale = STORAGE == 2 ? *reinterpret_cast<const float *>(buf + p.scale_off) : 1.0f;
      for (int j = lane; j < p.dim; j += 32) {
        const float qj = qv[j];
        const float xj = load_elem<STORAGE>(buf, j, scale);
        if (METRIC == 0) {
          const float d = __fsub_rn(qj, xj);
          a = __fmaf_rn(d, d, a);
        } else {
          a = __fmaf_rn(qj, xj, a);
          if (METRIC == 2) l2 = __fmaf_rn(xj, xj, l2);
        }
      }
      acc[0] = a;
      len[0] = l2;
    } else {
      constexpr int P = H / 2;  // row pairs
      uint64_t a2[P], l2[P];
      float sc[H];
#pragma unroll
      for (int i = 0; i < P; ++i) a2[i] = l2[i] = 0ull;
#pragma unroll
      for (int i = 0; i < H; ++i)
        sc[i] = STORAGE == 2 ? *reinterpret_cast<const float *>(buf + static_cast<size_t>(i) * rb + p.scale_off) : 1.0f;
#pragma unroll 2
      for (int j = lane; j < p.dim; j += 32) {
        const float qj = qv[j];
        const uint64_t qq = f2_pack(qj, qj);
#pragma unroll
        for (int i = 0; i < P; ++i) {
          if (2 * i < cnt) {  // warp-uniform
            const float x0 = load_elem<STORAGE>(buf + static_cast<size_t>(2 * i) * rb, j, sc[2 * i]);
            const float x1 = load_elem<STORAGE>(buf + static_cast<size_t>(2 * i + 1) * rb, j, sc[2 * i + 1]);
            const uint64_t xx = f2_pack(x0, x1);
            if (METRIC == 0) {
              const uint64_t d = f2_sub(qq, xx);
              a2[i] = f2_fma(d, d, a2[i]);
            } else {
              a2[i] = f2_fma(qq, xx, a2[i]);
              if (METRIC == 2) l2[i] = f2_fma(xx, xx, l2[i]);
            }
          }
        }
      }
#pragma unroll
      for (int i = 0; i < P; ++i) {
        f2_unpack(a2[i], acc[2 * i], acc[2 * i + 1]);
        f2_unpack(l2[i], len[2 * i], len[2 * i + 1]);
      }
    }
    // Row r's sums are in lanes r*(32/H) .. ; candidate first + i takes row i.
    const float t = butterfly_rows<H>(acc, lane);
    const float ln = METRIC == 2 ? butterfly_rows<H>(len, lane) : 0.0f;
    const int src = ((lane - first) & (H - 1)) * (32 / H);
    const float ts = __shfl_sync(FULL, t, src);
    const float ls = METRIC == 2 ? __shfl_sync(FULL, ln, src) : 0.0f;
    if (lane >= first && lane < first + cnt) out = finish_distance<METRIC>(ts, ls);
    __syncwarp();
    if (c + 2 < nchunks) issue(c + 2);
  }
  return true;
}

// FP32 distances (reference arithmetic) of up to 4 rows loaded straight from
// global memory, lane-strided and coalesced; result i in every lane.
template <int METRIC>
__device__ __forceinline__ void fp32_distances4(const Params &p, const float *qv,
                                                const uint32_t ids[4], int cnt, float d[4],
                                                int lane) {
  float acc[4], len[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    acc[i] = 0.0f;
    len[i] = 0.0f;
  }
  for (int j = lane; j < p.dim; j += 32) {
    const float qj = qv[j];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      if (i < cnt) {
        const float *row = reinterpret_cast<const float *>(
            reinterpret_cast<const uint8_t *>(p.rows_f32) + static_cast<uint64_t>(ids[i]) * p.f32_row_bytes);
        const float xj = __ldg(row + j);
        if (METRIC == 0) {
          const float dd = __fsub_rn(qj, xj);
          acc[i] = __fmaf_rn(dd, dd, acc[i]);
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
    for (int i = 0; i < 4; ++i) {
      acc[i] = __fadd_rn(acc[i], __shfl_xor_sync(FULL, acc[i], o));
      if (METRIC == 2) len[i] = __fadd_rn(len[i], __shfl_xor_sync(FULL, len[i], o));
    }
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) d[i] = finish_distance<METRIC>(acc[i], len[i]);
}

__device__ __forceinline__ uint64_t warp_min_u64(uint64_t x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const uint64_t y = __shfl_xor_sync(FULL, x, o);
    x = y < x ? y : x;
  }
  return x;
}

__device__ __forceinline__ float key_float(uint64_t k) {
  const uint32_t b = key_dist(k);
  return __uint_as_float((b & 0x80000000u) ? (b & 0x7fffffffu) : ~b);
}

// Early-exit network, warp-parallel: lane j owns hidden unit j of both layers.
// BF16 weights in shared memory, FP32 arithmetic.  Returns the logit.
__device__ __forceinline__ float mlp_logit(const __nv_bfloat16 *w, const float f[MLP_IN], int lane) {
  float h1 = __bfloat162float(w[MLP_B1 + lane]);
#pragma unroll
  for (int i = 0; i < MLP_IN; ++i) h1 = __fmaf_rn(__bfloat162float(w[MLP_W1 + lane * MLP_IN + i]), f[i], h1);
  h1 = fmaxf(h1, 0.0f);
  float h2 = __bfloat162float(w[MLP_B2 + lane]);
#pragma unroll
  for (int i = 0; i < MLP_H; ++i)
    h2 = __fmaf_rn(__bfloat162float(w[MLP_W2 + lane * MLP_H + i]), __shfl_sync(FULL, h1, i), h2);
  h2 = fmaxf(h2, 0.0f);
  float z = __fmul_rn(__bfloat162float(w[MLP_W3 + lane]), h2);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) z = __fadd_rn(z, __shfl_xor_sync(FULL, z, o));
  return __fadd_rn(z, __bfloat162float(w[MLP_B3]));
}

// The plain kernel keeps the reference's FixHash (bit parity); the learned
// kernel, which makes no parity claim, uses the smaller exact set.  Both are
// sized per query from its pq.
template <bool LEARNED>
struct VisitedOf {
  using type = VisitedHash;
  __device__ static VisitedHash make(int32_t *tab, int pq) {
    const int cap = 8 * pq;
    return VisitedHash{tab, cap, ~0ull / static_cast<uint64_t>(cap)};
  }
};
template <>
struct VisitedOf<true> {
  using type = ExactVisited;
  __device__ static ExactVisited make(int32_t *tab, int pq) {
    int lg = 5;
    while ((1 << lg) < 4 * pq) ++lg;
    return ExactVisited{tab, 1 << lg, lg};
  }
};

// The warp's shared-memory slice and barrier phases.
struct WarpCtx {
  uint8_t *stage;
  uint64_t *mbar;
  uint32_t *cbuf;
  float *qv;
  int32_t *tab;
  const __nv_bfloat16 *wmlp;
  uint32_t ph0, ph1;
};

struct QueryStats {
  int hops, evals, version;
};

// One query: the search of warp_astar_accelerator.h:111-335 with the query
// vector at qsrc, queue bound pq, k ids written ascending to o.  `trace`
// (LEARNED) receives the per-hop features or is null.  False if a bulk copy
// never completed.  MULTI: the reference's N_MULTIPROBE / FINISH_CNT knobs
// (p.probes, p.finish_cnt) as run-time values.
template <int METRIC, int STORAGE, int H, int S, bool LEARNED, bool MULTI = false>
__device__ __forceinline__ bool run_query(const Params &p, WarpCtx &w, const float *qsrc, const uint32_t *starts,
                                          int ns, int pq, int k, uint64_t *o, float *trace, QueryStats &st,
                                          int lane, const uint32_t *qcode = nullptr) {
  Code8 qc;
#pragma unroll
  for (int i = 0; i < 8; ++i) qc.w[i] = STORAGE == 3 ? qcode[i] : 0u;
  typename VisitedOf<LEARNED>::type vh = VisitedOf<LEARNED>::make(w.tab, pq);
  RegQueue<S> Q, T;  // candidate queue and top-pq list, ascending (distance, id)
  constexpr int C = RegQueue<S>::C;
  const int nslots = 1 << p.shift;
  for (int j = lane; j < p.dim; j += 32) w.qv[j] = qsrc[j];
  vh.clear(lane);
  // Start vertices: vertex 0 (the reference's), or the ns entry points the
  // pre-pass chose (lane i holds start i).  Prefetch the first start's row.
  if (!starts) ns = 1;
  const uint32_t sid = (starts && lane < ns) ? starts[lane] : 0u;
  uint32_t next_id = __shfl_sync(FULL, sid, 0);
  uint32_t a_next = lane < nslots ? __ldg(p.adj + (static_cast<uint64_t>(next_id) << p.shift) + lane) : 0u;

  // warp_astar_accelerator.h:115-176: distances to the starts, queue = {starts}.
  float cd;
  if (!gather_distances<METRIC, STORAGE, H>(p, w.stage, w.mbar, w.ph0, w.ph1, w.qv, ns, sid, cd, lane, qc)) {
    return false;
  }
  const float d0 = __shfl_sync(FULL, cd, 0);
  int qn = 0, tn = 0;
  Q.clear();
  T.clear();
  // T holds pq keys at all times: tn real ones (ascending, from position
  // C - pq) followed by pq - tn "infinite" keys, so every insertion evicts
  // the window's maximum (an infinite one while tn < pq).
#pragma unroll
  for (int j = 0; j < S; ++j) T.v[j] = (lane * S + j) >= C - pq ? ~0ull : 0ull;
  // Q likewise holds pq keys: qn real ones from position C - pq, then
  // infinite ones; a pop shifts the window one place left.
#pragma unroll
  for (int j = 0; j < S; ++j) Q.v[j] = (lane * S + j) >= C - pq ? ~0ull : 0ull;
  for (int i = 0; i < ns; ++i) {  // in start order, as the oracle queues them
    const uint32_t id = __shfl_sync(FULL, sid, i);
    Q.insert_evict(make_key(__shfl_sync(FULL, cd, i), id), lane);
    vh.add(id, lane);
  }
  qn = ns;
  if (ns > 1) {  // the first pop is the nearest start: prefetch its row instead
    const uint32_t mid = key_id(warp_min_u64(lane < ns ? make_key(cd, sid) : ~0ull));
    if (mid != next_id) {
      next_id = mid;
      a_next = lane < nslots ? __ldg(p.adj + (static_cast<uint64_t>(mid) << p.shift) + lane) : 0u;
    }
  }
  int hops = 0, evals = ns;
  int version = 0;           // number of changes of the top-k set (LEARNED)
  int last_change = 0;       // hop of the latest change (LEARNED)
  uint64_t kth_key = ~0ull;  // k-th smallest key of T, ~0 while tn < k (LEARNED)

  int finished = 0;  // MULTI: finish tests that held (finished[cid], :190-192)
  while (qn > 0) {
    if constexpr (MULTI) {
      // :182-228 up to p.probes pops per iteration.  Only the first takes the
      // finish test, which counts; the search ends when p.finish_cnt tests
      // held.  Every pop goes to the top-pq list, and the unvisited
      // neighbours of all of them are listed, in pop and row order (a vertex
      // adjacent to two pops may be listed twice, as in the reference),
      // before any distance is computed.
      int m = 0;
      bool fin = false;
      const int avail = qn;
      for (int kp = 0; kp < p.probes && kp < avail; ++kp) {
        uint64_t qh;
        const uint64_t now = Q.pop_window(C - pq, lane, &qh);
        --qn;
        const uint32_t now_id = key_id(now);
        const uint32_t a = (kp == 0 && now_id == next_id)
                               ? a_next
                               : (lane < nslots ? __ldg(p.adj + (static_cast<uint64_t>(now_id) << p.shift) + lane) : 0u);
        const int now_home = vh.slot(now_id);
        vh.del_at(now_id, now_home, lane);
        if (kp == 0 && tn == pq && key_dist(T.max()) <= key_dist(now) && ++finished >= p.finish_cnt) {
          fin = true;
          break;
        }
        ++hops;
        // :198-210 a later pop can lie above the list maximum; then it is
        // the key that leaves (add, then delete, as the reference does).
        const uint64_t tmax = T.max();
        const uint64_t ev = now < tmax ? tmax : now;
        T.insert_evict(now, lane);
        vh.add_at(now_id, now_home, lane);
        if (tn < pq) ++tn;
        else vh.del(key_id(ev), lane);
        const int deg = static_cast<int>(__shfl_sync(FULL, a, 0));
        const bool fresh = lane >= 1 && lane <= deg && !vh.test(a);
        const unsigned fm = __ballot_sync(FULL, fresh);
        if (fresh) w.cbuf[m + __popc(fm & lanemask_lt())] = a;
        m += __popc(fm);
      }
      if (fin) break;
      __syncwarp();
      // :237-322 distances and select-insert, 32 candidates at a time, in
      // list order (the distances do not depend on the queue, so this is the
      // reference's all-distances-then-all-inserts order).
      for (int r0 = 0; r0 < m; r0 += 32) {
        const int mr = min(32, m - r0);
        const uint32_t cid = lane < mr ? w.cbuf[r0 + lane] : 0u;
        if (!gather_distances<METRIC, STORAGE, H>(p, w.stage, w.mbar, w.ph0, w.ph1, w.qv, mr, cid, cd, lane, qc))
          return false;
        evals += mr;
        const uint64_t ck = lane < mr ? make_key(cd, cid) : ~0ull;
        const int chome = vh.slot(cid);
        if (p.double_check) {
          // :297-322 with :307-310: a candidate already in the visited hash
          // (listed by an earlier pop of this iteration, or twice in one row)
          // is skipped, so the hash calls interleave with the insertions.
          for (int c = 0; c < mr; ++c) {
            const uint64_t key = __shfl_sync(FULL, ck, c);
            const uint64_t qmax = Q.max();
            if (key_dist(qmax) < key_dist(key)) continue;
            const uint32_t id = key_id(key);
            if (vh.test(id)) continue;
            const uint64_t ev = key < qmax ? qmax : key;
            Q.insert_evict(key, lane);
            if (qn < pq) ++qn;
            vh.add_at(id, __shfl_sync(FULL, chome, c), lane);
            if (ev != ~0ull) vh.del(key_id(ev), lane);
          }
          __syncwarp();
          continue;
        }
        uint64_t my_ev = ~0ull;
        unsigned ins = 0u;
        for (int c = 0; c < mr; ++c) {
          const uint64_t key = __shfl_sync(FULL, ck, c);
          const uint64_t qmax = Q.max();
          if (key_dist(qmax) < key_dist(key)) continue;
          const uint64_t ev = key < qmax ? qmax : key;
          Q.insert_evict(key, lane);
          ins |= 1u << c;
          if (lane == c) my_ev = ev;
          if (qn < pq) ++qn;
        }
        if (ins) {
          const int ehome = my_ev != ~0ull ? vh.slot(key_id(my_ev)) : 0;
          do {
            const int c = __ffs(ins) - 1;
            ins &= ins - 1u;
            vh.add_at(__shfl_sync(FULL, cid, c), __shfl_sync(FULL, chome, c), lane);
            const uint64_t ev = __shfl_sync(FULL, my_ev, c);
            if (ev != ~0ull) vh.del_at(key_id(ev), __shfl_sync(FULL, ehome, c), lane);
          } while (ins);
        }
        __syncwarp();
      }
      // the next iteration's first pop is the queue head: load its row now
      if (qn > 0) {
        next_id = key_id(Q.at(C - pq, lane));
        a_next = lane < nslots ? __ldg(p.adj + (static_cast<uint64_t>(next_id) << p.shift) + lane) : 0u;
      }
      continue;
    }
    // :186-193 pop the minimum, drop it from the visited hash.
    uint64_t qh;  // queue minimum after the pop
    const uint64_t now = Q.pop_window(C - pq, lane, &qh);
    --qn;
    const uint32_t now_id = key_id(now);
    uint32_t a = a_next;
    if (now_id != next_id)  // not taken: the prefetch predicts the pop exactly
      a = lane < nslots ? __ldg(p.adj + (static_cast<uint64_t>(now_id) << p.shift) + lane) : 0u;
    const int now_home = vh.slot(now_id);
    vh.del_at(now_id, now_home, lane);
    // :191 finish test (<=) against the list maximum.
    if (tn == pq && key_dist(T.max()) <= key_dist(now)) break;
    ++hops;
    // LEARNED: does `now` enter the current top-k?  (Only such an entry
    // changes the k-th key: T drops its maximum, never a top-k key.)
    const bool enters = LEARNED && now < kth_key;
    if (enters) {
      ++version;
      last_change = hops;
    }
    // :198-210 move it to the top-pq list (when full, `now` is below the
    // list maximum, which is the one dropped).
    {
      const uint64_t ev = T.max();
      T.insert_evict(now, lane);
      vh.add_at(now_id, now_home, lane);
      if (tn < pq) ++tn;
      else vh.del(key_id(ev), lane);
    }
    if (enters && tn >= k) kth_key = T.at(C - pq + k - 1, lane);
    // :211-224 neighbours not in the visited hash, in row order.
    const int deg = static_cast<int>(__shfl_sync(FULL, a, 0));
    const bool isnb = lane >= 1 && lane <= deg;
    const bool fresh = isnb && !vh.test(a);
    const unsigned fm = __ballot_sync(FULL, fresh);
    const int m = __popc(fm);
    if (fresh) w.cbuf[__popc(fm & lanemask_lt())] = a;
    __syncwarp();
    const uint32_t cid = lane < m ? w.cbuf[lane] : 0u;
    // :237-287 distances.
    if (!gather_distances<METRIC, STORAGE, H>(p, w.stage, w.mbar, w.ph0, w.ph1, w.qv, m, cid, cd, lane, qc))
      return false;
    evals += m;
    // The next vertex popped is the smaller of the queue head and the best
    // candidate (the select-insert rule can only reject candidates above a
    // full queue's maximum); start loading its adjacency row now so that it
    // arrives while the candidates are inserted.
    const uint64_t ck = lane < m ? make_key(cd, cid) : ~0ull;
    const uint64_t cmin = warp_min_u64(ck);
    const uint64_t nk = cmin < qh ? cmin : qh;
    if (nk != ~0ull) {
      next_id = key_id(nk);
      a_next = lane < nslots ? __ldg(p.adj + (static_cast<uint64_t>(next_id) << p.shift) + lane) : 0u;
    }
    // :297-322 select-insert in candidate order, in two passes.  The queue
    // pass applies the select-insert rule and the insertions and notes, in
    // lane c, the key candidate c's insertion pushed out (~0: none, the
    // queue was not full).  Below pq live keys the window's maximum is an
    // infinite key, which leaves and is never below a candidate; at pq, the
    // select-insert rule, then the larger of the key and the maximum leaves
    // (:315-320).  The hash pass then makes the reference's visited-hash
    // calls in the reference's order -- add(candidate), delete(pushed-out
    // key) per inserted candidate -- with every home slot computed up front,
    // one lane per key.  (Queue and hash are independent, so splitting the
    // passes changes neither.)
    const int chome = vh.slot(cid);
    uint64_t my_ev = ~0ull;
    unsigned ins = 0u;
    for (int c = 0; c < m; ++c) {
      const uint64_t key = __shfl_sync(FULL, ck, c);
      const uint64_t qmax = Q.max();
      if (key_dist(qmax) < key_dist(key)) continue;
      const uint64_t ev = key < qmax ? qmax : key;
      Q.insert_evict(key, lane);
      ins |= 1u << c;
      if (lane == c) my_ev = ev;
      if (qn < pq) ++qn;
    }
    if (ins) {
      const int ehome = my_ev != ~0ull ? vh.slot(key_id(my_ev)) : 0;
      do {
        const int c = __ffs(ins) - 1;
        ins &= ins - 1u;
        vh.add_at(__shfl_sync(FULL, cid, c), __shfl_sync(FULL, chome, c), lane);
        const uint64_t ev = __shfl_sync(FULL, my_ev, c);
        if (ev != ~0ull) vh.del_at(key_id(ev), __shfl_sync(FULL, ehome, c), lane);
      } while (ins);
    }
    if (LEARNED) {
      const bool check = p.mlp && hops >= p.exit_min_hops && (hops % p.exit_every) == 0 && tn >= k;
      if (trace || check) {
      // Per-hop state: hop count, k-th and best distance, queue-head gap,
      // hops since the top-k last changed, distance evaluations.  Distances
      // enter through scale-free, bounded quantities: the top-k spread and
      // the queue-head gap relative to the progress span d0 - best (signed
      // logs).
      const float kth = key_float(tn >= k ? kth_key : T.at(C - pq + tn - 1, lane));
      const float best = key_float(T.at(C - pq, lane));
      const float head = nk != ~0ull ? key_float(nk) : kth;
      const float span = fabsf(d0 - best) + 1e-6f * (fabsf(d0) + fabsf(best)) + 1e-30f;
      const float r1 = (kth - best) / span;
      const float r3 = (head - kth) / span;
      float f[MLP_IN];
      f[0] = __log2f(1.0f + static_cast<float>(hops)) * 0.1f;
      f[1] = copysignf(log1pf(fabsf(r1)), r1);
      f[2] = __log2f(1.0f + static_cast<float>(hops - last_change)) * 0.1f;
      f[3] = copysignf(log1pf(fabsf(r3)), r3);
      f[4] = __log2f(1.0f + static_cast<float>(evals)) * 0.1f;
      if (trace && hops <= p.trace_hops && lane < TRACE_FIELDS) {
        float v = lane < MLP_IN ? f[0] : static_cast<float>(version);
#pragma unroll
        for (int i = 1; i < MLP_IN; ++i) v = lane == i ? f[i] : v;
        trace[static_cast<size_t>(hops - 1) * TRACE_FIELDS + lane] = v;
      }
      if (check && mlp_logit(w.wmlp, f, lane) >= p.exit_threshold) break;  // converged
      }
      if (p.exit_max_hops > 0 && hops >= p.exit_max_hops) break;
    }
  }

  if (STORAGE != 0 && p.rerank > 0) {
    // FP32 re-rank of the best `rerank` entries of the list, then the first k.
    const int R = min(max(p.rerank, k), tn);
    int rn = 0;
    Q.clear();
    for (int base = 0; base < R; base += 4) {
      uint32_t ids[4];
      const int cnt = min(4, R - base);
#pragma unroll
      for (int i = 0; i < 4; ++i) ids[i] = i < cnt ? key_id(T.at(C - pq + base + i, lane)) : 0u;
      float d[4];
      fp32_distances4<METRIC>(p, w.qv, ids, cnt, d, lane);
#pragma unroll
      for (int i = 0; i < 4; ++i)
        if (i < cnt) {
          Q.insert_grow(make_key(d[i], ids[i]), lane);
          ++rn;
        }
    }
#pragma unroll
    for (int j = 0; j < S; ++j) {
      const int r = Q.rank_of(j, rn, lane);
      if (r >= 0 && r < k) o[r] = static_cast<uint64_t>(key_id(Q.v[j]));
    }
    for (int i = rn + lane; i < k; i += 32) o[i] = ~0ull;
  } else {
    // :331-335 ascending ids; slots past the list length get UINT64_MAX.
#pragma unroll
    for (int j = 0; j < S; ++j) {
      const int r = T.rank_of(j, pq, lane);
      if (r >= 0 && r < k && r < tn) o[r] = static_cast<uint64_t>(key_id(T.v[j]));
    }
    for (int i = tn + lane; i < k; i += 32) o[i] = ~0ull;
  }
  st.hops = hops;
  st.evals = evals;
  st.version = version;
  return true;
}

// Small queues (S <= 4, pq < 128) ask for six resident blocks (24 warps per
// SM, at most 80 registers; the per-warp shared memory of such pq fits).
// Measured on the headline search: 5 -> 6 blocks 10 % faster; 8 blocks (64
// registers) 3 % slower than 6.
template <int METRIC, int STORAGE, int S, bool LEARNED>
struct MinBlocks {
  static constexpr int value = S > 4 ? 1 : 6;
};

template <int METRIC, int STORAGE, int H, int S, bool LEARNED, bool MULTI = false>
__global__ void __launch_bounds__(MAX_WARPS_PER_BLOCK * 32, (MinBlocks<METRIC, STORAGE, S, LEARNED>::value))
    search_kernel(const Params p) {
  extern __shared__ __align__(128) uint8_t smem_raw[];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const int nwarps = blockDim.x >> 5;
  uint8_t *ws = smem_raw + static_cast<size_t>(wib) * p.warp_bytes;
  WarpCtx w;
  w.stage = ws;
  w.mbar = reinterpret_cast<uint64_t *>(ws + p.off_mbar);
  w.cbuf = reinterpret_cast<uint32_t *>(ws + p.off_cand);
  w.qv = reinterpret_cast<float *>(ws + p.off_q);
  w.tab = reinterpret_cast<int32_t *>(ws + p.off_hash);
  __nv_bfloat16 *wmlp = reinterpret_cast<__nv_bfloat16 *>(smem_raw + static_cast<size_t>(nwarps) * p.warp_bytes);
  w.wmlp = wmlp;
  if (LEARNED) {
    if (p.mlp)
      for (int i = threadIdx.x; i < MLP_NPARAM; i += blockDim.x) wmlp[i] = p.mlp[i];
    __syncthreads();
  }
  if (lane == 0) {
    mbar_init(&w.mbar[0], 1);
    mbar_init(&w.mbar[1], 1);
    fence_mbar_init();
  }
  __syncwarp();
  w.ph0 = 0;
  w.ph1 = 0;

  for (;;) {
    uint32_t qid = 0;
    if (lane == 0) qid = atomicAdd(p.counter, 1u);
    qid = __shfl_sync(FULL, qid, 0);
    if (qid >= static_cast<uint32_t>(p.nq)) break;
    float *trace = nullptr;
    if (LEARNED && p.trace) trace = p.trace + static_cast<size_t>(qid) * p.trace_hops * TRACE_FIELDS;
    QueryStats st;
    if (!run_query<METRIC, STORAGE, H, S, LEARNED, MULTI>(p, w, p.queries + static_cast<size_t>(qid) * p.dim,
                                                   p.starts ? p.starts + static_cast<size_t>(qid) * p.n_starts
                                                            : nullptr,
                                                   p.n_starts, p.pq,
                                                   p.k, p.out + static_cast<size_t>(qid) * p.k, trace, st,
                                                   lane, STORAGE == 3 ? p.qcodes + static_cast<size_t>(qid) * 8
                                                                      : nullptr)) {
      if (lane == 0) atomicOr(p.error, 1);
      return;
    }
    if (lane == 0) {
      if (p.hops) p.hops[qid] = st.hops;
      if (p.evals) p.evals[qid] = st.evals;
      if (LEARNED && p.trace_final) {
        p.trace_final[2 * qid] = st.version;
        p.trace_final[2 * qid + 1] = min(st.hops, p.trace_hops);
      }
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------------------
// Host-side launch helpers shared by the per-storage translation units.
// ---------------------------------------------------------------------------

// Launch shape per (kernel, bytes per block): warps per block in {4, 2, 1}
// that keeps the most warps resident per SM (search.cu).
int get_shape(const void *fn, uint32_t warp_bytes, uint32_t extra_bytes, int *wpb, int *grid_cap);

template <int METRIC, int STORAGE, int H, int S, bool LEARNED, bool MULTI = false>
int launch_kernel(const Params &p, cudaStream_t stream) {
  auto kern = search_kernel<METRIC, STORAGE, H, S, LEARNED, MULTI>;
  const uint32_t extra = LEARNED ? static_cast<uint32_t>(MLP_NPARAM * sizeof(__nv_bfloat16) + 64) : 0u;
  int wpb = 0, cap = 0;
  int e = get_shape(reinterpret_cast<const void *>(kern), p.warp_bytes, extra, &wpb, &cap);
  if (e != 0) return e;
  const int want = (p.nq + wpb - 1) / wpb;
  const int grid = want < cap ? (want > 0 ? want : 1) : cap;
  cudaError_t ce = cudaMemsetAsync(p.counter, 0, sizeof(uint32_t), stream);
  if (ce != cudaSuccess) return ce;
  kern<<<grid, wpb * 32, static_cast<size_t>(p.warp_bytes) * wpb + extra, stream>>>(p);
  return cudaGetLastError();
}

template <int METRIC, int STORAGE, int H, bool LEARNED, bool MULTI = false>
int launch_by_s(const Params &p, int S, cudaStream_t s) {
  switch (S) {
    case 1: return launch_kernel<METRIC, STORAGE, H, 1, LEARNED, MULTI>(p, s);
    case 2: return launch_kernel<METRIC, STORAGE, H, 2, LEARNED, MULTI>(p, s);
    case 4: return launch_kernel<METRIC, STORAGE, H, 4, LEARNED, MULTI>(p, s);
    case 8: return launch_kernel<METRIC, STORAGE, H, 8, LEARNED, MULTI>(p, s);
    case 16: return launch_kernel<METRIC, STORAGE, H, 16, LEARNED, MULTI>(p, s);
    case 32: return launch_kernel<METRIC, STORAGE, H, 32, LEARNED, MULTI>(p, s);
    default: return -1;
  }
}

template <int STORAGE, bool LEARNED, bool MULTI = false>
int launch_storage(const Params &p, int metric, int H, int S, cudaStream_t s) {
  const int h = H == 1 ? 0 : (H == 2 ? 1 : (H == 4 ? 2 : -1));
  if (h < 0) return -1;
  switch (metric * 3 + h) {
    case 0: return launch_by_s<0, STORAGE, 1, LEARNED, MULTI>(p, S, s);
    case 1: return launch_by_s<0, STORAGE, 2, LEARNED, MULTI>(p, S, s);
    case 2: return launch_by_s<0, STORAGE, 4, LEARNED, MULTI>(p, S, s);
    case 3: return launch_by_s<1, STORAGE, 1, LEARNED, MULTI>(p, S, s);
    case 4: return launch_by_s<1, STORAGE, 2, LEARNED, MULTI>(p, S, s);
    case 5: return launch_by_s<1, STORAGE, 4, LEARNED, MULTI>(p, S, s);
    case 6: return launch_by_s<2, STORAGE, 1, LEARNED, MULTI>(p, S, s);
    case 7: return launch_by_s<2, STORAGE, 2, LEARNED, MULTI>(p, S, s);
    case 8: return launch_by_s<2, STORAGE, 4, LEARNED, MULTI>(p, S, s);
    default: return -1;
  }
}

// One per translation unit (search_f32.cu, search_bf16.cu, search_fp8.cu,
// search_bits.cu, search_learned.cu, search_multi.cu).
int launch_f32(const Params &p, int metric, int H, int S, cudaStream_t s);
int launch_bf16(const Params &p, int metric, int H, int S, cudaStream_t s);
int launch_fp8(const Params &p, int metric, int H, int S, cudaStream_t s);
int launch_bits(const Params &p, int metric, int S, cudaStream_t s);
int launch_learned(const Params &p, int storage, int metric, int H, int S, cudaStream_t s);
int launch_multi(const Params &p, int metric, int H, int S, cudaStream_t s);

}  // namespace song
