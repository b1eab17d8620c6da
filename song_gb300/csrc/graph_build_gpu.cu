// graph_build_gpu.cu -- the graph builder with each batch's searches on the GPU.
//
// The builder (graph_build.cpp) inserts vertices in batches; every new vertex
// runs the reference's CPU best-first search (graph.h:169-216) with result
// size `budget` against the graph as it stood before its batch.  This file
// runs those searches on the GPU, one warp per new vertex, and leaves the edge
// bookkeeping (graph.h:116-167) to graph_build.cpp.  The GPU search is the CPU
// search restated exactly, so the GPU builder writes the same graph as the CPU
// builder with the same batch_div, bit for bit:
//
//  * distances as data.h:28-62 computes them: float differences / products
//    (no contraction), accumulated in double in dimension order; cosine
//    divides by the two squared norms, each a float sum in dimension order;
//  * the queue is unbounded and ordered by (distance, id) like
//    std::pair<double, size_t>, the result list keeps the `budget` smallest
//    popped vertices by the same order, the search stops when the list is full
//    and its largest distance is below the next queue distance, and a vertex
//    enters the visited set when it is queued and never leaves it.
//
// A candidate farther than the maximum of a full result list is marked
// visited but not queued: the list's maximum only falls, so such a candidate
// could only ever be popped to end the search, which the next larger queue
// entry (or an empty queue) does just the same.
//
// One lane per candidate computes its distance (the double sum must run in
// dimension order); lane 0 keeps the two heaps.  Per warp: the result list
// and the query row in shared memory, the visited set (open addressing,
// insert-only, atomicCAS) and the queue heap in a device scratch region whose
// size is checked; a search that would overflow it flags the batch, which the
// host repeats with larger regions.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <vector>

#include "graph_build.h"
#include "internal.h"
#include "song_gb300.h"

namespace song {
namespace {

constexpr unsigned FULLM = 0xffffffffu;
constexpr uint32_t VIS_EMPTY = 0xffffffffu;
constexpr int BUILD_WARPS = 4;  // warps per block

struct QE {
  double d;
  uint32_t id;
  uint32_t pad;
};

__device__ __forceinline__ bool qless(const QE &a, const QE &b) {
  return a.d < b.d || (a.d == b.d && a.id < b.id);
}

struct BuildArgs {
  const float *data;     // n x dim
  const float *norms;    // cos: per-row squared norm (float, dimension order); else null
  const uint32_t *adj;   // n << shift
  int dim, metric, shift;
  uint64_t first;        // new vertices first .. first + count - 1
  uint32_t count;
  uint64_t limit;        // vertices inserted before the batch
  int budget;            // result size k of the search
  int out_k;             // ids written per vertex (search_degree)
  uint32_t *out;         // count x out_k
  int32_t *out_cnt;      // count
  uint32_t *vis;         // per warp: vis_cap slots
  uint32_t vis_cap;      // power of two
  int vis_log2;
  QE *q;                 // per warp: q_cap entries
  uint32_t q_cap;
  uint32_t *counter;
  int32_t *error;        // 1: visited set full, 2: queue full
};

// data.h:28-62 with a = base row, v = the query (in shared memory).
__device__ __forceinline__ double cpu_distance(const BuildArgs &p, const float *a, const float *v, float lena,
                                               float lenv) {
  double ret = 0.0;
  if (p.metric == SONG_METRIC_L2) {
    for (int i = 0; i < p.dim; ++i) {
      const float diff = __fsub_rn(__ldg(a + i), v[i]);
      ret = __dadd_rn(ret, static_cast<double>(__fmul_rn(diff, diff)));
    }
    return ret;
  }
  if (p.metric == SONG_METRIC_IP) {
    for (int i = 0; i < p.dim; ++i) ret = __dsub_rn(ret, static_cast<double>(__fmul_rn(__ldg(a + i), v[i])));
    return ret;
  }
  for (int i = 0; i < p.dim; ++i) ret = __dadd_rn(ret, static_cast<double>(__fmul_rn(__ldg(a + i), v[i])));
  const double sign = ret < 0 ? 1.0 : -1.0;
  return __dmul_rn(sign, __ddiv_rn(__ddiv_rn(__dmul_rn(ret, ret), static_cast<double>(lena)),
                                   static_cast<double>(lenv)));
}

// Insert-only visited set; true when id was not yet present.
__device__ __forceinline__ bool vis_insert(uint32_t *tab, uint32_t cap, int log2cap, uint32_t id) {
  uint32_t s = (id * 0x9E3779B1u) >> (32 - log2cap);
  for (uint32_t i = 0; i < cap; ++i) {
    const uint32_t old = atomicCAS(tab + s, VIS_EMPTY, id);
    if (old == VIS_EMPTY) return true;
    if (old == id) return false;
    s = (s + 1) & (cap - 1);
  }
  return false;  // unreachable: the fill is bounded below cap
}

// Min-heap (queue) and max-heap (result list) of QE, operated by one lane.
__device__ __forceinline__ void minheap_push(QE *h, uint32_t &n, const QE &e) {
  uint32_t i = n++;
  while (i > 0) {
    const uint32_t par = (i - 1) >> 1;
    const QE pe = h[par];
    if (!qless(e, pe)) break;
    h[i] = pe;
    i = par;
  }
  h[i] = e;
}

__device__ __forceinline__ void minheap_pop(QE *h, uint32_t &n) {
  const QE last = h[--n];
  uint32_t i = 0;
  for (;;) {
    uint32_t c = 2 * i + 1;
    if (c >= n) break;
    if (c + 1 < n && qless(h[c + 1], h[c])) ++c;
    const QE ce = h[c];
    if (!qless(ce, last)) break;
    h[i] = ce;
    i = c;
  }
  if (n > 0) h[i] = last;
}

__device__ __forceinline__ void maxheap_push(QE *h, int &n, const QE &e) {
  int i = n++;
  while (i > 0) {
    const int par = (i - 1) >> 1;
    const QE pe = h[par];
    if (!qless(pe, e)) break;
    h[i] = pe;
    i = par;
  }
  h[i] = e;
}

// Replace the maximum by e (e below it) and restore the heap.
__device__ __forceinline__ void maxheap_replace_top(QE *h, int n, const QE &e) {
  int i = 0;
  for (;;) {
    int c = 2 * i + 1;
    if (c >= n) break;
    if (c + 1 < n && qless(h[c], h[c + 1])) ++c;
    const QE ce = h[c];
    if (!qless(e, ce)) break;
    h[i] = ce;
    i = c;
  }
  h[i] = e;
}

__global__ void __launch_bounds__(BUILD_WARPS * 32) build_search_kernel(const BuildArgs p) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const size_t per_warp = static_cast<size_t>(p.budget) * sizeof(QE) + ((static_cast<size_t>(p.dim) * 4 + 15) & ~15ull);
  QE *T = reinterpret_cast<QE *>(smem + per_warp * wib);
  float *qv = reinterpret_cast<float *>(smem + per_warp * wib + static_cast<size_t>(p.budget) * sizeof(QE));
  const uint64_t gw = static_cast<uint64_t>(blockIdx.x) * BUILD_WARPS + wib;
  uint32_t *vis = p.vis + gw * p.vis_cap;
  QE *Q = p.q + gw * p.q_cap;
  const uint32_t vis_limit = p.vis_cap - (p.vis_cap >> 2);  // fill at most 3/4
  const uint32_t nslots = 1u << p.shift;

  for (;;) {
    uint32_t t = 0;
    if (lane == 0) t = atomicAdd(p.counter, 1u);
    t = __shfl_sync(FULLM, t, 0);
    if (t >= p.count) break;
    const uint64_t v = p.first + t;
    if (p.limit == 0) {  // the first vertex: nothing to search
      if (lane == 0) p.out_cnt[t] = 0;
      continue;
    }
    for (uint32_t i = lane; i < p.vis_cap; i += 32) vis[i] = VIS_EMPTY;
    const float *vrow = p.data + v * static_cast<uint64_t>(p.dim);
    for (int i = lane; i < p.dim; i += 32) qv[i] = vrow[i];
    const float lenv = p.norms ? p.norms[v] : 0.0f;
    __syncwarp();

    uint32_t qn = 0, vis_n = 1;
    int tn = 0;
    bool overflow = false;
    if (lane == 0) {
      vis_insert(vis, p.vis_cap, p.vis_log2, 0u);
      QE e;
      e.d = cpu_distance(p, p.data, qv, p.norms ? p.norms[0] : 0.0f, lenv);
      e.id = 0;
      e.pad = 0;
      minheap_push(Q, qn, e);
    }
    qn = __shfl_sync(FULLM, qn, 0);
    // Every lane holds the same qn, tn, vis_n and overflow at every branch:
    // lane 0 changes the heaps, and each change is broadcast before any lane
    // tests them.  The iteration cap is the reference's (graph.h:186).
    for (int iter = 0; iter < 1000000 && qn > 0; ++iter) {
      // graph.h:186-195: stop, or pop the minimum into the result list.
      QE now;
      int stop = 0;
      if (lane == 0) {
        now = Q[0];
        if (tn == p.budget && T[0].d < now.d) {
          stop = 1;
        } else {
          minheap_pop(Q, qn);
          if (tn < p.budget) maxheap_push(T, tn, now);
          else if (qless(now, T[0])) maxheap_replace_top(T, tn, now);
        }
      }
      stop = __shfl_sync(FULLM, stop, 0);
      if (stop) break;
      tn = __shfl_sync(FULLM, tn, 0);
      qn = __shfl_sync(FULLM, qn, 0);
      const uint32_t now_id = __shfl_sync(FULLM, lane == 0 ? now.id : 0u, 0);
      // graph.h:196-205: unvisited neighbours, one per lane.
      const uint32_t *row = p.adj + (static_cast<uint64_t>(now_id) << p.shift);
      const uint32_t deg = __ldg(row);
      uint32_t s = 0;
      bool fresh = false;
      for (uint32_t base = 1; base <= deg; base += 32) {
        const uint32_t slot = base + lane;
        s = 0;
        fresh = false;
        if (slot <= deg && slot < nslots) {
          s = __ldg(row + slot);
          fresh = vis_insert(vis, p.vis_cap, p.vis_log2, s);
        }
        const unsigned fm = __ballot_sync(FULLM, fresh);
        vis_n += __popc(fm);
        if (vis_n > vis_limit) overflow = true;
        double d = 0.0;
        if (fresh) d = cpu_distance(p, p.data + static_cast<uint64_t>(s) * p.dim, qv, p.norms ? p.norms[s] : 0.0f, lenv);
        // Queue the fresh candidates (lane order; the heap order does not
        // depend on it), skipping those beyond a full list's maximum.
        const double tmax = __shfl_sync(FULLM, (lane == 0 && tn == p.budget) ? T[0].d : 0.0, 0);
        const bool full = tn == p.budget;
        unsigned qm = __ballot_sync(FULLM, fresh && !(full && tmax < d));
        if (qn + __popc(qm) > p.q_cap) {
          overflow = true;
          qm = 0;
        }
        while (qm) {
          const int src = __ffs(qm) - 1;
          qm &= qm - 1;
          const double dd = __shfl_sync(FULLM, d, src);
          const uint32_t ss = __shfl_sync(FULLM, s, src);
          if (lane == 0) {
            QE e;
            e.d = dd;
            e.id = ss;
            e.pad = 0;
            minheap_push(Q, qn, e);
          }
        }
        qn = __shfl_sync(FULLM, qn, 0);
      }
      if (overflow) break;
    }
    if (overflow) {
      if (lane == 0) atomicOr(p.error, vis_n > vis_limit ? 1 : 2);
      continue;
    }
    // graph.h:207-215: the list in ascending order (in-place heap sort).
    if (lane == 0) {
      for (int i = tn - 1; i > 0; --i) {
        const QE top = T[0];
        maxheap_replace_top(T, i, T[i]);
        T[i] = top;
      }
    }
    __syncwarp();
    const int num = min(tn, p.out_k);
    for (int i = lane; i < num; i += 32) p.out[static_cast<uint64_t>(t) * p.out_k + i] = T[i].id;
    if (lane == 0) p.out_cnt[t] = tn;
    __syncwarp();
  }
}

// Squared norms of all rows, each a float sum in dimension order (data.h:50-62).
__global__ void row_norms_kernel(const float *data, uint64_t n, int dim, float *out) {
  for (uint64_t r = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; r < n;
       r += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
    const float *a = data + r * static_cast<uint64_t>(dim);
    float len = 0.0f;
    for (int i = 0; i < dim; ++i) len = __fadd_rn(len, __fmul_rn(a[i], a[i]));
    out[r] = len;
  }
}

// Scatter of changed adjacency rows: rows[i] (uint32 x 2^shift) goes to row ids[i].
__global__ void scatter_rows_kernel(const uint32_t *rows, const uint64_t *ids, uint64_t count, int shift,
                                    uint32_t *adj) {
  const uint32_t w = 1u << shift;
  const uint64_t total = count * w;
  for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < total;
       i += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
    const uint64_t r = i >> shift;
    adj[(ids[r] << shift) + (i & (w - 1))] = rows[i];
  }
}

struct DevBuf {
  void *p = nullptr;
  ~DevBuf() {
    if (p) cudaFree(p);
  }
};

struct HostPinned {
  void *p = nullptr;
  ~HostPinned() {
    if (p) cudaFreeHost(p);
  }
};

}  // namespace
}  // namespace song

extern "C" int song_graph_build_gpu(const float *data, uint64_t n, int dim, int metric, int shift,
                                    int search_degree, int fixed_degree, int budget, int batch_div,
                                    int device, int nthreads, uint64_t *graph_out) {
  using namespace song;
  clear_error();
  if (!data || !graph_out || n == 0 || dim <= 0) return fail(SONG_ERR_ARG, "graph build: null buffer or empty data");
  if (metric < SONG_METRIC_L2 || metric > SONG_METRIC_COS) return fail(SONG_ERR_ARG, "graph build: bad metric");
  if (shift < 1 || shift > 10) return fail(SONG_ERR_ARG, "graph build: shift must be 1..10");
  if (fixed_degree < 1 || fixed_degree > (1 << shift) - 1)
    return fail(SONG_ERR_ARG, "graph build: fixed_degree must be 1..2^shift-1");
  if (search_degree < 1 || search_degree > fixed_degree || budget < search_degree)
    return fail(SONG_ERR_ARG, "graph build: need 1 <= search_degree <= fixed_degree and budget >= search_degree");
  if (budget > 1024) return fail(SONG_ERR_ARG, "graph build: budget above 1024");
  if (batch_div < 0) return fail(SONG_ERR_ARG, "graph build: batch_div < 0");
  if (n >= (1ull << 32) - 1) return fail(SONG_ERR_ARG, "graph build: more than 2^32-2 vertices");
  if (nthreads < 1) nthreads = 1;
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return fail(SONG_ERR_CUDA, "graph build: cudaSetDevice: %s", cudaGetErrorString(e));
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  if (sms <= 0) sms = 1;

  GraphBuilder *gb = graph_builder_create(data, n, dim, metric, shift, search_degree, fixed_degree, budget);
  if (!gb) return fail(SONG_ERR_OOM, "graph build: host edge arrays");
  struct Guard {
    GraphBuilder *g;
    ~Guard() { graph_builder_free(g); }
  } guard{gb};

  const size_t per_warp_smem = static_cast<size_t>(budget) * sizeof(QE) + ((static_cast<size_t>(dim) * 4 + 15) & ~15ull);
  const size_t smem = per_warp_smem * BUILD_WARPS;
  int optin = 0;
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
  if (smem > static_cast<size_t>(optin)) return fail(SONG_ERR_ARG, "graph build: dim/budget need too much shared memory");
  e = cudaFuncSetAttribute(build_search_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
  if (e != cudaSuccess) return fail(SONG_ERR_CUDA, "graph build: %s", cudaGetErrorString(e));
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, build_search_kernel, BUILD_WARPS * 32, smem);
  if (per_sm < 1) return fail(SONG_ERR_ARG, "graph build: kernel does not fit on an SM");
  per_sm = std::min(per_sm, 8);  // 32 warps per SM: enough to hide the heap latency, bounded scratch
  const uint64_t blocks = static_cast<uint64_t>(sms) * per_sm;
  const uint64_t warps = blocks * BUILD_WARPS;

  cudaStream_t st;
  e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  if (e != cudaSuccess) return fail(SONG_ERR_CUDA, "graph build: %s", cudaGetErrorString(e));
  struct StreamGuard {
    cudaStream_t s;
    ~StreamGuard() { cudaStreamDestroy(s); }
  } sg{st};

  const uint64_t max_batch = batch_div == 0 ? 1 : std::max<uint64_t>(1, n / batch_div) + 1;
  const uint32_t w = 1u << shift;
  DevBuf d_data, d_norms, d_adj, d_out, d_cnt, d_ctl, d_vis, d_q, d_rows, d_ids;
  HostPinned h_out, h_cnt, h_err, h_rows, h_ids;
  const size_t rows_cap = static_cast<size_t>(max_batch) * (search_degree + 1);
#define SONG_GB_CK(call)                                                          \
  do {                                                                            \
    cudaError_t e_ = (call);                                                      \
    if (e_ != cudaSuccess)                                                        \
      return fail(e_ == cudaErrorMemoryAllocation ? SONG_ERR_OOM : SONG_ERR_CUDA, \
                  "graph build: %s: %s", #call, cudaGetErrorString(e_));          \
  } while (0)
  SONG_GB_CK(song::dev_malloc(&d_data.p, sizeof(float) * n * dim));
  SONG_GB_CK(song::dev_malloc(&d_adj.p, sizeof(uint32_t) * (n << shift)));
  SONG_GB_CK(song::dev_malloc(&d_out.p, sizeof(uint32_t) * max_batch * search_degree));
  SONG_GB_CK(song::dev_malloc(&d_cnt.p, sizeof(int32_t) * max_batch));
  SONG_GB_CK(song::dev_malloc(&d_ctl.p, 256));
  SONG_GB_CK(song::dev_malloc(&d_rows.p, sizeof(uint32_t) * rows_cap * w));
  SONG_GB_CK(song::dev_malloc(&d_ids.p, sizeof(uint64_t) * rows_cap));
  SONG_GB_CK(cudaMallocHost(&h_out.p, sizeof(uint32_t) * max_batch * search_degree));
  SONG_GB_CK(cudaMallocHost(&h_cnt.p, sizeof(int32_t) * max_batch));
  SONG_GB_CK(cudaMallocHost(&h_err.p, 256));
  SONG_GB_CK(cudaMallocHost(&h_rows.p, sizeof(uint32_t) * rows_cap * w));
  SONG_GB_CK(cudaMallocHost(&h_ids.p, sizeof(uint64_t) * rows_cap));
  SONG_GB_CK(cudaMemcpyAsync(d_data.p, data, sizeof(float) * n * dim, cudaMemcpyHostToDevice, st));
  SONG_GB_CK(cudaMemsetAsync(d_adj.p, 0, sizeof(uint32_t) * (n << shift), st));
  if (metric == SONG_METRIC_COS) {
    SONG_GB_CK(song::dev_malloc(&d_norms.p, sizeof(float) * n));
    row_norms_kernel<<<sms * 8, 256, 0, st>>>(static_cast<const float *>(d_data.p), n, dim,
                                              static_cast<float *>(d_norms.p));
    SONG_GB_CK(cudaGetLastError());
  }
  int vis_log2 = 13, q_log2 = 12;  // grown when a batch overflows
  auto alloc_scratch = [&]() -> int {
    if (d_vis.p) cudaFree(d_vis.p);
    if (d_q.p) cudaFree(d_q.p);
    d_vis.p = d_q.p = nullptr;
    cudaError_t e1 = song::dev_malloc(&d_vis.p, sizeof(uint32_t) * (warps << vis_log2));
    if (e1 == cudaSuccess) e1 = song::dev_malloc(&d_q.p, sizeof(QE) * (warps << q_log2));
    if (e1 != cudaSuccess)
      return fail(e1 == cudaErrorMemoryAllocation ? SONG_ERR_OOM : SONG_ERR_CUDA, "graph build: scratch: %s",
                  cudaGetErrorString(e1));
    return SONG_OK;
  };
  int rc = alloc_scratch();
  if (rc != SONG_OK) return rc;

  uint32_t *h_out32 = static_cast<uint32_t *>(h_out.p);
  int32_t *h_cnt32 = static_cast<int32_t *>(h_cnt.p);
  int32_t *h_err32 = static_cast<int32_t *>(h_err.p);
  std::vector<uint64_t> touched;
  const uint64_t *edges = graph_builder_edges(gb);
  uint64_t a = 0;
  while (a < n) {
    const uint64_t bs = batch_div == 0 ? 1 : std::max<uint64_t>(1, a / static_cast<uint64_t>(batch_div));
    const uint64_t end = std::min<uint64_t>(n, a + bs);
    for (int attempt = 0;; ++attempt) {
      BuildArgs p;
      p.data = static_cast<const float *>(d_data.p);
      p.norms = static_cast<const float *>(d_norms.p);
      p.adj = static_cast<const uint32_t *>(d_adj.p);
      p.dim = dim;
      p.metric = metric;
      p.shift = shift;
      p.first = a;
      p.count = static_cast<uint32_t>(end - a);
      p.limit = a;
      p.budget = budget;
      p.out_k = search_degree;
      p.out = static_cast<uint32_t *>(d_out.p);
      p.out_cnt = static_cast<int32_t *>(d_cnt.p);
      p.vis = static_cast<uint32_t *>(d_vis.p);
      p.vis_cap = 1u << vis_log2;
      p.vis_log2 = vis_log2;
      p.q = static_cast<QE *>(d_q.p);
      p.q_cap = 1u << q_log2;
      p.counter = static_cast<uint32_t *>(d_ctl.p);
      p.error = static_cast<int32_t *>(d_ctl.p) + 1;
      SONG_GB_CK(cudaMemsetAsync(d_ctl.p, 0, 8, st));
      const uint64_t grid = std::min<uint64_t>(blocks, (end - a + BUILD_WARPS - 1) / BUILD_WARPS);
      build_search_kernel<<<static_cast<unsigned>(grid), BUILD_WARPS * 32, smem, st>>>(p);
      SONG_GB_CK(cudaGetLastError());
      SONG_GB_CK(cudaMemcpyAsync(h_err32, p.error, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
      SONG_GB_CK(cudaMemcpyAsync(h_cnt32, d_cnt.p, sizeof(int32_t) * (end - a), cudaMemcpyDeviceToHost, st));
      SONG_GB_CK(cudaMemcpyAsync(h_out32, d_out.p, sizeof(uint32_t) * (end - a) * search_degree,
                                 cudaMemcpyDeviceToHost, st));
      SONG_GB_CK(cudaStreamSynchronize(st));
      if (*h_err32 == 0) break;
      if (attempt >= 6) return fail(SONG_ERR_OOM, "graph build: search scratch still too small after growing");
      if (*h_err32 & 1) ++vis_log2;
      if (*h_err32 & 2) ++q_log2;
      rc = alloc_scratch();
      if (rc != SONG_OK) return rc;
    }
    touched.clear();
    graph_builder_apply(gb, a, end, h_out32, h_cnt32, search_degree, nthreads, &touched);
    // upload the changed rows
    uint32_t *hr = static_cast<uint32_t *>(h_rows.p);
    uint64_t *hi = static_cast<uint64_t *>(h_ids.p);
    const uint64_t nt = touched.size();  // <= (end - a) * (search_degree + 1) <= rows_cap
    for (uint64_t i = 0; i < nt; ++i) {
      const uint64_t *src = edges + (touched[i] << shift);
      for (uint32_t j = 0; j < w; ++j) hr[i * w + j] = static_cast<uint32_t>(src[j]);
      hi[i] = touched[i];
    }
    SONG_GB_CK(cudaMemcpyAsync(d_rows.p, hr, sizeof(uint32_t) * nt * w, cudaMemcpyHostToDevice, st));
    SONG_GB_CK(cudaMemcpyAsync(d_ids.p, hi, sizeof(uint64_t) * nt, cudaMemcpyHostToDevice, st));
    const uint64_t blocks_s = std::min<uint64_t>(4096, (nt * w + 255) / 256);
    if (nt > 0) {
      scatter_rows_kernel<<<static_cast<unsigned>(blocks_s), 256, 0, st>>>(
          static_cast<const uint32_t *>(d_rows.p), static_cast<const uint64_t *>(d_ids.p), nt, shift,
          static_cast<uint32_t *>(d_adj.p));
      SONG_GB_CK(cudaGetLastError());
    }
    a = end;
  }
  SONG_GB_CK(cudaStreamSynchronize(st));
#undef SONG_GB_CK
  std::memcpy(graph_out, edges, sizeof(uint64_t) * (static_cast<size_t>(n) << shift));
  return SONG_OK;
}
