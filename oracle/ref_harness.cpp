// ref_harness.cpp -- C entry points around the REFERENCE's own source files.
//
// TEST INFRASTRUCTURE ONLY.  Built by oracle/build_ref.sh, in this container
// only (the reference tree is not present on the GPU host), into oracle/_ref/.
// It compiles, unmodified and where they lie in the reference tree:
//   config.h, data.h, graph.h      -- the CPU graph builder (graph.h:149-167)
//                                     and CPU best-first search (graph.h:169-216)
//   smmh2.h, bin_heap.h, fixhash.h -- the kernel's candidate queue, top-pq heap
//                                     and visited hash, made host-callable by
//                                     defining __device__ away.
// The search loop of warp_astar_accelerator.h:111-335 is a __global__ kernel
// and cannot run here; ref_kernel_search() below walks the same steps on one
// host thread and drives the reference containers with them, so that their
// tie order and their hash behaviour are the reference's.  It exists to pin
// oracle/song_oracle.c and to produce the golden fixtures in tests/golden/.
//
// Graph constants: build with -DREF_FIXED_DEGREE=.. -DREF_SHIFT=.. -DREF_SEARCH_DEGREE=..
// to get the degree-16 variant (README.md:79-80 sanctions editing config.h).
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <utility>
#include <vector>

#include "config.h"
#ifdef REF_FIXED_DEGREE
#undef FIXED_DEGREE
#define FIXED_DEGREE REF_FIXED_DEGREE
#endif
#ifdef REF_SHIFT
#undef FIXED_DEGREE_SHIFT
#define FIXED_DEGREE_SHIFT REF_SHIFT
#endif
#ifdef REF_SEARCH_DEGREE
#undef SEARCH_DEGREE
#define SEARCH_DEGREE REF_SEARCH_DEGREE
#endif
#include "data.h"
#include "graph.h"

#define __device__
#define __ENABLE_VISITED_DEL
#include "bin_heap.h"
#include "fixhash.h"
#include "smmh2.h"

namespace {

// astar_accelerator.h:19-38 cannot be included on the host (it declares a
// __global__ kernel); this is the same pair type, compared on .first only.
template <class A, class B>
struct KernelPair {
  A first;
  B second;
  KernelPair() {}
  bool operator<(const KernelPair &kp) const { return first < kp.first; }
  bool operator>(const KernelPair &kp) const { return first > kp.first; }
};

using KP = KernelPair<dist_t, idx_t>;

std::vector<std::pair<int, value_t>> dense_to_pairs(const float *v, int dim) {
  std::vector<std::pair<int, value_t>> p;
  p.reserve(dim);
  for (int i = 0; i < dim; ++i) p.push_back(std::make_pair(i, v[i]));
  return p;
}

template <int DT>
std::unique_ptr<GraphWrapper> make_graph(Data *d) {
  return std::unique_ptr<GraphWrapper>(new FixedDegreeGraph<DT>(d));
}

std::unique_ptr<GraphWrapper> graph_for(int metric, Data *d) {
  if (metric == 0) return make_graph<0>(d);
  if (metric == 1) return make_graph<1>(d);
  return make_graph<2>(d);
}

// Kernel distance, warp_astar_accelerator.h:237-287 with nvcc's default
// contraction of tmp += a * b into a fused multiply-add.
float kdist(int metric, int dim, const float *q, const float *x) {
  float t[32], l[32];
  for (int lane = 0; lane < 32; ++lane) {
    float a = 0, b = 0;
    for (int j = lane; j < dim; j += 32) {
      if (metric == 0) {
        float d = q[j] - x[j];
        a = std::fma(d, d, a);
      } else {
        a = std::fma(q[j], x[j], a);
        if (metric == 2) b = std::fma(x[j], x[j], b);
      }
    }
    t[lane] = a;
    l[lane] = b;
  }
  for (int off = 16; off > 0; off /= 2) {
    float nt[32], nl[32];
    for (int lane = 0; lane < 32; ++lane) {
      nt[lane] = t[lane] + t[lane ^ off];
      nl[lane] = l[lane] + l[lane ^ off];
    }
    std::memcpy(t, nt, sizeof t);
    std::memcpy(l, nl, sizeof l);
  }
  if (metric == 0) return t[0];
  if (metric == 1) return -t[0];
  int sign = t[0] < 0 ? 1 : -1;
  if (l[0] != 0) return sign * t[0] * t[0] / l[0];
  return 0;
}

// probes / finish_cnt: the N_MULTIPROBE / FINISH_CNT knobs of
// warp_astar_accelerator.h:29-30 (both 1 there); dcheck: the
// __ENABLE_MULTIPROBE_DOUBLE_CHECK switch (:307-310, off there).  An iteration pops up to
// `probes` vertices (:184), only its first pop takes the finish test, which
// counts (:190-192) and ends the search at finish_cnt (:196,227); the
// unvisited neighbours of all the iteration's pops are listed (:211-224)
// before the distances (:237-287) and the select-insert (:297-322).
template <int TOPK>
int kernel_search_one(const float *data, const uint64_t *graph, int dim, int shift, int metric,
                      const float *qv, uint64_t *out, int *hops_out, int *evals_out, int probes,
                      int finish_cnt, int dcheck) {
  const int QUEUE_SIZE = TOPK;
  FixHash<int, TOPK * 4 * 2> *pbf = new FixHash<int, TOPK * 4 * 2>();
  std::vector<KP> q(QUEUE_SIZE + 2), topk(TOPK + 1);
  std::vector<idx_t> index_list;
  std::vector<value_t> dist_list;
  int heap_size = 1, topk_heap_size = 0, hops = 0, evals = 1;
  float start_distance = kdist(metric, dim, qv, data);
  {
    KP kp;
    kp.first = start_distance;
    kp.second = 0;
    smmh2::insert(q.data(), heap_size, kp);
    pbf->add(0);
  }
  int finished = 0;
  while (heap_size > 1) {
    index_list.clear();
    const int current = heap_size - 1;
    for (int k = 0; k < probes && k < current; ++k) {
      KP now = smmh2::pop_min(q.data(), heap_size);
      pbf->del(now.second);
      if (k == 0 && topk_heap_size == TOPK && (topk[0].first <= now.first)) ++finished;
      if (finished >= finish_cnt) break;
      ++hops;
      topk[topk_heap_size++] = now;
      push_heap(topk.data(), topk.data() + topk_heap_size);
      pbf->add(now.second);
      if (topk_heap_size > TOPK) {
        pbf->del(topk[0].second);
        pop_heap(topk.data(), topk.data() + topk_heap_size);
        --topk_heap_size;
      }
      uint64_t offset = now.second << shift;
      int degree = graph[offset];
      for (int i = 1; i <= degree; ++i) {
        idx_t idx = graph[offset + i];
        if (pbf->test(idx)) continue;
        index_list.push_back(idx);
      }
    }
    if (finished >= finish_cnt) break;
    dist_list.resize(index_list.size());
    for (size_t i = 0; i < index_list.size(); ++i)
      dist_list[i] = kdist(metric, dim, qv, data + index_list[i] * (uint64_t)dim);
    evals += (int)index_list.size();
    for (size_t i = 0; i < index_list.size(); ++i) {
      dist_t d = dist_list[i];
      KP kp;
      kp.first = d;
      kp.second = index_list[i];
      if (heap_size >= QUEUE_SIZE + 1 && q[2].first < kp.first) continue;
      if (dcheck && pbf->test(kp.second)) continue;
      smmh2::insert(q.data(), heap_size, kp);
      pbf->add(kp.second);
      if (heap_size >= QUEUE_SIZE + 2) {
        pbf->del(q[2].second);
        smmh2::pop_max(q.data(), heap_size);
      }
    }
  }
  for (int i = 0; i < TOPK; ++i) out[i] = UINT64_MAX;
  int filled = topk_heap_size;
  for (int i = 0; i < filled; ++i) {
    KP e = pop_heap(topk.data(), topk.data() + filled - i);
    out[filled - 1 - i] = e.second;
  }
  delete pbf;
  *hops_out = hops;
  *evals_out = evals;
  return filled;
}

template <int P>
int dispatch(int pq, const float *data, const uint64_t *graph, int dim, int shift, int metric,
             const float *qv, uint64_t *out, int *h, int *e, int probes, int finish_cnt, int dcheck) {
  if (pq == P) return kernel_search_one<P>(data, graph, dim, shift, metric, qv, out, h, e, probes, finish_cnt, dcheck);
  return -2;
}

template <class H>
void run_fixhash_ops(H *h, const int32_t *ops, const int32_t *keys, int count, int32_t *results) {
  for (int i = 0; i < count; ++i) {
    results[i] = -1;
    if (ops[i] == 0) h->add(keys[i]);
    else if (ops[i] == 1) h->del(keys[i]);
    else results[i] = h->test(keys[i]) ? 1 : 0;
  }
}

}  // namespace

extern "C" {

int ref_graph_shift() { return FIXED_DEGREE_SHIFT; }
int ref_graph_fixed_degree() { return FIXED_DEGREE; }
int ref_graph_search_degree() { return SEARCH_DEGREE; }

// Sequential reference build (graph.h:149-167) in insertion order 0..n-1,
// exactly as main.cc's build_callback does; the graph is dumped with the
// reference's own dump() into graph_path.
int ref_build_graph(const float *data, uint64_t n, int dim, int metric, const char *graph_path,
                    const char *data_path) {
  Data d(n, dim);
  std::unique_ptr<GraphWrapper> g = graph_for(metric, &d);
  for (uint64_t i = 0; i < n; ++i) {
    std::vector<std::pair<int, value_t>> p = dense_to_pairs(data + i * (uint64_t)dim, dim);
    d.add(i, p);
    g->add_vertex(i, p);
  }
  g->dump(graph_path);
  d.dump(data_path);
  return 0;
}

// CPU best-first search (graph.h:169-216) over a loaded index, k results per
// query (UINT64_MAX past the result length).
int ref_cpu_search(const char *graph_path, const char *data_path, uint64_t n, int dim, int metric,
                   const float *queries, int nq, int k, uint64_t *out) {
  Data d(n, dim);
  d.load(data_path);
  std::unique_ptr<GraphWrapper> g = graph_for(metric, &d);
  g->load(graph_path);
  for (int i = 0; i < nq; ++i) {
    std::vector<idx_t> r;
    g->search_top_k(dense_to_pairs(queries + (uint64_t)i * dim, dim), k, r);
    for (int j = 0; j < k; ++j) out[(uint64_t)i * k + j] = j < (int)r.size() ? r[j] : UINT64_MAX;
  }
  return 0;
}

// Kernel search steps driven through the reference containers, with the
// N_MULTIPROBE / FINISH_CNT / __ENABLE_MULTIPROBE_DOUBLE_CHECK knobs as
// run-time values (1, 1, 0: the reference's defaults).
int ref_kernel_search_multi(const float *data, const uint64_t *graph, uint64_t n, int dim, int shift,
                            int metric, const float *queries, int nq, int pq, int probes, int finish_cnt,
                            int dcheck, uint64_t *out, int32_t *hops, int32_t *evals, int32_t *popped) {
  (void)n;
  if (probes < 1 || finish_cnt < 1) return -1;
  for (int i = 0; i < nq; ++i) {
    int h = 0, e = 0, r = -2;
    const float *qv = queries + (uint64_t)i * dim;
    uint64_t *o = out + (uint64_t)i * pq;
#define SONG_REF_P(P) \
  if (r == -2) r = dispatch<P>(pq, data, graph, dim, shift, metric, qv, o, &h, &e, probes, finish_cnt, dcheck);
    SONG_REF_P(2) SONG_REF_P(4) SONG_REF_P(8) SONG_REF_P(10) SONG_REF_P(16) SONG_REF_P(32)
    SONG_REF_P(50) SONG_REF_P(64) SONG_REF_P(100) SONG_REF_P(128) SONG_REF_P(150)
    SONG_REF_P(200) SONG_REF_P(256) SONG_REF_P(300) SONG_REF_P(400)
#undef SONG_REF_P
    if (r == -2) return -1;
    if (hops) hops[i] = h;
    if (evals) evals[i] = e;
    if (popped) popped[i] = r;
  }
  return 0;
}

int ref_kernel_search(const float *data, const uint64_t *graph, uint64_t n, int dim, int shift,
                      int metric, const float *queries, int nq, int pq, uint64_t *out,
                      int32_t *hops, int32_t *evals, int32_t *popped) {
  return ref_kernel_search_multi(data, graph, n, dim, shift, metric, queries, nq, pq, 1, 1, 0, out, hops, evals,
                                 popped);
}

// The reference FixHash on its own: ops[i] = 0 add, 1 del, 2 test of keys[i];
// results[i] = test answer (0/1) for tests, -1 otherwise.  cap = 8 * pq for
// pq in {8, 100}.
int ref_fixhash_ops(int pq, const int32_t *ops, const int32_t *keys, int count, int32_t *results) {
  if (pq == 8) {
    std::unique_ptr<FixHash<int, 64>> h(new FixHash<int, 64>());
    run_fixhash_ops(h.get(), ops, keys, count, results);
  } else if (pq == 100) {
    std::unique_ptr<FixHash<int, 800>> h(new FixHash<int, 800>());
    run_fixhash_ops(h.get(), ops, keys, count, results);
  } else {
    return -1;
  }
  return 0;
}

}  // extern "C"
