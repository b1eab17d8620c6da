// graph_build.cpp -- builder of fixed-degree proximity graphs in the bfsg.graph
// layout (n << shift uint64 slots per file; slot 0 = out-degree, then
// zero-based neighbour ids).
//
// It follows the reference's CPU builder, FixedDegreeGraph::add_vertex
// (graph.h:149-167): every new vertex runs a best-first search with result
// size `budget` (graph.h:169-216, CONSTRUCT_SEARCH_BUDGET, config.h:27), keeps
// the `search_degree` nearest results as out-edges sorted by distance
// (rank_edges, graph.h:116-124, with the reference's own quicksort so that
// equal distances land where the reference puts them), and adds reverse edges
// (add_edge, graph.h:126-137): appended while the row holds fewer than
// `fixed_degree`, re-ranked when it fills, and afterwards replacing the
// farthest edge when closer (rank_and_switch, graph.h:32-55).
//
// batch_div == 0 inserts vertices one at a time, which reproduces the
// reference's graph exactly.  batch_div > 0 inserts them in batches of
// max(1, inserted / batch_div): the searches of one batch run in parallel
// against the graph as it stood before the batch, then the batch's edges are
// applied as if one vertex at a time in id order.  The result is
// deterministic for a given batch_div (independent of the thread count) but
// is not the sequential graph.
//
// Applying a batch in parallel is exact: a batch's vertices only add reverse
// edges to rows of vertices inserted before the batch, a row's updates
// depend on nothing but that row, and each row receives its updates in
// vertex-id order, as the sequential loop would give them.
//
// The searches of a batch can also run on the GPU (graph_build_gpu.cu, the
// same search restated exactly); this file then only applies the edges.
//
// Distances are the reference's CPU ones (data.h:28-62): float products
// accumulated in double; cosine divides by both squared norms kept in float.
// This file must be compiled without floating-point contraction.
#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#include "graph_build.h"
#include "song_gb300.h"

namespace {

struct Builder {
  const float *data;
  uint64_t n;
  int dim, metric, shift, search_degree, fixed_degree, budget;
  std::vector<uint64_t> edges;
  std::vector<double> edge_dist;

  const float *row(uint64_t i) const { return data + i * (uint64_t)dim; }

  // a: base row, v: the other vector (query or second base row)
  double dist(const float *a, const float *v) const {
    double ret = 0.0;
    if (metric == SONG_METRIC_L2) {
      for (int i = 0; i < dim; ++i) {
        float diff = a[i] - v[i];
        float sq = diff * diff;
        ret += (double)sq;
      }
      return ret;
    }
    if (metric == SONG_METRIC_IP) {
      for (int i = 0; i < dim; ++i) {
        float p = a[i] * v[i];
        ret -= (double)p;
      }
      return ret;
    }
    float lena = 0.0f, lenv = 0.0f;
    for (int i = 0; i < dim; ++i) {
      float p = a[i] * v[i];
      ret += (double)p;
      float pa = a[i] * a[i];
      lena = lena + pa;
      float pv = v[i] * v[i];
      lenv = lenv + pv;
    }
    int sign = ret < 0 ? 1 : -1;
    return (double)sign * (ret * ret / (double)lena / (double)lenv);
  }

  // graph.h:98-114, kept as written (Hoare partition, middle pivot).
  void qsort_range(size_t l, size_t r) {
    size_t mid = (l + r) >> 1;
    long long i = (long long)l, j = (long long)r;
    double k = edge_dist[mid];
    do {
      while (edge_dist[i] < k) ++i;
      while (k < edge_dist[j]) --j;
      if (i <= j) {
        std::swap(edge_dist[i], edge_dist[j]);
        std::swap(edges[i], edges[j]);
        ++i;
        --j;
      }
    } while (i <= j);
    if ((size_t)i < r) qsort_range((size_t)i, r);
    if (j >= 0 && l < (size_t)j) qsort_range(l, (size_t)j);
  }

  void rank_edges(size_t off) {
    uint64_t deg = edges[off];
    const float *a = row(off >> shift);
    for (uint64_t i = 0; i < deg; ++i) edge_dist[off + i + 1] = dist(a, row(edges[off + i + 1]));
    if (deg > 0) qsort_range(off + 1, off + deg);
  }

  void rank_and_switch(uint64_t v, uint64_t u) {
    double curr = dist(row(v), row(u));
    size_t off = (size_t)v << shift;
    size_t last = off + edges[off];
    if (curr >= edge_dist[last]) return;
    edges[last] = u;
    edge_dist[last] = curr;
    for (size_t i = last - 1; i > off; --i) {
      if (edge_dist[i] > edge_dist[i + 1]) {
        std::swap(edges[i], edges[i + 1]);
        std::swap(edge_dist[i], edge_dist[i + 1]);
      } else {
        break;
      }
    }
  }

  void add_edge(uint64_t v, uint64_t u) {
    size_t off = (size_t)v << shift;
    if (edges[off] < (uint64_t)fixed_degree) {
      ++edges[off];
      edges[off + edges[off]] = u;
      if (edges[off] == (uint64_t)fixed_degree) rank_edges(off);
    } else {
      rank_and_switch(v, u);
    }
  }

  // Edges of the new vertices a..e-1 (nb(v): its search result, ascending),
  // row-parallel over nthreads; the rows changed are appended to *touched.
  template <class NB>
  void apply_batch(uint64_t a, uint64_t e, NB nb, int nthreads, std::vector<uint64_t> *touched) {
    const uint64_t m = e - a;
    std::vector<std::pair<uint64_t, uint64_t>> upd;  // (target row, new vertex)
    for (uint64_t v = a; v < e; ++v) {
      const uint64_t *ids;
      int cnt;
      nb(v, &ids, &cnt);
      const int num = std::min<int>(search_degree, cnt);
      for (int i = 0; i < num; ++i) upd.push_back({ids[i], v});
    }
    std::sort(upd.begin(), upd.end());
    std::vector<size_t> starts;  // one group per distinct target row
    for (size_t i = 0; i < upd.size(); ++i)
      if (i == 0 || upd[i].first != upd[i - 1].first) starts.push_back(i);
    starts.push_back(upd.size());
    const size_t groups = starts.size() - 1;
    auto own = [&](uint64_t v) {
      const uint64_t *ids;
      int cnt;
      nb(v, &ids, &cnt);
      const int num = std::min<int>(search_degree, cnt);
      size_t off = (size_t)v << shift;
      edges[off] = (uint64_t)num;
      for (int i = 0; i < num; ++i) edges[off + i + 1] = ids[i];
      rank_edges(off);
    };
    auto rev = [&](size_t g) {
      for (size_t i = starts[g]; i < starts[g + 1]; ++i) add_edge(upd[i].first, upd[i].second);
    };
    const uint64_t work = m + groups;
    int nt = (int)std::min<uint64_t>((uint64_t)std::max(1, nthreads), work / 16 + 1);
    if (nt <= 1) {
      for (uint64_t v = a; v < e; ++v) own(v);
      for (size_t g = 0; g < groups; ++g) rev(g);
    } else {
      std::atomic<uint64_t> next(0);
      auto worker = [&]() {
        for (;;) {
          uint64_t i = next.fetch_add(1);
          if (i >= work) break;
          if (i < m) own(a + i);
          else rev((size_t)(i - m));
        }
      };
      std::vector<std::thread> th;
      for (int t = 0; t < nt; ++t) th.emplace_back(worker);
      for (auto &x : th) x.join();
    }
    if (touched) {
      for (uint64_t v = a; v < e; ++v) touched->push_back(v);
      for (size_t g = 0; g < groups; ++g) touched->push_back(upd[starts[g]].first);
    }
  }

  void apply(uint64_t v, const std::vector<uint64_t> &nb) {
    int num = std::min<int>(search_degree, (int)nb.size());
    size_t off = (size_t)v << shift;
    edges[off] = (uint64_t)num;
    for (int i = 0; i < num; ++i) edges[off + i + 1] = nb[i];
    rank_edges(off);
    for (int i = 0; i < num; ++i) add_edge(nb[i], v);
  }
};

struct Pair {
  double d;
  uint64_t id;
};
inline bool pless(const Pair &a, const Pair &b) { return a.d < b.d || (a.d == b.d && a.id < b.id); }
struct MinCmp {
  bool operator()(const Pair &a, const Pair &b) const { return pless(b, a); }
};
struct MaxCmp {
  bool operator()(const Pair &a, const Pair &b) const { return pless(a, b); }
};

// Best-first search of graph.h:169-216 over the vertices inserted so far
// (`limit` of them; a search with limit 0 finds nothing).
struct Searcher {
  const Builder *b;
  std::vector<uint8_t> visited;
  std::vector<uint64_t> touched;
  std::vector<Pair> q, t;

  explicit Searcher(const Builder *bb) : b(bb), visited(bb->n, 0) {}

  void search(const float *qv, uint64_t limit, int k, std::vector<uint64_t> &result) {
    result.clear();
    q.clear();
    t.clear();
    touched.clear();
    if (limit > 0) {
      visited[0] = 1;
      touched.push_back(0);
      q.push_back({b->dist(b->row(0), qv), 0});
    }
    for (int iter = 0; iter < 1000000 && !q.empty(); ++iter) {
      Pair now = q.front();
      if ((int)t.size() == k && t.front().d < now.d) break;
      std::pop_heap(q.begin(), q.end(), MinCmp());
      q.pop_back();
      t.push_back(now);
      std::push_heap(t.begin(), t.end(), MaxCmp());
      if ((int)t.size() > k) {
        std::pop_heap(t.begin(), t.end(), MaxCmp());
        t.pop_back();
      }
      size_t off = (size_t)now.id << b->shift;
      uint64_t degree = b->edges[off];
      for (uint64_t i = 0; i < degree; ++i) {
        uint64_t s = b->edges[off + i + 1];
        if (visited[s]) continue;
        q.push_back({b->dist(b->row(s), qv), s});
        std::push_heap(q.begin(), q.end(), MinCmp());
        visited[s] = 1;
        touched.push_back(s);
      }
    }
    std::sort(t.begin(), t.end(), pless);
    for (const Pair &p : t) result.push_back(p.id);
    for (uint64_t s : touched) visited[s] = 0;
  }
};

}  // namespace

extern "C" int song_graph_build(const float *data, uint64_t n, int dim, int metric, int shift,
                                int search_degree, int fixed_degree, int budget, int batch_div,
                                int nthreads, uint64_t *graph_out) {
  if (!data || !graph_out || n == 0 || dim <= 0) return SONG_ERR_ARG;
  if (metric < SONG_METRIC_L2 || metric > SONG_METRIC_COS) return SONG_ERR_ARG;
  if (shift < 1 || shift > 10) return SONG_ERR_ARG;
  if (fixed_degree < 1 || fixed_degree > (1 << shift) - 1) return SONG_ERR_ARG;
  if (search_degree < 1 || search_degree > fixed_degree || budget < search_degree) return SONG_ERR_ARG;
  if (batch_div < 0 || (n << shift) >= (1ull << 40)) return SONG_ERR_ARG;
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 256) nthreads = 256;

  Builder b;
  b.data = data;
  b.n = n;
  b.dim = dim;
  b.metric = metric;
  b.shift = shift;
  b.search_degree = search_degree;
  b.fixed_degree = fixed_degree;
  b.budget = budget;
  try {
    b.edges.assign((size_t)n << shift, 0);
    b.edge_dist.assign((size_t)n << shift, 0.0);
  } catch (...) {
    return SONG_ERR_OOM;
  }

  if (batch_div == 0) {
    Searcher s(&b);
    std::vector<uint64_t> nb;
    for (uint64_t v = 0; v < n; ++v) {
      // data.h:139-144 sets curr_num = max(curr_num, idx) before add_vertex,
      // so vertex v searches from vertex 0 when v > 0.
      s.search(b.row(v), v, budget, nb);
      b.apply(v, nb);
    }
  } else {
    std::vector<Searcher> searchers;
    searchers.reserve(nthreads);
    for (int t = 0; t < nthreads; ++t) searchers.emplace_back(&b);
    std::vector<std::vector<uint64_t>> res;
    uint64_t a = 0;
    while (a < n) {
      uint64_t bs = std::max<uint64_t>(1, a / (uint64_t)batch_div);
      uint64_t e = std::min<uint64_t>(n, a + bs);
      res.assign(e - a, std::vector<uint64_t>());
      std::atomic<uint64_t> next(a);
      int nt = (int)std::min<uint64_t>((uint64_t)nthreads, e - a);
      auto work = [&](int tid) {
        for (;;) {
          uint64_t v = next.fetch_add(1);
          if (v >= e) break;
          searchers[tid].search(b.row(v), a, budget, res[v - a]);
        }
      };
      if (nt <= 1) {
        work(0);
      } else {
        std::vector<std::thread> th;
        for (int t = 0; t < nt; ++t) th.emplace_back(work, t);
        for (auto &x : th) x.join();
      }
      b.apply_batch(a, e, [&](uint64_t v, const uint64_t **ids, int *cnt) {
        *ids = res[v - a].data();
        *cnt = (int)res[v - a].size();
      }, nthreads, nullptr);
      a = e;
    }
  }
  std::memcpy(graph_out, b.edges.data(), sizeof(uint64_t) * ((size_t)n << shift));
  return SONG_OK;
}

// ---------------------------------------------------------------------------
// Interface for the GPU searches (graph_build.h)
// ---------------------------------------------------------------------------

namespace song {

struct GraphBuilder {
  Builder b;
};

GraphBuilder *graph_builder_create(const float *data, uint64_t n, int dim, int metric, int shift,
                                   int search_degree, int fixed_degree, int budget) {
  GraphBuilder *g = nullptr;
  try {
    g = new GraphBuilder();
    Builder &b = g->b;
    b.data = data;
    b.n = n;
    b.dim = dim;
    b.metric = metric;
    b.shift = shift;
    b.search_degree = search_degree;
    b.fixed_degree = fixed_degree;
    b.budget = budget;
    b.edges.assign((size_t)n << shift, 0);
    b.edge_dist.assign((size_t)n << shift, 0.0);
  } catch (...) {
    delete g;
    return nullptr;
  }
  return g;
}

void graph_builder_free(GraphBuilder *g) { delete g; }

void graph_builder_apply(GraphBuilder *g, uint64_t a, uint64_t e, const uint32_t *ids, const int32_t *cnt,
                         int ld, int nthreads, std::vector<uint64_t> *touched) {
  std::vector<uint64_t> wide((size_t)(e - a) * (size_t)ld);
  for (size_t i = 0; i < wide.size(); ++i) wide[i] = ids[i];
  g->b.apply_batch(a, e, [&](uint64_t v, const uint64_t **p, int *c) {
    *p = wide.data() + (size_t)(v - a) * (size_t)ld;
    *c = cnt[v - a];
  }, nthreads, touched);
}

const uint64_t *graph_builder_edges(const GraphBuilder *g) { return g->b.edges.data(); }

}  // namespace song
