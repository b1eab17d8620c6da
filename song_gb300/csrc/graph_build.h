// graph_build.h -- the CPU half of the graph builder (graph_build.cpp) as
// used by the GPU builder (graph_build_gpu.cu): edge bookkeeping of
// FixedDegreeGraph::add_vertex (graph.h:149-167) applied one batch at a time.
#pragma once

#include <cstdint>
#include <vector>

namespace song {

struct GraphBuilder;

// nullptr when the edge arrays cannot be allocated.
GraphBuilder *graph_builder_create(const float *data, uint64_t n, int dim, int metric, int shift,
                                   int search_degree, int fixed_degree, int budget);
void graph_builder_free(GraphBuilder *g);

// Applies the search results of the new vertices a..e-1: vertex v's result is
// ids[(v-a)*ld .. (v-a)*ld + cnt[v-a] - 1], ascending by distance (only the
// first search_degree are used).  Rows changed are appended to *touched.
void graph_builder_apply(GraphBuilder *g, uint64_t a, uint64_t e, const uint32_t *ids, const int32_t *cnt,
                         int ld, int nthreads, std::vector<uint64_t> *touched);

// n << shift slots: the graph as built so far.
const uint64_t *graph_builder_edges(const GraphBuilder *g);

}  // namespace song
