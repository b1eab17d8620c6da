/*
 * song_oracle.h -- CPU oracle for the batched best-first graph search.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product (song_gb300/, include/)
 * links, imports or calls this code; only tests/, __graft_entry__.smoke() and
 * the cpu_baseline / reference legs of bench.py do, and only as the correctness reference or
 * the timed CPU baseline.
 *
 * It restates, in plain C, three algorithms of sunbelbd/song:
 *
 *  1. the warp search kernel  (warp_astar_accelerator.h:41-341), with its
 *     symmetric min-max candidate queue (smmh2.h:3-164), its top-pq binary
 *     max-heap (bin_heap.h:3-47) and its open-addressing visited hash with
 *     backward-shift delete (fixhash.h:3-109, default build flags
 *     -D__ENABLE_FIXHASH -D__ENABLE_VISITED_DEL, Makefile:21).
 *     Mode ORC_MODE_REF keeps the reference's heap structures, so the order
 *     in which equal distances leave the queues is the reference's own.
 *     Mode ORC_MODE_LEX is the GB300 kernel's specification: the same search,
 *     the same visited-hash operation sequence, but the queues are kept sorted
 *     by the key (distance, id), so equal distances leave in id order.  The two
 *     modes agree on every query in which no decision compares two different
 *     ids at the same distance; orc_classify() finds the first decision at
 *     which they part and says whether it is such a tie.
 *
 *  2. the CPU best-first search (graph.h:169-216) that the reference's graph
 *     builder runs and that song.cpu times: unbounded queue, permanent visited
 *     set, std::pair ordering (distance, id).
 *
 *  3. the distance arithmetic of each: the kernel's lane-strided FP32 sums
 *     with the xor butterfly (warp_astar_accelerator.h:115-163, :237-287) and
 *     the CPU's float products accumulated in double (data.h:28-62).
 *
 * Parity with the reference is pinned by tests/golden/ fixtures produced by
 * the reference's own containers and CPU code (oracle/ref_harness.cpp).
 */
#ifndef SONG_ORACLE_H
#define SONG_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_L2 = 0, ORC_IP = 1, ORC_COS = 2,       /* KernelFixedDegreeGraph<0|1|2> */
       ORC_HAMMING = 3 };                         /* rows are 256-bit codes (8 words, dim = 8) */
/* ORC_MODE_LEX_EXACT: LEX with an exact visited multiset instead of FixHash
 * (the learned/low-precision kernel's visited set, which never loses an entry). */
enum { ORC_MODE_REF = 0, ORC_MODE_LEX = 1, ORC_MODE_LEX_EXACT = 2 };

/* Output slot that the search did not fill (fewer than pq vertices popped). */
#define ORC_NO_ID UINT64_MAX

/* Event kinds of the per-query decision log used by orc_classify(). */
enum {
  ORC_EV_POP = 1,     /* candidate queue minimum removed            */
  ORC_EV_FINISH = 2,  /* search stopped on the popped vertex          */
  ORC_EV_TEVICT = 3,  /* top-pq maximum dropped                       */
  ORC_EV_SKIP = 4,    /* candidate rejected by the select-insert test */
  ORC_EV_INSERT = 5,  /* candidate inserted                           */
  ORC_EV_QEVICT = 6,  /* candidate queue maximum dropped              */
  ORC_EV_TEST = 7,    /* neighbour passed the visited test            */
  ORC_EV_OUT = 8      /* one output slot, ascending                   */
};

typedef struct {
  int32_t kind;
  uint32_t pad;
  uint64_t id;
  float dist;
  uint32_t pad2;
} orc_event;

/* Index view: bfsg.data (n x dim float32) and bfsg.graph (n << shift uint64,
 * slot 0 = out-degree, then zero-based neighbour ids). */
typedef struct {
  const float *data;
  const uint64_t *graph;
  uint64_t n;
  int32_t dim;
  int32_t shift;
  int32_t metric;
  int32_t pad;
} orc_index;

/* Kernel distance of one base row x to query q: lane l of a 32-wide warp sums
 * dims l, l+32, ... with fused multiply-add (use_fma=1, nvcc's default
 * contraction) or separate multiply and add (use_fma=0); partial sums are
 * combined by the xor butterfly 16,8,4,2,1. */
float orc_kernel_distance(int metric, int dim, const float *q, const float *x, int use_fma);

/* CPU distance of data.h:28-62 (x = base row, q = query). */
double orc_cpu_distance(int metric, int dim, const float *x, const float *q);

/* Batched kernel-semantics search.  out: nq x pq ids (ascending distance);
 * hops/evals/popped may be NULL.  Returns 0, or -1 on bad arguments. */
int orc_kernel_search(const orc_index *ix, const float *queries, int nq, int pq, int mode,
                      int use_fma, uint64_t *out, int32_t *hops, int32_t *evals,
                      int32_t *popped, int nthreads);

/* orc_kernel_search with query i starting from the ns vertices
 * starts[i*ns .. i*ns+ns-1] (queued and marked visited in that order before
 * the first pop) instead of vertex 0 (starts NULL: vertex 0 for all). */
int orc_kernel_search_from(const orc_index *ix, const float *queries, int nq, const uint64_t *starts, int ns,
                           int pq, int mode, int use_fma, uint64_t *out, int32_t *hops, int32_t *evals,
                           int32_t *popped, int nthreads);

/* orc_kernel_search_from with the reference's search knobs: `probes`
 * (N_MULTIPROBE, warp_astar_accelerator.h:29; 1..ORC_MAX_PROBES) vertices
 * popped per iteration -- only an iteration's first pop takes the finish
 * test, and the neighbours of all its pops are filtered before their
 * distances are computed and select-inserted in order (:184-232);
 * `finish_cnt` (FINISH_CNT, :30; >= 1): the search ends when the finish test
 * has held that many times (:190-197); `double_check`
 * (__ENABLE_MULTIPROBE_DOUBLE_CHECK, :307-310): the select-insert skips a
 * candidate already in the visited set. */
#define ORC_MAX_PROBES 4
int orc_kernel_search_multi(const orc_index *ix, const float *queries, int nq, const uint64_t *starts, int ns,
                            int pq, int probes, int finish_cnt, int double_check, int mode, int use_fma,
                            uint64_t *out, int32_t *hops, int32_t *evals, int32_t *popped, int nthreads);

/* Entry-point choice: starts[i*ns ..] = the ns entries with the smallest
 * kernel distance to query i, ascending by (distance, id). */
int orc_nearest_entry(const orc_index *ix, const float *queries, int nq, const uint64_t *entries, int ne,
                      int ns, int use_fma, uint64_t *starts);

/* Two-level entry choice: entries[0..coarse-1] are coarse entries, each its
 * own cluster; every other entry joins its nearest coarse entry's cluster
 * (the entry's row as the query, ties to the smaller id).  Query i probes its
 * `probes` nearest coarse entries and gets the ns nearest entries of those
 * clusters in starts[i*ns ..] (ascending; ns <= probes <= coarse), on
 * nthreads threads. */
int orc_nearest_entry_2level(const orc_index *ix, const float *queries, int nq, const uint64_t *entries, int ne,
                             int coarse, int probes, int ns, int use_fma, uint64_t *starts, int nthreads);

/* One query with its decision log (at most cap events; *n_events gets the
 * number produced, which may exceed cap). */
int orc_kernel_search_log(const orc_index *ix, const float *query, int pq, int mode, int use_fma,
                          uint64_t *out, orc_event *log, int cap, int *n_events);
int orc_kernel_search_log_multi(const orc_index *ix, const float *query, int pq, int probes, int finish_cnt,
                                int double_check, int mode, int use_fma, uint64_t *out, orc_event *log, int cap, int *n_events);

/* One LEX / LEX_EXACT query with the learned search kernel's per-hop trace:
 * for hop h < min(hops, trace_hops), trace[h*ORC_TRACE_FIELDS + 0..4] are the
 * early-exit features after hop h+1 and [.. + 5] the number of changes of the
 * top-k set so far; *final_version gets that number at the end and *traced
 * min(hops, trace_hops).  out: pq ids.  Returns 0, or -1 on bad arguments. */
#define ORC_TRACE_FIELDS 6
int orc_kernel_search_trace(const orc_index *ix, const float *query, int pq, int k, int mode,
                            int use_fma, int trace_hops, float *trace, int32_t *final_version,
                            int32_t *traced, uint64_t *out, int32_t *hops, int32_t *evals);

/* Compare the REF and LEX logs of one query.  Returns 0 if identical, 1 if the
 * first difference is a tie (same event kind, same distance, different id),
 * 2 if it is anything else.  *at gets the index of the first difference. */
int orc_classify(const orc_event *a, int na, const orc_event *b, int nb, int *at);

/* CPU best-first search of graph.h:169-216 with result size k.  out: nq x k
 * (ORC_NO_ID past the result length); explored may be NULL. */
/* 256-bit sign codes of n rows from 256 hyperplanes (planes: 256 x dim),
 * codes: n x 8 words, bit i = (row . plane_i >= 0) summed as the kernel sums. */
int orc_hash_codes(const float *rows, uint64_t n, int dim, const float *planes, int use_fma, uint32_t *codes);

/* The reference's CPU graph builder (graph.h:149-167 with graph.h:32-55,
 * 98-137): batch_div 0 inserts one vertex at a time (the reference's graph);
 * batch_div > 0 inserts batches of max(1, inserted / batch_div) vertices,
 * each searched against the graph before its batch on nthreads threads and
 * applied in id order.  graph_out: n << shift uint64 (bfsg.graph layout). */
int orc_graph_build(const float *data, uint64_t n, int dim, int metric, int shift, int search_degree,
                    int fixed_degree, int budget, int batch_div, int nthreads, uint64_t *graph_out);

int orc_cpu_search(const orc_index *ix, const float *queries, int nq, int k, uint64_t *out,
                   int32_t *explored, int nthreads);

/* The visited hash on its own, for unit tests: a table of 8*pq int32 slots. */
int orc_fixhash_hash(int cap, uint64_t x);
void orc_fixhash_init(int32_t *tab, int cap);
void orc_fixhash_add(int32_t *tab, int cap, int32_t x);
int orc_fixhash_test(const int32_t *tab, int cap, int32_t x);
void orc_fixhash_del(int32_t *tab, int cap, int32_t x);

#ifdef __cplusplus
}
#endif
#endif
