/*
 * song_gb300.h -- C ABI of the GB300 (sm_103a) batched best-first graph search.
 *
 * A drop-in for the GPU search path of sunbelbd/song:
 *
 *   GraphWrapper::search_top_k_batch(queries, k, results)          kernelgraph.h:20, :269-272
 *     -> WarpAStarAccelerator::astar_multi_start_search_batch(
 *            queries, k, results, h_data, h_graph, vertex_offset_shift, num, dim)
 *                                                                   warp_astar_accelerator.h:347-423
 *     -> warp_independent_search_kernel<<<nq, 32>>>(...)            warp_astar_accelerator.h:41-341
 *
 * Inputs are the reference's own formats: base vectors as bfsg.data (n x dim
 * float32, row-major; data.h:164-175) and the graph as bfsg.graph (n << shift
 * uint64 slots, slot 0 = out-degree, then zero-based neighbour ids;
 * README.md:83-89, kernelgraph.h:255-267).  Results are zero-based ids in
 * ascending distance order, the first k of the pq_size best, as the
 * reference CLI prints them (main.cu:28-32).
 *
 * The reference fixes pq_size (TOPK), dim (DIM) and the metric at compile
 * time (fill_parameters.sh:35-65); here they are run-time arguments.
 *
 * Every call returns a status code.  An index is uploaded once and stays
 * resident.  One index may be searched from one host thread at a time; a
 * search is ordered on the stream it is given.
 */
#ifndef SONG_GB300_H
#define SONG_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  The reference has no error reporting at all
 * (warp_astar_accelerator.h:353-423 checks no CUDA call). */
#define SONG_OK 0
#define SONG_ERR_ARG 1     /* an argument is out of range or the graph is malformed */
#define SONG_ERR_OOM 2     /* device or host allocation failed                    */
#define SONG_ERR_TIMEOUT 3 /* a bounded device wait gave up                       */
#define SONG_ERR_CUDA 4    /* a CUDA runtime call failed                          */
#define SONG_ERR_IO 5      /* a file could not be opened or was too short         */

/* Metrics: the reference's __USE_L2_DIST / __USE_IP_DIST / __USE_COS_DIST
 * (Makefile:3, fill_parameters.sh:55-65), in KernelFixedDegreeGraph<0|1|2>
 * order (main.cu:66-75).  L2 = squared Euclidean; IP = negative inner
 * product; COS = -sign(q.x) (q.x)^2 / |x|^2 as the GPU kernel computes it
 * (warp_astar_accelerator.h:275-281). */
#define SONG_METRIC_L2 0
#define SONG_METRIC_IP 1
#define SONG_METRIC_COS 2

/* Device storage of the base vectors.  F32 is the reference's value_t
 * (config.h:11).  BF16 and FP8 (E4M3 with one float scale per vector) are
 * additions with no counterpart in the reference; their final candidates are
 * re-ranked with FP32 distances. */
#define SONG_STORAGE_F32 0
#define SONG_STORAGE_BF16 1
#define SONG_STORAGE_FP8 2
/* 256-bit sign codes searched by Hamming distance: the reference's bit-hash
 * path (hash_warp_no_heap_astar_accelerator.h:22-41 codes, __popc distances
 * :96-104, 226-235) as a row format of the same search; needs the index's
 * hyperplanes (song_index_set_hash_planes) before the first search, and
 * re-ranks the final candidates with FP32 distances of the index's metric. */
#define SONG_STORAGE_BITS 3
#define SONG_HASH_BITS 256

/* Limits of this implementation. */
#define SONG_MAX_PQ 1023   /* the reference's FixHash casts its slot to short: 8*pq < 32768 */
#define SONG_MAX_SHIFT 5   /* up to 31 neighbours per vertex, as FIXED_DEGREE (config.h:22) */

typedef struct song_index song_index;

/* Human-readable text of a status code. */
const char *song_status_string(int status);

/* Text of the last error raised on the calling host thread ("" if none). */
const char *song_last_error(void);

/* Create a resident index on CUDA device `device` from host arrays in the
 * reference layouts.  `graph` has n << shift uint64 entries; every degree must
 * be <= (1 << shift) - 1 and every neighbour id < n.  `data` is n x dim.
 * Replaces the per-call upload of warp_astar_accelerator.h:353-356. */
int song_index_create(const uint64_t *graph, const float *data, uint64_t n, int dim, int shift,
                      int metric, int storage, int device, song_index **out);

/* The same from bfsg.graph / bfsg.data files (kernelgraph.h:262-267,
 * data.h:170-175).  As in the reference, n and dim are not stored in the
 * files and must be given. */
int song_index_load(const char *graph_path, const char *data_path, uint64_t n, int dim, int shift,
                    int metric, int storage, int device, song_index **out);

int song_index_free(song_index *index);

/* Properties of an index (any pointer may be NULL). */
int song_index_info(const song_index *index, uint64_t *n, int *dim, int *shift, int *metric,
                    int *storage, uint64_t *device_bytes);

/* Batched search with HOST buffers: copies nq x dim float queries to the
 * device, searches, copies nq x k uint64 ids back, and returns when done.
 * 2 <= pq <= SONG_MAX_PQ, 1 <= k <= pq.  hops and evals (nq int32 each) may be
 * NULL; they receive per query the number of vertices expanded and of
 * distances computed.  This is the e2e call that replaces
 * astar_multi_start_search_batch (warp_astar_accelerator.h:347). */
int song_search(song_index *index, const float *queries, int nq, int pq, int k, uint64_t *out,
                int32_t *hops, int32_t *evals);

/* Batched search with DEVICE buffers, enqueued on `stream` (a cudaStream_t,
 * NULL = the legacy default stream) without synchronising.  Searches of one
 * index must not overlap on the device (issue them on one stream, or order
 * the streams): they share the index's work counter, error flag and, with
 * entry points set, its buffer of chosen starts. */
int song_search_device(song_index *index, const float *d_queries, int nq, int pq, int k,
                       uint64_t *d_out, int32_t *d_hops, int32_t *d_evals, void *stream);

/* One-shot form with the reference's own argument list
 * (warp_astar_accelerator.h:347): uploads data and graph, searches, frees.
 * results: nq x pq ids, as d_result (warp_astar_accelerator.h:334).  The
 * reference's `k` argument is ignored there and has no counterpart here. */
int song_astar_search_batch(const float *queries, int nq, int pq, uint64_t *results,
                            const float *h_data, const uint64_t *h_graph, int vertex_offset_shift,
                            uint64_t num, int dim, int metric);

/* Graph construction (graph.h:149-167 with config.h:22-27 constants as
 * arguments): fills graph_out (n << shift uint64) in the bfsg.graph layout.
 * batch_div = 0 reproduces the reference's sequential insertion exactly;
 * batch_div > 0 inserts in deterministic parallel batches of
 * max(1, inserted / batch_div) vertices on nthreads host threads. */
int song_graph_build(const float *data, uint64_t n, int dim, int metric, int shift,
                     int search_degree, int fixed_degree, int budget, int batch_div, int nthreads,
                     uint64_t *graph_out);

/* The same construction with each batch's searches (graph.h:169-216) on GPU
 * `device`, one warp per new vertex, and the edge updates on nthreads host
 * threads: graph_out equals song_graph_build's for the same arguments, bit
 * for bit.  budget <= 1024, n < 2^32 - 1. */
int song_graph_build_gpu(const float *data, uint64_t n, int dim, int metric, int shift,
                         int search_degree, int fixed_degree, int budget, int batch_div, int device,
                         int nthreads, uint64_t *graph_out);

/* Low-precision storage (BF16 / FP8): number of the best final candidates
 * re-ranked with exact FP32 distances before the first k are returned.
 * -1 (default) = all pq, 0 = none (results in the storage's precision).
 * No counterpart in the reference. */
int song_index_set_rerank(song_index *index, int rerank);

/* Stored rows (bytes as searched: F32, BF16, or FP8 bytes followed by the
 * row's float scale), rows first .. first+count-1; *row_bytes gets the row
 * size (out may be NULL to query it).  No counterpart in the reference. */
int song_index_rows(const song_index *index, uint64_t first, uint64_t count, void *out,
                    size_t out_bytes, int *row_bytes);

/* Learned early exit (no counterpart in the reference).  A network
 * 5 -> 32 -> 32 -> 1 (ReLU) reads, after every `every`-th hop from hop
 * `min_hops` on, the query's state (log hop count; the top-k spread and the
 * queue-head gap relative to the progress span d0 - best, as signed logs;
 * log of the hops since the top-k set last changed; log distance
 * evaluations) and
 * stops the search when its logit >= threshold; queries it
 * never trusts run the plain search to its finish rule.  weights: the
 * SONG_MLP_PARAMS FP32 parameters (W1[32][5], b1[32], W2[32][32], b2[32],
 * w3[32], b3), stored on the device in BF16; NULL switches the exit off.
 * F32 and BF16 storage. */
#define SONG_MLP_PARAMS 1281
int song_index_set_early_exit(song_index *index, const float *weights, float threshold,
                              int min_hops, int every);

/* Hyperplanes of a SONG_STORAGE_BITS index (hash_warp_no_heap_astar_accelerator.h:
 * 22-41; bithash.h:8-65): planes holds SONG_HASH_BITS rows of dim floats.
 * Bit i of a vector's code is set when its dot product with plane i is >= 0,
 * the dot product summed as the search sums distances (lane l of a warp takes
 * dimensions l, l+32, ... with fused multiply-adds; the 32 partial sums meet
 * in the xor butterfly).  Computes the codes of all base vectors; queries are
 * coded the same way on every search. */
int song_index_set_hash_planes(song_index *index, const float *planes);

/* The reference kernel's multi-probe knobs as run-time values (compile-time
 * macros there; generate_template.sh:17-18 and fill_parameters.sh:36-37 set
 * the first two).  All at their defaults -- (1, 1, 0), as in the reference --
 * select the plain search.
 *   probes (N_MULTIPROBE, warp_astar_accelerator.h:29; 1..SONG_MAX_PROBES):
 *     vertices popped per iteration; only an iteration's first pop takes the
 *     finish test, and the unvisited neighbours of all its pops are listed
 *     before their distances are computed and select-inserted in order
 *     (:182-322).  A vertex adjacent to two pops is listed twice and, without
 *     double_check, can enter the queue and the result twice, as in the
 *     reference.
 *   finish_cnt (FINISH_CNT, :30; >= 1): the search ends when the finish test
 *     has held that many times; a pop that passes it before then is expanded
 *     like any other (:190-197,227).
 *   double_check (__ENABLE_MULTIPROBE_DOUBLE_CHECK, :307-310; 0 or 1): the
 *     select-insert skips a candidate already in the visited hash.
 * F32 storage.  Does not combine with early exit, a hop limit, tracing or a
 * server: those reject an index with any knob away from its default. */
#define SONG_MAX_PROBES 4
int song_index_set_multiprobe(song_index *index, int probes, int finish_cnt, int double_check);

/* Fixed hop budget (0 = off): stop every query after max_hops expansions.
 * A baseline heuristic to compare the learned exit against; no counterpart
 * in the reference.  F32 and BF16 storage. */
int song_index_set_hop_limit(song_index *index, int max_hops);

/* Stage timing, the counterpart of the reference's __ENABLE_MEASURE stage
 * timers (warp_astar_accelerator.h:32-38,358-408).  With enable != 0 every
 * later search on the index records CUDA events on its launch stream around
 * the entry-point choice and around the search kernel; song_index_timing
 * waits for the last search's events and returns both stages in
 * milliseconds (entry_ms 0 without entry points).  enable = 0 stops the
 * recording; the events are released with the index. */
int song_index_set_timing(song_index *index, int enable);
int song_index_timing(song_index *index, float *entry_ms, float *search_ms);

/* Entry points (warp_astar_accelerator.h:173 always starts at vertex 0, which
 * stays the default).  With count > 0 entry vertex ids, every query of
 * song_search, song_search_device and song_search_trace_device starts from
 * the `starts` entries nearest to it (the search's own distance on the FP32
 * rows, ties to the smaller id), chosen on the GPU before the search: they
 * enter the candidate queue and the visited set nearest first, and the search
 * itself is unchanged.  1 <= starts <= min(SONG_MAX_STARTS, count) and
 * starts <= pq.  count = 0 restores vertex 0.  A server created on the
 * index afterwards makes the same choice inside its persistent warps (its
 * requests then need pq >= starts), and the entries cannot change while it
 * exists.  song_search_noalloc always starts at vertex 0.  No counterpart in
 * the reference. */
#define SONG_MAX_ENTRIES 65536
#define SONG_MAX_STARTS 8
int song_index_set_entries(song_index *index, const uint64_t *ids, int count, int starts);

/* Two-level entry points, for large entry sets (no counterpart in the
 * reference).  ids[0..coarse-1] are coarse entries, each its own cluster;
 * every other entry joins the cluster of its nearest coarse entry (its FP32
 * row as the query, ties to the smaller id), computed here on the GPU.  Each
 * query then probes its `probes` nearest coarse entries and starts from the
 * `starts` nearest entries of those clusters (starts <= probes <= min(
 * SONG_MAX_STARTS, coarse)): one pass over the coarse rows and the probed
 * clusters instead of all entries.  Distinct ids; rows of up to 4840 floats.
 * Replaces any entries set before; song_index_set_entries(ix, NULL, 0, 1)
 * clears them. */
#define SONG_MAX_ENTRIES_2LEVEL (1 << 20)
#define SONG_MAX_COARSE 16384
int song_index_set_entries_2level(song_index *index, const uint64_t *ids, int count, int coarse, int probes,
                                  int starts);

/* Training of the early-exit network (no counterpart in the reference), all
 * buffers on the device, ordered on `stream`: x n x 5 features, y n labels
 * (0/1), w n sample weights or NULL, perm epochs x n sample indices or NULL
 * (in order), Adam with learning rate lr on minibatches of `batch`, loss
 * weighted binary cross-entropy on the logit.  params (SONG_MLP_PARAMS FP32)
 * are read as the start point and overwritten; loss (epochs floats, may be
 * NULL) receives the mean minibatch loss of each epoch. */
int song_mlp_train_device(const float *d_x, const float *d_y, const float *d_w, int64_t n,
                          const int32_t *d_perm, int epochs, int batch, float lr, float *d_params,
                          float *d_loss, void *stream);

/* Mean gradient and loss of the training objective over n samples (host
 * buffers; w may be NULL), computed by the training kernels.  For checks. */
int song_mlp_grad(const float *x, const float *y, const float *w, int n, const float *params,
                  float *grad_out, float *loss_out);

/* Logits of n samples (host buffers), FP32 weights, by the training kernels. */
int song_mlp_forward(const float *x, int n, const float *params, float *logits_out);

/* The plain search with per-hop tracing, DEVICE buffers on `stream`: for
 * query q and hop h < trace_hops, trace[(q*trace_hops + h)*6 + 0..4] are the
 * early-exit features after hop h+1 and [.. + 5] the number of changes of the
 * top-k set so far; final[2q] = that count at the end, final[2q+1] = hops
 * traced.  A hop's label "top-k already final" is trace[..5] == final[2q]. */
int song_search_trace_device(song_index *index, const float *d_queries, int nq, int pq, int k,
                             int trace_hops, float *d_trace, int32_t *d_final, uint64_t *d_out,
                             int32_t *d_hops, int32_t *d_evals, void *stream);

/* Continuous-batching server over one resident index (no counterpart in the
 * reference).  A persistent kernel on `sm_fraction` of the GPU's warp slots
 * searches queries as soon as they are published; requests of 1..slot_queries
 * queries with their own pq (<= max_pq) and k (<= max_k) are admitted while
 * one of `slots` query/result slots is free and otherwise wait, in order, for
 * one (admission by memory).  Queries and ids stay in mapped pinned host
 * memory.  A request's ids are exactly what song_search returns for it alone.
 * F32 storage.  One host thread at a time per server. */
typedef struct song_server song_server;
int song_server_create(song_index *index, int max_pq, int max_k, int slots, int slot_queries,
                       float sm_fraction, song_server **out);
/* Copies the queries and queues the request; *ticket identifies it. */
int song_server_submit(song_server *server, const float *queries, int nq, int pq, int k,
                       uint64_t *ticket);
/* Up to `max` tickets of requests completed since the last poll. */
int song_server_poll(song_server *server, uint64_t *tickets, int max, int *n_done);
/* The nq x k ids of a completed request; frees its slot for waiting requests. */
int song_server_result(song_server *server, uint64_t ticket, uint64_t *out, int *nq, int *k);
/* Drains published work, stops the kernel and frees the server. */
int song_server_destroy(song_server *server);
/* Warps that find no work for `polls` polls (~0.5 us apart; default 2^21,
 * about a second) leave; the next submission relaunches the kernel.  Taken
 * by the next launch. */
int song_server_set_idle_polls(song_server *server, uint32_t polls);
/* *running = 1 while the server's kernel has warps on the GPU. */
int song_server_running(song_server *server, int *running);
/* Waits up to timeout_ms for a request to complete: SONG_OK, or
 * SONG_ERR_TIMEOUT if it has not completed by then (it stays queued). */
int song_server_wait(song_server *server, uint64_t ticket, int timeout_ms);

/* Size of the fixed device scratch array used by song_search_noalloc. */
#define SONG_NOALLOC_SCRATCH_BYTES (16u << 20)

/* song_search without any device allocation.  No counterpart in the
 * reference: for callers that cannot let a library call cudaMalloc (a service
 * whose GPU memory is already owned by its own pool or budget, or a request
 * path that must not pay for an allocation that may synchronise the device).
 * Host buffers as in song_search; the device copies of queries and ids and
 * the kernel's work counter and error flag live in one file-scope device
 * array of SONG_NOALLOC_SCRATCH_BYTES per GPU, held until process exit.  A
 * batch may use 256 + round_up(nq*dim*4, 256) + nq*k*8 bytes of it; larger
 * batches return SONG_ERR_ARG.  The array's device address is looked up on
 * the first call on each device (make that call before any stream capture).
 * Calls overlapping on one GPU share the array and race: serialise them. */
int song_search_noalloc(song_index *index, const float *queries, int nq, int pq, int k,
                        uint64_t *out);

/* Test hooks for the failure paths (no counterpart in the reference).
 * song_debug_fail_alloc(n): the n-th next device allocation of the library
 * fails as out of memory (0: none).  song_debug_set_wait: the search kernel's
 * bounded waits give up after wait_limit polls (default 2^24), and every
 * batch of row copies expects extra_tx bytes (a multiple of 16) that no copy
 * delivers -- a wait that cannot complete; the call then returns
 * SONG_ERR_TIMEOUT and the index stays usable.  song_debug_server_hold(1):
 * admitted requests are kept from the kernel until song_debug_server_hold(0). */
int song_debug_fail_alloc(int n);
int song_debug_set_wait(song_index *index, uint32_t wait_limit, uint32_t extra_tx);
int song_debug_server_hold(song_server *server, int hold);

/* Head phase of the two-level entry choice (song_index_set_entries_2level).
 * By default it scores queries against the coarse entries with a TF32
 * tensor-core product and re-scores, with the search's exact arithmetic, the
 * shortlist whose error intervals reach the probes-th best -- the same
 * clusters as an exact scan.  song_debug_head_path(index, 0) switches to the
 * exact CUDA-core scan of every coarse entry (1: back); *prepared (may be
 * NULL) tells whether the tensor path exists for the index (it needs
 * dim % 4 == 0).  song_debug_head_stats(index, enable, stats): with enable,
 * later searches count [0] queries, [1] coarse entries re-scored exactly,
 * [2] queries whose shortlist overflowed into a full scan; stats (3 values,
 * may be NULL) receives the counts since the previous call, which restart at
 * zero.  song_debug_head_scores: the tensor-core scores alone, d_scores[q*ld
 * + h] = approximate dot product of query q and coarse entry h (device
 * buffers; ld >= the coarse entries, a multiple of 4). */
int song_debug_head_path(song_index *index, int use_tensor_cores, int *prepared);
int song_debug_head_stats(song_index *index, int enable, unsigned long long *stats);
int song_debug_head_scores(song_index *index, const float *d_queries, int nq, float *d_scores, int ld);

/* The visited-hash slot function of the reference's default build
 * (fixhash.h:20-24) evaluated on the device for `count` ids, for tests. */
int song_debug_fixhash(const uint32_t *ids, int count, int pq, int32_t *slots_out);

#ifdef __cplusplus
}
#endif
#endif /* SONG_GB300_H */
