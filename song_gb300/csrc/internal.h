// internal.h -- declarations shared by the C-ABI layer and the kernels.
#pragma once

#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace song {

// Device layout of one resident index.
struct DeviceIndex {
  uint64_t n = 0;
  int dim = 0;
  int shift = 0;
  int metric = 0;
  int storage = 0;
  int dpad = 0;             // elements per stored row (row_bytes / element size)
  uint32_t row_bytes = 0;   // bytes per stored row, a multiple of 16
  const void *rows = nullptr;        // n rows of row_bytes
  uint32_t scale_off = 0;            // FP8: byte offset of the per-row float scale
  const float *rows_f32 = nullptr;   // FP32 rows (rerank; == rows for F32 storage)
  uint32_t f32_row_bytes = 0;
  const uint32_t *adj = nullptr;     // n << shift uint32: slot 0 = degree
};

struct SearchCall {
  const float *queries = nullptr;  // nq x dim, device
  int nq = 0;
  int pq = 0;
  int k = 0;
  uint64_t *out = nullptr;         // nq x k, device
  int32_t *hops = nullptr;         // nq or null
  int32_t *evals = nullptr;        // nq or null
  uint32_t *counter = nullptr;     // one uint32 of device scratch (work counter)
  int32_t *error = nullptr;        // one int32 device error flag
  int rerank = 0;                  // low-precision storage: FP32 re-rank of the best `rerank`
  const __nv_bfloat16 *mlp = nullptr;  // early-exit network (device, BF16) or null
  float exit_threshold = 0.0f;     // stop when the network's logit >= this
  int exit_min_hops = 0;
  int exit_every = 1;
  int exit_max_hops = 0;           // > 0: fixed hop budget (comparison heuristic)
  float *trace = nullptr;          // per-hop features, nq x trace_hops x 6, or null
  int trace_hops = 0;
  int32_t *trace_final = nullptr;  // nq x 2: final top-k version, hops traced
  const uint32_t *starts = nullptr;  // nq x n_starts start vertices (entry points), null = vertex 0
  int n_starts = 1;
  const uint32_t *qcodes = nullptr;  // BITS storage: nq x 8 query code words
  uint32_t wait_limit = 1u << 24;  // polls of a bounded mbarrier wait
  uint32_t extra_tx = 0;           // test hook (song_debug_set_wait)
  int probes = 1;                  // N_MULTIPROBE (song_index_set_multiprobe)
  int finish_cnt = 1;              // FINISH_CNT
  int double_check = 0;            // __ENABLE_MULTIPROBE_DOUBLE_CHECK
};

// Launch the plain search.  Returns a cudaError_t-compatible code (0 ok) or
// -1 when the shape is unsupported; sets *smem_per_warp if non-null.
int launch_search(const DeviceIndex &ix, const SearchCall &c, cudaStream_t stream);

// Shared-memory bytes one warp needs for (ix, pq).
uint32_t search_warp_bytes(const DeviceIndex &ix, int pq, bool multi = false);
// Whether an index's knobs select the multi-probe kernel.
inline bool multi_knobs(int probes, int finish_cnt, int double_check) {
  return probes > 1 || finish_cnt > 1 || double_check != 0;
}

int launch_debug_fixhash(const uint32_t *ids, int count, int pq, int32_t *out, cudaStream_t s);

// BITS storage: the 256-bit codes of n vectors (search_bits.cu).
int launch_hash_codes(const float *rows, uint64_t n, int stride, int dim, const float *planes, int pstride,
                      uint32_t *codes, cudaStream_t s);

}  // namespace song

struct song_index;

namespace song {
// Head phase of the two-level entry choice on the tensor cores (head_mma.cu).
bool heads_mma_prepare(song_index *ix, int coarse);
bool heads_mma_usable(const song_index *ix, const float *queries, int np);
cudaError_t launch_heads_mma(song_index *ix, const float *queries, int nq, int np, uint32_t *probe_out,
                             cudaStream_t s);
cudaError_t launch_head_scores_only(song_index *ix, const float *queries, int nq, float *scores, int ld,
                                    cudaStream_t s);

}  // namespace song

namespace song {
// Makes `dev` current for the scope and restores the caller's device.
struct DeviceGuard {
  int prev = -1;
  bool ok = true;
  explicit DeviceGuard(int dev) {
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    if (prev != dev) ok = cudaSetDevice(dev) == cudaSuccess;
  }
  ~DeviceGuard() {
    int cur = -1;
    if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
  }
};

// Device allocations of the library go through here, so that a test can make
// one fail (song_debug_fail_alloc).
cudaError_t dev_malloc(void **p, size_t bytes);
template <class T>
cudaError_t dev_malloc(T **p, size_t bytes) {
  return dev_malloc(reinterpret_cast<void **>(p), bytes);
}

// Error reporting of the C ABI (capi.cu): records the message for
// song_last_error() on the calling thread and returns `code`.
int fail(int code, const char *fmt, ...);
void clear_error();
int check_search_args(const song_index *ix, int nq, int pq, int k);
// Copies the index's search settings (re-rank count, early-exit network) into c.
void apply_index_settings(const song_index *ix, SearchCall &c);
}  // namespace song

// The opaque handle of include/song_gb300.h.
struct song_index {
  int device = 0;
  song::DeviceIndex dx;
  void *d_rows = nullptr;
  uint32_t *d_adj = nullptr;
  float *d_rows_f32 = nullptr;
  int rerank = -1;                  // -1: all pq candidates (default), 0: none
  __nv_bfloat16 *d_mlp = nullptr;   // early-exit network, null = off
  float exit_threshold = 0.0f;
  int exit_min_hops = 0;
  int exit_every = 1;
  int max_hops = 0;                 // fixed hop budget, 0 = off
  uint32_t wait_limit = 1u << 24;   // polls of the kernel's bounded waits (song_debug_set_wait)
  uint32_t extra_tx = 0;            // test hook: bytes no copy delivers (song_debug_set_wait)
  int probes = 1;                   // song_index_set_multiprobe
  int finish_cnt = 1;
  int double_check = 0;
  uint32_t *d_counter = nullptr;
  int32_t *d_error = nullptr;
  cudaStream_t stream = nullptr;
  // device staging for the host-buffer entry point song_search
  float *d_q = nullptr;
  size_t cap_q = 0;
  uint64_t *d_out = nullptr;
  size_t cap_out = 0;
  int32_t *d_stats = nullptr;
  size_t cap_stats = 0;
  // entry points (song_index_set_entries): ids, their FP32 rows, per-call starts
  uint32_t *d_entry_ids = nullptr;
  float *d_entry_rows = nullptr;
  int n_entries = 0;
  int n_starts = 1;  // start vertices per query (nearest entries)
  // two-level choice (n_coarse > 0): d_entry_rows / d_entry_ids hold all
  // entries in cluster order, d_offsets the clusters, d_coarse_rows the
  // coarse entries sorted by id
  int n_coarse = 0;
  int n_probes = 0;
  float *d_coarse_rows = nullptr;
  uint32_t *d_offsets = nullptr;
  uint32_t *d_cl_count = nullptr;      // probes per cluster (per call)
  uint32_t *d_cl_order = nullptr;      // clusters by descending size (the cluster phase's task order)
  // head phase on the tensor cores (head_mma.cu): tensor map of the coarse
  // rows (a CUtensorMap), their squared norms, the per-chunk score buffer
  unsigned char head_map[128] = {};
  bool heads_mma = false;              // prepared for this index
  bool heads_mma_enabled = true;       // song_debug_head_path
  float *d_head_n2 = nullptr;
  float *d_head_scores = nullptr;
  size_t cap_head_scores = 0;
  bool head_stats_on = false;          // song_debug_head_stats
  unsigned long long *d_head_stats = nullptr;
  uint32_t *d_entry_work = nullptr;    // per-call lists of the two-level choice
  size_t cap_entry_work = 0;
  int servers = 0;  // servers using the entries (song_server_create); they stay fixed meanwhile
  // stage timing (song_index_set_timing): events before the entry choice,
  // before the search kernel, after it
  bool timing = false;
  cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
  bool timed_entries = false;
  // BITS storage: hyperplanes (SONG_HASH_BITS x f32 row width) and per-call query codes
  float *d_planes = nullptr;
  bool has_planes = false;
  uint32_t *d_qcodes = nullptr;
  size_t cap_qcodes = 0;
  uint32_t *d_starts = nullptr;
  size_t cap_starts = 0;
  uint64_t device_bytes = 0;
};

namespace song {
// Entry points: with entries set on the index, picks every query's start
// vertex (entries.cu) on stream s and points c.starts at them; otherwise
// leaves c.starts null.  Returns a SONG_* status.
int prepare_starts(song_index *ix, SearchCall &c, cudaStream_t s);
}  // namespace song
