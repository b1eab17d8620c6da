// capi.cu -- the extern "C" boundary (include/song_gb300.h): resident index,
// search entry points with host or device buffers, and the one-shot form with
// the reference's argument list.
#include <cuda_bf16.h>
#include <cuda_fp8.h>
#include <cuda_runtime.h>

#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "internal.h"
#include "song_gb300.h"

namespace {
thread_local std::string g_last_error;
}  // namespace

namespace song {

int fail(int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

void clear_error() { g_last_error.clear(); }

namespace {
std::atomic<long long> g_fail_alloc{0};  // song_debug_fail_alloc: allocations left until one fails
}  // namespace

cudaError_t dev_malloc(void **p, size_t bytes) {
  if (g_fail_alloc.load() > 0 && g_fail_alloc.fetch_sub(1) == 1) {
    *p = nullptr;
    return cudaErrorMemoryAllocation;
  }
  return cudaMalloc(p, bytes);
}

int check_search_args(const song_index *ix, int nq, int pq, int k) {
  if (!ix) return fail(SONG_ERR_ARG, "null index");
  if (nq < 0) return fail(SONG_ERR_ARG, "nq must be >= 0");
  if (pq < 2 || pq > SONG_MAX_PQ) return fail(SONG_ERR_ARG, "pq must be in [2, %d]", SONG_MAX_PQ);
  if (k < 1 || k > pq) return fail(SONG_ERR_ARG, "k must be in [1, pq]");
  uint32_t wb = search_warp_bytes(ix->dx, pq, multi_knobs(ix->probes, ix->finish_cnt, ix->double_check));
  if (wb > 227u * 1024u)
    return fail(SONG_ERR_ARG, "pq %d with dim %d needs %u B of shared memory per warp", pq,
                ix->dx.dim, wb);
  return SONG_OK;
}

}  // namespace song

namespace {
using song::DeviceGuard;
using song::fail;
using song::check_search_args;

#define SONG_CUDA(call)                                                                   \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess)                                                                \
      return fail(e_ == cudaErrorMemoryAllocation ? SONG_ERR_OOM : SONG_ERR_CUDA, "%s: %s", \
                  #call, cudaGetErrorString(e_));                                         \
  } while (0)

template <class T>
int grow(T **p, size_t *cap, size_t need, uint64_t *acct) {
  if (need <= *cap) return SONG_OK;
  if (*p) {
    cudaFree(*p);
    *acct -= *cap * sizeof(T);
  }
  *p = nullptr;
  *cap = 0;
  size_t n = need < 1024 ? 1024 : need;
  SONG_CUDA(song::dev_malloc(reinterpret_cast<void **>(p), n * sizeof(T)));
  *cap = n;
  *acct += n * sizeof(T);
  return SONG_OK;
}

void release(song_index *ix) {
  if (!ix) return;
  if (ix->d_rows_f32 && static_cast<void *>(ix->d_rows_f32) != ix->d_rows) cudaFree(ix->d_rows_f32);
  cudaFree(ix->d_rows);
  cudaFree(ix->d_adj);
  cudaFree(ix->d_mlp);
  cudaFree(ix->d_counter);
  cudaFree(ix->d_error);
  cudaFree(ix->d_q);
  cudaFree(ix->d_out);
  cudaFree(ix->d_stats);
  cudaFree(ix->d_entry_ids);
  cudaFree(ix->d_entry_rows);
  cudaFree(ix->d_coarse_rows);
  cudaFree(ix->d_offsets);
  cudaFree(ix->d_cl_count);
  cudaFree(ix->d_cl_order);
  cudaFree(ix->d_entry_work);
  cudaFree(ix->d_starts);
  cudaFree(ix->d_planes);
  cudaFree(ix->d_qcodes);
  cudaFree(ix->d_head_n2);
  cudaFree(ix->d_head_scores);
  cudaFree(ix->d_head_stats);
  for (cudaEvent_t &e : ix->ev)
    if (e) cudaEventDestroy(e);
  if (ix->stream) cudaStreamDestroy(ix->stream);
  delete ix;
}

int launch(song_index *ix, const float *d_q, int nq, int pq, int k, uint64_t *d_out,
           int32_t *d_hops, int32_t *d_evals, cudaStream_t s) {
  song::SearchCall c;
  c.queries = d_q;
  c.nq = nq;
  c.pq = pq;
  c.k = k;
  c.out = d_out;
  c.hops = d_hops;
  c.evals = d_evals;
  c.counter = ix->d_counter;
  c.error = ix->d_error;
  song::apply_index_settings(ix, c);
  if (ix->dx.storage == SONG_STORAGE_BITS) {
    // the queries' 256-bit codes, on the search's stream
    if (!ix->has_planes) return fail(SONG_ERR_ARG, "SONG_STORAGE_BITS index without hash planes");
    int rc = grow(&ix->d_qcodes, &ix->cap_qcodes, static_cast<size_t>(nq) * 8, &ix->device_bytes);
    if (rc) return rc;
    const int e = song::launch_hash_codes(d_q, static_cast<uint64_t>(nq), ix->dx.dim, ix->dx.dim, ix->d_planes,
                                          static_cast<int>(ix->dx.f32_row_bytes / 4), ix->d_qcodes, s);
    if (e != 0) return fail(SONG_ERR_CUDA, "query codes: %s", cudaGetErrorString((cudaError_t)e));
    c.qcodes = ix->d_qcodes;
  }
  // the error flag collects the bounded waits of the entry choice and of the search
  SONG_CUDA(cudaMemsetAsync(ix->d_error, 0, sizeof(int32_t), s));
  if (ix->timing) SONG_CUDA(cudaEventRecord(ix->ev[0], s));
  int rc = song::prepare_starts(ix, c, s);
  if (rc != SONG_OK) return rc;
  if (ix->timing) {
    SONG_CUDA(cudaEventRecord(ix->ev[1], s));
    ix->timed_entries = c.starts != nullptr;
  }
  int e = song::launch_search(ix->dx, c, s);
  if (e == -1) return fail(SONG_ERR_ARG, "unsupported search shape");
  if (e != 0) return fail(SONG_ERR_CUDA, "search launch: %s", cudaGetErrorString((cudaError_t)e));
  if (ix->timing) SONG_CUDA(cudaEventRecord(ix->ev[2], s));
  return SONG_OK;
}


// BF16 rows: round-to-nearest-even conversion of every element, zero padding.
__global__ void to_bf16_kernel(const float *in, uint32_t in_row_floats, uint64_t n, int dim, int dpad,
                               __nv_bfloat16 *out) {
  const uint64_t total = n * static_cast<uint64_t>(dpad);
  for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < total;
       i += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
    const uint64_t r = i / dpad;
    const int j = static_cast<int>(i - r * dpad);
    out[i] = __float2bfloat16_rn(j < dim ? in[r * in_row_floats + j] : 0.0f);
  }
}

// FP8 rows, one warp per row: scale = max|x| / 448 (the largest finite E4M3
// value; 1 for a zero row), elements x / scale converted with saturation to
// E4M3, the scale stored as a float at scale_off.
__global__ void to_fp8_kernel(const float *in, uint32_t in_row_floats, uint64_t n, int dim,
                              uint8_t *out, uint32_t out_row_bytes, uint32_t scale_off) {
  const int lane = threadIdx.x & 31;
  const uint64_t warp = (blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x) >> 5;
  const uint64_t nwarps = (static_cast<uint64_t>(gridDim.x) * blockDim.x) >> 5;
  for (uint64_t r = warp; r < n; r += nwarps) {
    const float *x = in + r * in_row_floats;
    float amax = 0.0f;
    for (int j = lane; j < dim; j += 32) amax = fmaxf(amax, fabsf(x[j]));
    for (int o = 16; o > 0; o >>= 1) amax = fmaxf(amax, __shfl_xor_sync(0xffffffffu, amax, o));
    const float scale = amax > 0.0f ? amax / 448.0f : 1.0f;
    uint8_t *y = out + r * out_row_bytes;
    for (int j = lane; j < static_cast<int>(scale_off); j += 32)
      y[j] = j < dim ? static_cast<uint8_t>(__nv_cvt_float_to_fp8(x[j] / scale, __NV_SATFINITE, __NV_E4M3)) : 0;
    for (int j = static_cast<int>(scale_off) + lane; j < static_cast<int>(out_row_bytes); j += 32) y[j] = 0;
    __syncwarp();
    if (lane == 0) *reinterpret_cast<float *>(y + scale_off) = scale;
  }
}

}  // namespace

namespace song {
void apply_index_settings(const song_index *ix, SearchCall &c) {
  c.rerank = ix->dx.storage == SONG_STORAGE_F32 ? 0 : (ix->rerank < 0 ? c.pq : ix->rerank);
  c.mlp = ix->d_mlp;
  c.exit_threshold = ix->exit_threshold;
  c.exit_min_hops = ix->exit_min_hops;
  c.exit_every = ix->exit_every;
  c.exit_max_hops = ix->max_hops;
  c.wait_limit = ix->wait_limit;
  c.extra_tx = ix->extra_tx;
  c.probes = ix->probes;
  c.finish_cnt = ix->finish_cnt;
  c.double_check = ix->double_check;
}
}  // namespace song

namespace {
}  // namespace

extern "C" {

const char *song_status_string(int status) {
  switch (status) {
    case SONG_OK: return "ok";
    case SONG_ERR_ARG: return "invalid argument";
    case SONG_ERR_OOM: return "out of memory";
    case SONG_ERR_TIMEOUT: return "device wait timed out";
    case SONG_ERR_CUDA: return "CUDA error";
    case SONG_ERR_IO: return "I/O error";
    default: return "unknown status";
  }
}

const char *song_last_error(void) { return g_last_error.c_str(); }

int song_index_create(const uint64_t *graph, const float *data, uint64_t n, int dim, int shift,
                      int metric, int storage, int device, song_index **out) {
  g_last_error.clear();
  if (!out) return fail(SONG_ERR_ARG, "null output pointer");
  *out = nullptr;
  if (!graph || !data) return fail(SONG_ERR_ARG, "null graph or data");
  if (n < 1 || n > 0x7fffffffull) return fail(SONG_ERR_ARG, "n must be in [1, 2^31)");
  if (dim < 1 || dim > 65536) return fail(SONG_ERR_ARG, "dim must be in [1, 65536]");
  if (shift < 1 || shift > SONG_MAX_SHIFT)
    return fail(SONG_ERR_ARG, "shift must be in [1, %d]", SONG_MAX_SHIFT);
  if (metric < SONG_METRIC_L2 || metric > SONG_METRIC_COS) return fail(SONG_ERR_ARG, "bad metric");
  if (storage < SONG_STORAGE_F32 || storage > SONG_STORAGE_BITS) return fail(SONG_ERR_ARG, "bad storage %d", storage);

  // The reference reads degree and ids unchecked (warp_astar_accelerator.h:212-214);
  // a malformed row would make it read out of bounds, so reject it here.
  const uint64_t slots = n << shift;
  const uint64_t maxdeg = (1ull << shift) - 1;
  std::vector<uint32_t> adj(slots, 0u);
  for (uint64_t v = 0; v < n; ++v) {
    const uint64_t *row = graph + (v << shift);
    const uint64_t deg = row[0];
    if (deg > maxdeg)
      return fail(SONG_ERR_ARG, "vertex %llu has degree %llu > %llu", (unsigned long long)v,
                  (unsigned long long)deg, (unsigned long long)maxdeg);
    uint32_t *arow = adj.data() + (v << shift);
    arow[0] = static_cast<uint32_t>(deg);
    for (uint64_t i = 1; i <= deg; ++i) {
      if (row[i] >= n)
        return fail(SONG_ERR_ARG, "vertex %llu has neighbour %llu >= n", (unsigned long long)v,
                    (unsigned long long)row[i]);
      arow[i] = static_cast<uint32_t>(row[i]);
    }
  }

  DeviceGuard g(device);
  if (!g.ok) return fail(SONG_ERR_CUDA, "cannot select device %d", device);
  song_index *ix = new song_index();
  ix->device = device;
  song::DeviceIndex &dx = ix->dx;
  dx.n = n;
  dx.dim = dim;
  dx.shift = shift;
  dx.metric = metric;
  dx.storage = storage;
  const int dpad4 = (dim + 3) / 4 * 4;
  dx.f32_row_bytes = static_cast<uint32_t>(dpad4) * 4u;
  if (storage == SONG_STORAGE_F32) {
    dx.dpad = dpad4;
    dx.row_bytes = dx.f32_row_bytes;
  } else if (storage == SONG_STORAGE_BF16) {
    dx.dpad = (dim + 7) / 8 * 8;
    dx.row_bytes = static_cast<uint32_t>(dx.dpad) * 2u;
  } else if (storage == SONG_STORAGE_BITS) {
    dx.dpad = SONG_HASH_BITS / 32;  // code words
    dx.row_bytes = SONG_HASH_BITS / 8;
  } else {
    dx.dpad = (dim + 15) / 16 * 16;
    dx.scale_off = static_cast<uint32_t>(dx.dpad);
    dx.row_bytes = dx.scale_off + 16u;
  }
  auto bail = [&](int code) {
    release(ix);
    return code;
  };
  cudaError_t e;
#define SONG_CUDA_IX(call)                                                                  \
  do {                                                                                      \
    e = (call);                                                                             \
    if (e != cudaSuccess)                                                                   \
      return bail(fail(e == cudaErrorMemoryAllocation ? SONG_ERR_OOM : SONG_ERR_CUDA, "%s: %s", \
                       #call, cudaGetErrorString(e)));                                      \
  } while (0)
  SONG_CUDA_IX(cudaStreamCreateWithFlags(&ix->stream, cudaStreamNonBlocking));
  const size_t f32_bytes = static_cast<size_t>(n) * dx.f32_row_bytes;
  SONG_CUDA_IX(song::dev_malloc(reinterpret_cast<void **>(&ix->d_rows_f32), f32_bytes));
  ix->device_bytes += f32_bytes;
  SONG_CUDA_IX(cudaMemsetAsync(ix->d_rows_f32, 0, f32_bytes, ix->stream));
  SONG_CUDA_IX(cudaMemcpy2DAsync(ix->d_rows_f32, dx.f32_row_bytes, data, sizeof(float) * dim,
                                 sizeof(float) * dim, n, cudaMemcpyHostToDevice, ix->stream));
  if (storage == SONG_STORAGE_F32) {
    ix->d_rows = ix->d_rows_f32;
  } else {
    // Low-precision rows for the search; the FP32 rows stay for the re-rank.
    const size_t rows_bytes = static_cast<size_t>(n) * dx.row_bytes;
    SONG_CUDA_IX(song::dev_malloc(&ix->d_rows, rows_bytes));
    ix->device_bytes += rows_bytes;
    const uint32_t in_floats = dx.f32_row_bytes / 4u;
    if (storage == SONG_STORAGE_BITS)  // codes follow from the planes (song_index_set_hash_planes)
      SONG_CUDA_IX(cudaMemsetAsync(ix->d_rows, 0, rows_bytes, ix->stream));
    else if (storage == SONG_STORAGE_BF16)
      to_bf16_kernel<<<4 * 152, 256, 0, ix->stream>>>(ix->d_rows_f32, in_floats, n, dim, dx.dpad,
                                                      static_cast<__nv_bfloat16 *>(ix->d_rows));
    else
      to_fp8_kernel<<<4 * 152, 256, 0, ix->stream>>>(ix->d_rows_f32, in_floats, n, dim,
                                                     static_cast<uint8_t *>(ix->d_rows), dx.row_bytes,
                                                     dx.scale_off);
    SONG_CUDA_IX(cudaGetLastError());
  }
  SONG_CUDA_IX(song::dev_malloc(&ix->d_adj, slots * sizeof(uint32_t)));
  ix->device_bytes += slots * sizeof(uint32_t);
  SONG_CUDA_IX(cudaMemcpyAsync(ix->d_adj, adj.data(), slots * sizeof(uint32_t),
                               cudaMemcpyHostToDevice, ix->stream));
  SONG_CUDA_IX(song::dev_malloc(&ix->d_counter, 256));
  SONG_CUDA_IX(song::dev_malloc(&ix->d_error, 256));
  ix->device_bytes += 512;
  SONG_CUDA_IX(cudaMemsetAsync(ix->d_error, 0, 256, ix->stream));
  SONG_CUDA_IX(cudaStreamSynchronize(ix->stream));
#undef SONG_CUDA_IX
  dx.rows = ix->d_rows;
  dx.rows_f32 = ix->d_rows_f32;
  dx.adj = ix->d_adj;
  *out = ix;
  return SONG_OK;
}

int song_index_load(const char *graph_path, const char *data_path, uint64_t n, int dim, int shift,
                    int metric, int storage, int device, song_index **out) {
  g_last_error.clear();
  if (!graph_path || !data_path || !out) return fail(SONG_ERR_ARG, "null argument");
  if (n < 1 || dim < 1 || shift < 1 || shift > SONG_MAX_SHIFT)
    return fail(SONG_ERR_ARG, "bad n, dim or shift");
  std::vector<uint64_t> graph(static_cast<size_t>(n) << shift);
  std::vector<float> data(static_cast<size_t>(n) * dim);
  FILE *fg = fopen(graph_path, "rb");
  if (!fg) return fail(SONG_ERR_IO, "cannot open %s", graph_path);
  size_t got = fread(graph.data(), sizeof(uint64_t), graph.size(), fg);
  fclose(fg);
  if (got != graph.size()) return fail(SONG_ERR_IO, "%s: short read", graph_path);
  FILE *fd = fopen(data_path, "rb");
  if (!fd) return fail(SONG_ERR_IO, "cannot open %s", data_path);
  got = fread(data.data(), sizeof(float), data.size(), fd);
  fclose(fd);
  if (got != data.size()) return fail(SONG_ERR_IO, "%s: short read", data_path);
  return song_index_create(graph.data(), data.data(), n, dim, shift, metric, storage, device, out);
}

int song_index_free(song_index *index) {
  if (!index) return SONG_OK;
  DeviceGuard g(index->device);
  release(index);
  return SONG_OK;
}

int song_index_info(const song_index *ix, uint64_t *n, int *dim, int *shift, int *metric,
                    int *storage, uint64_t *device_bytes) {
  if (!ix) return fail(SONG_ERR_ARG, "null index");
  if (n) *n = ix->dx.n;
  if (dim) *dim = ix->dx.dim;
  if (shift) *shift = ix->dx.shift;
  if (metric) *metric = ix->dx.metric;
  if (storage) *storage = ix->dx.storage;
  if (device_bytes) *device_bytes = ix->device_bytes;
  return SONG_OK;
}

int song_search(song_index *ix, const float *queries, int nq, int pq, int k, uint64_t *out,
                int32_t *hops, int32_t *evals) {
  g_last_error.clear();
  int rc = check_search_args(ix, nq, pq, k);
  if (rc) return rc;
  if (nq == 0) return SONG_OK;
  if (!queries || !out) return fail(SONG_ERR_ARG, "null queries or out");
  DeviceGuard g(ix->device);
  if (!g.ok) return fail(SONG_ERR_CUDA, "cannot select device %d", ix->device);
  const size_t qn = static_cast<size_t>(nq) * ix->dx.dim;
  const size_t on = static_cast<size_t>(nq) * k;
  if ((rc = grow(&ix->d_q, &ix->cap_q, qn, &ix->device_bytes))) return rc;
  if ((rc = grow(&ix->d_out, &ix->cap_out, on, &ix->device_bytes))) return rc;
  const bool stats = hops || evals;
  if (stats && (rc = grow(&ix->d_stats, &ix->cap_stats, 2 * static_cast<size_t>(nq),
                          &ix->device_bytes)))
    return rc;
  cudaStream_t s = ix->stream;
  SONG_CUDA(cudaMemcpyAsync(ix->d_q, queries, qn * sizeof(float), cudaMemcpyHostToDevice, s));
  rc = launch(ix, ix->d_q, nq, pq, k, ix->d_out, stats ? ix->d_stats : nullptr,
              stats ? ix->d_stats + nq : nullptr, s);
  if (rc) return rc;
  SONG_CUDA(cudaMemcpyAsync(out, ix->d_out, on * sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
  if (hops)
    SONG_CUDA(cudaMemcpyAsync(hops, ix->d_stats, nq * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  if (evals)
    SONG_CUDA(cudaMemcpyAsync(evals, ix->d_stats + nq, nq * sizeof(int32_t),
                              cudaMemcpyDeviceToHost, s));
  int32_t err = 0;
  SONG_CUDA(cudaMemcpyAsync(&err, ix->d_error, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  SONG_CUDA(cudaStreamSynchronize(s));
  if (err) return fail(SONG_ERR_TIMEOUT, "a bulk copy wait timed out in the search kernel");
  return SONG_OK;
}

int song_search_device(song_index *ix, const float *d_queries, int nq, int pq, int k,
                       uint64_t *d_out, int32_t *d_hops, int32_t *d_evals, void *stream) {
  g_last_error.clear();
  int rc = check_search_args(ix, nq, pq, k);
  if (rc) return rc;
  if (nq == 0) return SONG_OK;
  if (!d_queries || !d_out) return fail(SONG_ERR_ARG, "null queries or out");
  DeviceGuard g(ix->device);
  if (!g.ok) return fail(SONG_ERR_CUDA, "cannot select device %d", ix->device);
  return launch(ix, d_queries, nq, pq, k, d_out, d_hops, d_evals,
                static_cast<cudaStream_t>(stream));
}

int song_astar_search_batch(const float *queries, int nq, int pq, uint64_t *results,
                            const float *h_data, const uint64_t *h_graph, int vertex_offset_shift,
                            uint64_t num, int dim, int metric) {
  song_index *ix = nullptr;
  int rc = song_index_create(h_graph, h_data, num, dim, vertex_offset_shift, metric,
                             SONG_STORAGE_F32, 0, &ix);
  if (rc) return rc;
  rc = song_search(ix, queries, nq, pq, pq, results, nullptr, nullptr);
  std::string keep = g_last_error;
  song_index_free(ix);
  g_last_error = keep;
  return rc;
}

int song_debug_fail_alloc(int n) {
  g_last_error.clear();
  if (n < 0) return fail(SONG_ERR_ARG, "n must be >= 0");
  song::g_fail_alloc.store(n);
  return SONG_OK;
}

int song_debug_set_wait(song_index *ix, uint32_t wait_limit, uint32_t extra_tx) {
  g_last_error.clear();
  if (!ix) return fail(SONG_ERR_ARG, "null index");
  if (wait_limit < 1) return fail(SONG_ERR_ARG, "wait_limit must be >= 1");
  if (extra_tx % 16 != 0 || extra_tx > (1u << 16)) return fail(SONG_ERR_ARG, "extra_tx must be a multiple of 16, <= 65536");
  ix->wait_limit = wait_limit;
  ix->extra_tx = extra_tx;
  return SONG_OK;
}

int song_debug_head_path(song_index *ix, int use_tensor_cores, int *prepared) {
  g_last_error.clear();
  if (!ix) return fail(SONG_ERR_ARG, "null index");
  ix->heads_mma_enabled = use_tensor_cores != 0;
  if (prepared) *prepared = ix->heads_mma ? 1 : 0;
  return SONG_OK;
}

int song_debug_head_stats(song_index *ix, int enable, unsigned long long *stats) {
  g_last_error.clear();
  if (!ix) return fail(SONG_ERR_ARG, "null index");
  DeviceGuard g(ix->device);
  if (!g.ok) return fail(SONG_ERR_CUDA, "cannot select device %d", ix->device);
  if (enable && !ix->d_head_stats) {
    SONG_CUDA(song::dev_malloc(reinterpret_cast<void **>(&ix->d_head_stats), 3 * sizeof(unsigned long long)));
    SONG_CUDA(cudaMemset(ix->d_head_stats, 0, 3 * sizeof(unsigned long long)));
  }
  if (stats) {
    stats[0] = stats[1] = stats[2] = 0;
    if (ix->d_head_stats) {
      SONG_CUDA(cudaStreamSynchronize(ix->stream));
      SONG_CUDA(cudaDeviceSynchronize());
      SONG_CUDA(cudaMemcpy(stats, ix->d_head_stats, 3 * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
      SONG_CUDA(cudaMemset(ix->d_head_stats, 0, 3 * sizeof(unsigned long long)));
    }
  }
  ix->head_stats_on = enable != 0;
  return SONG_OK;
}

int song_debug_head_scores(song_index *ix, const float *d_queries, int nq, float *d_scores, int ld) {
  g_last_error.clear();
  if (!ix || nq < 0 || (nq > 0 && (!d_queries || !d_scores))) return fail(SONG_ERR_ARG, "bad arguments");
  if (!ix->heads_mma) return fail(SONG_ERR_ARG, "no tensor-core head phase on this index");
  if (ld < ix->n_coarse || ld % 4 != 0) return fail(SONG_ERR_ARG, "ld must be >= the coarse entries and a multiple of 4");
  if (nq == 0) return SONG_OK;
  DeviceGuard g(ix->device);
  if (!g.ok) return fail(SONG_ERR_CUDA, "cannot select device %d", ix->device);
  SONG_CUDA(cudaMemsetAsync(ix->d_error, 0, sizeof(int32_t), ix->stream));
  cudaError_t e = song::launch_head_scores_only(ix, d_queries, nq, d_scores, ld, ix->stream);
  if (e == cudaErrorInvalidValue) return fail(SONG_ERR_ARG, "queries must be 16-byte aligned");
  SONG_CUDA(e);
  SONG_CUDA(cudaStreamSynchronize(ix->stream));
  int32_t err = 0;
  SONG_CUDA(cudaMemcpy(&err, ix->d_error, sizeof err, cudaMemcpyDeviceToHost));
  if (err) return fail(SONG_ERR_CUDA, "a bulk copy or the matrix multiply never completed (bounded wait)");
  return SONG_OK;
}

int song_debug_fixhash(const uint32_t *ids, int count, int pq, int32_t *slots_out) {
  g_last_error.clear();
  if (count < 0 || pq < 2 || pq > SONG_MAX_PQ || (count > 0 && (!ids || !slots_out)))
    return fail(SONG_ERR_ARG, "bad arguments");
  if (count == 0) return SONG_OK;
  uint32_t *d_ids = nullptr;
  int32_t *d_out = nullptr;
  SONG_CUDA(song::dev_malloc(&d_ids, count * sizeof(uint32_t)));
  cudaError_t e = song::dev_malloc(&d_out, count * sizeof(int32_t));
  if (e == cudaSuccess)
    e = cudaMemcpy(d_ids, ids, count * sizeof(uint32_t), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    int le = song::launch_debug_fixhash(d_ids, count, pq, d_out, 0);
    e = static_cast<cudaError_t>(le);
  }
  if (e == cudaSuccess)
    e = cudaMemcpy(slots_out, d_out, count * sizeof(int32_t), cudaMemcpyDeviceToHost);
  cudaFree(d_ids);
  cudaFree(d_out);
  if (e != cudaSuccess) return fail(SONG_ERR_CUDA, "debug fixhash: %s", cudaGetErrorString(e));
  return SONG_OK;
}


int song_index_set_rerank(song_index *ix, int rerank) {
  g_last_error.clear();
  if (!ix) return fail(SONG_ERR_ARG, "null index");
  if (rerank < -1 || rerank > SONG_MAX_PQ) return fail(SONG_ERR_ARG, "rerank must be in [-1, %d]", SONG_MAX_PQ);
  ix->rerank = rerank;
  return SONG_OK;
}

int song_index_set_early_exit(song_index *ix, const float *weights, float threshold, int min_hops,
                              int every) {
  g_last_error.clear();
  if (!ix) return fail(SONG_ERR_ARG, "null index");
  DeviceGuard g(ix->device);
  if (!g.ok) return fail(SONG_ERR_CUDA, "cannot select device %d", ix->device);
  if (!weights) {
    cudaFree(ix->d_mlp);
    ix->d_mlp = nullptr;
    return SONG_OK;
  }
  if (every < 1 || min_hops < 0) return fail(SONG_ERR_ARG, "every must be >= 1 and min_hops >= 0");
  if (ix->dx.storage >= SONG_STORAGE_FP8) return fail(SONG_ERR_ARG, "early exit is built for F32 and BF16 storage");
  if (song::multi_knobs(ix->probes, ix->finish_cnt, ix->double_check))
    return fail(SONG_ERR_ARG, "early exit does not combine with multi-probe search");
  std::vector<__nv_bfloat16> w(SONG_MLP_PARAMS);
  for (int i = 0; i < SONG_MLP_PARAMS; ++i) w[i] = __float2bfloat16_rn(weights[i]);
  if (!ix->d_mlp) {
    SONG_CUDA(song::dev_malloc(reinterpret_cast<void **>(&ix->d_mlp), sizeof(__nv_bfloat16) * SONG_MLP_PARAMS));
    ix->device_bytes += sizeof(__nv_bfloat16) * SONG_MLP_PARAMS;
  }
  SONG_CUDA(cudaMemcpy(ix->d_mlp, w.data(), sizeof(__nv_bfloat16) * SONG_MLP_PARAMS, cudaMemcpyHostToDevice));
  ix->exit_threshold = threshold;
  ix->exit_min_hops = min_hops;
  ix->exit_every = every;
  return SONG_OK;
}

int song_index_set_timing(song_index *ix, int enable) {
  g_last_error.clear();
  if (!ix) return fail(SONG_ERR_ARG, "null index");
  DeviceGuard g(ix->device);
  if (!g.ok) return fail(SONG_ERR_CUDA, "cannot select device %d", ix->device);
  if (enable)
    for (cudaEvent_t &e : ix->ev)
      if (!e) SONG_CUDA(cudaEventCreate(&e));
  ix->timing = enable != 0;
  ix->timed_entries = false;
  return SONG_OK;
}

int song_index_timing(song_index *ix, float *entry_ms, float *search_ms) {
  g_last_error.clear();
  if (!ix || !ix->ev[2]) return fail(SONG_ERR_ARG, "timing is not enabled on this index");
  DeviceGuard g(ix->device);
  if (!g.ok) return fail(SONG_ERR_CUDA, "cannot select device %d", ix->device);
  SONG_CUDA(cudaEventSynchronize(ix->ev[2]));
  float a = 0.0f, b = 0.0f;
  if (ix->timed_entries) SONG_CUDA(cudaEventElapsedTime(&a, ix->ev[0], ix->ev[1]));
  SONG_CUDA(cudaEventElapsedTime(&b, ix->ev[1], ix->ev[2]));
  if (entry_ms) *entry_ms = a;
  if (search_ms) *search_ms = b;
  return SONG_OK;
}

int song_index_set_multiprobe(song_index *ix, int probes, int finish_cnt, int double_check) {
  g_last_error.clear();
  if (!ix) return fail(SONG_ERR_ARG, "null index");
  if (probes < 1 || probes > SONG_MAX_PROBES || finish_cnt < 1)
    return fail(SONG_ERR_ARG, "probes must be in [1, %d] and finish_cnt >= 1", SONG_MAX_PROBES);
  const bool multi = song::multi_knobs(probes, finish_cnt, double_check);
  if (multi && ix->dx.storage != SONG_STORAGE_F32)
    return fail(SONG_ERR_ARG, "multi-probe search is built for F32 storage");
  if (multi && (ix->d_mlp || ix->max_hops > 0))
    return fail(SONG_ERR_ARG, "multi-probe search does not combine with early exit or a hop limit");
  ix->probes = probes;
  ix->finish_cnt = finish_cnt;
  ix->double_check = double_check != 0;
  return SONG_OK;
}

int song_index_set_hop_limit(song_index *ix, int max_hops) {
  g_last_error.clear();
  if (!ix) return fail(SONG_ERR_ARG, "null index");
  if (max_hops < 0) return fail(SONG_ERR_ARG, "max_hops must be >= 0");
  if (max_hops > 0 && ix->dx.storage >= SONG_STORAGE_FP8)
    return fail(SONG_ERR_ARG, "the hop limit is built for F32 and BF16 storage");
  if (max_hops > 0 && song::multi_knobs(ix->probes, ix->finish_cnt, ix->double_check))
    return fail(SONG_ERR_ARG, "a hop limit does not combine with multi-probe search");
  ix->max_hops = max_hops;
  return SONG_OK;
}

int song_search_trace_device(song_index *ix, const float *d_queries, int nq, int pq, int k,
                             int trace_hops, float *d_trace, int32_t *d_final, uint64_t *d_out,
                             int32_t *d_hops, int32_t *d_evals, void *stream) {
  g_last_error.clear();
  int rc = check_search_args(ix, nq, pq, k);
  if (rc) return rc;
  if (nq == 0) return SONG_OK;
  if (!d_queries || !d_out || !d_trace || !d_final || trace_hops < 1)
    return fail(SONG_ERR_ARG, "null buffer or trace_hops < 1");
  if (ix->dx.storage >= SONG_STORAGE_FP8) return fail(SONG_ERR_ARG, "tracing is built for F32 and BF16 storage");
  if (song::multi_knobs(ix->probes, ix->finish_cnt, ix->double_check))
    return fail(SONG_ERR_ARG, "tracing records the single-probe search: reset the multi-probe knobs first");
  DeviceGuard g(ix->device);
  if (!g.ok) return fail(SONG_ERR_CUDA, "cannot select device %d", ix->device);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  song::SearchCall c;
  c.queries = d_queries;
  c.nq = nq;
  c.pq = pq;
  c.k = k;
  c.out = d_out;
  c.hops = d_hops;
  c.evals = d_evals;
  c.counter = ix->d_counter;
  c.error = ix->d_error;
  song::apply_index_settings(ix, c);
  c.mlp = nullptr;  // traces record the full search
  c.exit_max_hops = 0;
  c.trace = d_trace;
  c.trace_hops = trace_hops;
  c.trace_final = d_final;
  rc = song::prepare_starts(ix, c, s);
  if (rc != SONG_OK) return rc;
  SONG_CUDA(cudaMemsetAsync(ix->d_error, 0, sizeof(int32_t), s));
  int e = song::launch_search(ix->dx, c, s);
  if (e == -1) return fail(SONG_ERR_ARG, "unsupported search shape");
  if (e != 0) return fail(SONG_ERR_CUDA, "trace launch: %s", cudaGetErrorString((cudaError_t)e));
  return SONG_OK;
}

int song_index_rows(const song_index *ix, uint64_t first, uint64_t count, void *out, size_t out_bytes,
                    int *row_bytes) {
  g_last_error.clear();
  if (!ix) return fail(SONG_ERR_ARG, "null index");
  if (row_bytes) *row_bytes = static_cast<int>(ix->dx.row_bytes);
  if (!out) return SONG_OK;
  const size_t need = static_cast<size_t>(count) * ix->dx.row_bytes;
  if (first > ix->dx.n || count > ix->dx.n - first || out_bytes < need)
    return fail(SONG_ERR_ARG, "rows out of range or buffer too small");
  DeviceGuard g(ix->device);
  if (!g.ok) return fail(SONG_ERR_CUDA, "cannot select device %d", ix->device);
  SONG_CUDA(cudaMemcpy(out, static_cast<const uint8_t *>(ix->d_rows) + first * ix->dx.row_bytes, need,
                       cudaMemcpyDeviceToHost));
  return SONG_OK;
}

}  // extern "C"
