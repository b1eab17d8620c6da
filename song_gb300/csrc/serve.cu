// serve.cu -- continuous-batching search service (no counterpart in the
// reference, whose only entry point is one synchronous batch,
// warp_astar_accelerator.h:347-423).
//
// One server per resident index.  A persistent kernel (serve_kernel) keeps a
// share of the GPU's warps polling a ring of work entries that the host
// publishes; each entry is one query with its own pq and k.  Requests of 1..N
// queries are admitted while a slot of the server's query/result memory is
// free (admission by memory); otherwise they wait in a host FIFO and are
// admitted as earlier requests complete.  New requests' queries go straight to
// the polling warps, so their work overlaps with requests already on the
// device.  Queries are read from, and ids written to, mapped pinned host memory
// (zero-copy); a per-slot completion counter is bumped after each query with
// system-scope release ordering, and the host polls it.
//
// Waits are bounded: a warp that finds no work for `idle_polls` polls (about
// a second by default; song_server_set_idle_polls) exits (an idle exit, not
// an error); when every warp has exited the host relaunches the kernel on the
// next submission.  The host's own wait for a request, song_server_wait, is
// bounded too and returns SONG_ERR_TIMEOUT.  Warps claim an entry only after it is
// published, so an exiting warp never holds unprocessed work.
#include <cuda_runtime.h>

#include <atomic>
#include <chrono>
#include <cstdint>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <vector>

#include "internal.h"
#include "entry_choice.cuh"
#include "search_kernel.cuh"
#include "song_gb300.h"

namespace song {
namespace {

constexpr uint32_t SERVE_IDLE_POLLS = 1u << 21;  // default; x ~0.5 us backoff: about a second idle

struct ServeEntry {
  uint64_t query;    // device-visible address of the query vector
  uint64_t out;      // device-visible address of the k result ids
  uint32_t slot;     // completion counter
  uint16_t pq, k;
};

struct ServeCtl {
  uint32_t published;  // entries published (host writes, release)
  uint32_t closing;    // host sets 1 to stop the kernel once the ring is drained
  uint32_t pad[14];
};

__device__ __forceinline__ uint32_t ld_acquire_sys(const uint32_t *p) {
  uint32_t v;
  asm volatile("ld.acquire.sys.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ uint32_t ld_volatile(const uint32_t *p) {
  return *reinterpret_cast<const volatile uint32_t *>(p);
}

// The entry choice of entries.cu (flat or two-level, same definition, same
// arithmetic) made by one warp for one query staged in qv (zero-padded to
// entry_dpad floats): the p.n_starts starts, nearest first, into out[].
template <int METRIC>
__device__ __forceinline__ void serve_choose_starts(const Params &p, const float *qv, uint32_t *out, int lane) {
  const int d4 = p.entry_dpad >> 2;
  const float4 *q4 = reinterpret_cast<const float4 *>(qv);
  constexpr int NL = 8;  // SONG_MAX_STARTS
  float bd[NL];
  uint32_t bi[NL];
#pragma unroll
  for (int m = 0; m < NL; ++m) {
    bd[m] = __int_as_float(0x7f800000);
    bi[m] = 0xffffffffu;
  }
  if (p.n_coarse > 0) {
    // heads (sorted by id: the position is the tie order), then the clusters
    float hd[NL];
    uint32_t hi[NL];
#pragma unroll
    for (int m = 0; m < NL; ++m) {
      hd[m] = __int_as_float(0x7f800000);
      hi[m] = 0xffffffffu;
    }
    for (int c = lane; c < p.n_coarse; c += 32)
      list_insert<NL>(hd, hi,
                      entry_distance<METRIC, true>(
                          reinterpret_cast<const float4 *>(p.coarse_rows + static_cast<size_t>(c) * p.entry_dpad), q4, d4),
                      static_cast<uint32_t>(c));
    int h = 0;
    uint32_t mine = 0;
    for (int r = 0; r < p.n_probes; ++r) {
      const uint32_t c = list_take<NL>(hd, hi, h);
      if (lane == r) mine = c;
    }
    for (int r = 0; r < p.n_probes; ++r) {
      const uint32_t c = __shfl_sync(FULL, mine, r);
      const uint32_t end = p.entry_offsets[c + 1];
      for (uint32_t e = p.entry_offsets[c] + lane; e < end; e += 32)
        list_insert<NL>(bd, bi,
                        entry_distance<METRIC, true>(
                            reinterpret_cast<const float4 *>(p.entry_rows + static_cast<size_t>(e) * p.entry_dpad), q4, d4),
                        p.entry_ids[e]);
    }
  } else {
    for (int e = lane; e < p.n_entries; e += 32)
      list_insert<NL>(bd, bi,
                      entry_distance<METRIC, true>(
                          reinterpret_cast<const float4 *>(p.entry_rows + static_cast<size_t>(e) * p.entry_dpad), q4, d4),
                      p.entry_ids[e]);
  }
  int h = 0;
  for (int r = 0; r < p.n_starts; ++r) {
    const uint32_t id = list_take<NL>(bd, bi, h);
    if (lane == 0) out[r] = id;
  }
  __syncwarp();
}

template <int METRIC, int STORAGE, int H, int S>
__global__ void __launch_bounds__(MAX_WARPS_PER_BLOCK * 32, 1)
    serve_kernel(const Params p, const ServeEntry *ring, uint32_t ring_mask, const ServeCtl *ctl,
                 uint32_t *next, uint32_t *done, uint32_t idle_polls) {
  extern __shared__ __align__(128) uint8_t smem_raw[];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  uint8_t *ws = smem_raw + static_cast<size_t>(wib) * p.warp_bytes;
  WarpCtx w;
  w.stage = ws;
  w.mbar = reinterpret_cast<uint64_t *>(ws + p.off_mbar);
  w.cbuf = reinterpret_cast<uint32_t *>(ws + p.off_cand);
  w.qv = reinterpret_cast<float *>(ws + p.off_q);
  w.tab = reinterpret_cast<int32_t *>(ws + p.off_hash);
  w.wmlp = nullptr;
  if (lane == 0) {
    mbar_init(&w.mbar[0], 1);
    mbar_init(&w.mbar[1], 1);
    fence_mbar_init();
  }
  __syncwarp();
  w.ph0 = 0;
  w.ph1 = 0;
  for (;;) {
    uint32_t idx = 0;
    int state = 0;  // 1 claimed, 2 closing, 3 idle
    if (lane == 0) {
      for (uint32_t polls = 0;; ++polls) {
        const uint32_t pub = ld_acquire_sys(&ctl->published);
        const uint32_t cur = ld_volatile(next);
        if (cur < pub) {
          if (atomicCAS(next, cur, cur + 1) == cur) {
            idx = cur;
            state = 1;
            break;
          }
          continue;
        }
        if (ld_volatile(&ctl->closing)) {
          state = 2;
          break;
        }
        if (polls >= idle_polls) {
          state = 3;
          break;
        }
        __nanosleep(500);
      }
    }
    state = __shfl_sync(FULL, state, 0);
    idx = __shfl_sync(FULL, idx, 0);
    if (state != 1) return;
    (void)ld_acquire_sys(&ctl->published);  // every lane: order the entry's and query's reads
    const ServeEntry e = ring[idx & ring_mask];
    QueryStats st;
    const uint32_t *starts = nullptr;
    if (p.entry_rows) {  // entry points: the starts go to the candidate buffer, which run_query reads first
      const float *qsrc = reinterpret_cast<const float *>(e.query);
      for (int j = lane; j < p.entry_dpad; j += 32) w.qv[j] = j < p.dim ? qsrc[j] : 0.0f;
      __syncwarp();
      serve_choose_starts<METRIC>(p, w.qv, w.cbuf, lane);
      starts = w.cbuf;
    }
    if (!run_query<METRIC, STORAGE, H, S, false>(p, w, reinterpret_cast<const float *>(e.query), starts,
                                                 p.n_starts, e.pq, e.k,
                                                 reinterpret_cast<uint64_t *>(e.out), nullptr, st, lane)) {
      if (lane == 0) atomicOr(p.error, 1);
      return;
    }
    __threadfence_system();  // the ids before the completion count
    __syncwarp();
    if (lane == 0) atomicAdd_system(&done[e.slot], 1u);
  }
}

int queue_segment(int pq) {
  int s = 1;
  while (32 * s < pq + 1) s <<= 1;
  return s;
}

uint32_t align_up(uint32_t x, uint32_t a) { return (x + a - 1) / a * a; }

template <int METRIC, int STORAGE, int H, int S>
cudaError_t launch_serve(const Params &p, const ServeEntry *ring, uint32_t mask, const ServeCtl *ctl,
                         uint32_t *next, uint32_t *done, float fraction, uint32_t idle, cudaStream_t s) {
  auto kern = serve_kernel<METRIC, STORAGE, H, S>;
  int wpb = 0, cap = 0;
  int e = get_shape(reinterpret_cast<const void *>(kern), p.warp_bytes, 0u, &wpb, &cap);
  if (e != 0) return e == -1 ? cudaErrorInvalidConfiguration : static_cast<cudaError_t>(e);
  int grid = static_cast<int>(fraction * cap + 0.5f);
  if (grid < 1) grid = 1;
  if (grid > cap) grid = cap;
  kern<<<grid, wpb * 32, static_cast<size_t>(p.warp_bytes) * wpb, s>>>(p, ring, mask, ctl, next, done, idle);
  return cudaGetLastError();
}

template <int METRIC, int H>
cudaError_t launch_serve_s(int S, const Params &p, const ServeEntry *ring, uint32_t mask, const ServeCtl *ctl,
                           uint32_t *next, uint32_t *done, float f, uint32_t idle, cudaStream_t s) {
  switch (S) {
    case 1:
    case 2:
    case 4: return launch_serve<METRIC, 0, H, 4>(p, ring, mask, ctl, next, done, f, idle, s);
    case 8: return launch_serve<METRIC, 0, H, 8>(p, ring, mask, ctl, next, done, f, idle, s);
    case 16: return launch_serve<METRIC, 0, H, 16>(p, ring, mask, ctl, next, done, f, idle, s);
    default: return launch_serve<METRIC, 0, H, 32>(p, ring, mask, ctl, next, done, f, idle, s);
  }
}

cudaError_t launch_serve_any(int metric, int H, int S, const Params &p, const ServeEntry *ring, uint32_t mask,
                             const ServeCtl *ctl, uint32_t *next, uint32_t *done, float f, uint32_t idle,
                             cudaStream_t s) {
  switch (metric * 2 + (H == 4 ? 1 : 0)) {
    case 0: return launch_serve_s<0, 2>(S, p, ring, mask, ctl, next, done, f, idle, s);
    case 1: return launch_serve_s<0, 4>(S, p, ring, mask, ctl, next, done, f, idle, s);
    case 2: return launch_serve_s<1, 2>(S, p, ring, mask, ctl, next, done, f, idle, s);
    case 3: return launch_serve_s<1, 4>(S, p, ring, mask, ctl, next, done, f, idle, s);
    case 4: return launch_serve_s<2, 2>(S, p, ring, mask, ctl, next, done, f, idle, s);
    default: return launch_serve_s<2, 4>(S, p, ring, mask, ctl, next, done, f, idle, s);
  }
}

}  // namespace
}  // namespace song

struct song_server {
  struct Slot {
    bool busy = false;
    bool complete = false;
    uint64_t ticket = 0;
    int nq = 0, pq = 0, k = 0;
  };
  struct Pending {
    uint64_t ticket;
    int nq, pq, k;
    std::vector<float> queries;
  };
  song_index *ix = nullptr;
  int max_pq = 0, max_k = 0, nslots = 0, slot_queries = 0, S = 0, H = 0;
  float fraction = 1.0f;
  cudaStream_t stream = nullptr;
  song::Params params{};
  // mapped pinned host memory
  float *h_q = nullptr;
  uint64_t *h_out = nullptr;
  song::ServeEntry *h_ring = nullptr;
  song::ServeCtl *h_ctl = nullptr;
  uint32_t *h_done = nullptr;
  float *d_q = nullptr;
  uint64_t *d_out = nullptr;
  song::ServeEntry *d_ring = nullptr;
  song::ServeCtl *d_ctl = nullptr;
  uint32_t *d_done = nullptr;
  uint32_t *d_next = nullptr;  // device memory
  uint32_t ring_mask = 0;
  uint32_t published = 0;
  bool running = false;
  bool holds_entries = false;  // counted in ix->servers: the index's entries stay fixed
  uint32_t idle_polls = song::SERVE_IDLE_POLLS;
  bool hold = false;           // test hook: admitted requests are not published while set
  uint64_t next_ticket = 1;
  std::vector<Slot> slots;
  std::deque<Pending> pending;
  std::deque<uint64_t> completed;
  std::mutex mu;
};

namespace {

using song::fail;

int relaunch_if_idle(song_server *s) {
  if (s->running) {
    const cudaError_t q = cudaStreamQuery(s->stream);
    if (q == cudaErrorNotReady) return SONG_OK;
    if (q != cudaSuccess) return fail(SONG_ERR_CUDA, "serve kernel: %s", cudaGetErrorString(q));
    s->running = false;
  }
  // Every warp has left and none holds a claim, so the claim counter already
  // counts exactly the processed entries: the new launch continues from it.
  cudaError_t e = song::launch_serve_any(s->ix->dx.metric, s->H, s->S, s->params, s->d_ring, s->ring_mask, s->d_ctl,
                                         s->d_next, s->d_done, s->fraction, s->idle_polls, s->stream);
  if (e != cudaSuccess) return fail(SONG_ERR_CUDA, "serve launch: %s", cudaGetErrorString(e));
  s->running = true;
  return SONG_OK;
}

void admit(song_server *s, int slot_i, song_server::Pending &r) {
  song_server::Slot &sl = s->slots[slot_i];
  sl.busy = true;
  sl.complete = false;
  sl.ticket = r.ticket;
  sl.nq = r.nq;
  sl.pq = r.pq;
  sl.k = r.k;
  const int dim = s->ix->dx.dim;
  float *q = s->h_q + static_cast<size_t>(slot_i) * s->slot_queries * dim;
  std::memcpy(q, r.queries.data(), sizeof(float) * r.nq * dim);
  __atomic_store_n(&s->h_done[slot_i], 0u, __ATOMIC_RELAXED);
  for (int i = 0; i < r.nq; ++i) {
    song::ServeEntry &e = s->h_ring[(s->published + i) & s->ring_mask];
    e.query = reinterpret_cast<uint64_t>(s->d_q + (static_cast<size_t>(slot_i) * s->slot_queries + i) * dim);
    e.out = reinterpret_cast<uint64_t>(s->d_out + (static_cast<size_t>(slot_i) * s->slot_queries + i) * s->max_k);
    e.slot = static_cast<uint32_t>(slot_i);
    e.pq = static_cast<uint16_t>(r.pq);
    e.k = static_cast<uint16_t>(r.k);
  }
  s->published += static_cast<uint32_t>(r.nq);
  if (s->hold) return;  // the entries wait in the ring until the hold is released
  std::atomic_thread_fence(std::memory_order_release);
  __atomic_store_n(&s->h_ctl->published, s->published, __ATOMIC_RELEASE);
}

int free_slot(const song_server *s) {
  for (int i = 0; i < s->nslots; ++i)
    if (!s->slots[i].busy) return i;
  return -1;
}

void admit_pending(song_server *s) {
  while (!s->pending.empty()) {
    const int fs = free_slot(s);
    if (fs < 0) return;
    admit(s, fs, s->pending.front());
    s->pending.pop_front();
  }
}

}  // namespace

extern "C" {

int song_server_create(song_index *ix, int max_pq, int max_k, int nslots, int slot_queries, float sm_fraction,
                       song_server **out) {
  song::clear_error();
  if (!ix || !out) return fail(SONG_ERR_ARG, "null argument");
  *out = nullptr;
  if (max_pq < 2 || max_pq > SONG_MAX_PQ || max_k < 1 || max_k > max_pq || nslots < 1 || slot_queries < 1 ||
      sm_fraction <= 0.0f || sm_fraction > 1.0f)
    return fail(SONG_ERR_ARG, "bad server limits");
  if (ix->dx.storage != SONG_STORAGE_F32) return fail(SONG_ERR_ARG, "the server is built for F32 storage");
  if (song::multi_knobs(ix->probes, ix->finish_cnt, ix->double_check))
    return fail(SONG_ERR_ARG, "the server runs the single-probe search: reset the multi-probe knobs first");
  int prev = -1;
  cudaGetDevice(&prev);
  if (prev != ix->device) cudaSetDevice(ix->device);
  song_server *s = new song_server();
  s->ix = ix;
  s->max_pq = max_pq;
  s->max_k = max_k;
  s->nslots = nslots;
  s->slot_queries = slot_queries;
  s->fraction = sm_fraction;
  s->slots.resize(nslots);
  const song::DeviceIndex &dx = ix->dx;
  const int dim = dx.dim;
  uint32_t ring = 1;
  while (ring < static_cast<uint32_t>(nslots) * static_cast<uint32_t>(slot_queries)) ring <<= 1;
  s->ring_mask = ring - 1;
  const size_t qbytes = sizeof(float) * static_cast<size_t>(nslots) * slot_queries * dim;
  const size_t obytes = sizeof(uint64_t) * static_cast<size_t>(nslots) * slot_queries * max_k;
  cudaError_t e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
  const unsigned fl = cudaHostAllocMapped | cudaHostAllocPortable;
  if (e == cudaSuccess) e = cudaHostAlloc(reinterpret_cast<void **>(&s->h_q), qbytes, fl);
  if (e == cudaSuccess) e = cudaHostAlloc(reinterpret_cast<void **>(&s->h_out), obytes, fl);
  if (e == cudaSuccess) e = cudaHostAlloc(reinterpret_cast<void **>(&s->h_ring), sizeof(song::ServeEntry) * ring, fl);
  if (e == cudaSuccess) e = cudaHostAlloc(reinterpret_cast<void **>(&s->h_ctl), sizeof(song::ServeCtl), fl);
  if (e == cudaSuccess) e = cudaHostAlloc(reinterpret_cast<void **>(&s->h_done), sizeof(uint32_t) * nslots, fl);
  if (e == cudaSuccess) e = cudaHostGetDevicePointer(reinterpret_cast<void **>(&s->d_q), s->h_q, 0);
  if (e == cudaSuccess) e = cudaHostGetDevicePointer(reinterpret_cast<void **>(&s->d_out), s->h_out, 0);
  if (e == cudaSuccess) e = cudaHostGetDevicePointer(reinterpret_cast<void **>(&s->d_ring), s->h_ring, 0);
  if (e == cudaSuccess) e = cudaHostGetDevicePointer(reinterpret_cast<void **>(&s->d_ctl), s->h_ctl, 0);
  if (e == cudaSuccess) e = cudaHostGetDevicePointer(reinterpret_cast<void **>(&s->d_done), s->h_done, 0);
  if (e == cudaSuccess) e = song::dev_malloc(&s->d_next, 256);
  if (e == cudaSuccess) e = cudaMemsetAsync(s->d_next, 0, 256, s->stream);
  if (e != cudaSuccess) {
    int rc = fail(e == cudaErrorMemoryAllocation ? SONG_ERR_OOM : SONG_ERR_CUDA, "server create: %s",
                  cudaGetErrorString(e));
    song_server_destroy(s);
    if (prev >= 0 && prev != ix->device) cudaSetDevice(prev);
    return rc;
  }
  std::memset(s->h_ctl, 0, sizeof(song::ServeCtl));
  std::memset(s->h_done, 0, sizeof(uint32_t) * nslots);
  // kernel parameters: the search layout for the largest pq
  s->S = song::queue_segment(max_pq);
  s->H = dx.row_bytes <= 1024 ? 4 : 2;
  song::Params &p = s->params;
  std::memset(&p, 0, sizeof p);
  p.rows = static_cast<const uint8_t *>(dx.rows);
  p.row_bytes = dx.row_bytes;
  p.scale_off = dx.scale_off;
  p.rows_f32 = dx.rows_f32;
  p.f32_row_bytes = dx.f32_row_bytes;
  p.adj = dx.adj;
  p.shift = dx.shift;
  p.dim = dim;
  p.error = ix->d_error;
  p.wait_limit = ix->wait_limit;
  p.extra_tx = ix->extra_tx;
  p.probes = 1;
  p.finish_cnt = 1;
  p.double_check = 0;
  p.n_starts = 1;
  if (ix->n_entries > 0) {  // the index's entry points, fixed for the server's life
    p.entry_rows = ix->d_entry_rows;
    p.entry_ids = ix->d_entry_ids;
    p.n_entries = ix->n_entries;
    p.coarse_rows = ix->d_coarse_rows;
    p.n_coarse = ix->n_coarse;
    p.entry_offsets = ix->d_offsets;
    p.n_probes = ix->n_probes;
    p.n_starts = ix->n_starts;
    p.entry_dpad = static_cast<int>(dx.f32_row_bytes / 4);
    ++ix->servers;
    s->holds_entries = true;
  }
  uint32_t off = 2u * s->H * dx.row_bytes;
  off = song::align_up(off, 16);
  p.off_mbar = off;
  off += 16;
  p.off_cand = off;
  off += 32 * 4;
  off = song::align_up(off, 16);
  p.off_q = off;
  off += song::align_up(static_cast<uint32_t>(dim) * 4u, 16);
  p.off_hash = off;
  off += 4u * 8u * static_cast<uint32_t>(max_pq);
  p.warp_bytes = song::align_up(off, 128);
  if (p.warp_bytes > 227u * 1024u) {
    song_server_destroy(s);
    return fail(SONG_ERR_ARG, "max_pq %d with dim %d does not fit a warp's shared memory", max_pq, dim);
  }
  int rc = relaunch_if_idle(s);
  if (prev >= 0 && prev != ix->device) cudaSetDevice(prev);
  if (rc) {
    song_server_destroy(s);
    return rc;
  }
  *out = s;
  return SONG_OK;
}

int song_server_submit(song_server *s, const float *queries, int nq, int pq, int k, uint64_t *ticket) {
  song::clear_error();
  if (!s || !queries || !ticket) return fail(SONG_ERR_ARG, "null argument");
  if (nq < 1 || nq > s->slot_queries) return fail(SONG_ERR_ARG, "nq must be in [1, %d]", s->slot_queries);
  if (pq < 2 || pq > s->max_pq || k < 1 || k > pq || k > s->max_k) return fail(SONG_ERR_ARG, "bad pq or k");
  if (pq < s->params.n_starts) return fail(SONG_ERR_ARG, "pq must be at least the %d entry starts", s->params.n_starts);
  std::lock_guard<std::mutex> lk(s->mu);
  int prev = -1;
  cudaGetDevice(&prev);
  if (prev != s->ix->device) cudaSetDevice(s->ix->device);
  song_server::Pending r;
  const uint64_t t = s->next_ticket++;
  r.ticket = t;
  r.nq = nq;
  r.pq = pq;
  r.k = k;
  r.queries.assign(queries, queries + static_cast<size_t>(nq) * s->ix->dx.dim);
  s->pending.push_back(std::move(r));
  admit_pending(s);
  int rc = relaunch_if_idle(s);
  if (prev >= 0 && prev != s->ix->device) cudaSetDevice(prev);
  *ticket = t;
  return rc;
}

int song_server_poll(song_server *s, uint64_t *tickets, int max, int *n_done) {
  song::clear_error();
  if (!s || !n_done || (max > 0 && !tickets)) return fail(SONG_ERR_ARG, "null argument");
  std::lock_guard<std::mutex> lk(s->mu);
  bool outstanding = false;
  for (int i = 0; i < s->nslots; ++i) {
    song_server::Slot &sl = s->slots[i];
    if (sl.busy && !sl.complete) outstanding = true;
    if (sl.busy && !sl.complete &&
        __atomic_load_n(&s->h_done[i], __ATOMIC_ACQUIRE) >= static_cast<uint32_t>(sl.nq)) {
      sl.complete = true;
      s->completed.push_back(sl.ticket);
    }
  }
  int n = 0;
  while (n < max && !s->completed.empty()) {
    tickets[n++] = s->completed.front();
    s->completed.pop_front();
  }
  *n_done = n;
  if (outstanding) {
    // a kernel whose warps all left on an idle wait just before new entries
    // were published is started again here
    int prev = -1;
    cudaGetDevice(&prev);
    if (prev != s->ix->device) cudaSetDevice(s->ix->device);
    const int rc = relaunch_if_idle(s);
    if (prev >= 0 && prev != s->ix->device) cudaSetDevice(prev);
    if (rc) return rc;
  }
  int32_t err = 0;
  // a search-kernel failure flag (a bounded copy wait that gave up)
  if (cudaMemcpy(&err, s->ix->d_error, sizeof(int32_t), cudaMemcpyDeviceToHost) == cudaSuccess && (err & 1))
    return fail(SONG_ERR_TIMEOUT, "a bulk copy wait timed out in the serve kernel");
  return SONG_OK;
}

int song_server_result(song_server *s, uint64_t ticket, uint64_t *out, int *nq, int *k) {
  song::clear_error();
  if (!s || !out) return fail(SONG_ERR_ARG, "null argument");
  std::lock_guard<std::mutex> lk(s->mu);
  for (int i = 0; i < s->nslots; ++i) {
    song_server::Slot &sl = s->slots[i];
    if (sl.busy && sl.ticket == ticket) {
      if (!sl.complete) return fail(SONG_ERR_ARG, "request %llu not complete", (unsigned long long)ticket);
      for (int q = 0; q < sl.nq; ++q)
        std::memcpy(out + static_cast<size_t>(q) * sl.k,
                    s->h_out + (static_cast<size_t>(i) * s->slot_queries + q) * s->max_k, sizeof(uint64_t) * sl.k);
      if (nq) *nq = sl.nq;
      if (k) *k = sl.k;
      sl.busy = false;
      sl.complete = false;
      int prev = -1;
      cudaGetDevice(&prev);
      if (prev != s->ix->device) cudaSetDevice(s->ix->device);
      admit_pending(s);
      int rc = relaunch_if_idle(s);
      if (prev >= 0 && prev != s->ix->device) cudaSetDevice(prev);
      return rc;
    }
  }
  return fail(SONG_ERR_ARG, "unknown request %llu", (unsigned long long)ticket);
}

int song_server_set_idle_polls(song_server *s, uint32_t polls) {
  song::clear_error();
  if (!s || polls < 1) return fail(SONG_ERR_ARG, "null server or polls < 1");
  std::lock_guard<std::mutex> lk(s->mu);
  s->idle_polls = polls;  // taken by the next launch
  return SONG_OK;
}

int song_server_running(song_server *s, int *running) {
  song::clear_error();
  if (!s || !running) return fail(SONG_ERR_ARG, "null argument");
  std::lock_guard<std::mutex> lk(s->mu);
  if (s->running) {
    const cudaError_t q = cudaStreamQuery(s->stream);
    if (q == cudaSuccess) s->running = false;
    else if (q != cudaErrorNotReady) return fail(SONG_ERR_CUDA, "serve kernel: %s", cudaGetErrorString(q));
  }
  *running = s->running ? 1 : 0;
  return SONG_OK;
}

int song_server_wait(song_server *s, uint64_t ticket, int timeout_ms) {
  song::clear_error();
  if (!s || timeout_ms < 0) return fail(SONG_ERR_ARG, "null server or negative timeout");
  const auto t0 = std::chrono::steady_clock::now();
  for (;;) {
    {
      std::lock_guard<std::mutex> lk(s->mu);
      int found = -1;
      for (int i = 0; i < s->nslots; ++i)
        if (s->slots[i].busy && s->slots[i].ticket == ticket) found = i;
      bool queued = false;
      for (const auto &r : s->pending) queued = queued || r.ticket == ticket;
      if (found < 0 && !queued) return fail(SONG_ERR_ARG, "unknown request %llu", (unsigned long long)ticket);
      if (found >= 0 && s->slots[found].complete) return SONG_OK;
      if (found >= 0 && __atomic_load_n(&s->h_done[found], __ATOMIC_ACQUIRE) >=
                            static_cast<uint32_t>(s->slots[found].nq)) {
        s->slots[found].complete = true;  // as song_server_poll marks it; poll reports it too
        s->completed.push_back(ticket);
        return SONG_OK;
      }
      int prev = -1;
      cudaGetDevice(&prev);
      if (prev != s->ix->device) cudaSetDevice(s->ix->device);
      const int rc = s->hold ? SONG_OK : relaunch_if_idle(s);
      if (prev >= 0 && prev != s->ix->device) cudaSetDevice(prev);
      if (rc) return rc;
    }
    const auto ms = std::chrono::duration_cast<std::chrono::milliseconds>(std::chrono::steady_clock::now() - t0);
    if (ms.count() >= timeout_ms)
      return fail(SONG_ERR_TIMEOUT, "request %llu not complete after %d ms", (unsigned long long)ticket, timeout_ms);
    std::this_thread::sleep_for(std::chrono::microseconds(50));
  }
}

int song_debug_server_hold(song_server *s, int hold) {
  song::clear_error();
  if (!s) return fail(SONG_ERR_ARG, "null server");
  std::lock_guard<std::mutex> lk(s->mu);
  s->hold = hold != 0;
  if (s->hold) return SONG_OK;
  // release: publish what was admitted meanwhile and make sure warps run
  std::atomic_thread_fence(std::memory_order_release);
  __atomic_store_n(&s->h_ctl->published, s->published, __ATOMIC_RELEASE);
  int prev = -1;
  cudaGetDevice(&prev);
  if (prev != s->ix->device) cudaSetDevice(s->ix->device);
  const int rc = relaunch_if_idle(s);
  if (prev >= 0 && prev != s->ix->device) cudaSetDevice(prev);
  return rc;
}

int song_server_destroy(song_server *s) {
  if (!s) return SONG_OK;
  int prev = -1;
  cudaGetDevice(&prev);
  if (s->ix && prev != s->ix->device) cudaSetDevice(s->ix->device);
  if (s->h_ctl) __atomic_store_n(&s->h_ctl->closing, 1u, __ATOMIC_RELEASE);
  if (s->stream) {
    cudaStreamSynchronize(s->stream);
    cudaStreamDestroy(s->stream);
  }
  cudaFreeHost(s->h_q);
  cudaFreeHost(s->h_out);
  cudaFreeHost(s->h_ring);
  cudaFreeHost(s->h_ctl);
  cudaFreeHost(s->h_done);
  cudaFree(s->d_next);
  if (s->holds_entries) --s->ix->servers;
  if (s->ix && prev >= 0 && prev != s->ix->device) cudaSetDevice(prev);
  delete s;
  return SONG_OK;
}

}  // extern "C"
