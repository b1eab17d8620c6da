// noalloc.cu -- song_search_noalloc: the host-buffer batched search without
// any device allocation.
//
// song_search stages the queries and the result ids in device buffers that
// the index allocates with cudaMalloc on first use and whenever a larger
// batch arrives, and the search kernel keeps its work counter and error flag
// in two more such allocations.  Some programs cannot let a library do that:
// a service that has already handed the whole GPU to its own memory pool (so
// a foreign cudaMalloc fails or breaks the pool's budget), or a latency-
// critical request path that must not pay for cudaMalloc, which may
// synchronise the device.  This entry point gives them the same search with
// all of that scratch taken from one fixed array compiled into the library:
//
//   * g_noalloc_scratch below, SONG_NOALLOC_SCRATCH_BYTES (16 MiB), is a
//     file-scope __device__ array; every GPU that loads the library holds it
//     until the process exits.
//   * Layout per call: [0, 8) work counter + error flag (cleared on the
//     stream before each launch), [256, ...) the queries, then the ids.
//     A batch needs 256 + round_up(nq * dim * 4, 256) + nq * k * 8 bytes;
//     larger batches are rejected with SONG_ERR_ARG.
//   * Each device has its own copy of the array.  Every call on a device uses
//     that copy and leaves its contents behind; calls whose work overlaps on
//     the same GPU (for example from two host threads at once) race on it,
//     so callers must serialise them.
//   * The device address of the array is looked up once per device, on the
//     first call made with that device current (cudaGetSymbolAddress; the
//     array's name in host code is only a host-side stand-in and must never
//     be handed to a kernel).  That first call should come before any stream
//     capture is started on the device.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "internal.h"
#include "song_gb300.h"

namespace {

static __device__ __align__(256) unsigned char g_noalloc_scratch[SONG_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void *g_scratch_addr[kMaxDevices] = {};

// Device address of g_noalloc_scratch on the current device.
int scratch_address(void **out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return song::fail(SONG_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return song::fail(SONG_ERR_ARG, "device %d out of range", dev);
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_scratch_addr[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return song::fail(SONG_ERR_CUDA, "cudaGetSymbolAddress(scratch): %s", cudaGetErrorString(e));
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return SONG_OK;
}

size_t round_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

}  // namespace

extern "C" int song_search_noalloc(song_index *ix, const float *queries, int nq, int pq, int k,
                                   uint64_t *out) {
  song::clear_error();
  int rc = song::check_search_args(ix, nq, pq, k);
  if (rc) return rc;
  if (nq == 0) return SONG_OK;
  if (!queries || !out) return song::fail(SONG_ERR_ARG, "null queries or out");
  const size_t qbytes = static_cast<size_t>(nq) * ix->dx.dim * sizeof(float);
  const size_t obytes = static_cast<size_t>(nq) * k * sizeof(uint64_t);
  const size_t need = 256 + round_up(qbytes, 256) + obytes;
  if (need > SONG_NOALLOC_SCRATCH_BYTES)
    return song::fail(SONG_ERR_ARG,
                      "batch needs %zu bytes of scratch (nq %d, dim %d, k %d); song_search_noalloc has "
                      "%zu: split the batch or use song_search",
                      need, nq, ix->dx.dim, k, static_cast<size_t>(SONG_NOALLOC_SCRATCH_BYTES));

  int prev = -1;
  cudaGetDevice(&prev);
  if (prev != ix->device && cudaSetDevice(ix->device) != cudaSuccess)
    return song::fail(SONG_ERR_CUDA, "cannot select device %d", ix->device);
  void *base = nullptr;
  rc = scratch_address(&base);
  unsigned char *b = static_cast<unsigned char *>(base);
  cudaStream_t s = ix->stream;
  cudaError_t e = cudaSuccess;
  int32_t err = 0;
  if (rc == SONG_OK) {
    uint32_t *counter = reinterpret_cast<uint32_t *>(b);
    int32_t *error = reinterpret_cast<int32_t *>(b + 4);
    float *d_q = reinterpret_cast<float *>(b + 256);
    uint64_t *d_out = reinterpret_cast<uint64_t *>(b + 256 + round_up(qbytes, 256));
    e = cudaMemsetAsync(b, 0, 8, s);  // counter and error flag start at zero
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_q, queries, qbytes, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
      song::SearchCall c;
      c.queries = d_q;
      c.nq = nq;
      c.pq = pq;
      c.k = k;
      c.out = d_out;
      c.counter = counter;
      c.error = error;
      song::apply_index_settings(ix, c);
      int le = song::launch_search(ix->dx, c, s);
      if (le == -1) rc = song::fail(SONG_ERR_ARG, "unsupported search shape");
      else e = static_cast<cudaError_t>(le);
    }
    if (rc == SONG_OK && e == cudaSuccess)
      e = cudaMemcpyAsync(out, d_out, obytes, cudaMemcpyDeviceToHost, s);
    if (rc == SONG_OK && e == cudaSuccess)
      e = cudaMemcpyAsync(&err, error, sizeof(int32_t), cudaMemcpyDeviceToHost, s);
    if (rc == SONG_OK && e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (rc == SONG_OK && e != cudaSuccess)
      rc = song::fail(SONG_ERR_CUDA, "song_search_noalloc: %s", cudaGetErrorString(e));
    if (rc == SONG_OK && err)
      rc = song::fail(SONG_ERR_TIMEOUT, "a bulk copy wait timed out in the search kernel");
  }
  if (prev >= 0 && prev != ix->device) cudaSetDevice(prev);
  return rc;
}
