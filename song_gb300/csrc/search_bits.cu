// search_bits.cu -- the 256-bit code row format (SONG_STORAGE_BITS): codes of
// vectors from the index's hyperplanes, and the search kernel instances that
// rank candidates by Hamming distance (the reference's bit-hash path,
// hash_warp_no_heap_astar_accelerator.h:22-41 for the codes, :96-104 and
// :226-235 for the __popc distances).
#include <cuda_runtime.h>

#include <vector>

#include "internal.h"
#include "search_kernel.cuh"
#include "song_gb300.h"

namespace song {

// One warp per vector: bit i of the code is (x . plane_i >= 0), the dot
// product summed as the search sums distances (lane l: dimensions l, l+32,
// ... with fused multiply-adds; the partials meet in the xor butterfly).  32
// planes at a time share one transposed butterfly, and a ballot of the 32
// signs is the code word.  rows: n vectors of `stride` floats (dim used);
// planes: SONG_HASH_BITS rows of pstride floats; codes: n x 8 words.
__global__ void hash_codes_kernel(const float *rows, uint64_t n, int stride, int dim, const float *planes,
                                  int pstride, uint32_t *codes) {
  const int lane = threadIdx.x & 31;
  const uint64_t warp = (blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x) >> 5;
  const uint64_t nwarps = (static_cast<uint64_t>(gridDim.x) * blockDim.x) >> 5;
  for (uint64_t r = warp; r < n; r += nwarps) {
    const float *x = rows + r * static_cast<uint64_t>(stride);
    for (int g = 0; g < SONG_HASH_BITS / 32; ++g) {
      float v[32];
#pragma unroll
      for (int i = 0; i < 32; ++i) v[i] = 0.0f;
      for (int j = lane; j < dim; j += 32) {
        const float xj = __ldg(x + j);
#pragma unroll
        for (int i = 0; i < 32; ++i)
          v[i] = __fmaf_rn(xj, __ldg(planes + static_cast<size_t>(g * 32 + i) * pstride + j), v[i]);
      }
      const float t = butterfly_rows<32>(v, lane);  // plane g*32 + lane
      const unsigned b = __ballot_sync(FULL, t >= 0.0f);
      if (lane == 0) codes[r * 8 + g] = b;
    }
  }
}

int launch_hash_codes(const float *rows, uint64_t n, int stride, int dim, const float *planes, int pstride,
                      uint32_t *codes, cudaStream_t s) {
  if (n == 0) return 0;
  const uint64_t blocks = (n + 7) / 8;  // 8 warps per block
  hash_codes_kernel<<<static_cast<unsigned>(blocks < 8192 ? blocks : 8192), 256, 0, s>>>(rows, n, stride, dim,
                                                                                        planes, pstride, codes);
  return cudaGetLastError();
}

int launch_bits(const Params &p, int metric, int S, cudaStream_t s) {
  switch (metric) {
    case 0: return launch_by_s<0, 3, 1, false>(p, S, s);
    case 1: return launch_by_s<1, 3, 1, false>(p, S, s);
    case 2: return launch_by_s<2, 3, 1, false>(p, S, s);
    default: return -1;
  }
}

}  // namespace song

extern "C" int song_index_set_hash_planes(song_index *ix, const float *planes) {
  using namespace song;
  clear_error();
  if (!ix || !planes) return fail(SONG_ERR_ARG, "null index or planes");
  if (ix->dx.storage != SONG_STORAGE_BITS) return fail(SONG_ERR_ARG, "hash planes are for SONG_STORAGE_BITS indexes");
  DeviceGuard g(ix->device);
  if (!g.ok) return fail(SONG_ERR_CUDA, "cannot select device %d", ix->device);
  const int dim = ix->dx.dim;
  const int pstride = static_cast<int>(ix->dx.f32_row_bytes / 4);
  std::vector<float> h(static_cast<size_t>(SONG_HASH_BITS) * pstride, 0.0f);
  for (int i = 0; i < SONG_HASH_BITS; ++i)
    for (int j = 0; j < dim; ++j) h[static_cast<size_t>(i) * pstride + j] = planes[static_cast<size_t>(i) * dim + j];
  cudaError_t e = cudaSuccess;
  if (!ix->d_planes) {
    e = dev_malloc(&ix->d_planes, sizeof(float) * h.size());
    if (e != cudaSuccess) return fail(SONG_ERR_OOM, "hash planes: %s", cudaGetErrorString(e));
    ix->device_bytes += sizeof(float) * h.size();
  }
  e = cudaMemcpyAsync(ix->d_planes, h.data(), sizeof(float) * h.size(), cudaMemcpyHostToDevice, ix->stream);
  if (e == cudaSuccess)
    e = static_cast<cudaError_t>(launch_hash_codes(ix->dx.rows_f32, ix->dx.n, pstride, dim, ix->d_planes, pstride,
                                                   static_cast<uint32_t *>(ix->d_rows), ix->stream));
  if (e == cudaSuccess) e = cudaStreamSynchronize(ix->stream);
  if (e != cudaSuccess) return fail(SONG_ERR_CUDA, "hash codes: %s", cudaGetErrorString(e));
  ix->has_planes = true;
  return SONG_OK;
}
