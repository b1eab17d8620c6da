// search_f32.cu -- instantiates the search kernel for F32 storage (plain search).
#include "search_kernel.cuh"

namespace song {
int launch_f32(const Params &p, int metric, int H, int S, cudaStream_t s) {
  return launch_storage<0, false>(p, metric, H, S, s);
}
}  // namespace song
