// search_fp8.cu -- instantiates the search kernel for FP8 storage (plain search).
#include "search_kernel.cuh"

namespace song {
int launch_fp8(const Params &p, int metric, int H, int S, cudaStream_t s) {
  return launch_storage<2, false>(p, metric, H, S, s);
}
}  // namespace song
