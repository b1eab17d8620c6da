// search_bf16.cu -- instantiates the search kernel for BF16 storage (plain search).
#include "search_kernel.cuh"

namespace song {
int launch_bf16(const Params &p, int metric, int H, int S, cudaStream_t s) {
  return launch_storage<1, false>(p, metric, H, S, s);
}
}  // namespace song
