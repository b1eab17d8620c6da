// search_learned.cu -- instantiates the search kernel with per-hop features
// (trace capture and the early-exit network) for FP32 and BF16 storage.
#include "search_kernel.cuh"

namespace song {
int launch_learned(const Params &p, int storage, int metric, int H, int S, cudaStream_t s) {
  if (storage == 0) return launch_storage<0, true>(p, metric, H, S, s);
  if (storage == 1) return launch_storage<1, true>(p, metric, H, S, s);
  return -1;
}
}  // namespace song
