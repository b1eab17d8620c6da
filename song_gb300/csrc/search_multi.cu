// search_multi.cu -- instantiates the search kernel with the reference's
// N_MULTIPROBE / FINISH_CNT knobs (warp_astar_accelerator.h:29-30,178-232) as
// run-time values, for F32 storage (the reference's only storage).
#include "search_kernel.cuh"

namespace song {
int launch_multi(const Params &p, int metric, int H, int S, cudaStream_t s) {
  return launch_storage<0, false, true>(p, metric, H, S, s);
}
}  // namespace song
