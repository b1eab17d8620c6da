// ref_gpu_runner.cpp -- launches the REFERENCE's own GPU search kernel
// (warp_independent_search_kernel, warp_astar_accelerator.h:41-341), rebuilt
// for sm_100 into a cubin by oracle/build_ref_gpu.sh, through the CUDA driver
// API, the way astar_multi_start_search_batch does (warp_astar_accelerator.h:
// 347-423): data, graph and densified queries uploaded, <<<nq, 32>>>, ids
// copied back.
//
// TEST INFRASTRUCTURE ONLY: the test of the FMA assumption of the oracle
// and the reference GPU baseline.  Built on the GPU host by oracle/ref_gpu.py.
//
// Safety: the kernel allocates its queues and visited hash with device-side
// new (warp_astar_accelerator.h:85-99) and dereferences the result unchecked.
// The runner therefore raises the device heap (cuCtxSetLimit) to twice what
// all resident blocks can hold at once and verifies the limit before any
// launch; it refuses to launch otherwise.
#include <cuda.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace {

struct Measure {
  unsigned long long s1, s2, s3;
};

int fail(char *err, int errlen, const char *what, CUresult r) {
  const char *msg = nullptr;
  cuGetErrorString(r, &msg);
  snprintf(err, errlen, "%s: %s", what, msg ? msg : "?");
  return static_cast<int>(r) ? static_cast<int>(r) : -1;
}

#define CK(call)                                            \
  do {                                                      \
    CUresult r_ = (call);                                   \
    if (r_ != CUDA_SUCCESS) {                               \
      rc = fail(err, errlen, #call, r_);                    \
      goto done;                                            \
    }                                                       \
  } while (0)

}  // namespace

// heap_pq: the largest pq_size this process will launch; the device heap is
// sized for it on the first call (it cannot grow once a kernel used it).
extern "C" int refgpu_run(const char *cubin, int measure, const float *data, uint64_t n, int dim,
                          const uint64_t *graph, int shift, const float *queries, int nq, int pq,
                          int heap_pq, uint64_t *out, float *kernel_ms, int repeats, char *err,
                          int errlen) {
  int rc = 0;
  CUdevice dev;
  CUcontext ctx = nullptr;
  CUmodule mod = nullptr;
  CUfunction fn;
  CUdeviceptr d_data = 0, d_query = 0, d_result = 0, d_graph = 0, d_measure = 0;
  CUevent e0 = nullptr, e1 = nullptr;
  int sms = 0;
  size_t heap = 0, got = 0, per_block = 0, resident = 0;
  const char *name = measure ? "_Z30warp_independent_search_kernelPfS_PmS0_iiP7Measure"
                             : "_Z30warp_independent_search_kernelPfS_PmS0_ii";
  err[0] = 0;
  CK(cuInit(0));
  CK(cuDeviceGet(&dev, 0));
  CK(cuDevicePrimaryCtxRetain(&ctx, dev));
  CK(cuCtxPushCurrent(ctx));
  CK(cuDeviceGetAttribute(&sms, CU_DEVICE_ATTRIBUTE_MULTIPROCESSOR_COUNT, dev));
  // per block: dist_list[31] f32, q[pq+2] and topk[pq+1] of 16-byte pairs,
  // FixHash<int, 8*pq> (+ its 16 uint64 constants); x2 for allocator overhead.
  if (heap_pq < pq) heap_pq = pq;
  per_block = 2 * (31 * 4 + (static_cast<size_t>(heap_pq) + 2) * 16 + (static_cast<size_t>(heap_pq) + 1) * 16 +
                   static_cast<size_t>(heap_pq) * 8 * 4 + 128) + 1024;
  resident = static_cast<size_t>(sms) * 32;  // at most 32 one-warp blocks per SM
  heap = 2 * per_block * resident;
  if (heap < (1ull << 30)) heap = 1ull << 30;
  // The limit can only grow before the first kernel that uses device new;
  // later calls in the same process find it already large enough.
  CK(cuCtxGetLimit(&got, CU_LIMIT_MALLOC_HEAP_SIZE));
  if (got < heap) {
    CK(cuCtxSetLimit(CU_LIMIT_MALLOC_HEAP_SIZE, heap));
    CK(cuCtxGetLimit(&got, CU_LIMIT_MALLOC_HEAP_SIZE));
  }
  // what this launch needs (the limit above may be sized for a larger pq)
  heap = 2 * (2 * (31 * 4 + (static_cast<size_t>(pq) + 2) * 16 + (static_cast<size_t>(pq) + 1) * 16 +
                   static_cast<size_t>(pq) * 8 * 4 + 128) + 1024) * resident;
  if (got < heap) {
    snprintf(err, errlen, "device heap limit %zu < required %zu; not launching", got, heap);
    rc = -2;
    goto done;
  }
  CK(cuModuleLoad(&mod, cubin));
  CK(cuModuleGetFunction(&fn, mod, name));
  CK(cuMemAlloc(&d_data, sizeof(float) * n * dim));
  CK(cuMemAlloc(&d_graph, sizeof(uint64_t) * (n << shift)));
  CK(cuMemAlloc(&d_query, sizeof(float) * static_cast<size_t>(nq) * dim));
  CK(cuMemAlloc(&d_result, sizeof(uint64_t) * static_cast<size_t>(nq) * pq));
  CK(cuMemAlloc(&d_measure, sizeof(Measure)));
  CK(cuMemcpyHtoD(d_data, data, sizeof(float) * n * dim));
  CK(cuMemcpyHtoD(d_graph, graph, sizeof(uint64_t) * (n << shift)));
  CK(cuMemcpyHtoD(d_query, queries, sizeof(float) * static_cast<size_t>(nq) * dim));
  CK(cuMemsetD8(d_measure, 0, sizeof(Measure)));
  CK(cuEventCreate(&e0, CU_EVENT_DEFAULT));
  CK(cuEventCreate(&e1, CU_EVENT_DEFAULT));
  for (int r = 0; r < repeats; ++r) {
    int num_query = nq, voff = shift;
    void *args_m[] = {&d_data, &d_query, &d_result, &d_graph, &num_query, &voff, &d_measure};
    CK(cuEventRecord(e0, nullptr));
    CK(cuLaunchKernel(fn, static_cast<unsigned>(nq), 1, 1, 32, 1, 1, 0, nullptr, args_m, nullptr));
    CK(cuEventRecord(e1, nullptr));
    CK(cuEventSynchronize(e1));
    float ms = 0;
    CK(cuEventElapsedTime(&ms, e0, e1));
    if (kernel_ms) kernel_ms[r] = ms;
  }
  CK(cuMemcpyDtoH(out, d_result, sizeof(uint64_t) * static_cast<size_t>(nq) * pq));
done:
  if (e0) cuEventDestroy(e0);
  if (e1) cuEventDestroy(e1);
  if (d_data) cuMemFree(d_data);
  if (d_graph) cuMemFree(d_graph);
  if (d_query) cuMemFree(d_query);
  if (d_result) cuMemFree(d_result);
  if (d_measure) cuMemFree(d_measure);
  if (mod) cuModuleUnload(mod);
  if (ctx) {
    cuCtxPopCurrent(nullptr);
    cuDevicePrimaryCtxRelease(dev);
  }
  return rc;
}
