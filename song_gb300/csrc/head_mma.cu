// head_mma.cu -- head phase of the two-level entry choice on the tensor cores.
//
// The head phase picks, for every query, the `probes` coarse entries nearest
// by the search kernel's own distance (warp_astar_accelerator.h:237-287
// arithmetic), ties to the smaller position.  It is a dense nq x n_heads x dim
// contraction, so it runs in two steps whose result is the same as an exact
// scan's:
//
//  1. head_scores_kernel: s~ = q . x for all pairs, a TF32 tcgen05.mma GEMM
//     (FP32 accumulators in tensor memory).  128 x 128 tiles; the operands are
//     staged by TMA (cp.async.bulk.tensor.2d) as 128-byte-swizzled K-major
//     slabs of 32 floats, two slab pairs in flight; one thread issues the
//     copies and the MMAs.  In the epilogue each thread reads its query's row of
//     the accumulators (tcgen05.ld) and turns every score into an interval
//     [lo, hi] that provably holds the exact search distance (the TF32 error
//     bound below); it writes the lower bounds and the tile's `probes`
//     smallest upper bounds.
//  2. head_select_kernel: a warp per query takes U = the probes-th smallest
//     upper bound and re-scores every head with lo <= U -- a superset of the
//     exact answer -- with the exact FP32 arithmetic; more than HM_CAP such
//     heads, and it scores all heads.
//
// Error bound.  TF32 keeps 10 mantissa bits: each operand read by the MMA is
// within 2^-10 (relative) of its FP32 value even when it is truncated, so a
// product is within 2^-9 of the exact one and |s~ - q.x| <= 2^-9 *
// sum |q_i x_i| <= 2^-9 * |q||x| (Cauchy-Schwarz), plus the accumulation:
// 8-term block sums added into an FP32 accumulator, under 2^-20 * dim/8 of
// the same sum even with truncating adders (2^-16 at dim 128).  The
// intervals use (2^-9 + 2^-14) * |q||x| and widen every FP32 step of the
// distance formula by 2^-15 of its magnitude, far above its rounding.  A GPU
// test measures the actual error against the bound.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>

#include "device_common.cuh"
#include "internal.h"
#include "song_gb300.h"

namespace song {

namespace {

constexpr int HM_B = 128;     // queries (M) and heads (N) per tile
constexpr int HM_K = 32;      // floats per K slab: one 128-byte swizzle row
constexpr int HM_STAGES = 2;  // slab pairs in flight (67 KB of shared memory: three blocks per SM overlap
                              // one another's copies, products and epilogues)
constexpr uint32_t HM_SLAB = HM_B * HM_K * 4;  // 16 KB
// slabs, then barriers (128 B), then the tile's head norms (2 x 128 floats)
constexpr size_t HM_SMEM = 1024 + static_cast<size_t>(HM_STAGES) * 2 * HM_SLAB + 128 + 2 * HM_B * 4;
constexpr int HM_CAP = 256;   // heads re-scored from the shortlist; beyond it the warp scores all
constexpr int HM_SEL_WARPS = 8;
constexpr float HM_REL = 0x1.08p-9f;  // dot-product error bound, relative to |q||x| (2^-9 + 2^-14)
constexpr float HM_SLACK = 0x1p-15f; // widening of each FP32 step of the distance formula

// ---- inline PTX: TMA, tcgen05 ---------------------------------------------

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int x, int y, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
      "[%4];" ::"r"(smem_addr(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_addr(bar))
      : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Whole warp: allocate / free `cols` tensor-memory columns (a power of two >= 32).
__device__ __forceinline__ void tmem_alloc(uint32_t *slot, uint32_t cols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(slot)),
               "r"(cols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t cols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(cols) : "memory");
}

// D[tmem] (+)= A[smem] * B[smem]^T, one thread.
__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// `bar` completes once every MMA this thread issued before has completed.
__device__ __forceinline__ void mma_commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
               : "memory");
}

// Whole warp: lane l gets columns col .. col+31 of tensor-memory lane
// (warp's quarter * 32 + l), the address carrying the quarter in bits 16+.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&v)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
        "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
        "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),
        "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// Shared-memory matrix descriptor of a K-major operand slab written by TMA
// with 128-byte swizzling: rows of 128 bytes, 8-row groups 1024 bytes apart
// (stride byte offset), descriptor version 1, swizzle mode 2 (128 B).  The
// slab starts on a 1024-byte boundary; `addr` may sit 32*k bytes past it to
// select the k-th 8-float step of K (the swizzle acts on absolute address
// bits, as the TMA wrote them).
__device__ __forceinline__ uint64_t sw128_desc(uint32_t addr) {
  return static_cast<uint64_t>((addr & 0x3ffffu) >> 4) | (1ull << 16) | (static_cast<uint64_t>(1024 >> 4) << 32) |
         (1ull << 46) | (2ull << 61);
}

// Instruction descriptor, kind::tf32: D FP32 (bits 4-5 = 1), A and B TF32
// (bits 7-9, 10-12 = 2), both K-major (bits 15, 16 = 0), N >> 3 at bit 17,
// M >> 4 at bit 24.
constexpr uint32_t tf32_idesc(int m, int n) {
  return (1u << 4) | (2u << 7) | (2u << 10) | (static_cast<uint32_t>(n >> 3) << 17) |
         (static_cast<uint32_t>(m >> 4) << 24);
}

// [lo, hi] around the search distance of a query (squared norm qn2, norm qn)
// to a head (squared norm xn2, norm xn) from the approximate dot product s.
template <int METRIC>
__device__ __forceinline__ void head_interval(float s, float qn2, float qn, float xn2, float xn, float &lo,
                                              float &hi) {
  const float e = HM_REL * qn * xn + 1e-30f;
  if (METRIC == SONG_METRIC_L2) {
    const float d = qn2 + xn2 - 2.0f * s;
    const float eps = 2.0f * e + HM_SLACK * (qn2 + xn2 + 2.0f * fabsf(s));
    lo = d - eps;
    hi = d + eps;
  } else if (METRIC == SONG_METRIC_IP) {
    const float eps = e + HM_SLACK * qn * xn;
    lo = -s - eps;
    hi = -s + eps;
  } else {
    // d = -t|t| / len, decreasing in t; a head with a (near) zero norm is
    // always re-scored
    if (!(xn2 > 1e-30f)) {
      lo = -__int_as_float(0x7f800000);
      hi = __int_as_float(0x7f800000);
      return;
    }
    const float et = e + HM_SLACK * qn * xn;
    const float tp = s + et, tm = s - et;
    const float a = -tp * fabsf(tp) / xn2, b = -tm * fabsf(tm) / xn2;
    lo = a - HM_SLACK * fabsf(a) - 1e-30f;
    hi = b + HM_SLACK * fabsf(b) + 1e-30f;
  }
}

// Lane l's sorted list of the N smallest (value, id) pairs seen, static indexing.
template <int N>
__device__ __forceinline__ void best_insert(float (&bd)[N], uint32_t (&bi)[N], float d, uint32_t id) {
  if (!(d < bd[N - 1] || (d == bd[N - 1] && id < bi[N - 1]))) return;
#pragma unroll
  for (int m = N - 1; m > 0; --m) {
    const bool shift = d < bd[m - 1] || (d == bd[m - 1] && id < bi[m - 1]);
    const bool here = !shift && (d < bd[m] || (d == bd[m] && id < bi[m]));
    if (shift) {
      bd[m] = bd[m - 1];
      bi[m] = bi[m - 1];
    } else if (here) {
      bd[m] = d;
      bi[m] = id;
    }
  }
  if (d < bd[0] || (d == bd[0] && id < bi[0])) {
    bd[0] = d;
    bi[0] = id;
  }
}

// Warp-wide smallest (value, id) over the lanes' list heads at position h
// (per lane); the owning lane moves past it.
template <int N>
__device__ __forceinline__ void warp_take(const float (&bd)[N], const uint32_t (&bi)[N], int &h, float &wd,
                                          uint32_t &wid) {
  float d = __int_as_float(0x7f800000);
  uint32_t id = 0xffffffffu;
#pragma unroll
  for (int m = 0; m < N; ++m)
    if (m == h) {
      d = bd[m];
      id = bi[m];
    }
  wd = d;
  wid = id;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float od = __shfl_xor_sync(FULL, wd, o);
    const uint32_t oid = __shfl_xor_sync(FULL, wid, o);
    if (od < wd || (od == wd && oid < wid)) {
      wd = od;
      wid = oid;
    }
  }
  if (id == wid && d == wd && id != 0xffffffffu) ++h;
}

// Exact search distance (lane-strided FMA chain over dims, xor butterfly) of
// the query to R head rows at once (R = 8 or 32): row r is rows + idx(r) *
// dpad; lane l returns row l / (32 / R)'s distance.  Products taken two rows
// at a time through the paired FP32 instructions (the scalar roundings, in
// the scalar order); the R rows meet in one transposed butterfly.
template <int METRIC, int R, class Idx>
__device__ __forceinline__ float rows_distance(const float *qv, int dim, const float *rows, int dpad, Idx idx,
                                               int lane) {
  constexpr bool COS = METRIC == SONG_METRIC_COS;
  constexpr int P = R / 2;
  uint64_t acc[P], ln[P];
#pragma unroll
  for (int p = 0; p < P; ++p) acc[p] = ln[p] = 0ull;
  for (int j = lane; j < dim; j += 32) {
    const float qj = qv[j];
    const uint64_t qq = f2_pack(qj, qj);
#pragma unroll
    for (int p = 0; p < P; ++p) {
      const float x0 = __ldg(rows + static_cast<size_t>(idx(2 * p)) * dpad + j);
      const float x1 = __ldg(rows + static_cast<size_t>(idx(2 * p + 1)) * dpad + j);
      const uint64_t xx = f2_pack(x0, x1);
      if (METRIC == SONG_METRIC_L2) {
        const uint64_t df = f2_sub(qq, xx);
        acc[p] = f2_fma(df, df, acc[p]);
      } else {
        acc[p] = f2_fma(qq, xx, acc[p]);
        if (COS) ln[p] = f2_fma(xx, xx, ln[p]);
      }
    }
  }
  float v[R];
#pragma unroll
  for (int p = 0; p < P; ++p) f2_unpack(acc[p], v[2 * p], v[2 * p + 1]);
  const float t = butterfly_rows<R>(v, lane);
  if (METRIC == SONG_METRIC_L2) return t;
  if (METRIC == SONG_METRIC_IP) return -t;
  float lv[R];
#pragma unroll
  for (int p = 0; p < P; ++p) f2_unpack(ln[p], lv[2 * p], lv[2 * p + 1]);
  const float len = butterfly_rows<R>(lv, lane);
  if (len != 0.0f) {
    const float sign = t < 0.0f ? 1.0f : -1.0f;
    return __fdiv_rn(__fmul_rn(__fmul_rn(sign, t), t), len);
  }
  return 0.0f;
}

// ---- step 1: tensor-core scores, intervals in the epilogue ------------------

struct HeadScoreArgs {
  int rows;      // queries of this launch: q_row0 .. q_row0 + rows - 1
  int q_row0;
  int n_heads;
  int kchunks;   // ceil(dim / HM_K)
  float *out;    // OUT_RAW: rows x ld raw scores
  uint16_t *lo16;  // OUT_BOUNDS: rows x ld lower bounds, BF16 rounded down (ld a multiple of 8)
  int ld;
  float *tile_hi;       // OUT_BOUNDS: rows x tiles x NP smallest upper bounds of each head tile
  const float *q_n2;    // squared norms of all queries (OUT_BOUNDS)
  const float *head_n2; // squared norms of the heads (OUT_BOUNDS)
  int32_t *error;
  uint32_t wait_limit;
  uint32_t extra_tx;  // test hook: bytes every copy batch expects beyond its slabs (0 in use)
};

constexpr int OUT_RAW = 0, OUT_BOUNDS = 1;

// One 128 x 128 tile (blockIdx.x: queries, blockIdx.y: heads).  OUT_RAW
// writes s~[q][h]; OUT_BOUNDS writes the lower bound of every head's search
// distance (+inf past the last head) in BF16 rounded toward -inf -- still a
// lower bound, in half the bytes, so that a whole batch's bounds stay in L2
// -- and, per query, the NP smallest upper bounds of the tile.
template <int METRIC, int NP, int OUT>
__global__ void __launch_bounds__(128, 1)
    head_scores_kernel(const __grid_constant__ CUtensorMap tq, const __grid_constant__ CUtensorMap th,
                       const HeadScoreArgs a) {
  extern __shared__ uint8_t hm_raw[];
  uint8_t *sm = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(hm_raw) + 1023) & ~uintptr_t(1023));
  uint64_t *full = reinterpret_cast<uint64_t *>(sm + static_cast<size_t>(HM_STAGES) * 2 * HM_SLAB);
  uint64_t *empty = full + HM_STAGES;
  uint64_t *done = empty + HM_STAGES;
  uint32_t *tslot = reinterpret_cast<uint32_t *>(done + 1);
  int32_t *failed = reinterpret_cast<int32_t *>(tslot + 1);
  float *hx2 = reinterpret_cast<float *>(sm + static_cast<size_t>(HM_STAGES) * 2 * HM_SLAB + 128);  // [HM_B]
  float *hx = hx2 + HM_B;                                                                           // [HM_B]
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.x * HM_B, n0 = blockIdx.y * HM_B;
  if (OUT == OUT_BOUNDS) {
    const int h = n0 + tid;
    const float x2 = h < a.n_heads ? a.head_n2[h] : 0.0f;
    hx2[tid] = x2;
    hx[tid] = sqrtf(x2);
  }
  if (tid == 0) {
    for (int s = 0; s < HM_STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(done, 1);
    *failed = 0;
    fence_mbar_init();
  }
  if (warp == 0) tmem_alloc(tslot, HM_B);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;

  if (tid == 0) {
    constexpr uint32_t idesc = tf32_idesc(HM_B, HM_B);
    int issued = 0;
    auto issue = [&](int c) {
      const int s = c % HM_STAGES;
      uint8_t *A = sm + static_cast<size_t>(s) * 2 * HM_SLAB;
      mbar_arrive_expect_tx(&full[s], 2 * HM_SLAB + a.extra_tx);
      tma_load_2d(A, &tq, c * HM_K, a.q_row0 + m0, &full[s]);
      tma_load_2d(A + HM_SLAB, &th, c * HM_K, n0, &full[s]);
    };
    for (; issued < min(HM_STAGES, a.kchunks); ++issued) issue(issued);
    bool ok = true;
    int c = 0;
    for (; c < a.kchunks; ++c) {
      const int s = c % HM_STAGES;
      const uint32_t ph = static_cast<uint32_t>(c / HM_STAGES) & 1u;
      if (!mbar_wait(&full[s], ph, a.wait_limit)) {
        ok = false;
        break;
      }
      tc_fence_after();
      const uint32_t A = smem_addr(sm + static_cast<size_t>(s) * 2 * HM_SLAB), B = A + HM_SLAB;
#pragma unroll
      for (int k = 0; k < HM_K / 8; ++k)
        mma_tf32(tmem, sw128_desc(A + 32u * k), sw128_desc(B + 32u * k), idesc, (c | k) != 0 ? 1u : 0u);
      mma_commit(&empty[s]);
      if (issued < a.kchunks) {  // chunk c + HM_STAGES reuses stage s once the MMAs above have read it
        if (!mbar_wait(&empty[s], ph, a.wait_limit)) {
          ok = false;
          ++c;
          break;
        }
        issue(issued++);
      }
    }
    mma_commit(done);
    if (!ok) {
      // copies of chunks c .. issued-1 may still be landing in this block's
      // shared memory: wait for them (bounded) before the block leaves
      for (int r = c; r < issued; ++r)
        mbar_wait(&full[r % HM_STAGES], static_cast<uint32_t>(r / HM_STAGES) & 1u, a.wait_limit);
      *failed = 1;
    }
  }
  __syncthreads();
  const bool mma_done = mbar_wait(done, 0, a.wait_limit);
  // one decision for the whole block: the tensor-memory loads below are
  // warp-collective
  const bool all_ok = __syncthreads_and(mma_done && !*failed) != 0;
  tc_fence_after();
  if (!all_ok) {
    if (tid == 0) atomicOr(a.error, 1);
  } else {
    const int row = m0 + 32 * warp + lane;  // this thread's query (tensor-memory lane)
    const bool live = row < a.rows;
    float qn2 = 0.0f, qn = 0.0f;
    if (OUT == OUT_BOUNDS && live) {
      qn2 = a.q_n2[a.q_row0 + row];
      qn = sqrtf(qn2);
    }
    float best[NP];
#pragma unroll
    for (int m = 0; m < NP; ++m) best[m] = __int_as_float(0x7f800000);
#pragma unroll 1
    for (int j = 0; j < HM_B / 32; ++j) {
      uint32_t v[32];
      tmem_ld32(tmem + (static_cast<uint32_t>(32 * warp) << 16) + static_cast<uint32_t>(32 * j), v);
      const int col0 = n0 + 32 * j;
      float o[32];
#pragma unroll
      for (int i = 0; i < 32; ++i) {
        const float s = __uint_as_float(v[i]);
        if (OUT == OUT_RAW) {
          o[i] = s;
        } else {
          float lo = __int_as_float(0x7f800000), hi = lo;
          if (col0 + i < a.n_heads) head_interval<METRIC>(s, qn2, qn, hx2[32 * j + i], hx[32 * j + i], lo, hi);
          o[i] = lo;
          // the tile's NP smallest upper bounds (values only)
          if (hi < best[NP - 1]) {
            float x = hi;
#pragma unroll
            for (int m = 0; m < NP; ++m) {
              const float lo_v = fminf(best[m], x);
              x = fmaxf(best[m], x);
              best[m] = lo_v;
            }
          }
        }
      }
      if (OUT == OUT_RAW && live && col0 < a.ld) {
        float *dst = a.out + static_cast<size_t>(row) * a.ld + col0;
        if (col0 + 32 <= a.ld) {
#pragma unroll
          for (int i = 0; i < 32; i += 4) *reinterpret_cast<float4 *>(dst + i) = make_float4(o[i], o[i + 1], o[i + 2], o[i + 3]);
        } else {
#pragma unroll
          for (int i = 0; i < 32; ++i)
            if (col0 + i < a.ld) dst[i] = o[i];
        }
      }
      if (OUT == OUT_BOUNDS && live && col0 < a.ld) {
        uint16_t b[32];
#pragma unroll
        for (int i = 0; i < 32; ++i) b[i] = __bfloat16_as_ushort(__float2bfloat16_rd(o[i]));
        uint16_t *dst = a.lo16 + static_cast<size_t>(row) * a.ld + col0;
        if (col0 + 32 <= a.ld) {
#pragma unroll
          for (int i = 0; i < 32; i += 8)
            *reinterpret_cast<uint4 *>(dst + i) =
                make_uint4(b[i] | (static_cast<uint32_t>(b[i + 1]) << 16), b[i + 2] | (static_cast<uint32_t>(b[i + 3]) << 16),
                           b[i + 4] | (static_cast<uint32_t>(b[i + 5]) << 16), b[i + 6] | (static_cast<uint32_t>(b[i + 7]) << 16));
        } else {
#pragma unroll
          for (int i = 0; i < 32; ++i)
            if (col0 + i < a.ld) dst[i] = b[i];
        }
      }
    }
    if (OUT == OUT_BOUNDS && live) {
      float *hb = a.tile_hi + (static_cast<size_t>(row) * gridDim.y + blockIdx.y) * NP;
#pragma unroll
      for (int m = 0; m < NP; ++m) hb[m] = best[m];
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, HM_B);
}

// ---- step 2: U, the shortlist, exact re-scoring ------------------------------

// One warp per query: probe_out[q * probes ..] = its `probes` nearest heads
// (positions), ascending by (distance, position); cl_count counts probes per
// head.  lo16: rows x ld lower bounds in BF16 (+inf past the heads); tile_hi:
// rows x tiles x NP.  stats (or null): [0] queries, [1] heads re-scored, [2]
// full scans.
template <int METRIC, int NP>
__global__ void __launch_bounds__(HM_SEL_WARPS * 32)
    head_select_kernel(const float *queries, int dim, int q_row0, int rows, const uint16_t *lo16, int ld,
                       const float *tile_hi, int tiles, const float *heads, int dpad, int n_heads, int probes,
                       uint32_t *probe_out, uint32_t *cl_count, unsigned long long *stats) {
  __shared__ uint32_t cand[HM_SEL_WARPS][HM_CAP];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int r = blockIdx.x * HM_SEL_WARPS + w;
  if (r >= rows) return;  // whole warp
  const int q = q_row0 + r;
  const float *qv = queries + static_cast<size_t>(q) * dim;

  // U = the probes-th smallest upper bound over all heads: the tiles' lists
  // hold every head's bound that can be among them
  float U;
  {
    float hb[NP];
    uint32_t hid[NP];
#pragma unroll
    for (int m = 0; m < NP; ++m) {
      hb[m] = __int_as_float(0x7f800000);
      hid[m] = 0xffffffffu;
    }
    const float *th = tile_hi + static_cast<size_t>(r) * tiles * NP;
    for (int i = lane; i < tiles * NP; i += 32) best_insert<NP>(hb, hid, th[i], static_cast<uint32_t>(i));
    int hp = 0;
    U = __int_as_float(0x7f800000);
    for (int k = 0; k < probes; ++k) {
      uint32_t wid;
      warp_take<NP>(hb, hid, hp, U, wid);
    }
  }
  // the shortlist: every head whose lower bound is <= U, four 16-byte
  // groups of eight BF16 bounds per lane in flight
  const uint4 *lo8 = reinterpret_cast<const uint4 *>(lo16 + static_cast<size_t>(r) * ld);
  const int n8 = ld / 8;
  int count = 0;
  for (int i0 = 0; i0 < n8; i0 += 32 * 4) {
    uint4 v[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int i = i0 + 32 * k + lane;
      v[k] = i < n8 ? __ldg(lo8 + i) : make_uint4(0x7f807f80u, 0x7f807f80u, 0x7f807f80u, 0x7f807f80u);  // +inf
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const uint32_t wds[4] = {v[k].x, v[k].y, v[k].z, v[k].w};
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        const uint32_t bits = (c & 1) ? (wds[c >> 1] & 0xffff0000u) : (wds[c >> 1] << 16);
        const bool f = __uint_as_float(bits) <= U;  // a BF16 value widened exactly
        const unsigned b = __ballot_sync(FULL, f);
        if (f) {
          const int pos = count + __popc(b & ((1u << lane) - 1u));
          if (pos < HM_CAP) cand[w][pos] = static_cast<uint32_t>(8 * (i0 + 32 * k + lane) + c);
        }
        count += __popc(b);
      }
    }
  }
  __syncwarp();
  // exact distances of the shortlist (or of every head)
  float bd[NP];
  uint32_t bi[NP];
#pragma unroll
  for (int m = 0; m < NP; ++m) {
    bd[m] = __int_as_float(0x7f800000);
    bi[m] = 0xffffffffu;
  }
  // (fewer candidates than probes only happens to bounds that are not
  // finite, e.g. after a timed-out score kernel: scan everything then too)
  const bool full_scan = count > HM_CAP || count < probes;
  const int total = full_scan ? n_heads : count;
  // 32 rows per pass, the last few (the common shortlist of a handful of
  // heads) 8 at a time: a pass reads every one of its rows
  for (int g = 0; g < total;) {
    const int left = total - g;
    if (left > 8) {
      const int n = min(32, left);
      float d;
      if (full_scan) {
        d = rows_distance<METRIC, 32>(qv, dim, heads, dpad, [&](int i) { return min(g + i, n_heads - 1); }, lane);
      } else {
        const uint32_t *cl = cand[w] + g;
        d = rows_distance<METRIC, 32>(qv, dim, heads, dpad, [&](int i) { return cl[min(i, n - 1)]; }, lane);
      }
      if (lane < n) best_insert<NP>(bd, bi, d, full_scan ? static_cast<uint32_t>(g + lane) : cand[w][g + lane]);
      g += n;
    } else {
      const int n = left;
      float d;
      if (full_scan) {
        d = rows_distance<METRIC, 8>(qv, dim, heads, dpad, [&](int i) { return min(g + i, n_heads - 1); }, lane);
      } else {
        const uint32_t *cl = cand[w] + g;
        d = rows_distance<METRIC, 8>(qv, dim, heads, dpad, [&](int i) { return cl[min(i, n - 1)]; }, lane);
      }
      const int row = lane >> 2;  // lane l holds row l / 4
      if ((lane & 3) == 0 && row < n)
        best_insert<NP>(bd, bi, d, full_scan ? static_cast<uint32_t>(g + row) : cand[w][g + row]);
      g += n;
    }
  }
  int hp = 0;
  for (int k = 0; k < probes; ++k) {
    float wd;
    uint32_t wid;
    warp_take<NP>(bd, bi, hp, wd, wid);
    if (wid >= static_cast<uint32_t>(n_heads)) wid = 0;  // no finite distance (a query that is not finite)
    if (lane == 0) {
      probe_out[static_cast<size_t>(q) * probes + k] = wid;
      atomicAdd(cl_count + wid, 1u);
    }
  }
  if (stats && lane == 0) {
    atomicAdd(stats + 0, 1ull);
    atomicAdd(stats + 1, static_cast<unsigned long long>(total));
    if (full_scan) atomicAdd(stats + 2, 1ull);
  }
}

// Squared norm of each of n rows (stride floats apart; any order: the
// intervals carry slack), a warp per row.
__global__ void row_norms_kernel(const float *rows, int n, int dim, int stride, float *out) {
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (w >= n) return;
  const float *x = rows + static_cast<size_t>(w) * stride;
  float s = 0.0f;
  for (int j = lane; j < dim; j += 32) s = fmaf(x[j], x[j], s);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(FULL, s, o);
  if (lane == 0) out[w] = s;
}

using EncodeTiled = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                 const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encode_fn() {
  static EncodeTiled fn = []() -> EncodeTiled {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      return nullptr;
    return reinterpret_cast<EncodeTiled>(p);
  }();
  return fn;
}

// A 2-D FP32 tensor map of `rows` rows of `dim` floats, `stride` bytes apart,
// read in boxes of 32 floats x 128 rows with 128-byte swizzling; reads past
// the edges return zeros.
bool encode_rows(CUtensorMap *map, const float *base, int dim, uint64_t rows, uint64_t stride) {
  EncodeTiled fn = encode_fn();
  if (!fn || (reinterpret_cast<uintptr_t>(base) & 15u) || (stride & 15u) || rows == 0) return false;
  const cuuint64_t gdim[2] = {static_cast<cuuint64_t>(dim), rows};
  const cuuint64_t gstride[1] = {stride};
  const cuuint32_t box[2] = {HM_K, HM_B};
  const cuuint32_t estr[2] = {1, 1};
  return fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float *>(base), gdim, gstride, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int METRIC, int NP>
cudaError_t launch_chunk(const CUtensorMap &tq, const CUtensorMap &th, HeadScoreArgs a, const float *queries,
                         song_index *ix, int np, uint32_t *probe_out, cudaStream_t s) {
  auto kern = head_scores_kernel<METRIC, NP, OUT_BOUNDS>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(HM_SMEM));
  if (e != cudaSuccess) return e;
  const int tiles = (a.n_heads + HM_B - 1) / HM_B;
  kern<<<dim3((a.rows + HM_B - 1) / HM_B, tiles), 128, HM_SMEM, s>>>(tq, th, a);
  const int dpad = static_cast<int>(ix->dx.f32_row_bytes / 4);
  head_select_kernel<METRIC, NP><<<(a.rows + HM_SEL_WARPS - 1) / HM_SEL_WARPS, HM_SEL_WARPS * 32, 0, s>>>(
      queries, ix->dx.dim, a.q_row0, a.rows, a.lo16, a.ld, a.tile_hi, tiles, ix->d_coarse_rows, dpad, ix->n_coarse,
      np, probe_out, ix->d_cl_count, ix->head_stats_on ? ix->d_head_stats : nullptr);
  return cudaGetLastError();
}

}  // namespace

static_assert(sizeof(CUtensorMap) == sizeof(song_index::head_map), "tensor map storage");

bool heads_mma_prepare(song_index *ix, int coarse) {
  ix->heads_mma = false;
  const int dim = ix->dx.dim, dpad = static_cast<int>(ix->dx.f32_row_bytes / 4);
  if (coarse <= 0 || dim % 4 != 0) return false;
  CUtensorMap map;
  if (!encode_rows(&map, ix->d_coarse_rows, dim, static_cast<uint64_t>(coarse), static_cast<uint64_t>(dpad) * 4u))
    return false;
  cudaFree(ix->d_head_n2);
  ix->d_head_n2 = nullptr;
  if (song::dev_malloc(&ix->d_head_n2, sizeof(float) * coarse) != cudaSuccess) return false;
  row_norms_kernel<<<(coarse + 7) / 8, 256, 0, ix->stream>>>(ix->d_coarse_rows, coarse, dim, dpad, ix->d_head_n2);
  if (cudaGetLastError() != cudaSuccess) return false;
  std::memcpy(ix->head_map, &map, sizeof map);
  ix->heads_mma = true;
  return true;
}

bool heads_mma_usable(const song_index *ix, const float *queries, int np) {
  return ix->heads_mma && ix->heads_mma_enabled && np <= 8 && (reinterpret_cast<uintptr_t>(queries) & 15u) == 0;
}

cudaError_t launch_heads_mma(song_index *ix, const float *queries, int nq, int np, uint32_t *probe_out,
                             cudaStream_t s) {
  const int dim = ix->dx.dim, coarse = ix->n_coarse;
  CUtensorMap tq, th;
  if (!encode_rows(&tq, queries, dim, static_cast<uint64_t>(nq), static_cast<uint64_t>(dim) * 4u))
    return cudaErrorInvalidValue;
  std::memcpy(&th, ix->head_map, sizeof th);
  const int NPsel = np <= 1 ? 1 : (np <= 2 ? 2 : (np <= 4 ? 4 : 8));
  const int tiles = (coarse + HM_B - 1) / HM_B;
  // BF16 bounds of up to `chunk` queries at a time: at most 96 MB, which
  // stays in L2 between the two kernels (the whole batch at the headline)
  const int ld = (coarse + 7) & ~7;
  const int chunk = std::max(HM_B, std::min((nq + HM_B - 1) / HM_B * HM_B,
                                            static_cast<int>((96u << 20) / (2u * ld)) / HM_B * HM_B));
  // work area (256-byte aligned parts): query norms, bounds, tile lists
  auto up256 = [](size_t b) { return (b + 255) & ~size_t(255); };
  const size_t off_lo = up256(sizeof(float) * static_cast<size_t>(nq));
  const size_t off_hi = off_lo + up256(sizeof(uint16_t) * static_cast<size_t>(chunk) * ld);
  const size_t need = (off_hi + sizeof(float) * static_cast<size_t>(chunk) * tiles * 8 + 3) / 4;  // floats
  if (need > ix->cap_head_scores) {
    cudaFree(ix->d_head_scores);
    ix->d_head_scores = nullptr;
    ix->cap_head_scores = 0;
    cudaError_t e = song::dev_malloc(&ix->d_head_scores, sizeof(float) * need);
    if (e != cudaSuccess) return e;
    ix->cap_head_scores = need;
  }
  unsigned char *work = reinterpret_cast<unsigned char *>(ix->d_head_scores);
  float *q_n2 = ix->d_head_scores;
  uint16_t *bounds = reinterpret_cast<uint16_t *>(work + off_lo);
  float *tile_hi = reinterpret_cast<float *>(work + off_hi);
  row_norms_kernel<<<(nq + 7) / 8, 256, 0, s>>>(queries, nq, dim, dim, q_n2);
  for (int q0 = 0; q0 < nq; q0 += chunk) {
    HeadScoreArgs a;
    a.rows = std::min(chunk, nq - q0);
    a.q_row0 = q0;
    a.n_heads = coarse;
    a.kchunks = (dim + HM_K - 1) / HM_K;
    a.out = nullptr;
    a.lo16 = bounds;
    a.ld = ld;
    a.tile_hi = tile_hi;
    a.q_n2 = q_n2;
    a.head_n2 = ix->d_head_n2;
    a.error = ix->d_error;
    a.wait_limit = ix->wait_limit;
    a.extra_tx = ix->extra_tx;
    cudaError_t e = cudaSuccess;
#define SONG_CHUNK(M)                                                                     \
  switch (NPsel) {                                                                        \
    case 1: e = launch_chunk<M, 1>(tq, th, a, queries, ix, np, probe_out, s); break;      \
    case 2: e = launch_chunk<M, 2>(tq, th, a, queries, ix, np, probe_out, s); break;      \
    case 4: e = launch_chunk<M, 4>(tq, th, a, queries, ix, np, probe_out, s); break;      \
    default: e = launch_chunk<M, 8>(tq, th, a, queries, ix, np, probe_out, s); break;     \
  }
    switch (ix->dx.metric) {
      case SONG_METRIC_L2: SONG_CHUNK(SONG_METRIC_L2); break;
      case SONG_METRIC_IP: SONG_CHUNK(SONG_METRIC_IP); break;
      default: SONG_CHUNK(SONG_METRIC_COS); break;
    }
#undef SONG_CHUNK
    if (e != cudaSuccess) return e;
  }
  return cudaGetLastError();
}

// Approximate scores only (tests): scores[q * ld + h] for all queries, or
// cudaErrorInvalidValue when the tensor path is not available for this index.
cudaError_t launch_head_scores_only(song_index *ix, const float *queries, int nq, float *scores, int ld,
                                    cudaStream_t s) {
  const int dim = ix->dx.dim;
  CUtensorMap tq, th;
  if (!ix->heads_mma || !encode_rows(&tq, queries, dim, static_cast<uint64_t>(nq), static_cast<uint64_t>(dim) * 4u))
    return cudaErrorInvalidValue;
  std::memcpy(&th, ix->head_map, sizeof th);
  auto kern = head_scores_kernel<SONG_METRIC_L2, 1, OUT_RAW>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(HM_SMEM));
  if (e != cudaSuccess) return e;
  HeadScoreArgs a;
  std::memset(&a, 0, sizeof a);
  a.rows = nq;
  a.q_row0 = 0;
  a.n_heads = ix->n_coarse;
  a.kchunks = (dim + HM_K - 1) / HM_K;
  a.out = scores;
  a.lo16 = nullptr;
  a.ld = ld;
  a.error = ix->d_error;
  a.wait_limit = ix->wait_limit;
  a.extra_tx = ix->extra_tx;
  kern<<<dim3((nq + HM_B - 1) / HM_B, (ix->n_coarse + HM_B - 1) / HM_B), 128, HM_SMEM, s>>>(tq, th, a);
  return cudaGetLastError();
}

}  // namespace song
