// Batch forward pass of the closure MLP on the 5th-generation tensor cores
// (tcgen05.mma, accumulators in tensor memory).
//
// A block of four warps evaluates 128 samples per tile, one sample per
// thread row: the BF16 inputs and weights sit in shared memory in the
// canonical K-major layout without swizzle (8 x 16-byte core matrices), one
// elected thread issues the layer's MMAs (M = 128, K = 16 per instruction,
// N = 64 / 64 / 16), their completion arrives on an mbarrier, and each warp
// reads its 32 rows of the FP32 accumulator with tcgen05.ld, adds the bias,
// applies SiLU, rounds to BF16 and writes the next layer's operand.  The
// arithmetic per element is that of the warp-level path (lbm_mlp.cuh); only
// the order of the FP32 accumulation inside a layer may differ.
//
// Tensor memory: 64 columns per block, allocated by warp 0 at the start and
// freed at the end; the three layers' accumulators reuse them (every thread
// has read a layer's columns before the barrier that precedes the next
// layer's MMA).  Every mbarrier wait is bounded in time; a block whose
// wait gives up leaves after all its threads agree (no partial barrier) and
// counts the timeout.
#pragma once

#include "lbm_common.cuh"
#include "lbm_mlp.cuh"
#include "lbm_tc.cuh"

namespace lbm_mlp_tc {

using namespace lbm_mlp;
using namespace lbm_tc;

constexpr int kRows = 128;         // samples per tile (MMA M)
constexpr int kThreads = 128;      // one thread per sample row
constexpr uint32_t kTmemCols = 64;
constexpr int kN3 = 16;            // layer-3 outputs padded to the MMA's smallest N for M = 128

// waits that gave up (0 in a healthy run), read by lbm_mlp_tc_timeouts
__device__ unsigned int mlp_tc_timeouts;

struct Smem {
  __nv_bfloat16 w1[H * IN];   // [64][16]  layer-1 B operand (out x in)
  __nv_bfloat16 w2[H * H];    // [64][64]
  __nv_bfloat16 w3[kN3 * H];  // [16][64]  (rows 8..15 zero)
  __nv_bfloat16 x[kRows * IN];
  __nv_bfloat16 h[kRows * H];  // hidden activations of layer 1, then of layer 2
  float b1[H], b2[H], b3[OUT];
  uint64_t bar;
  uint32_t tmem_base;
};

__global__ void __launch_bounds__(kThreads) k_mlp_forward_tc(const __nv_bfloat16* __restrict__ x, int n,
                                                             const float* __restrict__ params, float* __restrict__ y) {
  __shared__ __align__(128) Smem sm;
  const int tid = threadIdx.x, warp = tid >> 5;
  unsigned char* w1b = reinterpret_cast<unsigned char*>(sm.w1);
  unsigned char* w2b = reinterpret_cast<unsigned char*>(sm.w2);
  unsigned char* w3b = reinterpret_cast<unsigned char*>(sm.w3);
  unsigned char* xb = reinterpret_cast<unsigned char*>(sm.x);
  unsigned char* hb = reinterpret_cast<unsigned char*>(sm.h);
  // weights: the BF16 rounding of the FP32 master block (as lbm_mlp_sync_weights)
  stage_bf16(w1b, params + PW1, H, H, IN, tid, kThreads);
  stage_bf16(w2b, params + PW2, H, H, H, tid, kThreads);
  stage_bf16(w3b, params + PW3, kN3, OUT, H, tid, kThreads);
  for (int i = tid; i < H; i += kThreads) {
    sm.b1[i] = params[PB1 + i];
    sm.b2[i] = params[PB2 + i];
  }
  for (int i = tid; i < OUT; i += kThreads) sm.b3[i] = params[PB3 + i];
  if (tid == 0) {
    lbm::mbar_init(&sm.bar, 1);
    lbm::mbar_init_fence();
  }
  if (warp == 0) tmem_alloc(&sm.tmem_base, kTmemCols);
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tmem = sm.tmem_base;
  const uint32_t lane_base = (uint32_t)(warp * 32) << 16;  // this warp's 32 accumulator rows
  const uint32_t xa = lbm::smem_addr(sm.x), ha = lbm::smem_addr(sm.h);
  const uint32_t w1a = lbm::smem_addr(sm.w1), w2a = lbm::smem_addr(sm.w2), w3a = lbm::smem_addr(sm.w3);
  uint32_t phase = 0;
  bool ok = true;
  const int tiles = (n + kRows - 1) / kRows;
  for (int tile = blockIdx.x; tile < tiles && ok; tile += gridDim.x) {
    const int row = tile * kRows + tid;
    // inputs of this thread's sample (zero past the end)
    {
      uint4 lo = make_uint4(0, 0, 0, 0), hi = lo;
      if (row < n) {
        lo = *reinterpret_cast<const uint4*>(x + (size_t)row * IN);
        hi = *reinterpret_cast<const uint4*>(x + (size_t)row * IN + 8);
      }
      *reinterpret_cast<uint4*>(xb + core_offset(tid, 0, IN)) = lo;
      *reinterpret_cast<uint4*>(xb + core_offset(tid, 8, IN)) = hi;
    }
    fence_async_smem();
    fence_before_sync();
    __syncthreads();
    // layer 1: D[0:64) = X (128 x 16) W1^T
    if (tid == 0) {
      fence_after_sync();
      mma_bf16(tmem, smem_desc(xa, 128, (IN / 8) * 128), smem_desc(w1a, 128, (IN / 8) * 128), instr_desc(kRows, H),
               0);
      mma_commit(&sm.bar);
    }
    if (!(ok = wait_mma(&sm.bar, phase))) break;
    fence_after_sync();
    epilogue_bf16<H>(tmem + lane_base, sm.b1, hb, tid, Silu());
    fence_async_smem();
    fence_before_sync();
    __syncthreads();
    // layer 2: D[0:64) = H1 (128 x 64) W2^T, four K = 16 steps
    if (tid == 0) {
      fence_after_sync();
#pragma unroll
      for (int kc = 0; kc < H / 16; ++kc)
        mma_bf16(tmem, smem_desc(ha + kc * 256, 128, (H / 8) * 128), smem_desc(w2a + kc * 256, 128, (H / 8) * 128),
                 instr_desc(kRows, H), kc > 0);
      mma_commit(&sm.bar);
    }
    if (!(ok = wait_mma(&sm.bar, phase))) break;
    fence_after_sync();
    epilogue_bf16<H>(tmem + lane_base, sm.b2, hb, tid, Silu());
    fence_async_smem();
    fence_before_sync();
    __syncthreads();
    // layer 3: D[0:16) = H2 (128 x 64) W3^T (outputs 8..15 are zero rows of W3)
    if (tid == 0) {
      fence_after_sync();
#pragma unroll
      for (int kc = 0; kc < H / 16; ++kc)
        mma_bf16(tmem, smem_desc(ha + kc * 256, 128, (H / 8) * 128), smem_desc(w3a + kc * 256, 128, (H / 8) * 128),
                 instr_desc(kRows, kN3), kc > 0);
      mma_commit(&sm.bar);
    }
    if (!(ok = wait_mma(&sm.bar, phase))) break;
    fence_after_sync();
    {
      float v[16];
      tmem_ld16(tmem + lane_base, v);
      if (row < n) {
#pragma unroll
        for (int j = 0; j < OUT; ++j) y[(size_t)row * OUT + j] = v[j] + sm.b3[j];
      }
    }
    fence_before_sync();
    __syncthreads();
  }
  if (!ok && tid == 0) atomicAdd(&mlp_tc_timeouts, 1u);
  fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    fence_after_sync();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
  }
}

}  // namespace lbm_mlp_tc
