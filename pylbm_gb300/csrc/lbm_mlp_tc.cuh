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

// ---------------------------------------------------------------------------
// One training step on the 5th-generation tensor cores.  A block takes
// 128-sample tiles, one sample per thread, and for each tile runs in shared
// and tensor memory only:
//   forward      Z1 = X W1^T, H1 = silu(Z1 + b1), Z2 = H1 W2^T, H2 = silu(..),
//                Y = H2 W3^T + b3 (pre-activations stay in tensor memory)
//   loss         dY = 2 (Y - T) / (6 n) on the 6 used outputs (BF16)
//   backward     dZ2 = (dY W3) silu'(Z2), dZ1 = (dZ2 W2) silu'(Z1)   (BF16)
//   gradients    [dZ1^T; dZ2^T] [X | H1 | 1] and [H2^T; ..] [dY | 1]: two
//                M = 128 MMAs per 16 samples whose diagonal blocks are dW1,
//                dW2 and the bias sums (the ones column), and dW3^T with the
//                b3 sums, accumulated in tensor memory over the block's tiles
// then adds its accumulated gradients to `grad` once.  The rounding points
// are those of k_mlp_fwd_bwd / k_mlp_wgrad (BF16 activations, gradients and
// operands, FP32 accumulation); only the accumulation order differs.
//
// Shared memory holds the tile's operands in interleaved buffers so that the
// same bytes serve the forward MMAs (K-major: sample rows, feature K) and the
// gradient MMAs (MN-major: feature rows, sample K): per 8-sample group,
//   Q: H2 (features 0-63) | dY (64-79) | ones (80-95) | zeros (96-127)
//   G: dZ1 (0-63) | dZ2 (64-127)
//   P: X (0-15) | H1 (16-79) | ones (80-95)
// in 16-byte core rows, core matrices 128 bytes apart along the features.
namespace train {
constexpr int kGroups = kRows / 8;
constexpr int kQGroup = 16 * 128, kGGroup = 16 * 128, kPGroup = 12 * 128;
constexpr int kQ = 0;
constexpr int kG = kQ + kGroups * kQGroup;
constexpr int kP = kG + kGroups * kGGroup;
constexpr int kW1 = kP + kGroups * kPGroup;  // [64][16]
constexpr int kW2 = kW1 + H * IN * 2;        // [64][64]
constexpr int kW3 = kW2 + H * H * 2;         // [16][64] (rows 8..15 zero)
constexpr int kW3T = kW3 + 16 * H * 2;       // [64][16]: W3^T, columns 8..15 zero
constexpr int kW2T = kW3T + H * 16 * 2;      // [64][64]: W2^T
constexpr int kBias = kW2T + H * H * 2;      // b1[64], b2[64], b3[8]
constexpr int kBar = kBias + (2 * H + OUT) * 4;
constexpr int kSmem = kBar + 16;
// tensor-memory columns: pre-activations, scratch accumulator, gradients
constexpr uint32_t kZ1 = 0, kZ2 = 64, kS = 128, kD1 = 256, kD2 = 384, kCols = 512;
// an MN-major operand of `cores` core matrices along MN read by the eight
// K = 16 MMAs of a tile from `start`: its last byte, and the last byte if the
// two strides were taken the other way round; both stay inside the block's
// shared memory
constexpr int mn_extent(int start, int cores, int group) { return start + 14 * group + group + cores * 128; }
constexpr int mn_extent_other(int start, int cores, int group) {
  return start + 14 * group + (cores - 1) * group + 256;
}
static_assert(mn_extent_other(kG, 16, kGGroup) <= kSmem && mn_extent(kG, 16, kGGroup) <= kP, "G extent");
static_assert(mn_extent_other(kP, 12, kPGroup) <= kSmem && mn_extent(kP, 12, kPGroup) <= kW1, "P extent");
static_assert(mn_extent_other(kQ, 16, kQGroup) <= kSmem && mn_extent(kQ, 16, kQGroup) <= kG, "Q extent");
static_assert(mn_extent_other(kQ + 1024, 4, kQGroup) <= kSmem, "dY extent");
static_assert(kBar % 8 == 0, "mbarrier alignment");
}  // namespace train

// dZ = acc * silu'(z + bias) over N columns (a multiple of 32), rounded to BF16
// into row `row` of a K-major operand with 8-row groups group_bytes apart
template <int N>
__device__ __forceinline__ void backward_epilogue(uint32_t t_acc, uint32_t t_z, const float* bias, unsigned char* dst,
                                                  int row, int group_bytes) {
#pragma unroll
  for (int c = 0; c < N; c += 32) {
    float a[32], z[32];
    tmem_ld32(t_acc + (uint32_t)c, a);
    tmem_ld32(t_z + (uint32_t)c, z);
#pragma unroll
    for (int j = 0; j < 32; ++j) a[j] *= silu_grad(z[j] + bias[c + j]);
#pragma unroll
    for (int j = 0; j < 32; j += 8) store8_bf16(dst, group_offset(row, c + j, group_bytes), a + j);
  }
}

__global__ void __launch_bounds__(kThreads, 1) k_mlp_train_tc(const __nv_bfloat16* __restrict__ x,
                                                              const float* __restrict__ target, int n,
                                                              const float* __restrict__ params,
                                                              float* __restrict__ grad, float* __restrict__ loss,
                                                              bool upstream) {
  using namespace train;
  extern __shared__ __align__(1024) unsigned char smem[];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  unsigned char* Q = smem + kQ;
  unsigned char* G = smem + kG;
  unsigned char* P = smem + kP;
  float* b1 = reinterpret_cast<float*>(smem + kBias);
  float* b2 = b1 + H;
  float* b3 = b2 + H;
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + kBar);
  uint32_t* tbase = reinterpret_cast<uint32_t*>(smem + kBar + 8);
  // weights: the forward operands and the transposed ones of the backward pass
  stage_bf16(smem + kW1, params + PW1, H, H, IN, tid, kThreads);
  stage_bf16(smem + kW2, params + PW2, H, H, H, tid, kThreads);
  stage_bf16(smem + kW3, params + PW3, kN3, OUT, H, tid, kThreads);
  for (int e = tid; e < H * 16; e += kThreads) {
    const int i = e >> 4, o = e & 15;
    store_bf16(smem + kW3T, core_offset(i, o, 16), o < OUT ? params[PW3 + o * H + i] : 0.0f);
  }
  for (int e = tid; e < H * H; e += kThreads) {
    const int i = e / H, o = e % H;
    store_bf16(smem + kW2T, core_offset(i, o, H), params[PW2 + o * H + i]);
  }
  for (int i = tid; i < H; i += kThreads) {
    b1[i] = params[PB1 + i];
    b2[i] = params[PB2 + i];
  }
  for (int i = tid; i < OUT; i += kThreads) b3[i] = params[PB3 + i];
  // constant cores: the ones column (feature 80) of P and Q, Q's zero pad
  {
    const uint4 one = make_uint4(0x3F80u, 0u, 0u, 0u), zero = make_uint4(0u, 0u, 0u, 0u);
    for (int e = tid; e < kGroups * 8 * 8; e += kThreads) {
      const int g = e >> 6, r = (e >> 3) & 7, c = e & 7;  // c: P core 10, 11, Q core 10..15
      if (c < 2)
        *reinterpret_cast<uint4*>(P + g * kPGroup + (10 + c) * 128 + r * 16) = c == 0 ? one : zero;
      else
        *reinterpret_cast<uint4*>(Q + g * kQGroup + (8 + c) * 128 + r * 16) = c == 2 ? one : zero;
    }
  }
  if (tid == 0) {
    lbm::mbar_init(bar, 1);
    lbm::mbar_init_fence();
  }
  if (warp == 0) tmem_alloc(tbase, kCols);
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tmem = *tbase;
  const uint32_t lanes = (uint32_t)(warp * 32) << 16;
  const uint32_t q = lbm::smem_addr(Q), gq = lbm::smem_addr(G), p = lbm::smem_addr(P);
  const uint32_t w1 = lbm::smem_addr(smem + kW1), w2 = lbm::smem_addr(smem + kW2), w3 = lbm::smem_addr(smem + kW3);
  const uint32_t w3t = lbm::smem_addr(smem + kW3T), w2t = lbm::smem_addr(smem + kW2T);
  const float scale = 2.0f / (6.0f * (float)n);
  float my_loss = 0.0f;
  uint32_t phase = 0;
  bool ok = true, first = true;
  const int tiles = (n + kRows - 1) / kRows;
  for (int tile = blockIdx.x; tile < tiles && ok; tile += gridDim.x) {
    const int row = tile * kRows + tid;
    const bool active = row < n;
    float tg[8];
    {
      uint4 lo = make_uint4(0, 0, 0, 0), hi = lo;
      float4 t0 = make_float4(0.f, 0.f, 0.f, 0.f), t1 = t0;
      if (active) {
        lo = *reinterpret_cast<const uint4*>(x + (size_t)row * IN);
        hi = *reinterpret_cast<const uint4*>(x + (size_t)row * IN + 8);
        t0 = *reinterpret_cast<const float4*>(target + (size_t)row * OUT);
        t1 = *reinterpret_cast<const float4*>(target + (size_t)row * OUT + 4);
      }
      *reinterpret_cast<uint4*>(P + group_offset(tid, 0, kPGroup)) = lo;
      *reinterpret_cast<uint4*>(P + group_offset(tid, 8, kPGroup)) = hi;
      tg[0] = t0.x; tg[1] = t0.y; tg[2] = t0.z; tg[3] = t0.w;
      tg[4] = t1.x; tg[5] = t1.y; tg[6] = t1.z; tg[7] = t1.w;
    }
    sync_for_mma();
    if (tid == 0) {  // Z1 = X W1^T
      fence_after_sync();
      mma_bf16(tmem + kZ1, smem_desc(p, 128, kPGroup), smem_desc(w1, 128, 256), instr_desc(kRows, H), 0);
      mma_commit(bar);
    }
    if (!(ok = wait_mma(bar, phase))) break;
    fence_after_sync();
    epilogue_bf16<H>(tmem + lanes + kZ1, b1, P + 256, tid, kPGroup, Silu());
    sync_for_mma();
    if (tid == 0) {  // Z2 = H1 W2^T
      fence_after_sync();
#pragma unroll
      for (int kc = 0; kc < H / 16; ++kc)
        mma_bf16(tmem + kZ2, smem_desc(p + 256 + kc * 256, 128, kPGroup), smem_desc(w2 + kc * 256, 128, 1024),
                 instr_desc(kRows, H), kc > 0);
      mma_commit(bar);
    }
    if (!(ok = wait_mma(bar, phase))) break;
    fence_after_sync();
    epilogue_bf16<H>(tmem + lanes + kZ2, b2, Q, tid, kQGroup, Silu());
    sync_for_mma();
    if (tid == 0) {  // Y = H2 W3^T
      fence_after_sync();
#pragma unroll
      for (int kc = 0; kc < H / 16; ++kc)
        mma_bf16(tmem + kS, smem_desc(q + kc * 256, 128, kQGroup), smem_desc(w3 + kc * 256, 128, 1024),
                 instr_desc(kRows, kN3), kc > 0);
      mma_commit(bar);
    }
    if (!(ok = wait_mma(bar, phase))) break;
    fence_after_sync();
    {
      float y[16], d[16];
      tmem_ld16(tmem + lanes + kS, y);
#pragma unroll
      for (int j = 0; j < 16; ++j) d[j] = 0.0f;
#pragma unroll
      for (int j = 0; j < 6; ++j) {
        if (upstream) {  // target holds dLoss/dy: the pass is a vector-Jacobian product
          const float g = active ? tg[j] : 0.0f;
          my_loss += g * (y[j] + b3[j]);
          d[j] = g;
        } else {
          const float diff = active ? y[j] + b3[j] - tg[j] : 0.0f;
          my_loss += diff * diff;
          d[j] = scale * diff;
        }
      }
      store8_bf16(Q, group_offset(tid, 64, kQGroup), d);
      store8_bf16(Q, group_offset(tid, 72, kQGroup), d + 8);
    }
    sync_for_mma();
    if (tid == 0) {  // dY W3 (K = 16)
      fence_after_sync();
      mma_bf16(tmem + kS, smem_desc(q + 1024, 128, kQGroup), smem_desc(w3t, 128, 256), instr_desc(kRows, H), 0);
      mma_commit(bar);
    }
    if (!(ok = wait_mma(bar, phase))) break;
    fence_after_sync();
    backward_epilogue<H>(tmem + lanes + kS, tmem + lanes + kZ2, b2, G + 1024, tid, kGGroup);
    sync_for_mma();
    if (tid == 0) {  // dZ2 W2 (K = 64)
      fence_after_sync();
#pragma unroll
      for (int kc = 0; kc < H / 16; ++kc)
        mma_bf16(tmem + kS, smem_desc(gq + 1024 + kc * 256, 128, kGGroup), smem_desc(w2t + kc * 256, 128, 1024),
                 instr_desc(kRows, H), kc > 0);
      mma_commit(bar);
    }
    if (!(ok = wait_mma(bar, phase))) break;
    fence_after_sync();
    backward_epilogue<H>(tmem + lanes + kS, tmem + lanes + kZ1, b1, G, tid, kGGroup);
    sync_for_mma();
    if (tid == 0) {  // gradients: K = the tile's samples, 16 per MMA
      fence_after_sync();
#pragma unroll
      for (int kc = 0; kc < kRows / 16; ++kc) {
        const uint32_t acc = (!first || kc > 0) ? 1u : 0u;
        mma_bf16(tmem + kD1, smem_desc(gq + kc * 2 * kGGroup, kGGroup, 128),
                 smem_desc(p + kc * 2 * kPGroup, kPGroup, 128), instr_desc_mn(kRows, 96, true, true), acc);
        mma_bf16(tmem + kD2, smem_desc(q + kc * 2 * kQGroup, kQGroup, 128),
                 smem_desc(q + 1024 + kc * 2 * kQGroup, kQGroup, 128), instr_desc_mn(kRows, 32, true, true), acc);
      }
      mma_commit(bar);
    }
    // the next tile overwrites the operands only after these MMAs are done
    if (!(ok = wait_mma(bar, phase))) break;
    fence_after_sync();
    first = false;
  }
  for (int o = 16; o > 0; o >>= 1) my_loss += __shfl_xor_sync(0xffffffffu, my_loss, o);
  if (ok && lane == 0) atomicAdd(loss, upstream ? my_loss : my_loss / (6.0f * (float)n));
  if (ok) {
    // row tid of the accumulated gradients (columns per the buffers' features)
    if (warp < 2) {  // rows 0..63: dW1 (columns 0..15), b1 (80), dW3^T (D2 columns 0..7)
      float v[16];
      tmem_ld16(tmem + lanes + kD1, v);
#pragma unroll
      for (int c = 0; c < IN; ++c) atomicAdd(&grad[PW1 + tid * IN + c], v[c]);
      tmem_ld16(tmem + lanes + kD1 + 80, v);
      atomicAdd(&grad[PB1 + tid], v[0]);
      tmem_ld16(tmem + lanes + kD2, v);
#pragma unroll
      for (int o = 0; o < OUT; ++o) atomicAdd(&grad[PW3 + o * H + tid], v[o]);
    } else {  // rows 64..127: dW2 (columns 16..79), b2 (80), b3 (D2 column 16, rows 64..71)
      const int o = tid - H;
#pragma unroll
      for (int c = 0; c < H; c += 16) {
        float v[16];
        tmem_ld16(tmem + lanes + kD1 + 16 + (uint32_t)c, v);
#pragma unroll
        for (int j = 0; j < 16; ++j) atomicAdd(&grad[PW2 + o * H + c + j], v[j]);
      }
      float v[16];
      tmem_ld16(tmem + lanes + kD1 + 80, v);
      atomicAdd(&grad[PB2 + o], v[0]);
      tmem_ld16(tmem + lanes + kD2 + 16, v);
      if (o < OUT) atomicAdd(&grad[PB3 + o], v[0]);
    }
  }
  if (!ok && tid == 0) atomicAdd(&mlp_tc_timeouts, 1u);
  fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    fence_after_sync();
    tmem_dealloc(tmem, kCols);
  }
}

}  // namespace lbm_mlp_tc
