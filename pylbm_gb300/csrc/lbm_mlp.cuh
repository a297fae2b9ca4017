// Per-node MLP of the learned collision closure: warp-level BF16 tensor-core
// primitives (mma.sync m16n8k16, BF16 inputs, FP32 accumulation).
//
// Network: x (16 inputs, 9 used) -> 64 SiLU -> 64 SiLU -> y (8 outputs, 6 used).
// A warp evaluates 16 rows (nodes or samples) at a time.  The accumulator
// (D) fragments of two adjacent 8-column output tiles have exactly the
// register layout of the A fragment of one 16-column input tile, so hidden
// activations stay in registers from layer to layer.
//
// Weight layout in memory (both FP32 master and BF16 copies):
//   w1t [64][16], w2t [64][64], w3t [8][64]   ("out x in", B operands of the
//                                              forward GEMMs, k contiguous)
//   w2n [64][64], w3n [64][16]                ("in x out", B operands of the
//                                              backward data GEMMs; w3n pads
//                                              its 8 outputs to 16 with zeros)
//   b1 [64], b2 [64], b3 [8]                  (FP32 only)
#pragma once

#include <cuda_bf16.h>
#include <cstdint>

namespace lbm_mlp {

constexpr int IN = 16;
constexpr int H = 64;
constexpr int OUT = 8;

// offsets (elements) inside the BF16 weight block
constexpr int BW1T = 0;
constexpr int BW2T = BW1T + H * IN;
constexpr int BW3T = BW2T + H * H;
constexpr int BW2N = BW3T + OUT * H;
constexpr int BW3N = BW2N + H * H;
constexpr int BF16_WEIGHTS = BW3N + H * 16;

// offsets (floats) inside the FP32 parameter block (master weights + biases)
constexpr int PW1 = 0;             // [64][16]  (out x in)
constexpr int PB1 = PW1 + H * IN;
constexpr int PW2 = PB1 + H;       // [64][64]  (out x in)
constexpr int PB2 = PW2 + H * H;
constexpr int PW3 = PB2 + H;       // [8][64]   (out x in)
constexpr int PB3 = PW3 + OUT * H;
constexpr int NPARAM = PB3 + OUT;

__device__ __forceinline__ void mma16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t*>(&v);
}

__device__ __forceinline__ float bf16_round(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

// sigmoid(z) = (1 + tanh(z/2)) / 2 with the hardware tanh approximation
// (one MUFU instruction, max relative error ~2^-11, below the BF16 rounding
// of the activations); training and inference use the same function.
__device__ __forceinline__ float tanh_approx(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

__device__ __forceinline__ float sigmoidf_(float z) { return fmaf(0.5f, tanh_approx(0.5f * z), 0.5f); }

__device__ __forceinline__ float silu(float z) { return z * sigmoidf_(z); }

struct Silu {
  __device__ __forceinline__ float operator()(float z) const { return silu(z); }
};

__device__ __forceinline__ float silu_grad(float z) {
  const float s = sigmoidf_(z);
  return s * (1.0f + z * (1.0f - s));
}

// The BF16 copies of the weight matrices are stored in fragment order: for
// an [N][K] matrix, the B fragment (n-tile nt, k-tile kt) of lane l is the
// pair of 32-bit words at ((nt * K/16 + kt) * 32 + l) * 2, holding
//   b0 = (W[nt*8+g][kt*16+2t], W[nt*8+g][kt*16+2t+1])
//   b1 = (W[nt*8+g][kt*16+8+2t], W[nt*8+g][kt*16+8+2t+1]),  g = l/4, t = l%4,
// so a warp reads one fragment as 32 consecutive 64-bit words (no shared
// memory bank conflicts).  frag_source maps a position of that layout back to
// (n, k) of the matrix.
__device__ __forceinline__ void frag_source(int idx, int K, int& n, int& k) {
  const int j = idx & 3;
  const int lane = (idx >> 2) & 31;
  const int tile = idx >> 7;
  const int KT = K / 16;
  const int nt = tile / KT, kt = tile % KT;
  const int g = lane >> 2, t = lane & 3;
  n = nt * 8 + g;
  k = kt * 16 + 2 * t + (j & 1) + ((j & 2) ? 8 : 0);
}

__device__ __forceinline__ void load_b(const __nv_bfloat16* w, int K, int nt, int kt, int lane, uint32_t& b0,
                                       uint32_t& b1) {
  const uint2 v = reinterpret_cast<const uint2*>(w)[(nt * (K / 16) + kt) * 32 + lane];
  b0 = v.x;
  b1 = v.y;
}

// A fragment of k-tile j from the D fragments of output tiles 2j and 2j+1
__device__ __forceinline__ void d_to_a(const float (&d0)[4], const float (&d1)[4], uint32_t (&a)[4]) {
  a[0] = pack_bf16(d0[0], d0[1]);
  a[1] = pack_bf16(d0[2], d0[3]);
  a[2] = pack_bf16(d1[0], d1[1]);
  a[3] = pack_bf16(d1[2], d1[3]);
}

// Forward pass of one 16-row tile.  xa: A fragment of the (normalised, BF16)
// inputs.  Returns the output D fragment (columns 0..7), and optionally the
// pre-activations z1, z2 (D fragments) for the backward pass.
template <bool KEEP>
__device__ __forceinline__ void forward_tile(const uint32_t (&xa)[4], const __nv_bfloat16* __restrict__ wb,
                                             const float* __restrict__ b1, const float* __restrict__ b2,
                                             const float* __restrict__ b3, int lane, float (&y)[4],
                                             float (&z1)[8][4], float (&z2)[8][4], uint32_t (&h1a)[4][4],
                                             uint32_t (&h2a)[4][4]) {
  const int t = lane & 3;
  float acc[8][4];
#pragma unroll
  for (int nt = 0; nt < 8; ++nt) {
    const float c0 = b1[nt * 8 + 2 * t], c1 = b1[nt * 8 + 2 * t + 1];
    acc[nt][0] = c0;
    acc[nt][1] = c1;
    acc[nt][2] = c0;
    acc[nt][3] = c1;
    uint32_t bb0, bb1;
    load_b(wb + BW1T, IN, nt, 0, lane, bb0, bb1);
    mma16816(acc[nt], xa, bb0, bb1);
  }
#pragma unroll
  for (int nt = 0; nt < 8; ++nt)
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      if (KEEP) z1[nt][i] = acc[nt][i];
      acc[nt][i] = silu(acc[nt][i]);
    }
#pragma unroll
  for (int j = 0; j < 4; ++j) d_to_a(acc[2 * j], acc[2 * j + 1], h1a[j]);
#pragma unroll
  for (int nt = 0; nt < 8; ++nt) {
    const float c0 = b2[nt * 8 + 2 * t], c1 = b2[nt * 8 + 2 * t + 1];
    acc[nt][0] = c0;
    acc[nt][1] = c1;
    acc[nt][2] = c0;
    acc[nt][3] = c1;
#pragma unroll
    for (int kt = 0; kt < 4; ++kt) {
      uint32_t bb0, bb1;
      load_b(wb + BW2T, H, nt, kt, lane, bb0, bb1);
      mma16816(acc[nt], h1a[kt], bb0, bb1);
    }
  }
#pragma unroll
  for (int nt = 0; nt < 8; ++nt)
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      if (KEEP) z2[nt][i] = acc[nt][i];
      acc[nt][i] = silu(acc[nt][i]);
    }
#pragma unroll
  for (int j = 0; j < 4; ++j) d_to_a(acc[2 * j], acc[2 * j + 1], h2a[j]);
  {
    const float c0 = b3[2 * t], c1 = b3[2 * t + 1];
    y[0] = c0;
    y[1] = c1;
    y[2] = c0;
    y[3] = c1;
#pragma unroll
    for (int kt = 0; kt < 4; ++kt) {
      uint32_t bb0, bb1;
      load_b(wb + BW3T, H, 0, kt, lane, bb0, bb1);
      mma16816(y, h2a[kt], bb0, bb1);
    }
  }
}

}  // namespace lbm_mlp
