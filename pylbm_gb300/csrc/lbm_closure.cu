// Training and batch inference of the learned-closure MLP (part of
// liblbm_gb300.so).  BF16 inputs, weights and activations; FP32 accumulation
// on the tensor cores (lbm_mlp.cuh); FP32 master weights and Adam.
//
// One training step on a batch of n samples (n a multiple of 16):
//   k_mlp_fwd_bwd   per 16-sample tile: forward, MSE loss on the 6 outputs,
//                   backward through the data path; writes the BF16
//                   activations H1, H2 and gradients dY, dH1, dH2
//   k_mlp_wgrad     weight gradients dW = G^T A reduced over the batch on the
//                   tensor cores (per-block partials, FP32 atomics), biases
//                   as column sums
//   k_mlp_adam      Adam on the FP32 master block, then the BF16 copies in
//                   both layouts the GEMMs use
#include "lbm_common.cuh"
#include "lbm_mlp.cuh"
#include "lbm_mlp_tc.cuh"

using namespace lbm;
using namespace lbm_mlp;

namespace {

constexpr int kWarps = 4;
constexpr int kChunk = 64;  // samples staged per k-loop iteration of the weight gradients

struct Scratch {
  __nv_bfloat16* h1;   // [n][64]
  __nv_bfloat16* h2;   // [n][64]
  __nv_bfloat16* dh1;  // [n][64]
  __nv_bfloat16* dh2;  // [n][64]
  __nv_bfloat16* dy;   // [n][8]
};

size_t scratch_bytes_for(int n) { return (size_t)n * (4 * H + OUT) * sizeof(__nv_bfloat16); }

Scratch carve(void* base, int n) {
  Scratch s;
  __nv_bfloat16* p = (__nv_bfloat16*)base;
  s.h1 = p;
  s.h2 = p + (size_t)n * H;
  s.dh1 = p + (size_t)2 * n * H;
  s.dh2 = p + (size_t)3 * n * H;
  s.dy = p + (size_t)4 * n * H;
  return s;
}

__device__ __forceinline__ void load_x_frag(const __nv_bfloat16* x, int r0, int lane, uint32_t (&a)[4]) {
  const int g = lane >> 2, t = lane & 3;
  a[0] = *reinterpret_cast<const uint32_t*>(x + (size_t)(r0 + g) * IN + 2 * t);
  a[1] = *reinterpret_cast<const uint32_t*>(x + (size_t)(r0 + g + 8) * IN + 2 * t);
  a[2] = *reinterpret_cast<const uint32_t*>(x + (size_t)(r0 + g) * IN + 8 + 2 * t);
  a[3] = *reinterpret_cast<const uint32_t*>(x + (size_t)(r0 + g + 8) * IN + 8 + 2 * t);
}

__device__ __forceinline__ void store_a_frag(__nv_bfloat16* dst, int ld, int r0, int j, int lane,
                                             const uint32_t (&a)[4]) {
  const int g = lane >> 2, t = lane & 3;
  *reinterpret_cast<uint32_t*>(dst + (size_t)(r0 + g) * ld + 16 * j + 2 * t) = a[0];
  *reinterpret_cast<uint32_t*>(dst + (size_t)(r0 + g + 8) * ld + 16 * j + 2 * t) = a[1];
  *reinterpret_cast<uint32_t*>(dst + (size_t)(r0 + g) * ld + 16 * j + 8 + 2 * t) = a[2];
  *reinterpret_cast<uint32_t*>(dst + (size_t)(r0 + g + 8) * ld + 16 * j + 8 + 2 * t) = a[3];
}

__global__ void __launch_bounds__(32 * kWarps) k_mlp_fwd_bwd(const __nv_bfloat16* __restrict__ x,
                                                            const float* __restrict__ target, int n,
                                                            const __nv_bfloat16* __restrict__ wb,
                                                            const float* __restrict__ params, Scratch s,
                                                            float* __restrict__ loss) {
  __shared__ __align__(16) __nv_bfloat16 w_s[BF16_WEIGHTS];
  __shared__ float b_s[2 * H + OUT];
  for (int i = threadIdx.x; i < BF16_WEIGHTS; i += blockDim.x) w_s[i] = wb[i];
  for (int i = threadIdx.x; i < H; i += blockDim.x) {
    b_s[i] = params[PB1 + i];
    b_s[H + i] = params[PB2 + i];
  }
  for (int i = threadIdx.x; i < OUT; i += blockDim.x) b_s[2 * H + i] = params[PB3 + i];
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int g = lane >> 2, t = lane & 3;
  const float scale = 2.0f / (6.0f * (float)n);
  float local_loss = 0.0f;
  const int ntiles = n / 16;
  for (int tile = blockIdx.x * kWarps + warp; tile < ntiles; tile += gridDim.x * kWarps) {
    const int r0 = tile * 16;
    uint32_t xa[4];
    load_x_frag(x, r0, lane, xa);
    float y[4], z1[8][4], z2[8][4];
    uint32_t h1a[4][4], h2a[4][4];
    forward_tile<true>(xa, w_s, b_s, b_s + H, b_s + 2 * H, lane, y, z1, z2, h1a, h2a);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      store_a_frag(s.h1, H, r0, j, lane, h1a[j]);
      store_a_frag(s.h2, H, r0, j, lane, h2a[j]);
    }
    // loss and dL/dy on the 6 used outputs (columns 2t, 2t+1)
    float dy[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int row = r0 + g + (i >= 2 ? 8 : 0);
      const int col = 2 * t + (i & 1);
      const float diff = col < 6 ? y[i] - target[(size_t)row * OUT + col] : 0.0f;
      local_loss += diff * diff;
      dy[i] = scale * diff;
    }
    uint32_t dya[4];
    dya[0] = pack_bf16(dy[0], dy[1]);
    dya[1] = pack_bf16(dy[2], dy[3]);
    dya[2] = 0u;
    dya[3] = 0u;
    *reinterpret_cast<uint32_t*>(s.dy + (size_t)(r0 + g) * OUT + 2 * t) = dya[0];
    *reinterpret_cast<uint32_t*>(s.dy + (size_t)(r0 + g + 8) * OUT + 2 * t) = dya[1];
    // dH2 = (dY W3) * silu'(z2)
    float acc[8][4];
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
      acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.0f;
      uint32_t bb0, bb1;
      load_b(w_s + BW3N, 16, nt, 0, lane, bb0, bb1);
      mma16816(acc[nt], dya, bb0, bb1);
#pragma unroll
      for (int i = 0; i < 4; ++i) acc[nt][i] *= silu_grad(z2[nt][i]);
    }
    uint32_t d2a[4][4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      d_to_a(acc[2 * j], acc[2 * j + 1], d2a[j]);
      store_a_frag(s.dh2, H, r0, j, lane, d2a[j]);
    }
    // dH1 = (dH2 W2) * silu'(z1)
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
      acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.0f;
#pragma unroll
      for (int kt = 0; kt < 4; ++kt) {
        uint32_t bb0, bb1;
        load_b(w_s + BW2N, H, nt, kt, lane, bb0, bb1);
        mma16816(acc[nt], d2a[kt], bb0, bb1);
      }
#pragma unroll
      for (int i = 0; i < 4; ++i) acc[nt][i] *= silu_grad(z1[nt][i]);
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      uint32_t a[4];
      d_to_a(acc[2 * j], acc[2 * j + 1], a);
      store_a_frag(s.dh1, H, r0, j, lane, a);
    }
  }
  // block-reduce the loss
  for (int o = 16; o > 0; o >>= 1) local_loss += __shfl_xor_sync(0xffffffffu, local_loss, o);
  if (lane == 0) atomicAdd(loss, local_loss / (6.0f * (float)n));
}

// G^T A over a chunk of samples staged in shared memory: A fragment of G^T
// (rows = G columns, cols = samples) and B fragment of A (k = samples).
__device__ __forceinline__ void frag_gt(const __nv_bfloat16* g_s, int ldg, int mt, int kk, int lane, uint32_t (&a)[4]) {
  const int gg = lane >> 2, t = lane & 3;
  const int i0 = mt * 16 + gg, i1 = i0 + 8;
  const int k0 = kk * 16 + 2 * t;
  auto at = [&](int k, int i) { return g_s[k * ldg + i]; };
  __nv_bfloat162 v;
  v = __halves2bfloat162(at(k0, i0), at(k0 + 1, i0));
  a[0] = *reinterpret_cast<uint32_t*>(&v);
  v = __halves2bfloat162(at(k0, i1), at(k0 + 1, i1));
  a[1] = *reinterpret_cast<uint32_t*>(&v);
  v = __halves2bfloat162(at(k0 + 8, i0), at(k0 + 9, i0));
  a[2] = *reinterpret_cast<uint32_t*>(&v);
  v = __halves2bfloat162(at(k0 + 8, i1), at(k0 + 9, i1));
  a[3] = *reinterpret_cast<uint32_t*>(&v);
}

__device__ __forceinline__ void frag_b(const __nv_bfloat16* a_s, int lda, int nt, int kk, int lane, uint32_t& b0,
                                       uint32_t& b1) {
  const int gg = lane >> 2, t = lane & 3;
  const int j = nt * 8 + gg;
  const int k0 = kk * 16 + 2 * t;
  __nv_bfloat162 v = __halves2bfloat162(a_s[k0 * lda + j], a_s[(k0 + 1) * lda + j]);
  b0 = *reinterpret_cast<uint32_t*>(&v);
  v = __halves2bfloat162(a_s[(k0 + 8) * lda + j], a_s[(k0 + 9) * lda + j]);
  b1 = *reinterpret_cast<uint32_t*>(&v);
}

__global__ void __launch_bounds__(32 * kWarps) k_mlp_wgrad(const __nv_bfloat16* __restrict__ x, int n, Scratch s,
                                                           int samples_per_block, float* __restrict__ grad) {
  __shared__ __align__(16) __nv_bfloat16 sx[kChunk * IN];
  __shared__ __align__(16) __nv_bfloat16 sh1[kChunk * H];
  __shared__ __align__(16) __nv_bfloat16 sh2[kChunk * H];
  __shared__ __align__(16) __nv_bfloat16 sd1[kChunk * H];
  __shared__ __align__(16) __nv_bfloat16 sd2[kChunk * H];
  __shared__ __align__(16) __nv_bfloat16 sdy[kChunk * 16];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int gg = lane >> 2, t = lane & 3;
  float a2[8][4], a1[2][4], a3[8][4];  // dW2t rows (warp's m-tile) x 64, dW1t x 16, dW3t (warp 0)
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) a2[i][j] = a3[i][j] = 0.0f;
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) a1[i][j] = 0.0f;
  float bsum1 = 0.0f, bsum2 = 0.0f, bsum3 = 0.0f;
  const int begin = blockIdx.x * samples_per_block;
  const int end = min(n, begin + samples_per_block);
  for (int c0 = begin; c0 < end; c0 += kChunk) {
    const int rows = min(kChunk, end - c0);
    __syncthreads();
    for (int i = threadIdx.x; i < kChunk * H; i += blockDim.x) {
      const int r = i / H, c = i % H;
      const bool ok = r < rows;
      const size_t gi = (size_t)(c0 + r) * H + c;
      sh1[i] = ok ? s.h1[gi] : __float2bfloat16(0.0f);
      sh2[i] = ok ? s.h2[gi] : __float2bfloat16(0.0f);
      sd1[i] = ok ? s.dh1[gi] : __float2bfloat16(0.0f);
      sd2[i] = ok ? s.dh2[gi] : __float2bfloat16(0.0f);
    }
    for (int i = threadIdx.x; i < kChunk * 16; i += blockDim.x) {
      const int r = i / 16, c = i % 16;
      const bool ok = r < rows;
      sx[i] = ok ? x[(size_t)(c0 + r) * IN + c] : __float2bfloat16(0.0f);
      sdy[i] = (ok && c < OUT) ? s.dy[(size_t)(c0 + r) * OUT + c] : __float2bfloat16(0.0f);
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kChunk / 16; ++kk) {
      uint32_t ga[4];
      // dW2t[o][i] += sum_n dH2[n][o] H1[n][i]   (warp = m-tile of o)
      frag_gt(sd2, H, warp, kk, lane, ga);
#pragma unroll
      for (int nt = 0; nt < 8; ++nt) {
        uint32_t b0, b1;
        frag_b(sh1, H, nt, kk, lane, b0, b1);
        mma16816(a2[nt], ga, b0, b1);
      }
      // dW1t[o][i] += sum_n dH1[n][o] X[n][i]
      frag_gt(sd1, H, warp, kk, lane, ga);
#pragma unroll
      for (int nt = 0; nt < 2; ++nt) {
        uint32_t b0, b1;
        frag_b(sx, 16, nt, kk, lane, b0, b1);
        mma16816(a1[nt], ga, b0, b1);
      }
      if (warp == 0) {
        // dW3t[o][i] += sum_n dY[n][o] H2[n][i]   (o padded to 16)
        frag_gt(sdy, 16, 0, kk, lane, ga);
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
          uint32_t b0, b1;
          frag_b(sh2, H, nt, kk, lane, b0, b1);
          mma16816(a3[nt], ga, b0, b1);
        }
      }
    }
    // bias gradients: column sums (thread i < 64 sums column i of dH1/dH2, i < 8 of dY)
    if (threadIdx.x < H) {
      for (int r = 0; r < rows; ++r) {
        bsum1 += __bfloat162float(sd1[r * H + threadIdx.x]);
        bsum2 += __bfloat162float(sd2[r * H + threadIdx.x]);
        if (threadIdx.x < OUT) bsum3 += __bfloat162float(sdy[r * 16 + threadIdx.x]);
      }
    }
  }
  // flush partials (D fragment: rows gg, gg+8 of the m-tile; cols 2t, 2t+1 of the n-tile)
  const int o0 = warp * 16 + gg, o1 = o0 + 8;
#pragma unroll
  for (int nt = 0; nt < 8; ++nt) {
    const int c = nt * 8 + 2 * t;
    atomicAdd(&grad[PW2 + o0 * H + c], a2[nt][0]);
    atomicAdd(&grad[PW2 + o0 * H + c + 1], a2[nt][1]);
    atomicAdd(&grad[PW2 + o1 * H + c], a2[nt][2]);
    atomicAdd(&grad[PW2 + o1 * H + c + 1], a2[nt][3]);
  }
#pragma unroll
  for (int nt = 0; nt < 2; ++nt) {
    const int c = nt * 8 + 2 * t;
    atomicAdd(&grad[PW1 + o0 * IN + c], a1[nt][0]);
    atomicAdd(&grad[PW1 + o0 * IN + c + 1], a1[nt][1]);
    atomicAdd(&grad[PW1 + o1 * IN + c], a1[nt][2]);
    atomicAdd(&grad[PW1 + o1 * IN + c + 1], a1[nt][3]);
  }
  if (warp == 0) {
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
      const int c = nt * 8 + 2 * t;
      if (gg < OUT) {  // rows 0..7 of dW3t; rows 8..15 are the zero padding
        atomicAdd(&grad[PW3 + gg * H + c], a3[nt][0]);
        atomicAdd(&grad[PW3 + gg * H + c + 1], a3[nt][1]);
      }
    }
  }
  if (threadIdx.x < H) {
    atomicAdd(&grad[PB1 + threadIdx.x], bsum1);
    atomicAdd(&grad[PB2 + threadIdx.x], bsum2);
    if (threadIdx.x < OUT) atomicAdd(&grad[PB3 + threadIdx.x], bsum3);
  }
}

// FP32 master block -> BF16 copies in fragment order (lbm_mlp.cuh):
//   w1t = W1 [64 out][16 in], w2t = W2 [64][64], w3t = W3 [8][64]      (forward)
//   w2n = W2^T [64 in][64 out], w3n = W3^T [64 in][16 (8 out + zeros)]   (backward)
__global__ void k_mlp_sync(const float* __restrict__ p, __nv_bfloat16* __restrict__ wb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  int n, k;
  if (i < H * IN) {
    frag_source(i, IN, n, k);
    wb[BW1T + i] = __float2bfloat16_rn(p[PW1 + n * IN + k]);
  }
  if (i < H * H) {
    frag_source(i, H, n, k);
    wb[BW2T + i] = __float2bfloat16_rn(p[PW2 + n * H + k]);
    wb[BW2N + i] = __float2bfloat16_rn(p[PW2 + k * H + n]);  // transposed: n = in, k = out
  }
  if (i < OUT * H) {
    frag_source(i, H, n, k);
    wb[BW3T + i] = __float2bfloat16_rn(p[PW3 + n * H + k]);
  }
  if (i < H * 16) {
    frag_source(i, 16, n, k);  // n = in (64), k = out (16, padded)
    wb[BW3N + i] = k < OUT ? __float2bfloat16_rn(p[PW3 + k * H + n]) : __float2bfloat16(0.0f);
  }
}

struct AdamArgs {
  float lr, beta1, beta2, eps, bc1, bc2;
  int n;
};

__global__ void k_mlp_adam(float* __restrict__ p, float* __restrict__ m, float* __restrict__ v,
                           float* __restrict__ grad, AdamArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const float gr = grad[i];
  const float mm = a.beta1 * m[i] + (1.0f - a.beta1) * gr;
  const float vv = a.beta2 * v[i] + (1.0f - a.beta2) * gr * gr;
  m[i] = mm;
  v[i] = vv;
  p[i] -= a.lr * (mm / a.bc1) / (sqrtf(vv / a.bc2) + a.eps);
  grad[i] = 0.0f;
}

__global__ void __launch_bounds__(32 * kWarps) k_mlp_infer(const __nv_bfloat16* __restrict__ x, int n,
                                                           const __nv_bfloat16* __restrict__ wb,
                                                           const float* __restrict__ params, float* __restrict__ y) {
  __shared__ __align__(16) __nv_bfloat16 w_s[BF16_WEIGHTS];
  __shared__ float b_s[2 * H + OUT];
  for (int i = threadIdx.x; i < BF16_WEIGHTS; i += blockDim.x) w_s[i] = wb[i];
  for (int i = threadIdx.x; i < H; i += blockDim.x) {
    b_s[i] = params[PB1 + i];
    b_s[H + i] = params[PB2 + i];
  }
  for (int i = threadIdx.x; i < OUT; i += blockDim.x) b_s[2 * H + i] = params[PB3 + i];
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int g = lane >> 2, t = lane & 3;
  for (int tile = blockIdx.x * kWarps + warp; tile < n / 16; tile += gridDim.x * kWarps) {
    const int r0 = tile * 16;
    uint32_t xa[4];
    load_x_frag(x, r0, lane, xa);
    float out[4], z1[8][4], z2[8][4];
    uint32_t h1a[4][4], h2a[4][4];
    forward_tile<false>(xa, w_s, b_s, b_s + H, b_s + 2 * H, lane, out, z1, z2, h1a, h2a);
    y[(size_t)(r0 + g) * OUT + 2 * t] = out[0];
    y[(size_t)(r0 + g) * OUT + 2 * t + 1] = out[1];
    y[(size_t)(r0 + g + 8) * OUT + 2 * t] = out[2];
    y[(size_t)(r0 + g + 8) * OUT + 2 * t + 1] = out[3];
  }
}

int grid_for(int tiles) {
  int g = (tiles + kWarps - 1) / kWarps;
  return g < 1 ? 1 : (g > 4096 ? 4096 : g);
}

}  // namespace

extern "C" {

int lbm_mlp_sizes(int32_t* nparam, int32_t* nweights_bf16) {
  if (nparam) *nparam = NPARAM;
  if (nweights_bf16) *nweights_bf16 = BF16_WEIGHTS;
  return LBM_OK;
}

int lbm_mlp_scratch_bytes(int32_t n, size_t* bytes) {
  if (!bytes || n < 0) return fail(LBM_ERR_ARG, "lbm_mlp_scratch_bytes: bad argument");
  *bytes = scratch_bytes_for(n);
  return LBM_OK;
}

int lbm_mlp_sync_weights(const float* params, void* wbf16, void* stream) {
  if (!params || !wbf16) return fail(LBM_ERR_ARG, "lbm_mlp_sync_weights: NULL");
  k_mlp_sync<<<(H * H + 255) / 256, 256, 0, (cudaStream_t)stream>>>(params, (__nv_bfloat16*)wbf16);
  return launch_check("lbm_mlp_sync_weights");
}

int lbm_mlp_forward(const void* x, int32_t n, const void* wbf16, const float* params, float* y, void* stream) {
  if (!x || !wbf16 || !params || !y) return fail(LBM_ERR_ARG, "lbm_mlp_forward: NULL");
  if (n < 0 || n % 16) return fail(LBM_ERR_ARG, "lbm_mlp_forward: n=%d must be a multiple of 16", n);
  if (n == 0) return LBM_OK;
  k_mlp_infer<<<grid_for(n / 16), 32 * kWarps, 0, (cudaStream_t)stream>>>(
      (const __nv_bfloat16*)x, n, (const __nv_bfloat16*)wbf16, params, y);
  return launch_check("lbm_mlp_forward");
}

int lbm_mlp_forward_tc(const void* x, int32_t n, const float* params, float* y, void* stream) {
  if (!x || !params || !y) return fail(LBM_ERR_ARG, "lbm_mlp_forward_tc: NULL");
  if (n < 0) return fail(LBM_ERR_ARG, "lbm_mlp_forward_tc: n=%d", n);
  if (n == 0) return LBM_OK;
  int dev = 0, sms = 0;
  int rc = cuda_check(cudaGetDevice(&dev), "lbm_mlp_forward_tc: cudaGetDevice");
  if (!rc) rc = cuda_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "lbm_mlp_forward_tc");
  if (rc) return rc;
  const int tiles = (n + lbm_mlp_tc::kRows - 1) / lbm_mlp_tc::kRows;
  // eight blocks per SM hold 8 x 64 of the 512 tensor-memory columns
  const int blocks = tiles < 8 * sms ? tiles : 8 * sms;
  lbm_mlp_tc::k_mlp_forward_tc<<<blocks, lbm_mlp_tc::kThreads, 0, (cudaStream_t)stream>>>(
      (const __nv_bfloat16*)x, n, params, y);
  return launch_check("lbm_mlp_forward_tc");
}

static int train_tc(const void* x, const float* target, int32_t n, const float* params, float* grad, float* loss,
                    void* stream, bool upstream, const char* who) {
  if (!x || !target || !params || !grad || !loss) return fail(LBM_ERR_ARG, "%s: NULL", who);
  if (n <= 0) return fail(LBM_ERR_ARG, "%s: n=%d", who, n);
  int dev = 0, sms = 0;
  int rc = cuda_check(cudaGetDevice(&dev), who);
  if (!rc) rc = cuda_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), who);
  if (rc) return rc;
  static bool sized[64];  // dynamic shared memory above 48 KB, allowed once per device
  if (dev < 0 || dev >= 64 || !sized[dev]) {
    rc = cuda_check(cudaFuncSetAttribute(lbm_mlp_tc::k_mlp_train_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         lbm_mlp_tc::train::kSmem),
                    who);
    if (rc) return rc;
    if (dev >= 0 && dev < 64) sized[dev] = true;
  }
  cudaStream_t st = (cudaStream_t)stream;
  rc = cuda_check(cudaMemsetAsync(loss, 0, sizeof(float), st), who);
  if (rc) return rc;
  // one block per SM: each holds all 512 tensor-memory columns
  const int tiles = (n + lbm_mlp_tc::kRows - 1) / lbm_mlp_tc::kRows;
  const int blocks = tiles < sms ? tiles : sms;
  lbm_mlp_tc::k_mlp_train_tc<<<blocks, lbm_mlp_tc::kThreads, lbm_mlp_tc::train::kSmem, st>>>(
      (const __nv_bfloat16*)x, target, n, params, grad, loss, upstream);
  return launch_check(who);
}

int lbm_mlp_gradients_tc(const void* x, const float* target, int32_t n, const float* params, float* grad, float* loss,
                         void* stream) {
  return train_tc(x, target, n, params, grad, loss, stream, false, "lbm_mlp_gradients_tc");
}

int lbm_mlp_vjp_tc(const void* x, const float* dy, int32_t n, const float* params, float* grad, float* dot,
                   void* stream) {
  return train_tc(x, dy, n, params, grad, dot, stream, true, "lbm_mlp_vjp_tc");
}

int lbm_mlp_tc_timeouts(uint32_t* count) {
  if (!count) return fail(LBM_ERR_ARG, "lbm_mlp_tc_timeouts: NULL");
  return cuda_check(cudaMemcpyFromSymbol(count, lbm_mlp_tc::mlp_tc_timeouts, sizeof(uint32_t)),
                    "lbm_mlp_tc_timeouts");
}

int lbm_mlp_gradients(const void* x, const float* target, int32_t n, const void* wbf16, const float* params,
                      float* grad, float* loss, void* scratch, size_t scratch_bytes, void* stream) {
  if (!x || !target || !wbf16 || !params || !grad || !loss || !scratch)
    return fail(LBM_ERR_ARG, "lbm_mlp_gradients: NULL");
  if (n <= 0 || n % 16) return fail(LBM_ERR_ARG, "lbm_mlp_gradients: n=%d must be a positive multiple of 16", n);
  if (scratch_bytes < scratch_bytes_for(n))
    return fail(LBM_ERR_ARG, "lbm_mlp_gradients: scratch %zu < %zu bytes", scratch_bytes, scratch_bytes_for(n));
  cudaStream_t st = (cudaStream_t)stream;
  Scratch s = carve(scratch, n);
  int rc = cuda_check(cudaMemsetAsync(loss, 0, sizeof(float), st), "lbm_mlp_gradients: clear loss");
  if (rc) return rc;
  k_mlp_fwd_bwd<<<grid_for(n / 16), 32 * kWarps, 0, st>>>((const __nv_bfloat16*)x, target, n,
                                                          (const __nv_bfloat16*)wbf16, params, s, loss);
  rc = launch_check("lbm_mlp_gradients: forward/backward");
  if (rc) return rc;
  const int per = 2048;
  k_mlp_wgrad<<<(n + per - 1) / per, 32 * kWarps, 0, st>>>((const __nv_bfloat16*)x, n, s, per, grad);
  return launch_check("lbm_mlp_gradients: weight gradients");
}

int lbm_mlp_adam(float* params, float* m, float* v, float* grad, float lr, float beta1, float beta2, float eps,
                 int32_t step, void* wbf16, void* stream) {
  if (!params || !m || !v || !grad || !wbf16) return fail(LBM_ERR_ARG, "lbm_mlp_adam: NULL");
  if (step < 1) return fail(LBM_ERR_ARG, "lbm_mlp_adam: step=%d must start at 1", step);
  AdamArgs a;
  a.lr = lr;
  a.beta1 = beta1;
  a.beta2 = beta2;
  a.eps = eps;
  a.bc1 = 1.0f - powf(beta1, (float)step);
  a.bc2 = 1.0f - powf(beta2, (float)step);
  a.n = NPARAM;
  cudaStream_t st = (cudaStream_t)stream;
  k_mlp_adam<<<(NPARAM + 255) / 256, 256, 0, st>>>(params, m, v, grad, a);
  int rc = launch_check("lbm_mlp_adam");
  if (rc) return rc;
  return lbm_mlp_sync_weights(params, wbf16, stream);
}

}  // extern "C"
