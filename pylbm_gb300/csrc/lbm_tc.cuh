// 5th-generation tensor-core building blocks (tcgen05, sm_100+ / sm_103a):
// shared-memory operand layout and descriptors, the kind::f16 MMA issued by
// one thread, its commit to an mbarrier, the tensor-memory fences and loads.
#pragma once

#include "lbm_common.cuh"

namespace lbm_tc {

// byte offset of element (r, k) of an [R][K] BF16 operand in the K-major
// no-swizzle layout: core matrices of 8 rows x 8 elements (128 bytes, rows
// 16 bytes apart), K-adjacent core matrices 128 bytes apart, row groups of 8
// (K / 8) * 128 bytes apart
__device__ __forceinline__ uint32_t core_offset(int r, int k, int K) {
  return (uint32_t)((((r >> 3) * (K >> 3) + (k >> 3)) << 7) + ((r & 7) << 4) + ((k & 7) << 1));
}

// shared-memory matrix descriptor: start address, leading byte offset (the
// K-direction core-matrix step), stride byte offset (the 8-row step),
// descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, N and M
__host__ __device__ constexpr uint32_t instr_desc(int m, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

// the same with A and/or B MN-major (bits 15 / 16: the operand's M or N index
// is the contiguous one).  The MN-major no-swizzle layout: core matrices of
// 8 K-rows x 8 MN-elements (16-byte rows), the stride byte offset steps
// between core matrices along MN, the leading byte offset between groups of
// 8 along K.
__host__ __device__ constexpr uint32_t instr_desc_mn(int m, int n, bool a_mn, bool b_mn) {
  return instr_desc(m, n) | (a_mn ? 1u << 15 : 0u) | (b_mn ? 1u << 16 : 0u);
}

// byte offset of element (r, k) of a K-major operand whose 8-row groups are
// group_bytes apart (core_offset is the dense case, group_bytes = K / 8 * 128)
__device__ __forceinline__ uint32_t group_offset(int r, int k, int group_bytes) {
  return (uint32_t)((r >> 3) * group_bytes + ((k >> 3) << 7) + ((r & 7) << 4) + ((k & 7) << 1));
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.u32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   lbm::smem_addr(bar))
               : "memory");
}

__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// 16 / 32 consecutive accumulator columns of this thread's row (its warp's
// lanes).  The load and its wait sit in one asm statement, so no use of the
// registers can be scheduled before the data has arrived.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void store_bf16(unsigned char* base, uint32_t off, float v) {
  *reinterpret_cast<__nv_bfloat16*>(base + off) = __float2bfloat16_rn(v);
}

// eight consecutive K elements of one row (one 16-byte core-matrix row),
// rounded to BF16, in one shared-memory store; off = core_offset(r, k, K)
// with k a multiple of 8
__device__ __forceinline__ void store8_bf16(unsigned char* base, uint32_t off, const float* v) {
  uint4 w;
  __nv_bfloat162 p;
  p = __floats2bfloat162_rn(v[0], v[1]);
  w.x = *reinterpret_cast<uint32_t*>(&p);
  p = __floats2bfloat162_rn(v[2], v[3]);
  w.y = *reinterpret_cast<uint32_t*>(&p);
  p = __floats2bfloat162_rn(v[4], v[5]);
  w.z = *reinterpret_cast<uint32_t*>(&p);
  p = __floats2bfloat162_rn(v[6], v[7]);
  w.w = *reinterpret_cast<uint32_t*>(&p);
  *reinterpret_cast<uint4*>(base + off) = w;
}

// a row-major FP32 [rows][K] matrix (rows from `valid` on are zero) into the
// K-major core-matrix layout in BF16, eight elements per thread and step;
// K a multiple of 8
__device__ __forceinline__ void stage_bf16(unsigned char* dst, const float* __restrict__ src, int rows, int valid,
                                           int K, int tid, int nthreads) {
  const bool vec = (reinterpret_cast<uintptr_t>(src) & 15u) == 0;
  for (int i = tid; i < rows * (K >> 3); i += nthreads) {
    const int r = i / (K >> 3), k = (i % (K >> 3)) << 3;
    float v[8];
    if (r >= valid) {
#pragma unroll
      for (int j = 0; j < 8; ++j) v[j] = 0.0f;
    } else if (vec) {
      const float4 a = *reinterpret_cast<const float4*>(src + (size_t)r * K + k);
      const float4 b = *reinterpret_cast<const float4*>(src + (size_t)r * K + k + 4);
      v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
      v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
    } else {
#pragma unroll
      for (int j = 0; j < 8; ++j) v[j] = src[(size_t)r * K + k + j];
    }
    store8_bf16(dst, core_offset(r, k, K), v);
  }
}

// the epilogue of a hidden layer: N accumulator columns of this thread's row
// (N a multiple of 32), plus bias, through the activation, rounded to BF16
// into row `row` of the next layer's [..][N] K-major A operand
template <int N, class Act>
__device__ __forceinline__ void epilogue_bf16(uint32_t taddr, const float* bias, unsigned char* dst, int row,
                                              int group_bytes, Act act) {
#pragma unroll
  for (int c = 0; c < N; c += 32) {
    float v[32];
    tmem_ld32(taddr + (uint32_t)c, v);
#pragma unroll
    for (int j = 0; j < 32; ++j) v[j] = act(v[j] + bias[c + j]);
#pragma unroll
    for (int j = 0; j < 32; j += 8) store8_bf16(dst, group_offset(row, c + j, group_bytes), v + j);
  }
}

template <int N, class Act>
__device__ __forceinline__ void epilogue_bf16(uint32_t taddr, const float* bias, unsigned char* dst, int row,
                                              Act act) {
  epilogue_bf16<N>(taddr, bias, dst, row, N / 8 * 128, act);
}

// the block's generic-proxy shared-memory writes made visible to the tensor
// cores, and its tensor-memory reads ordered, before one thread issues MMAs
__device__ __forceinline__ void sync_for_mma() {
  fence_async_smem();
  fence_before_sync();
  __syncthreads();
}

// wait for the block's MMA commit of the current phase; false when any thread
// of the block gave up (every thread returns the same answer)
__device__ __forceinline__ bool wait_mma(uint64_t* bar, uint32_t& phase) {
  const bool ok = lbm::mbar_wait(bar, phase & 1);
  ++phase;
  return __syncthreads_and(ok) != 0;
}

// warp-wide: ncols columns of tensor memory (a power of two, 32..512); the
// base address lands in *dst (shared memory)
__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(lbm::smem_addr(dst)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

// warp-wide: free what tmem_alloc returned
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

}  // namespace lbm_tc
