// Shared device helpers: storage conversions, the lattice geometry passed by
// value to kernels, and the per-thread error message used by both libraries.
#pragma once

#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <cuda_bf16.h>

#include <cstdarg>
#include <cstdint>
#include <cstdio>

#include "lbm_gb300.h"

namespace lbm {

// ---------------------------------------------------------------- errors
struct ErrorSlot {
  char msg[512];
};

inline ErrorSlot& error_slot() {
  static thread_local ErrorSlot slot = {{0}};
  return slot;
}

inline int fail(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(error_slot().msg, sizeof(error_slot().msg), fmt, ap);
  va_end(ap);
  return code;
}

inline int cuda_check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    return fail(LBM_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
  }
  return LBM_OK;
}

inline int launch_check(const char* what) {
  return cuda_check(cudaGetLastError(), what);
}

inline size_t dtype_size(int dt) {
  switch (dt) {
    case LBM_F64: return 8;
    case LBM_F32: return 4;
    case LBM_F16: return 2;
    case LBM_BF16: return 2;
    default: return 0;
  }
}

// ---------------------------------------------------------------- storage
template <typename S> struct Store;

template <> struct Store<double> {
  static constexpr int code = LBM_F64;
  __device__ __forceinline__ static double load(const double* p) { return __ldg(p); }
  __device__ __forceinline__ static double load_plain(const double* p) { return *p; }
  __device__ __forceinline__ static void store(double* p, double v) { *p = v; }
};

template <> struct Store<float> {
  static constexpr int code = LBM_F32;
  __device__ __forceinline__ static float load(const float* p) { return __ldg(p); }
  __device__ __forceinline__ static float load_plain(const float* p) { return *p; }
  __device__ __forceinline__ static void store(float* p, float v) { *p = v; }
};

template <> struct Store<__half> {
  static constexpr int code = LBM_F16;
  __device__ __forceinline__ static float load(const __half* p) { return __half2float(__ldg(p)); }
  __device__ __forceinline__ static float load_plain(const __half* p) { return __half2float(*p); }
  __device__ __forceinline__ static void store(__half* p, float v) { *p = __float2half_rn(v); }
};

template <> struct Store<__nv_bfloat16> {
  static constexpr int code = LBM_BF16;
  __device__ __forceinline__ static float load(const __nv_bfloat16* p) {
    return __bfloat162float(__ldg(p));
  }
  __device__ __forceinline__ static float load_plain(const __nv_bfloat16* p) {
    return __bfloat162float(*p);
  }
  __device__ __forceinline__ static void store(__nv_bfloat16* p, float v) {
    *p = __float2bfloat16_rn(v);
  }
};

// ---------------------------------------------------------------- node pairs
// Two nodes' FP32 values processed together with the packed FP32x2
// instructions of sm_100+ (FADD2/FMUL2/FFMA2): the generated per-node algebra
// is instantiated with this type to update two neighbouring nodes at once.
struct F2 {
  float2 v;
  __device__ __forceinline__ F2() {}
  __device__ __forceinline__ F2(float a, float b) { v = make_float2(a, b); }
  __device__ __forceinline__ explicit F2(float a) { v = make_float2(a, a); }
  __device__ __forceinline__ explicit F2(double a) { v = make_float2((float)a, (float)a); }
  __device__ __forceinline__ explicit F2(int a) { v = make_float2((float)a, (float)a); }
};

// Adds and multiply-adds are packed.  A packed multiply whose result feeds a
// packed add is fused into one multiply-add by ptxas on sm_103a even when
// both carry an explicit .rn (measured: the pair then rounds once), while
// the scalar code of a module built with -fmad=false rounds twice; products
// are therefore two scalar multiplies, which are never contracted, and the
// two-node kernels round exactly as the one-node kernels.
__device__ __forceinline__ F2 operator+(F2 a, F2 b) {
  F2 r;
  asm("{\n\t.reg .b64 A, B, D;\n\tmov.b64 A, {%2, %3};\n\tmov.b64 B, {%4, %5};\n\t"
      "add.rn.f32x2 D, A, B;\n\tmov.b64 {%0, %1}, D;\n\t}"
      : "=f"(r.v.x), "=f"(r.v.y)
      : "f"(a.v.x), "f"(a.v.y), "f"(b.v.x), "f"(b.v.y));
  return r;
}
__device__ __forceinline__ F2 operator*(F2 a, F2 b) { return F2(__fmul_rn(a.v.x, b.v.x), __fmul_rn(a.v.y, b.v.y)); }
__device__ __forceinline__ F2 operator-(F2 a) { return F2(-a.v.x, -a.v.y); }
__device__ __forceinline__ F2 operator-(F2 a, F2 b) { return a + (-b); }
__device__ __forceinline__ F2 operator/(F2 a, F2 b) { return F2(a.v.x / b.v.x, a.v.y / b.v.y); }
__device__ __forceinline__ F2& operator+=(F2& a, F2 b) { a = a + b; return a; }
__device__ __forceinline__ F2 sqrt(F2 a) { return F2(sqrtf(a.v.x), sqrtf(a.v.y)); }
__device__ __forceinline__ F2 pow(F2 a, F2 e) { return F2(powf(a.v.x, e.v.x), powf(a.v.y, e.v.y)); }

// a*b + c with one rounding.  Scheme modules are compiled without implicit
// contraction, so these are the only fused multiply-adds of the generated
// algebra and every kernel instantiating it rounds the same way; the pair
// form rounds each lane exactly as the scalar form.
template <typename R>
__device__ __forceinline__ R lbm_fma(R a, R b, R c);
template <>
__device__ __forceinline__ double lbm_fma<double>(double a, double b, double c) { return __fma_rn(a, b, c); }
template <>
__device__ __forceinline__ float lbm_fma<float>(float a, float b, float c) { return __fmaf_rn(a, b, c); }
template <>
__device__ __forceinline__ F2 lbm_fma<F2>(F2 a, F2 b, F2 c) {
  F2 r;
  asm("{\n\t.reg .b64 A, B, C, D;\n\tmov.b64 A, {%2, %3};\n\tmov.b64 B, {%4, %5};\n\tmov.b64 C, {%6, %7};\n\t"
      "fma.rn.f32x2 D, A, B, C;\n\tmov.b64 {%0, %1}, D;\n\t}"
      : "=f"(r.v.x), "=f"(r.v.y)
      : "f"(a.v.x), "f"(a.v.y), "f"(b.v.x), "f"(b.v.y), "f"(c.v.x), "f"(c.v.y));
  return r;
}

// ---------------------------------------------------------------- geometry
// Kernel-side copy of lbm_lattice (without the shift table).
struct Geo {
  int dim;
  int nv;
  int n[3];
  int h[3];
  long long stride[3];
  long long vstride;
  long long origin;
};

inline Geo make_geo(const lbm_lattice& l) {
  Geo g;
  g.dim = l.dim;
  g.nv = l.nv;
  for (int d = 0; d < 3; ++d) {
    g.n[d] = l.n[d];
    g.h[d] = l.halo[d];
    g.stride[d] = l.stride[d];
  }
  g.vstride = l.vstride;
  g.origin = l.origin;
  return g;
}

// Validate a lattice descriptor against its own invariants.
inline int check_lattice(const lbm_lattice* l, const char* who) {
  if (!l) return fail(LBM_ERR_ARG, "%s: lattice is NULL", who);
  if (l->dim < 1 || l->dim > 3) return fail(LBM_ERR_ARG, "%s: dim=%d", who, l->dim);
  if (l->nv < 1 || l->nv > LBM_MAX_Q) return fail(LBM_ERR_ARG, "%s: nv=%d", who, l->nv);
  if (dtype_size(l->dtype) == 0) return fail(LBM_ERR_ARG, "%s: dtype=%d", who, l->dtype);
  for (int d = 0; d < 3; ++d) {
    if (l->n[d] < 1) return fail(LBM_ERR_ARG, "%s: n[%d]=%d", who, d, l->n[d]);
    if (l->halo[d] < 0) return fail(LBM_ERR_ARG, "%s: halo[%d]=%d", who, d, l->halo[d]);
    if (d < l->dim && l->halo[d] > l->n[d])
      return fail(LBM_ERR_ARG, "%s: halo[%d]=%d exceeds n=%d", who, d, l->halo[d], l->n[d]);
    if (d >= l->dim && (l->n[d] != 1 || l->halo[d] != 0))
      return fail(LBM_ERR_ARG, "%s: unused axis %d must have n=1, halo=0", who, d);
  }
  if (l->stride[l->dim - 1] != 1) return fail(LBM_ERR_ARG, "%s: last axis must be contiguous", who);
  // the last element of the last population must lie inside the allocation
  long long last = (long long)(l->nv - 1) * l->vstride + l->origin;
  for (int d = 0; d < l->dim; ++d) last += (long long)(l->n[d] + 2 * l->halo[d] - 1) * l->stride[d];
  if (l->origin < 0 || last >= l->elements)
    return fail(LBM_ERR_ARG, "%s: strides exceed the allocation (%lld >= %lld)", who, last,
                (long long)l->elements);
  return LBM_OK;
}

// ---------------------------------------------------------------- async copies
// Bulk copies global -> shared on the TMA unit (cp.async.bulk) completing on
// an mbarrier, and the mbarrier operations around them.  Every wait is
// bounded in time: after kWaitCycles SM clocks it gives up and returns false
// (the caller records the timeout and leaves), so no kernel can spin forever.
constexpr long long kWaitCycles = 4000000000LL;  // about two seconds at 2 GHz

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
// 16 bytes global -> shared without registers (both addresses 16-byte
// aligned); complete after cp_async_wait_all
__device__ __forceinline__ void cp_async16(void* smem_dst, const void* gsrc) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_addr(smem_dst)), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
// the initialised barriers become visible to the async proxy (the copy engine)
__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_test(uint64_t* bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return done != 0;
}
// wait for the phase of the given parity to complete; false after the time bound
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  if (mbar_test(bar, parity)) return true;
  const long long t0 = clock64();
  while (!mbar_test(bar, parity))
    if (clock64() - t0 > kWaitCycles) return false;
  return true;
}
// `bytes` (a multiple of 16) from global src to shared dst, both 16-byte aligned
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_addr(dst)),
               "l"(src), "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}

// Element offset of halo coordinates (i0, i1, i2) of population 0.
__host__ __device__ __forceinline__ long long node_offset(const Geo& g, int i0, int i1, int i2) {
  return g.origin + (long long)i0 * g.stride[0] + (long long)i1 * g.stride[1] +
         (long long)i2 * g.stride[2];
}

}  // namespace lbm
