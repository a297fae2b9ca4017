// Kernel templates of a per-scheme module (lbm_scheme_<id>.so).
//
// The generated translation unit defines, before including this file:
//   LBM_DIM, LBM_Q, LBM_NCONS, LBM_NPRM, LBM_VMAX, LBM_SHIFTED,
//   LBM_FOR_EACH_V(X)    X(k, vx, vy, vz) for every population,
//   lbm_moments / lbm_populations / lbm_relax / lbm_equilibrium_abs /
//   lbm_relax_abs / lbm_collide  (per-node algebra of the scheme),
//   lbm_host_shift[], lbm_host_mref[]  (stored shift and its moments),
//   LBM_STORAGE (double, float, __half or __nv_bfloat16) and LBM_COMPUTE.
//
// One thread updates one interior node: it pulls the Q populations
// f_k(x - v_k) (structure of arrays, so each load of a warp is a contiguous
// run along the last axis), computes the moments, relaxes them and writes the
// Q new populations at x.  The two step kernels differ only in where the
// pulled neighbours come from: ghost layers filled beforehand
// (k_step_ghost), or the interior wrapped periodically (k_step_periodic).
#pragma once

#include "lbm_common.cuh"
#include "lbm_mlp.cuh"
#include "lbm_tc.cuh"

#include <type_traits>

#ifndef LBM_BLOCK
#define LBM_BLOCK 128
#endif

namespace lbm_scheme {

using lbm::Geo;
using lbm::Store;

// bounded waits of this module's kernels that gave up (0 in a healthy run)
__device__ unsigned int lbm_wait_timeouts;
using S = LBM_STORAGE;
using R = LBM_COMPUTE;

constexpr int kPrm = LBM_NPRM > 0 ? LBM_NPRM : 1;

struct StepArgs {
  Geo g;
  long long pull[LBM_Q];  // element offset of the pulled value of population k
  R prm[kPrm];
};

struct MomentArgs {
  Geo g;    // populations
  Geo gm;   // float64 moments
  double prm[kPrm];
};

// interior node handled by this thread, as halo coordinates
__device__ __forceinline__ bool my_node(const Geo& g, int& i0, int& i1, int& i2) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
#if LBM_DIM == 1
  if (t >= g.n[0]) return false;
  i0 = t + g.h[0];
  i1 = 0;
  i2 = 0;
#elif LBM_DIM == 2
  if (t >= g.n[1]) return false;
  i0 = blockIdx.y + g.h[0];
  i1 = t + g.h[1];
  i2 = 0;
#else
  if (t >= g.n[2]) return false;
  i0 = blockIdx.z + g.h[0];
  i1 = blockIdx.y + g.h[1];
  i2 = t + g.h[2];
#endif
  return true;
}

// every node of the halo-extended box (moment transforms)
__device__ __forceinline__ bool my_cell(const Geo& g, int& i0, int& i1, int& i2) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
#if LBM_DIM == 1
  if (t >= g.n[0] + 2 * g.h[0]) return false;
  i0 = t;
  i1 = 0;
  i2 = 0;
#elif LBM_DIM == 2
  if (t >= g.n[1] + 2 * g.h[1]) return false;
  i0 = blockIdx.y;
  i1 = t;
  i2 = 0;
#else
  if (t >= g.n[2] + 2 * g.h[2]) return false;
  i0 = blockIdx.z;
  i1 = blockIdx.y;
  i2 = t;
#endif
  return true;
}

__global__ void __launch_bounds__(LBM_BLOCK) k_step_ghost(const S* __restrict__ f, S* __restrict__ fnew,
                                                          StepArgs a) {
  int i0, i1, i2;
  if (!my_node(a.g, i0, i1, i2)) return;
  const long long o = lbm::node_offset(a.g, i0, i1, i2);
  R g[LBM_Q];
#pragma unroll
  for (int k = 0; k < LBM_Q; ++k) g[k] = (R)Store<S>::load(f + o + a.pull[k]);
  lbm_collide<R>(g, a.prm);
#pragma unroll
  for (int k = 0; k < LBM_Q; ++k) Store<S>::store(fnew + o + (long long)k * a.g.vstride, g[k]);
}

// offset of the pulled neighbour along one axis, wrapped into the interior
__device__ __forceinline__ long long wrap_off(int i, int s, int n, int h, long long stride) {
  int j = i - s;
  if (j < h) j += n;
  if (j >= n + h) j -= n;
  return (long long)(j - i) * stride;
}

__global__ void __launch_bounds__(LBM_BLOCK) k_step_periodic(const S* __restrict__ f, S* __restrict__ fnew,
                                                             StepArgs a) {
  int i0, i1, i2;
  if (!my_node(a.g, i0, i1, i2)) return;
  const long long o = lbm::node_offset(a.g, i0, i1, i2);
  long long off0[2 * LBM_VMAX + 1], off1[2 * LBM_VMAX + 1], off2[2 * LBM_VMAX + 1];
#pragma unroll
  for (int s = -LBM_VMAX; s <= LBM_VMAX; ++s) {
    off0[s + LBM_VMAX] = LBM_DIM > 0 ? wrap_off(i0, s, a.g.n[0], a.g.h[0], a.g.stride[0]) : 0;
    off1[s + LBM_VMAX] = LBM_DIM > 1 ? wrap_off(i1, s, a.g.n[1], a.g.h[1], a.g.stride[1]) : 0;
    off2[s + LBM_VMAX] = LBM_DIM > 2 ? wrap_off(i2, s, a.g.n[2], a.g.h[2], a.g.stride[2]) : 0;
  }
  R g[LBM_Q];
#define LBM_PULL_WRAP(k, vx, vy, vz)                                                            \
  g[k] = (R)Store<S>::load(f + o + (long long)(k) * a.g.vstride + off0[(vx) + LBM_VMAX] +      \
                           off1[(vy) + LBM_VMAX] + off2[(vz) + LBM_VMAX]);
  LBM_FOR_EACH_V(LBM_PULL_WRAP)
#undef LBM_PULL_WRAP
  lbm_collide<R>(g, a.prm);
#pragma unroll
  for (int k = 0; k < LBM_Q; ++k) Store<S>::store(fnew + o + (long long)k * a.g.vstride, g[k]);
}

// ---------------------------------------------------------------------------
// Bounce-back box walls folded into the pull.  On a box whose boundary links
// are all bounce-back links of its walls, the ghost slot (k, x - v_k) a wall
// node x pulls from would hold f_k'(x) + c (k' opposite to k) after the
// boundary launch, with c given by k and the walls the slot lies beyond
// (host: boundary.box_wall_table).  The step reads f_k'(x) and adds c itself,
// in the boundary launch's arithmetic, and rounds the value through the
// storage type as the ghost store would: the populations equal those of the
// boundary launch followed by k_step_ghost bit for bit, without the launch
// and without reading or writing ghost slots.
struct WallArgs {
  R c[LBM_Q][27];  // constant by population and wall signature 9 (o0+1) + 3 (o1+1) + (o2+1)
  int sym[LBM_Q];  // opposite population
};

// v rounded to the storage type and back, in registers: what a store to the
// ghost slot and the step's load of it would give
template <typename T> struct StorageRound {
  __device__ __forceinline__ static R apply(R v) { return v; }  // float / double: exact
};
template <> struct StorageRound<__half> {
  __device__ __forceinline__ static R apply(R v) { return (R)__half2float(__float2half_rn((float)v)); }
};
template <> struct StorageRound<__nv_bfloat16> {
  __device__ __forceinline__ static R apply(R v) { return (R)__bfloat162float(__float2bfloat16_rn((float)v)); }
};
__device__ __forceinline__ R through_storage(R v) { return StorageRound<S>::apply(v); }

// wall offset of the source of a node at (lo, hi) faces for a velocity component
__device__ __forceinline__ int wall_off(int v, bool lo, bool hi) { return (v > 0 && lo) ? -1 : ((v < 0 && hi) ? 1 : 0); }

__global__ void __launch_bounds__(LBM_BLOCK) k_step_walls(const S* __restrict__ f, S* __restrict__ fnew,
                                                          StepArgs a, WallArgs w) {
  int i0, i1, i2;
  if (!my_node(a.g, i0, i1, i2)) return;
  const long long o = lbm::node_offset(a.g, i0, i1, i2);
  const bool lo0 = i0 == a.g.h[0], hi0 = i0 == a.g.h[0] + a.g.n[0] - 1;
  const bool lo1 = LBM_DIM > 1 && i1 == a.g.h[1], hi1 = LBM_DIM > 1 && i1 == a.g.h[1] + a.g.n[1] - 1;
  const bool lo2 = LBM_DIM > 2 && i2 == a.g.h[2], hi2 = LBM_DIM > 2 && i2 == a.g.h[2] + a.g.n[2] - 1;
  R g[LBM_Q];
  // walls normal to the outer axes are uniform over a row (a block's rows);
  // the two walls normal to the contiguous axis touch one thread per row end
#if LBM_DIM == 3
  const bool outer = lo0 || hi0 || lo1 || hi1, loL = lo2, hiL = hi2;
  constexpr int wL = 1;
#define LBM_VC(vx, vy, vz) (vz)
#elif LBM_DIM == 2
  const bool outer = lo0 || hi0, loL = lo1, hiL = hi1;
  constexpr int wL = 3;
#define LBM_VC(vx, vy, vz) (vy)
#else
  const bool outer = false, loL = lo0, hiL = hi0;
  constexpr int wL = 9;
#define LBM_VC(vx, vy, vz) (vx)
#endif
  (void)lo2;
  (void)hi2;
  if (!outer) {
    // the plain pull (a row end reads its ghost neighbour, replaced below)
#pragma unroll
    for (int k = 0; k < LBM_Q; ++k) g[k] = (R)Store<S>::load(f + o + a.pull[k]);
    if (loL || hiL) {
#define LBM_FIX_END(k, vx, vy, vz)                                                                      \
  {                                                                                                     \
    const int sig = 13 + wL * wall_off(LBM_VC(vx, vy, vz), loL, hiL);                                   \
    if (sig != 13)                                                                                      \
      g[k] = through_storage((R)Store<S>::load(f + o + (long long)w.sym[k] * a.g.vstride) + w.c[k][sig]); \
  }
      LBM_FOR_EACH_V(LBM_FIX_END)
#undef LBM_FIX_END
    }
  } else {
#define LBM_PULL_WALL(k, vx, vy, vz)                                                                       \
  {                                                                                                        \
    const int sig = 9 * (wall_off(vx, lo0, hi0) + 1) + 3 * (wall_off(vy, lo1, hi1) + 1) +                 \
                    (wall_off(vz, lo2, hi2) + 1);                                                          \
    if (sig == 13)                                                                                         \
      g[k] = (R)Store<S>::load(f + o + a.pull[k]);                                                         \
    else                                                                                                   \
      g[k] = through_storage((R)Store<S>::load(f + o + (long long)w.sym[k] * a.g.vstride) + w.c[k][sig]); \
  }
    LBM_FOR_EACH_V(LBM_PULL_WALL)
#undef LBM_PULL_WALL
  }
#undef LBM_VC
  lbm_collide<R>(g, a.prm);
#pragma unroll
  for (int k = 0; k < LBM_Q; ++k) Store<S>::store(fnew + o + (long long)k * a.g.vstride, g[k]);
}

// ---------------------------------------------------------------------------
// Two nodes per thread (16-bit storage).  A thread owns nodes z and z+1 of the
// contiguous axis (z even), loads each population of both as one 32-bit word,
// and runs the generated algebra once on F2 = two FP32 lanes (packed FP32x2
// instructions), halving the load/store/convert/address instructions and the
// additions per node of the issue-bound 16-bit path.  Populations moving
// along the contiguous axis read the neighbouring word; where the periodic
// wrap breaks adjacency (row ends) the one wrapped value is read on its own.
template <typename T> struct Pair;
template <> struct Pair<__half> {
  __device__ __forceinline__ static float2 load(const __half* p) {
    return __half22float2(*reinterpret_cast<const __half2*>(p));
  }
  __device__ __forceinline__ static float one(const __half* p) { return __half2float(*p); }
  __device__ __forceinline__ static void store(__half* p, float2 v) {
    *reinterpret_cast<__half2*>(p) = __floats2half2_rn(v.x, v.y);
  }
};
template <> struct Pair<__nv_bfloat16> {
  __device__ __forceinline__ static float2 load(const __nv_bfloat16* p) {
    return __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(p));
  }
  __device__ __forceinline__ static float one(const __nv_bfloat16* p) { return __bfloat162float(*p); }
  __device__ __forceinline__ static void store(__nv_bfloat16* p, float2 v) {
    *reinterpret_cast<__nv_bfloat162*>(p) = __floats2bfloat162_rn(v.x, v.y);
  }
};
template <> struct Pair<float> {
  __device__ __forceinline__ static float2 load(const float* p) { return *reinterpret_cast<const float2*>(p); }
  __device__ __forceinline__ static float one(const float* p) { return *p; }
  __device__ __forceinline__ static void store(float* p, float2 v) { *reinterpret_cast<float2*>(p) = v; }
};

#if defined(LBM_PAIRS) && LBM_VMAX == 1
#define LBM_HAS_PAIRS 1
// pulled pair of population plane `p` (already offset to node z of this row
// and to the outer-axis neighbour), velocity component vl along the contiguous axis
__device__ __forceinline__ lbm::F2 pull_pair(const S* __restrict__ p, int vl, int z, int nL) {
  float lo, hi;
  if (vl == 0) {
    const float2 w = Pair<S>::load(p);
    lo = w.x;
    hi = w.y;
  } else if (vl > 0) {  // sources z-1, z
    const float2 w = Pair<S>::load(p);
    hi = w.x;
    lo = z > 0 ? Pair<S>::load(p - 2).y : Pair<S>::one(p + (nL - 1));
  } else {  // sources z+1, z+2
    const float2 w = Pair<S>::load(p);
    lo = w.y;
    hi = z + 2 < nL ? Pair<S>::load(p + 2).x : Pair<S>::one(p - z);
  }
  return lbm::F2(lo, hi);
}

// the velocity component along the last axis and the outer offset of population k
#if LBM_DIM == 1
#define LBM_VL(vx, vy, vz) (vx)
#define LBM_OUTER(vx, vy, vz) 0LL
#elif LBM_DIM == 2
#define LBM_VL(vx, vy, vz) (vy)
#define LBM_OUTER(vx, vy, vz) off0[(vx) + 1]
#else
#define LBM_VL(vx, vy, vz) (vz)
#define LBM_OUTER(vx, vy, vz) (off0[(vx) + 1] + off1[(vy) + 1])
#endif

// the pulled values of the two nodes (z, z + 1) of a row, periodic wrap
__device__ __forceinline__ void pull_pairs(const S* __restrict__ f, const Geo& g, int i0, int i1, int i2, int z,
                                           int nL, lbm::F2 (&gv)[LBM_Q]) {
  const long long o = lbm::node_offset(g, i0, i1, i2);
  long long off0[3] = {0, 0, 0}, off1[3] = {0, 0, 0};
#pragma unroll
  for (int s = -1; s <= 1; ++s) {
    if (LBM_DIM > 1) off0[s + 1] = wrap_off(i0, s, g.n[0], g.h[0], g.stride[0]);
    if (LBM_DIM > 2) off1[s + 1] = wrap_off(i1, s, g.n[1], g.h[1], g.stride[1]);
  }
  (void)off1;
#define LBM_PULL_PAIR(k, vx, vy, vz) \
  gv[k] = pull_pair(f + o + (long long)(k) * g.vstride + LBM_OUTER(vx, vy, vz), LBM_VL(vx, vy, vz), z, nL);
  LBM_FOR_EACH_V(LBM_PULL_PAIR)
#undef LBM_PULL_PAIR
}

__device__ __forceinline__ void collide_store_pairs(S* __restrict__ fnew, const Geo& g, const lbm::F2 (&prm)[kPrm],
                                                    int i0, int i1, int i2, lbm::F2 (&gv)[LBM_Q]) {
  const long long o = lbm::node_offset(g, i0, i1, i2);
  lbm_collide<lbm::F2>(gv, prm);
#pragma unroll
  for (int k = 0; k < LBM_Q; ++k) Pair<S>::store(fnew + o + (long long)k * g.vstride, gv[k].v);
}

__device__ __forceinline__ void step_pair(const S* __restrict__ f, S* __restrict__ fnew, const Geo& g,
                                          const lbm::F2 (&prm)[kPrm], int i0, int i1, int i2, int z, int nL) {
  lbm::F2 gv[LBM_Q];
  pull_pairs(f, g, i0, i1, i2, z, nL, gv);
  collide_store_pairs(fnew, g, prm, i0, i1, i2, gv);
}

// eight resident blocks of LBM_BLOCK threads per SM: 64 registers, no spills
// for the D3Q19 collide (BF16 storage +1.7 %, the FP16 cube's step +2.8 %;
// nine blocks spill and lose 8 %)
#ifndef LBM_PAIRS_MIN_BLOCKS
#define LBM_PAIRS_MIN_BLOCKS 8
#endif

// Bounded domains: the pull reads the ghost layer (refreshed and written by
// the boundary methods before the step), so the two sources of a pair need
// no wrap.  For z = 0 the word at p - 2 holds (z - 2, z - 1): z - 1 is the
// ghost, z - 2 the last element of the row before (in the buffer: every
// interior row follows a ghost plane).  For the last pair the word at p + 2
// holds (n, n + 1): n is the ghost, n + 1 lies in the row after.
__device__ __forceinline__ lbm::F2 pull_pair_ghost(const S* __restrict__ p, int vl) {
  const float2 w = Pair<S>::load(p);
  if (vl == 0) return lbm::F2(w.x, w.y);
  if (vl > 0) return lbm::F2(Pair<S>::load(p - 2).y, w.x);
  return lbm::F2(w.y, Pair<S>::load(p + 2).x);
}

#if LBM_DIM == 1
#define LBM_OUTER_GHOST(vx, vy, vz) 0LL
#elif LBM_DIM == 2
#define LBM_OUTER_GHOST(vx, vy, vz) (-(long long)(vx) * a.g.stride[0])
#else
#define LBM_OUTER_GHOST(vx, vy, vz) (-((long long)(vx) * a.g.stride[0] + (long long)(vy) * a.g.stride[1]))
#endif

__global__ void __launch_bounds__(LBM_BLOCK, LBM_PAIRS_MIN_BLOCKS) k_step_ghost_pairs(const S* __restrict__ f,
                                                                                    S* __restrict__ fnew,
                                                                                    StepArgs a) {
  const int z = 2 * (blockIdx.x * blockDim.x + threadIdx.x);
  const int nL = a.g.n[LBM_DIM - 1];
  if (z >= nL) return;
  int i0, i1, i2;
#if LBM_DIM == 1
  i0 = z + a.g.h[0];
  i1 = i2 = 0;
#elif LBM_DIM == 2
  i0 = blockIdx.y + a.g.h[0];
  i1 = z + a.g.h[1];
  i2 = 0;
#else
  i0 = blockIdx.z + a.g.h[0];
  i1 = blockIdx.y + a.g.h[1];
  i2 = z + a.g.h[2];
#endif
  lbm::F2 prm[kPrm];
#pragma unroll
  for (int p = 0; p < kPrm; ++p) prm[p] = lbm::F2((float)a.prm[p]);
  const long long o = lbm::node_offset(a.g, i0, i1, i2);
  lbm::F2 gv[LBM_Q];
#define LBM_PULL_GHOST(k, vx, vy, vz) \
  gv[k] = pull_pair_ghost(f + o + (long long)(k) * a.g.vstride + LBM_OUTER_GHOST(vx, vy, vz), LBM_VL(vx, vy, vz));
  LBM_FOR_EACH_V(LBM_PULL_GHOST)
#undef LBM_PULL_GHOST
  collide_store_pairs(fnew, a.g, prm, i0, i1, i2, gv);
}

// the box-wall fold for two nodes (z, z + 1) per thread (16-bit storage)
__global__ void __launch_bounds__(LBM_BLOCK, LBM_PAIRS_MIN_BLOCKS) k_step_walls_pairs(const S* __restrict__ f,
                                                                                     S* __restrict__ fnew,
                                                                                     StepArgs a, WallArgs w) {
  constexpr int L = LBM_DIM - 1;
  const int z = 2 * (blockIdx.x * blockDim.x + threadIdx.x);
  const int nL = a.g.n[L];
  if (z >= nL) return;
  int i0, i1, i2;
#if LBM_DIM == 1
  i0 = z + a.g.h[0];
  i1 = i2 = 0;
#elif LBM_DIM == 2
  i0 = blockIdx.y + a.g.h[0];
  i1 = z + a.g.h[1];
  i2 = 0;
#else
  i0 = blockIdx.z + a.g.h[0];
  i1 = blockIdx.y + a.g.h[1];
  i2 = z + a.g.h[2];
#endif
  lbm::F2 prm[kPrm];
#pragma unroll
  for (int p = 0; p < kPrm; ++p) prm[p] = lbm::F2((float)a.prm[p]);
  const long long o = lbm::node_offset(a.g, i0, i1, i2);
  // faces of the outer axes (shared by both nodes) and of the contiguous axis (per node)
  const bool lo0 = LBM_DIM > 1 && i0 == a.g.h[0], hi0 = LBM_DIM > 1 && i0 == a.g.h[0] + a.g.n[0] - 1;
  const bool lo1 = LBM_DIM > 2 && i1 == a.g.h[1], hi1 = LBM_DIM > 2 && i1 == a.g.h[1] + a.g.n[1] - 1;
  const bool first = z == 0, last = z + 2 == nL;
  lbm::F2 gv[LBM_Q];
  // wall signature 9 (o0+1) + 3 (o1+1) + (o2+1): the outer axes' part, and the
  // weight of the contiguous axis
#if LBM_DIM == 1
#define LBM_WALL_BASE(vx, vy, vz) 13
  constexpr int wL = 9;
#elif LBM_DIM == 2
#define LBM_WALL_BASE(vx, vy, vz) (9 * (wall_off(vx, lo0, hi0) + 1) + 4)
  constexpr int wL = 3;
#else
#define LBM_WALL_BASE(vx, vy, vz) (9 * (wall_off(vx, lo0, hi0) + 1) + 3 * (wall_off(vy, lo1, hi1) + 1) + 1)
  constexpr int wL = 1;
#endif
#define LBM_PULL_WALL_PAIR(k, vx, vy, vz)                                                             \
  {                                                                                                   \
    const int vl = LBM_VL(vx, vy, vz);                                                                \
    const int base = LBM_WALL_BASE(vx, vy, vz);                                                       \
    const int s0 = base + wL * wall_off(vl, first, false);                                            \
    const int s1 = base + wL * wall_off(vl, false, last);                                             \
    gv[k] = pull_pair_ghost(f + o + (long long)(k) * a.g.vstride + LBM_OUTER_GHOST(vx, vy, vz), vl); \
    if (s0 != 13 || s1 != 13) {                                                                       \
      const float2 bb = Pair<S>::load(f + o + (long long)w.sym[k] * a.g.vstride);                     \
      if (s0 != 13) gv[k].v.x = through_storage(bb.x + w.c[k][s0]);                                 \
      if (s1 != 13) gv[k].v.y = through_storage(bb.y + w.c[k][s1]);                                 \
    }                                                                                                 \
  }
  if (!(lo0 || hi0 || lo1 || hi1)) {
    // no wall normal to the outer axes (uniform over the row): the plain
    // two-node pull of the ghost kernel; at a row end the one value whose
    // source is the wall normal to the contiguous axis is replaced, so only
    // that thread's few loads diverge
#define LBM_PULL_GHOST_W(k, vx, vy, vz) \
  gv[k] = pull_pair_ghost(f + o + (long long)(k) * a.g.vstride + LBM_OUTER_GHOST(vx, vy, vz), LBM_VL(vx, vy, vz));
    LBM_FOR_EACH_V(LBM_PULL_GHOST_W)
#undef LBM_PULL_GHOST_W
    if (first || last) {
#define LBM_FIX_END_PAIR(k, vx, vy, vz)                                                       \
  {                                                                                           \
    const int vl = LBM_VL(vx, vy, vz);                                                        \
    if ((first && vl > 0) || (last && vl < 0)) {                                             \
      const float2 bb = Pair<S>::load(f + o + (long long)w.sym[k] * a.g.vstride);             \
      if (first && vl > 0) gv[k].v.x = through_storage(bb.x + w.c[k][13 - wL]);               \
      if (last && vl < 0) gv[k].v.y = through_storage(bb.y + w.c[k][13 + wL]);                \
    }                                                                                         \
  }
      LBM_FOR_EACH_V(LBM_FIX_END_PAIR)
#undef LBM_FIX_END_PAIR
    }
  } else {
    LBM_FOR_EACH_V(LBM_PULL_WALL_PAIR)
  }
#undef LBM_PULL_WALL_PAIR
#undef LBM_WALL_BASE
  collide_store_pairs(fnew, a.g, prm, i0, i1, i2, gv);
}

#ifndef LBM_ENSEMBLE_ROW_PAIRS
#define LBM_ENSEMBLE_ROW_PAIRS 1
#endif
__global__ void __launch_bounds__(LBM_BLOCK, LBM_PAIRS_MIN_BLOCKS) k_step_periodic_pairs(const S* __restrict__ f, S* __restrict__ fnew,
                                                                   StepArgs a) {
  constexpr int L = LBM_DIM - 1;
  const int z = 2 * (blockIdx.x * blockDim.x + threadIdx.x);
  const int nL = a.g.n[L];
  if (z >= nL) return;
  int i0, i1, i2;
#if LBM_DIM == 1
  i0 = z + a.g.h[0];
  i1 = i2 = 0;
#elif LBM_DIM == 2
  i0 = blockIdx.y + a.g.h[0];
  i1 = z + a.g.h[1];
  i2 = 0;
#else
  i0 = blockIdx.z + a.g.h[0];
  i1 = blockIdx.y + a.g.h[1];
  i2 = z + a.g.h[2];
#endif
  lbm::F2 prm[kPrm];
#pragma unroll
  for (int p = 0; p < kPrm; ++p) prm[p] = lbm::F2((float)a.prm[p]);
  step_pair(f, fnew, a.g, prm, i0, i1, i2, z, nL);
}

// ---------------------------------------------------------------------------
// Staged periodic step (16-bit storage, two nodes per thread).  A persistent
// block owns a sequence of interior rows (all axes but the contiguous one);
// for each row one producer thread issues Q bulk copies on the TMA unit --
// for population k, the interior row the pull reads (the row at x - v_k,
// wrapped periodically along the outer axes) -- into one of kStages shared
// buffers, completing on that stage's "full" mbarrier.  Four consumer warps
// wait on it, take each node's Q values from shared memory (the wrap along
// the contiguous axis is an index into the staged row), collide two nodes
// per thread and store them, then release the stage on its "empty" mbarrier.
// The copies of the next stages are in flight while a row is computed, with
// no registers held for them: the one-node-per-load kernels are limited by
// the loads a thread can keep in flight at the occupancy its registers allow.
// Every wait is bounded (lbm::mbar_wait); a timed-out wait is counted in
// lbm_wait_timeouts and the block leaves after its copies have landed.
constexpr int kStages = 4;
constexpr int kConsumers = 4;  // warps
constexpr int kStagedThreads = 32 * (1 + kConsumers);

__device__ __forceinline__ void staged_row_coords(const Geo& g, int r, int& i0, int& i1) {
#if LBM_DIM == 3
  i0 = r / g.n[1];
  i1 = r - i0 * g.n[1];
#else
  i0 = r;
  i1 = 0;
#endif
}

// interior coordinate c shifted by -v and wrapped into [0, n)
__device__ __forceinline__ int wrap_back(int c, int v, int n) {
  int j = c - v;
  return j < 0 ? j + n : (j >= n ? j - n : j);
}

// the two pulled values of nodes (z, z+1) from a staged row of nL values
__device__ __forceinline__ lbm::F2 staged_pair(const S* __restrict__ row, int vl, int z, int nL) {
  if (vl == 0) {
    const float2 w = Pair<S>::load(row + z);
    return lbm::F2(w.x, w.y);
  }
  const int a = wrap_back(z, vl, nL), b = wrap_back(z + 1, vl, nL);
  return lbm::F2(Pair<S>::one(row + a), Pair<S>::one(row + b));
}

__global__ void __launch_bounds__(kStagedThreads) k_step_periodic_staged(const S* __restrict__ f,
                                                                        S* __restrict__ fnew, StepArgs a) {
  constexpr int L = LBM_DIM - 1;
  extern __shared__ __align__(128) unsigned char staged_smem[];
  const Geo& g = a.g;
  const int nL = g.n[L];
  const int rows = LBM_DIM == 3 ? g.n[0] * g.n[1] : g.n[0];
  const uint32_t row_bytes = (uint32_t)nL * sizeof(S);
  S* buf = reinterpret_cast<S*>(staged_smem);
  uint64_t* full = reinterpret_cast<uint64_t*>(staged_smem + (size_t)kStages * LBM_Q * row_bytes);
  uint64_t* empty = full + kStages;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      lbm::mbar_init(&full[s], 1);
      lbm::mbar_init(&empty[s], kConsumers);
    }
    lbm::mbar_init_fence();
  }
  __syncthreads();
  if (warp == 0) {
    if (lane != 0) return;
    // producer: the Q source rows of every row this block owns
    int it = 0;
    bool ok = true;
    for (int r = blockIdx.x; r < rows; r += gridDim.x, ++it) {
      const int s = it % kStages;
      if (it >= kStages && !lbm::mbar_wait(&empty[s], ((it / kStages) - 1) & 1)) {
        ok = false;
        break;
      }
      lbm::mbar_expect_tx(&full[s], LBM_Q * row_bytes);
      int x0, x1;
      staged_row_coords(g, r, x0, x1);
#define LBM_STAGE_ROW(k, vx, vy, vz)                                                                  \
  {                                                                                                   \
    const int s0 = wrap_back(x0, LBM_DIM == 3 ? (vx) : (LBM_DIM == 2 ? (vx) : 0), g.n[0]) + g.h[0];   \
    const int s1 = LBM_DIM == 3 ? wrap_back(x1, (vy), g.n[1]) + g.h[1] : 0;                           \
    const S* src = f + (long long)(k) * g.vstride + lbm::node_offset(g, s0, s1, 0) + g.h[L];          \
    lbm::bulk_load(buf + ((size_t)s * LBM_Q + (k)) * nL, src, row_bytes, &full[s]);                   \
  }
      LBM_FOR_EACH_V(LBM_STAGE_ROW)
#undef LBM_STAGE_ROW
    }
    if (!ok) atomicAdd(&lbm_wait_timeouts, 1u);
    // the copies still in flight land before the block's shared memory goes away
    for (int j = it - 1; j >= 0 && j >= it - kStages; --j)
      if (!lbm::mbar_wait(&full[j % kStages], (j / kStages) & 1)) {
        atomicAdd(&lbm_wait_timeouts, 1u);
        break;
      }
    return;
  }
  // consumers
  lbm::F2 prm[kPrm];
#pragma unroll
  for (int p = 0; p < kPrm; ++p) prm[p] = lbm::F2((float)a.prm[p]);
  const int t = threadIdx.x - 32;
  int it = 0;
  for (int r = blockIdx.x; r < rows; r += gridDim.x, ++it) {
    const int s = it % kStages;
    if (!lbm::mbar_wait(&full[s], (it / kStages) & 1)) {
      if (lane == 0) atomicAdd(&lbm_wait_timeouts, 1u);
      break;
    }
    int x0, x1;
    staged_row_coords(g, r, x0, x1);
    const S* stage = buf + (size_t)s * LBM_Q * nL;
    for (int z = 2 * t; z < nL; z += 2 * 32 * kConsumers) {
      lbm::F2 gv[LBM_Q];
#define LBM_PULL_STAGED(k, vx, vy, vz) gv[k] = staged_pair(stage + (size_t)(k) * nL, LBM_VL(vx, vy, vz), z, nL);
      LBM_FOR_EACH_V(LBM_PULL_STAGED)
#undef LBM_PULL_STAGED
#if LBM_DIM == 3
      collide_store_pairs(fnew, g, prm, x0 + g.h[0], x1 + g.h[1], z + g.h[2], gv);
#else
      collide_store_pairs(fnew, g, prm, x0 + g.h[0], z + g.h[1], 0, gv);
#endif
    }
    __syncwarp();
    if (lane == 0) lbm::mbar_arrive(&empty[s]);
  }
}

#else
#define LBM_HAS_PAIRS 0
#endif

// halo coordinates of interior row r (all axes but the last) and column col
__device__ __forceinline__ void row_coords(const Geo& g, int r, int col, int (&idx)[3]) {
  constexpr int L = LBM_DIM - 1;
  idx[0] = idx[1] = idx[2] = 0;
  int q = r;
#pragma unroll
  for (int d = L - 1; d >= 1; --d) {
    idx[d] = q % g.n[d] + g.h[d];
    q /= g.n[d];
  }
  if (L >= 1) idx[0] = q + g.h[0];  // r < rows: the outermost index needs no modulo
  idx[L] = col + g.h[L];
}

__device__ __forceinline__ void step_node(const S* __restrict__ f, S* __restrict__ fnew, const Geo& g,
                                          const R (&prm)[kPrm], int i0, int i1, int i2) {
  const long long o = lbm::node_offset(g, i0, i1, i2);
  long long off0[2 * LBM_VMAX + 1], off1[2 * LBM_VMAX + 1], off2[2 * LBM_VMAX + 1];
#pragma unroll
  for (int s = -LBM_VMAX; s <= LBM_VMAX; ++s) {
    off0[s + LBM_VMAX] = LBM_DIM > 0 ? wrap_off(i0, s, g.n[0], g.h[0], g.stride[0]) : 0;
    off1[s + LBM_VMAX] = LBM_DIM > 1 ? wrap_off(i1, s, g.n[1], g.h[1], g.stride[1]) : 0;
    off2[s + LBM_VMAX] = LBM_DIM > 2 ? wrap_off(i2, s, g.n[2], g.h[2], g.stride[2]) : 0;
  }
  R gv[LBM_Q];
#define LBM_PULL_ENS(k, vx, vy, vz)                                                              \
  gv[k] = (R)Store<S>::load(f + o + (long long)(k) * g.vstride + off0[(vx) + LBM_VMAX] +        \
                            off1[(vy) + LBM_VMAX] + off2[(vz) + LBM_VMAX]);
  LBM_FOR_EACH_V(LBM_PULL_ENS)
#undef LBM_PULL_ENS
  R p[kPrm];
#pragma unroll
  for (int i = 0; i < kPrm; ++i) p[i] = prm[i];
  lbm_collide<R>(gv, p);
#pragma unroll
  for (int k = 0; k < LBM_Q; ++k) Store<S>::store(fnew + o + (long long)k * g.vstride, gv[k]);
}

// Ensemble step: blocks stride over a tile list that covers every instance;
// a tile is rows_per_tile rows x span nodes of the last axis of one instance
// (span = blockDim.x, or 2 blockDim.x for LBM_INSTANCE_PAIRS, where a thread
// updates two neighbouring nodes).  The per-node work is the periodic step
// above with the instance's own geometry and run-time parameters.
// kPairsOnly: every instance carries LBM_INSTANCE_PAIRS (the caller checks),
// so the kernel holds the two-node path alone (fewer registers).
template <bool kPairsOnly>
__global__ void __launch_bounds__(LBM_ENSEMBLE_MAX_BLOCK) k_step_ensemble(S* __restrict__ arena,
                                                                          const lbm_instance* __restrict__ inst,
                                                                          const int* __restrict__ tile_inst,
                                                                          int ntiles, int rows_per_tile, int parity) {
  constexpr int L = LBM_DIM - 1;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const lbm_instance* I = inst + tile_inst[tile];
    const int local = tile - I->tile_begin;
    const int rt = local / I->col_tiles;
    const int ct = local - rt * I->col_tiles;
    const bool two = (I->flags & LBM_INSTANCE_PAIRS) != 0;
    const int base = ct * (two ? 2 * (int)blockDim.x : (int)blockDim.x);
    const int nL = I->n[L];
    Geo g;
    g.dim = LBM_DIM;
    g.nv = LBM_Q;
    for (int d = 0; d < 3; ++d) {
      g.n[d] = I->n[d];
      g.h[d] = I->halo[d];
      g.stride[d] = I->stride[d];
    }
    g.vstride = I->vstride;
    g.origin = I->origin;
    const S* __restrict__ f = arena + I->offset[parity];
    S* __restrict__ fnew = arena + I->offset[parity ^ 1];
    const int r0 = rt * rows_per_tile;
    const int r1 = min(I->rows, r0 + rows_per_tile);
#if LBM_HAS_PAIRS
    bool aligned = two && nL % 2 == 0 && (g.origin + g.h[L]) % 2 == 0 && g.vstride % 2 == 0 &&
                   I->offset[0] % 2 == 0 && I->offset[1] % 2 == 0;
#pragma unroll
    for (int d = 0; d < L; ++d) aligned = aligned && g.stride[d] % 2 == 0;
    if (aligned) {
      const int z = base + 2 * (int)threadIdx.x;
      if (z >= nL) continue;
      lbm::F2 prm2[kPrm];
#pragma unroll
      for (int p = 0; p < kPrm; ++p) prm2[p] = lbm::F2((float)I->prm[p < LBM_MAX_PRM ? p : 0]);
      int r = r0;
#if LBM_ENSEMBLE_ROW_PAIRS
      // two rows at a time: both rows' loads are issued before either collide
      for (; r + 1 < r1; r += 2) {
        int a[3], b[3];
        row_coords(g, r, z, a);
        row_coords(g, r + 1, z, b);
        lbm::F2 ga[LBM_Q], gb[LBM_Q];
        pull_pairs(f, g, a[0], a[1], a[2], z, nL, ga);
        pull_pairs(f, g, b[0], b[1], b[2], z, nL, gb);
        collide_store_pairs(fnew, g, prm2, a[0], a[1], a[2], ga);
        collide_store_pairs(fnew, g, prm2, b[0], b[1], b[2], gb);
      }
#endif
      for (; r < r1; ++r) {
        int idx[3];
        row_coords(g, r, z, idx);
        step_pair(f, fnew, g, prm2, idx[0], idx[1], idx[2], z, nL);
      }
      continue;
    }
#endif
    if (kPairsOnly) continue;  // not reached: the caller checked every instance
    R prm[kPrm];
#pragma unroll
    for (int p = 0; p < kPrm; ++p) prm[p] = (R)I->prm[p < LBM_MAX_PRM ? p : 0];
    for (int c = 0; c < (two ? 2 : 1); ++c) {
      const int col = base + (int)threadIdx.x + c * (int)blockDim.x;
      if (col >= nL) break;
      for (int r = r0; r < r1; ++r) {
        int idx[3];
        row_coords(g, r, col, idx);
        step_node(f, fnew, g, prm, idx[0], idx[1], idx[2]);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Periodic step with the learned collision closure: after the relaxation the
// non-conserved moments receive the MLP's correction, computed from the
// node's pre-collision moments.  Each warp stages the normalised moments of
// its 32 nodes in shared memory and evaluates the MLP on the tensor cores as
// two 16-row tiles (lbm_mlp.cuh); conserved moments are never changed.
struct ClosureArgs {
  const __nv_bfloat16* w;  // BF16 weight block (forward part read)
  const float* params;     // FP32 parameter block (biases read)
  float mu_in[16], isig_in[16];
  float mu_out[8], sig_out[8];
  long long nodes;         // interior nodes
  // guard: a node whose corrections are not finite or exceed
  // ratio * (largest change the relaxation itself made) + floor keeps the
  // plain MRT collision and is counted (ratio <= 0: no guard)
  float guard_ratio, guard_floor;
  int* fallbacks;          // device counter of guarded nodes, or null
  // rate form (rate_form != 0): output j scales the relaxation's own change
  // of moment j, corr_j = lam_j (m_relaxed_j - m_j) with
  // lam_j = lam_lo[j] + (lam_hi[j] - lam_lo[j]) sigmoid(y_j sig_out[j] + mu_out[j]),
  // so the effective rate s_j (1 + lam_j) stays inside the caller's bounds
  int rate_form;
  float lam_lo[8], lam_hi[8];
};

// correction of non-conserved moment j from the network output y (bias
// included) and the relaxation's change d of that moment
__device__ __forceinline__ float closure_correction(const ClosureArgs& c, int j, float y, float d) {
  const float z = y * c.sig_out[j] + c.mu_out[j];
  if (!c.rate_form) return z;
  const float lam = c.lam_lo[j] + (c.lam_hi[j] - c.lam_lo[j]) / (1.0f + __expf(-z));
  return lam * d;
}

constexpr int kClosureWarps = 8;
// nodes per warp and pass: 32 (every lane pulls, relaxes and stores a node;
// the MLP runs as two 16-row tiles) or 16 (lanes 16..31 only join the MLP)
#ifndef LBM_CLOSURE_WARP_NODES
#define LBM_CLOSURE_WARP_NODES 32
#endif
constexpr int kClosureWarpNodes = LBM_CLOSURE_WARP_NODES;
static_assert(kClosureWarpNodes == 16 || kClosureWarpNodes == 32, "16 or 32 nodes per warp");
#ifndef LBM_CLOSURE_MIN_BLOCKS
// no register cap: capping at 64 or 80 registers spills and was slower
#define LBM_CLOSURE_MIN_BLOCKS 1
#endif

__global__ void __launch_bounds__(32 * kClosureWarps, LBM_CLOSURE_MIN_BLOCKS) k_step_periodic_closure(const S* __restrict__ f,
                                                                               S* __restrict__ fnew, StepArgs a,
                                                                               ClosureArgs c) {
#if LBM_Q <= 16 && (LBM_Q - LBM_NCONS) <= 8
  using namespace lbm_mlp;
  __shared__ __align__(16) __nv_bfloat16 w_s[BW2N];
  __shared__ __align__(16) float b_s[2 * H + OUT];
  __shared__ __align__(16) __nv_bfloat16 x_s[kClosureWarps][32 * IN];
  __shared__ float y_s[kClosureWarps][kClosureWarpNodes * OUT];
  static_assert((BW2N * sizeof(__nv_bfloat16)) % 16 == 0, "weight block must be a whole number of 16-byte words");
  static_assert(PB1 % 4 == 0 && PB2 % 4 == 0 && PB3 % 4 == 0 && H % 4 == 0 && OUT % 4 == 0, "16-byte bias chunks");
  // weights and biases reach shared memory by cp.async while the warps pull
  // their first nodes (both blocks 16-byte aligned, checked by the host);
  // the block waits for them just before its first MLP evaluation
  {
    const char* src = reinterpret_cast<const char*>(c.w);
    char* dst = reinterpret_cast<char*>(w_s);
    for (int i = threadIdx.x; i < (int)(BW2N * sizeof(__nv_bfloat16) / 16); i += blockDim.x)
      lbm::cp_async16(dst + 16 * i, src + 16 * i);
    char* bd = reinterpret_cast<char*>(b_s);
    for (int i = threadIdx.x; i < (2 * H + OUT) / 4; i += blockDim.x) {
      const float* bs = i < H / 4 ? c.params + PB1 + 4 * i
                        : i < H / 2 ? c.params + PB2 + 4 * (i - H / 4)
                                    : c.params + PB3 + 4 * (i - H / 2);
      lbm::cp_async16(bd + 16 * i, bs);
    }
    lbm::cp_async_commit();
  }
  bool staged = false;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int gq = lane >> 2, tq = lane & 3;
  const Geo& g = a.g;
  // kClosureWarpNodes nodes per warp: lane l owns node l of the warp's run
  // (l < kClosureWarpNodes); all 32 lanes evaluate the MLP, one 16-row MMA
  // tile after the other
  const long long per_block = kClosureWarpNodes * kClosureWarps;
  for (long long base = (long long)blockIdx.x * per_block; base < c.nodes; base += (long long)gridDim.x * per_block) {
    const long long node = base + warp * kClosureWarpNodes + lane;
    const bool active = lane < kClosureWarpNodes && node < c.nodes;
    int idx[3] = {0, 0, 0};
    long long q = active ? node : 0;
    for (int d = LBM_DIM - 1; d >= 0; --d) {
      idx[d] = (int)(q % g.n[d]) + g.h[d];
      q /= g.n[d];
    }
    const long long o = lbm::node_offset(g, idx[0], idx[1], idx[2]);
    R gv[LBM_Q], m[LBM_Q];
    if (active) {
      long long off0[2 * LBM_VMAX + 1], off1[2 * LBM_VMAX + 1], off2[2 * LBM_VMAX + 1];
#pragma unroll
      for (int s = -LBM_VMAX; s <= LBM_VMAX; ++s) {
        off0[s + LBM_VMAX] = LBM_DIM > 0 ? wrap_off(idx[0], s, g.n[0], g.h[0], g.stride[0]) : 0;
        off1[s + LBM_VMAX] = LBM_DIM > 1 ? wrap_off(idx[1], s, g.n[1], g.h[1], g.stride[1]) : 0;
        off2[s + LBM_VMAX] = LBM_DIM > 2 ? wrap_off(idx[2], s, g.n[2], g.h[2], g.stride[2]) : 0;
      }
#define LBM_PULL_CL(k, vx, vy, vz)                                                              \
  gv[k] = (R)Store<S>::load(f + o + (long long)(k) * g.vstride + off0[(vx) + LBM_VMAX] +        \
                            off1[(vy) + LBM_VMAX] + off2[(vz) + LBM_VMAX]);
      LBM_FOR_EACH_V(LBM_PULL_CL)
#undef LBM_PULL_CL
      lbm_moments<R>(gv, m);
    } else {
#pragma unroll
      for (int k = 0; k < LBM_Q; ++k) m[k] = (R)0;
    }
    // normalised pre-collision moments (absolute values) -> BF16 row of this lane
    if (lane < kClosureWarpNodes) {
      __nv_bfloat16* xr = &x_s[warp][lane * IN];
#pragma unroll
      for (int k = 0; k < IN; ++k) {
        float v = 0.0f;
        if (k < LBM_Q && active)
          v = ((float)m[k] + (float)lbm_dev_mref[k < LBM_Q ? k : 0] - c.mu_in[k]) * c.isig_in[k];
        xr[k] = __float2bfloat16_rn(v);
      }
    }
    if (!staged) {  // every block runs the same passes: a block-wide wait
      lbm::cp_async_wait_all();
      __syncthreads();
      staged = true;
    } else {
      __syncwarp();
    }
#pragma unroll 1
    for (int t = 0; t < kClosureWarpNodes / 16; ++t) {
      const __nv_bfloat16* xt = &x_s[warp][t * 16 * IN];
      uint32_t xa[4];
      xa[0] = *reinterpret_cast<const uint32_t*>(xt + gq * IN + 2 * tq);
      xa[1] = *reinterpret_cast<const uint32_t*>(xt + (gq + 8) * IN + 2 * tq);
      xa[2] = *reinterpret_cast<const uint32_t*>(xt + gq * IN + 8 + 2 * tq);
      xa[3] = *reinterpret_cast<const uint32_t*>(xt + (gq + 8) * IN + 8 + 2 * tq);
      float y[4], z1[8][4], z2[8][4];
      uint32_t h1a[4][4], h2a[4][4];
      forward_tile<false>(xa, w_s, b_s, b_s + H, b_s + 2 * H, lane, y, z1, z2, h1a, h2a);
      float* yt = &y_s[warp][t * 16 * OUT];
      yt[gq * OUT + 2 * tq] = y[0];
      yt[gq * OUT + 2 * tq + 1] = y[1];
      yt[(gq + 8) * OUT + 2 * tq] = y[2];
      yt[(gq + 8) * OUT + 2 * tq + 1] = y[3];
    }
    __syncwarp();
    if (active) {
      R pre[LBM_Q - LBM_NCONS];
#pragma unroll
      for (int j = 0; j < LBM_Q - LBM_NCONS; ++j) pre[j] = m[LBM_NCONS + j];
      lbm_relax<R>(m, a.prm);
      float corr[LBM_Q - LBM_NCONS];
      float change = 0.0f;
#pragma unroll
      for (int j = 0; j < LBM_Q - LBM_NCONS; ++j) {
        const float d = (float)(m[LBM_NCONS + j] - pre[j]);
        corr[j] = closure_correction(c, j, y_s[warp][lane * OUT + j], d);
        change = fmaxf(change, fabsf(d));
      }
      bool ok = true;
      if (c.guard_ratio > 0.0f) {
        const float limit = c.guard_ratio * change + c.guard_floor;
#pragma unroll
        for (int j = 0; j < LBM_Q - LBM_NCONS; ++j) ok = ok && fabsf(corr[j]) <= limit;  // false for NaN
      }
      if (ok) {
#pragma unroll
        for (int j = 0; j < LBM_Q - LBM_NCONS; ++j) m[LBM_NCONS + j] += (R)corr[j];
      } else if (c.fallbacks) {
        atomicAdd(c.fallbacks, 1);
      }
      lbm_populations<R>(m, gv);
#pragma unroll
      for (int k = 0; k < LBM_Q; ++k) Store<S>::store(fnew + o + (long long)k * g.vstride, gv[k]);
    }
    __syncwarp();
  }
  if (!staged) lbm::cp_async_wait_all();  // a block without nodes
#endif
}

// ---------------------------------------------------------------------------
// The closure step on the 5th-generation tensor cores.  A block of 128
// threads takes 128 consecutive interior nodes per tile, one node per
// thread: each thread pulls its node and computes its moments, the block's
// normalised moments form the 128 x 16 A operand of the MLP's first layer in
// shared memory, one thread issues the three layers' tcgen05 MMAs (FP32
// accumulators in tensor memory, lbm_tc.cuh), each warp reads back its 32
// rows, and every thread relaxes its node, adds the correction (with the
// same guard as k_step_periodic_closure) and stores it.  Weights come from
// the FP32 master block rounded to BF16 (the values of the warp kernel's
// fragment copy); only the FP32 accumulation order inside a layer differs.
#if LBM_Q <= 16 && (LBM_Q - LBM_NCONS) <= 8
constexpr int kTcRows = 128;
constexpr uint32_t kTcCols = 64;  // the three layers reuse columns 0..63
struct ClosureTcSmem {
  __nv_bfloat16 w1[lbm_mlp::H * lbm_mlp::IN];
  __nv_bfloat16 w2[lbm_mlp::H * lbm_mlp::H];
  __nv_bfloat16 w3[16 * lbm_mlp::H];
  __nv_bfloat16 x[kTcRows * lbm_mlp::IN];
  __nv_bfloat16 h[kTcRows * lbm_mlp::H];
  float b1[lbm_mlp::H], b2[lbm_mlp::H], b3[lbm_mlp::OUT];
  uint64_t bar;
  uint32_t tmem_base;
};

__global__ void __launch_bounds__(kTcRows) k_step_periodic_closure_tc(const S* __restrict__ f, S* __restrict__ fnew,
                                                                     StepArgs a, ClosureArgs c) {
  using namespace lbm_mlp;
  using namespace lbm_tc;
  __shared__ __align__(128) ClosureTcSmem sm;
  const int tid = threadIdx.x, warp = tid >> 5;
  unsigned char* w1b = reinterpret_cast<unsigned char*>(sm.w1);
  unsigned char* w2b = reinterpret_cast<unsigned char*>(sm.w2);
  unsigned char* w3b = reinterpret_cast<unsigned char*>(sm.w3);
  unsigned char* xb = reinterpret_cast<unsigned char*>(sm.x);
  unsigned char* hb = reinterpret_cast<unsigned char*>(sm.h);
  stage_bf16(w1b, c.params + PW1, H, H, IN, tid, kTcRows);
  stage_bf16(w2b, c.params + PW2, H, H, H, tid, kTcRows);
  stage_bf16(w3b, c.params + PW3, 16, OUT, H, tid, kTcRows);
  for (int i = tid; i < H; i += kTcRows) {
    sm.b1[i] = c.params[PB1 + i];
    sm.b2[i] = c.params[PB2 + i];
  }
  for (int i = tid; i < OUT; i += kTcRows) sm.b3[i] = c.params[PB3 + i];
  if (tid == 0) {
    lbm::mbar_init(&sm.bar, 1);
    lbm::mbar_init_fence();
  }
  if (warp == 0) tmem_alloc(&sm.tmem_base, kTcCols);
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tmem = sm.tmem_base;
  const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
  const uint32_t xa = lbm::smem_addr(sm.x), ha = lbm::smem_addr(sm.h);
  const uint32_t w1a = lbm::smem_addr(sm.w1), w2a = lbm::smem_addr(sm.w2), w3a = lbm::smem_addr(sm.w3);
  const Geo& g = a.g;
  uint32_t phase = 0;
  bool ok = true;
  const long long tiles = (c.nodes + kTcRows - 1) / kTcRows;
  for (long long tile = blockIdx.x; tile < tiles && ok; tile += gridDim.x) {
    const long long node = tile * kTcRows + tid;
    const bool active = node < c.nodes;
    int idx[3] = {0, 0, 0};
    long long q = active ? node : 0;
    for (int d = LBM_DIM - 1; d >= 0; --d) {
      idx[d] = (int)(q % g.n[d]) + g.h[d];
      q /= g.n[d];
    }
    const long long o = lbm::node_offset(g, idx[0], idx[1], idx[2]);
    R gv[LBM_Q], m[LBM_Q];
    if (active) {
      long long off0[2 * LBM_VMAX + 1], off1[2 * LBM_VMAX + 1], off2[2 * LBM_VMAX + 1];
#pragma unroll
      for (int s = -LBM_VMAX; s <= LBM_VMAX; ++s) {
        off0[s + LBM_VMAX] = LBM_DIM > 0 ? wrap_off(idx[0], s, g.n[0], g.h[0], g.stride[0]) : 0;
        off1[s + LBM_VMAX] = LBM_DIM > 1 ? wrap_off(idx[1], s, g.n[1], g.h[1], g.stride[1]) : 0;
        off2[s + LBM_VMAX] = LBM_DIM > 2 ? wrap_off(idx[2], s, g.n[2], g.h[2], g.stride[2]) : 0;
      }
#define LBM_PULL_TC(k, vx, vy, vz)                                                              \
  gv[k] = (R)Store<S>::load(f + o + (long long)(k) * g.vstride + off0[(vx) + LBM_VMAX] +        \
                            off1[(vy) + LBM_VMAX] + off2[(vz) + LBM_VMAX]);
      LBM_FOR_EACH_V(LBM_PULL_TC)
#undef LBM_PULL_TC
      lbm_moments<R>(gv, m);
    } else {
#pragma unroll
      for (int k = 0; k < LBM_Q; ++k) m[k] = (R)0;
    }
    // this node's normalised pre-collision moments: row tid of the A operand
    {
      float v[IN];
#pragma unroll
      for (int k = 0; k < IN; ++k) {
        v[k] = 0.0f;
        if (k < LBM_Q && active)
          v[k] = ((float)m[k < LBM_Q ? k : 0] + (float)lbm_dev_mref[k < LBM_Q ? k : 0] - c.mu_in[k]) * c.isig_in[k];
      }
      store8_bf16(xb, core_offset(tid, 0, IN), v);
      store8_bf16(xb, core_offset(tid, 8, IN), v + 8);
    }
    fence_async_smem();
    fence_before_sync();
    __syncthreads();
    if (tid == 0) {
      fence_after_sync();
      mma_bf16(tmem, smem_desc(xa, 128, (IN / 8) * 128), smem_desc(w1a, 128, (IN / 8) * 128),
               instr_desc(kTcRows, H), 0);
      mma_commit(&sm.bar);
    }
    if (!(ok = wait_mma(&sm.bar, phase))) break;
    fence_after_sync();
    epilogue_bf16<H>(tmem + lane_base, sm.b1, hb, tid, Silu());
    fence_async_smem();
    fence_before_sync();
    __syncthreads();
    if (tid == 0) {
      fence_after_sync();
#pragma unroll
      for (int kc = 0; kc < H / 16; ++kc)
        mma_bf16(tmem, smem_desc(ha + kc * 256, 128, (H / 8) * 128),
                 smem_desc(w2a + kc * 256, 128, (H / 8) * 128), instr_desc(kTcRows, H), kc > 0);
      mma_commit(&sm.bar);
    }
    if (!(ok = wait_mma(&sm.bar, phase))) break;
    fence_after_sync();
    epilogue_bf16<H>(tmem + lane_base, sm.b2, hb, tid, Silu());
    fence_async_smem();
    fence_before_sync();
    __syncthreads();
    if (tid == 0) {
      fence_after_sync();
#pragma unroll
      for (int kc = 0; kc < H / 16; ++kc)
        mma_bf16(tmem, smem_desc(ha + kc * 256, 128, (H / 8) * 128), smem_desc(w3a + kc * 256, 128, (H / 8) * 128),
                 instr_desc(kTcRows, 16), kc > 0);
      mma_commit(&sm.bar);
    }
    if (!(ok = wait_mma(&sm.bar, phase))) break;
    fence_after_sync();
    float y[16];
    tmem_ld16(tmem + lane_base, y);
    if (active) {
      R pre[LBM_Q - LBM_NCONS];
#pragma unroll
      for (int j = 0; j < LBM_Q - LBM_NCONS; ++j) pre[j] = m[LBM_NCONS + j];
      lbm_relax<R>(m, a.prm);
      float corr[LBM_Q - LBM_NCONS];
      float change = 0.0f;
#pragma unroll
      for (int j = 0; j < LBM_Q - LBM_NCONS; ++j) {
        const float d = (float)(m[LBM_NCONS + j] - pre[j]);
        corr[j] = closure_correction(c, j, y[j] + sm.b3[j], d);
        change = fmaxf(change, fabsf(d));
      }
      bool keep = true;
      if (c.guard_ratio > 0.0f) {
        const float limit = c.guard_ratio * change + c.guard_floor;
#pragma unroll
        for (int j = 0; j < LBM_Q - LBM_NCONS; ++j) keep = keep && fabsf(corr[j]) <= limit;  // false for NaN
      }
      if (keep) {
#pragma unroll
        for (int j = 0; j < LBM_Q - LBM_NCONS; ++j) m[LBM_NCONS + j] += (R)corr[j];
      } else if (c.fallbacks) {
        atomicAdd(c.fallbacks, 1);
      }
      lbm_populations<R>(m, gv);
#pragma unroll
      for (int k = 0; k < LBM_Q; ++k) Store<S>::store(fnew + o + (long long)k * g.vstride, gv[k]);
    }
    fence_before_sync();
    __syncthreads();
  }
  if (!ok && tid == 0) atomicAdd(&lbm_wait_timeouts, 1u);
  fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    fence_after_sync();
    tmem_dealloc(tmem, kTcCols);
  }
}
#endif

__global__ void __launch_bounds__(LBM_BLOCK) k_transport(const S* __restrict__ f, S* __restrict__ fnew,
                                                         StepArgs a) {
  int i0, i1, i2;
  if (!my_node(a.g, i0, i1, i2)) return;
  const long long o = lbm::node_offset(a.g, i0, i1, i2);
#pragma unroll
  for (int k = 0; k < LBM_Q; ++k) fnew[o + (long long)k * a.g.vstride] = f[o + a.pull[k]];
}

// Arithmetic of the moment transforms.  Shifted storage holds deviations
// g = f - feq(c0), whose moments M g are small: they are computed in the
// module's FP32 arithmetic (the step kernel's own algebra) and the FP64
// moments of the shift, mref = M feq(c0), are added once per moment, so the
// float64 moment array costs one conversion and one add per written moment
// instead of FP64 algebra per node (GB300's FP64 rate is a small fraction of
// its FP32 rate).  Unshifted storage keeps the whole transform in FP64.
#if LBM_SHIFTED
using RM = R;
#else
using RM = double;
#endif

__global__ void __launch_bounds__(LBM_BLOCK) k_f2m(const S* __restrict__ f, double* __restrict__ m,
                                                   MomentArgs a) {
  int i0, i1, i2;
  if (!my_cell(a.g, i0, i1, i2)) return;
  const long long o = lbm::node_offset(a.g, i0, i1, i2);
  const long long om = lbm::node_offset(a.gm, i0, i1, i2);
  RM g[LBM_Q], mm[LBM_Q];
#pragma unroll
  for (int k = 0; k < LBM_Q; ++k) g[k] = (RM)Store<S>::load(f + o + (long long)k * a.g.vstride);
  lbm_moments<RM>(g, mm);
#pragma unroll
  for (int k = 0; k < LBM_Q; ++k) m[om + (long long)k * a.gm.vstride] = (double)mm[k] + lbm_dev_mref[k];
}

// the conserved moments alone (what output and conservation checks read): the
// compiler drops the algebra of the other moments
__global__ void __launch_bounds__(LBM_BLOCK) k_f2m_conserved(const S* __restrict__ f, double* __restrict__ m,
                                                             MomentArgs a) {
  int i0, i1, i2;
  if (!my_cell(a.g, i0, i1, i2)) return;
  const long long o = lbm::node_offset(a.g, i0, i1, i2);
  const long long om = lbm::node_offset(a.gm, i0, i1, i2);
  RM g[LBM_Q], mm[LBM_Q];
#pragma unroll
  for (int k = 0; k < LBM_Q; ++k) g[k] = (RM)Store<S>::load(f + o + (long long)k * a.g.vstride);
  lbm_moments<RM>(g, mm);
#pragma unroll
  for (int k = 0; k < LBM_NCONS; ++k) m[om + (long long)k * a.gm.vstride] = (double)mm[k] + lbm_dev_mref[k];
}

// the conserved moments of the interior nodes straight into a dense array
// out[c][i0][i1][i2] (last axis fastest): what output reads, in one pass
__global__ void __launch_bounds__(LBM_BLOCK) k_f2m_conserved_dense(const S* __restrict__ f, double* __restrict__ out,
                                                                   MomentArgs a) {
  int i0, i1, i2;
  if (!my_node(a.g, i0, i1, i2)) return;
  const long long o = lbm::node_offset(a.g, i0, i1, i2);
  RM g[LBM_Q], mm[LBM_Q];
#pragma unroll
  for (int k = 0; k < LBM_Q; ++k) g[k] = (RM)Store<S>::load(f + o + (long long)k * a.g.vstride);
  lbm_moments<RM>(g, mm);
  const long long plane = (long long)a.g.n[0] * a.g.n[1] * a.g.n[2];
  const long long at = ((long long)(i0 - a.g.h[0]) * a.g.n[1] + (i1 - a.g.h[1])) * a.g.n[2] + (i2 - a.g.h[2]);
#pragma unroll
  for (int c = 0; c < LBM_NCONS; ++c) out[c * plane + at] = (double)mm[c] + lbm_dev_mref[c];
}

__global__ void __launch_bounds__(LBM_BLOCK) k_m2f(const double* __restrict__ m, S* __restrict__ f,
                                                   MomentArgs a) {
  int i0, i1, i2;
  if (!my_cell(a.g, i0, i1, i2)) return;
  const long long o = lbm::node_offset(a.g, i0, i1, i2);
  const long long om = lbm::node_offset(a.gm, i0, i1, i2);
  RM mm[LBM_Q], g[LBM_Q];
  // M^-1 (m - mref) = f - shift: the stored deviations directly
#pragma unroll
  for (int k = 0; k < LBM_Q; ++k) mm[k] = (RM)(m[om + (long long)k * a.gm.vstride] - lbm_dev_mref[k]);
  lbm_populations<RM>(mm, g);
#pragma unroll
  for (int k = 0; k < LBM_Q; ++k) Store<S>::store(f + o + (long long)k * a.g.vstride, (R)g[k]);
}

// pylbm's initialisation from the conserved moments (equilibrium, then m2f)
// in one pass over the halo box: planes 0..nconsm-1 of m are read, the
// populations written, the other planes of m neither read nor written.
// Shifted storage computes the equilibrium of the deviations in the module's
// FP32 arithmetic (one FP64 subtraction per conserved moment); unshifted
// storage runs exactly the operations of k_equilibrium followed by k_m2f.
__global__ void __launch_bounds__(LBM_BLOCK) k_init_conserved(const double* __restrict__ m, S* __restrict__ f,
                                                              MomentArgs a) {
  int i0, i1, i2;
  if (!my_cell(a.g, i0, i1, i2)) return;
  const long long o = lbm::node_offset(a.g, i0, i1, i2);
  const long long om = lbm::node_offset(a.gm, i0, i1, i2);
  RM mm[LBM_Q], g[LBM_Q];
#pragma unroll
  for (int k = 0; k < LBM_Q; ++k) mm[k] = (RM)0;
#if LBM_SHIFTED
  RM prm[kPrm];
#pragma unroll
  for (int p = 0; p < kPrm; ++p) prm[p] = (RM)a.prm[p];
#pragma unroll
  for (int c = 0; c < LBM_NCONS; ++c) mm[c] = (RM)(m[om + (long long)c * a.gm.vstride] - lbm_dev_mref[c]);
  lbm_equilibrium_dev<RM>(mm, prm);
#else
#pragma unroll
  for (int c = 0; c < LBM_NCONS; ++c) mm[c] = m[om + (long long)c * a.gm.vstride];
  lbm_equilibrium_abs<double>(mm, a.prm);
#pragma unroll
  for (int k = 0; k < LBM_Q; ++k) mm[k] = (RM)(mm[k] - lbm_dev_mref[k]);
#endif
  lbm_populations<RM>(mm, g);
#pragma unroll
  for (int k = 0; k < LBM_Q; ++k) Store<S>::store(f + o + (long long)k * a.g.vstride, (R)g[k]);
}

__global__ void __launch_bounds__(LBM_BLOCK) k_equilibrium(double* __restrict__ m, MomentArgs a) {
  int i0, i1, i2;
  if (!my_cell(a.gm, i0, i1, i2)) return;
  const long long om = lbm::node_offset(a.gm, i0, i1, i2);
  double mm[LBM_Q];
#pragma unroll
  for (int k = 0; k < LBM_Q; ++k) mm[k] = m[om + (long long)k * a.gm.vstride];
  lbm_equilibrium_abs<double>(mm, a.prm);
#pragma unroll
  for (int k = LBM_NCONS; k < LBM_Q; ++k) m[om + (long long)k * a.gm.vstride] = mm[k];
}

__global__ void __launch_bounds__(LBM_BLOCK) k_relaxation(double* __restrict__ m, MomentArgs a) {
  int i0, i1, i2;
  if (!my_cell(a.gm, i0, i1, i2)) return;
  const long long om = lbm::node_offset(a.gm, i0, i1, i2);
  double mm[LBM_Q];
#pragma unroll
  for (int k = 0; k < LBM_Q; ++k) mm[k] = m[om + (long long)k * a.gm.vstride];
  lbm_relax_abs<double>(mm, a.prm);
#pragma unroll
  for (int k = LBM_NCONS; k < LBM_Q; ++k) m[om + (long long)k * a.gm.vstride] = mm[k];
}

// pylbm's standalone source_term: the conserved moments of the interior
// nodes advance over half a time step by explicit Euler
__global__ void __launch_bounds__(LBM_BLOCK) k_source_term(double* __restrict__ m, MomentArgs a) {
  int i0, i1, i2;
  if (!my_node(a.gm, i0, i1, i2)) return;
  const long long om = lbm::node_offset(a.gm, i0, i1, i2);
  double mm[LBM_Q];
#pragma unroll
  for (int k = 0; k < LBM_Q; ++k) mm[k] = m[om + (long long)k * a.gm.vstride];
  lbm_source_half<double>(mm, a.prm);
#pragma unroll
  for (int k = 0; k < LBM_NCONS; ++k) m[om + (long long)k * a.gm.vstride] = mm[k];
}

// ------------------------------------------------------------------ host
// need_halo: the stencil reach in ghost layers, for the kernels that pull
// neighbours; the pointwise transforms (f2m, m2f) take any halo, including
// none (pylbm evaluates its boundary equilibria on such arrays).
inline int check_pop_lattice(const lbm_lattice* lat, const char* who, bool need_halo = true) {
  int rc = lbm::check_lattice(lat, who);
  if (rc) return rc;
  if (lat->dim != LBM_DIM || lat->nv != LBM_Q)
    return lbm::fail(LBM_ERR_ARG, "%s: lattice dim=%d nv=%d, scheme has dim=%d nv=%d", who, lat->dim,
                     lat->nv, LBM_DIM, LBM_Q);
  if (lat->dtype != Store<S>::code)
    return lbm::fail(LBM_ERR_ARG, "%s: lattice dtype %d, module stores %d", who, lat->dtype, Store<S>::code);
  for (int d = 0; d < LBM_DIM && need_halo; ++d)
    if (lat->halo[d] < LBM_VMAX)
      return lbm::fail(LBM_ERR_ARG, "%s: halo[%d]=%d below the stencil reach %d", who, d, lat->halo[d], LBM_VMAX);
  return LBM_OK;
}

inline int check_moment_lattice(const lbm_lattice* lat, const lbm_lattice* mlat, const char* who) {
  int rc = lbm::check_lattice(mlat, who);
  if (rc) return rc;
  if (mlat->dtype != LBM_F64) return lbm::fail(LBM_ERR_ARG, "%s: moments must be float64", who);
  if (mlat->dim != LBM_DIM || mlat->nv != LBM_Q) return lbm::fail(LBM_ERR_ARG, "%s: moment lattice shape", who);
  if (lat) {
    for (int d = 0; d < 3; ++d)
      if (lat->n[d] != mlat->n[d] || lat->halo[d] != mlat->halo[d])
        return lbm::fail(LBM_ERR_ARG, "%s: moment and population lattices differ on axis %d", who, d);
  }
  return LBM_OK;
}

inline dim3 node_grid(const lbm_lattice& l, bool with_halo) {
  const int L = LBM_DIM - 1;
  const int e = with_halo ? 2 : 0;
  unsigned gx = (unsigned)((l.n[L] + e * l.halo[L] + LBM_BLOCK - 1) / LBM_BLOCK);
  unsigned gy = 1, gz = 1;
#if LBM_DIM == 2
  gy = (unsigned)(l.n[0] + e * l.halo[0]);
#elif LBM_DIM == 3
  gy = (unsigned)(l.n[1] + e * l.halo[1]);
  gz = (unsigned)(l.n[0] + e * l.halo[0]);
#endif
  return dim3(gx, gy, gz);
}

// Two-node words need an even row length and every pair (z, z+1), z even, on a
// 4-byte boundary: even element offsets of the row start, strides and planes.
inline bool pairs_fit(const lbm_lattice& l, const void* f, const void* fnew) {
  const int L = LBM_DIM - 1;
  if (l.n[L] % 2 || (l.origin + l.halo[L]) % 2 || l.vstride % 2) return false;
  for (int d = 0; d < L; ++d)
    if (l.stride[d] % 2) return false;
  return ((uintptr_t)f % 4 == 0) && ((uintptr_t)fnew % 4 == 0);
}

#if LBM_HAS_PAIRS
// the staged step applies: 2D or 3D rows whose bytes and starts suit bulk copies
inline bool staged_fits(const lbm_lattice& l, const void* f, const void* fnew) {
  const int L = LBM_DIM - 1;
  if (LBM_DIM < 2 || !pairs_fit(l, f, fnew)) return false;
  const long long es = (long long)sizeof(S);
  if ((l.n[L] * es) % 16 || l.n[L] > 1024) return false;  // row bytes: multiple of 16, stage within shared memory
  if (((l.origin + l.halo[L]) * es) % 16 || (l.vstride * es) % 16) return false;
  for (int d = 0; d < L; ++d)
    if ((l.stride[d] * es) % 16) return false;
  return ((uintptr_t)f % 16 == 0);
}

inline size_t staged_smem_bytes(const lbm_lattice& l) {
  return (size_t)kStages * LBM_Q * l.n[LBM_DIM - 1] * sizeof(S) + 2 * kStages * sizeof(uint64_t);
}
#endif

inline StepArgs make_step_args(const lbm_lattice& l, const double* prm) {
  StepArgs a;
  a.g = lbm::make_geo(l);
#define LBM_PULL_OFF(k, vx, vy, vz) \
  a.pull[k] = (long long)(k) * l.vstride - ((long long)(vx) * l.stride[0] + (long long)(vy) * l.stride[1] + (long long)(vz) * l.stride[2]);
  LBM_FOR_EACH_V(LBM_PULL_OFF)
#undef LBM_PULL_OFF
  for (int i = 0; i < kPrm; ++i) a.prm[i] = (i < LBM_NPRM && prm) ? (R)prm[i] : (R)0;
  return a;
}

}  // namespace lbm_scheme

extern "C" {

const char* lbm_scheme_last_error(void) { return lbm::error_slot().msg; }

int lbm_scheme_describe(int32_t* nv, int32_t* dim, int32_t* nprm, int32_t* storage, int32_t* compute,
                        double* shift, double* mref) {
  if (nv) *nv = LBM_Q;
  if (dim) *dim = LBM_DIM;
  if (nprm) *nprm = LBM_NPRM;
  if (storage) *storage = lbm::Store<lbm_scheme::S>::code;
  if (compute) *compute = std::is_same<lbm_scheme::R, double>::value ? LBM_F64 : LBM_F32;
  for (int k = 0; k < LBM_Q; ++k) {
    if (shift) shift[k] = lbm_host_shift[k];
    if (mref) mref[k] = lbm_host_mref[k];
  }
  return LBM_OK;
}

// 0 (default): the direct-load kernels; 1: periodic 16-bit steps use the
// staged kernel where the rows fit
static int g_step_variant = 0;

#if LBM_Q <= 16 && (LBM_Q - LBM_NCONS) <= 8
// blocks per SM of the tensor-core closure step: 0 = the resource bound
// below, else a fixed count; always within the 512 / kTcCols tensor-memory
// allocations an SM can hold at once, so no allocation waits on another
// block.  The bound comes from the kernel's registers and shared memory and
// the SM's limits (the runtime's occupancy query answers 1 block per SM for
// this kernel although several run side by side).
static int g_closure_tc_occupancy = 0;

static int closure_tc_blocks_per_sm(int dev, int* used, int* bound_out) {
  static int cache[64];  // the resource bound per device ordinal, 0 until computed
  int bound = dev >= 0 && dev < 64 ? cache[dev] : 0;
  if (bound == 0) {
    const char* who = "closure_tc_blocks_per_sm";
    cudaFuncAttributes fa;
    int regs = 0, smem = 0, reserved = 0, threads = 0;
    int rc = lbm::cuda_check(cudaFuncGetAttributes(&fa, lbm_scheme::k_step_periodic_closure_tc), who);
    if (!rc) rc = lbm::cuda_check(cudaDeviceGetAttribute(&regs, cudaDevAttrMaxRegistersPerMultiprocessor, dev), who);
    if (!rc)
      rc = lbm::cuda_check(cudaDeviceGetAttribute(&smem, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev), who);
    if (!rc) rc = lbm::cuda_check(cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev), who);
    if (!rc)
      rc = lbm::cuda_check(cudaDeviceGetAttribute(&threads, cudaDevAttrMaxThreadsPerMultiProcessor, dev), who);
    if (rc) return rc;
    const int rows = lbm_scheme::kTcRows;
    const int regs_block = ((fa.numRegs + 7) / 8) * 8 * rows;  // registers are allocated 256 per warp
    bound = (int)(512 / lbm_scheme::kTcCols);
    if (regs_block > 0 && regs / regs_block < bound) bound = regs / regs_block;
    if (smem / (int)(fa.sharedSizeBytes + reserved) < bound) bound = smem / (int)(fa.sharedSizeBytes + reserved);
    if (threads / rows < bound) bound = threads / rows;
    if (bound < 1) bound = 1;
    if (dev >= 0 && dev < 64) cache[dev] = bound;
  }
  int n = g_closure_tc_occupancy > 0 ? g_closure_tc_occupancy : bound;
  if (n > (int)(512 / lbm_scheme::kTcCols)) n = (int)(512 / lbm_scheme::kTcCols);
  if (used) *used = n;
  if (bound_out) *bound_out = bound;
  return LBM_OK;
}
#endif

int lbm_scheme_set_closure_tc_occupancy(int32_t blocks_per_sm) {
  if (blocks_per_sm < 0 || blocks_per_sm > 8)
    return lbm::fail(LBM_ERR_ARG, "lbm_scheme_set_closure_tc_occupancy: %d (0..8)", blocks_per_sm);
#if LBM_Q <= 16 && (LBM_Q - LBM_NCONS) <= 8
  g_closure_tc_occupancy = blocks_per_sm;
  return LBM_OK;
#else
  return lbm::fail(LBM_ERR_UNSUPPORTED, "lbm_scheme_set_closure_tc_occupancy: no closure step in this scheme");
#endif
}

int lbm_scheme_closure_tc_occupancy(int32_t* bound, int32_t* used) {
  if (!bound || !used) return lbm::fail(LBM_ERR_ARG, "lbm_scheme_closure_tc_occupancy: NULL");
#if LBM_Q <= 16 && (LBM_Q - LBM_NCONS) <= 8
  int dev = 0, q = 0, u = 0;
  int rc = lbm::cuda_check(cudaGetDevice(&dev), "lbm_scheme_closure_tc_occupancy");
  if (!rc) rc = closure_tc_blocks_per_sm(dev, &u, &q);
  if (rc) return rc;
  *bound = q;
  *used = u;
  return LBM_OK;
#else
  return lbm::fail(LBM_ERR_UNSUPPORTED, "lbm_scheme_closure_tc_occupancy: no closure step in this scheme");
#endif
}

int lbm_scheme_set_step_variant(int32_t variant) {
  if (variant < 0 || variant > 1) return lbm::fail(LBM_ERR_ARG, "lbm_scheme_set_step_variant: %d", variant);
  g_step_variant = variant;
  return LBM_OK;
}

int lbm_scheme_wait_timeouts(uint32_t* count) {
  if (!count) return lbm::fail(LBM_ERR_ARG, "lbm_scheme_wait_timeouts: NULL");
  return lbm::cuda_check(cudaMemcpyFromSymbol(count, lbm_scheme::lbm_wait_timeouts, sizeof(uint32_t)),
                         "lbm_scheme_wait_timeouts");
}

static int step_common(const void* f, void* fnew, const lbm_lattice* lat, const double* prm, void* stream,
                       bool periodic, const char* who) {
  using namespace lbm_scheme;
  int rc = check_pop_lattice(lat, who);
  if (rc) return rc;
  if (!f || !fnew) return lbm::fail(LBM_ERR_ARG, "%s: NULL populations", who);
  if (f == fnew) return lbm::fail(LBM_ERR_ARG, "%s: f and fnew must be distinct buffers", who);
  if (LBM_NPRM > 0 && !prm) return lbm::fail(LBM_ERR_ARG, "%s: %d parameters expected", who, LBM_NPRM);
  StepArgs a = make_step_args(*lat, prm);
  dim3 grid = node_grid(*lat, false);
  cudaStream_t s = (cudaStream_t)stream;
#if LBM_HAS_PAIRS
  if (periodic && g_step_variant == 1 && staged_fits(*lat, f, fnew)) {
    const size_t smem = staged_smem_bytes(*lat);
    // shared-memory limit and resident blocks per SM, looked up once per device and size
    static int cache_dev = -1, cache_blocks = 0;
    static size_t cache_smem = 0;
    int dev = 0;
    rc = lbm::cuda_check(cudaGetDevice(&dev), who);
    if (rc) return rc;
    if (dev != cache_dev || smem != cache_smem) {
      int sms = 0, per_sm = 0;
      rc = lbm::cuda_check(cudaFuncSetAttribute(k_step_periodic_staged, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                (int)smem),
                           who);
      if (!rc) rc = lbm::cuda_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), who);
      if (!rc)
        rc = lbm::cuda_check(
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_step_periodic_staged, kStagedThreads, smem),
            who);
      if (rc) return rc;
      cache_dev = dev;
      cache_smem = smem;
      cache_blocks = sms * (per_sm > 0 ? per_sm : 1);
    }
    const int rows = LBM_DIM == 3 ? lat->n[0] * lat->n[1] : lat->n[0];
    const int blocks = cache_blocks < rows ? cache_blocks : rows;
    k_step_periodic_staged<<<blocks, kStagedThreads, smem, s>>>((const S*)f, (S*)fnew, a);
    return lbm::launch_check(who);
  }
  if (pairs_fit(*lat, f, fnew)) {
    grid.x = (unsigned)((lat->n[LBM_DIM - 1] / 2 + LBM_BLOCK - 1) / LBM_BLOCK);
    if (periodic)
      k_step_periodic_pairs<<<grid, LBM_BLOCK, 0, s>>>((const S*)f, (S*)fnew, a);
    else
      k_step_ghost_pairs<<<grid, LBM_BLOCK, 0, s>>>((const S*)f, (S*)fnew, a);
    return lbm::launch_check(who);
  }
#endif
  if (periodic)
    k_step_periodic<<<grid, LBM_BLOCK, 0, s>>>((const S*)f, (S*)fnew, a);
  else
    k_step_ghost<<<grid, LBM_BLOCK, 0, s>>>((const S*)f, (S*)fnew, a);
  return lbm::launch_check(who);
}

int lbm_one_time_step(const void* f, void* fnew, const lbm_lattice* lat, const double* prm, void* stream) {
  return step_common(f, fnew, lat, prm, stream, false, "lbm_one_time_step");
}

int lbm_one_time_step_periodic(const void* f, void* fnew, const lbm_lattice* lat, const double* prm,
                               void* stream) {
  return step_common(f, fnew, lat, prm, stream, true, "lbm_one_time_step_periodic");
}

int lbm_one_time_step_walls(const void* f, void* fnew, const lbm_lattice* lat, const double* prm,
                            const double* table, const int32_t* sym, void* stream) {
  using namespace lbm_scheme;
  const char* who = "lbm_one_time_step_walls";
  int rc = check_pop_lattice(lat, who);
  if (rc) return rc;
  if (!f || !fnew || f == fnew) return lbm::fail(LBM_ERR_ARG, "%s: bad population buffers", who);
  if (!table || !sym) return lbm::fail(LBM_ERR_ARG, "%s: NULL wall table", who);
  if (LBM_NPRM > 0 && !prm) return lbm::fail(LBM_ERR_ARG, "%s: %d parameters expected", who, LBM_NPRM);
  if (LBM_VMAX != 1) return lbm::fail(LBM_ERR_UNSUPPORTED, "%s: stencils reaching one node only", who);
  for (int d = 0; d < LBM_DIM; ++d)
    if (lat->halo[d] != 1) return lbm::fail(LBM_ERR_ARG, "%s: halo[%d]=%d, one ghost layer expected", who, d, lat->halo[d]);
  WallArgs w;
  for (int k = 0; k < LBM_Q; ++k) {
    if (sym[k] < 0 || sym[k] >= LBM_Q) return lbm::fail(LBM_ERR_ARG, "%s: sym[%d]=%d", who, k, sym[k]);
    w.sym[k] = sym[k];
    for (int j = 0; j < 27; ++j) w.c[k][j] = (R)table[k * 27 + j];
  }
  StepArgs a = make_step_args(*lat, prm);
  dim3 grid = node_grid(*lat, false);
  cudaStream_t s = (cudaStream_t)stream;
#if LBM_HAS_PAIRS
  if (pairs_fit(*lat, f, fnew)) {
    grid.x = (unsigned)((lat->n[LBM_DIM - 1] / 2 + LBM_BLOCK - 1) / LBM_BLOCK);
    k_step_walls_pairs<<<grid, LBM_BLOCK, 0, s>>>((const S*)f, (S*)fnew, a, w);
    return lbm::launch_check(who);
  }
#endif
  k_step_walls<<<grid, LBM_BLOCK, 0, s>>>((const S*)f, (S*)fnew, a, w);
  return lbm::launch_check(who);
}

int lbm_transport(const void* f, void* fnew, const lbm_lattice* lat, void* stream) {
  using namespace lbm_scheme;
  int rc = check_pop_lattice(lat, "lbm_transport");
  if (rc) return rc;
  if (!f || !fnew || f == fnew) return lbm::fail(LBM_ERR_ARG, "lbm_transport: bad buffers");
  StepArgs a = make_step_args(*lat, nullptr);
  k_transport<<<node_grid(*lat, false), LBM_BLOCK, 0, (cudaStream_t)stream>>>((const S*)f, (S*)fnew, a);
  return lbm::launch_check("lbm_transport");
}

static lbm_scheme::MomentArgs make_moment_args(const lbm_lattice* lat, const lbm_lattice* mlat, const double* prm) {
  lbm_scheme::MomentArgs a;
  a.g = lbm::make_geo(lat ? *lat : *mlat);
  a.gm = lbm::make_geo(*mlat);
  for (int i = 0; i < lbm_scheme::kPrm; ++i) a.prm[i] = (i < LBM_NPRM && prm) ? prm[i] : 0.0;
  return a;
}

int lbm_f2m(const void* f, const lbm_lattice* lat, double* m, const lbm_lattice* mlat, void* stream) {
  using namespace lbm_scheme;
  int rc = check_pop_lattice(lat, "lbm_f2m", false);
  if (!rc) rc = check_moment_lattice(lat, mlat, "lbm_f2m");
  if (rc) return rc;
  if (!f || !m) return lbm::fail(LBM_ERR_ARG, "lbm_f2m: NULL buffer");
  MomentArgs a = make_moment_args(lat, mlat, nullptr);
  k_f2m<<<node_grid(*lat, true), LBM_BLOCK, 0, (cudaStream_t)stream>>>((const S*)f, m, a);
  return lbm::launch_check("lbm_f2m");
}

int lbm_f2m_conserved(const void* f, const lbm_lattice* lat, double* m, const lbm_lattice* mlat, void* stream) {
  using namespace lbm_scheme;
  int rc = check_pop_lattice(lat, "lbm_f2m_conserved", false);
  if (!rc) rc = check_moment_lattice(lat, mlat, "lbm_f2m_conserved");
  if (rc) return rc;
  if (!f || !m) return lbm::fail(LBM_ERR_ARG, "lbm_f2m_conserved: NULL buffer");
  MomentArgs a = make_moment_args(lat, mlat, nullptr);
  k_f2m_conserved<<<node_grid(*lat, true), LBM_BLOCK, 0, (cudaStream_t)stream>>>((const S*)f, m, a);
  return lbm::launch_check("lbm_f2m_conserved");
}

int lbm_m2f(const double* m, const lbm_lattice* mlat, void* f, const lbm_lattice* lat, void* stream) {
  using namespace lbm_scheme;
  int rc = check_pop_lattice(lat, "lbm_m2f", false);
  if (!rc) rc = check_moment_lattice(lat, mlat, "lbm_m2f");
  if (rc) return rc;
  if (!f || !m) return lbm::fail(LBM_ERR_ARG, "lbm_m2f: NULL buffer");
  MomentArgs a = make_moment_args(lat, mlat, nullptr);
  k_m2f<<<node_grid(*lat, true), LBM_BLOCK, 0, (cudaStream_t)stream>>>(m, (S*)f, a);
  return lbm::launch_check("lbm_m2f");
}

int lbm_equilibrium(double* m, const lbm_lattice* mlat, const double* prm, void* stream) {
  using namespace lbm_scheme;
  int rc = check_moment_lattice(nullptr, mlat, "lbm_equilibrium");
  if (rc) return rc;
  if (!m) return lbm::fail(LBM_ERR_ARG, "lbm_equilibrium: NULL buffer");
  if (LBM_NPRM > 0 && !prm) return lbm::fail(LBM_ERR_ARG, "lbm_equilibrium: parameters expected");
  MomentArgs a = make_moment_args(nullptr, mlat, prm);
  k_equilibrium<<<node_grid(*mlat, true), LBM_BLOCK, 0, (cudaStream_t)stream>>>(m, a);
  return lbm::launch_check("lbm_equilibrium");
}

int lbm_f2m_conserved_dense(const void* f, const lbm_lattice* lat, double* out, void* stream) {
  using namespace lbm_scheme;
  int rc = check_pop_lattice(lat, "lbm_f2m_conserved_dense", false);
  if (rc) return rc;
  if (!f || !out) return lbm::fail(LBM_ERR_ARG, "lbm_f2m_conserved_dense: NULL buffer");
  MomentArgs a = make_moment_args(lat, lat, nullptr);
  k_f2m_conserved_dense<<<node_grid(*lat, false), LBM_BLOCK, 0, (cudaStream_t)stream>>>((const S*)f, out, a);
  return lbm::launch_check("lbm_f2m_conserved_dense");
}

int lbm_init_conserved(const double* m, const lbm_lattice* mlat, void* f, const lbm_lattice* lat, const double* prm,
                       void* stream) {
  using namespace lbm_scheme;
  int rc = check_pop_lattice(lat, "lbm_init_conserved", false);
  if (!rc) rc = check_moment_lattice(lat, mlat, "lbm_init_conserved");
  if (rc) return rc;
  if (!f || !m) return lbm::fail(LBM_ERR_ARG, "lbm_init_conserved: NULL buffer");
  if (LBM_NPRM > 0 && !prm) return lbm::fail(LBM_ERR_ARG, "lbm_init_conserved: parameters expected");
  MomentArgs a = make_moment_args(lat, mlat, prm);
  k_init_conserved<<<node_grid(*lat, true), LBM_BLOCK, 0, (cudaStream_t)stream>>>(m, (S*)f, a);
  return lbm::launch_check("lbm_init_conserved");
}

int lbm_source_term(double* m, const lbm_lattice* mlat, const double* prm, void* stream) {
  using namespace lbm_scheme;
  int rc = check_moment_lattice(nullptr, mlat, "lbm_source_term");
  if (rc) return rc;
  if (!LBM_HAS_SOURCE) return lbm::fail(LBM_ERR_UNSUPPORTED, "lbm_source_term: the scheme has no source terms");
  if (!m) return lbm::fail(LBM_ERR_ARG, "lbm_source_term: NULL buffer");
  if (LBM_NPRM > 0 && !prm) return lbm::fail(LBM_ERR_ARG, "lbm_source_term: parameters expected");
  MomentArgs a = make_moment_args(nullptr, mlat, prm);
  k_source_term<<<node_grid(*mlat, false), LBM_BLOCK, 0, (cudaStream_t)stream>>>(m, a);
  return lbm::launch_check("lbm_source_term");
}

static int closure_common(const void* f, void* fnew, const lbm_lattice* lat, const double* prm, const void* wbf16,
                          const float* params, const float* norm, const float* guard, const float* rate,
                          int32_t* fallbacks, int32_t grid, void* stream, bool tc, const char* who);

int lbm_one_time_step_periodic_closure(const void* f, void* fnew, const lbm_lattice* lat, const double* prm,
                                       const void* wbf16, const float* params, const float* norm,
                                       const float* guard, const float* rate, int32_t* fallbacks, int32_t grid,
                                       void* stream) {
  return closure_common(f, fnew, lat, prm, wbf16, params, norm, guard, rate, fallbacks, grid, stream, false,
                        "lbm_one_time_step_periodic_closure");
}

int lbm_one_time_step_periodic_closure_tc(const void* f, void* fnew, const lbm_lattice* lat, const double* prm,
                                          const float* params, const float* norm, const float* guard,
                                          const float* rate, int32_t* fallbacks, void* stream) {
  return closure_common(f, fnew, lat, prm, nullptr, params, norm, guard, rate, fallbacks, 0, stream, true,
                        "lbm_one_time_step_periodic_closure_tc");
}

static int closure_common(const void* f, void* fnew, const lbm_lattice* lat, const double* prm, const void* wbf16,
                          const float* params, const float* norm, const float* guard, const float* rate,
                          int32_t* fallbacks, int32_t grid, void* stream, bool tc, const char* who) {
  using namespace lbm_scheme;
  int rc = check_pop_lattice(lat, who);
  if (rc) return rc;
  if (LBM_Q > 16 || LBM_Q - LBM_NCONS > 8)
    return lbm::fail(LBM_ERR_UNSUPPORTED, "%s: the closure MLP takes at most 16 moments and 8 corrections", who);
  if (!f || !fnew || f == fnew || (!tc && !wbf16) || !params || !norm)
    return lbm::fail(LBM_ERR_ARG, "%s: bad pointers", who);
  if (!tc && (((uintptr_t)wbf16 | (uintptr_t)params) & 15u))
    return lbm::fail(LBM_ERR_ARG, "%s: wbf16 and params must be 16-byte aligned", who);
  if (LBM_NPRM > 0 && !prm) return lbm::fail(LBM_ERR_ARG, "%s: %d parameters expected", who, LBM_NPRM);
  StepArgs a = make_step_args(*lat, prm);
  ClosureArgs c;
  c.w = (const __nv_bfloat16*)wbf16;
  c.params = params;
  for (int i = 0; i < 16; ++i) {
    c.mu_in[i] = norm[i];
    c.isig_in[i] = norm[16 + i];
  }
  for (int i = 0; i < 8; ++i) {
    c.mu_out[i] = norm[32 + i];
    c.sig_out[i] = norm[40 + i];
  }
  c.nodes = (long long)lat->n[0] * lat->n[1] * lat->n[2];
  c.guard_ratio = guard ? guard[0] : 0.0f;
  c.guard_floor = guard ? guard[1] : 0.0f;
  c.fallbacks = fallbacks;
  c.rate_form = rate != nullptr;
  for (int i = 0; i < 8; ++i) {
    c.lam_lo[i] = rate ? rate[i] : 0.0f;
    c.lam_hi[i] = rate ? rate[8 + i] : 0.0f;
    if (rate && !(c.lam_lo[i] <= c.lam_hi[i] && c.lam_lo[i] >= -1.0f))
      return lbm::fail(LBM_ERR_ARG, "%s: rate bounds of output %d: [%g, %g] (need -1 <= lo <= hi)", who, i,
                       (double)c.lam_lo[i], (double)c.lam_hi[i]);
  }
#if LBM_Q <= 16 && (LBM_Q - LBM_NCONS) <= 8
  if (tc) {
    int dev = 0, sms = 0;
    int rc2 = lbm::cuda_check(cudaGetDevice(&dev), who);
    if (!rc2) rc2 = lbm::cuda_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), who);
    if (rc2) return rc2;
    int per_sm = 0;
    rc2 = closure_tc_blocks_per_sm(dev, &per_sm, nullptr);
    if (rc2) return rc2;
    const long long tiles = (c.nodes + kTcRows - 1) / kTcRows;
    const long long cap = (long long)per_sm * sms;
    const long long blocks = tiles < cap ? tiles : cap;
    k_step_periodic_closure_tc<<<(unsigned)blocks, kTcRows, 0, (cudaStream_t)stream>>>((const S*)f, (S*)fnew, a, c);
    return lbm::launch_check(who);
  }
#endif
  const long long per = kClosureWarpNodes * kClosureWarps;
  long long blocks = (c.nodes + per - 1) / per;
  if (grid > 0 && blocks > grid) blocks = grid;
  k_step_periodic_closure<<<(unsigned)blocks, 32 * kClosureWarps, 0, (cudaStream_t)stream>>>((const S*)f, (S*)fnew,
                                                                                             a, c);
  return lbm::launch_check(who);
}

static int ensemble_step(void* arena, const lbm_instance* inst, const int32_t* tile_instance, int32_t ntiles,
                         int32_t rows_per_tile, int32_t block, int32_t grid, int32_t parity, void* stream,
                         bool pairs_only, const char* who) {
  using namespace lbm_scheme;
  if (!arena || !inst || !tile_instance) return lbm::fail(LBM_ERR_ARG, "%s: NULL argument", who);
  if (ntiles < 0 || rows_per_tile < 1 || block < 32 || block > LBM_ENSEMBLE_MAX_BLOCK || (block % 32) || grid < 0 ||
      (parity != 0 && parity != 1))
    return lbm::fail(LBM_ERR_ARG, "%s: ntiles=%d rows_per_tile=%d block=%d grid=%d parity=%d", who, ntiles,
                     rows_per_tile, block, grid, parity);
  if (LBM_NPRM > LBM_MAX_PRM) return lbm::fail(LBM_ERR_UNSUPPORTED, "%s: too many parameters", who);
  if (ntiles == 0) return LBM_OK;
  unsigned blocks = (unsigned)(grid > 0 ? (grid < ntiles ? grid : ntiles) : ntiles);
  if (pairs_only) {
    if (!LBM_HAS_PAIRS) return lbm::fail(LBM_ERR_UNSUPPORTED, "%s: module without the two-node path", who);
    k_step_ensemble<true><<<blocks, block, 0, (cudaStream_t)stream>>>((S*)arena, inst, tile_instance, ntiles,
                                                                      rows_per_tile, parity);
  } else {
    k_step_ensemble<false><<<blocks, block, 0, (cudaStream_t)stream>>>((S*)arena, inst, tile_instance, ntiles,
                                                                       rows_per_tile, parity);
  }
  return lbm::launch_check(who);
}

int lbm_ensemble_step(void* arena, const lbm_instance* inst, const int32_t* tile_instance, int32_t ntiles,
                      int32_t rows_per_tile, int32_t block, int32_t grid, int32_t parity, void* stream) {
  return ensemble_step(arena, inst, tile_instance, ntiles, rows_per_tile, block, grid, parity, stream, false,
                       "lbm_ensemble_step");
}

int lbm_ensemble_step_pairs(void* arena, const lbm_instance* inst, const int32_t* tile_instance, int32_t ntiles,
                            int32_t rows_per_tile, int32_t block, int32_t grid, int32_t parity, void* stream) {
  return ensemble_step(arena, inst, tile_instance, ntiles, rows_per_tile, block, grid, parity, stream, true,
                       "lbm_ensemble_step_pairs");
}

int lbm_relaxation(double* m, const lbm_lattice* mlat, const double* prm, void* stream) {
  using namespace lbm_scheme;
  int rc = check_moment_lattice(nullptr, mlat, "lbm_relaxation");
  if (rc) return rc;
  if (!m) return lbm::fail(LBM_ERR_ARG, "lbm_relaxation: NULL buffer");
  if (LBM_NPRM > 0 && !prm) return lbm::fail(LBM_ERR_ARG, "lbm_relaxation: parameters expected");
  MomentArgs a = make_moment_args(nullptr, mlat, prm);
  k_relaxation<<<node_grid(*mlat, true), LBM_BLOCK, 0, (cudaStream_t)stream>>>(m, a);
  return lbm::launch_check("lbm_relaxation");
}

}  // extern "C"
