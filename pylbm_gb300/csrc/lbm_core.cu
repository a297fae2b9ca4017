// liblbm_gb300.so: scheme-independent runtime of the GB300 pylbm backend.
//
// Device memory, streams, the periodic ghost refresh, the boundary-node
// kernels and FP64 conservation sums.  Everything is reached through the C
// ABI declared in include/lbm_gb300.h.
#include "lbm_common.cuh"

#include <cstring>
#include <mutex>
#include <type_traits>

using namespace lbm;

namespace {

constexpr int kThreads = 256;

// ---------------------------------------------------------------- halo
// Slab decomposition of the ghost shell: slab (axis a, side s) holds the
// h[a] ghost layers of that side with every other axis at full halo extent.
// Cells at edges and corners belong to several slabs; each slab writes the
// same value there (the fully wrapped interior node), so the overlap is benign
// and the result equals pylbm's sequential x-then-y-then-z exchange.
struct HaloPlan {
  long long slab_cells[6];
  long long slab_begin[7];
  int nslab;
  int only;  // -1: every axis, wrapped along every axis; else this axis alone
};

__device__ __forceinline__ int wrap_index(int i, int n, int h) {
  if (i < h) return i + n;
  if (i >= n + h) return i - n;
  return i;
}

template <typename S>
__global__ void __launch_bounds__(kThreads) k_update_halo(S* __restrict__ f, Geo g, HaloPlan p) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= p.slab_begin[p.nslab]) return;
  int k = blockIdx.y;
  int slab = 0;
  while (slab + 1 < p.nslab && t >= p.slab_begin[slab + 1]) ++slab;
  long long r = t - p.slab_begin[slab];
  int axis = p.only >= 0 ? p.only : slab >> 1, side = slab & 1;
  int ext[3], idx[3];
  for (int d = 0; d < 3; ++d) ext[d] = g.n[d] + 2 * g.h[d];
  ext[axis] = g.h[axis];
  // decompose r with the last axis fastest
  for (int d = 2; d >= 0; --d) {
    idx[d] = (int)(r % ext[d]);
    r /= ext[d];
  }
  if (side) idx[axis] += g.n[axis] + g.h[axis];
  int src[3];
  for (int d = 0; d < 3; ++d)
    src[d] = (d < g.dim && (p.only < 0 || d == p.only)) ? wrap_index(idx[d], g.n[d], g.h[d]) : idx[d];
  long long o_dst = (long long)k * g.vstride + node_offset(g, idx[0], idx[1], idx[2]);
  long long o_src = (long long)k * g.vstride + node_offset(g, src[0], src[1], src[2]);
  f[o_dst] = f[o_src];
}

// ---------------------------------------------------------------- boundary
struct BcArgs {
  const int* iload;
  const int* istore;
  const double* rhs;
  int ncond;
  double sign;  // +1 bounce-back / Neumann, -1 anti-bounce-back
  double shift[LBM_MAX_Q];
};

template <typename S>
__device__ __forceinline__ void bc_link(S* f, const Geo& g, const BcArgs& a, int c) {
  const int w = g.dim + 1;
  const int* st = a.istore + (long long)c * w;
  const int* ld = a.iload + (long long)c * w;
  int is[3] = {0, 0, 0}, il[3] = {0, 0, 0};
  for (int d = 0; d < g.dim; ++d) {
    is[d] = st[1 + d];
    il[d] = ld[1 + d];
  }
  const int ks = st[0], kl = ld[0];
  long long os = (long long)ks * g.vstride + node_offset(g, is[0], is[1], is[2]);
  long long ol = (long long)kl * g.vstride + node_offset(g, il[0], il[1], il[2]);
  double fl = (double)Store<S>::load_plain(f + ol) + a.shift[kl];
  double v = a.sign * fl + (a.rhs ? a.rhs[c] : 0.0);
  Store<S>::store(f + os, (decltype(Store<S>::load_plain(f)))(v - a.shift[ks]));
}

template <typename S>
__global__ void __launch_bounds__(kThreads) k_boundary(S* __restrict__ f, Geo g, BcArgs a) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < a.ncond) bc_link(f, g, a, c);
}

// one thread, links in list order: the reference's sequential semantics
template <typename S>
__global__ void k_boundary_ordered(S* __restrict__ f, Geo g, BcArgs a) {
  if (blockIdx.x == 0 && threadIdx.x == 0)
    for (int c = 0; c < a.ncond; ++c) bc_link(f, g, a, c);
}

// ---------------------------------------------------------------- Bouzidi
struct BouzidiArgs {
  const int* iload0;
  const int* iload1;
  const int* istore;
  const double* rhs;
  const double* dist;
  double* scratch;  // copy semantics: values of every link before any store
  int ncond;
  int anti;         // 0: bounce-back (+d f0), 1: anti-bounce-back (-d f0)
  double shift[LBM_MAX_Q];
};

// element offset and velocity of one (k, i0[, i1[, i2]]) row of a link list
__device__ __forceinline__ long long link_slot(const Geo& g, const int* row, int& k) {
  int i[3] = {0, 0, 0};
  for (int d = 0; d < g.dim; ++d) i[d] = row[1 + d];
  k = row[0];
  return (long long)k * g.vstride + node_offset(g, i[0], i[1], i[2]);
}

// ((1-d) f1 +/- d f0) + rhs with separate roundings, in pylbm's printed order
template <typename S>
__device__ __forceinline__ double bouzidi_value(const S* f, const Geo& g, const BouzidiArgs& a, int c) {
  const int w = g.dim + 1;
  int k0, k1;
  const long long o0 = link_slot(g, a.iload0 + (long long)c * w, k0);
  const long long o1 = link_slot(g, a.iload1 + (long long)c * w, k1);
  const double f0 = (double)Store<S>::load_plain(f + o0) + a.shift[k0];
  const double f1 = (double)Store<S>::load_plain(f + o1) + a.shift[k1];
  const double d = a.dist[c];
  const double t1 = __dmul_rn(__dsub_rn(1.0, d), f1);
  const double t0 = __dmul_rn(d, f0);
  return __dadd_rn(a.anti ? __dsub_rn(t1, t0) : __dadd_rn(t1, t0), a.rhs[c]);
}

template <typename S>
__device__ __forceinline__ void bouzidi_store(S* f, const Geo& g, const BouzidiArgs& a, int c, double v) {
  int ks;
  const long long os = link_slot(g, a.istore + (long long)c * (g.dim + 1), ks);
  Store<S>::store(f + os, (decltype(Store<S>::load_plain(f)))(v - a.shift[ks]));
}

template <typename S>
__global__ void __launch_bounds__(kThreads) k_bouzidi(S* __restrict__ f, Geo g, BouzidiArgs a) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < a.ncond) bouzidi_store(f, g, a, c, bouzidi_value(f, g, a, c));
}

template <typename S>
__global__ void __launch_bounds__(kThreads) k_bouzidi_gather(const S* __restrict__ f, Geo g, BouzidiArgs a) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < a.ncond) a.scratch[c] = bouzidi_value(f, g, a, c);
}

template <typename S>
__global__ void __launch_bounds__(kThreads) k_bouzidi_scatter(S* __restrict__ f, Geo g, BouzidiArgs a) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < a.ncond) bouzidi_store(f, g, a, c, a.scratch[c]);
}

template <typename S>
__global__ void k_bouzidi_ordered(S* __restrict__ f, Geo g, BouzidiArgs a) {
  if (blockIdx.x == 0 && threadIdx.x == 0)
    for (int c = 0; c < a.ncond; ++c) bouzidi_store(f, g, a, c, bouzidi_value(f, g, a, c));
}

// ---------------------------------------------------------------- batched boundary methods
struct BatchArgs {
  const lbm_bc_method* methods;
  int nmethods;
  int total;
  double shift[LBM_MAX_Q];
};

// one thread per link of the batch; the same arithmetic as the per-method kernels
template <typename S>
__global__ void __launch_bounds__(kThreads) k_boundary_batch(S* __restrict__ f, Geo g, BatchArgs a) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= a.total) return;
  int m = 0;
  while (m + 1 < a.nmethods && c >= a.methods[m + 1].first) ++m;
  const lbm_bc_method M = a.methods[m];
  const int l = c - M.first;
  const int w = g.dim + 1;
  const bool flat = (M.flags & LBM_BC_FLAT) != 0;
  int ks = 0, k0 = 0;
  const long long os = flat ? (long long)M.istore[l] : link_slot(g, M.istore + (long long)l * w, ks);
  const long long o0 = flat ? (long long)M.iload0[l] : link_slot(g, M.iload0 + (long long)l * w, k0);
  if (M.kind == LBM_BC_GHOST_COPY) {
    f[os] = f[o0];
    return;
  }
  if (!std::is_same<S, double>::value && (M.flags & LBM_BC_FLOAT_FORM)) {
    // stored deviations in FP32: the shifts are folded into c by the caller
    const float c = reinterpret_cast<const float*>(M.rhs)[l];
    const float g0 = (float)Store<S>::load_plain(f + o0);
    float v;
    if (M.kind == LBM_BC_BOUZIDI_BOUNCE_BACK || M.kind == LBM_BC_BOUZIDI_ANTI_BOUNCE_BACK) {
      int k1 = 0;
      const long long o1 = flat ? (long long)M.iload1[l] : link_slot(g, M.iload1 + (long long)l * w, k1);
      const float g1 = (float)Store<S>::load_plain(f + o1);
      const float d = reinterpret_cast<const float*>(M.dist)[l];
      const float t1 = __fmul_rn(__fsub_rn(1.0f, d), g1);
      const float t0 = __fmul_rn(d, g0);
      v = __fadd_rn(M.kind == LBM_BC_BOUZIDI_ANTI_BOUNCE_BACK ? __fsub_rn(t1, t0) : __fadd_rn(t1, t0), c);
    } else {
      v = __fadd_rn(M.kind == LBM_BC_ANTI_BOUNCE_BACK ? -g0 : g0, c);
    }
    Store<S>::store(f + os, (decltype(Store<S>::load_plain(f)))v);
    return;
  }
  // flat offsets carry no population index: the caller sets them for unshifted storage only
  const double f0 = (double)Store<S>::load_plain(f + o0) + (flat ? 0.0 : a.shift[k0]);
  double v;
  if (M.kind == LBM_BC_BOUZIDI_BOUNCE_BACK || M.kind == LBM_BC_BOUZIDI_ANTI_BOUNCE_BACK) {
    int k1 = 0;
    const long long o1 = flat ? (long long)M.iload1[l] : link_slot(g, M.iload1 + (long long)l * w, k1);
    const double f1 = (double)Store<S>::load_plain(f + o1) + (flat ? 0.0 : a.shift[k1]);
    const double d = M.dist[l];
    const double t1 = __dmul_rn(__dsub_rn(1.0, d), f1);
    const double t0 = __dmul_rn(d, f0);
    v = __dadd_rn(M.kind == LBM_BC_BOUZIDI_ANTI_BOUNCE_BACK ? __dsub_rn(t1, t0) : __dadd_rn(t1, t0), M.rhs[l]);
  } else {
    const double sign = M.kind == LBM_BC_ANTI_BOUNCE_BACK ? -1.0 : 1.0;
    v = sign * f0 + (M.kind == LBM_BC_NEUMANN ? 0.0 : M.rhs[l]);
  }
  Store<S>::store(f + os, (decltype(Store<S>::load_plain(f)))(v - (flat ? 0.0 : a.shift[ks])));
}

// ---------------------------------------------------------------- gather
// One strided box of one plane (population or moment) into a dense array:
// element (i0, i1, i2) of the box is interior node start + i * step.
struct GatherBox {
  int start[3], count[3], step[3];
  long long total;
};

template <typename S>
__global__ void __launch_bounds__(kThreads) k_gather(const S* __restrict__ f, Geo g, int k, GatherBox b,
                                                     S* __restrict__ out) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= b.total) return;
  long long r = t;
  int idx[3];
  for (int d = 2; d >= 0; --d) {
    const int i = (int)(r % b.count[d]);
    r /= b.count[d];
    idx[d] = d < g.dim ? b.start[d] + i * b.step[d] + g.h[d] : 0;
  }
  out[t] = f[(long long)k * g.vstride + node_offset(g, idx[0], idx[1], idx[2])];
}

// ---------------------------------------------------------------- planes
// Whole planes between the padded layout and a dense array
// dense[plane][i0][i1][i2] over the interior or the halo-extended box, last
// axis fastest.  One thread per element of a box row: x runs along the last
// axis, y over the rows of the middle axis (3D) or over the first axis (2D),
// z over planes x first-axis rows (3D).  Every thread reads and writes one
// element, so both sides are coalesced along the row.
struct PlaneBox {
  int first;        // first plane of the lattice
  int n[3];         // box extent per axis (1 beyond dim)
  int lo[3];        // halo coordinate of the box's first node per axis
};

template <typename S, bool kToLattice>
__global__ void __launch_bounds__(kThreads) k_planes(S* __restrict__ f, Geo g, PlaneBox b,
                                                     S* __restrict__ dense) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int L = g.dim - 1;
  if (x >= b.n[L]) return;
  int idx[3] = {0, 0, 0};
  long long plane, row;
  if (g.dim == 3) {
    const int z = blockIdx.z;
    plane = z / b.n[0];
    idx[0] = z - (int)plane * b.n[0];
    idx[1] = blockIdx.y;
    row = ((long long)plane * b.n[0] + idx[0]) * b.n[1] + idx[1];
  } else if (g.dim == 2) {
    plane = blockIdx.z;
    idx[0] = blockIdx.y;
    row = (long long)plane * b.n[0] + idx[0];
  } else {
    plane = blockIdx.z;
    row = plane;
  }
  idx[L] = x;
  const long long dense_at = row * b.n[L] + x;
  const long long lat_at = (long long)(b.first + plane) * g.vstride +
                           node_offset(g, idx[0] + b.lo[0], idx[1] + b.lo[1], idx[2] + b.lo[2]);
  if (kToLattice)
    f[lat_at] = dense[dense_at];
  else
    dense[dense_at] = f[lat_at];
}

// ---------------------------------------------------------------- FP64 rate
// Eight independent FP64 FMA chains per thread (enough independent work to
// cover the pipe's latency at any occupancy); the result is written so the
// chains are not removed.  x <- x * a + b with a just below 1 stays bounded.
constexpr int kFmaChains = 8;
constexpr int kFmaBlocksPerSm = 8;

__global__ void __launch_bounds__(kThreads) k_fp64_fma(double* __restrict__ out, int iters, double a, double b) {
  double x[kFmaChains];
#pragma unroll
  for (int c = 0; c < kFmaChains; ++c) x[c] = 1e-3 * (threadIdx.x + c);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int c = 0; c < kFmaChains; ++c) x[c] = fma(x[c], a, b);
  }
  double acc = 0.0;
#pragma unroll
  for (int c = 0; c < kFmaChains; ++c) acc += x[c];
  out[(long long)blockIdx.x * blockDim.x + threadIdx.x] = acc;
}

// ---------------------------------------------------------------- sums
// Stage 1: block b of population k sums rows [b*rows_per_block, ...) of the
// interior with FP64 warp shuffles; stage 2 adds the per-block partials.
struct SumPlan {
  long long rows;           // interior rows (all axes but the last)
  long long rows_per_block;
  int blocks;               // per population
  int row_len;              // interior length of the last axis
};

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <typename S>
__global__ void __launch_bounds__(kThreads) k_sums_stage1(const S* __restrict__ f, Geo g, SumPlan p,
                                                          double* __restrict__ partials,
                                                          int* __restrict__ nonfinite) {
  const int k = blockIdx.y;
  const int L = g.dim - 1;
  double acc = 0.0;
  bool bad = false;
  long long r0 = (long long)blockIdx.x * p.rows_per_block;
  long long r1 = r0 + p.rows_per_block;
  if (r1 > p.rows) r1 = p.rows;
  for (long long r = r0; r < r1; ++r) {
    // row r -> interior coordinates of the axes before the last
    int idx[3] = {0, 0, 0};
    long long q = r;
    for (int d = L - 1; d >= 0; --d) {
      idx[d] = (int)(q % g.n[d]) + g.h[d];
      q /= g.n[d];
    }
    idx[L] = g.h[L];
    const S* row = f + (long long)k * g.vstride + node_offset(g, idx[0], idx[1], idx[2]);
    for (int i = threadIdx.x; i < p.row_len; i += blockDim.x) {
      double v = (double)Store<S>::load(row + i);
      bad |= !isfinite(v);
      acc += v;
    }
  }
  __shared__ double red[kThreads / 32];
  __shared__ int badflag;
  if (threadIdx.x == 0) badflag = 0;
  __syncthreads();
  if (bad) atomicOr(&badflag, 1);
  acc = warp_sum(acc);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = threadIdx.x < (kThreads / 32) ? red[threadIdx.x] : 0.0;
    v = warp_sum(v);
    if (threadIdx.x == 0) {
      partials[(long long)k * p.blocks + blockIdx.x] = v;
      if (badflag) atomicAdd(nonfinite, 1);
    }
  }
}

struct ShiftTable {
  double v[LBM_MAX_Q];
};

__global__ void __launch_bounds__(kThreads) k_sums_stage2(const double* __restrict__ partials, int blocks,
                                                          long long count, ShiftTable shift,
                                                          double* __restrict__ sums) {
  const int k = blockIdx.x;
  double acc = 0.0;
  for (int i = threadIdx.x; i < blocks; i += blockDim.x) acc += partials[(long long)k * blocks + i];
  __shared__ double red[kThreads / 32];
  acc = warp_sum(acc);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = threadIdx.x < (kThreads / 32) ? red[threadIdx.x] : 0.0;
    v = warp_sum(v);
    if (threadIdx.x == 0) sums[k] = v + (double)count * shift.v[k];
  }
}

// ---------------------------------------------------------------- restriction
struct RestrictArgs {
  double shift[LBM_MAX_Q];
  int factor;
  int nc[3];        // coarse interior sizes (1 beyond dim)
  long long cells;  // product of nc
};

template <typename S>
__global__ void __launch_bounds__(kThreads) k_restrict(const S* __restrict__ f, Geo g, RestrictArgs r,
                                                       double* __restrict__ out) {
  const long long cell = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (cell >= r.cells) return;
  const int k = blockIdx.y;
  int c[3];
  long long q = cell;
  for (int d = 2; d >= 0; --d) {
    c[d] = (int)(q % r.nc[d]);
    q /= r.nc[d];
  }
  const int f0 = g.dim > 0 ? r.factor : 1, f1 = g.dim > 1 ? r.factor : 1, f2 = g.dim > 2 ? r.factor : 1;
  double acc = 0.0;
  for (int a = 0; a < f0; ++a)
    for (int b = 0; b < f1; ++b)
      for (int e = 0; e < f2; ++e) {
        const int i0 = c[0] * f0 + a + g.h[0], i1 = c[1] * f1 + b + g.h[1], i2 = c[2] * f2 + e + g.h[2];
        acc += (double)Store<S>::load(f + (long long)k * g.vstride + node_offset(g, i0, i1, i2));
      }
  out[(long long)k * r.cells + cell] = acc / (double)(f0 * f1 * f2) + r.shift[k];
}

SumPlan make_sum_plan(const lbm_lattice& l) {
  SumPlan p;
  const int L = l.dim - 1;
  p.row_len = l.n[L];
  p.rows = 1;
  for (int d = 0; d < L; ++d) p.rows *= l.n[d];
  // about 8 rows of work per block, at most 4096 blocks per population
  long long target = (p.rows + 4095) / 4096;
  long long per = target > 8 ? target : 8;
  if (per > p.rows) per = p.rows;
  p.rows_per_block = per;
  p.blocks = (int)((p.rows + per - 1) / per);
  return p;
}

template <typename F>
int dispatch_dtype(int dt, F&& fn) {
  switch (dt) {
    case LBM_F64: return fn((double*)nullptr);
    case LBM_F32: return fn((float*)nullptr);
    case LBM_F16: return fn((__half*)nullptr);
    case LBM_BF16: return fn((__nv_bfloat16*)nullptr);
    default: return fail(LBM_ERR_ARG, "unknown dtype %d", dt);
  }
}

int boundary_common(void* f, const int32_t* iload0, const int32_t* istore, int32_t ncond,
                    const double* rhs, const lbm_lattice* lat, int32_t ordered, double sign,
                    const char* who, void* stream) {
  int rc = check_lattice(lat, who);
  if (rc) return rc;
  if (ncond < 0) return fail(LBM_ERR_ARG, "%s: ncond=%d", who, ncond);
  if (ncond == 0) return LBM_OK;
  if (!f || !iload0 || !istore) return fail(LBM_ERR_ARG, "%s: NULL array", who);
  BcArgs a;
  a.iload = iload0;
  a.istore = istore;
  a.rhs = rhs;
  a.ncond = ncond;
  a.sign = sign;
  for (int k = 0; k < LBM_MAX_Q; ++k) a.shift[k] = k < lat->nv ? lat->shift[k] : 0.0;
  Geo g = make_geo(*lat);
  cudaStream_t s = (cudaStream_t)stream;
  return dispatch_dtype(lat->dtype, [&](auto* tag) {
    using S = std::remove_pointer_t<decltype(tag)>;
    if (ordered) {
      k_boundary_ordered<S><<<1, 1, 0, s>>>((S*)f, g, a);
    } else {
      int blocks = (ncond + kThreads - 1) / kThreads;
      k_boundary<S><<<blocks, kThreads, 0, s>>>((S*)f, g, a);
    }
    return launch_check(who);
  });
}

}  // namespace

extern "C" {

const char* lbm_version(void) { return "pylbm_gb300 0.1.0 (sm_103a)"; }

const char* lbm_last_error(void) { return error_slot().msg; }

int lbm_lattice_init(lbm_lattice* lat, int32_t dim, int32_t nv, int32_t dtype, const int32_t* n,
                     const int32_t* halo) {
  if (!lat || !n || !halo) return fail(LBM_ERR_ARG, "lbm_lattice_init: NULL argument");
  if (dim < 1 || dim > 3) return fail(LBM_ERR_ARG, "lbm_lattice_init: dim=%d", dim);
  if (nv < 1 || nv > LBM_MAX_Q) return fail(LBM_ERR_ARG, "lbm_lattice_init: nv=%d", nv);
  size_t es = dtype_size(dtype);
  if (!es) return fail(LBM_ERR_ARG, "lbm_lattice_init: dtype=%d", dtype);
  std::memset(lat, 0, sizeof(*lat));
  lat->dim = dim;
  lat->nv = nv;
  lat->dtype = dtype;
  for (int d = 0; d < 3; ++d) {
    lat->n[d] = d < dim ? n[d] : 1;
    lat->halo[d] = d < dim ? halo[d] : 0;
    if (lat->n[d] < 1 || lat->halo[d] < 0)
      return fail(LBM_ERR_ARG, "lbm_lattice_init: n[%d]=%d halo[%d]=%d", d, lat->n[d], d, lat->halo[d]);
  }
  const long long align = (long long)(32 / es);  // 32-byte rows
  const int L = dim - 1;
  const long long h = lat->halo[L];
  const long long lead = ((h + align - 1) / align) * align;
  const long long pitch = ((lead + lat->n[L] + h + align - 1) / align) * align;
  long long s = pitch;
  for (int d = 2; d >= 0; --d) {
    if (d > L) {
      lat->stride[d] = 0;
    } else if (d == L) {
      lat->stride[d] = 1;
    } else {
      lat->stride[d] = s;
      s *= (long long)(lat->n[d] + 2 * lat->halo[d]);
    }
  }
  long long box = (L == 0) ? pitch : s;
  const long long valign = 128 / (long long)es;  // populations start on 128-byte boundaries
  lat->vstride = ((box + valign - 1) / valign) * valign;
  lat->origin = lead - h;
  lat->elements = (long long)nv * lat->vstride;
  return LBM_OK;
}

int lbm_device_count(int32_t* count) {
  int c = 0;
  int rc = cuda_check(cudaGetDeviceCount(&c), "cudaGetDeviceCount");
  if (count) *count = rc ? 0 : c;
  return rc;
}

int lbm_device_info(int32_t* sm_count, char* name, int32_t name_len) {
  int dev = 0;
  int rc = cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
  if (rc) return rc;
  cudaDeviceProp prop;
  rc = cuda_check(cudaGetDeviceProperties(&prop, dev), "cudaGetDeviceProperties");
  if (rc) return rc;
  if (sm_count) *sm_count = prop.multiProcessorCount;
  if (name && name_len > 0) {
    std::strncpy(name, prop.name, (size_t)name_len - 1);
    name[name_len - 1] = '\0';
  }
  return LBM_OK;
}

int lbm_set_device(int32_t device) { return cuda_check(cudaSetDevice(device), "cudaSetDevice"); }

int lbm_device_synchronize(void) { return cuda_check(cudaDeviceSynchronize(), "cudaDeviceSynchronize"); }

int lbm_alloc(void** ptr, size_t bytes) {
  if (!ptr) return fail(LBM_ERR_ARG, "lbm_alloc: NULL ptr");
  *ptr = nullptr;
  if (bytes == 0) bytes = 256;
  return cuda_check(cudaMalloc(ptr, bytes), "cudaMalloc");
}

int lbm_free(void* ptr) {
  if (!ptr) return LBM_OK;
  return cuda_check(cudaFree(ptr), "cudaFree");
}

int lbm_memcpy(void* dst, const void* src, size_t bytes, int32_t kind, void* stream) {
  if (bytes == 0) return LBM_OK;
  if (!dst || !src) return fail(LBM_ERR_ARG, "lbm_memcpy: NULL pointer");
  cudaMemcpyKind k;
  switch (kind) {
    case LBM_H2D: k = cudaMemcpyHostToDevice; break;
    case LBM_D2H: k = cudaMemcpyDeviceToHost; break;
    case LBM_D2D: k = cudaMemcpyDeviceToDevice; break;
    default: return fail(LBM_ERR_ARG, "lbm_memcpy: kind=%d", kind);
  }
  return cuda_check(cudaMemcpyAsync(dst, src, bytes, k, (cudaStream_t)stream), "cudaMemcpyAsync");
}

int lbm_memset(void* ptr, int32_t value, size_t bytes, void* stream) {
  if (bytes == 0) return LBM_OK;
  if (!ptr) return fail(LBM_ERR_ARG, "lbm_memset: NULL pointer");
  return cuda_check(cudaMemsetAsync(ptr, value, bytes, (cudaStream_t)stream), "cudaMemsetAsync");
}

int lbm_stream_create(void** stream) {
  if (!stream) return fail(LBM_ERR_ARG, "lbm_stream_create: NULL");
  cudaStream_t s;
  // a blocking stream: work on it is ordered with the legacy default stream,
  // so callers that mix both (e.g. NULL-stream copies) stay race-free
  int rc = cuda_check(cudaStreamCreateWithFlags(&s, cudaStreamDefault), "cudaStreamCreate");
  *stream = rc ? nullptr : (void*)s;
  return rc;
}

int lbm_stream_destroy(void* stream) {
  if (!stream) return LBM_OK;
  return cuda_check(cudaStreamDestroy((cudaStream_t)stream), "cudaStreamDestroy");
}

int lbm_stream_synchronize(void* stream) {
  return cuda_check(cudaStreamSynchronize((cudaStream_t)stream), "cudaStreamSynchronize");
}

int lbm_host_device_pointer(void* host, void** device) {
  if (!host || !device) return fail(LBM_ERR_ARG, "lbm_host_device_pointer: NULL pointer");
  *device = nullptr;
  cudaPointerAttributes attr;
  int rc = cuda_check(cudaPointerGetAttributes(&attr, host), "lbm_host_device_pointer: cudaPointerGetAttributes");
  if (rc) return rc;
  if (attr.type != cudaMemoryTypeHost || !attr.devicePointer)
    return fail(LBM_ERR_UNSUPPORTED, "lbm_host_device_pointer: not page-locked host memory mapped for the device");
  *device = attr.devicePointer;
  return LBM_OK;
}

int lbm_host_alloc(void** ptr, size_t bytes) {
  if (!ptr) return fail(LBM_ERR_ARG, "lbm_host_alloc: NULL ptr");
  *ptr = nullptr;
  return cuda_check(cudaMallocHost(ptr, bytes ? bytes : 256), "cudaMallocHost");
}

int lbm_host_free(void* ptr) {
  if (!ptr) return LBM_OK;
  return cuda_check(cudaFreeHost(ptr), "cudaFreeHost");
}

int lbm_event_create(void** event) {
  if (!event) return fail(LBM_ERR_ARG, "lbm_event_create: NULL");
  cudaEvent_t e;
  int rc = cuda_check(cudaEventCreate(&e), "cudaEventCreate");
  *event = rc ? nullptr : (void*)e;
  return rc;
}

int lbm_event_destroy(void* event) {
  if (!event) return LBM_OK;
  return cuda_check(cudaEventDestroy((cudaEvent_t)event), "cudaEventDestroy");
}

int lbm_event_record(void* event, void* stream) {
  if (!event) return fail(LBM_ERR_ARG, "lbm_event_record: NULL event");
  return cuda_check(cudaEventRecord((cudaEvent_t)event, (cudaStream_t)stream), "cudaEventRecord");
}

int lbm_event_elapsed_ms(void* start, void* end, float* ms) {
  if (!start || !end || !ms) return fail(LBM_ERR_ARG, "lbm_event_elapsed_ms: NULL");
  int rc = cuda_check(cudaEventSynchronize((cudaEvent_t)end), "cudaEventSynchronize");
  if (rc) return rc;
  return cuda_check(cudaEventElapsedTime(ms, (cudaEvent_t)start, (cudaEvent_t)end), "cudaEventElapsedTime");
}

int lbm_graph_begin(void* stream) {
  if (!stream) return fail(LBM_ERR_ARG, "lbm_graph_begin: capture needs a created stream, not NULL");
  return cuda_check(cudaStreamBeginCapture((cudaStream_t)stream, cudaStreamCaptureModeThreadLocal),
                    "cudaStreamBeginCapture");
}

int lbm_graph_end(void* stream, void** graph_exec) {
  if (!stream || !graph_exec) return fail(LBM_ERR_ARG, "lbm_graph_end: NULL argument");
  *graph_exec = nullptr;
  cudaGraph_t graph = nullptr;
  int rc = cuda_check(cudaStreamEndCapture((cudaStream_t)stream, &graph), "cudaStreamEndCapture");
  if (rc) return rc;
  cudaGraphExec_t exec = nullptr;
  rc = cuda_check(cudaGraphInstantiate(&exec, graph, 0), "cudaGraphInstantiate");
  cudaGraphDestroy(graph);
  if (rc) return rc;
  *graph_exec = (void*)exec;
  return LBM_OK;
}

int lbm_graph_launch(void* graph_exec, void* stream) {
  if (!graph_exec) return fail(LBM_ERR_ARG, "lbm_graph_launch: NULL graph");
  return cuda_check(cudaGraphLaunch((cudaGraphExec_t)graph_exec, (cudaStream_t)stream), "cudaGraphLaunch");
}

int lbm_graph_destroy(void* graph_exec) {
  if (!graph_exec) return LBM_OK;
  return cuda_check(cudaGraphExecDestroy((cudaGraphExec_t)graph_exec), "cudaGraphExecDestroy");
}

static int update_halo(void* f, const lbm_lattice* lat, int only, void* stream, const char* who) {
  int rc = check_lattice(lat, who);
  if (rc) return rc;
  if (!f) return fail(LBM_ERR_ARG, "%s: f is NULL", who);
  if (only >= lat->dim) return fail(LBM_ERR_ARG, "%s: axis %d of a %d-D lattice", who, only, lat->dim);
  HaloPlan p;
  p.nslab = 0;
  p.only = only;
  p.slab_begin[0] = 0;
  for (int a = 0; a < lat->dim; ++a) {
    if (only >= 0 && a != only) continue;
    long long cells = lat->halo[a];
    for (int d = 0; d < 3; ++d)
      if (d != a) cells *= (long long)(lat->n[d] + 2 * lat->halo[d]);
    for (int side = 0; side < 2; ++side) {
      p.slab_cells[p.nslab] = cells;
      p.slab_begin[p.nslab + 1] = p.slab_begin[p.nslab] + cells;
      ++p.nslab;
    }
  }
  long long total = p.slab_begin[p.nslab];
  if (total == 0) return LBM_OK;
  Geo g = make_geo(*lat);
  dim3 grid((unsigned)((total + kThreads - 1) / kThreads), (unsigned)lat->nv);
  cudaStream_t s = (cudaStream_t)stream;
  return dispatch_dtype(lat->dtype, [&](auto* tag) {
    using S = std::remove_pointer_t<decltype(tag)>;
    k_update_halo<S><<<grid, kThreads, 0, s>>>((S*)f, g, p);
    return launch_check(who);
  });
}

int lbm_update_halo(void* f, const lbm_lattice* lat, void* stream) {
  return update_halo(f, lat, -1, stream, "lbm_update_halo");
}

int lbm_update_halo_axis(void* f, const lbm_lattice* lat, int32_t axis, void* stream) {
  if (axis < 0) return fail(LBM_ERR_ARG, "lbm_update_halo_axis: axis %d", axis);
  return update_halo(f, lat, axis, stream, "lbm_update_halo_axis");
}

int lbm_bounce_back(void* f, const int32_t* iload0, const int32_t* istore, int32_t ncond,
                    const double* rhs, const lbm_lattice* lat, int32_t ordered, void* stream) {
  return boundary_common(f, iload0, istore, ncond, rhs, lat, ordered, 1.0, "lbm_bounce_back", stream);
}

int lbm_anti_bounce_back(void* f, const int32_t* iload0, const int32_t* istore, int32_t ncond,
                         const double* rhs, const lbm_lattice* lat, int32_t ordered, void* stream) {
  return boundary_common(f, iload0, istore, ncond, rhs, lat, ordered, -1.0, "lbm_anti_bounce_back",
                         stream);
}

int lbm_neumann(void* f, const int32_t* iload0, const int32_t* istore, int32_t ncond,
                const lbm_lattice* lat, int32_t ordered, void* stream) {
  return boundary_common(f, iload0, istore, ncond, nullptr, lat, ordered, 1.0, "lbm_neumann", stream);
}

static int bouzidi_common(void* f, const int32_t* iload0, const int32_t* iload1, const int32_t* istore,
                          int32_t ncond, const double* rhs, const double* dist, const lbm_lattice* lat,
                          double* scratch, int anti, int ordered, const char* who, void* stream) {
  int rc = check_lattice(lat, who);
  if (rc) return rc;
  if (ncond < 0) return fail(LBM_ERR_ARG, "%s: ncond=%d", who, ncond);
  if (ncond == 0) return LBM_OK;
  if (!f || !iload0 || !iload1 || !istore || !rhs || !dist) return fail(LBM_ERR_ARG, "%s: NULL array", who);
  BouzidiArgs a;
  a.iload0 = iload0;
  a.iload1 = iload1;
  a.istore = istore;
  a.rhs = rhs;
  a.dist = dist;
  a.scratch = scratch;
  a.ncond = ncond;
  a.anti = anti;
  for (int k = 0; k < LBM_MAX_Q; ++k) a.shift[k] = k < lat->nv ? lat->shift[k] : 0.0;
  Geo g = make_geo(*lat);
  cudaStream_t s = (cudaStream_t)stream;
  const int blocks = (ncond + kThreads - 1) / kThreads;
  return dispatch_dtype(lat->dtype, [&](auto* tag) {
    using S = std::remove_pointer_t<decltype(tag)>;
    if (ordered) {
      k_bouzidi_ordered<S><<<1, 1, 0, s>>>((S*)f, g, a);
    } else if (scratch) {
      k_bouzidi_gather<S><<<blocks, kThreads, 0, s>>>((const S*)f, g, a);
      k_bouzidi_scatter<S><<<blocks, kThreads, 0, s>>>((S*)f, g, a);
    } else {
      k_bouzidi<S><<<blocks, kThreads, 0, s>>>((S*)f, g, a);
    }
    return launch_check(who);
  });
}

int lbm_boundary_batch(void* f, const lbm_lattice* lat, const lbm_bc_method* methods, int32_t nmethods,
                       int32_t total_links, void* stream) {
  int rc = check_lattice(lat, "lbm_boundary_batch");
  if (rc) return rc;
  if (total_links < 0 || nmethods < 0) return fail(LBM_ERR_ARG, "lbm_boundary_batch: negative size");
  if (total_links == 0) return LBM_OK;
  if (!f || !methods || nmethods == 0) return fail(LBM_ERR_ARG, "lbm_boundary_batch: NULL argument");
  BatchArgs a;
  a.methods = methods;
  a.nmethods = nmethods;
  a.total = total_links;
  for (int k = 0; k < LBM_MAX_Q; ++k) a.shift[k] = k < lat->nv ? lat->shift[k] : 0.0;
  Geo g = make_geo(*lat);
  cudaStream_t s = (cudaStream_t)stream;
  return dispatch_dtype(lat->dtype, [&](auto* tag) {
    using S = std::remove_pointer_t<decltype(tag)>;
    k_boundary_batch<S><<<(total_links + kThreads - 1) / kThreads, kThreads, 0, s>>>((S*)f, g, a);
    return launch_check("lbm_boundary_batch");
  });
}

int lbm_bouzidi_bounce_back(void* f, const int32_t* iload0, const int32_t* iload1, const int32_t* istore,
                            int32_t ncond, const double* rhs, const double* dist, const lbm_lattice* lat,
                            double* scratch, void* stream) {
  return bouzidi_common(f, iload0, iload1, istore, ncond, rhs, dist, lat, scratch, 0, 0,
                        "lbm_bouzidi_bounce_back", stream);
}

int lbm_bouzidi_anti_bounce_back(void* f, const int32_t* iload0, const int32_t* iload1, const int32_t* istore,
                                 int32_t ncond, const double* rhs, const double* dist, const lbm_lattice* lat,
                                 int32_t ordered, void* stream) {
  return bouzidi_common(f, iload0, iload1, istore, ncond, rhs, dist, lat, nullptr, 1, ordered,
                        "lbm_bouzidi_anti_bounce_back", stream);
}

int lbm_gather(const void* f, const lbm_lattice* lat, int32_t k, const int32_t* start, const int32_t* count,
               const int32_t* step, void* out, void* stream) {
  int rc = check_lattice(lat, "lbm_gather");
  if (rc) return rc;
  if (!f || !out || !start || !count || !step) return fail(LBM_ERR_ARG, "lbm_gather: NULL argument");
  if (k < 0 || k >= lat->nv) return fail(LBM_ERR_ARG, "lbm_gather: plane %d of %d", k, lat->nv);
  GatherBox b;
  b.total = 1;
  for (int d = 0; d < 3; ++d) {
    if (d < lat->dim) {
      const long long last = (long long)start[d] + (long long)(count[d] - 1) * step[d];
      if (count[d] < 1 || start[d] < 0 || start[d] >= lat->n[d] || last < 0 || last >= lat->n[d])
        return fail(LBM_ERR_ARG, "lbm_gather: axis %d start %d count %d step %d outside 0..%d", d, start[d],
                    count[d], step[d], lat->n[d] - 1);
      b.start[d] = start[d];
      b.count[d] = count[d];
      b.step[d] = step[d];
    } else {
      b.start[d] = 0;
      b.count[d] = 1;
      b.step[d] = 1;
    }
    b.total *= b.count[d];
  }
  Geo g = make_geo(*lat);
  cudaStream_t s = (cudaStream_t)stream;
  return dispatch_dtype(lat->dtype, [&](auto* tag) {
    using S = std::remove_pointer_t<decltype(tag)>;
    k_gather<S><<<(unsigned)((b.total + kThreads - 1) / kThreads), kThreads, 0, s>>>((const S*)f, g, k, b,
                                                                                      (S*)out);
    return launch_check("lbm_gather");
  });
}

int lbm_copy_planes(void* f, const lbm_lattice* lat, int32_t first, int32_t count, int32_t with_halo,
                    void* dense, int32_t to_lattice, void* stream) {
  int rc = check_lattice(lat, "lbm_copy_planes");
  if (rc) return rc;
  if (!f || !dense) return fail(LBM_ERR_ARG, "lbm_copy_planes: NULL buffer");
  if (first < 0 || count < 1 || first + count > lat->nv)
    return fail(LBM_ERR_ARG, "lbm_copy_planes: planes %d..%d of %d", first, first + count - 1, lat->nv);
  PlaneBox b;
  b.first = first;
  for (int d = 0; d < 3; ++d) {
    b.n[d] = d < lat->dim ? lat->n[d] + (with_halo ? 2 * lat->halo[d] : 0) : 1;
    b.lo[d] = d < lat->dim && !with_halo ? lat->halo[d] : 0;
  }
  const int L = lat->dim - 1;
  // planes go in chunks whose z extent (planes x first-axis rows in 3D) fits the grid
  const int per_plane_z = lat->dim == 3 ? b.n[0] : 1;
  const int chunk = per_plane_z > 65535 ? 0 : 65535 / per_plane_z;
  const unsigned gy = lat->dim == 3 ? (unsigned)b.n[1] : lat->dim == 2 ? (unsigned)b.n[0] : 1u;
  if (chunk < 1 || gy > 65535u)
    return fail(LBM_ERR_UNSUPPORTED, "lbm_copy_planes: box rows beyond the 65535 grid limit");
  Geo g = make_geo(*lat);
  cudaStream_t s = (cudaStream_t)stream;
  return dispatch_dtype(lat->dtype, [&](auto* tag) {
    using S = std::remove_pointer_t<decltype(tag)>;
    const long long plane_elems = (long long)b.n[0] * b.n[1] * b.n[2];
    for (int c0 = 0; c0 < count; c0 += chunk) {
      const int c = count - c0 < chunk ? count - c0 : chunk;
      PlaneBox bc = b;
      bc.first = first + c0;
      dim3 grid((unsigned)((b.n[L] + kThreads - 1) / kThreads), gy, (unsigned)(c * per_plane_z));
      S* d = (S*)dense + (long long)c0 * plane_elems;
      if (to_lattice)
        k_planes<S, true><<<grid, kThreads, 0, s>>>((S*)f, g, bc, d);
      else
        k_planes<S, false><<<grid, kThreads, 0, s>>>((S*)f, g, bc, d);
      int rc2 = launch_check("lbm_copy_planes");
      if (rc2) return rc2;
    }
    return (int)LBM_OK;
  });
}

int lbm_fp64_fma_scratch_bytes(size_t* bytes) {
  int dev = 0, sms = 0;
  int rc = cuda_check(cudaGetDevice(&dev), "lbm_fp64_fma_scratch_bytes: cudaGetDevice");
  if (!rc) rc = cuda_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev),
                           "lbm_fp64_fma_scratch_bytes: SM count");
  if (rc) return rc;
  if (!bytes) return fail(LBM_ERR_ARG, "lbm_fp64_fma_scratch_bytes: NULL");
  *bytes = (size_t)sms * kFmaBlocksPerSm * kThreads * sizeof(double);
  return LBM_OK;
}

int lbm_fp64_fma_rate(double* scratch, int32_t iters, double* flops_per_s, float* ms, void* stream) {
  if (!scratch || !flops_per_s || iters < 1) return fail(LBM_ERR_ARG, "lbm_fp64_fma_rate: bad argument");
  int dev = 0, sms = 0;
  int rc = cuda_check(cudaGetDevice(&dev), "lbm_fp64_fma_rate: cudaGetDevice");
  if (!rc) rc = cuda_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev),
                           "lbm_fp64_fma_rate: SM count");
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  const int blocks = sms * kFmaBlocksPerSm;
  cudaEvent_t e0, e1;
  rc = cuda_check(cudaEventCreate(&e0), "lbm_fp64_fma_rate: event");
  if (rc) return rc;
  rc = cuda_check(cudaEventCreate(&e1), "lbm_fp64_fma_rate: event");
  if (rc) {
    cudaEventDestroy(e0);
    return rc;
  }
  k_fp64_fma<<<blocks, kThreads, 0, s>>>(scratch, iters, 0.9999999, 1e-7);  // warm-up
  cudaEventRecord(e0, s);
  k_fp64_fma<<<blocks, kThreads, 0, s>>>(scratch, iters, 0.9999999, 1e-7);
  cudaEventRecord(e1, s);
  rc = launch_check("lbm_fp64_fma_rate");
  float t = 0.f;
  if (!rc) rc = cuda_check(cudaEventSynchronize(e1), "lbm_fp64_fma_rate: synchronize");
  if (!rc) rc = cuda_check(cudaEventElapsedTime(&t, e0, e1), "lbm_fp64_fma_rate: elapsed");
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) return rc;
  const double flops = 2.0 * kFmaChains * (double)iters * blocks * kThreads;
  *flops_per_s = flops / (t * 1e-3);
  if (ms) *ms = t;
  return LBM_OK;
}

int lbm_restrict(const void* f, const lbm_lattice* lat, double* out, int32_t factor, void* stream) {
  int rc = check_lattice(lat, "lbm_restrict");
  if (rc) return rc;
  if (!f || !out) return fail(LBM_ERR_ARG, "lbm_restrict: NULL");
  if (factor < 1) return fail(LBM_ERR_ARG, "lbm_restrict: factor=%d", factor);
  RestrictArgs r;
  r.factor = factor;
  r.cells = 1;
  for (int d = 0; d < 3; ++d) {
    if (d < lat->dim) {
      if (lat->n[d] % factor) return fail(LBM_ERR_ARG, "lbm_restrict: n[%d]=%d not divisible by %d", d, lat->n[d], factor);
      r.nc[d] = lat->n[d] / factor;
    } else {
      r.nc[d] = 1;
    }
    r.cells *= r.nc[d];
  }
  for (int k = 0; k < LBM_MAX_Q; ++k) r.shift[k] = k < lat->nv ? lat->shift[k] : 0.0;
  Geo g = make_geo(*lat);
  dim3 grid((unsigned)((r.cells + kThreads - 1) / kThreads), (unsigned)lat->nv);
  cudaStream_t s = (cudaStream_t)stream;
  return dispatch_dtype(lat->dtype, [&](auto* tag) {
    using S = std::remove_pointer_t<decltype(tag)>;
    k_restrict<S><<<grid, kThreads, 0, s>>>((const S*)f, g, r, out);
    return launch_check("lbm_restrict");
  });
}

int lbm_population_sums_scratch_bytes(const lbm_lattice* lat, size_t* bytes) {
  int rc = check_lattice(lat, "lbm_population_sums_scratch_bytes");
  if (rc) return rc;
  if (!bytes) return fail(LBM_ERR_ARG, "lbm_population_sums_scratch_bytes: NULL");
  SumPlan p = make_sum_plan(*lat);
  // one FP64 partial sum per block and population
  *bytes = (size_t)lat->nv * (size_t)p.blocks * sizeof(double);
  return LBM_OK;
}

int lbm_population_sums(const void* f, const lbm_lattice* lat, double* sums, int32_t* nonfinite,
                        void* partials, size_t partials_bytes, void* stream) {
  int rc = check_lattice(lat, "lbm_population_sums");
  if (rc) return rc;
  if (!f || !sums || !nonfinite || !partials) return fail(LBM_ERR_ARG, "lbm_population_sums: NULL");
  size_t need = 0;
  lbm_population_sums_scratch_bytes(lat, &need);
  if (partials_bytes < need)
    return fail(LBM_ERR_ARG, "lbm_population_sums: scratch has %zu bytes, needs %zu", partials_bytes, need);
  SumPlan p = make_sum_plan(*lat);
  cudaStream_t s = (cudaStream_t)stream;
  double* part = (double*)partials;
  ShiftTable shift;
  for (int k = 0; k < LBM_MAX_Q; ++k) shift.v[k] = k < lat->nv ? lat->shift[k] : 0.0;
  rc = cuda_check(cudaMemsetAsync(nonfinite, 0, sizeof(int32_t), s), "lbm_population_sums: clear flag");
  if (rc) return rc;
  long long count = p.rows * (long long)p.row_len;
  Geo g = make_geo(*lat);
  rc = dispatch_dtype(lat->dtype, [&](auto* tag) {
    using S = std::remove_pointer_t<decltype(tag)>;
    dim3 grid((unsigned)p.blocks, (unsigned)lat->nv);
    k_sums_stage1<S><<<grid, kThreads, 0, s>>>((const S*)f, g, p, part, (int*)nonfinite);
    return launch_check("lbm_population_sums stage 1");
  });
  if (rc) return rc;
  k_sums_stage2<<<lat->nv, kThreads, 0, s>>>(part, p.blocks, count, shift, sums);
  return launch_check("lbm_population_sums stage 2");
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free variant of lbm_population_sums.
//
// Some callers cannot call cudaMalloc: a host application whose own memory
// manager owns every device allocation (the library may only use what it is
// handed), or a time-critical loop in which the implicit device
// synchronisation of cudaMalloc/cudaFree is not acceptable.  For them the
// per-block partial sums live in a fixed file-scope device array instead of
// caller-provided scratch.  The array is 1 MiB (131072 FP64 partials: any
// lattice with nv * blocks within that, e.g. every lattice with nv <= 32) and
// every GPU that loads this library holds it until the process exits.
//
// In host code the array's name is only a host-side stand-in, so its device
// address is looked up once per device (cudaGetSymbolAddress, with that device
// current) on the first call made on that device; that first call should come
// before any stream capture.  The address is cached together with the unique
// id of the context it was looked up in (cuCtxGetId): after a device reset the
// library's module lives in a new context, the ids differ and the first call
// in the new context looks the address up again (so that call, too, belongs
// before any capture).  All calls share the one array: calls that
// overlap on the GPU (e.g. on two streams) race on it.  Nothing in it needs to
// start at zero -- every partial is written before it is read -- and the
// non-finite counter is the caller's output, cleared by the call.
// ---------------------------------------------------------------------------
namespace {

constexpr size_t kNoAllocScratchBytes = size_t(1) << 20;
static __device__ __align__(256) double g_noalloc_partials[kNoAllocScratchBytes / sizeof(double)];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mutex;
struct NoAllocSlot {
  unsigned long long context_id;  // cuCtxGetId of the context the address belongs to
  void* address;
};
NoAllocSlot g_noalloc_slot[kMaxDevices] = {};

// cuCtxGetId through the runtime's driver entry point (no link to libcuda).
typedef int (*CtxGetIdFn)(void* ctx, unsigned long long* id);

int current_context_id(unsigned long long* id) {
  static CtxGetIdFn fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    int rc = cuda_check(cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q),
                        "lbm_population_sums_noalloc: driver entry point cuCtxGetId");
    if (rc) return rc;
    if (q != cudaDriverEntryPointSuccess || !p)
      return fail(LBM_ERR_UNSUPPORTED, "lbm_population_sums_noalloc: the driver has no cuCtxGetId");
    fn = (CtxGetIdFn)p;
  }
  // no current context: a plain status, the caller decides whether that is an error
  return fn(nullptr, id) == 0 ? LBM_OK : LBM_ERR_CUDA;
}

int noalloc_scratch_address(void** out) {
  int dev = 0;
  int rc = cuda_check(cudaGetDevice(&dev), "lbm_population_sums_noalloc: cudaGetDevice");
  if (rc) return rc;
  if (dev < 0 || dev >= kMaxDevices)
    return fail(LBM_ERR_UNSUPPORTED, "lbm_population_sums_noalloc: device %d beyond %d", dev, kMaxDevices);
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  NoAllocSlot& slot = g_noalloc_slot[dev];
  unsigned long long ctx = 0;
  // before the runtime has made a context current on this thread the id is
  // unavailable; the lookup below makes the device's primary context current
  bool have_ctx = slot.address && current_context_id(&ctx) == LBM_OK;
  if (!have_ctx || ctx != slot.context_id) {
    void* p = nullptr;
    rc = cuda_check(cudaGetSymbolAddress(&p, g_noalloc_partials),
                    "lbm_population_sums_noalloc: cudaGetSymbolAddress");
    if (rc) return rc;
    if (current_context_id(&ctx) != LBM_OK)
      return fail(LBM_ERR_CUDA, "lbm_population_sums_noalloc: no current context after the symbol lookup");
    slot.context_id = ctx;
    slot.address = p;
  }
  *out = slot.address;
  return LBM_OK;
}

}  // namespace

extern "C" size_t lbm_population_sums_noalloc_max_bytes(void) { return kNoAllocScratchBytes; }

extern "C" int lbm_population_sums_noalloc(const void* f, const lbm_lattice* lat, double* sums,
                                           int32_t* nonfinite, void* stream) {
  int rc = check_lattice(lat, "lbm_population_sums_noalloc");
  if (rc) return rc;
  size_t need = 0;
  rc = lbm_population_sums_scratch_bytes(lat, &need);
  if (rc) return rc;
  if (need > kNoAllocScratchBytes)
    return fail(LBM_ERR_ARG,
                "lbm_population_sums_noalloc: this lattice needs %zu bytes of partial sums, the built-in "
                "scratch holds %zu; use lbm_population_sums with caller-provided scratch",
                need, kNoAllocScratchBytes);
  void* scratch = nullptr;
  rc = noalloc_scratch_address(&scratch);
  if (rc) return rc;
  return lbm_population_sums(f, lat, sums, nonfinite, scratch, kNoAllocScratchBytes, stream);
}
