/*
 * lbm_gb300.h -- C ABI of the GB300 stream+collide backend for pylbm.
 *
 * Two shared libraries export this ABI:
 *
 *   liblbm_gb300.so      scheme-independent runtime: device memory, streams,
 *                        the periodic ghost refresh, the boundary-node kernels
 *                        and the FP64 conservation sums.
 *   lbm_scheme_<id>.so   one per scheme and storage type, generated and
 *                        compiled from the scheme's sympy description (as
 *                        pylbm compiles one Cython module per scheme), holding
 *                        the fused pull-stream + collide and the moment
 *                        transforms.
 *
 * Conventions: every entry point returns LBM_OK (0) or an error code and never
 * throws or aborts; lbm_last_error() / lbm_scheme_last_error() give the message
 * of the last failure of the calling thread.  Pointers named f, fnew, m, rhs,
 * istore, iload0 and sums are DEVICE pointers; lbm_lattice and prm are HOST
 * pointers read during the call.  `stream` is a cudaStream_t (NULL = legacy
 * default stream).  Calls only enqueue work unless stated otherwise.
 *
 * Population storage: structure of arrays, one array per population, each a
 * halo-extended box with the last axis contiguous (pylbm's index order
 * f[k, ix, iy, iz], pylbm/storage.py:423 SOA).  Element (k, i0, i1, i2) in
 * halo coordinates lives at
 *     k*vstride + origin + i0*stride[0] + i1*stride[1] + i2*stride[2]
 * where the stride of the last axis is 1 and rows of the last axis are padded
 * so that interior rows start on 32-byte boundaries (lbm_lattice_init).
 * With shifted storage the stored value is f_k - shift[k].
 */
#ifndef LBM_GB300_H
#define LBM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LBM_MAX_Q 64

enum lbm_status {
  LBM_OK = 0,
  LBM_ERR_ARG = 1,         /* invalid argument (sizes, types, null pointers) */
  LBM_ERR_CUDA = 2,        /* a CUDA runtime call failed */
  LBM_ERR_NONFINITE = 3,   /* a NaN or Inf was found in the populations */
  LBM_ERR_TIMEOUT = 4,     /* a bounded device-side wait gave up */
  LBM_ERR_UNSUPPORTED = 5  /* configuration not handled by this build */
};

enum lbm_dtype { LBM_F64 = 0, LBM_F32 = 1, LBM_F16 = 2, LBM_BF16 = 3 };

enum lbm_copy_kind { LBM_H2D = 0, LBM_D2H = 1, LBM_D2D = 2 };

typedef struct lbm_lattice {
  int32_t dim;                /* 1, 2 or 3 */
  int32_t nv;                 /* number of populations */
  int32_t dtype;              /* enum lbm_dtype of the stored values */
  int32_t reserved;
  int32_t n[3];               /* interior nodes per axis (1 beyond dim) */
  int32_t halo[3];            /* ghost layers per axis (0 beyond dim) */
  int64_t stride[3];          /* element stride per axis; stride[dim-1] == 1 */
  int64_t vstride;            /* element stride between populations */
  int64_t origin;             /* element offset of halo index (0,0,0) */
  int64_t elements;           /* total elements of the allocation (nv*vstride) */
  double shift[LBM_MAX_Q];    /* stored value = f_k - shift[k] */
} lbm_lattice;

/* ------------------------------------------------------------------ */
/* liblbm_gb300.so: runtime                                             */
/* ------------------------------------------------------------------ */

const char* lbm_version(void);
const char* lbm_last_error(void);

/* Fill the strides of the padded structure-of-arrays layout described
 * above for `dim` axes of n[d] interior nodes and halo[d] ghost layers;
 * shift[] is zeroed.  Host-only. */
int lbm_lattice_init(lbm_lattice* lat, int32_t dim, int32_t nv, int32_t dtype,
                     const int32_t* n, const int32_t* halo);

int lbm_device_count(int32_t* count);
/* Multiprocessor count and name of the current device (name NUL-terminated). */
int lbm_device_info(int32_t* sm_count, char* name, int32_t name_len);
int lbm_set_device(int32_t device);
int lbm_device_synchronize(void);

/* Device memory and copies (replace the pyopencl arrays of pylbm's LOOPY
 * containers, pylbm/storage.py:109-157, pylbm/boundary.py:378-397). */
int lbm_alloc(void** ptr, size_t bytes);
int lbm_free(void* ptr);
int lbm_memcpy(void* dst, const void* src, size_t bytes, int32_t kind, void* stream);
int lbm_memset(void* ptr, int32_t value, size_t bytes, void* stream);
int lbm_stream_create(void** stream); /* blocking: ordered with the legacy default stream */
int lbm_stream_destroy(void* stream);
int lbm_stream_synchronize(void* stream);

/* Pinned host memory (for host<->device copies that overlap compute). */
int lbm_host_alloc(void** ptr, size_t bytes);
int lbm_host_free(void* ptr);
/* The device address of page-locked host memory (from lbm_host_alloc), for
 * kernels that read or write it directly over the host link; LBM_ERR_UNSUPPORTED
 * when the memory is not mapped for the device. */
int lbm_host_device_pointer(void* host, void** device);

/* CUDA events on a stream, for device-side timing. */
int lbm_event_create(void** event);
int lbm_event_destroy(void* event);
int lbm_event_record(void* event, void* stream);
int lbm_event_elapsed_ms(void* start, void* end, float* ms); /* synchronizes on `end` */

/* CUDA graphs: capture the work enqueued on `stream` (not the legacy default
 * stream) between lbm_graph_begin and lbm_graph_end into an executable
 * graph, then replay it with lbm_graph_launch.  Used to replay a fixed
 * sequence of steps (ghost refresh, boundary kernels, step kernel) with one
 * launch. */
int lbm_graph_begin(void* stream);
int lbm_graph_end(void* stream, void** graph_exec);
int lbm_graph_launch(void* graph_exec, void* stream);
int lbm_graph_destroy(void* graph_exec);

/* Periodic ghost refresh of every axis: ghost layer i of an axis receives
 * interior layer i +/- n (pylbm/storage.py:307-367 Array.update, a periodic
 * halo exchange with itself on one process; LOOPY kernels update_x/y/z
 * :370-420).  Boundary kernels run afterwards and overwrite the ghost
 * populations they own, as in Simulation.boundary_condition
 * (pylbm/simulation.py:374-390). */
int lbm_update_halo(void* f, const lbm_lattice* lat, void* stream);

/* One axis of that refresh, as pylbm's per-axis exchange makes it
 * (pylbm/storage.py:331-367 one pass of the loop over d; LOOPY update_x,
 * update_y, update_z :370-420): the two ghost slabs of `axis`, over the full
 * extent (ghosts included) of the other axes, receive the interior layers
 * n away along `axis` only.  Axes 0, 1, 2 in that order equal
 * lbm_update_halo. */
int lbm_update_halo_axis(void* f, const lbm_lattice* lat, int32_t axis, void* stream);

/* Boundary-node kernels.  istore and iload0 are int32 arrays of shape
 * (ncond, dim+1): velocity index then halo coordinates, the layout pylbm
 * gives them after BoundaryMethod.fix_iload (pylbm/boundary.py:226-235).
 * rhs is float64 (ncond).  Values are physical (shift applied inside).
 *   bounce_back:       f[istore] =  f[iload0] + rhs   (pylbm/boundary.py:430-464)
 *   anti_bounce_back:  f[istore] = -f[iload0] + rhs   (pylbm/boundary.py:646-680)
 *   neumann:           f[istore] =  f[iload0]         (pylbm/boundary.py:787-818,
 *                      also neumannx/y/z, which differ only in iload0)
 * The links of one call must not read a population another link of the
 * same call writes (true for lists built by pylbm's Boundary); `ordered`=1
 * processes the links one after the other instead. */
int lbm_bounce_back(void* f, const int32_t* iload0, const int32_t* istore, int32_t ncond,
                    const double* rhs, const lbm_lattice* lat, int32_t ordered, void* stream);
int lbm_anti_bounce_back(void* f, const int32_t* iload0, const int32_t* istore, int32_t ncond,
                         const double* rhs, const lbm_lattice* lat, int32_t ordered, void* stream);
int lbm_neumann(void* f, const int32_t* iload0, const int32_t* istore, int32_t ncond,
                const lbm_lattice* lat, int32_t ordered, void* stream);

/* Bouzidi interpolated walls (second-order wall position from the link's
 * wall distance).  iload1 is a second load list of the same layout and
 * dist[c] the interpolation weight of link c (pylbm's BoundaryMethod.s:
 * 2q for q < 1/2, 1/(2q) otherwise, pylbm/boundary.py:508-534).  With
 * d = dist[c], f0 = f[iload0[c]], f1 = f[iload1[c]], evaluated in this order
 * without fused multiply-adds as pylbm's generated code does:
 *   bouzidi_bounce_back:       f[istore] = ((1-d) f1 + d f0) + rhs
 *                              (pylbm/boundary.py:570-618; the loads read a
 *                              copy of f taken before the method runs)
 *   bouzidi_anti_bounce_back:  f[istore] = ((1-d) f1 - d f0) + rhs
 *                              (pylbm/boundary.py:707-756; loads read f
 *                              itself, links in list order)
 * Bounce-back: `scratch` (ncond doubles, device) gives the copy semantics
 * by computing every link before storing any; NULL is allowed when no link
 * loads a population another link of the call stores.  Anti-bounce-back:
 * `ordered` as for lbm_bounce_back. */
int lbm_bouzidi_bounce_back(void* f, const int32_t* iload0, const int32_t* iload1, const int32_t* istore,
                            int32_t ncond, const double* rhs, const double* dist, const lbm_lattice* lat,
                            double* scratch, void* stream);
int lbm_bouzidi_anti_bounce_back(void* f, const int32_t* iload0, const int32_t* iload1, const int32_t* istore,
                                 int32_t ncond, const double* rhs, const double* dist, const lbm_lattice* lat,
                                 int32_t ordered, void* stream);

/* Every boundary method of a step in one launch.  `methods` (device,
 * nmethods entries) describes each method's lists as for the calls above;
 * link c of the batch belongs to the method whose [first, first + ncond)
 * holds c.  All links read the populations as they are before the call, so
 * the batch equals the methods applied one after the other only when no
 * link loads a population that a link of the batch stores (the caller
 * checks; pylbm's lists for a wall, an inflow and an outflow satisfy it).
 * Ordered (sequential) methods are not batched. */
#define LBM_BC_BOUNCE_BACK 1
#define LBM_BC_ANTI_BOUNCE_BACK 2
#define LBM_BC_NEUMANN 3
#define LBM_BC_BOUZIDI_BOUNCE_BACK 4
#define LBM_BC_BOUZIDI_ANTI_BOUNCE_BACK 5
/* f[istore] = f[iload0] as stored (no conversion, no shift): the periodic
 * ghost copies of lbm_update_halo restricted to the ghost populations that a
 * later read observes (a pull of an interior node or a boundary load that no
 * boundary store precedes).  Interior results equal those of the full
 * refresh bit for bit; the other ghost populations keep stale values. */
#define LBM_BC_GHOST_COPY 6

/* Flag of lbm_bc_method.flags for FP32 / FP16 / BF16 storage: `rhs` and
 * `dist` point to float arrays and the link computes in FP32 on the stored
 * deviations g = f - shift: g_s = +/- g_0 + c (bounce-back, anti-bounce-back,
 * Neumann) or g_s = ((1 - d) g_1 +/- d g_0) + c (Bouzidi), where the caller
 * folds the shifts into c = +/- shift[k_0] + rhs - shift[k_s] (Bouzidi:
 * (1 - d) shift[k_1] +/- d shift[k_0] + rhs - shift[k_s]) in float64 and
 * rounds it once.  No float64 arithmetic runs on the device. */
#define LBM_BC_FLOAT_FORM 1
/* Flag of lbm_bc_method.flags: iload0, iload1 and istore hold one int32 per
 * link, the element offset k * vstride + node offset of the slot, instead of
 * rows (k, i0, ...).  The population index is then unknown to the kernel,
 * so the caller sets it with LBM_BC_FLOAT_FORM or with unshifted storage. */
#define LBM_BC_FLAT 2

typedef struct lbm_bc_method {
  int32_t kind;               /* LBM_BC_* */
  int32_t ncond;
  int32_t first;              /* index of the method's first link in the batch */
  int32_t flags;              /* LBM_BC_FLOAT_FORM or 0 */
  const int32_t* iload0;
  const int32_t* iload1;      /* Bouzidi only */
  const int32_t* istore;
  const double* rhs;          /* not for Neumann (float* with LBM_BC_FLOAT_FORM) */
  const double* dist;         /* Bouzidi only (float* with LBM_BC_FLOAT_FORM) */
} lbm_bc_method;

int lbm_boundary_batch(void* f, const lbm_lattice* lat, const lbm_bc_method* methods, int32_t nmethods,
                       int32_t total_links, void* stream);

/* ------------------------------------------------------------------ */
/* Domain construction on the device (pylbm/domain.py:87-620 and the  */
/* link lists of pylbm/boundary.py:23-160): fluid/solid map, per-link */
/* wall distance and label, and the boundary links they define.  The   */
/* arrays cover the halo-extended box, last axis contiguous, no        */
/* padding; for each unique velocity u of the stencil,                 */
/* distance[u][node] is the fraction of the link node -> node + v_u    */
/* before a wall (999 where none) and flag[u][node] that wall's label  */
/* (999 where none); in_or_out is 999 in the fluid, -1 elsewhere.      */
/* Arithmetic follows the host rules operation by operation (IEEE,     */
/* no fused multiply-adds), so the arrays equal the host ones bit for  */
/* bit.                                                                */
/* ------------------------------------------------------------------ */

typedef struct lbm_domain {
  int32_t dim;                /* 1, 2 or 3 */
  int32_t nu;                 /* unique velocities */
  int32_t n[3];               /* halo-extended nodes per axis (1 beyond dim) */
  int32_t halo[3];            /* ghost layers per axis */
  int32_t vel[LBM_MAX_Q][3];  /* unique velocities */
  double dx;                  /* space step */
} lbm_domain;

#define LBM_ELEMENT_CIRCLE 1        /* p = cx, cy, radius; one label */
#define LBM_ELEMENT_PARALLELOGRAM 2 /* p = point x, y, v1 x, y, v2 x, y; labels of the 4 edges */
#define LBM_ELEMENT_SPHERE 3        /* p = cx, cy, cz, radius; one label (3D domains) */
/* The kinds below take the constants of their ray equations from the host
 * (pylbm_gb300/geometry.py ``device_params``), per element in p and per
 * unique velocity u in vq[u]; the device repeats only the per-node terms. */
#define LBM_ELEMENT_ELLIPSE 4   /* p = cx, cy, sxx, syy, sxy, det2 (syy X^2 + sxx Y^2 - sxy XY = det2);
                                   vq[u][0] = the ray quadratic's coefficient; one label
                                   (pylbm/elements/ellipse.py) */
#define LBM_ELEMENT_TRIANGLE 5  /* p = point x, y, v1 x, y, v2 x, y; labels of the 3 edges
                                   (pylbm/elements/triangle.py) */
#define LBM_ELEMENT_ELLIPSOID 6 /* p = cx, cy, cz, cxx, cyy, czz, cxy, cyz, czx, d; vq[u] = the ray
                                   quadratic's coefficient and the 3 factors of its linear one;
                                   one label (pylbm/elements/ellipsoid.py) */
#define LBM_ELEMENT_CYLINDER 7  /* p = center x, y, z, the inverse frame matrix (9, row-major), the
                                   section (0 disc, 1 triangle, 2 square); vq[u] = velocity u in the
                                   frame and, for the disc, the side's ray quadratic coefficient;
                                   labels: the sides, bottom, top (pylbm/elements/cylinder.py) */

typedef struct lbm_element {
  int32_t kind;
  int32_t isfluid;            /* 1: the element carves fluid out of solid */
  int32_t label[6];
  double p[24];
  int32_t lo[3], hi[3];       /* halo-coordinate region [lo, hi) the element touches */
  double vq[LBM_MAX_Q][4];    /* per unique velocity constants (kinds 4..7) */
} lbm_element;

/* in_or_out = -1 with 999 on the interior, distance = 999, flag = 999
 * (pylbm/domain.py:87-160). */
int lbm_domain_reset(const lbm_domain* d, double* in_or_out, double* distance, int32_t* flag, void* stream);

/* Box walls: for every axis and every unique velocity leaving the box
 * through a side whose label is not -2, the first |v| interior layers get
 * distance (i + 1/2)/|v| and that side's label where this is shorter than
 * the current distance (pylbm/domain.py:463-521). */
int lbm_domain_box(const lbm_domain* d, const int32_t* box_label, double* distance, int32_t* flag, void* stream);

/* One obstacle (pylbm/domain.py:523-620): nodes of the element become solid
 * (fluid for isfluid elements), then each fluid node of the region whose
 * link v_u ends in a solid node and crosses the element's boundary within
 * one link gets the crossing fraction and edge label (shortest wins).
 * `coords` holds the halo coordinates of axis 0, then 1, then 2. */
int lbm_domain_element(const lbm_domain* d, const lbm_element* e, const double* coords, double* in_or_out,
                       double* distance, int32_t* flag, void* stream);

/* Links starting in solid nodes are removed (pylbm/domain.py ``clean``). */
int lbm_domain_clean(const lbm_domain* d, const double* in_or_out, double* distance, int32_t* flag,
                     void* stream);

/* Boundary links of one label and one unique velocity u, in row-major node
 * order (np.where of pylbm/boundary.py:23-47): every node with
 * flag[u][node] == label gives the row node + vsym (its halo coordinates)
 * and distance[u][node].  Two passes: lbm_links_count writes the count of
 * each block of lbm_links_block() nodes (blocks = ceil(nodes / block));
 * the caller prefix-sums them into offsets and lbm_links_fill writes rows
 * (count, dim) int32 and distances (count) float64. */
int32_t lbm_links_block(void);
int lbm_links_count(const lbm_domain* d, const int32_t* flag, int32_t u, int32_t label, int32_t* block_counts,
                    void* stream);
int lbm_links_fill(const lbm_domain* d, const int32_t* flag, const double* distance, int32_t u, int32_t label,
                   const int32_t* vsym, const int32_t* block_offsets, int32_t* rows, double* dist, void* stream);

/* A strided box of one plane k of a lattice (populations in their storage
 * type, or float64 moments) copied into a dense device array out, last axis
 * fastest: out[i0][i1][i2] = plane k at interior node start + i * step
 * (step may be negative; every selected node must be interior).  Reading a
 * slice of sim.m or sim.F then moves only the slice to the host
 * (pylbm/simulation.py:216-256 m / F, followed by the caller's indexing). */
int lbm_gather(const void* f, const lbm_lattice* lat, int32_t k, const int32_t* start, const int32_t* count,
               const int32_t* step, void* out, void* stream);

/* Planes first..first+count-1 of a lattice (raw stored values: populations
 * in their storage type, or float64 moments) copied between the padded
 * layout and a dense device array dense[plane][i0][i1][i2], last axis
 * fastest, over the interior (with_halo = 0) or the halo-extended box
 * (with_halo = 1); to_lattice = 1 writes the lattice from dense, 0 reads it
 * into dense.  Assigning whole moment planes (sim.m_halo[k] = array) and
 * reading the conserved fields then cross the host link as one contiguous
 * copy each (pylbm/simulation.py:200-224 m_halo / m, whose numpy arrays are
 * dense). */
int lbm_copy_planes(void* f, const lbm_lattice* lat, int32_t first, int32_t count, int32_t with_halo,
                    void* dense, int32_t to_lattice, void* stream);

/* Measured FP64 FMA rate of the current device: eight independent DFMA
 * chains per thread, 8 blocks of 256 threads per SM, `iters` iterations,
 * timed with CUDA events on `stream` after one warm-up launch; writes the
 * rate (flop/s, an FMA counting two) and the launch time.  `scratch` is
 * device memory of lbm_fp64_fma_scratch_bytes() bytes.  The roof of the
 * FP64 paths (the parity form of the step), which GB300's FP64 rate bounds
 * before its HBM does.  No reference counterpart. */
int lbm_fp64_fma_scratch_bytes(size_t* bytes);
int lbm_fp64_fma_rate(double* scratch, int32_t iters, double* flops_per_s, float* ms, void* stream);

/* Block average of the interior populations over factor^dim nodes into a
 * dense float64 array out[nv][n0/factor][n1/factor][n2/factor] (physical
 * values, last axis contiguous): restriction of a fine run onto a coarse
 * lattice (training data of the learned closure; no reference counterpart). */
int lbm_restrict(const void* f, const lbm_lattice* lat, double* out, int32_t factor, void* stream);

/* FP64 sums over the interior nodes of every population (physical values),
 * the conservation diagnostic of the build (mass/momentum = M . sums).
 * `partials` is caller-provided device scratch of at least
 * lbm_population_sums_scratch_bytes() bytes.  sums (nv doubles) and
 * nonfinite (one int32, set to the number of blocks that saw a NaN/Inf) are
 * device pointers.  No reference counterpart: pylbm has no such check. */
int lbm_population_sums_scratch_bytes(const lbm_lattice* lat, size_t* bytes);
int lbm_population_sums(const void* f, const lbm_lattice* lat, double* sums, int32_t* nonfinite,
                        void* partials, size_t partials_bytes, void* stream);

/* Same sums for callers that cannot call cudaMalloc (a host application
 * whose memory manager owns every device allocation, or a time-critical loop
 * that cannot afford cudaMalloc's implicit synchronisation): the partial sums
 * live in a fixed 1 MiB device array inside the library (see
 * lbm_population_sums_noalloc_max_bytes), held by every GPU that loads the
 * library until exit.  Lattices whose partials exceed it are rejected with
 * LBM_ERR_ARG.  The first call on a device looks up the array's address for
 * that device; make it before any stream capture.  The address is kept with
 * the id of the context it belongs to, so after a device reset the first
 * call in the new context looks it up again (again before any capture).
 * All calls share the
 * array: calls that overlap on the GPU race.  Allocates nothing.
 * No counterpart in the reference (pylbm has no conservation check). */
int lbm_population_sums_noalloc(const void* f, const lbm_lattice* lat, double* sums,
                                int32_t* nonfinite, void* stream);
size_t lbm_population_sums_noalloc_max_bytes(void);

/* ------------------------------------------------------------------ */
/* Learned collision closure (no reference counterpart): a per-node    */
/* MLP x(16, 9 used) -> 64 SiLU -> 64 SiLU -> y(8, 6 used) evaluated on */
/* the tensor cores with BF16 operands and FP32 accumulation.           */
/* params: FP32 block of lbm_mlp_sizes().nparam floats                  */
/*   W1[64][16] b1[64] W2[64][64] b2[64] W3[8][64] b3[8]  (out x in);   */
/* wbf16: the BF16 copies the kernels read (lbm_mlp_sync_weights).      */
/* x: BF16 [n][16]; y, target: FP32 [n][8]; n a multiple of 16.         */
/* ------------------------------------------------------------------ */
int lbm_mlp_sizes(int32_t* nparam, int32_t* nweights_bf16);
int lbm_mlp_scratch_bytes(int32_t n, size_t* bytes);
int lbm_mlp_sync_weights(const float* params, void* wbf16, void* stream);
int lbm_mlp_forward(const void* x, int32_t n, const void* wbf16, const float* params, float* y, void* stream);
/* The same forward pass on the 5th-generation tensor cores: tiles of 128
 * samples, tcgen05.mma with the FP32 accumulators in tensor memory, BF16
 * weights from the FP32 master block params (rounded as
 * lbm_mlp_sync_weights rounds them); any n >= 0.  Outputs equal those of
 * lbm_mlp_forward up to the FP32 accumulation order inside a layer.
 * lbm_mlp_tc_timeouts reads the count of its bounded waits that gave up. */
int lbm_mlp_forward_tc(const void* x, int32_t n, const float* params, float* y, void* stream);
int lbm_mlp_tc_timeouts(uint32_t* count);
/* Adds dLoss/dparams to grad (FP32 atomics; zero it first) for the loss
 * mean over samples and the 6 used outputs of (y - target)^2; writes the
 * loss to *loss (device).  scratch: lbm_mlp_scratch_bytes(n) bytes. */
int lbm_mlp_gradients(const void* x, const float* target, int32_t n, const void* wbf16, const float* params,
                      float* grad, float* loss, void* scratch, size_t scratch_bytes, void* stream);
/* The same gradients and loss from one kernel on the 5th-generation tensor
 * cores: per 128-sample tile the forward pass, the loss, the backward pass
 * and the weight gradients run in shared and tensor memory (no scratch; the
 * gradients accumulate in tensor memory over a block's tiles and reach grad
 * once per block).  Any n > 0; the rounding points of lbm_mlp_gradients, the
 * FP32 accumulation order differs.  Bounded waits as lbm_mlp_forward_tc. */
int lbm_mlp_gradients_tc(const void* x, const float* target, int32_t n, const float* params, float* grad, float* loss,
                         void* stream);
/* Vector-Jacobian product of the MLP on the same tensor-core kernel: adds
 * to grad the gradient with respect to params of sum over samples of dy . y,
 * y the outputs lbm_mlp_forward_tc returns for x and dy (n x 8 FP32, the
 * first 6 columns used) a given gradient of some loss with respect to y;
 * *dot (device) receives sum dy . y.
 * This is the backward step of an MLP that sits inside a differentiated
 * computation (a training loss over several closure time steps); no
 * counterpart in pylbm, which has no learned closure (its relaxation is
 * pylbm/algorithm/base.py:404-428). */
int lbm_mlp_vjp_tc(const void* x, const float* dy, int32_t n, const float* params, float* grad, float* dot,
                   void* stream);
/* Adam update of params (moments m, v), zeroes grad, refreshes wbf16. */
int lbm_mlp_adam(float* params, float* m, float* v, float* grad, float lr, float beta1, float beta2, float eps,
                 int32_t step, void* wbf16, void* stream);

/* ------------------------------------------------------------------ */
/* lbm_scheme_<id>.so: per-scheme module (generated constants + the     */
/* kernel templates of pylbm_gb300/csrc/scheme_kernels.cuh)            */
/* ------------------------------------------------------------------ */

const char* lbm_scheme_last_error(void);

/* Number of populations, dimension, number of run-time parameters,
 * storage and compute types, and shift/mref (nv doubles each: the stored
 * shift feq(c0) and its moments). */
int lbm_scheme_describe(int32_t* nv, int32_t* dim, int32_t* nprm, int32_t* storage,
                        int32_t* compute, double* shift, double* mref);

/* One LBM step on the interior nodes: pull f_k(x - v_k), m = M f, relax
 * the non-conserved moments toward m_eq(conserved) at rates s, fnew = M^-1 m
 * (pylbm/algorithm/pull.py:11-59, pylbm/algorithm/base.py:551-600; generated
 * routine `one_time_step(f, fnew, nx, ny[, nz])`).  prm holds the run-time
 * parameters (free symbols of the scheme, sorted by name).  f must have its
 * ghost layers filled (lbm_update_halo + boundary kernels). */
int lbm_one_time_step(const void* f, void* fnew, const lbm_lattice* lat, const double* prm,
                      void* stream);

/* Same step for domains periodic along every axis: the pull wraps inside the
 * interior, ghost layers are neither read nor written (no halo pass). */
int lbm_one_time_step_periodic(const void* f, void* fnew, const lbm_lattice* lat,
                               const double* prm, void* stream);

/* One step on a box whose boundary links are all bounce-back links of its
 * walls (pylbm/boundary.py:400-469 applied in the pull): a wall node pulling
 * population k from beyond a wall takes f_k'(x) + table[k * 27 + sig] (k' =
 * sym[k], the opposite population; sig = 9 (o0+1) + 3 (o1+1) + (o2+1), o_d =
 * -1 / 0 / +1 where the source lies below / inside / above the interior along
 * axis d), rounded through the storage type: the same populations as the
 * boundary launch (lbm_boundary_batch, bounce-back links) followed by
 * lbm_one_time_step, bit for bit, in one launch that neither reads nor writes
 * ghost slots.  table: nv * 27 constants (host) in the boundary launch's
 * arithmetic (float64 right-hand sides, or for shifted storage the FP32
 * per-link constants of LBM_BC_FLOAT_FORM); one ghost layer per axis. */
int lbm_one_time_step_walls(const void* f, void* fnew, const lbm_lattice* lat, const double* prm,
                            const double* table, const int32_t* sym, void* stream);

/* Step kernel choice of this module: 1 runs periodic steps of 16-bit
 * storage in the staged kernel where the rows allow it (bulk copies of each
 * pulled row into shared memory on the TMA unit, ahead of the compute), 0
 * (default) the direct-load kernels; both give the same results bit for bit.
 * No reference counterpart. */
int lbm_scheme_set_step_variant(int32_t variant);
/* Blocks per SM of the tensor-core closure step
 * (lbm_one_time_step_periodic_closure_tc): 0 (default) takes the bound set
 * by the kernel's registers and shared memory, 1..8 a fixed count.  Either
 * is capped at 8, the tensor-memory allocations of 64 columns an SM holds at
 * once.  No reference counterpart. */
int lbm_scheme_set_closure_tc_occupancy(int32_t blocks_per_sm);
/* The resource bound for the current device and the blocks per SM the
 * launch uses. */
int lbm_scheme_closure_tc_occupancy(int32_t* bound, int32_t* used);
/* Number of bounded waits of this module's kernels that gave up (0 in a
 * healthy run; a kernel whose wait times out leaves without completing). */
int lbm_scheme_wait_timeouts(uint32_t* count);

/* Periodic step with the learned collision closure (no reference
 * counterpart): after the relaxation, the non-conserved moments k >= nconsm
 * receive corr_j = y_j * sig_out[j] + mu_out[j], y = MLP((m - mu_in) * isig_in)
 * of the node's pre-collision moments m.  norm (host, 48 floats): mu_in[16],
 * isig_in[16], mu_out[8], sig_out[8].  wbf16/params: the MLP blocks of
 * lbm_mlp_* (device).  guard (host, 2 floats, or NULL for none): a node
 * whose corrections are not all finite and within guard[0] * (the largest
 * change the relaxation made to its non-conserved moments) + guard[1] keeps
 * the plain MRT collision (bit for bit that of lbm_one_time_step_periodic)
 * and adds one to *fallbacks (device int32, or NULL).  rate (host, 16
 * floats, or NULL for the additive form above): the rate form, lo[8] then
 * hi[8] with -1 <= lo <= hi; output j then scales the relaxation's own
 * change of moment j, corr_j = lam_j * (m_relaxed_j - m_j) with
 * lam_j = lo[j] + (hi[j] - lo[j]) * sigmoid(y_j * sig_out[j] + mu_out[j]),
 * i.e. the node relaxes moment j at the rate s_j * (1 + lam_j), inside
 * bounds the caller chooses (effective rates below 2 keep the collision
 * stable).  grid > 0 caps the number of blocks (persistent loop).  Needs
 * nv <= 16 and nv - nconsm <= 8. */
int lbm_one_time_step_periodic_closure(const void* f, void* fnew, const lbm_lattice* lat, const double* prm,
                                       const void* wbf16, const float* params, const float* norm,
                                       const float* guard, const float* rate, int32_t* fallbacks, int32_t grid,
                                       void* stream);
/* The same step with the MLP on the 5th-generation tensor cores: 128 nodes
 * per block tile, one node per thread, the three layers as tcgen05 MMAs with
 * FP32 accumulators in tensor memory; BF16 weights from the FP32 master block
 * params (no BF16 copy needed).  Same guard, rate form and fallback count;
 * the corrections equal those of the warp-level kernel up to the FP32
 * accumulation order inside a layer. */
int lbm_one_time_step_periodic_closure_tc(const void* f, void* fnew, const lbm_lattice* lat, const double* prm,
                                          const float* params, const float* norm, const float* guard,
                                          const float* rate, int32_t* fallbacks, void* stream);

/* Pure pull streaming on the interior (pylbm/algorithm/base.py:289-296). */
int lbm_transport(const void* f, void* fnew, const lbm_lattice* lat, void* stream);

/* Moments of every node, halo included: m = M f (pylbm/algorithm/base.py:
 * 336-344).  m is float64 in its own lattice layout `mlat` (same n/halo). */
int lbm_f2m(const void* f, const lbm_lattice* lat, double* m, const lbm_lattice* mlat,
            void* stream);

/* The conserved moments alone (planes 0 .. nconsm-1 of m; the others are left
 * as they are): what output and conservation checks read, at a fraction of
 * the float64 arithmetic of lbm_f2m. */
int lbm_f2m_conserved(const void* f, const lbm_lattice* lat, double* m, const lbm_lattice* mlat, void* stream);

/* The conserved moments of the interior nodes written straight into a dense
 * float64 array out[c][i0][i1][i2] (nconsm planes, last axis fastest), in one
 * pass over the populations: the read of sim.m[rho] etc. without the moment
 * array (pylbm/simulation.py:216-224).  out may be device memory or
 * page-locked host memory mapped for the device (lbm_host_device_pointer). */
int lbm_f2m_conserved_dense(const void* f, const lbm_lattice* lat, double* out, void* stream);

/* Populations from moments: f = M^-1 m (pylbm/algorithm/base.py:346-379). */
int lbm_m2f(const double* m, const lbm_lattice* mlat, void* f, const lbm_lattice* lat,
            void* stream);

/* Non-conserved moments set to their equilibrium (pylbm/algorithm/base.py:
 * 381-402); conserved moments are inputs. */
int lbm_equilibrium(double* m, const lbm_lattice* mlat, const double* prm, void* stream);

/* Moment-space relaxation m <- m + s (m_eq - m) (pylbm/algorithm/base.py:404-437). */
int lbm_relaxation(double* m, const lbm_lattice* mlat, const double* prm, void* stream);

/* Populations at the equilibrium of the conserved moments (planes
 * 0..nconsm-1 of m, read only), over the whole halo box: pylbm's
 * initialisation, equilibrium then m2f (pylbm/simulation.py:258-320), in one
 * pass without writing the other moments.  Unshifted storage computes
 * exactly lbm_equilibrium followed by lbm_m2f; shifted storage evaluates the
 * equilibrium of the deviations in FP32. */
int lbm_init_conserved(const double* m, const lbm_lattice* mlat, void* f, const lbm_lattice* lat,
                       const double* prm, void* stream);

/* Source terms over half a time step on the interior nodes: each conserved
 * moment with a source gets m_c += dt/2 S_c(m) (explicit Euler,
 * pylbm/algorithm/base.py:439-504 and algorithm/ode.py:11-16; dt is the
 * run-time parameter "dt").  LBM_ERR_UNSUPPORTED for schemes without
 * source terms (pylbm generates no source_term routine for them). */
int lbm_source_term(double* m, const lbm_lattice* mlat, const double* prm, void* stream);

/* ------------------------------------------------------------------ */
/* Batched ensembles: many independent periodic simulations of one    */
/* scheme, each with its own grid size and run-time parameters, in one */
/* persistent launch per step.  No reference counterpart (pylbm runs   */
/* one simulation per process).                                        */
/* ------------------------------------------------------------------ */

#define LBM_MAX_PRM 8

typedef struct lbm_instance {
  int64_t offset[2];          /* element offsets of the two population buffers in the arena */
  int32_t n[3];               /* interior nodes per axis (1 beyond dim) */
  int32_t halo[3];            /* ghost layers per axis */
  int64_t stride[3];          /* as in lbm_lattice */
  int64_t vstride;
  int64_t origin;
  int32_t rows;               /* interior rows: product of n over all axes but the last */
  int32_t col_tiles;          /* tiles across the last axis: ceil(n_last / span) */
  int32_t tile_begin;         /* index of this instance's first tile */
  int32_t flags;              /* LBM_INSTANCE_* bits */
  double prm[LBM_MAX_PRM];    /* run-time parameters of this instance */
} lbm_instance;

/* A tile of this instance spans 2 x block nodes of the last axis (span =
 * 2 block, else span = block): each thread updates two neighbouring nodes.
 * Modules with 16-bit storage then load and store both nodes as one 32-bit
 * word and relax them with packed FP32x2 arithmetic when n_last, origin +
 * halo_last, vstride, the outer strides and both buffer offsets are even;
 * otherwise the thread updates the two nodes one after the other. */
#define LBM_INSTANCE_PAIRS 1

/* One periodic step of every instance.  `arena` holds all populations (the
 * storage type of the module), `inst` (device, ninst entries) describes them
 * and `tile_instance` (device, ntiles entries) maps each tile to its
 * instance; a tile is `rows_per_tile` rows x `span` consecutive nodes of the
 * last axis (span = block, or 2 x block with LBM_INSTANCE_PAIRS).  `parity`
 * selects which of the two buffers is read (then the other is written).
 * `grid` blocks of `block` threads (32 to LBM_ENSEMBLE_MAX_BLOCK, a multiple
 * of 32) stride over the tiles (grid = 0: one block per tile). */
#define LBM_ENSEMBLE_MAX_BLOCK 256
int lbm_ensemble_step(void* arena, const lbm_instance* inst, const int32_t* tile_instance, int32_t ntiles,
                      int32_t rows_per_tile, int32_t block, int32_t grid, int32_t parity, void* stream);

/* The same step when every instance carries LBM_INSTANCE_PAIRS (the caller
 * checks; 16-bit storage modules only): a kernel with the two-node path
 * alone, which needs fewer registers. */
int lbm_ensemble_step_pairs(void* arena, const lbm_instance* inst, const int32_t* tile_instance, int32_t ntiles,
                            int32_t rows_per_tile, int32_t block, int32_t grid, int32_t parity, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* LBM_GB300_H */
