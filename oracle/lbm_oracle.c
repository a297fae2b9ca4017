/*
 * lbm_oracle.c -- CPU restatement of pylbm's per-step hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker the GPU kernels are
 * compared with (tests/, __graft_entry__.smoke() and the CPU-baseline leg of
 * bench.py); the pylbm_gb300 package never links or calls it.
 *
 * Arrays follow the NumPy layout of pylbm's SOA container
 * (pylbm/storage.py:423): f[k][i0][i1][i2] with the last axis contiguous,
 * halo-extended (n[d] + 2*h[d] nodes per axis), no padding, float64.
 *
 * Every function restates one reference routine:
 *   oracle_update_halo   pylbm/storage.py:307-367   (Array.update: per axis, in
 *                        order x, y, z, full extent of the other axes, periodic)
 *   oracle_boundary      pylbm/boundary.py:430-464 / :646-680 / :787-818
 *                        (f[istore] = sign*f[iload0] + rhs, links in order)
 *   oracle_bouzidi       pylbm/boundary.py:472-623 / :687-760 (interpolated
 *                        bounce-back / anti-bounce-back)
 *   oracle_one_time_step pylbm/algorithm/pull.py:11-59 with
 *                        pylbm/algorithm/base.py:298-428: pull f(x - v_k),
 *                        m = M f, m_k = (1 - s_k) m_k + s_k meq_k(m_cons) for
 *                        every moment, fnew = M^-1 m, on the interior nodes
 *   oracle_f2m / _m2f    pylbm/algorithm/base.py:336-379 (whole halo box)
 *   oracle_equilibrium   pylbm/algorithm/base.py:381-402
 *
 * The equilibrium is passed as a table of monomials of the conserved moments
 * (exponents may be negative, e.g. qx^2 rho^-1):
 *   meq_k = sum_{t: term_row[t]==k} coef[t] * prod_c m_c^expo[t][c]
 * Conserved moments are the first ncons moments (pylbm/scheme.py:225-241)
 * and keep their value (their equilibrium is themselves).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORACLE_MAX_Q 64
#define ORACLE_MAX_CONS 8

typedef struct {
  int dim, nv, ncons;
  int n[3], h[3];
  long long ext[3];    /* n + 2h per axis (1 beyond dim) */
  long long stride[3]; /* element strides (last axis 1) */
  long long vstride;   /* elements per population */
} og;

static og make_geo(int dim, int nv, int ncons, const int* n, const int* h) {
  og g;
  memset(&g, 0, sizeof(g));
  g.dim = dim;
  g.nv = nv;
  g.ncons = ncons;
  for (int d = 0; d < 3; ++d) {
    g.n[d] = d < dim ? n[d] : 1;
    g.h[d] = d < dim ? h[d] : 0;
    g.ext[d] = g.n[d] + 2 * g.h[d];
  }
  g.stride[2] = 1;
  g.stride[1] = g.ext[2];
  g.stride[0] = g.ext[1] * g.ext[2];
  g.vstride = g.ext[0] * g.ext[1] * g.ext[2];
  /* express dims < 3 with the used axes first */
  if (dim == 2) {
    g.stride[0] = g.ext[1];
    g.stride[1] = 1;
    g.stride[2] = 0;
  } else if (dim == 1) {
    g.stride[0] = 1;
    g.stride[1] = 0;
    g.stride[2] = 0;
  }
  return g;
}

static inline long long off3(const og* g, long long i0, long long i1, long long i2) {
  return i0 * g->stride[0] + i1 * g->stride[1] + i2 * g->stride[2];
}

/* Array.update: for each axis d, the h[d] first ghost layers receive the
 * last h[d] interior layers and the last ghost layers the first interior
 * layers; the other axes are copied over their full (halo) extent. */
void oracle_update_halo(double* f, int dim, int nv, const int* n, const int* h) {
  og g = make_geo(dim, nv, 0, n, h);
  for (int d = 0; d < dim; ++d) {
    for (int k = 0; k < nv; ++k) {
      double* fk = f + (long long)k * g.vstride;
      for (long long i0 = 0; i0 < g.ext[0]; ++i0)
        for (long long i1 = 0; i1 < g.ext[1]; ++i1)
          for (long long i2 = 0; i2 < g.ext[2]; ++i2) {
            long long idx[3] = {i0, i1, i2};
            long long c = idx[d];
            long long src;
            if (c < g.h[d]) {
              src = c + g.n[d];
            } else if (c >= g.n[d] + g.h[d]) {
              src = c - g.n[d];
            } else {
              continue;
            }
            long long sidx[3] = {i0, i1, i2};
            sidx[d] = src;
            fk[off3(&g, idx[0], idx[1], idx[2])] = fk[off3(&g, sidx[0], sidx[1], sidx[2])];
          }
    }
  }
}

/* f[istore[c]] = sign * f[iload[c]] + rhs[c], c = 0..ncond-1 in order. */
void oracle_boundary(double* f, int dim, int nv, const int* n, const int* h, const int32_t* iload,
                     const int32_t* istore, int ncond, const double* rhs, double sign) {
  og g = make_geo(dim, nv, 0, n, h);
  const int w = dim + 1;
  for (int c = 0; c < ncond; ++c) {
    const int32_t* st = istore + (long long)c * w;
    const int32_t* ld = iload + (long long)c * w;
    long long is[3] = {0, 0, 0}, il[3] = {0, 0, 0};
    for (int d = 0; d < dim; ++d) {
      is[d] = st[1 + d];
      il[d] = ld[1 + d];
    }
    double v = sign * f[(long long)ld[0] * g.vstride + off3(&g, il[0], il[1], il[2])];
    if (rhs) v += rhs[c];
    f[(long long)st[0] * g.vstride + off3(&g, is[0], is[1], is[2])] = v;
  }
}

/* Bouzidi links (pylbm/boundary.py:570-618 and :707-756), in pylbm's printed
 * order ((1 - d) f1 +/- d f0) + rhs.  anti = 0: bounce-back, whose loads read
 * a copy of f taken before the method (pylbm/boundary.py:536-559, fcopy);
 * anti = 1: anti-bounce-back, loads and stores in f, links in order. */
void oracle_bouzidi(double* f, int dim, int nv, const int* n, const int* h, const int32_t* iload0,
                    const int32_t* iload1, const int32_t* istore, int ncond, const double* rhs,
                    const double* dist, int anti) {
  og g = make_geo(dim, nv, 0, n, h);
  const int w = dim + 1;
  const double* src = f;
  double* copy = NULL;
  if (!anti) {
    copy = (double*)malloc(sizeof(double) * (size_t)g.vstride * (size_t)nv);
    memcpy(copy, f, sizeof(double) * (size_t)g.vstride * (size_t)nv);
    src = copy;
  }
  for (int c = 0; c < ncond; ++c) {
    long long o[3];
    const int32_t* rows[3] = {iload0 + (long long)c * w, iload1 + (long long)c * w, istore + (long long)c * w};
    for (int r = 0; r < 3; ++r) {
      long long i[3] = {0, 0, 0};
      for (int d = 0; d < dim; ++d) i[d] = rows[r][1 + d];
      o[r] = (long long)rows[r][0] * g.vstride + off3(&g, i[0], i[1], i[2]);
    }
    const double d = dist[c];
    const double t1 = (1 - d) * src[o[1]];
    const double t0 = d * src[o[0]];
    f[o[2]] = (anti ? t1 - t0 : t1 + t0) + rhs[c];
  }
  free(copy);
}

typedef struct {
  int nterms;
  const int32_t* row;    /* moment index of each term */
  const double* coef;    /* coefficient */
  const int32_t* expo;   /* nterms x ncons exponents */
} oracle_eq;

static double ipow(double x, int e) {
  double r = 1.0;
  int a = e < 0 ? -e : e;
  for (int i = 0; i < a; ++i) r *= x;
  return e < 0 ? 1.0 / r : r;
}

static void equilibrium_node(const og* g, const oracle_eq* eq, const double* m, double* meq) {
  for (int k = 0; k < g->nv; ++k) meq[k] = 0.0;
  for (int t = 0; t < eq->nterms; ++t) {
    double v = eq->coef[t];
    for (int c = 0; c < g->ncons; ++c) {
      int e = eq->expo[(long long)t * g->ncons + c];
      if (e) v *= ipow(m[c], e);
    }
    meq[eq->row[t]] += v;
  }
  for (int c = 0; c < g->ncons; ++c) meq[c] = m[c];
}

/* One pull step on the interior nodes (every node, fluid or solid, as the
 * reference does with check_isfluid=False). */
void oracle_one_time_step(const double* f, double* fnew, int dim, int nv, int ncons, const int* n, const int* h,
                          const int32_t* vel /* nv x 3 */, const double* M, const double* invM,
                          const double* s, int nterms, const int32_t* eq_row, const double* eq_coef,
                          const int32_t* eq_expo, int nthreads) {
  og g = make_geo(dim, nv, ncons, n, h);
  oracle_eq eq = {nterms, eq_row, eq_coef, eq_expo};
  long long pull[ORACLE_MAX_Q];
  for (int k = 0; k < nv; ++k)
    pull[k] = (long long)k * g.vstride -
              ((long long)vel[3 * k] * g.stride[0] + (long long)vel[3 * k + 1] * g.stride[1] +
               (long long)vel[3 * k + 2] * g.stride[2]);
  (void)nthreads;
#pragma omp parallel for schedule(static) num_threads(nthreads > 0 ? nthreads : 1)
  for (long long i0 = g.h[0]; i0 < g.h[0] + g.n[0]; ++i0) {
    double fl[ORACLE_MAX_Q], m[ORACLE_MAX_Q], meq[ORACLE_MAX_Q];
    for (long long i1 = g.h[1]; i1 < g.h[1] + g.n[1]; ++i1)
      for (long long i2 = g.h[2]; i2 < g.h[2] + g.n[2]; ++i2) {
        long long o = off3(&g, i0, i1, i2);
        for (int k = 0; k < nv; ++k) fl[k] = f[o + pull[k]];
        for (int i = 0; i < nv; ++i) {
          double acc = 0.0;
          for (int k = 0; k < nv; ++k) acc += M[i * nv + k] * fl[k];
          m[i] = acc;
        }
        equilibrium_node(&g, &eq, m, meq);
        for (int i = 0; i < nv; ++i) m[i] = (1.0 - s[i]) * m[i] + s[i] * meq[i];
        for (int k = 0; k < nv; ++k) {
          double acc = 0.0;
          for (int i = 0; i < nv; ++i) acc += invM[k * nv + i] * m[i];
          fnew[(long long)k * g.vstride + o] = acc;
        }
      }
  }
}

/* m = M f on every node of the halo box. */
void oracle_f2m(const double* f, double* m, int dim, int nv, const int* n, const int* h, const double* M) {
  og g = make_geo(dim, nv, 0, n, h);
  for (long long o = 0; o < g.vstride; ++o)
    for (int i = 0; i < nv; ++i) {
      double acc = 0.0;
      for (int k = 0; k < nv; ++k) acc += M[i * nv + k] * f[(long long)k * g.vstride + o];
      m[(long long)i * g.vstride + o] = acc;
    }
}

/* f = M^-1 m on every node of the halo box. */
void oracle_m2f(const double* m, double* f, int dim, int nv, const int* n, const int* h, const double* invM) {
  oracle_f2m(m, f, dim, nv, n, h, invM);
}

/* non-conserved moments set to their equilibrium on every node. */
void oracle_equilibrium(double* m, int dim, int nv, int ncons, const int* n, const int* h, int nterms,
                        const int32_t* eq_row, const double* eq_coef, const int32_t* eq_expo) {
  og g = make_geo(dim, nv, ncons, n, h);
  oracle_eq eq = {nterms, eq_row, eq_coef, eq_expo};
  double mm[ORACLE_MAX_Q], meq[ORACLE_MAX_Q];
  for (long long o = 0; o < g.vstride; ++o) {
    for (int i = 0; i < nv; ++i) mm[i] = m[(long long)i * g.vstride + o];
    equilibrium_node(&g, &eq, mm, meq);
    for (int i = ncons; i < nv; ++i) m[(long long)i * g.vstride + o] = meq[i];
  }
}
