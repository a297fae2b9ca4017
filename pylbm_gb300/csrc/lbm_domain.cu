// Domain construction on the device: fluid/solid map, per-link wall
// distances and labels, and the boundary links they define.
//
// Same rules as the host Domain/Boundary (pylbm/domain.py:87-620,
// pylbm/boundary.py:23-160); every floating-point operation is written
// with an explicit IEEE intrinsic (no contraction) in the order the host
// evaluates it, so both give identical arrays.
#include "lbm_common.cuh"

using namespace lbm;

namespace {

constexpr int kThreads = 256;
constexpr double kValIn = 999.0;
constexpr double kValOut = -1.0;
constexpr double kFar = 1.0e16;  // "no intersection" of the element distance rules

__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dvd(double a, double b) { return __ddiv_rn(a, b); }

struct Box {
  int dim, nu;
  int n[3];
  long long stride[3];
  long long nodes;
};

inline Box make_box(const lbm_domain& d) {
  Box b;
  b.dim = d.dim;
  b.nu = d.nu;
  for (int k = 0; k < 3; ++k) b.n[k] = k < d.dim ? d.n[k] : 1;
  b.stride[2] = 1;
  b.stride[1] = b.n[2];
  b.stride[0] = (long long)b.n[1] * b.n[2];
  b.nodes = (long long)b.n[0] * b.n[1] * b.n[2];
  return b;
}

// node -> (i0, i1, i2) of the (up to) 3D box; unused axes have n = 1
__device__ __forceinline__ void unflatten(const Box& b, long long node, int (&i)[3]) {
  i[2] = (int)(node % b.n[2]);
  long long r = node / b.n[2];
  i[1] = (int)(r % b.n[1]);
  i[0] = (int)(r / b.n[1]);
}

// ------------------------------------------------------------------ reset
__global__ void k_reset(Box b, lbm_domain d, double* ioo, double* dist, int* flag) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= b.nodes) return;
  int i[3];
  unflatten(b, t, i);
  bool inner = true;
  for (int a = 0; a < b.dim; ++a) inner = inner && i[a] >= d.halo[a] && i[a] < b.n[a] - d.halo[a];
  ioo[t] = inner ? kValIn : kValOut;
  for (int u = 0; u < b.nu; ++u) {
    dist[u * b.nodes + t] = kValIn;
    flag[u * b.nodes + t] = 999;
  }
}

// ------------------------------------------------------------------ box walls
struct BoxLabels {
  int label[6];
};

// one thread per (u, node): the candidates of the axes in order, strict "shorter" rule
__global__ void k_box(Box b, lbm_domain d, BoxLabels L, double* dist, int* flag) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= b.nodes * b.nu) return;
  const int u = (int)(t / b.nodes);
  const long long node = t - (long long)u * b.nodes;
  int i[3];
  unflatten(b, node, i);
  for (int a = 0; a < b.dim; ++a)
    if (i[a] < d.halo[a] || i[a] >= b.n[a] - d.halo[a]) return;  // interior nodes only
  double dv = dist[t];
  int fv = flag[t];
  for (int a = 0; a < b.dim; ++a) {
    const int c = d.vel[u][a];
    const int nin = b.n[a] - 2 * d.halo[a];
    const int ia = i[a] - d.halo[a];
    if (c < 0 && L.label[2 * a] != -2) {
      if (ia < -c) {
        const double dd = dvd(add((double)ia, 0.5), (double)(-c));
        if (dv > dd) {
          dv = dd;
          fv = L.label[2 * a];
        }
      }
    } else if (c > 0 && L.label[2 * a + 1] != -2) {
      const int from_end = nin - 1 - ia;
      if (from_end < c) {
        const double dd = dvd(add((double)from_end, 0.5), (double)c);
        if (dv > dd) {
          dv = dd;
          fv = L.label[2 * a + 1];
        }
      }
    }
  }
  dist[t] = dv;
  flag[t] = fv;
}

// ------------------------------------------------------------------ elements
struct Region {
  int lo[3], hi[3];
  long long nodes;
};

__device__ __forceinline__ void region_node(const Region& r, long long t, int (&i)[3]) {
  const int n1 = r.hi[1] - r.lo[1], n2 = r.hi[2] - r.lo[2];
  i[2] = r.lo[2] + (int)(t % n2);
  const long long q = t / n2;
  i[1] = r.lo[1] + (int)(q % n1);
  i[0] = r.lo[0] + (int)(q / n1);
}

// cxx X^2 + cyy Y^2 + czz Z^2 + cxy XY + cyz YZ + czx ZX, left to right
// (ellipsoid coefficients p[3..8])
__device__ __forceinline__ double quadric_form(const lbm_element& e, double X, double Y, double Z) {
  return add(add(add(add(add(mul(e.p[3], mul(X, X)), mul(e.p[4], mul(Y, Y))), mul(e.p[5], mul(Z, Z))),
                     mul(mul(e.p[6], X), Y)),
                 mul(mul(e.p[7], Y), Z)),
             mul(mul(e.p[8], Z), X));
}

// (x, y, z) in a cylinder's frame: the inverse frame matrix p[3..11] applied
// to the offset from the centre p[0..2]
__device__ __forceinline__ void to_frame(const lbm_element& e, double x, double y, double z, double (&f)[3]) {
  const double xx = sub(x, e.p[0]), yy = sub(y, e.p[1]), zz = sub(z, e.p[2]);
  for (int r = 0; r < 3; ++r)
    f[r] = add(add(mul(e.p[3 + 3 * r], xx), mul(e.p[4 + 3 * r], yy)), mul(e.p[5 + 3 * r], zz));
}

// the cylinder's section in its frame: unit disc, unit triangle, unit square
__device__ __forceinline__ bool section_inside(int section, double x, double y) {
  if (section == 0) return add(mul(x, x), mul(y, y)) <= 1.0;
  if (section == 1) return x >= 0 && y >= 0 && add(x, y) <= 1;
  return x >= 0 && y >= 0 && x <= 1 && y <= 1;
}

__device__ __forceinline__ bool inside(const lbm_element& e, double x, double y, double z) {
  if (e.kind == LBM_ELEMENT_SPHERE) {
    const double px = sub(x, e.p[0]), py = sub(y, e.p[1]), pz = sub(z, e.p[2]);
    return add(add(mul(px, px), mul(py, py)), mul(pz, pz)) <= mul(e.p[3], e.p[3]);
  }
  if (e.kind == LBM_ELEMENT_CIRCLE) {
    const double px = sub(x, e.p[0]), py = sub(y, e.p[1]);
    return add(mul(px, px), mul(py, py)) <= mul(e.p[2], e.p[2]);
  }
  if (e.kind == LBM_ELEMENT_ELLIPSE) {
    const double px = sub(x, e.p[0]), py = sub(y, e.p[1]);
    return sub(add(mul(mul(px, px), e.p[3]), mul(mul(py, py), e.p[2])), mul(mul(px, py), e.p[4])) <= e.p[5];
  }
  if (e.kind == LBM_ELEMENT_ELLIPSOID) {
    const double X = sub(x, e.p[0]), Y = sub(y, e.p[1]), Z = sub(z, e.p[2]);
    return quadric_form(e, X, Y, Z) <= e.p[9];
  }
  if (e.kind == LBM_ELEMENT_CYLINDER) {
    double f[3];
    to_frame(e, x, y, z, f);
    return section_inside((int)e.p[12], f[0], f[1]) && fabs(f[2]) <= 1.0;
  }
  // parallelogram and triangle: barycentric coordinates in (v1, v2)
  const double dx = sub(x, e.p[0]), dy = sub(y, e.p[1]);
  const double inv = dvd(1.0, sub(mul(e.p[2], e.p[5]), mul(e.p[3], e.p[4])));
  const double a = mul(sub(mul(dx, e.p[5]), mul(dy, e.p[4])), inv);
  const double bb = mul(sub(mul(dy, e.p[2]), mul(dx, e.p[3])), inv);
  if (e.kind == LBM_ELEMENT_TRIANGLE) return a >= 0 && bb >= 0 && add(a, bb) <= 1;
  return a >= 0 && bb >= 0 && a <= 1 && bb <= 1;
}

// First crossing of the ray (x, y[, z]) + t v, t in (0, dmax], with the
// element boundary: t (or -1) and the label of the crossed edge (or -1).

// roots of the ellipse rule (pylbm/elements/utils.py:93-150): the smallest
// non-negative root of qa t^2 + qb t + qc, none when qa == 0
__device__ __forceinline__ double ellipse_crossing(double px, double py, double vx, double vy, double sxx,
                                                  double syy, double sxy, double det2, double qa, double dmax,
                                                  int label, int& border) {
  const double qb = sub(add(mul(mul(mul(2.0, px), vx), syy), mul(mul(mul(2.0, py), vy), sxx)),
                        mul(add(mul(px, vy), mul(py, vx)), sxy));
  const double qc = sub(sub(add(mul(mul(px, px), syy), mul(mul(py, py), sxx)), mul(mul(px, py), sxy)), det2);
  const double disc = sub(mul(qb, qb), mul(mul(4.0, qa), qc));
  const bool ok = disc >= 0;
  const double root = __dsqrt_rn(ok ? disc : 0.0);
  double t1 = kFar, t2 = kFar;
  if (qa != 0) {
    t1 = ok ? dvd(sub(-qb, root), mul(2.0, qa)) : kFar;
    t2 = ok ? dvd(add(-qb, root), mul(2.0, qa)) : kFar;
  }
  if (t1 < 0) t1 = kFar;
  if (t2 < 0) t2 = kFar;
  double t = ok ? fmin(t1, t2) : -1.0;
  if (t == kFar) t = -1.0;
  border = -1;
  if (t > 0 && t <= dmax) {
    border = label;
    return t;
  }
  return -1.0;
}

// segments q_k + s w_k, s in [0, 1], tried in order, a later one winning only
// when strictly closer (pylbm/elements/utils.py:21-90)
__device__ __forceinline__ double lines_crossing(double px, double py, double vx, double vy, int n,
                                                const double (*q)[2], const double (*w)[2], const int* labels,
                                                double dmax, int& border) {
  double alpha = kFar;
  border = -1;
  for (int k = 0; k < n; ++k) {
    const double det = sub(mul(vy, w[k][0]), mul(vx, w[k][1]));
    if (det == 0) continue;
    const double inv = dvd(1.0, det);
    const double c1 = sub(q[k][0], px), c2 = sub(q[k][1], py);
    const double t = mul(add(mul(-w[k][1], c1), mul(w[k][0], c2)), inv);
    const double s = mul(add(mul(-vy, c1), mul(vx, c2)), inv);
    if (t > 0 && s >= 0 && s <= 1 && t <= dmax && alpha > t) {
      alpha = t;
      border = labels[k];
    }
  }
  if (alpha == kFar) {
    border = -1;
    return -1.0;
  }
  return alpha;
}

// the ellipsoid rule (pylbm/elements/utils.py:160-230): quadratic
// coefficient qa and linear factors (bx, by, bz) of the ray, implicit-form
// coefficients c[0..5] = cxx, cyy, czz, cxy, cyz, czx and right side dd
__device__ __forceinline__ double quadric_crossing(double X, double Y, double Z, const double (&c)[6], double dd,
                                                  double qa, double bx, double by, double bz, double dmax,
                                                  int label, int& border) {
  const double qb = add(add(mul(bx, X), mul(by, Y)), mul(bz, Z));
  const double qc =
      sub(add(add(add(add(add(mul(c[0], mul(X, X)), mul(c[1], mul(Y, Y))), mul(c[2], mul(Z, Z))), mul(mul(c[3], X), Y)),
                  mul(mul(c[4], Y), Z)),
              mul(mul(c[5], Z), X)),
          dd);
  double disc = sub(mul(qb, qb), mul(mul(4.0, qa), qc));
  const bool ok = disc >= 0;
  double t1 = kFar, t2 = kFar;
  if (ok) {
    disc = __dsqrt_rn(disc);
    t1 = dvd(sub(-qb, disc), mul(2.0, qa));
    t2 = dvd(add(-qb, disc), mul(2.0, qa));
  }
  if (t1 < 0) t1 = kFar;
  if (t2 < 0) t2 = kFar;
  double t = ok ? fmin(t1, t2) : -1.0;
  if (t == kFar) t = -1.0;
  border = -1;
  if (t > 0 && t <= dmax) {
    border = label;
    return t;
  }
  return -1.0;
}

// the sphere as the host evaluates the ellipsoid quadratic with the
// semi-axes r e_x, r e_y, r e_z (cross products, then the coefficients, term
// by term in the host's order)
__device__ __forceinline__ double sphere_crossing(const lbm_element& e, double x, double y, double z, double v0,
                                                 double v1, double v2, double dmax, int& border) {
  const double r = e.p[3];
  const double a[3] = {mul(r, 1.0), mul(r, 0.0), mul(r, 0.0)};
  const double b[3] = {mul(r, 0.0), mul(r, 1.0), mul(r, 0.0)};
  const double c[3] = {mul(r, 0.0), mul(r, 0.0), mul(r, 1.0)};
  auto cross = [](const double (&u)[3], const double (&w)[3], double (&out)[3]) {
    out[0] = sub(mul(u[1], w[2]), mul(u[2], w[1]));
    out[1] = sub(mul(u[2], w[0]), mul(u[0], w[2]));
    out[2] = sub(mul(u[0], w[1]), mul(u[1], w[0]));
  };
  double c12[3], c23[3], c31[3];
  cross(a, b, c12);
  cross(b, c, c23);
  cross(c, a, c31);
  const double in = add(add(mul(a[0], c23[0]), mul(a[1], c23[1])), mul(a[2], c23[2]));
  const double dd = mul(in, in);
  double co[6];
  co[0] = add(add(mul(c12[0], c12[0]), mul(c23[0], c23[0])), mul(c31[0], c31[0]));
  co[1] = add(add(mul(c12[1], c12[1]), mul(c23[1], c23[1])), mul(c31[1], c31[1]));
  co[2] = add(add(mul(c12[2], c12[2]), mul(c23[2], c23[2])), mul(c31[2], c31[2]));
  co[3] = mul(2.0, add(add(mul(c12[0], c12[1]), mul(c23[0], c23[1])), mul(c31[0], c31[1])));
  co[4] = mul(2.0, add(add(mul(c12[1], c12[2]), mul(c23[1], c23[2])), mul(c31[1], c31[2])));
  co[5] = mul(2.0, add(add(mul(c12[2], c12[0]), mul(c23[2], c23[0])), mul(c31[2], c31[0])));
  const double qa = add(add(add(add(add(mul(co[0], mul(v0, v0)), mul(co[1], mul(v1, v1))), mul(co[2], mul(v2, v2))),
                                mul(mul(co[3], v0), v1)),
                            mul(mul(co[4], v1), v2)),
                        mul(mul(co[5], v2), v0));
  const double bx = add(add(mul(mul(2.0, co[0]), v0), mul(co[3], v1)), mul(co[5], v2));
  const double by = add(add(mul(mul(2.0, co[1]), v1), mul(co[4], v2)), mul(co[3], v0));
  const double bz = add(add(mul(mul(2.0, co[2]), v2), mul(co[5], v0)), mul(co[4], v1));
  return quadric_crossing(sub(x, e.p[0]), sub(y, e.p[1]), sub(z, e.p[2]), co, dd, qa, bx, by, bz, dmax, e.label[0],
                          border);
}

__device__ __forceinline__ double ellipsoid_crossing(const lbm_element& e, double x, double y, double z, int u,
                                                    double dmax, int& border) {
  const double co[6] = {e.p[3], e.p[4], e.p[5], e.p[6], e.p[7], e.p[8]};
  return quadric_crossing(sub(x, e.p[0]), sub(y, e.p[1]), sub(z, e.p[2]), co, e.p[9], e.vq[u][0], e.vq[u][1],
                          e.vq[u][2], e.vq[u][3], dmax, e.label[0], border);
}

// a cylinder (pylbm/elements/cylinder.py:104-216): in its frame, the side is
// the section's boundary crossed between the caps z = -1 and z = 1, the caps
// count where the crossing lies in the section; the first of the three wins
// (ties: bottom, then top, then side)
__device__ __forceinline__ double cylinder_crossing(const lbm_element& e, double x, double y, double z, int u,
                                                   double dmax, int& border) {
  double f[3];
  to_frame(e, x, y, z, f);
  const double vx = e.vq[u][0], vy = e.vq[u][1], vz = e.vq[u][2];
  const int section = (int)e.p[12];
  const int sides = section == 0 ? 1 : (section == 1 ? 3 : 4);
  double alpha;
  if (section == 0) {
    alpha = ellipse_crossing(sub(f[0], 0.0), sub(f[1], 0.0), vx, vy, 1.0, 1.0, 0.0, 1.0, e.vq[u][3], dmax,
                             e.label[0], border);
  } else {
    const double tq[3][2] = {{0, 0}, {0, 0}, {1, 0}}, tw[3][2] = {{1, 0}, {0, 1}, {-1, 1}};
    const double sq[4][2] = {{0, 0}, {0, 0}, {1, 0}, {0, 1}}, sw[4][2] = {{1, 0}, {0, 1}, {0, 1}, {1, 0}};
    alpha = lines_crossing(f[0], f[1], vx, vy, sides, section == 1 ? tq : sq, section == 1 ? tw : sw, e.label, dmax,
                           border);
  }
  if (alpha < 0) alpha = kFar;
  if (alpha > 0 && fabs(add(f[2], mul(alpha, vz))) > 1.0) {
    alpha = kFar;
    border = -1;
  }
  const double den = add(vz, vz == 0 ? 1.0e-16 : 0.0);
  double top = dvd(sub(1.0, f[2]), den);
  if (top < 0 || top > dmax || !section_inside(section, add(f[0], mul(top, vx)), add(f[1], mul(top, vy))))
    top = kFar;
  double bottom = dvd(-add(1.0, f[2]), den);
  if (bottom < 0 || bottom > dmax ||
      !section_inside(section, add(f[0], mul(bottom, vx)), add(f[1], mul(bottom, vy))))
    bottom = kFar;
  alpha = fmin(fmin(alpha, top), bottom);
  if (alpha == top) border = e.label[sides + 1];
  if (alpha == bottom) border = e.label[sides];
  return alpha == kFar ? -1.0 : alpha;
}

__device__ __forceinline__ double crossing(const lbm_element& e, double x, double y, double vx, double vy, int u,
                                          double dmax, int& border) {
  border = -1;
  if (e.kind == LBM_ELEMENT_CIRCLE) {
    // ellipse {c + cos(a) v1 + sin(a) v2} with v1 = (r, 0), v2 = (0, r)
    const double r = e.p[2];
    const double v1x = mul(r, 1.0), v1y = mul(r, 0.0), v2x = mul(r, 0.0), v2y = mul(r, 1.0);
    const double sxx = add(mul(v1x, v1x), mul(v2x, v2x));
    const double syy = add(mul(v1y, v1y), mul(v2y, v2y));
    const double sxy = mul(2.0, add(mul(v1x, v1y), mul(v2x, v2y)));
    const double det = sub(mul(v1x, v2y), mul(v1y, v2x));
    const double qa = sub(add(mul(mul(vx, vx), syy), mul(mul(vy, vy), sxx)), mul(mul(vx, vy), sxy));
    return ellipse_crossing(sub(x, e.p[0]), sub(y, e.p[1]), vx, vy, sxx, syy, sxy, mul(det, det), qa, dmax,
                            e.label[0], border);
  }
  if (e.kind == LBM_ELEMENT_ELLIPSE)
    return ellipse_crossing(sub(x, e.p[0]), sub(y, e.p[1]), vx, vy, e.p[2], e.p[3], e.p[4], e.p[5], e.vq[u][0], dmax,
                            e.label[0], border);
  const double px = sub(x, e.p[0]), py = sub(y, e.p[1]);
  if (e.kind == LBM_ELEMENT_TRIANGLE) {
    // edges from the point along v1 and v2, then from v1 along v2 - v1
    const double q[3][2] = {{0.0, 0.0}, {0.0, 0.0}, {e.p[2], e.p[3]}};
    const double w[3][2] = {{e.p[2], e.p[3]}, {e.p[4], e.p[5]}, {sub(e.p[4], e.p[2]), sub(e.p[5], e.p[3])}};
    return lines_crossing(px, py, vx, vy, 3, q, w, e.label, dmax, border);
  }
  // parallelogram: the four edges point + s w, s in [0, 1], in the host order
  const double q[4][2] = {{0.0, 0.0}, {0.0, 0.0}, {e.p[4], e.p[5]}, {e.p[2], e.p[3]}};
  const double w[4][2] = {{e.p[2], e.p[3]}, {e.p[4], e.p[5]}, {e.p[2], e.p[3]}, {e.p[4], e.p[5]}};
  return lines_crossing(px, py, vx, vy, 4, q, w, e.label, dmax, border);
}

__device__ __forceinline__ long long box_offset(const Box& b, const int (&i)[3]) {
  return (long long)i[0] * b.stride[0] + (long long)i[1] * b.stride[1] + i[2];
}

__global__ void k_element_map(Box b, Region r, lbm_element e, const double* __restrict__ c0,
                              const double* __restrict__ c1, const double* __restrict__ c2, double* ioo) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= r.nodes) return;
  int i[3];
  region_node(r, t, i);
  const bool in = inside(e, c0[i[0]], c1[i[1]], c2 ? c2[i[2]] : 0.0);
  if (in) ioo[box_offset(b, i)] = e.isfluid ? kValIn : kValOut;
}

__global__ void k_element_links(Box b, lbm_domain d, Region r, lbm_element e, const double* __restrict__ c0,
                                const double* __restrict__ c1, const double* __restrict__ c2,
                                const double* __restrict__ ioo, double* dist, int* flag) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= r.nodes * b.nu) return;
  const int u = (int)(t / r.nodes);
  const int vx = d.vel[u][0], vy = d.vel[u][1], vz = d.vel[u][2];
  if (vx == 0 && vy == 0 && vz == 0) return;
  int i[3];
  region_node(r, t - (long long)u * r.nodes, i);
  const double x = c0[i[0]], y = c1[i[1]], z = c2 ? c2[i[2]] : 0.0;
  const bool in = inside(e, x, y, z);
  const bool solid = e.isfluid ? !in : in;
  const long long o = box_offset(b, i);
  int j[3] = {i[0] + vx, i[1] + vy, i[2] + vz};
  const bool out = ioo[box_offset(b, j)] == kValOut;
  int border;
  double alpha;
  if (e.kind == LBM_ELEMENT_SPHERE)
    alpha = sphere_crossing(e, x, y, z, mul(d.dx, (double)vx), mul(d.dx, (double)vy), mul(d.dx, (double)vz), 1.0,
                            border);
  else if (e.kind == LBM_ELEMENT_ELLIPSOID)
    alpha = ellipsoid_crossing(e, x, y, z, u, 1.0, border);
  else if (e.kind == LBM_ELEMENT_CYLINDER)
    alpha = cylinder_crossing(e, x, y, z, u, 1.0, border);
  else
    alpha = crossing(e, x, y, mul(d.dx, (double)vx), mul(d.dx, (double)vy), u, 1.0, border);
  const bool sel = alpha > 0 && !solid && out;
  double dk = dist[(long long)u * b.nodes + o];
  int fk = flag[(long long)u * b.nodes + o];
  if (e.isfluid) {
    if (!out && ioo[o] == kValIn) {
      dk = kValIn;
      fk = 999;
    }
  } else if (solid) {
    dk = kValIn;
    fk = 999;
  }
  const bool keep = e.isfluid ? (alpha > dk || dk == kValIn) : (alpha < dk);
  if (sel && keep) {
    dk = alpha;
    fk = border;
  }
  dist[(long long)u * b.nodes + o] = dk;
  flag[(long long)u * b.nodes + o] = fk;
}

__global__ void k_clean(Box b, const double* __restrict__ ioo, double* dist, int* flag) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= b.nodes * b.nu) return;
  const long long node = t % b.nodes;
  if (ioo[node] == kValOut && dist[t] > 0) {
    dist[t] = kValIn;
    flag[t] = 999;
  }
}

// ------------------------------------------------------------------ link lists
__global__ void __launch_bounds__(kThreads) k_links_count(Box b, const int* __restrict__ flag, int u, int label,
                                                          int* counts) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const bool hit = t < b.nodes && flag[(long long)u * b.nodes + t] == label;
  const int c = __syncthreads_count(hit);
  if (threadIdx.x == 0) counts[blockIdx.x] = c;
}

__global__ void __launch_bounds__(kThreads) k_links_fill(Box b, const int* __restrict__ flag,
                                                         const double* __restrict__ dist, int u, int label,
                                                         int3 vsym, const int* __restrict__ offsets, int* rows,
                                                         double* out_dist) {
  __shared__ int warp_total[kThreads / 32];
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const bool hit = t < b.nodes && flag[(long long)u * b.nodes + t] == label;
  const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned ballot = __ballot_sync(0xffffffffu, hit);
  if (lane == 0) warp_total[warp] = __popc(ballot);
  __syncthreads();
  int before = 0;
  for (unsigned w = 0; w < warp; ++w) before += warp_total[w];
  if (!hit) return;
  const int pos = offsets[blockIdx.x] + before + __popc(ballot & ((1u << lane) - 1u));
  int i[3];
  unflatten(b, t, i);
  const int vs[3] = {vsym.x, vsym.y, vsym.z};
  for (int a = 0; a < b.dim; ++a) rows[(long long)pos * b.dim + a] = i[a] + vs[a];
  out_dist[pos] = dist[(long long)u * b.nodes + t];
}

int check_domain(const lbm_domain* d, const char* who) {
  if (!d) return fail(LBM_ERR_ARG, "%s: NULL domain", who);
  if (d->dim < 1 || d->dim > 3 || d->nu < 1 || d->nu > LBM_MAX_Q)
    return fail(LBM_ERR_ARG, "%s: dim=%d nu=%d", who, d->dim, d->nu);
  for (int a = 0; a < 3; ++a) {
    if (d->n[a] < 1 || (a >= d->dim && d->n[a] != 1)) return fail(LBM_ERR_ARG, "%s: n[%d]=%d", who, a, d->n[a]);
    if (a < d->dim && (d->halo[a] < 1 || 2 * d->halo[a] >= d->n[a]))
      return fail(LBM_ERR_ARG, "%s: halo[%d]=%d for n=%d", who, a, d->halo[a], d->n[a]);
  }
  for (int u = 0; u < d->nu; ++u)
    for (int a = 0; a < 3; ++a) {
      const int reach = a < d->dim ? d->halo[a] : 0;
      if (d->vel[u][a] < -reach || d->vel[u][a] > reach)
        return fail(LBM_ERR_ARG, "%s: velocity %d reaches beyond the halo", who, u);
    }
  return LBM_OK;
}

inline unsigned blocks_for(long long n) { return (unsigned)((n + kThreads - 1) / kThreads); }

}  // namespace

extern "C" {

int32_t lbm_links_block(void) { return kThreads; }

int lbm_domain_reset(const lbm_domain* d, double* in_or_out, double* distance, int32_t* flag, void* stream) {
  int rc = check_domain(d, "lbm_domain_reset");
  if (rc) return rc;
  if (!in_or_out || !distance || !flag) return fail(LBM_ERR_ARG, "lbm_domain_reset: NULL array");
  Box b = make_box(*d);
  k_reset<<<blocks_for(b.nodes), kThreads, 0, (cudaStream_t)stream>>>(b, *d, in_or_out, distance, flag);
  return launch_check("lbm_domain_reset");
}

int lbm_domain_box(const lbm_domain* d, const int32_t* box_label, double* distance, int32_t* flag, void* stream) {
  int rc = check_domain(d, "lbm_domain_box");
  if (rc) return rc;
  if (!box_label || !distance || !flag) return fail(LBM_ERR_ARG, "lbm_domain_box: NULL argument");
  Box b = make_box(*d);
  BoxLabels L;
  for (int k = 0; k < 6; ++k) L.label[k] = k < 2 * d->dim ? box_label[k] : -2;
  k_box<<<blocks_for(b.nodes * b.nu), kThreads, 0, (cudaStream_t)stream>>>(b, *d, L, distance, flag);
  return launch_check("lbm_domain_box");
}

int lbm_domain_element(const lbm_domain* d, const lbm_element* e, const double* coords, double* in_or_out,
                       double* distance, int32_t* flag, void* stream) {
  int rc = check_domain(d, "lbm_domain_element");
  if (rc) return rc;
  if (!e || !coords || !in_or_out || !distance || !flag) return fail(LBM_ERR_ARG, "lbm_domain_element: NULL argument");
  if (e->kind < LBM_ELEMENT_CIRCLE || e->kind > LBM_ELEMENT_CYLINDER)
    return fail(LBM_ERR_ARG, "lbm_domain_element: kind %d", e->kind);
  if (e->kind == LBM_ELEMENT_CYLINDER && (e->p[12] < 0 || e->p[12] > 2))
    return fail(LBM_ERR_ARG, "lbm_domain_element: cylinder section %g", e->p[12]);
  const bool solid3d =
      e->kind == LBM_ELEMENT_SPHERE || e->kind == LBM_ELEMENT_ELLIPSOID || e->kind == LBM_ELEMENT_CYLINDER;
  if (d->dim != (solid3d ? 3 : 2))
    return fail(LBM_ERR_UNSUPPORTED, "lbm_domain_element: element kind %d on a %dD domain", e->kind, d->dim);
  Region r;
  r.nodes = 1;
  for (int a = 0; a < 3; ++a) {
    r.lo[a] = a < d->dim ? e->lo[a] : 0;
    r.hi[a] = a < d->dim ? e->hi[a] : 1;
    // the region stays in the interior, so node + v stays in the box
    if (a < d->dim && (r.lo[a] < d->halo[a] || r.hi[a] > d->n[a] - d->halo[a]))
      return fail(LBM_ERR_ARG, "lbm_domain_element: region [%d, %d) outside the interior of axis %d", r.lo[a],
                  r.hi[a], a);
    if (r.hi[a] <= r.lo[a]) return LBM_OK;
    r.nodes *= r.hi[a] - r.lo[a];
  }
  Box b = make_box(*d);
  cudaStream_t s = (cudaStream_t)stream;
  const double* c0 = coords;
  const double* c1 = coords + d->n[0];
  const double* c2 = d->dim == 3 ? coords + d->n[0] + d->n[1] : nullptr;
  k_element_map<<<blocks_for(r.nodes), kThreads, 0, s>>>(b, r, *e, c0, c1, c2, in_or_out);
  rc = launch_check("lbm_domain_element");
  if (rc) return rc;
  k_element_links<<<blocks_for(r.nodes * b.nu), kThreads, 0, s>>>(b, *d, r, *e, c0, c1, c2, in_or_out, distance,
                                                                  flag);
  return launch_check("lbm_domain_element");
}

int lbm_domain_clean(const lbm_domain* d, const double* in_or_out, double* distance, int32_t* flag, void* stream) {
  int rc = check_domain(d, "lbm_domain_clean");
  if (rc) return rc;
  if (!in_or_out || !distance || !flag) return fail(LBM_ERR_ARG, "lbm_domain_clean: NULL array");
  Box b = make_box(*d);
  k_clean<<<blocks_for(b.nodes * b.nu), kThreads, 0, (cudaStream_t)stream>>>(b, in_or_out, distance, flag);
  return launch_check("lbm_domain_clean");
}

int lbm_links_count(const lbm_domain* d, const int32_t* flag, int32_t u, int32_t label, int32_t* block_counts,
                    void* stream) {
  int rc = check_domain(d, "lbm_links_count");
  if (rc) return rc;
  if (!flag || !block_counts || u < 0 || u >= d->nu) return fail(LBM_ERR_ARG, "lbm_links_count: bad argument");
  Box b = make_box(*d);
  k_links_count<<<blocks_for(b.nodes), kThreads, 0, (cudaStream_t)stream>>>(b, flag, u, label, block_counts);
  return launch_check("lbm_links_count");
}

int lbm_links_fill(const lbm_domain* d, const int32_t* flag, const double* distance, int32_t u, int32_t label,
                   const int32_t* vsym, const int32_t* block_offsets, int32_t* rows, double* dist, void* stream) {
  int rc = check_domain(d, "lbm_links_fill");
  if (rc) return rc;
  if (!flag || !distance || !vsym || !block_offsets || !rows || !dist || u < 0 || u >= d->nu)
    return fail(LBM_ERR_ARG, "lbm_links_fill: bad argument");
  Box b = make_box(*d);
  int3 vs = make_int3(vsym[0], d->dim > 1 ? vsym[1] : 0, d->dim > 2 ? vsym[2] : 0);
  k_links_fill<<<blocks_for(b.nodes), kThreads, 0, (cudaStream_t)stream>>>(b, flag, distance, u, label, vs,
                                                                          block_offsets, rows, dist);
  return launch_check("lbm_links_fill");
}

}  // extern "C"
