"""Geometric elements used to build the solid/fluid map of a domain.

The reference describes obstacles by elements with ``get_bounds``,
``point_inside`` and a ray distance ``distance(grid, v, dmax)`` returning the
fraction of the lattice link before the wall and the wall label
(pylbm/elements/circle.py:24, pylbm/elements/utils.py:93 ``distance_ellipse``;
pylbm/elements/parallelogram.py:21 with utils.py:40 ``distance_lines``).
Boundary link lists are derived from those distances, so the ray/obstacle
intersection follows the same quadratic (same coefficients, same smallest
positive root, links whose root lies in (0, dmax]) to give identical lists.
"""
import numpy as np

_FAR = 1.0e16  # root value meaning "no intersection" (pylbm/elements/utils.py:15)


class Element:
    number_of_bounds = 1

    def __init__(self, label=0, isfluid=False):
        self.isfluid = bool(isfluid)
        self.label = [label] * self.number_of_bounds if isinstance(label, (int, np.integer)) else list(label)


def _ellipse_ray(x, y, v, center, v1, v2, dmax, label):
    """Smallest positive ray parameter t with (x, y) + t v on the ellipse.

    The ellipse is {c + cos(a) v1 + sin(a) v2}; its implicit form gives the
    quadratic a t^2 + b t + c = 0 below.
    """
    px = x - center[0]
    py = y - center[1]
    sxx = v1[0] ** 2 + v2[0] ** 2
    syy = v1[1] ** 2 + v2[1] ** 2
    sxy = 2 * (v1[0] * v1[1] + v2[0] * v2[1])
    det2 = (v1[0] * v2[1] - v1[1] * v2[0]) ** 2
    qa = v[0] ** 2 * syy + v[1] ** 2 * sxx - v[0] * v[1] * sxy
    qb = 2 * px * v[0] * syy + 2 * py * v[1] * sxx - (px * v[1] + py * v[0]) * sxy
    qc = px ** 2 * syy + py ** 2 * sxx - px * py * sxy - det2
    disc = qb ** 2 - 4 * qa * qc
    ok = disc >= 0
    root = np.sqrt(np.where(ok, disc, 0.0))
    shape = ok.shape
    t1 = np.full(shape, _FAR)
    t2 = np.full(shape, _FAR)
    if qa != 0:
        t1 = np.where(ok, (-qb - root) / (2 * qa), _FAR)
        t2 = np.where(ok, (-qb + root) / (2 * qa), _FAR)
    t1 = np.where(t1 < 0, _FAR, t1)
    t2 = np.where(t2 < 0, _FAR, t2)
    t = np.where(ok, np.minimum(t1, t2), -1.0)
    t = np.where(t == _FAR, -1.0, t)
    hit = t > 0 if dmax is None else np.logical_and(t > 0, t <= dmax)
    alpha = np.where(hit, t, -1.0)
    border = np.where(hit, float(label[0]), -1.0)
    return alpha, border


class Circle(Element):
    """Disc obstacle (pylbm/elements/circle.py:24); the edge counts as inside."""

    number_of_bounds = 1

    def __init__(self, center, radius, label=0, isfluid=False):
        if radius < 0:
            raise ValueError("the radius of the circle should be positive")
        self.dim = 2
        self.center = np.asarray(center, dtype=np.float64)
        self.radius = float(radius)
        super().__init__(label, isfluid)

    def get_bounds(self):
        return self.center - self.radius, self.center + self.radius

    def point_inside(self, grid):
        x, y = grid
        return (x - self.center[0]) ** 2 + (y - self.center[1]) ** 2 <= self.radius ** 2

    def distance(self, grid, v, dmax=None):
        x, y = grid
        r = self.radius
        return _ellipse_ray(x, y, v, self.center, r * np.array([1, 0]), r * np.array([0, 1]), dmax, self.label)


def _line_hits(px, py, v, q, w):
    """Ray (px, py) + t v against the segment q + s w, s in [0, 1]: (t, s) by
    Cramer's rule, or None for parallel lines."""
    det = v[1] * w[0] - v[0] * w[1]
    if det == 0:
        return None
    inv = 1.0 / det
    c1 = q[0] - px
    c2 = q[1] - py
    return (-w[1] * c1 + w[0] * c2) * inv, (-v[1] * c1 + v[0] * c2) * inv


class Parallelogram(Element):
    """Parallelogram {point + a v1 + b v2, a, b in [0, 1]} (pylbm/elements/parallelogram.py:21).

    Four edges, each with its own label (edges from the point along v1 and
    v2, then the opposite ones); the edges count as inside.
    """

    number_of_bounds = 4

    def __init__(self, point, vecta, vectb, label=0, isfluid=False):
        self.dim = 2
        self.point = np.asarray(point, dtype=np.float64)
        self.v1 = np.asarray(vecta, dtype=np.float64)
        self.v2 = np.asarray(vectb, dtype=np.float64)
        super().__init__(label, isfluid)

    def get_bounds(self):
        box = np.asarray([self.point, self.point + self.v1, self.point + self.v1 + self.v2, self.point + self.v2])
        return np.min(box, axis=0), np.max(box, axis=0)

    def point_inside(self, grid):
        x, y = grid
        dx, dy = x - self.point[0], y - self.point[1]
        inv = 1.0 / (self.v1[0] * self.v2[1] - self.v1[1] * self.v2[0])
        a = (dx * self.v2[1] - dy * self.v2[0]) * inv
        b = (dy * self.v1[0] - dx * self.v1[1]) * inv
        return (a >= 0) & (b >= 0) & (a <= 1) & (b <= 1)

    def distance(self, grid, v, dmax=None):
        x, y = grid
        px, py = x - self.point[0], y - self.point[1]
        shape = (x.size, y.size) if x.shape[1] == 1 and y.shape[0] == 1 else x.shape
        alpha = np.full(shape, _FAR)
        border = -np.ones(shape)
        zero = np.zeros(2)
        for q, w, lab in ((zero, self.v1, self.label[0]), (zero, self.v2, self.label[1]),
                          (self.v2, self.v1, self.label[2]), (self.v1, self.v2, self.label[3])):
            hit = _line_hits(px, py, v, q, w)
            if hit is None:
                continue
            t, s = hit
            ok = (t > 0) & (s >= 0) & (s <= 1)
            if dmax is not None:
                ok &= t <= dmax
            closer = np.where(ok & (alpha > t))
            alpha[closer] = t[closer]
            border[closer] = lab
        alpha[alpha == _FAR] = -1.0
        return alpha, border


class Sphere(Element):
    """Ball obstacle (pylbm/elements/sphere.py:24); the surface counts as inside.

    The ray distance follows the ellipsoid quadratic of pylbm
    (pylbm/elements/utils.py:171 ``distance_ellipsoid``) with the three
    semi-axes r e_x, r e_y, r e_z, term by term in the same order.
    """

    number_of_bounds = 1

    def __init__(self, center, radius, label=0, isfluid=False):
        if radius < 0:
            raise ValueError("the radius of the sphere should be positive")
        self.dim = 3
        self.center = np.asarray(center, dtype=np.float64)
        self.radius = float(radius)
        super().__init__(label, isfluid)

    def get_bounds(self):
        return self.center - self.radius, self.center + self.radius

    def point_inside(self, grid):
        x, y, z = grid
        return ((x - self.center[0]) ** 2 + (y - self.center[1]) ** 2 + (z - self.center[2]) ** 2) <= self.radius ** 2

    def distance(self, grid, v, dmax=None):
        x, y, z = grid
        shape = (x.size, y.size, z.size)
        r = self.radius
        e1, e2, e3 = r * np.array([1, 0, 0]), r * np.array([0, 1, 0]), r * np.array([0, 0, 1])
        X, Y, Z = x - self.center[0], y - self.center[1], z - self.center[2]
        c12, c23, c31 = np.cross(e1, e2), np.cross(e2, e3), np.cross(e3, e1)
        dd = np.inner(e1, c23) ** 2
        cxx = c12[0] ** 2 + c23[0] ** 2 + c31[0] ** 2
        cyy = c12[1] ** 2 + c23[1] ** 2 + c31[1] ** 2
        czz = c12[2] ** 2 + c23[2] ** 2 + c31[2] ** 2
        cxy = 2 * (c12[0] * c12[1] + c23[0] * c23[1] + c31[0] * c31[1])
        cyz = 2 * (c12[1] * c12[2] + c23[1] * c23[2] + c31[1] * c31[2])
        czx = 2 * (c12[2] * c12[0] + c23[2] * c23[0] + c31[2] * c31[0])
        qa = cxx * v[0] ** 2 + cyy * v[1] ** 2 + czz * v[2] ** 2 + cxy * v[0] * v[1] + cyz * v[1] * v[2] \
            + czx * v[2] * v[0]
        qb = (2 * cxx * v[0] + cxy * v[1] + czx * v[2]) * X + (2 * cyy * v[1] + cyz * v[2] + cxy * v[0]) * Y \
            + (2 * czz * v[2] + czx * v[0] + cyz * v[1]) * Z
        qc = cxx * X ** 2 + cyy * Y ** 2 + czz * Z ** 2 + cxy * X * Y + cyz * Y * Z + czx * Z * X - dd
        disc = np.broadcast_to(qb ** 2 - 4 * qa * qc, shape).copy()
        ok = disc >= 0
        disc[ok] = np.sqrt(disc[ok])
        qbb = np.broadcast_to(qb, shape)
        t1 = np.full(shape, _FAR)
        t2 = np.full(shape, _FAR)
        t1[ok] = (-qbb[ok] - disc[ok]) / (2 * qa)
        t2[ok] = (-qbb[ok] + disc[ok]) / (2 * qa)
        t1[t1 < 0] = _FAR
        t2[t2 < 0] = _FAR
        t = -np.ones(shape)
        t[ok] = np.minimum(t1[ok], t2[ok])
        t[t == _FAR] = -1
        hit = t > 0 if dmax is None else np.logical_and(t > 0, t <= dmax)
        alpha = -np.ones(shape)
        border = -np.ones(shape)
        alpha[hit] = t[hit]
        border[hit] = self.label[0]
        return alpha, border
