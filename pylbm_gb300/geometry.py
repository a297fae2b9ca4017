"""Geometric elements used to build the solid/fluid map of a domain.

The reference describes obstacles by elements with ``get_bounds``,
``point_inside`` and a ray distance ``distance(grid, v, dmax)`` returning the
fraction of the lattice link before the wall and the wall label
(pylbm/elements/circle.py:24, pylbm/elements/utils.py:93 ``distance_ellipse``;
pylbm/elements/parallelogram.py:21 with utils.py:40 ``distance_lines``).
Boundary link lists are derived from those distances, so the ray/obstacle
intersection follows the same quadratic (same coefficients, same smallest
positive root, links whose root lies in (0, dmax]) to give identical lists.

All of pylbm's analytic elements are here: Circle, Ellipse, Parallelogram,
Triangle (2D), Sphere, Ellipsoid, CylinderCircle, CylinderEllipse,
CylinderTriangle and Parallelepiped (3D).  The elements the device builds
beyond the circle, parallelogram and sphere describe themselves to it with
``device_params``: the per-element and per-velocity constants of their ray
equations, computed here by the same expressions their ``distance`` uses,
so the device only repeats the per-node arithmetic.
"""
import numpy as np

_FAR = 1.0e16  # root value meaning "no intersection" (pylbm/elements/utils.py:15)


class Element:
    number_of_bounds = 1

    def __init__(self, label=0, isfluid=False):
        self.isfluid = bool(isfluid)
        self.label = [label] * self.number_of_bounds if isinstance(label, (int, np.integer)) else list(label)


def _ellipse_coeffs(v1, v2):
    """(sxx, syy, sxy, det2) of the implicit form of {cos(a) v1 + sin(a) v2}:
    syy X^2 + sxx Y^2 - sxy X Y = det2 (pylbm/elements/utils.py:93-121)."""
    sxx = v1[0] ** 2 + v2[0] ** 2
    syy = v1[1] ** 2 + v2[1] ** 2
    sxy = 2 * (v1[0] * v1[1] + v2[0] * v2[1])
    det2 = (v1[0] * v2[1] - v1[1] * v2[0]) ** 2
    return sxx, syy, sxy, det2


def _ellipse_qa(v, co):
    """Quadratic coefficient of the ray equation (depends on v only)."""
    sxx, syy, sxy, _ = co
    return v[0] ** 2 * syy + v[1] ** 2 * sxx - v[0] * v[1] * sxy


def _ellipse_ray(x, y, v, center, v1, v2, dmax, label, co=None, qa=None):
    """Smallest positive ray parameter t with (x, y) + t v on the ellipse.

    The ellipse is {c + cos(a) v1 + sin(a) v2}; its implicit form gives the
    quadratic qa t^2 + qb t + qc = 0 below.
    """
    sxx, syy, sxy, det2 = co = _ellipse_coeffs(v1, v2) if co is None else co
    qa = _ellipse_qa(v, co) if qa is None else qa
    px = x - center[0]
    py = y - center[1]
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
    Cramer's rule, or None for parallel lines (pylbm/elements/utils.py:21-37)."""
    det = v[1] * w[0] - v[0] * w[1]
    if det == 0:
        return None
    inv = 1.0 / det
    c1 = q[0] - px
    c2 = q[1] - py
    return (-w[1] * c1 + w[0] * c2) * inv, (-v[1] * c1 + v[0] * c2) * inv


def _lines_ray(px, py, v, segments, dmax):
    """First crossing of the ray (px, py) + t v, t in (0, dmax], with a set of
    segments [(q, w, label), ...] tried in order, a later one winning only
    when strictly closer (pylbm/elements/utils.py:40-90).  Returns the ray
    parameter (-1 where none) and the label (-1 where none)."""
    shape = (px.size, py.size) if px.shape[1] == 1 and py.shape[0] == 1 else px.shape
    alpha = np.full(shape, _FAR)
    border = -np.ones(shape)
    for q, w, lab in segments:
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
        zero = np.zeros(2)
        return _lines_ray(x - self.point[0], y - self.point[1], v,
                          ((zero, self.v1, self.label[0]), (zero, self.v2, self.label[1]),
                           (self.v2, self.v1, self.label[2]), (self.v1, self.v2, self.label[3])), dmax)


class Ellipse(Element):
    """Ellipse {center + cos(a) v1 + sin(a) v2} with orthogonal v1, v2
    (pylbm/elements/ellipse.py:23); the edge counts as inside."""

    number_of_bounds = 1

    def __init__(self, center, v1, v2, label=0, isfluid=False):
        if abs(v1[0] * v2[0] + v1[1] * v2[1]) > 1.0e-14:
            raise ValueError("the vectors of the ellipse are not orthogonal")
        self.dim = 2
        self.center = np.asarray(center, dtype=np.float64)
        self.v1 = np.asarray(v1, dtype=np.float64)
        self.v2 = np.asarray(v2, dtype=np.float64)
        super().__init__(label, isfluid)

    def get_bounds(self):
        r = max(np.linalg.norm(self.v1), np.linalg.norm(self.v2))
        return self.center - r, self.center + r

    def point_inside(self, grid):
        x, y = grid
        sxx, syy, sxy, det2 = _ellipse_coeffs(self.v1, self.v2)
        px, py = x - self.center[0], y - self.center[1]
        return px ** 2 * syy + py ** 2 * sxx - px * py * sxy <= det2

    def distance(self, grid, v, dmax=None):
        x, y = grid
        return _ellipse_ray(x, y, v, self.center, self.v1, self.v2, dmax, self.label)

    def device_params(self, dx, velocities):
        co = _ellipse_coeffs(self.v1, self.v2)
        qa = [_ellipse_qa(dx * vk, co) for vk in velocities]
        return [*self.center, *co], self.label[:1], [(a, 0.0, 0.0, 0.0) for a in qa]


class Triangle(Element):
    """Triangle {point + a v1 + b v2, a, b >= 0, a + b <= 1}
    (pylbm/elements/triangle.py:24); edges along v1, along v2 and the third
    one, each with its own label; the edges count as inside."""

    number_of_bounds = 3

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
        return (a >= 0) & (b >= 0) & (a + b <= 1)

    def distance(self, grid, v, dmax=None):
        x, y = grid
        zero = np.zeros(2)
        return _lines_ray(x - self.point[0], y - self.point[1], v,
                          ((zero, self.v1, self.label[0]), (zero, self.v2, self.label[1]),
                           (self.v1, self.v2 - self.v1, self.label[2])), dmax)

    def device_params(self, dx, velocities):
        return [*self.point, *self.v1, *self.v2], self.label[:3], [(0.0,) * 4 for _ in velocities]


def _ellipsoid_coeffs(v1, v2, v3):
    """(cxx, cyy, czz, cxy, cyz, czx, d) of the implicit form of the
    ellipsoid {a v1 + b v2 + c v3, a^2 + b^2 + c^2 = 1}:
    cxx X^2 + cyy Y^2 + czz Z^2 + cxy XY + cyz YZ + czx ZX = d
    (pylbm/elements/utils.py:171-198)."""
    c12, c23, c31 = np.cross(v1, v2), np.cross(v2, v3), np.cross(v3, v1)
    d = np.inner(v1, c23) ** 2
    cxx = c12[0] ** 2 + c23[0] ** 2 + c31[0] ** 2
    cyy = c12[1] ** 2 + c23[1] ** 2 + c31[1] ** 2
    czz = c12[2] ** 2 + c23[2] ** 2 + c31[2] ** 2
    cxy = 2 * (c12[0] * c12[1] + c23[0] * c23[1] + c31[0] * c31[1])
    cyz = 2 * (c12[1] * c12[2] + c23[1] * c23[2] + c31[1] * c31[2])
    czx = 2 * (c12[2] * c12[0] + c23[2] * c23[0] + c31[2] * c31[0])
    return cxx, cyy, czz, cxy, cyz, czx, d


def _ellipsoid_ray_constants(v, co):
    """The ray equation's quadratic coefficient and the three factors of its
    linear coefficient (X, Y, Z multiply them); they depend on v only."""
    cxx, cyy, czz, cxy, cyz, czx, _ = co
    qa = cxx * v[0] ** 2 + cyy * v[1] ** 2 + czz * v[2] ** 2 + cxy * v[0] * v[1] + cyz * v[1] * v[2] \
        + czx * v[2] * v[0]
    bx = 2 * cxx * v[0] + cxy * v[1] + czx * v[2]
    by = 2 * cyy * v[1] + cyz * v[2] + cxy * v[0]
    bz = 2 * czz * v[2] + czx * v[0] + cyz * v[1]
    return qa, bx, by, bz


def _ellipsoid_ray(grid, v, center, co, dmax, label):
    """Smallest positive t with (x, y, z) + t v on the ellipsoid of
    implicit-form coefficients co (pylbm/elements/utils.py:160-230)."""
    x, y, z = grid
    shape = (x.size, y.size, z.size)
    cxx, cyy, czz, cxy, cyz, czx, dd = co
    qa, bx, by, bz = _ellipsoid_ray_constants(v, co)
    X, Y, Z = x - center[0], y - center[1], z - center[2]
    qb = bx * X + by * Y + bz * Z
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
    border[hit] = label[0]
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
        r = self.radius
        co = _ellipsoid_coeffs(r * np.array([1, 0, 0]), r * np.array([0, 1, 0]), r * np.array([0, 0, 1]))
        return _ellipsoid_ray(grid, v, self.center, co, dmax, self.label)


class Ellipsoid(Element):
    """Ellipsoid {center + a v1 + b v2 + c v3, a^2 + b^2 + c^2 <= 1} with
    orthogonal v1, v2, v3 (pylbm/elements/ellipsoid.py:24); the surface
    counts as inside."""

    number_of_bounds = 1

    def __init__(self, center, v1, v2, v3, label=0, isfluid=False):
        dots = (np.dot(v1, v2), np.dot(v2, v3), np.dot(v3, v1))
        if max(abs(float(p)) for p in dots) > 1.0e-14:
            raise ValueError("the vectors of the ellipsoid are not orthogonal")
        self.dim = 3
        self.center = np.asarray(center, dtype=np.float64)
        self.v1 = np.asarray(v1, dtype=np.float64)
        self.v2 = np.asarray(v2, dtype=np.float64)
        self.v3 = np.asarray(v3, dtype=np.float64)
        super().__init__(label, isfluid)

    def get_bounds(self):
        r = max(np.linalg.norm(self.v1), np.linalg.norm(self.v2), np.linalg.norm(self.v3))
        return self.center - r, self.center + r

    def point_inside(self, grid):
        x, y, z = grid
        cxx, cyy, czz, cxy, cyz, czx, d = _ellipsoid_coeffs(self.v1, self.v2, self.v3)
        X, Y, Z = x - self.center[0], y - self.center[1], z - self.center[2]
        return cxx * X ** 2 + cyy * Y ** 2 + czz * Z ** 2 + cxy * X * Y + cyz * Y * Z + czx * Z * X <= d

    def distance(self, grid, v, dmax=None):
        co = _ellipsoid_coeffs(self.v1, self.v2, self.v3)
        return _ellipsoid_ray(grid, v, self.center, co, dmax, self.label)

    def device_params(self, dx, velocities):
        co = _ellipsoid_coeffs(self.v1, self.v2, self.v3)
        return [*self.center, *co], self.label[:1], [_ellipsoid_ray_constants(dx * vk, co) for vk in velocities]


# ----------------------------------------------------------------- cylinders
# A cylinder is a plane section extruded along w: in the frame (v1, v2, w)
# centred on `center` it is {(x, y) in the section, -1 <= z <= 1}, where the
# section is the unit disc (circle and ellipse bases), the unit triangle
# {x, y >= 0, x + y <= 1} or the unit square (pylbm/elements/cylinder.py:27-270,
# pylbm/elements/base.py:136-608).

SECTION_ROUND, SECTION_TRIANGLE, SECTION_SQUARE = 0, 1, 2
_UNIT_CIRCLE = (np.zeros(2), np.asarray([1, 0]), np.asarray([0, 1]))
_SECTION_SEGMENTS = {
    SECTION_TRIANGLE: (([0, 0], [1, 0]), ([0, 0], [0, 1]), ([1, 0], [-1, 1])),
    SECTION_SQUARE: (([0, 0], [1, 0]), ([0, 0], [0, 1]), ([1, 0], [0, 1]), ([0, 1], [1, 0])),
}


def _section_inside(kind, x, y):
    if kind == SECTION_ROUND:
        return (x ** 2 + y ** 2) <= 1.0
    if kind == SECTION_TRIANGLE:
        return np.logical_and(np.logical_and(x >= 0, y >= 0), x + y <= 1)
    return np.logical_and(np.logical_and(x >= 0, y >= 0), np.logical_and(x <= 1, y <= 1))


def _section_qa(v):
    return _ellipse_qa(v, _ellipse_coeffs(_UNIT_CIRCLE[1], _UNIT_CIRCLE[2]))


def _section_ray(kind, x, y, v, dmax, labels):
    if kind == SECTION_ROUND:
        c, v1, v2 = _UNIT_CIRCLE
        return _ellipse_ray(x, y, v, c, v1, v2, dmax, labels)
    segments = tuple((q, w, lab) for (q, w), lab in zip(_SECTION_SEGMENTS[kind], labels))
    return _lines_ray(x, y, v, segments, dmax)


class _Cylinder(Element):
    dim = 3
    section = SECTION_ROUND

    def _frame(self, center, v1, v2, w):
        self.center = np.asarray(center, dtype=np.float64)
        self.v1 = np.asarray(v1, dtype=np.float64)
        self.v2 = np.asarray(v2, dtype=np.float64)
        self.w = np.asarray(w, dtype=np.float64)
        A = np.empty((3, 3))
        A[:, 0], A[:, 1], A[:, 2] = self.v1, self.v2, self.w
        self.A = A
        self.iA = np.linalg.inv(A)

    def _section_bounds(self):
        box = np.asarray([self.center, self.center + self.v1, self.center + self.v1 + self.v2, self.center + self.v2])
        return np.min(box, axis=0), np.max(box, axis=0)

    def get_bounds(self):
        half = [0.5 * abs(self.w[k]) for k in range(len(self.w))]
        lo, hi = self._section_bounds()
        return lo - half, hi + half

    def _to_frame(self, grid):
        x, y, z = grid
        xx, yy, zz = x - self.center[0], y - self.center[1], z - self.center[2]
        iA = self.iA
        return (iA[0, 0] * xx + iA[0, 1] * yy + iA[0, 2] * zz,
                iA[1, 0] * xx + iA[1, 1] * yy + iA[1, 2] * zz,
                iA[2, 0] * xx + iA[2, 1] * yy + iA[2, 2] * zz)

    def frame_velocity(self, v):
        """The ray direction in the cylinder's frame."""
        return self.iA.dot(np.asarray(v))

    def point_inside(self, grid):
        xc, yc, zc = self._to_frame(grid)
        return np.logical_and(_section_inside(self.section, xc, yc), np.abs(zc) <= 1.0)

    def distance(self, grid, v, dmax=None):
        xc, yc, zc = self._to_frame(grid)
        vc = self.frame_velocity(v)
        # the side: the section's boundary, the crossing kept between the caps
        alpha, border = _section_ray(self.section, xc, yc, vc[:-1], dmax, self.label[:-2])
        alpha = np.array(alpha, dtype=np.float64)
        border = np.array(border, dtype=np.float64)
        alpha[alpha < 0] = _FAR
        off = np.logical_and(alpha > 0, np.abs(zc + alpha * vc[2]) > 1.0)
        alpha[off] = _FAR
        border[off] = -1.0
        # the caps z = 1 and z = -1, where the crossing lies in the section
        shift = 1.0e-16 if vc[2] == 0 else 0.0
        caps = []
        for t in ((1.0 - zc) / (vc[2] + shift), -(1.0 + zc) / (vc[2] + shift)):
            miss = np.logical_or(np.logical_or(t < 0, t > dmax),
                                 np.logical_not(_section_inside(self.section, xc + t * vc[0], yc + t * vc[1])))
            t = np.array(np.broadcast_to(t, alpha.shape), dtype=np.float64)
            t[np.broadcast_to(miss, alpha.shape)] = _FAR
            caps.append(t)
        top, bottom = caps
        alpha = np.amin([alpha, top, bottom], axis=0)
        border[alpha == top] = self.label[-1]
        border[alpha == bottom] = self.label[-2]
        alpha[alpha == _FAR] = -1.0
        return alpha, border

    def device_params(self, dx, velocities):
        table = []
        for vk in velocities:
            vc = self.frame_velocity(dx * vk)
            table.append((vc[0], vc[1], vc[2], _section_qa(vc[:-1]) if self.section == SECTION_ROUND else 0.0))
        return [*self.center, *self.iA.ravel(), float(self.section)], list(self.label), table


class CylinderCircle(_Cylinder):
    """Cylinder of circular section, axis w through center (the section
    {center + cos(a) v1 + sin(a) v2}, |v1| = |v2|), between center - w and
    center + w (pylbm/elements/cylinder.py:272); labels: side, bottom, top."""

    number_of_bounds = 3

    def __init__(self, center, v1, v2, w, label=0, isfluid=False):
        if np.linalg.norm(v1) != np.linalg.norm(v2):
            raise ValueError("the vectors of the circular section must have the same norm")
        self._frame(center, v1, v2, w)
        super().__init__(label, isfluid)

    def _section_bounds(self):
        r = np.linalg.norm(self.v1)
        return self.center - r, self.center + r


class CylinderEllipse(_Cylinder):
    """Cylinder of elliptic section {center + cos(a) v1 + sin(a) v2}
    (v1, v2 orthogonal), between center - w and center + w
    (pylbm/elements/cylinder.py:345); labels: side, bottom, top."""

    number_of_bounds = 3

    def __init__(self, center, v1, v2, w, label=0, isfluid=False):
        if abs(np.inner(np.asarray(v1), np.asarray(v2))) > 1.0e-10:
            raise ValueError("the vectors of the elliptic section have to be orthogonal")
        self._frame(center, v1, v2, w)
        super().__init__(label, isfluid)

    def _section_bounds(self):
        r = max(np.linalg.norm(self.v1), np.linalg.norm(self.v2))
        return self.center - r, self.center + r


class CylinderTriangle(_Cylinder):
    """Cylinder of triangular section {center + a v1 + b v2, a, b >= 0,
    a + b <= 1} between center - w and center + w
    (pylbm/elements/cylinder.py:423); labels: the three sides, bottom, top."""

    number_of_bounds = 5
    section = SECTION_TRIANGLE

    def __init__(self, center, v1, v2, w, label=0, isfluid=False):
        self._frame(center, v1, v2, w)
        super().__init__(label, isfluid)


class Parallelepiped(_Cylinder):
    """Parallelepiped {point + a v0 + b v1 + c v2, a, b, c in [0, 1]}: a
    cylinder of section (v0, v1) along w = v2 / 2 centred on point + w
    (pylbm/elements/cylinder.py:496); labels: the four sides, bottom, top."""

    number_of_bounds = 6
    section = SECTION_SQUARE

    def __init__(self, point, v0, v1, v2, label=0, isfluid=False):
        self.point = np.asarray(point, dtype=np.float64)
        w = 0.5 * np.asarray(v2)
        self._frame(self.point + w, v0, v1, w)
        super().__init__(label, isfluid)
