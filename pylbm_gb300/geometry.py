"""Geometric elements used to build the solid/fluid map of a domain.

The reference describes obstacles by elements with ``get_bounds``,
``point_inside`` and a ray distance ``distance(grid, v, dmax)`` returning the
fraction of the lattice link before the wall and the wall label
(pylbm/elements/circle.py:24, pylbm/elements/utils.py:93 ``distance_ellipse``).
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
