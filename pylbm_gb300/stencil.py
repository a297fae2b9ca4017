"""Velocity numbering and stencils, the same numbering pylbm uses.

pylbm identifies every lattice velocity by an integer (pylbm/stencil.py:119
``Velocity``; numbering in ``_set_num``/``_set_coord``, :285-374).  Scheme
dictionaries name their velocities by these integers, so the numbering is an
interface and is reproduced exactly here:

* 1D: 0, +1, -1, +2, -2, ...
* 2D: rings of growing Chebyshev radius n; inside a ring the four axis
  velocities, then the four diagonals, then the eight (n, j) velocities for
  j = 1..n-1 in the order (n,j), (j,n), (-j,n), (-n,j), (-n,-j), (-j,-n),
  (j,-n), (n,-j).
* 3D: for k = 0, 1, ...; i <= k; j <= i: every distinct permutation of the
  sorted triple (j, i, k) in lexicographic order, and for each permutation the
  sign choices (+ before -) of its non-zero entries, first component outermost.

The class below keeps only what the CUDA backend needs: the velocities of each
elementary scheme, the unique velocities, ``nv_ptr``, the symmetric index map
(pylbm/stencil.py:817 ``get_symmetric``) and ``vmax`` (:716).
"""
import itertools

import numpy as np


def _velocities_2d():
    yield (0, 0)
    n = 1
    while True:
        yield from [(n, 0), (0, n), (-n, 0), (0, -n)]
        yield from [(n, n), (-n, n), (-n, -n), (n, -n)]
        for j in range(1, n):
            yield from [(n, j), (j, n), (-j, n), (-n, j),
                        (-n, -j), (-j, -n), (j, -n), (n, -j)]
        n += 1


def _velocities_3d():
    for k in itertools.count():
        for i in range(k + 1):
            for j in range(i + 1):
                for perm in sorted(set(itertools.permutations((j, i, k)))):
                    signs = [(1, -1) if c else (1,) for c in perm]
                    for sg in itertools.product(*signs):
                        yield tuple(s * c for s, c in zip(sg, perm))


def _velocities_1d():
    yield (0,)
    n = 1
    while True:
        yield (n,)
        yield (-n,)
        n += 1


_GENERATORS = {1: _velocities_1d, 2: _velocities_2d, 3: _velocities_3d}
_TABLES = {}


def _table(dim, upto):
    tab = _TABLES.setdefault(dim, [])
    if len(tab) <= upto:
        tab.clear()
        gen = _GENERATORS[dim]()
        for _ in range(max(upto + 1, 64)):
            tab.append(next(gen))
    return tab


def velocity(dim, num):
    """Coordinates of velocity number ``num`` in dimension ``dim``."""
    if num < 0:
        raise ValueError("velocity numbers are non-negative")
    return _table(dim, num)[num]


def velocity_number(v):
    """Number of the velocity with coordinates ``v`` (inverse of ``velocity``)."""
    v = tuple(int(c) for c in v)
    dim = len(v)
    radius = max(abs(c) for c in v) if v else 0
    upto = (2 * radius + 1) ** dim
    tab = _table(dim, upto)
    try:
        return tab.index(v)
    except ValueError as exc:
        raise ValueError(f"velocity {v} not found") from exc


class Stencil:
    """Velocities of the elementary schemes of a pylbm dictionary.

    Mirrors the attributes of pylbm's ``Stencil`` (pylbm/stencil.py:444) that
    the hot path uses: ``dim``, ``nv``, ``nv_ptr``, ``unum`` (unique velocity
    numbers), ``unum2index``, ``num`` (per scheme), ``get_all_velocities``,
    ``get_symmetric`` and ``vmax``.
    """

    def __init__(self, dim, schemes_velocities):
        self.dim = int(dim)
        self.nums = [np.asarray(list(v), dtype=np.int64) for v in schemes_velocities]
        self.nstencils = len(self.nums)
        self.nv = [len(v) for v in self.nums]
        self.nv_ptr = np.concatenate([[0], np.cumsum(self.nv)]).astype(np.int64)
        unique = np.unique(np.concatenate(self.nums)) if self.nums else np.zeros(0, np.int64)
        self.unum = unique
        self.unique_v = np.array([velocity(self.dim, int(n)) for n in unique], dtype=np.int64)
        self.unum2index = -1000 * np.ones(int(unique.max()) + 1 if unique.size else 1, dtype=np.int64)
        self.unum2index[unique] = np.arange(unique.size)
        for k, nums in enumerate(self.nums):
            for n in nums:
                sym = velocity_number(tuple(-c for c in velocity(self.dim, int(n))))
                if sym not in set(nums.tolist()):
                    raise ValueError(
                        f"velocity {int(n)} of scheme {k} has no symmetric velocity in that scheme")

    @classmethod
    def from_dico(cls, dico, dim):
        return cls(dim, [s["velocities"] for s in dico["schemes"]])

    @property
    def unvtot(self):
        return int(self.unum.size)

    @property
    def nvtot(self):
        return int(self.nv_ptr[-1])

    def num(self, k):
        return self.nums[k]

    def get_all_velocities(self):
        """All velocities of all schemes, shape (nvtot, dim) (pylbm/stencil.py:783)."""
        out = np.empty((self.nvtot, self.dim), dtype=np.int64)
        i = 0
        for nums in self.nums:
            for n in nums:
                out[i] = velocity(self.dim, int(n))
                i += 1
        return out

    def get_symmetric(self):
        """Index of -v_k inside the same elementary scheme (pylbm/stencil.py:817)."""
        ksym = np.empty(self.nvtot, dtype=np.int32)
        i = 0
        for s, nums in enumerate(self.nums):
            pos = {int(n): j for j, n in enumerate(nums)}
            for n in nums:
                sym = velocity_number(tuple(-c for c in velocity(self.dim, int(n))))
                ksym[i] = pos[sym] + self.nv_ptr[s]
                i += 1
        return ksym

    @property
    def vmax(self):
        """Largest |v| along each axis over the unique velocities (pylbm/stencil.py:716)."""
        return np.abs(self.unique_v).max(axis=0) if self.unique_v.size else np.zeros(self.dim, np.int64)
