"""Halo-extended lattice, fluid/solid map and per-link wall distances/labels.

Same contract as pylbm's ``Domain`` (pylbm/domain.py:87): nodes are cell
centres ``xmin + (i + 1/2) dx`` plus ``vmax`` ghost layers per side
(``create_coords`` :385-442); ``in_or_out`` is 999 in the fluid and -1 in
the solid/ghost layers; ``distance[k, node]`` is the fraction of the link
``node -> node + v_k`` before a wall and ``flag[k, node]`` that wall's label,
999 elsewhere.  Box walls are applied axis by axis with a strict
"only if shorter" rule (:463-521), obstacles after them (:523-620), then
flags on solid nodes are cleared (``clean``).  The boundary link lists built
from these arrays decide which populations the boundary kernels write, so
the rules (including their tie-breaking) are kept identical.
"""
import numpy as np

from .stencil import Stencil
from .scheme import _box_dim

VALIN = 999
VALOUT = -1


class Domain:
    """Lattice geometry of a dictionary.

    ``with_flags=False`` builds only sizes, halo and coordinates (no
    ``in_or_out``/``distance``/``flag`` arrays), enough for domains periodic
    along every axis, whose ghost layers no boundary method writes.
    """

    def __init__(self, dico, stencil=None, with_flags=True, device=False):
        self.valin = VALIN
        self.valout = VALOUT
        self.dim = _box_dim(dico)
        box = dico["box"]
        bounds = [box["x"]]
        if self.dim > 1:
            bounds.append(box["y"])
        if self.dim > 2:
            bounds.append(box["z"])
        self.bounds = np.asarray(bounds, dtype=np.float64)
        lab = box.get("label", -1)
        if isinstance(lab, (int, np.integer)):
            lab = [int(lab)] * (2 * self.dim)
        lab = list(lab)
        if len(lab) != 2 * self.dim:
            raise ValueError("the box label list must have 2*dim entries")
        self.box_label = lab
        self.dx = float(dico["space_step"])
        self.stencil = stencil if stencil is not None else Stencil.from_dico(dico, self.dim)
        self.elements = list(dico.get("elements", []) or [])
        for e in self.elements:
            if getattr(e, "dim", self.dim) != self.dim:
                raise ValueError("element and box dimensions differ")

        self.global_size = []
        for k in range(self.dim):
            n = (self.bounds[k][1] - self.bounds[k][0]) / self.dx
            if not float(n).is_integer():
                r = round(n)
                if abs(r - n) < self.dx:
                    n = r
                else:
                    raise ValueError(f"box length along axis {k} is not a multiple of the space step")
            self.global_size.append(int(n))
        self.halo = np.asarray(self.stencil.vmax, dtype=np.int64)
        if np.any(self.halo < 1):
            raise ValueError("every axis needs at least one non-zero velocity component")
        self.coords_halo = []
        for k in range(self.dim):
            h = int(self.halo[k])
            beg = self.dx * (h - 0.5)
            self.coords_halo.append(np.linspace(self.bounds[k][0] - beg, self.bounds[k][1] + beg,
                                                self.global_size[k] + 2 * h))
        self.coords = [c[int(h):-int(h)] for c, h in zip(self.coords_halo, self.halo)]
        self.device = bool(device) and with_flags
        if self.device:
            # the arrays are built and kept on the GPU (lbm_domain_* kernels);
            # boundary links are extracted there too (link_list)
            self.in_or_out = self.distance = self.flag = None
            self._build_on_device()
            return
        if not with_flags:
            if self.elements or any(l != -1 for l in self.box_label):
                raise ValueError("a domain without flags must be periodic along every axis")
            self.in_or_out = self.distance = self.flag = None
            return

        uv = self.stencil.unique_v
        nu = uv.shape[0]
        shape = self.shape_halo
        self.in_or_out = np.full(shape, float(VALOUT))
        inner = tuple(slice(int(h), -int(h)) for h in self.halo)
        self.in_or_out[inner] = VALIN
        self.distance = np.full([nu] + shape, float(VALIN))
        self.flag = np.full([nu] + shape, VALIN, dtype=np.int64)
        self._add_box(inner)
        for e in self.elements:
            self._add_element(e)
        self._clean()

    @property
    def shape_halo(self):
        return [int(c.size) for c in self.coords_halo]

    @property
    def shape_in(self):
        return [int(c.size) for c in self.coords]

    # one process owns the whole domain: the demos pass this to H5File, which ignores it
    mpi_topo = None

    # coordinate accessors of pylbm's Domain (pylbm/domain.py:318-361, 444-461)
    x = property(lambda self: self.coords[0], doc="x coordinates of the interior nodes")
    y = property(lambda self: self.coords[1], doc="y coordinates of the interior nodes")
    z = property(lambda self: self.coords[2], doc="z coordinates of the interior nodes")
    x_halo = property(lambda self: self.coords_halo[0], doc="x coordinates, ghost layers included")
    y_halo = property(lambda self: self.coords_halo[1], doc="y coordinates, ghost layers included")
    z_halo = property(lambda self: self.coords_halo[2], doc="z coordinates, ghost layers included")

    def get_bounds(self):
        """First and last interior coordinates per axis."""
        return (np.asarray([c[0] for c in self.coords]), np.asarray([c[-1] for c in self.coords]))

    def get_bounds_halo(self):
        """First and last coordinates per axis, ghost layers included."""
        return (np.asarray([c[0] for c in self.coords_halo]), np.asarray([c[-1] for c in self.coords_halo]))

    def list_of_labels(self):
        labs = np.unique(self.box_label)
        elabs = [l for e in self.elements for l in e.label]
        return np.union1d(labs, np.asarray(elabs, dtype=labs.dtype)) if elabs else labs

    def _add_box(self, inner):
        uv = self.stencil.unique_v
        dist = self.distance[(slice(None),) + inner]
        flag = self.flag[(slice(None),) + inner]
        for axis in range(self.dim):
            for k in range(uv.shape[0]):
                c = int(uv[k, axis])
                if c < 0 and self.box_label[2 * axis] != -2:
                    rows, lab = [(i, (i + 0.5) / -c) for i in range(-c)], self.box_label[2 * axis]
                elif c > 0 and self.box_label[2 * axis + 1] != -2:
                    rows, lab = [(-i - 1, (i + 0.5) / c) for i in range(c)], self.box_label[2 * axis + 1]
                else:
                    continue
                for row, d in rows:
                    sl = [slice(None)] * self.dim
                    sl[axis] = slice(row, row + 1 if row != -1 else None)  # a view, also in 1D
                    dv = dist[k][tuple(sl)]
                    fv = flag[k][tuple(sl)]
                    upd = dv > d
                    dv[upd] = d
                    fv[upd] = lab

    def _add_element(self, elem):
        vmax = self.halo
        lo, hi = elem.get_bounds()
        origin = np.array([c[0] for c in self.coords_halo])
        nmin = np.maximum(vmax, np.array((lo - origin) / self.dx, int) - vmax)
        nmax = np.minimum(vmax + np.asarray(self.shape_in), np.array((hi - origin) / self.dx, int) + vmax + 1)
        region = tuple(slice(a, b) for a, b in zip(nmin, nmax))
        ioo = self.in_or_out[region]
        grid = np.meshgrid(*(self.coords_halo[d][region[d]] for d in range(self.dim)),
                           sparse=True, indexing="ij")
        if not elem.isfluid:
            solid = elem.point_inside(grid)
            fluid = np.logical_not(solid)
            ioo[solid] = VALOUT
        else:
            fluid = elem.point_inside(grid)
            solid = np.logical_not(fluid)
            ioo[fluid] = VALIN
        uv = self.stencil.unique_v
        for k in range(uv.shape[0]):
            vk = uv[k]
            if not np.any(vk != 0):
                continue
            shifted = tuple(slice(a + vk[d], b + vk[d]) for d, (a, b) in enumerate(zip(nmin, nmax)))
            out_cells = self.in_or_out[shifted] == VALOUT
            alpha, border = elem.distance(grid, self.dx * vk, 1.0)
            sel = np.logical_and(alpha > 0, fluid)
            if out_cells.size:
                sel = np.logical_and(sel, out_cells)
            dk = self.distance[k][region]
            fk = self.flag[k][region]
            if elem.isfluid:
                back = np.logical_and(np.logical_not(out_cells), ioo == VALIN)
                dk[back] = VALIN
                fk[back] = VALIN
            else:
                dk[solid] = VALIN
                fk[solid] = VALIN
            idx = np.where(sel)
            if not elem.isfluid:
                keep = alpha[idx] < dk[idx]
            else:
                keep = np.logical_or(alpha[idx] > dk[idx], dk[idx] == VALIN)
            idx = tuple(i[keep] for i in idx)
            dk[idx] = alpha[idx]
            fk[idx] = border[idx]

    def _clean(self):
        solid = self.in_or_out == VALOUT
        for k in range(self.distance.shape[0]):
            sel = np.logical_and(self.distance[k] > 0, solid)
            self.distance[k][sel] = VALIN
            self.flag[k][sel] = VALIN

    # ------------------------------------------------------------------ device construction
    def _region(self, elem):
        """Halo-coordinate region [nmin, nmax) an element touches (same rule as _add_element)."""
        vmax = self.halo
        lo, hi = elem.get_bounds()
        origin = np.array([c[0] for c in self.coords_halo])
        nmin = np.maximum(vmax, np.array((lo - origin) / self.dx, int) - vmax)
        nmax = np.minimum(vmax + np.asarray(self.shape_in), np.array((hi - origin) / self.dx, int) + vmax + 1)
        return nmin, nmax

    def _element_desc(self, elem):
        from . import geometry, runtime
        e = runtime.ElementDesc()
        if isinstance(elem, geometry.Circle):
            e.kind = runtime.LBM_ELEMENT_CIRCLE
            vals = [elem.center[0], elem.center[1], elem.radius]
        elif isinstance(elem, geometry.Parallelogram):
            e.kind = runtime.LBM_ELEMENT_PARALLELOGRAM
            vals = [*elem.point, *elem.v1, *elem.v2]
        elif isinstance(elem, geometry.Sphere):
            e.kind = runtime.LBM_ELEMENT_SPHERE
            vals = [*elem.center, elem.radius]
        elif hasattr(elem, "device_params") and isinstance(elem, geometry.Element):
            kinds = {geometry.Ellipse: runtime.LBM_ELEMENT_ELLIPSE, geometry.Triangle: runtime.LBM_ELEMENT_TRIANGLE,
                     geometry.Ellipsoid: runtime.LBM_ELEMENT_ELLIPSOID}
            e.kind = kinds.get(type(elem), runtime.LBM_ELEMENT_CYLINDER)
            vals, labels, table = elem.device_params(self.dx, self.stencil.unique_v)
            for u, row in enumerate(table):
                for i, v in enumerate(row):
                    e.vq[u][i] = float(v)
        else:
            raise NotImplementedError(f"{type(elem).__name__} is not built on the device")
        for i, v in enumerate(vals):
            e.p[i] = float(v)
        for i, lab in enumerate(elem.label[:6]):
            e.label[i] = int(lab)
        e.isfluid = int(elem.isfluid)
        nmin, nmax = self._region(elem)
        for a in range(self.dim):
            e.lo[a], e.hi[a] = int(nmin[a]), int(nmax[a])
        return e

    def _build_on_device(self):
        import ctypes
        from . import runtime

        core = runtime.core()
        uv = self.stencil.unique_v
        d = runtime.DomainDesc()
        d.dim, d.nu, d.dx = self.dim, uv.shape[0], self.dx
        shape = self.shape_halo + [1] * (3 - self.dim)
        for a in range(3):
            d.n[a] = shape[a]
            d.halo[a] = int(self.halo[a]) if a < self.dim else 0
        for u in range(uv.shape[0]):
            for a in range(self.dim):
                d.vel[u][a] = int(uv[u, a])
        self._desc = d
        self._nodes = int(np.prod(shape))
        nu = uv.shape[0]
        self.d_in_or_out = runtime.DeviceBuffer(8 * self._nodes)
        self.d_distance = runtime.DeviceBuffer(8 * nu * self._nodes)
        self.d_flag = runtime.DeviceBuffer(4 * nu * self._nodes)
        self.d_coords = runtime.DeviceBuffer(8 * int(sum(shape[:self.dim])))
        self.d_coords.upload(np.ascontiguousarray(np.concatenate(self.coords_halo), dtype=np.float64))
        ref = ctypes.byref(d)
        runtime.check(core.lbm_domain_reset(ref, self.d_in_or_out.handle, self.d_distance.handle,
                                            self.d_flag.handle, None))
        labels = np.asarray(self.box_label + [-2] * (6 - len(self.box_label)), dtype=np.int32)
        runtime.check(core.lbm_domain_box(ref, labels.ctypes.data_as(ctypes.c_void_p), self.d_distance.handle,
                                          self.d_flag.handle, None))
        for elem in self.elements:
            e = self._element_desc(elem)
            runtime.check(core.lbm_domain_element(ref, ctypes.byref(e), self.d_coords.handle, self.d_in_or_out.handle,
                                                  self.d_distance.handle, self.d_flag.handle, None))
        runtime.check(core.lbm_domain_clean(ref, self.d_in_or_out.handle, self.d_distance.handle,
                                            self.d_flag.handle, None))
        runtime.check(core.lbm_device_synchronize())

    def link_list(self, label, u, vsym):
        """Nodes with flag[u] == label, row-major (np.where order), shifted by
        vsym: (dim, count) int64 halo coordinates and their distances."""
        import ctypes
        from . import runtime

        core = runtime.core()
        ref = ctypes.byref(self._desc)
        block = core.lbm_links_block()
        nblocks = -(-self._nodes // block)
        counts = runtime.DeviceBuffer(4 * nblocks)
        runtime.check(core.lbm_links_count(ref, self.d_flag.handle, int(u), int(label), counts.handle, None))
        host = np.empty(nblocks, dtype=np.int32)
        counts.download(host)
        offsets = np.zeros(nblocks, dtype=np.int32)
        np.cumsum(host[:-1], out=offsets[1:])
        total = int(host.sum())
        if total == 0:
            counts.free()
            return np.zeros((self.dim, 0), dtype=np.int64), np.zeros(0)
        counts.upload(offsets)
        rows = runtime.DeviceBuffer(4 * total * self.dim)
        dist = runtime.DeviceBuffer(8 * total)
        vs = np.zeros(3, dtype=np.int32)
        vs[:self.dim] = vsym
        runtime.check(core.lbm_links_fill(ref, self.d_flag.handle, self.d_distance.handle, int(u), int(label),
                                          vs.ctypes.data_as(ctypes.c_void_p), counts.handle, rows.handle,
                                          dist.handle, None))
        r = np.empty((total, self.dim), dtype=np.int32)
        dd = np.empty(total)
        rows.download(r)
        dist.download(dd)
        for b in (counts, rows, dist):
            b.free()
        return r.T.astype(np.int64), dd

    def download_arrays(self):
        """Host copies of the device arrays (in_or_out, distance, flag), as the host path builds them."""
        nu = self._desc.nu
        shape = self.shape_halo
        ioo = np.empty(self._nodes)
        dist = np.empty(nu * self._nodes)
        flag = np.empty(nu * self._nodes, dtype=np.int32)
        self.d_in_or_out.download(ioo)
        self.d_distance.download(dist)
        self.d_flag.download(flag)
        return ioo.reshape(shape), dist.reshape([nu] + shape), flag.reshape([nu] + shape).astype(np.int64)
