"""Boundary link lists and boundary methods (pylbm/boundary.py).

Link lists are built on the host once, exactly as the reference builds them:
for every label and every velocity k of a scheme, the fluid nodes x whose link
x -> x - v_k crosses a wall with that label give a store slot (k, x - v_k) in a
ghost or solid node (pylbm/boundary.py:23-47 ``BoundaryVelocity``); slots are
grouped per method class in the order labels, schemes, velocities are met
(:78-160).  Each method derives its load slots (``set_iload``) and its
right-hand side from the equilibrium at the wall points (``prepare_rhs``,
:238-305).  The lists are uploaded once; every step the device kernels of the
C ABI apply ``f[istore] = +/- f[iload0] + rhs`` (Bouzidi methods: an
interpolation between two loads).
"""
from collections import OrderedDict

import numpy as np
import sympy as sp


class _BoundaryVelocity:
    """Store slots of one label for one incoming velocity (pylbm/boundary.py:23-47)."""

    def __init__(self, domain, label, kunique):
        st = domain.stencil
        v = st.unique_v[kunique]
        vsym = -v
        from .stencil import velocity_number
        num = velocity_number(tuple(int(c) for c in vsym))
        ksym_u = int(st.unum2index[num])
        if getattr(domain, "device", False):  # flags on the GPU: extracted there, same order
            self.indices, self.distance = domain.link_list(label, ksym_u, vsym)
            return
        ind = np.where(domain.flag[ksym_u] == label)
        self.indices = np.array(ind, dtype=np.int64)
        if self.indices.size:
            self.indices = self.indices + vsym[:, np.newaxis]
        self.distance = np.array(domain.distance[(ksym_u,) + ind])


class _Moments:
    """Moment container handed to user boundary functions (``m[RHO] = ...``)."""

    def __init__(self, array, consm):
        self.array = array
        self.consm = consm

    def _key(self, key):
        if isinstance(key, (sp.Symbol, sp.IndexedBase)):
            return self.consm[key]
        if isinstance(key, str) and sp.Symbol(key) in self.consm:
            return self.consm[sp.Symbol(key)]
        return key

    def __getitem__(self, key):
        return self.array[self._key(key)]

    def __setitem__(self, key, value):
        self.array[self._key(key)] = value


class BoundaryMethod:
    """Common part of the boundary methods (pylbm/boundary.py:164-397).

    ``kind`` selects the device kernel: 'bounce_back', 'anti_bounce_back',
    'bouzidi_bounce_back', 'bouzidi_anti_bounce_back' or 'neumann'.
    """

    kind = None
    name = None

    def __init__(self, istore, ilabel, distance, stencil, value_bc, time_bc):
        self.istore = istore            # (dim+1, ncond) until fix_iload
        self.ilabel = ilabel
        self.distance = distance
        self.stencil = stencil
        self.feq = np.zeros((stencil.nvtot, istore.shape[1]))
        self.rhs = np.zeros(istore.shape[1])
        self.value_bc = {k: value_bc[k] for k in np.unique(ilabel)}
        self.time_bc = {k: time_bc[k] for k in np.unique(ilabel)}
        self.iload = []
        self._timed = []
        self.ncond = int(istore.shape[1])

    def set_iload(self):
        raise NotImplementedError

    def set_rhs(self):
        pass

    def fix_iload(self):
        """(dim+1, ncond) -> contiguous (ncond, dim+1) int32 (pylbm/boundary.py:226-235)."""
        self.iload = [np.ascontiguousarray(il.T, dtype=np.int32) for il in self.iload]
        self.istore = np.ascontiguousarray(self.istore.T, dtype=np.int32)

    def _wall_points(self, sim, sel):
        """Wall point of every selected link: x_g + (1 - distance) v_k dx."""
        dim = sim.domain.dim
        k = self.istore[0, sel]
        s = 1.0 - self.distance[sel]
        v = self.stencil.get_all_velocities()
        coords = []
        for d in range(dim):
            x = sim.domain.coords_halo[d][self.istore[d + 1, sel]] + s * v[k, d] * sim.domain.dx
            x = x.ravel()
            for _ in range(1, dim):
                x = x[:, np.newaxis]
            coords.append(x)
        return coords

    def _eval_value(self, sim, func, args, sel, t=None):
        n = sel.size
        shape = [sim.scheme.nv, n] + [1] * (sim.domain.dim - 1)
        m = _Moments(np.zeros(shape), sim.scheme.consm)
        f = _Moments(np.zeros(shape), sim.scheme.consm)
        if t is None:
            func(f, m, *args)
        else:
            func(f, m, t, *args)
        cons = m.array.reshape(sim.scheme.nv, n)[:sim.scheme.nconsm]
        if hasattr(sim, "feq_host"):
            return sim.feq_host(cons)
        return sim.scheme.feq_numpy(cons, sim.extra_parameters_str())

    def prepare_rhs(self, sim):
        """Equilibrium populations at the wall points of labels with a value."""
        self._timed = []
        for label, value in self.value_bc.items():
            if value is None:
                continue
            sel = np.where(self.ilabel == label)[0]
            coords = self._wall_points(sim, sel)
            func, extra = (value[0], tuple(value[1]) if len(value) > 1 else ()) if isinstance(value, tuple) else (value, ())
            args = tuple(coords) + extra
            t = 0.0 if self.time_bc[label] else None
            self.feq[:, sel] = self._eval_value(sim, func, args, sel, t)
            if self.time_bc[label]:
                self._timed.append((func, args, sel))

    def update_feq(self, sim):
        """Re-evaluate time-dependent boundary values (pylbm/boundary.py:307-321)."""
        for func, args, sel in self._timed:
            self.feq[:, sel] = self._eval_value(sim, func, args, sel, sim.t)
        return bool(self._timed)


class BounceBack(BoundaryMethod):
    """f_k(x_g) = f_k'(x_g + v_k) + feq_k - feq_k'  (pylbm/boundary.py:400-469)."""

    kind = "bounce_back"
    name = "bounce_back"

    def set_iload(self):
        k = self.istore[0]
        ksym = self.stencil.get_symmetric()[k][np.newaxis, :]
        v = self.stencil.get_all_velocities()
        self.iload.append(np.concatenate([ksym, self.istore[1:] + v[k].T]))

    def set_rhs(self):
        k = self.istore[:, 0]
        ksym = self.stencil.get_symmetric()[k]
        i = np.arange(k.size)
        self.rhs[:] = self.feq[k, i] - self.feq[ksym, i]


class AntiBounceBack(BounceBack):
    """f_k(x_g) = -f_k'(x_g + v_k) + feq_k + feq_k'  (pylbm/boundary.py:626-684)."""

    kind = "anti_bounce_back"
    name = "anti_bounce_back"

    def set_rhs(self):
        k = self.istore[:, 0]
        ksym = self.stencil.get_symmetric()[k]
        i = np.arange(k.size)
        self.rhs[:] = self.feq[k, i] + self.feq[ksym, i]


class BouzidiBounceBack(BoundaryMethod):
    """Interpolated bounce-back of Bouzidi, Firdaouss and Lallemand (pylbm/boundary.py:472-623).

    f_k(x_g) = (1 - s) f_l1 + s f_l0 + feq_k - feq_k', with the loads taken
    from the populations as they were before the method ran.  For a wall at
    distance q < 1/2 of the link: l0 = (k', x_g + v_k), l1 = (k', x_g + 2 v_k),
    s = 2q; otherwise l0 = (k', x_g + v_k), l1 = (k, x_g + v_k), s = 1/(2q)
    (``set_iload``, pylbm/boundary.py:508-534).
    """

    kind = "bouzidi_bounce_back"
    name = "Bouzidi_bounce_back"

    def __init__(self, *args, **kwargs):
        super().__init__(*args, **kwargs)
        self.s = np.empty(self.istore.shape[1])

    def set_iload(self):
        k = self.istore[0]
        ksym = self.stencil.get_symmetric()[k]
        v = self.stencil.get_all_velocities()
        iload1 = np.zeros(self.istore.shape, dtype=np.int32)
        iload2 = np.zeros(self.istore.shape, dtype=np.int32)
        near = self.distance < 0.5
        far = np.logical_not(near)
        iload1[0] = ksym
        iload2[0, near] = ksym[near]
        iload2[0, far] = k[far]
        iload1[1:] = self.istore[1:] + v[k].T
        iload2[1:, near] = self.istore[1:, near] + 2 * v[k[near]].T
        iload2[1:, far] = self.istore[1:, far] + v[k[far]].T
        self.s[near] = 2.0 * self.distance[near]
        self.s[far] = 0.5 / self.distance[far]
        self.iload.append(iload1)
        self.iload.append(iload2)

    def set_rhs(self):
        k = self.istore[:, 0]
        ksym = self.stencil.get_symmetric()[k]
        i = np.arange(k.size)
        self.rhs[:] = self.feq[k, i] - self.feq[ksym, i]


class BouzidiAntiBounceBack(BouzidiBounceBack):
    """Interpolated anti-bounce-back (pylbm/boundary.py:687-760).

    f_k(x_g) = (1 - s) f_l1 - s f_l0 + feq_k + feq_k', loads and stores in
    the populations themselves, links in list order.
    """

    kind = "bouzidi_anti_bounce_back"
    name = "Bouzidi_anti_bounce_back"

    def set_rhs(self):
        k = self.istore[:, 0]
        ksym = self.stencil.get_symmetric()[k]
        i = np.arange(k.size)
        self.rhs[:] = self.feq[k, i] + self.feq[ksym, i]


class Neumann(BoundaryMethod):
    """f_k(x_g) = f_k(x_g + v_k)  (pylbm/boundary.py:763-823)."""

    kind = "neumann"
    name = "neumann"

    def set_iload(self):
        k = self.istore[0]
        v = self.stencil.get_all_velocities()
        self.iload.append(np.concatenate([k[np.newaxis, :], self.istore[1:] + v[k].T]))


class _NeumannAxis(Neumann):
    axis = 0

    def set_iload(self):
        k = self.istore[0]
        v = self.stencil.get_all_velocities()
        ind = self.istore[1:].copy()
        ind[self.axis] += v[k].T[self.axis]
        self.iload.append(np.concatenate([k[np.newaxis, :], ind]))


class NeumannX(_NeumannAxis):
    """Neumann along x only (pylbm/boundary.py:826-847)."""
    name = "neumannx"
    axis = 0


class NeumannY(_NeumannAxis):
    """Neumann along y only (pylbm/boundary.py:850-871)."""
    name = "neumanny"
    axis = 1


class NeumannZ(_NeumannAxis):
    """Neumann along z only (pylbm/boundary.py:874-895)."""
    name = "neumannz"
    axis = 2


_BY_NAME = {c.__name__: c for c in (BounceBack, AntiBounceBack, BouzidiBounceBack, BouzidiAntiBounceBack,
                                     Neumann, NeumannX, NeumannY, NeumannZ)}


def resolve_method(cls):
    """Map a pylbm boundary class (or one of ours) to this module's class by name."""
    if isinstance(cls, type) and issubclass(cls, BoundaryMethod):
        return cls
    name = getattr(cls, "__name__", str(cls))
    if name in _BY_NAME:
        return _BY_NAME[name]
    raise NotImplementedError(f"boundary method {name} is not supported by the CUDA backend")


class Boundary:
    """Boundary link lists per method (pylbm/boundary.py:50-160)."""

    def __init__(self, domain, dico):
        self.domain = domain
        st = domain.stencil
        labels = [int(l) for l in domain.list_of_labels() if int(l) not in (-1, -2)]
        bv = {lab: [_BoundaryVelocity(domain, lab, k) for k in range(st.unvtot)] for lab in labels}
        dico_bound = dico.get("boundary_conditions", {}) or {}
        istore = OrderedDict()
        ilabel, distance = {}, {}
        value_bc, time_bc = {}, {}
        for lab in labels:
            if lab not in dico_bound:
                raise ValueError(f"no boundary condition given for label {lab}")
            value_bc[lab] = dico_bound[lab].get("value", None)
            time_bc[lab] = dico_bound[lab].get("time_bc", False)
            for ksch, cls in dico_bound[lab]["method"].items():
                meth = resolve_method(cls)
                for inum, num in enumerate(st.num(ksch)):
                    b = bv[lab][int(st.unum2index[num])]
                    if b.indices.size == 0:
                        continue
                    n = b.indices.shape[1]
                    vel = (inum + int(st.nv_ptr[ksch])) * np.ones((1, n), dtype=np.int64)
                    block = np.concatenate([vel, b.indices])
                    if meth not in istore:
                        istore[meth] = block.copy()
                        ilabel[meth] = lab * np.ones(n, dtype=np.int64)
                        distance[meth] = b.distance.copy()
                    else:
                        istore[meth] = np.concatenate([istore[meth], block], axis=1)
                        ilabel[meth] = np.concatenate([ilabel[meth], lab * np.ones(n, dtype=np.int64)])
                        distance[meth] = np.concatenate([distance[meth], b.distance])
        self.methods = [cls(istore[cls], ilabel[cls], distance[cls], st, value_bc, time_bc) for cls in istore]


def _sorted_unique(a):
    """Sorted distinct values of an int64 array (a sort, not a hash table)."""
    a = np.sort(a, kind="stable")
    return a[np.concatenate(([True], a[1:] != a[:-1]))] if a.size else a


def observed_ghost_copies(shape_in, halo, velocities, methods):
    """The periodic ghost copies of a step whose values something reads.

    pylbm refreshes every ghost population of every axis before the boundary
    methods (its MPI topology is periodic along all axes,
    pylbm/domain.py:373-383, pylbm/storage.py:307-367).  On a bounded domain
    most of those values are never read: a fluid node's pull from a ghost
    crosses a wall, so a boundary method stores that slot first.  A ghost
    population (k, g) is observed when

    * an interior node pulls it (x - v_k = g) and no method stores it, or
    * a method loads it and no earlier method stores it.

    Returns ``(istore, iload)``, int32 link arrays ``[k, i_0, ...]`` in halo
    coordinates with iload the periodic image of istore (the copy
    ``lbm_update_halo`` makes), or None when an axis is shorter than its halo
    (the periodic image is then itself a ghost and the full refresh decides).
    """
    n = np.asarray(shape_in, dtype=np.int64)
    h = np.asarray(halo, dtype=np.int64)
    dim = n.size
    if np.any(n < h):
        return None
    ext = n + 2 * h
    box = int(np.prod(ext))

    def keys(lst):
        lst = np.asarray(lst, dtype=np.int64).reshape(-1, dim + 1)
        return lst[:, 0] * box + np.ravel_multi_index(tuple(lst[:, 1:].T), tuple(ext))

    def is_ghost(lst):
        c = np.asarray(lst, dtype=np.int64).reshape(-1, dim + 1)[:, 1:]
        return np.any((c < h) | (c >= h + n), axis=1)

    stored = _sorted_unique(np.concatenate([keys(m.istore) for m in methods] + [np.zeros(0, np.int64)]))
    parts = []
    for k, v in enumerate(np.asarray(velocities, dtype=np.int64).reshape(-1, dim)):
        for d in np.flatnonzero(v):
            # interior nodes whose source x - v leaves the interior along axis d
            box_d = [np.arange(a, a + b) for a, b in zip(h, n)]
            box_d[d] = np.arange(h[d], h[d] + v[d]) if v[d] > 0 else np.arange(h[d] + n[d] + v[d], h[d] + n[d])
            src = np.meshgrid(*[c - s for c, s in zip(box_d, v)], indexing="ij")
            parts.append(k * box + np.ravel_multi_index(tuple(c.ravel() for c in src), tuple(ext)))
    pulled = _sorted_unique(np.concatenate(parts)) if parts else np.zeros(0, np.int64)
    needed = [np.setdiff1d(pulled, stored, assume_unique=True)]
    before = np.zeros(0, np.int64)
    for m in methods:
        for il in m.iload:
            g = is_ghost(il)
            needed.append(np.setdiff1d(_sorted_unique(keys(il)[g]), before, assume_unique=True))
        before = _sorted_unique(np.concatenate([before, keys(m.istore)]))
    needed = _sorted_unique(np.concatenate(needed))
    k, rem = np.divmod(needed, box)
    c = np.array(np.unravel_index(rem, tuple(ext)), dtype=np.int64).reshape(dim, -1)
    src = np.where(c < h[:, None], c + n[:, None], np.where(c >= (n + h)[:, None], c - n[:, None], c))
    istore = np.ascontiguousarray(np.column_stack([k, c.T]), dtype=np.int32)
    iload = np.ascontiguousarray(np.column_stack([k, src.T]), dtype=np.int32)
    return istore, iload


def batch_entries(methods, ext, ghost=None):
    """The links of one lbm_boundary_batch launch, equal to the ghost copies
    followed by the methods applied one after the other, or None.

    Every link of a batch reads the populations as they are before the
    launch.  Two kinds of load see a value another link writes in the
    sequential order, and are rewritten: a load of a copied ghost slot reads
    the copy's source, and a Neumann link whose load slot another
    (non-Neumann) method stores takes that method's formula for the slot and
    stores its result (the value the copy would have moved).  A slot stored
    twice, a load of a slot a non-Neumann link stores or a copy of a copy
    keep the methods sequential (None).

    ``methods``: boundary methods with (ncond, dim+1) lists; ``ext``: the
    slot extents [nv, n0 + 2 h0, ...]; ``ghost``: (istore, iload) of the
    observed ghost copies or None.  Returns (entries, ghost_joined) with
    entries of kind, iload (list of lists), istore, method (index whose rhs
    and distances the entry uses) and links (indices into that method's
    lists, None for all)."""
    ext = tuple(int(e) for e in ext)

    def keys(lst):
        lst = np.asarray(lst, dtype=np.int64).reshape(-1, len(ext))
        return np.ravel_multi_index(tuple(lst.T), ext)

    if not methods:
        return None
    empty = np.zeros(0, np.int64)
    st_keys = [keys(m.istore) for m in methods]
    stores = np.concatenate(st_keys + [empty])
    order = np.argsort(stores, kind="stable")
    st_sorted = stores[order]
    if st_sorted.size and (st_sorted[1:] == st_sorted[:-1]).any():
        return None  # a slot stored twice: the method order decides
    owner_m = np.concatenate([np.full(len(k), i) for i, k in enumerate(st_keys)] + [empty])
    owner_l = np.concatenate([np.arange(len(k)) for k in st_keys] + [empty])
    entries = []
    for i, m in enumerate(methods):
        loads = [keys(il) for il in m.iload]
        hits = [np.isin(k, stores) for k in loads]
        if not any(h.any() for h in hits):
            entries.append({"kind": m.kind, "iload": list(m.iload), "istore": m.istore, "method": i,
                            "links": None})
            continue
        if m.kind != "neumann":
            return None
        h = hits[0]
        src = order[np.searchsorted(st_sorted, loads[0][h])]
        pm, pl = owner_m[src], owner_l[src]
        if any(methods[p].kind == "neumann" for p in np.unique(pm)):
            return None  # a copy of a copy
        keep = np.flatnonzero(~h)
        if keep.size:
            entries.append({"kind": "neumann", "iload": [m.iload[0][keep]], "istore": m.istore[keep],
                            "method": i, "links": keep})
        for p in np.unique(pm):
            sel = pm == p
            links = pl[sel]
            entries.append({"kind": methods[p].kind, "iload": [il[links] for il in methods[p].iload],
                            "istore": m.istore[h][sel], "method": int(p), "links": links})
    joined = False
    if ghost is not None and not np.isin(keys(ghost[1]), stores).any():
        # the copies read interior slots that no method stores, so they join
        # the launch; a load of a copied ghost slot reads the copy's source
        gst = keys(ghost[0])
        gorder = np.argsort(gst)
        gsorted = gst[gorder]
        for e in entries:
            fwd = []
            for il in e["iload"]:
                kk = keys(il)
                pos = np.minimum(np.searchsorted(gsorted, kk), len(gsorted) - 1)
                hit = gsorted[pos] == kk
                if hit.any():
                    il = np.array(il, copy=True)
                    il[hit] = ghost[1][gorder[pos[hit]]]
                fwd.append(il)
            e["iload"] = fwd
        joined = True
    return entries, joined


def wall_signature(ghost, shape_in, halo):
    """Index 9 (o0 + 1) + 3 (o1 + 1) + (o2 + 1) of the walls a ghost slot lies
    beyond: o_d = -1 below the interior along axis d, +1 above it, else 0."""
    c = np.asarray(ghost, dtype=np.int64).reshape(len(shape_in), -1)
    n = np.asarray(shape_in, dtype=np.int64)[:, None]
    h = np.asarray(halo, dtype=np.int64)[:, None]
    o = np.where(c < h, -1, np.where(c >= n + h, 1, 0))
    o = np.concatenate([o, np.zeros((3 - len(shape_in), o.shape[1]), dtype=np.int64)])
    return 9 * (o[0] + 1) + 3 * (o[1] + 1) + (o[2] + 1)


def box_wall_table(methods, shape_in, halo, velocities, constants):
    """Bounce-back box walls folded into the pull.

    On a box whose every boundary link is a bounce-back link of a wall (no
    element, no periodic axis, no time-dependent value), the ghost slot
    (k, x - v_k) a wall node x pulls from holds f_k'(x) + c, k' = opposite
    of k, written by exactly one link, and c depends only on k and the walls
    the slot lies beyond.  The step can then read f_k'(x) + c itself instead
    of the ghost a boundary launch wrote (pylbm/boundary.py:400-469).

    ``constants[m]`` are the per-link constants of method m in the arithmetic
    of the boundary launch (float64 right-hand sides, or the FP32 constants of
    the stored deviations).  Returns the table c[k][signature] (27 entries per
    population, wall_signature) or None when the links do not have that form.
    """
    n = np.asarray(shape_in, dtype=np.int64)
    h = np.asarray(halo, dtype=np.int64)
    dim = n.size
    v = np.asarray(velocities, dtype=np.int64).reshape(-1, dim)
    nv = v.shape[0]
    if np.any(h != 1) or np.any(np.abs(v) > 1) or not methods:
        return None
    if any(m.kind != "bounce_back" or m._timed for m in methods):
        return None
    table = np.zeros((nv, 27))
    seen = np.zeros((nv, 27), dtype=bool)
    slots = []
    for m, const in zip(methods, constants):
        st = np.asarray(m.istore, dtype=np.int64).reshape(-1, dim + 1)
        il = np.asarray(m.iload[0], dtype=np.int64).reshape(-1, dim + 1)
        k = st[:, 0]
        # a bounce-back link loads the opposite population at the fluid node x_g + v_k
        if np.any(il[:, 1:] != st[:, 1:] + v[k]):
            return None
        sig = wall_signature(st[:, 1:].T, n, h)
        if np.any(sig == 13):  # a store into the interior
            return None
        const = np.asarray(const, dtype=np.float64)
        for kk, ss, cc in zip(k, sig, const):
            if seen[kk, ss] and table[kk, ss] != cc:
                return None
            table[kk, ss] = cc
            seen[kk, ss] = True
        slots.append(st[:, 0] * int(np.prod(n + 2 * h)) + np.ravel_multi_index(tuple(st[:, 1:].T), tuple(n + 2 * h)))
    slots = np.concatenate(slots)
    # exactly one link for every (population, interior node) whose source leaves the box
    expected = sum(int(np.prod(n)) - int(np.prod(n - np.abs(vk))) for vk in v)
    if slots.size != expected or np.unique(slots).size != slots.size:
        return None
    return table
