"""TreeMesh (host setup): a uniform initial refinement plus optional
refinement patches, periodic or not per dimension.

Element order is Trixi's: cells are created depth-first with children in
_child_signs order (x fastest, then y, then z; abstract_tree.jl:122-130,
206-248), and elements are the leaf cells in cell-id order
(abstract_tree.jl:154-174).  For a uniform refinement that is the Morton
(Z-order) curve with x as the lowest bit.  Interfaces are created per element
in the positive directions only (containers_2d.jl:228-284); L2 mortars per
large element in every direction towards a refined neighbour
(containers_2d.jl:660-810, containers_3d.jl:652-790).
"""
from __future__ import annotations

import ctypes

import numpy as np


def _morton_cells(ndims: int, level: int):
    """Cartesian index [E, ndims] of each leaf in depth-first (Morton) order."""
    E = 1 << (ndims * level)
    codes = np.arange(E, dtype=np.int64)
    cart = np.zeros((E, ndims), dtype=np.int64)
    for b in range(level):
        for d in range(ndims):
            bit = (codes >> (ndims * b + d)) & 1
            cart[:, d] |= bit << b
    return cart


class _NativeTree:
    """The refinement tree of a TreeMesh, held by the library (tg_tree_*: Trixi's
    refine!/coarsen! rules and the containers of the leaves, in C++)."""

    def __init__(self, ndims, level, cmin, cmax, periodicity):
        from . import _lib
        self._lib = _lib
        self.lib = _lib.load()
        self.ndims = ndims
        h = ctypes.c_void_p()
        lo = np.ascontiguousarray(cmin, dtype=np.float64)
        hi = np.ascontiguousarray(cmax, dtype=np.float64)
        per = np.ascontiguousarray([int(p) for p in periodicity] + [1] * (3 - ndims), dtype=np.int32)
        _lib.check(self.lib.tg_tree_create(ndims, level, _dp(lo), _dp(hi),
                                           per.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                           ctypes.byref(h)))
        self.h = h

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.tg_tree_destroy(self.h)
            self.h = None

    def refine_patch(self, kind, a, b):
        pa = np.zeros(3)
        pa[:self.ndims] = a
        if kind == "box":
            pb = np.zeros(3)
            pb[:self.ndims] = b
            self._lib.check(self.lib.tg_tree_refine_patch(self.h, 0, _dp(pa), _dp(pb), 0.0))
        else:
            self._lib.check(self.lib.tg_tree_refine_patch(self.h, 1, _dp(pa), None, float(b)))

    def nelements(self):
        n = ctypes.c_int64()
        self._lib.check(self.lib.tg_tree_nelements(self.h, ctypes.byref(n)))
        return n.value

    def elements(self):
        E = self.nelements()
        lev = np.zeros(E, dtype=np.int32)
        ctr = np.zeros((E, self.ndims))
        self._lib.check(self.lib.tg_tree_elements(
            self.h, lev.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), _dp(ctr)))
        return lev.astype(np.int64), ctr

    def containers(self):
        ni, nm = ctypes.c_int64(), ctypes.c_int64()
        self._lib.check(self.lib.tg_tree_counts(self.h, ctypes.byref(ni), ctypes.byref(nm)))
        ns = 1 << (self.ndims - 1)
        nb = np.zeros((ni.value, 2), dtype=np.int64)
        orient = np.zeros(ni.value, dtype=np.int64)
        mids = np.zeros((nm.value, ns + 1), dtype=np.int64)
        ls = np.zeros(nm.value, dtype=np.int64)
        mor = np.zeros(nm.value, dtype=np.int64)
        self._lib.check(self.lib.tg_tree_interfaces(self.h, _ip(nb), _ip(orient)))
        self._lib.check(self.lib.tg_tree_mortars(self.h, _ip(mids), _ip(ls), _ip(mor)))
        return (nb, orient), (mids, ls, mor)

    def adapt(self, controller_value, only_refine, only_coarsen):
        lam = np.ascontiguousarray(controller_value, dtype=np.int8)
        changed = ctypes.c_int32()
        self._lib.check(self.lib.tg_tree_adapt(self.h, lam.ctypes.data_as(ctypes.POINTER(ctypes.c_int8)),
                                               int(only_refine), int(only_coarsen),
                                               ctypes.byref(changed)))
        if not changed.value:
            return False, None, None
        E = self.nelements()
        src = np.zeros(E, dtype=np.int64)
        kind = np.zeros(E, dtype=np.int8)
        self._lib.check(self.lib.tg_tree_transfer_map(
            self.h, _ip(src), kind.ctypes.data_as(ctypes.POINTER(ctypes.c_int8))))
        return True, src, kind


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))


def _patch(p, ndims):
    """A refinement patch as in tree_mesh.jl:194-203: (type = "box",
    coordinates_min, coordinates_max) or (type = "sphere", center, radius)."""
    get = p.get if isinstance(p, dict) else (lambda k, default=None: getattr(p, k, default))
    kind = get("type")
    if kind == "box":
        lo = tuple(float(x) for x in get("coordinates_min"))
        hi = tuple(float(x) for x in get("coordinates_max"))
        if len(lo) != ndims or len(hi) != ndims or any(a >= b for a, b in zip(lo, hi)):
            raise ValueError("a box patch needs coordinates_min < coordinates_max per dimension")
        return ("box", lo, hi)
    if kind == "sphere":
        c = tuple(float(x) for x in get("center"))
        r = float(get("radius"))
        if len(c) != ndims or r < 0:
            raise ValueError("a sphere patch needs a center per dimension and a radius >= 0")
        return ("sphere", c, r)
    raise ValueError(f"unknown refinement patch type {kind!r}")


class TreeMesh:
    """TreeMesh(coordinates_min, coordinates_max; initial_refinement_level, periodicity),
    tree_mesh.jl:128-185 (uniform).  periodicity: a bool for all dimensions or one
    per dimension; faces at a non-periodic domain edge are boundaries."""

    def __init__(self, coordinates_min, coordinates_max, initial_refinement_level: int,
                 periodicity=True, n_cells_max=None, refinement_patches=()):
        cmin = tuple(float(x) for x in coordinates_min)
        cmax = tuple(float(x) for x in coordinates_max)
        if len(cmin) != len(cmax) or len(cmin) not in (2, 3):
            raise ValueError("TreeMesh needs 2 or 3 coordinates")
        if isinstance(periodicity, (tuple, list)):
            if len(periodicity) != len(cmin):
                raise ValueError("periodicity needs one entry per dimension")
            self.periodicity = tuple(bool(p) for p in periodicity)
        else:
            self.periodicity = (bool(periodicity),) * len(cmin)
        if initial_refinement_level < 0:
            raise ValueError("initial_refinement_level must be non-negative")
        length = cmax[0] - cmin[0]
        for d in range(1, len(cmin)):
            if not np.isclose(cmax[d] - cmin[d], length, rtol=np.sqrt(np.finfo(float).eps), atol=0):
                raise ValueError("The TreeMesh domain must be a hypercube")
        self.ndims = len(cmin)
        self.coordinates_min, self.coordinates_max = cmin, cmax
        self.initial_refinement_level = initial_refinement_level
        self.length_level_0 = length
        self.center_level_0 = tuple((a + b) / 2 for a, b in zip(cmin, cmax))
        self.cells_per_dim = 1 << initial_refinement_level
        self.refinement_patches = tuple(_patch(p, self.ndims) for p in refinement_patches)
        self._tree = None
        if self.refinement_patches:
            self._build_tree()
        else:
            self.cartesian = _morton_cells(self.ndims, initial_refinement_level)

    def _build_tree(self):
        """initialize!(mesh, initial_refinement_level, refinement_patches),
        tree_mesh.jl:186-215: uniform refinement, then each patch refines the
        leaves whose centre lies strictly inside it (refine_box!, refine_sphere!,
        abstract_tree.jl:405-447); the tree is the library's (tg_tree_*)."""
        t = _NativeTree(self.ndims, self.initial_refinement_level, self.coordinates_min,
                        self.coordinates_max, self.periodicity)
        for kind, a, b in self.refinement_patches:
            t.refine_patch(kind, a, b)
        self._tree = t
        self._refresh()

    def _refresh(self):
        self._levels, self._centers = self._tree.elements()
        self._interfaces, self._mortars = self._tree.containers()

    @property
    def nelements(self) -> int:
        if self._tree is not None:
            return len(self._levels)
        return self.cartesian.shape[0]

    def _ensure_tree(self):
        if self._tree is None:
            self._build_tree()
            del self.cartesian

    def adapt(self, controller_value, only_refine=False, only_coarsen=False):
        """One AMR pass on the tree (amr.jl:244-392): refine! the elements with
        controller_value > 0 (with rebalancing), then coarsen! the parents whose
        children all have controller_value < 0.  Returns (changed,
        source_element, kind) for the elements of the adapted mesh: kind 0 copies
        element source_element, 1 + q is child q of the refined element
        source_element, -1 the parent of the coarsened elements source_element ..
        source_element + 2^ndims - 1 (the layout tg_adapt_state takes)."""
        self._ensure_tree()
        lam = np.asarray(controller_value)
        if lam.shape != (self.nelements,):
            raise ValueError("one controller value per element")
        changed, src, kind = self._tree.adapt(lam, only_refine, only_coarsen)
        if changed:
            self._refresh()
        return changed, src, kind

    @property
    def is_uniform(self) -> bool:
        if self._tree is None:
            return True
        return bool(np.all(self._levels == self._levels[0]))

    def cell_centers(self):
        """Cell midpoints, computed like child_coordinates (abstract_tree.jl:668-674):
        each level adds sign * (parent_length / 2) / 2 to the parent centre."""
        if self._tree is not None:
            return self._centers.copy()
        L = self.initial_refinement_level
        centers = np.tile(np.array(self.center_level_0), (self.nelements, 1))
        length = self.length_level_0
        for lev in range(L):
            child_len = length / 2
            bit = (self.cartesian >> (L - 1 - lev)) & 1
            sign = np.where(bit == 1, 1.0, -1.0)
            centers = centers + sign * child_len / 2
            length = child_len
        return centers

    def element_length(self) -> float:
        """Edge length of the elements of a uniform mesh."""
        if not self.is_uniform:
            raise ValueError("the elements of this mesh have different sizes")
        return float(self.element_lengths()[0])

    def element_lengths(self):
        """length_at_cell of every element (length_level_0 / 2^level)."""
        if self._tree is not None:
            return self.length_level_0 / np.power(2.0, self._levels)
        return np.full(self.nelements, self.length_level_0 / (1 << self.initial_refinement_level))

    def element_levels(self):
        if self._tree is not None:
            return self._levels.copy()
        return np.full(self.nelements, self.initial_refinement_level, dtype=np.int64)

    def interfaces(self):
        """neighbor_ids [I, 2] (1-based, (left, right)) and orientations [I] (1-based),
        per element in order and positive directions only where a neighbour
        exists (init_interfaces!, containers_2d.jl:228-284)."""
        if self._tree is not None:
            return self._tree_interfaces()
        D, M, E = self.ndims, self.cells_per_dim, self.nelements
        lin = np.zeros(E, dtype=np.int64)
        mult = 1
        for d in range(D):
            lin += self.cartesian[:, d] * mult
            mult *= M
        c2e = np.empty(E, dtype=np.int64)
        c2e[lin] = np.arange(E)
        nb = np.zeros((E, D, 2), dtype=np.int64)
        orient = np.zeros((E, D), dtype=np.int64)
        exists = np.ones((E, D), dtype=bool)
        for d in range(D):
            c = self.cartesian.copy()
            if not self.periodicity[d]:
                exists[:, d] = c[:, d] + 1 < M
            c[:, d] = (c[:, d] + 1) % M
            l2 = np.zeros(E, dtype=np.int64)
            mult = 1
            for dd in range(D):
                l2 += c[:, dd] * mult
                mult *= M
            nb[:, d, 0] = np.arange(E) + 1
            nb[:, d, 1] = c2e[l2] + 1
            orient[:, d] = d + 1
        keep = exists.reshape(E * D)
        return nb.reshape(E * D, 2)[keep], orient.reshape(E * D)[keep]

    def _tree_interfaces(self):
        nb, orient = self._interfaces
        return nb.copy(), orient.copy()

    def mortars(self):
        """cache.mortars of L2 mortars (init_mortars!, containers_2d.jl:707-810,
        containers_3d.jl:652-790): neighbor_ids [M, 2^(ndims-1) + 1] (1-based; the
        small elements facing the large one in child order, then the large one),
        large_sides [M] (1: large element on the negative side), orientations [M]."""
        ns = 1 << (self.ndims - 1)
        if self._tree is None:
            return (np.zeros((0, ns + 1), dtype=np.int64), np.zeros(0, dtype=np.int64),
                    np.zeros(0, dtype=np.int64))
        ids, ls, orient = self._mortars
        return ids.copy(), ls.copy(), orient.copy()

    def __repr__(self):
        per = "periodic" if all(self.periodicity) else f"periodicity {self.periodicity}"
        return (f"TreeMesh{{{self.ndims}}} with {self.nelements} elements "
                f"(level {self.initial_refinement_level}, {per})")
