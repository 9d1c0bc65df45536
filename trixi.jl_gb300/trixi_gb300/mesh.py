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


class _Tree:
    """The refinement tree of a TreeMesh (abstract_tree.jl): cells keyed by
    (level, integer position); a same-level neighbour exists iff its key is
    present (periodic wrap per dimension), as Trixi's neighbour links record."""

    def __init__(self, ndims, periodicity, length0, center0):
        self.D = ndims
        self.periodicity = periodicity
        self.length0 = length0
        self.level, self.ix, self.center, self.child0 = [], [], [], []
        self.index = {}
        self._add(0, (0,) * ndims, tuple(center0))

    def _add(self, level, ix, c):
        self.index[(level, ix)] = len(self.level)
        self.level.append(level)
        self.ix.append(ix)
        self.center.append(c)
        self.child0.append(-1)

    def length(self, level):
        return self.length0 / (1 << level)

    def is_leaf(self, cell):
        return self.child0[cell] < 0

    def neighbour(self, cell, direction):
        """Same-level neighbour across face `direction` (0: -x, 1: +x, ...) or -1."""
        lev, ix = self.level[cell], list(self.ix[cell])
        d = direction // 2
        M = 1 << lev
        ix[d] += 1 if direction & 1 else -1
        if not 0 <= ix[d] < M:
            if not self.periodicity[d]:
                return -1
            ix[d] %= M
        return self.index.get((lev, tuple(ix)), -1)

    def parent(self, cell):
        lev = self.level[cell]
        if lev == 0:
            return -1
        return self.index[(lev - 1, tuple(i >> 1 for i in self.ix[cell]))]

    def _refine_cell(self, cell):
        # init_child! / child_coordinates (abstract_tree.jl:668-674)
        lev, ix, c = self.level[cell], self.ix[cell], self.center[cell]
        child_len = self.length(lev) / 2
        self.child0[cell] = len(self.level)
        for ch in range(1 << self.D):
            bits = [(ch >> d) & 1 for d in range(self.D)]
            self._add(lev + 1, tuple(2 * i + b for i, b in zip(ix, bits)),
                      tuple(cc + (1.0 if b else -1.0) * child_len / 2 for cc, b in zip(c, bits)))

    def refine(self, cells):
        """refine!(t, cell_ids): refine the given leaves, then rebalance! until no
        two face neighbours differ by more than one level (abstract_tree.jl:367-402,
        453-489)."""
        refined = sorted(set(cells))
        for c in refined:
            self._refine_cell(c)
        while refined:
            marks = set()
            for cell in refined:
                for direction in range(2 * self.D):
                    if self.neighbour(cell, direction) >= 0:
                        continue
                    p = self.parent(cell)
                    if p < 0:
                        continue
                    pn = self.neighbour(p, direction)
                    if pn >= 0:
                        marks.add(pn)
            refined = sorted(marks)
            for c in refined:
                self._refine_cell(c)

    def coarsen(self, parents):
        """coarsen!(t, cell_ids), abstract_tree.jl:516-618: parents whose children
        are all leaves, highest level first; a parent is kept when one of its
        children has a same-level neighbour with children across a face that is
        not shared with a sibling (the 2:1 rule).  Returns {parent: first child}
        of the coarsened parents."""
        order = sorted(parents, key=lambda c: self.level[c])  # stable, as Julia's sort
        done = {}
        nch = 1 << self.D
        while order:
            cell = order.pop()
            first = self.child0[cell]
            skip = False
            for ch in range(nch):
                c = first + ch
                for direction in range(2 * self.D):
                    if (ch >> (direction // 2)) & 1 != direction & 1:
                        continue  # the neighbour across this face is a sibling
                    nb = self.neighbour(c, direction)
                    if nb >= 0 and not self.is_leaf(nb):
                        skip = True
                        break
                if skip:
                    break
            if skip:
                continue
            for ch in range(nch):
                del self.index[(self.level[first + ch], self.ix[first + ch])]
            self.child0[cell] = -1
            done[cell] = first
        return done

    def leaves(self):
        """Leaf cells depth-first with children in _child_signs order."""
        out, stack = [], [0]
        nch = 1 << self.D
        while stack:
            cell = stack.pop()
            if self.child0[cell] < 0:
                out.append(cell)
            else:
                stack.extend(range(self.child0[cell] + nch - 1, self.child0[cell] - 1, -1))
        return out


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
        abstract_tree.jl:405-447)."""
        t = _Tree(self.ndims, self.periodicity, self.length_level_0, self.center_level_0)
        for _ in range(self.initial_refinement_level):
            t.refine(t.leaves())
        for kind, a, b in self.refinement_patches:
            sel = []
            for cell in t.leaves():
                c = t.center[cell]
                if kind == "box":
                    inside = all(lo < x < hi for x, lo, hi in zip(c, a, b))
                else:
                    inside = sum((x - y) ** 2 for x, y in zip(c, a)) < b * b
                if inside:
                    sel.append(cell)
            if sel:
                t.refine(sel)
        self._tree = t
        self._leaves = t.leaves()

    @property
    def nelements(self) -> int:
        if self._tree is not None:
            return len(self._leaves)
        return self.cartesian.shape[0]

    def _ensure_tree(self):
        if self._tree is None:
            self._build_tree()
            del self.cartesian

    def adapt(self, controller_value, only_refine=False, only_coarsen=False):
        """One AMR pass on the tree (amr.jl:244-392): refine! the leaves with
        controller_value > 0 (with rebalancing), then coarsen! the parents whose
        children all have controller_value < 0.  Returns (changed,
        source_element, kind) for the elements of the adapted mesh: kind 0 copies
        element source_element, 1 + q is child q of the refined element
        source_element, -1 the parent of the coarsened elements source_element ..
        source_element + 2^ndims - 1 (the layout tg_adapt_state takes)."""
        self._ensure_tree()
        t = self._tree
        lam = np.asarray(controller_value)
        if lam.shape != (len(self._leaves),):
            raise ValueError("one controller value per element")
        old_leaves = self._leaves
        old_elem = {c: e for e, c in enumerate(old_leaves)}
        to_refine = [old_leaves[e] for e in np.flatnonzero(lam > 0)]
        to_coarsen = [old_leaves[e] for e in np.flatnonzero(lam < 0)]
        changed = False
        former = {}
        if not only_coarsen and to_refine:
            t.refine(to_refine)
            changed = True
        if not only_refine and to_coarsen:
            count = {}
            parents = []
            nch = 1 << self.ndims
            for cell in to_coarsen:
                if t.level[cell] == 0 or not t.is_leaf(cell):
                    continue
                p = t.parent(cell)
                count[p] = count.get(p, 0) + 1
                if count[p] == nch:
                    parents.append(p)
            former = t.coarsen(sorted(parents))
            changed = changed or bool(former)
        if not changed:
            return False, None, None
        self._leaves = t.leaves()
        E = len(self._leaves)
        src = np.zeros(E, dtype=np.int64)
        kind = np.zeros(E, dtype=np.int8)
        for e, cell in enumerate(self._leaves):
            if cell in old_elem:
                src[e] = old_elem[cell]
            elif cell in former:
                src[e], kind[e] = old_elem[former[cell]], -1
            else:
                p = t.parent(cell)
                src[e], kind[e] = old_elem[p], 1 + (cell - t.child0[p])
        return True, src, kind

    @property
    def is_uniform(self) -> bool:
        if self._tree is None:
            return True
        return len({self._tree.level[c] for c in self._leaves}) == 1

    def cell_centers(self):
        """Cell midpoints, computed like child_coordinates (abstract_tree.jl:668-674):
        each level adds sign * (parent_length / 2) / 2 to the parent centre."""
        if self._tree is not None:
            return np.array([self._tree.center[c] for c in self._leaves], dtype=np.float64)
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
            return np.array([self._tree.length(self._tree.level[c]) for c in self._leaves])
        return np.full(self.nelements, self.length_level_0 / (1 << self.initial_refinement_level))

    def element_levels(self):
        if self._tree is not None:
            return np.array([self._tree.level[c] for c in self._leaves], dtype=np.int64)
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
        t, D = self._tree, self.ndims
        c2e = {c: e for e, c in enumerate(self._leaves)}
        nb, orient = [], []
        for e, cell in enumerate(self._leaves):
            for d in range(D):
                n = t.neighbour(cell, 2 * d + 1)
                if n >= 0 and t.is_leaf(n):
                    nb.append((e + 1, c2e[n] + 1))
                    orient.append(d + 1)
        return (np.array(nb, dtype=np.int64).reshape(-1, 2),
                np.array(orient, dtype=np.int64))

    def mortars(self):
        """cache.mortars of L2 mortars (init_mortars!, containers_2d.jl:707-810,
        containers_3d.jl:652-790): neighbor_ids [M, 2^(ndims-1) + 1] (1-based; the
        small elements facing the large one in child order, then the large one),
        large_sides [M] (1: large element on the negative side), orientations [M]."""
        D = self.ndims
        ns = 1 << (D - 1)
        if self._tree is None:
            return (np.zeros((0, ns + 1), dtype=np.int64), np.zeros(0, dtype=np.int64),
                    np.zeros(0, dtype=np.int64))
        t = self._tree
        c2e = {c: e for e, c in enumerate(self._leaves)}
        ids, ls, orient = [], [], []
        for e, cell in enumerate(self._leaves):
            for direction in range(2 * D):
                n = t.neighbour(cell, direction)
                if n < 0 or t.is_leaf(n):
                    continue
                d = direction // 2
                want = 0 if direction & 1 else 1
                small = [t.child0[n] + ch for ch in range(1 << D) if (ch >> d) & 1 == want]
                if not all(t.is_leaf(c) for c in small):
                    raise RuntimeError("refinement tree is not 2:1 balanced")
                ids.append([c2e[c] + 1 for c in small] + [e + 1])
                ls.append(1 if direction & 1 else 2)
                orient.append(d + 1)
        return (np.array(ids, dtype=np.int64).reshape(-1, ns + 1),
                np.array(ls, dtype=np.int64), np.array(orient, dtype=np.int64))

    def __repr__(self):
        per = "periodic" if all(self.periodicity) else f"periodicity {self.periodicity}"
        return (f"TreeMesh{{{self.ndims}}} with {self.nelements} elements "
                f"(level {self.initial_refinement_level}, {per})")
