"""Uniformly refined TreeMesh (host setup), periodic or not per dimension.

Element order is Trixi's: cells are created depth-first with children in
_child_signs order (x fastest, then y, then z; abstract_tree.jl:122-130,
206-248), and elements are the leaf cells in cell-id order
(abstract_tree.jl:154-174).  For a uniform refinement that is the Morton
(Z-order) curve with x as the lowest bit.  Interfaces are created per element
in the positive directions only (containers_2d.jl:228-284).
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


class TreeMesh:
    """TreeMesh(coordinates_min, coordinates_max; initial_refinement_level, periodicity),
    tree_mesh.jl:128-185 (uniform).  periodicity: a bool for all dimensions or one
    per dimension; faces at a non-periodic domain edge are boundaries."""

    def __init__(self, coordinates_min, coordinates_max, initial_refinement_level: int,
                 periodicity=True, n_cells_max=None):
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
        self.cartesian = _morton_cells(self.ndims, initial_refinement_level)

    @property
    def nelements(self) -> int:
        return self.cartesian.shape[0]

    def cell_centers(self):
        """Cell midpoints, computed like child_coordinates (abstract_tree.jl:668-674):
        each level adds sign * (parent_length / 2) / 2 to the parent centre."""
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
        return self.length_level_0 / (1 << self.initial_refinement_level)

    def interfaces(self):
        """neighbor_ids [I, 2] (1-based, (left, right)) and orientations [I] (1-based),
        per element in order and positive directions only where a neighbour
        exists (init_interfaces!, containers_2d.jl:228-284)."""
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

    def __repr__(self):
        per = "periodic" if all(self.periodicity) else f"periodicity {self.periodicity}"
        return (f"TreeMesh{{{self.ndims}}} with {self.nelements} elements "
                f"(level {self.initial_refinement_level}, {per})")
