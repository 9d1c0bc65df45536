"""Curvilinear 2D meshes (host setup): StructuredMesh and P4estMesh built
from a brick of trees.

StructuredMesh(cells_per_dimension, mapping | faces | (coordinates_min,
coordinates_max); periodicity) follows src/meshes/structured_mesh.jl: the
element of cell (cx, cy) is cx + nx cy (x fastest) and its nodes are the mapping
evaluated at the solver's LGL nodes of the cell's part of [-1, 1]^2
(dgsem_structured/containers_2d.jl:37-59).

P4estMesh(trees_per_dimension; polydeg, mapping | faces | coordinates,
initial_refinement_level, periodicity) follows p4est_mesh.jl:189-244: trees in
row order (connectivity_structured, :1149-1240), the mapping evaluated at the
LGL nodes of the mesh polydeg per tree (calc_tree_node_coordinates!,
:1618-1644), each tree refined uniformly with its quadrants in Morton order
(x the lowest bit, p4est's order within a tree), and the element nodes
interpolated from the tree nodes (dgsem_p4est/containers_2d.jl:29-89).

Both give the element node coordinates, the metric terms
(calc_jacobian_matrix!, calc_contravariant_vectors!, calc_inverse_jacobian!,
dgsem_structured/containers_2d.jl:61-152) and the interfaces of a brick whose
faces are all conforming and aligned.  Edges of the brick are periodic or
(per dimension) boundaries.
"""
from __future__ import annotations

import numpy as np

from .basis import gauss_lobatto_nodes_weights, polynomial_interpolation_matrix


def _linear_interpolate(s, left, right):
    # linear_interpolate, structured_mesh.jl:213-215
    return 0.5 * ((1 - s) * left + (1 + s) * right)


def coordinates2mapping(cmin, cmax):
    """coordinates2mapping, structured_mesh.jl:228-233."""
    def mapping(xi, eta):
        return (_linear_interpolate(xi, cmin[0], cmax[0]),
                _linear_interpolate(eta, cmin[1], cmax[1]))
    return mapping


def transfinite_mapping(faces):
    """transfinite_mapping(faces) of four face functions (structured_mesh.jl:254-300):
    faces[0..3] are the faces at xi = -1, xi = 1, eta = -1, eta = 1, each a
    function of the running coordinate in [-1, 1] returning (x, y)."""
    f1, f2, f3, f4 = faces

    def fv(f, s):
        r = f(s)
        return np.asarray(r[0], dtype=float), np.asarray(r[1], dtype=float)

    def mapping(x, y):
        x = np.asarray(x, dtype=float)
        y = np.asarray(y, dtype=float)
        c1, c2, c3, c4 = fv(f1, -1.0), fv(f2, -1.0), fv(f1, 1.0), fv(f2, 1.0)
        out = []
        for k in range(2):
            lin1 = _linear_interpolate(x, fv(f1, y)[k], fv(f2, y)[k])
            lin2 = _linear_interpolate(y, fv(f3, x)[k], fv(f4, x)[k])
            bil = 0.25 * (c1[k] * (1 - x) * (1 - y) + c2[k] * (1 + x) * (1 - y) +
                          c3[k] * (1 - x) * (1 + y) + c4[k] * (1 + x) * (1 + y))
            out.append(lin1 + lin2 - bil)
        return tuple(out)
    return mapping


def transfinite_mapping_3d(faces):
    """transfinite_mapping(faces) of six face functions (structured_mesh.jl:266-342):
    faces[0..5] at xi = -1, xi = 1, eta = -1, eta = 1, zeta = -1, zeta = 1, each a
    function of the two running coordinates returning (x, y, z)."""
    f = faces

    def fv(fun, s, t):
        r = fun(s, t)
        return [np.asarray(r[q], dtype=float) for q in range(3)]

    def li(s, a, b):
        return [_linear_interpolate(s, a[q], b[q]) for q in range(3)]

    def add(a, b):
        return [a[q] + b[q] for q in range(3)]

    def mapping(x, y, z):
        x, y, z = (np.asarray(v, dtype=float) for v in (x, y, z))
        lin = add(add(li(x, fv(f[0], y, z), fv(f[1], y, z)), li(y, fv(f[2], x, z), fv(f[3], x, z))),
                  li(z, fv(f[4], x, y), fv(f[5], x, y)))
        # correction_term_3d
        c_x = li(x, add(li(y, fv(f[2], -1, z), fv(f[3], -1, z)), li(z, fv(f[4], -1, y), fv(f[5], -1, y))),
                 add(li(y, fv(f[2], 1, z), fv(f[3], 1, z)), li(z, fv(f[4], 1, y), fv(f[5], 1, y))))
        c_y = li(y, add(li(x, fv(f[0], -1, z), fv(f[1], -1, z)), li(z, fv(f[4], x, -1), fv(f[5], x, -1))),
                 add(li(x, fv(f[0], 1, z), fv(f[1], 1, z)), li(z, fv(f[4], x, 1), fv(f[5], x, 1))))
        c_z = li(z, add(li(x, fv(f[0], y, -1), fv(f[1], y, -1)), li(y, fv(f[2], x, -1), fv(f[3], x, -1))),
                 add(li(x, fv(f[0], y, 1), fv(f[1], y, 1)), li(y, fv(f[2], x, 1), fv(f[3], x, 1))))
        corr = [0.5 * (c_x[q] + c_y[q] + c_z[q]) for q in range(3)]
        # trilinear_mapping
        corners = [fv(f[0], -1, -1), fv(f[1], -1, -1), fv(f[0], 1, -1), fv(f[1], 1, -1),
                   fv(f[0], -1, 1), fv(f[1], -1, 1), fv(f[0], 1, 1), fv(f[1], 1, 1)]
        sx, sy, sz = (1 - x, 1 + x), (1 - y, 1 + y), (1 - z, 1 + z)
        tri = [0.125 * (corners[0][q] * sx[0] * sy[0] * sz[0] + corners[1][q] * sx[1] * sy[0] * sz[0] +
                        corners[2][q] * sx[0] * sy[1] * sz[0] + corners[3][q] * sx[1] * sy[1] * sz[0] +
                        corners[4][q] * sx[0] * sy[0] * sz[1] + corners[5][q] * sx[1] * sy[0] * sz[1] +
                        corners[6][q] * sx[0] * sy[1] * sz[1] + corners[7][q] * sx[1] * sy[1] * sz[1])
               for q in range(3)]
        return tuple(lin[q] - corr[q] + tri[q] for q in range(3))
    return mapping


def _eval_mapping3(mapping, xi, eta, zeta):
    r = mapping(xi, eta, zeta)
    return tuple(np.array(np.broadcast_to(np.asarray(r[q], dtype=float), xi.shape)) for q in range(3))


def _eval_mapping(mapping, xi, eta):
    """Evaluates a mapping on arrays of reference coordinates; a mapping that
    only takes scalars is applied point by point."""
    try:
        r = mapping(xi, eta)
        x = np.broadcast_to(np.asarray(r[0], dtype=float), xi.shape)
        y = np.broadcast_to(np.asarray(r[1], dtype=float), xi.shape)
        return np.array(x), np.array(y)
    except (TypeError, ValueError):
        x = np.empty(xi.shape)
        y = np.empty(xi.shape)
        for idx in np.ndindex(xi.shape):
            r = mapping(float(xi[idx]), float(eta[idx]))
            x[idx], y[idx] = float(r[0]), float(r[1])
        return x, y


def _resolve_mapping(mapping, faces, coordinates_min, coordinates_max):
    given = sum(v is not None for v in (mapping, faces, coordinates_min))
    if given != 1 or (coordinates_min is None) != (coordinates_max is None):
        raise ValueError("exactly one of mapping, faces and coordinates_min/max must be given")
    if faces is not None:
        if len(faces) != 4:
            raise ValueError("a 2D mesh takes four faces")
        return transfinite_mapping(faces)
    if coordinates_min is not None:
        return coordinates2mapping(tuple(coordinates_min), tuple(coordinates_max))
    return mapping


def _periodicity(periodicity):
    if isinstance(periodicity, bool):
        return (periodicity, periodicity)
    return tuple(bool(p) for p in periodicity)


class _CurvedBrick2D:
    """A brick of elements on a uniform grid of mx x my cells with a
    mapping; subclasses fix the element order and the node coordinates."""
    ndims = 2
    curved = True

    def _setup_cells(self, cells):
        # cells: [E, 2] global cell index of each element in the fine grid
        self.cells = np.asarray(cells, dtype=np.int64)
        self.nelements = self.cells.shape[0]
        mx, my = self.grid
        c2e = np.empty(mx * my, dtype=np.int64)
        c2e[self.cells[:, 0] + mx * self.cells[:, 1]] = np.arange(self.nelements)
        self._c2e = c2e

    def neighbors(self):
        """[E, 4] (0-based) elements across the -x, +x, -y and +y faces; -1 on a
        face at a non-periodic edge of the brick."""
        mx, my = self.grid
        cx, cy = self.cells[:, 0], self.cells[:, 1]
        out = np.empty((self.nelements, 4), dtype=np.int64)
        out[:, 0] = self._c2e[(cx - 1) % mx + mx * cy]
        out[:, 1] = self._c2e[(cx + 1) % mx + mx * cy]
        out[:, 2] = self._c2e[cx + mx * ((cy - 1) % my)]
        out[:, 3] = self._c2e[cx + mx * ((cy + 1) % my)]
        if not self.periodicity[0]:
            out[cx == 0, 0] = -1
            out[cx == mx - 1, 1] = -1
        if not self.periodicity[1]:
            out[cy == 0, 2] = -1
            out[cy == my - 1, 3] = -1
        return out

    def interfaces(self):
        """neighbor_ids [I, 2] (1-based: element on the negative side, element on
        the positive side) and orientations [I] (1-based), per element in order,
        positive directions only."""
        nb = self.neighbors()
        E = self.nelements
        ids = np.empty((E, 2, 2), dtype=np.int64)
        ori = np.empty((E, 2), dtype=np.int64)
        for d in range(2):
            ids[:, d, 0] = np.arange(E) + 1
            ids[:, d, 1] = nb[:, 2 * d + 1] + 1
            ori[:, d] = d + 1
        keep = (nb[:, 1::2] >= 0).reshape(2 * E)
        return ids.reshape(2 * E, 2)[keep], ori.reshape(2 * E)[keep]

    def mortars(self):
        z = np.zeros((0, 3), dtype=np.int64)
        return z, np.zeros(0, dtype=np.int64), np.zeros(0, dtype=np.int64)

    @property
    def is_uniform(self):
        return True


def metric_terms(X, basis):
    """Jacobian matrix, contravariant vectors Ja^i and inverse Jacobian per node
    (dgsem_structured/containers_2d.jl:61-152) of node coordinates X[E, j, i, 2].
    Returns contravariant [E, j, i, 2 (i), 2 (x, y)] and inverse_jacobian [E, j, i]."""
    Dm = basis.derivative_matrix
    # x_xi, y_xi: derivative along i; x_eta, y_eta: along j
    d_xi = np.einsum("ik,ejkc->ejic", Dm, X)
    d_eta = np.einsum("jk,ekic->ejic", Dm, X)
    Ja = np.empty(X.shape[:3] + (2, 2))
    Ja[..., 0, 0] = d_eta[..., 1]
    Ja[..., 0, 1] = -d_eta[..., 0]
    Ja[..., 1, 0] = -d_xi[..., 1]
    Ja[..., 1, 1] = d_xi[..., 0]
    inv_j = 1.0 / (d_xi[..., 0] * d_eta[..., 1] - d_eta[..., 0] * d_xi[..., 1])
    return Ja, inv_j


def metric_terms_3d(X, basis):
    """Jacobian matrix, contravariant vectors in the invariant curl form and
    inverse Jacobian per node (dgsem_structured/containers_3d.jl:67-286) of node
    coordinates X[E, k, j, i, 3].  Returns contravariant [E, k, j, i, 3 (i), 3
    (x, y, z)] and inverse_jacobian [E, k, j, i]."""
    Dm = basis.derivative_matrix
    # J[..., c, d] = dX_c / dxi_d (d: 0 xi along i, 1 eta along j, 2 zeta along k)
    J = np.empty(X.shape[:4] + (3, 3))
    J[..., 0] = np.einsum("is,ekjsc->ekjic", Dm, X)
    J[..., 1] = np.einsum("js,eksic->ekjic", Dm, X)
    J[..., 2] = np.einsum("ks,esjic->ekjic", Dm, X)
    Ja = np.empty(X.shape[:4] + (3, 3))
    d_xi = lambda G: np.einsum("is,ekjs->ekji", Dm, G)
    d_eta = lambda G: np.einsum("js,eksi->ekji", Dm, G)
    d_zeta = lambda G: np.einsum("ks,esji->ekji", Dm, G)
    for n in range(3):
        m, l = (n + 1) % 3, (n + 2) % 3
        g = [X[..., m] * J[..., l, d] - X[..., l] * J[..., m, d] for d in range(3)]
        Ja[..., 0, n] = 0.5 * d_eta(g[2]) - 0.5 * d_zeta(g[1])
        Ja[..., 1, n] = 0.5 * d_zeta(g[0]) - 0.5 * d_xi(g[2])
        Ja[..., 2, n] = 0.5 * d_xi(g[1]) - 0.5 * d_eta(g[0])
    det = (J[..., 0, 0] * J[..., 1, 1] * J[..., 2, 2] + J[..., 0, 1] * J[..., 1, 2] * J[..., 2, 0] +
           J[..., 0, 2] * J[..., 1, 0] * J[..., 2, 1] - J[..., 0, 2] * J[..., 1, 1] * J[..., 2, 0] -
           J[..., 0, 1] * J[..., 1, 0] * J[..., 2, 2] - J[..., 0, 0] * J[..., 1, 2] * J[..., 2, 1])
    return Ja, 1.0 / det


class StructuredMesh(_CurvedBrick2D):
    """StructuredMesh(cells_per_dimension, mapping | faces | (cmin, cmax); periodicity).
    Three cells_per_dimension give a StructuredMesh3D."""

    def __new__(cls, cells_per_dimension, *args, **kwargs):
        if len(cells_per_dimension) == 3:
            return StructuredMesh3D(cells_per_dimension, *args, **kwargs)
        return super().__new__(cls)

    def __init__(self, cells_per_dimension, mapping=None, coordinates_max=None, *, faces=None,
                 coordinates_min=None, periodicity=True):
        if isinstance(mapping, (tuple, list)) and len(mapping) == 4 and callable(mapping[0]):
            faces, mapping = tuple(mapping), None
        elif isinstance(mapping, (tuple, list)) and coordinates_max is not None:
            coordinates_min, mapping = tuple(mapping), None
        self.mapping = _resolve_mapping(mapping, faces, coordinates_min, coordinates_max)
        nx, ny = (int(c) for c in cells_per_dimension)
        if len(cells_per_dimension) != 2:
            raise NotImplementedError("curvilinear meshes are 2D only")
        self.periodicity = _periodicity(periodicity)
        self.cells_per_dimension = (nx, ny)
        self.grid = (nx, ny)
        cx, cy = np.meshgrid(np.arange(nx), np.arange(ny), indexing="xy")
        self._setup_cells(np.stack([cx.ravel(), cy.ravel()], axis=1))

    def node_coordinates(self, basis):
        """calc_node_coordinates!, dgsem_structured/containers_2d.jl:37-59: [E, j, i, 2]."""
        nx, ny = self.grid
        dx, dy = 2.0 / nx, 2.0 / ny
        nodes = basis.nodes
        ox = -1 + self.cells[:, 0] * dx + dx / 2
        oy = -1 + self.cells[:, 1] * dy + dy / 2
        xi = ox[:, None, None] + (dx / 2 * nodes)[None, None, :]
        eta = oy[:, None, None] + (dy / 2 * nodes)[None, :, None]
        xi, eta = np.broadcast_arrays(xi, eta)
        x, y = _eval_mapping(self.mapping, np.ascontiguousarray(xi), np.ascontiguousarray(eta))
        return np.stack([x, y], axis=-1)

    def __repr__(self):
        return f"StructuredMesh{{2}}({self.grid[0]}x{self.grid[1]} cells)"


class StructuredMesh3D:
    """StructuredMesh with three cells_per_dimension (structured_mesh.jl): the
    mapping of three reference coordinates, six faces (transfinite) or
    coordinates_min/max.  Host setup of the element node coordinates
    (containers_3d.jl:37-65, cells x fastest), neighbours and interfaces.  The
    GPU path runs these in FP64."""
    ndims = 3
    curved = True

    def __init__(self, cells_per_dimension, mapping=None, coordinates_max=None, *, faces=None,
                 coordinates_min=None, periodicity=True):
        if isinstance(mapping, (tuple, list)) and len(mapping) == 6 and callable(mapping[0]):
            faces, mapping = tuple(mapping), None
        elif isinstance(mapping, (tuple, list)) and coordinates_max is not None:
            coordinates_min, mapping = tuple(mapping), None
        if faces is not None:
            self.mapping = transfinite_mapping_3d(faces)
        elif coordinates_min is not None:
            lo, hi = tuple(coordinates_min), tuple(coordinates_max)
            self.mapping = lambda a, b, c: (_linear_interpolate(a, lo[0], hi[0]),
                                            _linear_interpolate(b, lo[1], hi[1]),
                                            _linear_interpolate(c, lo[2], hi[2]))
        else:
            self.mapping = mapping
        self.grid = tuple(int(c) for c in cells_per_dimension)
        self.periodicity = ((periodicity,) * 3 if isinstance(periodicity, bool)
                            else tuple(bool(p) for p in periodicity))
        nx, ny, nz = self.grid
        self.nelements = nx * ny * nz
        e = np.arange(self.nelements)
        self.cells = np.stack([e % nx, (e // nx) % ny, e // (nx * ny)], axis=1)

    def interfaces(self):
        """neighbor_ids [I, 2] (1-based: element on the negative side, element on
        the positive side) and orientations [I] (1..3), per element in order,
        positive directions only."""
        nb = self.neighbors()
        E = self.nelements
        ids = np.empty((E, 3, 2), dtype=np.int64)
        ori = np.empty((E, 3), dtype=np.int64)
        for d in range(3):
            ids[:, d, 0] = np.arange(E) + 1
            ids[:, d, 1] = nb[:, 2 * d + 1] + 1
            ori[:, d] = d + 1
        keep = (nb[:, 1::2] >= 0).reshape(3 * E)
        return ids.reshape(3 * E, 2)[keep], ori.reshape(3 * E)[keep]

    def mortars(self):
        z = np.zeros((0, 5), dtype=np.int64)
        return z, np.zeros(0, dtype=np.int64), np.zeros(0, dtype=np.int64)

    @property
    def is_uniform(self):
        return True

    def neighbors(self):
        """[E, 6] (0-based) across -x, +x, -y, +y, -z, +z; -1 at a non-periodic edge."""
        g = self.grid
        out = np.empty((self.nelements, 6), dtype=np.int64)
        for d in range(3):
            for side, step in ((0, -1), (1, 1)):
                c = self.cells.copy()
                c[:, d] = (c[:, d] + step) % g[d]
                out[:, 2 * d + side] = c[:, 0] + g[0] * (c[:, 1] + g[1] * c[:, 2])
                if not self.periodicity[d]:
                    edge = self.cells[:, d] == (0 if side == 0 else g[d] - 1)
                    out[edge, 2 * d + side] = -1
        return out

    def node_coordinates(self, basis):
        """calc_node_coordinates! (containers_3d.jl:37-65): [E, k, j, i, 3]."""
        g = self.grid
        nodes = basis.nodes
        ref = []
        for d in range(3):
            dx = 2.0 / g[d]
            ref.append(-1 + self.cells[:, d] * dx + dx / 2)
        xi = ref[0][:, None, None, None] + (1.0 / g[0] * nodes)[None, None, None, :]
        eta = ref[1][:, None, None, None] + (1.0 / g[1] * nodes)[None, None, :, None]
        zeta = ref[2][:, None, None, None] + (1.0 / g[2] * nodes)[None, :, None, None]
        xi, eta, zeta = (np.ascontiguousarray(a) for a in np.broadcast_arrays(xi, eta, zeta))
        return np.stack(_eval_mapping3(self.mapping, xi, eta, zeta), axis=-1)

    def __repr__(self):
        return f"StructuredMesh{{3}}({self.grid[0]}x{self.grid[1]}x{self.grid[2]} cells)"


class P4estMesh(_CurvedBrick2D):
    """P4estMesh(trees_per_dimension; polydeg, mapping | faces | coordinates_min/max,
    initial_refinement_level, periodicity) on a brick of trees."""

    def __init__(self, trees_per_dimension, *, polydeg, mapping=None, faces=None,
                 coordinates_min=None, coordinates_max=None, initial_refinement_level=0,
                 periodicity=True):
        if len(trees_per_dimension) != 2:
            raise NotImplementedError("curvilinear meshes are 2D only")
        self.mapping = _resolve_mapping(mapping, faces, coordinates_min, coordinates_max)
        self.periodicity = _periodicity(periodicity)
        tx, ty = (int(t) for t in trees_per_dimension)
        L = int(initial_refinement_level)
        if L < 0 or L > 15:
            raise ValueError("initial_refinement_level must be in 0..15")
        self.trees_per_dimension = (tx, ty)
        self.level = L
        self.polydeg = int(polydeg)
        self.grid = (tx << L, ty << L)
        # calc_tree_node_coordinates!, p4est_mesh.jl:1618-1644: [tree, j, i, 2]
        self.nodes, _ = gauss_lobatto_nodes_weights(self.polydeg + 1)
        dx, dy = 2.0 / tx, 2.0 / ty
        gx, gy = np.meshgrid(np.arange(tx), np.arange(ty), indexing="xy")
        gx, gy = gx.ravel(), gy.ravel()
        xi = (-1 + gx * dx + dx / 2)[:, None, None] + (dx / 2 * self.nodes)[None, None, :]
        eta = (-1 + gy * dy + dy / 2)[:, None, None] + (dy / 2 * self.nodes)[None, :, None]
        xi, eta = np.broadcast_arrays(xi, eta)
        x, y = _eval_mapping(self.mapping, np.ascontiguousarray(xi), np.ascontiguousarray(eta))
        self.tree_node_coordinates = np.stack([x, y], axis=-1)
        # quadrants of each tree in Morton order (x the lowest bit)
        q = np.arange(1 << (2 * L), dtype=np.int64)
        qx = np.zeros_like(q)
        qy = np.zeros_like(q)
        for bit in range(L):
            qx |= ((q >> (2 * bit)) & 1) << bit
            qy |= ((q >> (2 * bit + 1)) & 1) << bit
        self._quad = np.stack([qx, qy], axis=1)
        tree = np.repeat(np.arange(tx * ty), 1 << (2 * L))
        quad = np.tile(self._quad, (tx * ty, 1))
        self._tree = tree
        cells = np.stack([(gx[tree] << L) + quad[:, 0], (gy[tree] << L) + quad[:, 1]], axis=1)
        self._setup_cells(cells)

    def node_coordinates(self, basis):
        """calc_node_coordinates!, dgsem_p4est/containers_2d.jl:29-89: the tree
        nodes interpolated to each quadrant's solver nodes, [E, j, i, 2]."""
        if basis.nnodes() < len(self.nodes):
            raise ValueError("The solver can't have a lower polydeg than the mesh")
        L = self.level
        ql = 2.0 ** -L
        out = np.empty((self.nelements, basis.nnodes(), basis.nnodes(), 2))
        mats = {}
        for k in range(1 << L):
            pts = 2 * (ql * 0.5 * (basis.nodes + 1) + k * ql) - 1
            mats[k] = polynomial_interpolation_matrix(self.nodes, pts)
        per_tree = 1 << (2 * L)
        ntrees = self.nelements // per_tree
        view = out.reshape((ntrees, per_tree) + out.shape[1:])
        T = self.tree_node_coordinates
        for q in range(per_tree):
            m1 = mats[int(self._quad[q, 0])]
            m2 = mats[int(self._quad[q, 1])]
            view[:, q] = np.einsum("ia,jb,tbac->tjic", m1, m2, T, optimize=True)
        return out

    def __repr__(self):
        tx, ty = self.trees_per_dimension
        return f"P4estMesh{{2}}({tx}x{ty} trees, level {self.level})"
