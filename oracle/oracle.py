"""ctypes wrapper of the CPU FP64 oracle (oracle/trixi_oracle.cpp).

TEST INFRASTRUCTURE ONLY.  The oracle restates Trixi.jl's DGSEM TreeMesh
Euler path on the CPU; only the test suite, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` may load it, and only as the checker or the
timed CPU reference -- never as part of the product path.

All arrays use Trixi's column-major layouts, exposed here as C-ordered numpy
arrays with the axes reversed: ``u[element, (k), j, i, v]``.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")

# enums mirrored from trixi_oracle.cpp
VI_WEAK, VI_FLUXDIFF, VI_SHOCKCAPTURING_HG = 0, 1, 2
(FLUX_CENTRAL, FLUX_RANOCHA, FLUX_SHIMA_ETAL, FLUX_LAX_FRIEDRICHS, FLUX_LAX_FRIEDRICHS_NAIVE,
 FLUX_HLLC, FLUX_CHANDRASHEKAR, FLUX_HLLE) = range(8)
SRC_NONE, SRC_CONVERGENCE_TEST = 0, 1
BC_PERIODIC, BC_DIRICHLET, BC_SLIP_WALL = 0, 1, 2
(IC_CONSTANT, IC_CONVERGENCE_TEST, IC_ISENTROPIC_VORTEX, IC_WEAK_BLAST_WAVE,
 IC_KELVIN_HELMHOLTZ, IC_TAYLOR_GREEN, IC_GAUSSIAN_BLAST,
 IC_ISENTROPIC_VORTEX_ADVECTED, IC_BLAST_WAVE, IC_DENSITY_PULSE, IC_SEDOV_BLAST_WAVE,
 IC_DENSITY_WAVE, IC_MEDIUM_SEDOV_3D) = range(13)

_lib = None
_PORTABLE_FLAGS = "g++ -O3 -fopenmp (portable)"


def select_build(kind: str = "portable") -> str:
    """Chooses which build of the oracle the next load uses and returns its
    compile flags: "portable" (the parity checker) or "native" (tuned for the
    host CPU by oracle/build.sh; used only for timing the CPU baseline).  Has
    no effect once a build is loaded."""
    global _LIB_PATH
    native = os.path.join(_HERE, "_build", "liboracle_native.so")
    if _lib is None and kind == "native" and os.path.exists(native):
        _LIB_PATH = native
    if _LIB_PATH == native:
        try:
            with open(os.path.join(_HERE, "_build", "liboracle_native.flags")) as f:
                return f.read().strip()
        except OSError:
            return "native"
    return _PORTABLE_FLAGS


def build() -> str:
    """Compile the oracle with its own recipe (oracle/build.sh)."""
    subprocess.run(["sh", os.path.join(_HERE, "build.sh")], check=True)
    return _LIB_PATH


def _load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_LIB_PATH):
        build()
    lib = ctypes.CDLL(_LIB_PATH)
    d, i, i64, vp = ctypes.c_double, ctypes.c_int, ctypes.c_int64, ctypes.c_void_p
    P = ctypes.POINTER
    lib.orc_create.restype = vp
    lib.orc_create.argtypes = [i, i, i, P(d), P(d), d, i, i, i, i, d, d, i, i]
    lib.orc_destroy.argtypes = [vp]
    lib.orc_set_threads.argtypes = [i]
    lib.orc_max_threads.restype = i
    for name in ("orc_nelements", "orc_ninterfaces", "orc_ndofs"):
        getattr(lib, name).restype = i64
        getattr(lib, name).argtypes = [vp]
    lib.orc_nnodes.restype = i
    lib.orc_nnodes.argtypes = [vp]
    lib.orc_get_basis.argtypes = [vp] + [P(d)] * 7
    lib.orc_get_mesh.argtypes = [vp, P(i64), P(i64), P(d), P(d)]
    lib.orc_initial_condition.argtypes = [vp, i, P(d), d, P(d)]
    lib.orc_rhs.argtypes = [vp, P(d), P(d), d]
    lib.orc_alpha.argtypes = [vp, P(d), P(d)]
    lib.orc_max_dt.restype = d
    lib.orc_max_dt.argtypes = [vp, P(d)]
    lib.orc_rk_stage.argtypes = [vp, P(d), P(d), P(d), i, d, d]
    lib.orc_solve.restype = i
    lib.orc_solve.argtypes = [vp, P(d), d, d, d, i64, P(d), P(i64)]
    lib.orc_error_norms.argtypes = [vp, P(d), d, i, P(d), P(d), P(d)]
    lib.orc_integrals.argtypes = [vp, P(d), P(d)]
    lib.orc_entropy_timederivative.restype = d
    lib.orc_entropy_timederivative.argtypes = [vp, P(d), d]
    lib.orc_set_boundaries.restype = i
    lib.orc_set_boundaries.argtypes = [vp, P(i), i, P(d)]
    lib.orc_set_refinement.restype = i
    lib.orc_set_refinement.argtypes = [vp, i, P(i), P(d)]
    lib.orc_nmortars.restype = i64
    lib.orc_nmortars.argtypes = [vp]
    lib.orc_get_mortars.argtypes = [vp, P(i64), P(i64), P(i64)]
    lib.orc_get_mortar_matrices.argtypes = [vp, P(d)]
    lib.orc_set_amr.argtypes = [vp, P(i), P(d)]
    lib.orc_adapt.restype = i
    lib.orc_adapt.argtypes = [vp, P(d), i, i]
    lib.orc_get_state.argtypes = [vp, P(d)]
    lib.orc_adapt_with.restype = i
    lib.orc_adapt_with.argtypes = [vp, P(d), P(i), i, i]
    lib.orc_amr_lambda.argtypes = [vp, P(d), P(i)]
    lib.orc_element_levels.argtypes = [vp, P(i)]
    lib.orc_solve_amr.restype = i
    lib.orc_solve_amr.argtypes = [vp, i, P(d), d, d, d, i64, P(d), P(i64)]
    lib.orc_curved_create.restype = vp
    lib.orc_curved_create.argtypes = [i, i64, P(d), P(i64), d, i, i, i, i]
    lib.orc_curved_destroy.argtypes = [vp]
    lib.orc_curved_set_dirichlet.argtypes = [vp, i, P(d)]
    lib.orc_curved_set_hg.argtypes = [vp, d, d, i, i]
    lib.orc_curved_alpha.argtypes = [vp, P(d), P(d)]
    lib.orc_curved_metric.argtypes = [vp, P(d), P(d)]
    lib.orc_curved_initial_condition.argtypes = [vp, i, P(d), d, P(d)]
    lib.orc_curved_rhs.argtypes = [vp, P(d), P(d), d]
    lib.orc_curved_max_dt.restype = d
    lib.orc_curved_max_dt.argtypes = [vp, P(d)]
    lib.orc_curved_solve.restype = i
    lib.orc_curved_solve.argtypes = [vp, P(d), d, d, d, i64, P(d), P(i64)]
    lib.orc_curved_errors.argtypes = [vp, P(d), d, i, P(d), P(d), P(d)]
    lib.orc_curved3_set_hg.argtypes = [vp, d, d, i, i]
    lib.orc_curved3_alpha.argtypes = [vp, P(d), P(d)]
    lib.orc_curved3_create.restype = vp
    lib.orc_curved3_create.argtypes = [i, i64, P(d), P(i64), d, i, i, i, i]
    lib.orc_curved3_destroy.argtypes = [vp]
    lib.orc_curved3_set_dirichlet.argtypes = [vp, i, P(d)]
    lib.orc_curved3_metric.argtypes = [vp, P(d), P(d)]
    lib.orc_curved3_initial_condition.argtypes = [vp, i, P(d), d, P(d)]
    lib.orc_curved3_rhs.argtypes = [vp, P(d), P(d), d]
    lib.orc_curved3_max_dt.restype = d
    lib.orc_curved3_max_dt.argtypes = [vp, P(d)]
    lib.orc_curved3_solve.restype = i
    lib.orc_curved3_solve.argtypes = [vp, P(d), d, d, d, i64, P(d), P(i64)]
    lib.orc_curved3_errors.argtypes = [vp, P(d), d, i, P(d), P(d), P(d)]
    _lib = lib
    return lib


def _p(a, ctype=ctypes.c_double):
    return a.ctypes.data_as(ctypes.POINTER(ctype))


class Oracle:
    """One semidiscretization of the oracle (mesh + basis + solver options)."""

    def __init__(self, ndims, polydeg, level, xmin, xmax, gamma=1.4,
                 volume_integral=VI_WEAK, volume_flux=FLUX_CENTRAL,
                 surface_flux=FLUX_LAX_FRIEDRICHS, fv_flux=None,
                 alpha_max=0.5, alpha_min=0.001, alpha_smooth=True,
                 source=SRC_NONE):
        lib = _load()
        self.lib = lib
        self.ndims, self.polydeg, self.n = ndims, polydeg, polydeg + 1
        self.nvar = ndims + 2
        xmin = np.ascontiguousarray(xmin, dtype=np.float64)
        xmax = np.ascontiguousarray(xmax, dtype=np.float64)
        if fv_flux is None:
            fv_flux = surface_flux
        h = lib.orc_create(ndims, polydeg, level, _p(xmin), _p(xmax), gamma,
                           volume_integral, volume_flux, surface_flux, fv_flux,
                           alpha_max, alpha_min, int(alpha_smooth), source)
        if not h:
            raise ValueError("oracle: unsupported configuration")
        self.h = h
        self.nelements = lib.orc_nelements(h)
        self.ninterfaces = lib.orc_ninterfaces(h)
        self.ndofs = lib.orc_ndofs(h)

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.orc_destroy(self.h)
            self.h = None

    @property
    def shape(self):
        return (self.nelements,) + (self.n,) * self.ndims + (self.nvar,)

    def basis(self):
        n = self.n
        vecs = [np.zeros(n) for _ in range(3)]
        mats = [np.zeros((n, n)) for _ in range(4)]  # column-major buffers
        self.lib.orc_get_basis(self.h, *[_p(v) for v in vecs], *[_p(m) for m in mats])
        names = ["nodes", "weights", "inverse_weights"]
        out = dict(zip(names, vecs))
        # buffers were written column-major: reinterpret as (n, n) Fortran arrays
        for name, m in zip(["derivative_matrix", "derivative_hat", "derivative_split",
                            "inverse_vandermonde_legendre"], mats):
            out[name] = m.reshape(-1).reshape((n, n), order="F").copy()
        return out

    def mesh(self):
        I, E = self.ninterfaces, self.nelements
        nb = np.zeros((I, 2), dtype=np.int64)
        orient = np.zeros(I, dtype=np.int64)
        invj = np.zeros(E)
        coords = np.zeros((E,) + (self.n,) * self.ndims + (self.ndims,))
        self.lib.orc_get_mesh(self.h, _p(nb, ctypes.c_int64), _p(orient, ctypes.c_int64),
                              _p(invj), _p(coords))
        return dict(neighbor_ids=nb, orientations=orient, inverse_jacobian=invj,
                    node_coordinates=coords)

    def initial_condition(self, ic, params=None, t=0.0):
        u = np.zeros(self.shape)
        par = None if params is None else np.ascontiguousarray(params, dtype=np.float64)
        self.lib.orc_initial_condition(self.h, ic, None if par is None else _p(par), t, _p(u))
        return u

    def rhs(self, u, t=0.0):
        u = np.ascontiguousarray(u, dtype=np.float64)
        du = np.zeros_like(u)
        self.lib.orc_rhs(self.h, _p(du), _p(u), t)
        return du

    def alpha(self, u):
        u = np.ascontiguousarray(u, dtype=np.float64)
        a = np.zeros(self.nelements)
        self.lib.orc_alpha(self.h, _p(u), _p(a))
        return a

    def max_dt(self, u):
        u = np.ascontiguousarray(u, dtype=np.float64)
        return self.lib.orc_max_dt(self.h, _p(u))

    def rk_stage(self, u, u_tmp, stage, t, dt):
        """In place: du = rhs(u, t + c_s dt); u_tmp = du - a_s u_tmp; u += b_s dt u_tmp."""
        du = np.zeros_like(u)
        self.lib.orc_rk_stage(self.h, _p(u), _p(u_tmp), _p(du), stage, t, dt)
        return du

    def solve(self, u, t0, t_end, cfl, max_steps=10**9):
        u = np.ascontiguousarray(u, dtype=np.float64).copy()
        t_out = ctypes.c_double(0)
        nsteps = ctypes.c_int64(0)
        rc = self.lib.orc_solve(self.h, _p(u), t0, t_end, cfl, max_steps,
                                ctypes.byref(t_out), ctypes.byref(nsteps))
        if rc != 0:
            raise FloatingPointError("oracle: time step size is NaN")
        return u, t_out.value, nsteps.value

    def error_norms(self, u, t, ic, params=None):
        u = np.ascontiguousarray(u, dtype=np.float64)
        l2 = np.zeros(self.nvar)
        linf = np.zeros(self.nvar)
        par = None if params is None else np.ascontiguousarray(params, dtype=np.float64)
        self.lib.orc_error_norms(self.h, _p(u), t, ic, None if par is None else _p(par),
                                 _p(l2), _p(linf))
        return l2, linf

    def integrals(self, u):
        """Domain totals of each conserved variable, then entropy, then kinetic energy."""
        u = np.ascontiguousarray(u, dtype=np.float64)
        out = np.zeros(self.nvar + 2)
        self.lib.orc_integrals(self.h, _p(u), _p(out))
        return out


def _entropy_timederivative(self, u, t=0.0):
    """Normalised integral of cons2entropy(u) . rhs(u, t) (analysis_dg2d.jl:460-472)."""
    u = np.ascontiguousarray(u, dtype=np.float64)
    return self.lib.orc_entropy_timederivative(self.h, _p(u), t)


Oracle.entropy_timederivative = _entropy_timederivative


def _set_boundaries(self, bc, ic=0, params=None):
    """periodicity = false: boundary condition per direction (-x, +x, -y, ...),
    BC_DIRICHLET with the values of initial condition `ic`, or BC_SLIP_WALL."""
    codes = np.ascontiguousarray(bc, dtype=np.int32)
    assert codes.size == 2 * self.ndims
    par = np.zeros(8)
    if params is not None:
        par[:len(params)] = params
    if self.lib.orc_set_boundaries(self.h, _p(codes, ctypes.c_int), int(ic), _p(par)) != 0:
        raise ValueError("oracle: invalid boundary condition")
    self.ninterfaces = self.lib.orc_ninterfaces(self.h)


Oracle.set_boundaries = _set_boundaries


def _set_refinement(self, patches):
    """Refinement patches after the initial refinement (TreeMesh
    refinement_patches): dicts with type "box" (coordinates_min,
    coordinates_max) or "sphere" (center, radius)."""
    kinds = np.zeros(max(1, len(patches)), dtype=np.int32)
    par = np.zeros(7 * max(1, len(patches)))
    for k, p in enumerate(patches):
        if p["type"] == "box":
            kinds[k] = 0
            par[7 * k:7 * k + self.ndims] = p["coordinates_min"]
            par[7 * k + 3:7 * k + 3 + self.ndims] = p["coordinates_max"]
        elif p["type"] == "sphere":
            kinds[k] = 1
            par[7 * k:7 * k + self.ndims] = p["center"]
            par[7 * k + 6] = p["radius"]
        else:
            raise ValueError(f"unknown refinement patch type {p['type']!r}")
    if self.lib.orc_set_refinement(self.h, len(patches), _p(kinds, ctypes.c_int), _p(par)) != 0:
        raise ValueError("oracle: invalid refinement patch")
    self.nelements = self.lib.orc_nelements(self.h)
    self.ninterfaces = self.lib.orc_ninterfaces(self.h)
    self.nmortars = self.lib.orc_nmortars(self.h)
    self.ndofs = self.lib.orc_ndofs(self.h)


def _mortars(self):
    """cache.mortars: neighbor_ids [M, 2^(ndims-1) + 1] (1-based, large last),
    large_sides [M] (1 or 2), orientations [M] (1-based)."""
    M = self.lib.orc_nmortars(self.h)
    ids = np.zeros((M, (1 << (self.ndims - 1)) + 1), dtype=np.int64)
    ls = np.zeros(M, dtype=np.int64)
    orient = np.zeros(M, dtype=np.int64)
    if M:
        self.lib.orc_get_mortars(self.h, _p(ids, ctypes.c_int64), _p(ls, ctypes.c_int64),
                                 _p(orient, ctypes.c_int64))
    return ids, ls, orient


def _mortar_matrices(self):
    """forward_upper, forward_lower, reverse_upper, reverse_lower as (n, n) arrays."""
    n = self.n
    out = np.zeros(4 * n * n)
    self.lib.orc_get_mortar_matrices(self.h, _p(out))
    return [out[k * n * n:(k + 1) * n * n].reshape(n, n).copy() for k in range(4)]


def _refresh(self):
    self.nelements = self.lib.orc_nelements(self.h)
    self.ninterfaces = self.lib.orc_ninterfaces(self.h)
    self.nmortars = self.lib.orc_nmortars(self.h)
    self.ndofs = self.lib.orc_ndofs(self.h)


def _set_amr(self, interval=5, adapt_initial_condition=True,
             adapt_initial_condition_only_refine=True, alpha_max=0.5, alpha_min=0.001,
             alpha_smooth=True, base_level=1, med_level=None, med_threshold=0.0,
             max_level=None, max_threshold=1.0, variable="density_pressure",
             indicator="hennemann_gassner"):
    """AMRCallback(semi, ControllerThreeLevel(semi, IndicatorHennemannGassner(...)))."""
    med_level = base_level if med_level is None else med_level
    max_level = base_level if max_level is None else max_level
    ints = np.array([interval, adapt_initial_condition, adapt_initial_condition_only_refine,
                     alpha_smooth, base_level, med_level, max_level,
                     {"density_pressure": 0, "density": 1}[variable],
                     {"hennemann_gassner": 0, "max": 1}[indicator]], dtype=np.int32)
    dbls = np.array([alpha_max, alpha_min, med_threshold, max_threshold], dtype=np.float64)
    self.lib.orc_set_amr(self.h, _p(ints, ctypes.c_int), _p(dbls))


def _adapt(self, u, only_refine=False, only_coarsen=False):
    """One AMR pass; returns (changed, new state)."""
    u = np.ascontiguousarray(u, dtype=np.float64)
    changed = bool(self.lib.orc_adapt(self.h, _p(u), int(only_refine), int(only_coarsen)))
    self.refresh()
    out = np.zeros(self.shape)
    self.lib.orc_get_state(self.h, _p(out))
    return changed, out


def _adapt_with(self, u, controller_value, only_refine=False, only_coarsen=False):
    """One AMR pass with given controller values; returns (changed, new state)."""
    u = np.ascontiguousarray(u, dtype=np.float64)
    lam = np.ascontiguousarray(controller_value, dtype=np.int32)
    changed = bool(self.lib.orc_adapt_with(self.h, _p(u), _p(lam, ctypes.c_int),
                                           int(only_refine), int(only_coarsen)))
    self.refresh()
    out = np.zeros(self.shape)
    self.lib.orc_get_state(self.h, _p(out))
    return changed, out


def _amr_lambda(self, u):
    u = np.ascontiguousarray(u, dtype=np.float64)
    out = np.zeros(self.nelements, dtype=np.int32)
    self.lib.orc_amr_lambda(self.h, _p(u), _p(out, ctypes.c_int))
    return out


Oracle.adapt_with = _adapt_with
Oracle.amr_lambda = _amr_lambda


def _element_levels(self):
    out = np.zeros(self.nelements, dtype=np.int32)
    self.lib.orc_element_levels(self.h, _p(out, ctypes.c_int))
    return out


def _solve_amr(self, ic, params, t0, t_end, cfl, max_steps=10**9):
    par = None if params is None else np.ascontiguousarray(params, dtype=np.float64)
    t_out = ctypes.c_double(0)
    nsteps = ctypes.c_int64(0)
    rc = self.lib.orc_solve_amr(self.h, ic, None if par is None else _p(par), t0, t_end, cfl,
                                max_steps, ctypes.byref(t_out), ctypes.byref(nsteps))
    self.refresh()
    if rc != 0:
        raise FloatingPointError("oracle: time step size is NaN")
    out = np.zeros(self.shape)
    self.lib.orc_get_state(self.h, _p(out))
    return out, t_out.value, nsteps.value


Oracle.refresh = _refresh
Oracle.set_amr = _set_amr
Oracle.adapt = _adapt
Oracle.element_levels = _element_levels
Oracle.solve_amr = _solve_amr
Oracle.set_refinement = _set_refinement
Oracle.mortars = _mortars
Oracle.mortar_matrices = _mortar_matrices


def set_threads(n: int) -> None:
    _load().orc_set_threads(int(n))


def max_threads() -> int:
    return _load().orc_max_threads()


class CurvedOracle:
    """CPU restatement of DGSEM on a curvilinear 2D mesh (StructuredMesh / P4estMesh
    brick): element node coordinates x[E, n, n, 2] (i fastest) and neighbours
    nbr[E, 4] (0-based, -x, +x, -y, +y).  State layout [E, n, n, 4]."""

    def __init__(self, polydeg, x, nbr, gamma=1.4, volume_integral=VI_WEAK,
                 volume_flux=FLUX_CENTRAL, surface_flux=FLUX_LAX_FRIEDRICHS, source=SRC_NONE):
        lib = _load()
        self.x = np.ascontiguousarray(x, dtype=np.float64)
        self.nbr = np.ascontiguousarray(nbr, dtype=np.int64)
        self.n = polydeg + 1
        self.E = self.x.shape[0]
        self.h = lib.orc_curved_create(polydeg, self.E, _p(self.x), _p(self.nbr, ctypes.c_int64),
                                       gamma, volume_integral, volume_flux, surface_flux, source)

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_curved_destroy(self.h)
            self.h = None

    @property
    def shape(self):
        return (self.E, self.n, self.n, 4)

    def set_hg(self, alpha_max, alpha_min, alpha_smooth, fv_flux):
        """IndicatorHennemannGassner(density_pressure) parameters and the FV flux of
        a VI_SHOCKCAPTURING_HG solver."""
        _lib.orc_curved_set_hg(self.h, alpha_max, alpha_min, int(alpha_smooth), fv_flux)

    def alpha(self, u):
        """Smoothed blending factors of state u (after set_hg)."""
        a = np.empty(self.E)
        _lib.orc_curved_alpha(self.h, _p(np.ascontiguousarray(u, dtype=np.float64)), _p(a))
        return a

    def set_dirichlet(self, ic, params=None):
        """BoundaryConditionDirichlet(initial condition ic) on every face without a
        neighbour (nbr < 0)."""
        par = np.zeros(8)
        if params is not None:
            par[:len(params)] = params
        _lib.orc_curved_set_dirichlet(self.h, ic, _p(par))

    def metric(self):
        Ja = np.empty((self.E, self.n, self.n, 2, 2))
        ij = np.empty((self.E, self.n, self.n))
        _lib.orc_curved_metric(self.h, _p(Ja), _p(ij))
        return Ja, ij

    def initial_condition(self, ic, t=0.0, params=None):
        u = np.empty(self.shape)
        par = np.ascontiguousarray(params if params is not None else np.zeros(8), dtype=np.float64)
        _lib.orc_curved_initial_condition(self.h, ic, _p(par), t, _p(u))
        return u

    def rhs(self, u, t=0.0):
        u = np.ascontiguousarray(u, dtype=np.float64)
        du = np.empty_like(u)
        _lib.orc_curved_rhs(self.h, _p(du), _p(u), t)
        return du

    def max_dt(self, u):
        return _lib.orc_curved_max_dt(self.h, _p(np.ascontiguousarray(u, dtype=np.float64)))

    def solve(self, u, t0, t_end, cfl, max_steps=2 ** 62):
        u = np.array(u, dtype=np.float64, copy=True)
        t = ctypes.c_double()
        k = ctypes.c_int64()
        rc = _lib.orc_curved_solve(self.h, _p(u), t0, t_end, cfl, max_steps, ctypes.byref(t),
                                   ctypes.byref(k))
        if rc != 0:
            raise FloatingPointError("NaN time step")
        return u, t.value, k.value

    def error_norms(self, u, t, ic, params=None):
        l2 = np.empty(4)
        linf = np.empty(4)
        par = np.ascontiguousarray(params if params is not None else np.zeros(8), dtype=np.float64)
        _lib.orc_curved_errors(self.h, _p(np.ascontiguousarray(u, dtype=np.float64)), t, ic,
                               _p(par), _p(l2), _p(linf))
        return l2, linf


class CurvedOracle3D:
    """CPU restatement of DGSEM on a curvilinear 3D StructuredMesh: element node
    coordinates x[E, n, n, n, 3] (i fastest) and neighbours nbr[E, 6] (0-based,
    -x, +x, -y, +y, -z, +z; -1 on a Dirichlet face).  State layout [E, n, n, n, 5]."""

    def __init__(self, polydeg, x, nbr, gamma=1.4, volume_integral=VI_WEAK,
                 volume_flux=FLUX_CENTRAL, surface_flux=FLUX_LAX_FRIEDRICHS, source=SRC_NONE):
        lib = _load()
        self.x = np.ascontiguousarray(x, dtype=np.float64)
        self.nbr = np.ascontiguousarray(nbr, dtype=np.int64)
        self.n = polydeg + 1
        self.E = self.x.shape[0]
        self.h = lib.orc_curved3_create(polydeg, self.E, _p(self.x),
                                        _p(self.nbr, ctypes.c_int64), gamma, volume_integral,
                                        volume_flux, surface_flux, source)

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_curved3_destroy(self.h)
            self.h = None

    @property
    def shape(self):
        return (self.E, self.n, self.n, self.n, 5)

    def set_hg(self, alpha_max, alpha_min, alpha_smooth, fv_flux):
        """IndicatorHennemannGassner(density_pressure) parameters and the FV flux of
        a VI_SHOCKCAPTURING_HG solver."""
        _lib.orc_curved3_set_hg(self.h, alpha_max, alpha_min, int(alpha_smooth), fv_flux)

    def alpha(self, u):
        """Smoothed blending factors of state u (after set_hg)."""
        a = np.empty(self.E)
        _lib.orc_curved3_alpha(self.h, _p(np.ascontiguousarray(u, dtype=np.float64)), _p(a))
        return a

    def set_dirichlet(self, ic, params=None):
        par = np.zeros(8)
        if params is not None:
            par[:len(params)] = params
        _lib.orc_curved3_set_dirichlet(self.h, ic, _p(par))

    def metric(self):
        Ja = np.empty((self.E, self.n, self.n, self.n, 3, 3))
        ij = np.empty((self.E, self.n, self.n, self.n))
        _lib.orc_curved3_metric(self.h, _p(Ja), _p(ij))
        return Ja, ij

    def initial_condition(self, ic, t=0.0, params=None):
        u = np.empty(self.shape)
        par = np.ascontiguousarray(params if params is not None else np.zeros(8), dtype=np.float64)
        _lib.orc_curved3_initial_condition(self.h, ic, _p(par), t, _p(u))
        return u

    def rhs(self, u, t=0.0):
        u = np.ascontiguousarray(u, dtype=np.float64)
        du = np.empty_like(u)
        _lib.orc_curved3_rhs(self.h, _p(du), _p(u), t)
        return du

    def max_dt(self, u):
        return _lib.orc_curved3_max_dt(self.h, _p(np.ascontiguousarray(u, dtype=np.float64)))

    def solve(self, u, t0, t_end, cfl, max_steps=2 ** 62):
        u = np.array(u, dtype=np.float64, copy=True)
        t = ctypes.c_double()
        k = ctypes.c_int64()
        rc = _lib.orc_curved3_solve(self.h, _p(u), t0, t_end, cfl, max_steps, ctypes.byref(t),
                                    ctypes.byref(k))
        if rc != 0:
            raise FloatingPointError("NaN time step")
        return u, t.value, k.value

    def error_norms(self, u, t, ic, params=None):
        l2 = np.empty(5)
        linf = np.empty(5)
        par = np.ascontiguousarray(params if params is not None else np.zeros(8), dtype=np.float64)
        _lib.orc_curved3_errors(self.h, _p(np.ascontiguousarray(u, dtype=np.float64)), t, ic,
                                _p(par), _p(l2), _p(linf))
        return l2, linf
