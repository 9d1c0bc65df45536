"""SemidiscretizationHyperbolic on the GB300 path.

Host-side mirror of src/semidiscretization/semidiscretization_hyperbolic.jl
and src/semidiscretization/semidiscretization.jl: the semidiscretization
builds the TreeMesh containers (elements, interfaces) on the host, hands them
with the basis to the C ABI (tg_ctx_create) and exposes rhs! / compute
coefficients / time stepping through the device context.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .equations import CompressibleEulerEquations2D
from .mesh import TreeMesh
from .solvers import DGSEM, VolumeIntegralShockCapturingHG


class BoundaryConditionPeriodic:
    code = _lib.TG_BOUNDARY_PERIODIC

    def __repr__(self):
        return "boundary_condition_periodic"


boundary_condition_periodic = BoundaryConditionPeriodic()


class BoundaryConditionDirichlet:
    """BoundaryConditionDirichlet(boundary_value_function), equations.jl:159-182: the
    values of an initial condition at the boundary node and time.  On the GPU
    path the function is one of the package's initial conditions."""
    code = _lib.TG_BOUNDARY_DIRICHLET

    def __init__(self, boundary_value_function):
        self.boundary_value_function = boundary_value_function

    def __repr__(self):
        return f"BoundaryConditionDirichlet({getattr(self.boundary_value_function, '__name__', '?')})"


class BoundaryConditionSlipWall:
    code = _lib.TG_BOUNDARY_SLIP_WALL

    def __repr__(self):
        return "boundary_condition_slip_wall"


# compressible_euler_2d.jl:322-393, 3d.jl:315-416
boundary_condition_slip_wall = BoundaryConditionSlipWall()

# initial conditions the device can evaluate for Dirichlet boundaries
_IC_CODES = {"initial_condition_constant": 0, "initial_condition_convergence_test": 1,
             "initial_condition_isentropic_vortex": 2, "initial_condition_weak_blast_wave": 3,
             "initial_condition_kelvin_helmholtz_instability": 4,
             "initial_condition_taylor_green_vortex": 5, "initial_condition_gaussian_blast": 6}


def _digest_boundary_conditions(bcs, mesh):
    """One boundary condition per direction (-x, +x, -y, +y[, -z, +z]) from a single
    condition, a tuple of 2D conditions or a dict with keys x_neg, x_pos, ...
    (digest_boundary_conditions, semidiscretization_hyperbolic.jl)."""
    D = mesh.ndims
    names = ["x_neg", "x_pos", "y_neg", "y_pos", "z_neg", "z_pos"][:2 * D]
    if isinstance(bcs, dict):
        per_dir = [bcs[k] for k in names]
    elif isinstance(bcs, (tuple, list)):
        if len(bcs) != 2 * D:
            raise ValueError(f"need {2 * D} boundary conditions")
        per_dir = list(bcs)
    else:
        per_dir = [bcs] * (2 * D)
    for k, bc in enumerate(per_dir):
        periodic_dir = mesh.periodicity[k // 2]
        if periodic_dir != isinstance(bc, BoundaryConditionPeriodic):
            raise ValueError(f"boundary condition {bc!r} of direction {names[k]} does not match "
                             f"the mesh periodicity {mesh.periodicity}")
    return per_dir


def _dptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ptr_of(x):
    """Address of a device or host buffer: torch tensor, numpy array or int."""
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        return x.data_ptr()
    if isinstance(x, np.ndarray):
        return x.ctypes.data
    raise TypeError(f"cannot take the address of {type(x)}")


def make_config(semi, precision="fp64", device=0, elements_per_block=0):
    """tg_config of a semidiscretization, and the arrays it points into (they
    must stay alive while the config is in use)."""
    dg, eq = semi.solver, semi.equations
    vi = dg.volume_integral
    b = dg.basis
    # keep every array alive while the config points at it
    keep = []

    def arr(a, dtype=np.float64):
        a = np.ascontiguousarray(a, dtype=dtype)
        keep.append(a)
        return a

    nb, orient = semi.neighbor_ids, semi.orientations
    cfg = _lib.tg_config()
    cfg.ndims = eq.ndims
    cfg.polydeg = b.polydeg
    cfg.nelements = semi.nelements
    cfg.ninterfaces = nb.shape[0]
    cfg.gamma = eq.gamma
    cfg.volume_integral = vi.code
    if isinstance(vi, VolumeIntegralShockCapturingHG):
        ind = vi.indicator
        cfg.volume_flux = vi.volume_flux_dg.code
        cfg.volume_flux_fv = vi.volume_flux_fv.code
        cfg.alpha_max, cfg.alpha_min = ind.alpha_max, ind.alpha_min
        cfg.alpha_smooth = int(ind.alpha_smooth)
    else:
        cfg.volume_flux = getattr(vi, "volume_flux", None).code if hasattr(vi, "volume_flux") else 0
        cfg.volume_flux_fv = dg.surface_flux.code
    cfg.surface_flux = dg.surface_flux.code
    cfg.source_terms = semi.source_terms.code if semi.source_terms is not None else 0
    cfg.precision = {"fp64": _lib.TG_PRECISION_FP64, "mixed": _lib.TG_PRECISION_MIXED}[precision]
    cfg.device = device
    # Julia column-major matrices: pass the transpose's C buffer
    cfg.nodes = _dptr(arr(b.nodes))
    cfg.weights = _dptr(arr(b.weights))
    cfg.inverse_weights = _dptr(arr(b.inverse_weights))
    cfg.derivative_hat = _dptr(arr(np.asfortranarray(b.derivative_hat).ravel(order="F")))
    cfg.derivative_split = _dptr(arr(np.asfortranarray(b.derivative_split).ravel(order="F")))
    cfg.inverse_vandermonde_legendre = _dptr(
        arr(np.asfortranarray(b.inverse_vandermonde_legendre).ravel(order="F")))
    cfg.neighbor_ids = arr(nb, np.int64).ctypes.data_as(ctypes.POINTER(ctypes.c_int64))
    cfg.orientations = arr(orient, np.int64).ctypes.data_as(ctypes.POINTER(ctypes.c_int64))
    cfg.inverse_jacobian = _dptr(arr(semi.inverse_jacobian))
    if getattr(semi, "curved", False):
        cfg.mesh_type = _lib.TG_MESH_CURVED
        cfg.contravariant_vectors = _dptr(arr(semi.contravariant_vectors))
    cfg.node_coordinates = _dptr(arr(semi.node_coordinates))
    cfg.elements_per_block = int(elements_per_block)
    mids = getattr(semi, "mortar_neighbor_ids", None)
    if mids is not None and len(mids):
        i64p = ctypes.POINTER(ctypes.c_int64)
        cfg.nmortars = mids.shape[0]
        cfg.mortar_neighbor_ids = arr(mids, np.int64).ctypes.data_as(i64p)
        cfg.mortar_large_sides = arr(semi.mortar_large_sides, np.int64).ctypes.data_as(i64p)
        cfg.mortar_orientations = arr(semi.mortar_orientations, np.int64).ctypes.data_as(i64p)
        m = dg.mortar
        for name in ("forward_upper", "forward_lower", "reverse_upper", "reverse_lower"):
            setattr(cfg, "mortar_" + name,
                    _dptr(arr(np.asfortranarray(getattr(m, name)).ravel(order="F"))))
    funcs = set()
    for k, bc in enumerate(getattr(semi, "boundary_conditions", [])):
        cfg.boundary_conditions[k] = bc.code
        if isinstance(bc, BoundaryConditionDirichlet):
            funcs.add(bc.boundary_value_function)
    if len(funcs) > 1:
        raise NotImplementedError("Dirichlet boundaries with different functions")
    if funcs:
        f = funcs.pop()
        name = getattr(f, "__name__", None)
        if name not in _IC_CODES:
            raise NotImplementedError(f"Dirichlet values from {name!r}: only the package's "
                                      "initial conditions run on the device")
        cfg.boundary_value_function = _IC_CODES[name]
        for k, v in enumerate(getattr(f, "params", ())):
            cfg.boundary_value_params[k] = v
    return cfg, keep


class DeviceContext:
    """One tg_ctx: device-resident state, stage buffers and step graphs."""

    def __init__(self, semi, precision="fp64", device=0, elements_per_block=0, _handle=None):
        lib = _lib.load()
        self.lib = lib
        self.semi = semi
        self._owned = _handle is None
        if _handle is None:
            cfg, self._keep = make_config(semi, precision, device, elements_per_block)
            h = ctypes.c_void_p()
            _lib.check(lib.tg_ctx_create(ctypes.byref(cfg), ctypes.byref(h)))
        else:
            h = ctypes.c_void_p(_handle)
        self.h = h
        self.precision = precision
        self.t = None

    def close(self):
        if getattr(self, "h", None):
            if self._owned:
                self.lib.tg_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        _lib.check(rc, self.h)

    # -- AMR ----------------------------------------------------------------
    def amr_indicator(self, alpha_max, alpha_min, alpha_smooth, variable=0):
        """The HG indicator of the state with these parameters (variable 0:
        density_pressure, 1: density), in FP64 (tg_amr_indicator)."""
        out = np.zeros(self.semi.nelements)
        self._check(self.lib.tg_amr_indicator(self.h, float(alpha_max), float(alpha_min),
                                              int(bool(alpha_smooth)), int(variable), _dptr(out)))
        return out

    def amr_indicator_max(self, variable=1):
        """IndicatorMax: the maximum of the variable (1: density, 0:
        density_pressure) over each element's nodes, in FP64."""
        out = np.zeros(self.semi.nelements)
        self._check(self.lib.tg_amr_indicator_max(self.h, int(variable), _dptr(out)))
        return out

    def adapt_from(self, src, source_element, kind):
        """This context's state from `src`'s by the AMR transfer map
        (tg_adapt_state) with the solver's L2 adaptor matrices."""
        m = self.semi.solver.mortar
        mats = [np.ascontiguousarray(np.asfortranarray(getattr(m, k)).ravel(order="F"))
                for k in ("forward_upper", "forward_lower", "reverse_upper", "reverse_lower")]
        src_e = np.ascontiguousarray(source_element, dtype=np.int64)
        kd = np.ascontiguousarray(kind, dtype=np.int8)
        self._check(self.lib.tg_adapt_state(
            self.h, src.h, src_e.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
            kd.ctypes.data_as(ctypes.POINTER(ctypes.c_int8)), *[_dptr(x) for x in mats]))

    # -- state --------------------------------------------------------------
    def upload(self, u):
        if isinstance(u, np.ndarray):
            u = np.ascontiguousarray(u, dtype=np.float64)
            assert u.size == self.semi.nvalues
        self._check(self.lib.tg_upload_state(self.h, _ptr_of(u)))

    def download(self, out=None):
        if out is None:
            out = np.empty(self.semi.u_shape)
        self._check(self.lib.tg_download_state(self.h, _ptr_of(out)))
        return out

    # -- transfers overlapping the stepping (page-locked host buffers: numpy
    #    arrays that stay alive, or raw addresses) ------------------------------
    def prefetch(self, slot, u_host):
        """Start copying a host state into staging slot 0 or 1 (returns at once)."""
        self._check(self.lib.tg_prefetch_state(self.h, int(slot), _ptr_of(u_host)))

    def load_prefetched(self, slot):
        """The prefetched state of `slot` becomes the context's state (in stream order)."""
        self._check(self.lib.tg_load_prefetched(self.h, int(slot)))

    def fetch(self, slot, u_host):
        """Enqueue the copy of the current state to a host buffer (returns at once)."""
        self._check(self.lib.tg_fetch_state(self.h, int(slot), _ptr_of(u_host)))

    def transfer_wait(self, slot, direction):
        """Block until slot's prefetch (direction 0) or fetch (direction 1) completed."""
        self._check(self.lib.tg_transfer_wait(self.h, int(slot), int(direction)))

    def transfer_join(self):
        """The context stream waits for every transfer issued so far."""
        self._check(self.lib.tg_transfer_join(self.h))

    def state_ptr(self) -> int:
        p = ctypes.c_void_p()
        self._check(self.lib.tg_state_device_ptr(self.h, ctypes.byref(p)))
        return p.value

    # -- evaluations --------------------------------------------------------
    def rhs(self, du, u, t):
        """rhs! with device buffers (torch CUDA tensors or raw device addresses)."""
        self._check(self.lib.tg_rhs(self.h, _ptr_of(du), _ptr_of(u), float(t)))

    def rhs_host(self, u, t=0.0):
        u = np.ascontiguousarray(u, dtype=np.float64)
        du = np.empty_like(u)
        self._check(self.lib.tg_rhs_host(self.h, _ptr_of(du), _ptr_of(u), float(t)))
        return du

    def max_dt(self, u=None) -> float:
        dt = ctypes.c_double()
        self._check(self.lib.tg_max_dt(self.h, None if u is None else _ptr_of(u), ctypes.byref(dt)))
        return dt.value

    def rk_stage(self, stage, t, dt):
        self._check(self.lib.tg_rk_stage(self.h, int(stage), float(t), float(dt)))

    def rk_stage_part(self, stage, t, dt, parts):
        """One pass of rk_stage (parts 1: clock + shock indicator, 2: element
        kernel and state advance, 3: both), for timing the passes alone."""
        self._check(self.lib.tg_rk_stage_part(self.h, int(stage), float(t), float(dt), int(parts)))

    def step(self, max_steps, cfl, t_end, t):
        tt = ctypes.c_double(t)
        n = ctypes.c_int64(0)
        self._check(self.lib.tg_step(self.h, int(max_steps), float(cfl), float(t_end),
                                     ctypes.byref(tt), ctypes.byref(n)))
        return tt.value, n.value

    def step_enqueue(self, nsteps, cfl, t_end, t_start):
        """tg_step without waiting: enqueue nsteps step graphs and return."""
        self._check(self.lib.tg_step_enqueue(self.h, int(nsteps), float(cfl), float(t_end),
                                             float(t_start)))

    def clock_read(self):
        """(t, steps since the clock was set up, reached t_end), after synchronising."""
        t = ctypes.c_double()
        n = ctypes.c_int64()
        f = ctypes.c_int32()
        self._check(self.lib.tg_clock_read(self.h, ctypes.byref(t), ctypes.byref(n),
                                           ctypes.byref(f)))
        return t.value, n.value, bool(f.value)

    def integrals(self):
        out = np.zeros(self.semi.equations.nvariables + 2)
        self._check(self.lib.tg_integrals(self.h, _dptr(out)))
        return out

    def error_norms(self, t, exact=None, u=None, analyzer=None):
        """calc_error_norms on the device (tg_error_norms): L2 and Linf errors of
        the context state (or of `u`, device buffer) against `exact` (default:
        the semidiscretization's initial condition) at time t, on the
        (2N+1)-node analyzer.  `exact` must be one of the package's initial
        conditions (they run on the device)."""
        from .basis import LobattoLegendreAnalyzer
        f = exact or self.semi.initial_condition
        name = getattr(f, "__name__", None)
        if name not in _IC_CODES:
            raise NotImplementedError(f"error norms on the device against {name!r}: only the "
                                      "package's initial conditions run on the device")
        an = analyzer or LobattoLegendreAnalyzer(self.semi.solver.basis)
        vand = np.ascontiguousarray(np.asfortranarray(an.vandermonde).ravel(order="F"))
        w = np.ascontiguousarray(an.weights, dtype=np.float64)
        par = np.zeros(4)
        for k, v in enumerate(getattr(f, "params", ())):
            par[k] = v
        nv = self.semi.equations.nvariables
        l2, linf = np.zeros(nv), np.zeros(nv)
        self._check(self.lib.tg_error_norms(self.h, None if u is None else _ptr_of(u), float(t),
                                            _IC_CODES[name], _dptr(par), len(w), _dptr(vand),
                                            _dptr(w), _dptr(l2), _dptr(linf)))
        return l2, linf

    def entropy_timederivative(self, t=0.0) -> float:
        """Normalised integral of cons2entropy(u) . rhs(u, t) of the device state."""
        out = ctypes.c_double()
        self._check(self.lib.tg_entropy_timederivative(self.h, float(t), ctypes.byref(out)))
        return out.value

    def alpha(self, u=None):
        a = np.zeros(self.semi.nelements)
        self._check(self.lib.tg_alpha(self.h, None if u is None else _ptr_of(u), _dptr(a)))
        return a

    def status(self) -> int:
        f = ctypes.c_int32()
        self._check(self.lib.tg_status(self.h, ctypes.byref(f)))
        return f.value

    def synchronize(self):
        self._check(self.lib.tg_synchronize(self.h))

    def autotune(self, iters=20):
        """Time every elements-per-block value of the element kernel on the
        uploaded state (unchanged) and keep the fastest; returns (epb, ms per stage)."""
        epb = ctypes.c_int32()
        ms = ctypes.c_double()
        self._check(self.lib.tg_ctx_autotune(self.h, int(iters), ctypes.byref(epb), ctypes.byref(ms)))
        return epb.value, ms.value

    def stream(self) -> int:
        """cudaStream_t of the context (for torch.cuda.ExternalStream)."""
        p = ctypes.c_void_p()
        self._check(self.lib.tg_stream(self.h, ctypes.byref(p)))
        return p.value

    def elements_per_block(self) -> int:
        v = ctypes.c_int32()
        self._check(self.lib.tg_elements_per_block(self.h, ctypes.byref(v)))
        return v.value


class SemidiscretizationHyperbolic:
    """SemidiscretizationHyperbolic(mesh, equations, initial_condition, solver;
    source_terms, boundary_conditions), semidiscretization_hyperbolic.jl:50-76."""

    def __init__(self, mesh: TreeMesh, equations: CompressibleEulerEquations2D, initial_condition,
                 solver: DGSEM, source_terms=None, boundary_conditions=boundary_condition_periodic,
                 precision="fp64", device=0, elements_per_block=0):
        if mesh.ndims != equations.ndims:
            raise ValueError("mesh and equations have different dimensions")
        self.boundary_conditions = _digest_boundary_conditions(boundary_conditions, mesh)
        if precision not in ("fp64", "mixed"):
            raise ValueError("precision must be 'fp64' or 'mixed'")
        self.mesh, self.equations, self.solver = mesh, equations, solver
        self.initial_condition = initial_condition
        self.source_terms = source_terms
        self.precision = precision
        self.device, self.elements_per_block = device, elements_per_block
        self._ctx = None
        self._setup_containers()

    def _setup_containers(self):
        """Element geometry, interfaces and mortars of the current mesh."""
        mesh, equations, solver = self.mesh, self.equations, self.solver
        D, n = equations.ndims, solver.nnodes()
        self.nelements = mesh.nelements
        self.nnodes_per_element = n ** D
        self.ndofs = self.nelements * self.nnodes_per_element
        self.nvalues = self.ndofs * equations.nvariables
        self.u_shape = (self.nelements,) + (n,) * D + (equations.nvariables,)
        self.curved = bool(getattr(mesh, "curved", False))
        if self.curved:
            # StructuredMesh / P4estMesh brick: per-node metric terms
            # (dgsem_structured/containers_2d.jl:9-35, dgsem_p4est/containers_2d.jl:9-27)
            from .curved_mesh import metric_terms, metric_terms_3d
            self.node_coordinates = mesh.node_coordinates(solver.basis)
            self.contravariant_vectors, self.inverse_jacobian = (
                metric_terms if D == 2 else metric_terms_3d)(self.node_coordinates, solver.basis)
            self.neighbor_ids, self.orientations = mesh.interfaces()
            (self.mortar_neighbor_ids, self.mortar_large_sides,
             self.mortar_orientations) = mesh.mortars()
            return
        # init_elements!, containers_2d.jl:85-127
        b = solver.basis
        reference_length = 0.0
        for w in b.weights:
            reference_length += 1.0 * w
        reference_offset = (b.nodes[0] + b.nodes[-1]) / 2
        jac = mesh.element_lengths() / reference_length  # per element
        self.inverse_jacobian = 1.0 / jac
        centers = mesh.cell_centers()
        X = np.empty((self.nelements,) + (n,) * D + (D,))
        rel = b.nodes - reference_offset
        jb = jac.reshape((-1,) + (1,) * D)
        for d in range(D):
            # axis of node index along d in the (e, k, j, i) array order
            ax = D - d
            shape = [1] * (D + 1)
            shape[ax] = n
            X[..., d] = centers[:, d].reshape((-1,) + (1,) * D) + jb * rel.reshape(shape)
        self.node_coordinates = X
        self.neighbor_ids, self.orientations = mesh.interfaces()
        (self.mortar_neighbor_ids, self.mortar_large_sides,
         self.mortar_orientations) = mesh.mortars()

    def adapt(self, controller_value, only_refine=False, only_coarsen=False):
        """One AMR pass (amr.jl:244-392): adapts the mesh, rebuilds the
        containers and a device context for them, and transfers the state of the
        current context on the device (tg_adapt_state).  Returns whether the
        mesh changed."""
        changed, src, kind = self.mesh.adapt(controller_value, only_refine, only_coarsen)
        if not changed:
            return False
        old = self._ctx
        self._setup_containers()
        self._ctx = None
        if old is not None:
            new = self.device_context
            new.adapt_from(old, src, kind)
            old.close()
        return True

    @property
    def device_context(self) -> DeviceContext:
        if self._ctx is None:
            self._ctx = DeviceContext(self, self.precision, self.device, self.elements_per_block)
        return self._ctx

    def compute_coefficients(self, t=0.0):
        """compute_coefficients(t, semi): the initial condition at the nodes (dg.jl:1280-1325)."""
        return np.ascontiguousarray(self.initial_condition(self.node_coordinates, t, self.equations))

    def rhs(self, du, u, t):
        """rhs!(du, u, semi, t) with device buffers."""
        self.device_context.rhs(du, u, t)

    def __repr__(self):
        return (f"SemidiscretizationHyperbolic({self.mesh!r}, {self.equations!r}, {self.solver!r}, "
                f"precision={self.precision})")


class ODEProblem:
    def __init__(self, f, u0, tspan, p):
        self.f, self.u0, self.tspan, self.p = f, u0, tuple(float(x) for x in tspan), p


def semidiscretize(semi: SemidiscretizationHyperbolic, tspan) -> ODEProblem:
    """semidiscretize(semi, tspan), semidiscretization.jl:102-153."""
    u0 = semi.compute_coefficients(tspan[0])
    return ODEProblem(semi.rhs, u0, tspan, semi)
