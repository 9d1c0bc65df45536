"""trixi_gb300 -- Trixi.jl's TreeMesh DGSEM Euler hot path on GB300 (sm_103a).

The names below mirror Trixi.jl's user API for that path, so that an elixir
such as examples/tree_3d_dgsem/elixir_euler_source_terms.jl reads the same:

    equations = CompressibleEulerEquations3D(1.4)
    solver = DGSEM(polydeg=3, surface_flux=flux_lax_friedrichs,
                   volume_integral=VolumeIntegralFluxDifferencing(flux_ranocha))
    mesh = TreeMesh((0.0,) * 3, (2.0,) * 3, initial_refinement_level=5)
    semi = SemidiscretizationHyperbolic(mesh, equations,
                                        initial_condition_convergence_test, solver,
                                        source_terms=source_terms_convergence_test)
    ode = semidiscretize(semi, (0.0, 1.0))
    sol = solve(ode, CarpenterKennedy2N54(williamson_condition=False), dt=1.0,
                callback=CallbackSet(StepsizeCallback(cfl=1.0)))

All numerics run in libtrixi_gb300.so (include/trixi_gb300.h); this package is
the host side: mesh/basis setup, the C-ABI binding and the driver loop.
"""
from ._lib import TrixiGB300Error, load as load_library  # noqa: F401
from .analysis import calc_error_norms  # noqa: F401
from .basis import LobattoLegendreAnalyzer, LobattoLegendreBasis, MortarL2  # noqa: F401
from .equations import (initial_condition_density_wave,  # noqa: F401
                        flux_chandrashekar, flux_hlle, initial_condition_sedov_blast_wave,  # noqa: F401
                        initial_condition_medium_sedov_blast_wave,  # noqa: F401
                        flux_hllc, initial_condition_isentropic_vortex_advected,  # noqa: F401
                        initial_condition_density_pulse,  # noqa: F401
                        initial_condition_blast_wave,  # noqa: F401
                        CompressibleEulerEquations2D, CompressibleEulerEquations3D,  # noqa: F401
                        FluxLaxFriedrichs, cons2prim, density, density_pressure, flux_central,
                        flux_lax_friedrichs, flux_ranocha, flux_shima_etal,
                        initial_condition_constant, initial_condition_convergence_test,
                        initial_condition_gaussian_blast, initial_condition_isentropic_vortex,
                        initial_condition_kelvin_helmholtz_instability,
                        initial_condition_taylor_green_vortex, initial_condition_weak_blast_wave,
                        max_abs_speed, max_abs_speed_naive, prim2cons,
                        source_terms_convergence_test)
from .mesh import TreeMesh  # noqa: F401
from .curved_mesh import P4estMesh, StructuredMesh  # noqa: F401
from .semidiscretization import (BoundaryConditionDirichlet, DeviceContext, ODEProblem,  # noqa: F401
                                 SemidiscretizationHyperbolic, boundary_condition_periodic,
                                 boundary_condition_slip_wall, semidiscretize)
from .solvers import (DGSEM, IndicatorHennemannGassner, IndicatorMax, VolumeIntegralFluxDifferencing,  # noqa: F401
                      VolumeIntegralShockCapturingHG, VolumeIntegralWeakForm)
from .time_integration import (AliveCallback, AnalysisCallback, CallbackSet,  # noqa: F401
                               CarpenterKennedy2N54, StepsizeCallback, SummaryCallback,
                               ode_default_options, solve)
from .ensemble import Ensemble  # noqa: F401
from .amr import AMRCallback, ControllerThreeLevel  # noqa: F401
