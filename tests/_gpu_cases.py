"""Builders shared by the GPU tests: a trixi_gb300 semidiscretization and the
matching oracle for the same mesh, basis and solver options."""
import numpy as np

import trixi_gb300 as T
from oracle import oracle as O

FLUX = {"central": (T.flux_central, O.FLUX_CENTRAL), "ranocha": (T.flux_ranocha, O.FLUX_RANOCHA),
        "shima_etal": (T.flux_shima_etal, O.FLUX_SHIMA_ETAL),
        "llf": (T.flux_lax_friedrichs, O.FLUX_LAX_FRIEDRICHS),
        "llf_naive": (T.FluxLaxFriedrichs(T.max_abs_speed_naive), O.FLUX_LAX_FRIEDRICHS_NAIVE),
        "hllc": (T.flux_hllc, O.FLUX_HLLC),
        "chandrashekar": (T.flux_chandrashekar, O.FLUX_CHANDRASHEKAR),
        "hlle": (T.flux_hlle, O.FLUX_HLLE)}
IC = {"convergence_test": (lambda p: T.initial_condition_convergence_test, O.IC_CONVERGENCE_TEST),
      "weak_blast_wave": (lambda p: T.initial_condition_weak_blast_wave, O.IC_WEAK_BLAST_WAVE),
      "kelvin_helmholtz": (lambda p: T.initial_condition_kelvin_helmholtz_instability,
                           O.IC_KELVIN_HELMHOLTZ),
      "isentropic_vortex": (lambda p: T.initial_condition_isentropic_vortex(*(p or [25.0, 5.0])),
                            O.IC_ISENTROPIC_VORTEX),
      "taylor_green": (lambda p: T.initial_condition_taylor_green_vortex(*(p or [0.1])),
                       O.IC_TAYLOR_GREEN),
      "constant": (lambda p: T.initial_condition_constant, O.IC_CONSTANT),
      "blast_wave": (lambda p: T.initial_condition_blast_wave, O.IC_BLAST_WAVE),
      "density_pulse": (lambda p: T.initial_condition_density_pulse, O.IC_DENSITY_PULSE),
      "sedov_blast_wave": (lambda p: T.initial_condition_sedov_blast_wave, O.IC_SEDOV_BLAST_WAVE),
      "density_wave": (lambda p: T.initial_condition_density_wave, O.IC_DENSITY_WAVE),
      "isentropic_vortex_advected": (
          lambda p: T.initial_condition_isentropic_vortex_advected(*(p or [25.0, 5.0])),
          O.IC_ISENTROPIC_VORTEX_ADVECTED),
      "gaussian_blast": (lambda p: T.initial_condition_gaussian_blast(*(p or [1e-5, 1.0, 0.25])),
                         O.IC_GAUSSIAN_BLAST)}


def build(c, precision="fp64", elements_per_block=0):
    D = c["ndims"]
    eq = T.CompressibleEulerEquations2D(1.4) if D == 2 else T.CompressibleEulerEquations3D(1.4)
    basis = T.LobattoLegendreBasis(c["polydeg"])
    sflux = FLUX[c["surface_flux"]][0]
    vflux = FLUX[c.get("volume_flux", "central")][0]
    if c["vi"] == "weak":
        vi = T.VolumeIntegralWeakForm()
        ovi = O.VI_WEAK
    elif c["vi"] == "fluxdiff":
        vi = T.VolumeIntegralFluxDifferencing(vflux)
        ovi = O.VI_FLUXDIFF
    else:
        ind = T.IndicatorHennemannGassner(eq, basis, alpha_max=c.get("alpha_max", 0.5),
                                          alpha_min=c.get("alpha_min", 0.001),
                                          alpha_smooth=c.get("alpha_smooth", True),
                                          variable=T.density_pressure)
        fvflux = FLUX[c.get("fv_flux", c["surface_flux"])][0]
        vi = T.VolumeIntegralShockCapturingHG(ind, volume_flux_dg=vflux, volume_flux_fv=fvflux)
        ovi = O.VI_SHOCKCAPTURING_HG
    solver = T.DGSEM(basis, sflux, vi)
    boundary = c.get("boundary")
    mesh = T.TreeMesh(c["xmin"], c["xmax"], initial_refinement_level=c["level"],
                      periodicity=boundary is None,
                      refinement_patches=c.get("refinement_patches", ()))
    src = T.source_terms_convergence_test if c.get("source") == "convergence_test" else None
    ic = IC[c["ic"]][0](c.get("ic_params"))
    bcs = {None: T.boundary_condition_periodic, "slip_wall": T.boundary_condition_slip_wall,
           "dirichlet": T.BoundaryConditionDirichlet(ic)}[boundary]
    semi = T.SemidiscretizationHyperbolic(mesh, eq, ic, solver, source_terms=src,
                                          boundary_conditions=bcs, precision=precision,
                                          elements_per_block=elements_per_block)
    orc = O.Oracle(D, c["polydeg"], c["level"], c["xmin"], c["xmax"], volume_integral=ovi,
                   volume_flux=FLUX[c.get("volume_flux", "central")][1],
                   surface_flux=FLUX[c["surface_flux"]][1],
                   alpha_max=c.get("alpha_max", 0.5), alpha_min=c.get("alpha_min", 0.001),
                   alpha_smooth=c.get("alpha_smooth", True),
                   fv_flux=FLUX[c["fv_flux"]][1] if c.get("fv_flux") else None,
                   source=O.SRC_CONVERGENCE_TEST if src is not None else O.SRC_NONE)
    if c.get("refinement_patches"):
        orc.set_refinement(c["refinement_patches"])
    if c.get("amr"):
        orc.set_amr(**c["amr"])
    if boundary is not None:
        code = dict(dirichlet=O.BC_DIRICHLET, slip_wall=O.BC_SLIP_WALL)[boundary]
        orc.set_boundaries([code] * (2 * D), IC[c["ic"]][1], c.get("ic_params"))
    return semi, orc


def amr_callback(semi, c):
    """AMRCallback + ControllerThreeLevel(IndicatorHennemannGassner) from a case's amr dict."""
    a = dict(c["amr"])
    variables = {"density_pressure": T.density_pressure, "density": T.density}
    if a.pop("indicator", "hennemann_gassner") == "max":
        ind = T.IndicatorMax(semi, variable=variables[a.pop("variable", "density")])
    else:
        ind = None
    ind = ind or T.IndicatorHennemannGassner(semi, alpha_max=a.pop("alpha_max", 0.5),
                                      alpha_min=a.pop("alpha_min", 0.001),
                                      alpha_smooth=a.pop("alpha_smooth", True),
                                      variable={"density_pressure": T.density_pressure,
                                                "density": T.density}[
                                          a.pop("variable", "density_pressure")])
    ctrl = T.ControllerThreeLevel(semi, ind, base_level=a.pop("base_level", 1),
                                  med_level=a.pop("med_level", None),
                                  med_threshold=a.pop("med_threshold", 0.0),
                                  max_level=a.pop("max_level", None),
                                  max_threshold=a.pop("max_threshold", 1.0))
    return T.AMRCallback(semi, ctrl, **a)


def perturbed_state(semi, seed=0, amp=1e-2):
    """A smooth initial state with a random relative perturbation (positivity kept)."""
    rng = np.random.default_rng(seed)
    u = semi.compute_coefficients(0.0)
    return u * (1.0 + amp * rng.uniform(-1, 1, size=u.shape))


def rel_err(a, b):
    """Max over variables of max|a - b| / max|b| (normwise per variable)."""
    nv = a.shape[-1]
    a2, b2 = a.reshape(-1, nv), b.reshape(-1, nv)
    return float(np.max(np.max(np.abs(a2 - b2), axis=0) / np.maximum(np.max(np.abs(b2), axis=0), 1e-300)))
