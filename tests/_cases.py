"""Shared helpers: turn a golden/elixir case description into oracle objects."""
import json
import os

HERE = os.path.dirname(os.path.abspath(__file__))


def load_goldens():
    with open(os.path.join(HERE, "golden", "trixi_goldens.json"), encoding="utf-8") as f:
        return json.load(f)


def oracle_from_case(O, c, **over):
    c = dict(c, **over)
    vi = dict(weak=O.VI_WEAK, fluxdiff=O.VI_FLUXDIFF, hg=O.VI_SHOCKCAPTURING_HG)[c["vi"]]
    fl = dict(central=O.FLUX_CENTRAL, ranocha=O.FLUX_RANOCHA, shima_etal=O.FLUX_SHIMA_ETAL,
              llf=O.FLUX_LAX_FRIEDRICHS, llf_naive=O.FLUX_LAX_FRIEDRICHS_NAIVE,
              hllc=O.FLUX_HLLC, chandrashekar=O.FLUX_CHANDRASHEKAR, hlle=O.FLUX_HLLE)
    src = O.SRC_CONVERGENCE_TEST if c.get("source") == "convergence_test" else O.SRC_NONE
    orc = O.Oracle(c["ndims"], c["polydeg"], c["level"], c["xmin"], c["xmax"],
                   volume_integral=vi, volume_flux=fl[c["volume_flux"]],
                   surface_flux=fl[c["surface_flux"]],
                   alpha_max=c.get("alpha_max", 0.5), alpha_min=c.get("alpha_min", 0.001),
                   alpha_smooth=c.get("alpha_smooth", True), source=src)
    if c.get("refinement_patches"):
        orc.set_refinement(c["refinement_patches"])
    if c.get("amr"):
        orc.set_amr(**c["amr"])
    if c.get("boundary"):
        code = dict(dirichlet=O.BC_DIRICHLET, slip_wall=O.BC_SLIP_WALL)[c["boundary"]]
        orc.set_boundaries([code] * (2 * c["ndims"]), ic_id(O, c["ic"]), c.get("ic_params"))
    return orc


def ic_id(O, name):
    return dict(constant=O.IC_CONSTANT, convergence_test=O.IC_CONVERGENCE_TEST,
                isentropic_vortex=O.IC_ISENTROPIC_VORTEX, weak_blast_wave=O.IC_WEAK_BLAST_WAVE,
                kelvin_helmholtz=O.IC_KELVIN_HELMHOLTZ, taylor_green=O.IC_TAYLOR_GREEN,
                gaussian_blast=O.IC_GAUSSIAN_BLAST,
                isentropic_vortex_advected=O.IC_ISENTROPIC_VORTEX_ADVECTED,
                blast_wave=O.IC_BLAST_WAVE, density_pulse=O.IC_DENSITY_PULSE,
                sedov_blast_wave=O.IC_SEDOV_BLAST_WAVE, density_wave=O.IC_DENSITY_WAVE)[name]
