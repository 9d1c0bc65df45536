"""Extract the L2/Linf goldens of Trixi.jl's TreeMesh, StructuredMesh and P4estMesh
Euler regression tests.

Run once in a checkout that has the Trixi.jl sources (read as text, nothing is
executed):

    python tests/golden/extract_goldens.py /path/to/Trixi.jl

It writes ``tests/golden/trixi_goldens.json``: for each selected ``@testitem``
the golden ``l2``/``linf`` vectors and the overridden keyword arguments, next
to the elixir settings (transcribed from the elixir files named in each entry)
that the oracle needs to reproduce the run.
"""
from __future__ import annotations

import json
import os
import re
import sys

# Elixir settings transcribed from examples/tree_{2,3}d_dgsem/*.jl.
# vi: weak | fluxdiff | hg ; fluxes: central | ranocha | shima_etal | llf | llf_naive | hllc | chandrashekar | hlle
CASES = {
    "TreeMesh2D Euler: elixir_euler_source_terms.jl": dict(
        file="test/test_tree_2d_euler.jl",
        elixir="examples/tree_2d_dgsem/elixir_euler_source_terms.jl",
        ndims=2, polydeg=3, level=4, xmin=[0.0, 0.0], xmax=[2.0, 2.0],
        ic="convergence_test", source="convergence_test", vi="weak",
        volume_flux="central", surface_flux="llf_naive", cfl=1.0, tspan=[0.0, 2.0]),
    "TreeMesh2D Euler: elixir_euler_ec.jl": dict(
        file="test/test_tree_2d_euler.jl",
        elixir="examples/tree_2d_dgsem/elixir_euler_ec.jl",
        ndims=2, polydeg=3, level=5, xmin=[-2.0, -2.0], xmax=[2.0, 2.0],
        ic="weak_blast_wave", source="none", vi="fluxdiff",
        volume_flux="ranocha", surface_flux="ranocha", cfl=1.0, tspan=[0.0, 0.4]),
    "TreeMesh2D Euler: elixir_euler_source_terms_nonperiodic.jl": dict(
        file="test/test_tree_2d_euler.jl",
        elixir="examples/tree_2d_dgsem/elixir_euler_source_terms_nonperiodic.jl",
        ndims=2, polydeg=3, level=4, xmin=[0.0, 0.0], xmax=[2.0, 2.0],
        ic="convergence_test", source="convergence_test", vi="weak",
        volume_flux="central", surface_flux="llf_naive", cfl=1.0, tspan=[0.0, 2.0],
        boundary="dirichlet"),
    "TreeMesh2D Euler: elixir_euler_ec.jl with boundary_condition_slip_wall": dict(
        file="test/test_tree_2d_euler.jl",
        elixir="examples/tree_2d_dgsem/elixir_euler_ec.jl",
        ndims=2, polydeg=3, level=5, xmin=[-2.0, -2.0], xmax=[2.0, 2.0],
        ic="weak_blast_wave", source="none", vi="fluxdiff",
        volume_flux="ranocha", surface_flux="ranocha", cfl=0.3, tspan=[0.0, 0.1],
        boundary="slip_wall"),
    "TreeMesh2D Euler: elixir_euler_shockcapturing.jl": dict(
        file="test/test_tree_2d_euler.jl",
        elixir="examples/tree_2d_dgsem/elixir_euler_shockcapturing.jl",
        ndims=2, polydeg=3, level=5, xmin=[-2.0, -2.0], xmax=[2.0, 2.0],
        ic="weak_blast_wave", source="none", vi="hg", volume_flux="shima_etal",
        surface_flux="llf_naive", alpha_max=0.5, alpha_min=0.001, alpha_smooth=True,
        cfl=1.0, tspan=[0.0, 1.0]),
    "TreeMesh2D Euler: elixir_euler_kelvin_helmholtz_instability.jl": dict(
        file="test/test_tree_2d_euler.jl",
        elixir="examples/tree_2d_dgsem/elixir_euler_kelvin_helmholtz_instability.jl",
        ndims=2, polydeg=3, level=5, xmin=[-1.0, -1.0], xmax=[1.0, 1.0],
        ic="kelvin_helmholtz", source="none", vi="hg", volume_flux="ranocha",
        surface_flux="llf_naive", alpha_max=0.002, alpha_min=0.0001, alpha_smooth=True,
        cfl=1.3, tspan=[0.0, 3.0]),
    "TreeMesh2D Euler: elixir_euler_vortex.jl": dict(
        file="test/test_tree_2d_euler.jl",
        elixir="examples/tree_2d_dgsem/elixir_euler_vortex.jl",
        ndims=2, polydeg=3, level=4, xmin=[-10.0, -10.0], xmax=[10.0, 10.0],
        ic="isentropic_vortex", ic_params=[25.0, 5.0], source="none", vi="weak",
        volume_flux="central", surface_flux="llf_naive", cfl=1.1, tspan=[0.0, 20.0]),
    "TreeMesh2D Euler: elixir_euler_vortex.jl one step with initial_condition_constant": dict(
        file="test/test_tree_2d_euler.jl",
        elixir="examples/tree_2d_dgsem/elixir_euler_vortex.jl",
        ndims=2, polydeg=3, level=4, xmin=[-10.0, -10.0], xmax=[10.0, 10.0],
        ic="constant", source="none", vi="weak",
        volume_flux="central", surface_flux="llf_naive", cfl=1.1, tspan=[0.0, 20.0]),
    "TreeMesh3D Euler: elixir_euler_source_terms.jl": dict(
        file="test/test_tree_3d_euler.jl",
        elixir="examples/tree_3d_dgsem/elixir_euler_source_terms.jl",
        ndims=3, polydeg=3, level=2, xmin=[0.0] * 3, xmax=[2.0] * 3,
        ic="convergence_test", source="convergence_test", vi="weak",
        volume_flux="central", surface_flux="llf_naive", cfl=0.6, tspan=[0.0, 5.0]),
    "TreeMesh3D Euler: elixir_euler_source_terms.jl with split_form": dict(
        file="test/test_tree_3d_euler.jl",
        elixir="examples/tree_3d_dgsem/elixir_euler_source_terms.jl",
        ndims=3, polydeg=3, level=2, xmin=[0.0] * 3, xmax=[2.0] * 3,
        ic="convergence_test", source="convergence_test", vi="fluxdiff",
        volume_flux="central", surface_flux="llf_naive", cfl=0.6, tspan=[0.0, 5.0]),
    "TreeMesh3D Euler: elixir_euler_taylor_green_vortex.jl": dict(
        file="test/test_tree_3d_euler.jl",
        elixir="examples/tree_3d_dgsem/elixir_euler_taylor_green_vortex.jl",
        ndims=3, polydeg=3, level=3, xmin=[-3.141592653589793] * 3,
        xmax=[3.141592653589793] * 3, ic="taylor_green", ic_params=[0.1], source="none",
        vi="fluxdiff", volume_flux="ranocha", surface_flux="llf_naive", cfl=1.4,
        tspan=[0.0, 10.0]),
    "TreeMesh2D Euler: elixir_euler_vortex_mortar_split.jl": dict(
        file="test/test_tree_2d_euler.jl",
        elixir="examples/tree_2d_dgsem/elixir_euler_vortex_mortar_split.jl",
        ndims=2, polydeg=3, level=4, xmin=[-10.0, -10.0], xmax=[10.0, 10.0],
        refinement_patches=[dict(type="box", coordinates_min=[0.0, -10.0],
                                 coordinates_max=[10.0, 10.0])],
        ic="isentropic_vortex", ic_params=[25.0, 5.0], source="none",
        vi="fluxdiff", volume_flux="shima_etal", surface_flux="llf_naive", cfl=1.4,
        tspan=[0.0, 1.0]),
    "TreeMesh2D Euler: elixir_euler_vortex_mortar.jl": dict(
        file="test/test_tree_2d_euler.jl",
        elixir="examples/tree_2d_dgsem/elixir_euler_vortex_mortar.jl",
        ndims=2, polydeg=3, level=4, xmin=[-10.0, -10.0], xmax=[10.0, 10.0],
        refinement_patches=[dict(type="box", coordinates_min=[0.0, -10.0],
                                 coordinates_max=[10.0, 10.0])],
        ic="isentropic_vortex_advected", ic_params=[25.0, 5.0], source="none",
        vi="weak", volume_flux="central", surface_flux="hllc", cfl=1.4, tspan=[0.0, 1.0]),
    "TreeMesh2D Euler: elixir_euler_vortex_mortar_shockcapturing.jl": dict(
        file="test/test_tree_2d_euler.jl",
        elixir="examples/tree_2d_dgsem/elixir_euler_vortex_mortar_shockcapturing.jl",
        ndims=2, polydeg=3, level=4, xmin=[-10.0, -10.0], xmax=[10.0, 10.0],
        refinement_patches=[dict(type="box", coordinates_min=[0.0, -10.0],
                                 coordinates_max=[10.0, 10.0])],
        ic="isentropic_vortex", ic_params=[25.0, 5.0], source="none",
        vi="hg", volume_flux="shima_etal", surface_flux="llf_naive", alpha_max=0.5,
        alpha_min=0.001, alpha_smooth=True, cfl=0.7, tspan=[0.0, 1.0]),
    "TreeMesh2D Euler: elixir_euler_blast_wave_amr.jl": dict(
        file="test/test_tree_2d_euler.jl",
        elixir="examples/tree_2d_dgsem/elixir_euler_blast_wave_amr.jl",
        ndims=2, polydeg=3, level=6, xmin=[-2.0, -2.0], xmax=[2.0, 2.0],
        ic="blast_wave", source="none", vi="hg", volume_flux="ranocha",
        surface_flux="llf_naive", alpha_max=0.5, alpha_min=0.001, alpha_smooth=True,
        cfl=0.9, tspan=[0.0, 12.5],
        amr=dict(interval=5, adapt_initial_condition=True,
                 adapt_initial_condition_only_refine=True, alpha_max=0.5, alpha_min=0.001,
                 alpha_smooth=True, base_level=4, max_level=6, max_threshold=0.01)),
    "TreeMesh3D Euler: elixir_euler_shockcapturing_amr.jl": dict(
        file="test/test_tree_3d_euler.jl",
        elixir="examples/tree_3d_dgsem/elixir_euler_shockcapturing_amr.jl",
        ndims=3, polydeg=3, level=3, xmin=[-2.0] * 3, xmax=[2.0] * 3,
        ic="weak_blast_wave", source="none", vi="hg", volume_flux="ranocha",
        surface_flux="ranocha", alpha_max=0.5, alpha_min=0.001, alpha_smooth=True,
        cfl=1.3, tspan=[0.0, 0.4],
        amr=dict(interval=1, adapt_initial_condition=True,
                 adapt_initial_condition_only_refine=True, alpha_max=0.5, alpha_min=0.001,
                 alpha_smooth=False, base_level=2, max_level=4, max_threshold=0.0003)),
    "TreeMesh2D Euler: elixir_euler_kelvin_helmholtz_instability_amr.jl": dict(
        file="test/test_tree_2d_euler.jl",
        elixir="examples/tree_2d_dgsem/elixir_euler_kelvin_helmholtz_instability_amr.jl",
        ndims=2, polydeg=3, level=5, xmin=[-1.0, -1.0], xmax=[1.0, 1.0],
        ic="kelvin_helmholtz", source="none", vi="hg", volume_flux="ranocha",
        surface_flux="llf_naive", alpha_max=0.002, alpha_min=0.0001, alpha_smooth=True,
        cfl=1.3, tspan=[0.0, 3.0],
        amr=dict(interval=1, adapt_initial_condition=True,
                 adapt_initial_condition_only_refine=True, alpha_max=1.0, alpha_min=0.0001,
                 alpha_smooth=False, variable="density", base_level=4, med_level=0,
                 med_threshold=0.0003, max_level=6, max_threshold=0.003)),
    "TreeMesh3D Euler: elixir_euler_amr.jl": dict(
        file="test/test_tree_3d_euler.jl",
        elixir="examples/tree_3d_dgsem/elixir_euler_amr.jl",
        ndims=3, polydeg=3, level=4, xmin=[-5.0] * 3, xmax=[5.0] * 3,
        ic="density_pulse", source="none", vi="weak", volume_flux="central",
        surface_flux="llf_naive", cfl=0.9, tspan=[0.0, 10.0],
        amr=dict(interval=5, adapt_initial_condition=True,
                 adapt_initial_condition_only_refine=True, indicator="max", variable="density",
                 base_level=4, med_level=5, med_threshold=1.05, max_level=6, max_threshold=1.3)),
    "TreeMesh2D Euler: elixir_euler_sedov_blast_wave.jl": dict(
        file="test/test_tree_2d_euler.jl",
        elixir="examples/tree_2d_dgsem/elixir_euler_sedov_blast_wave.jl",
        ndims=2, polydeg=3, level=6, xmin=[-2.0, -2.0], xmax=[2.0, 2.0],
        ic="sedov_blast_wave", source="none", vi="hg", volume_flux="chandrashekar",
        surface_flux="llf_naive", alpha_max=0.5, alpha_min=0.001, alpha_smooth=True,
        cfl=0.8, tspan=[0.0, 12.5],
        amr=dict(interval=5, adapt_initial_condition=True,
                 adapt_initial_condition_only_refine=True, alpha_max=0.5, alpha_min=0.001,
                 alpha_smooth=True, base_level=4, max_level=6, max_threshold=0.01)),
    "TreeMesh2D Euler: elixir_euler_sedov_blast_wave.jl (HLLE)": dict(
        file="test/test_tree_2d_euler.jl",
        elixir="examples/tree_2d_dgsem/elixir_euler_sedov_blast_wave.jl",
        ndims=2, polydeg=3, level=6, xmin=[-2.0, -2.0], xmax=[2.0, 2.0],
        ic="sedov_blast_wave", source="none", vi="hg", volume_flux="chandrashekar",
        surface_flux="hlle", alpha_max=0.5, alpha_min=0.001, alpha_smooth=True,
        cfl=0.8, tspan=[0.0, 12.5]),
    "TreeMesh2D Euler: elixir_euler_blast_wave.jl": dict(
        file="test/test_tree_2d_euler.jl",
        elixir="examples/tree_2d_dgsem/elixir_euler_blast_wave.jl",
        ndims=2, polydeg=3, level=6, xmin=[-2.0, -2.0], xmax=[2.0, 2.0],
        ic="blast_wave", source="none", vi="hg", volume_flux="ranocha",
        surface_flux="llf_naive", alpha_max=0.5, alpha_min=0.001, alpha_smooth=True,
        cfl=0.9, tspan=[0.0, 12.5]),
    "TreeMesh2D Euler: elixir_euler_vortex_shockcapturing.jl": dict(
        file="test/test_tree_2d_euler.jl",
        elixir="examples/tree_2d_dgsem/elixir_euler_vortex_shockcapturing.jl",
        ndims=2, polydeg=3, level=4, xmin=[-10.0, -10.0], xmax=[10.0, 10.0],
        ic="isentropic_vortex", ic_params=[25.0, 5.0], source="none", vi="hg",
        volume_flux="shima_etal", surface_flux="llf_naive", alpha_max=0.5, alpha_min=0.001,
        alpha_smooth=True, cfl=0.7, tspan=[0.0, 1.0]),
    "TreeMesh2D Euler: elixir_euler_density_wave.jl": dict(
        file="test/test_tree_2d_euler.jl",
        elixir="examples/tree_2d_dgsem/elixir_euler_density_wave.jl",
        ndims=2, polydeg=5, level=2, xmin=[-1.0, -1.0], xmax=[1.0, 1.0],
        ic="density_wave", source="none", vi="weak", volume_flux="central",
        surface_flux="central", cfl=1.6, tspan=[0.0, 2.0]),
    "TreeMesh2D Euler: elixir_euler_ec.jl with flux_chandrashekar": dict(
        file="test/test_tree_2d_euler.jl",
        elixir="examples/tree_2d_dgsem/elixir_euler_ec.jl",
        ndims=2, polydeg=3, level=5, xmin=[-2.0, -2.0], xmax=[2.0, 2.0],
        ic="weak_blast_wave", source="none", vi="fluxdiff", volume_flux="chandrashekar",
        surface_flux="chandrashekar", cfl=1.0, tspan=[0.0, 0.4]),
    "TreeMesh3D Euler: elixir_euler_ec.jl with flux_chandrashekar": dict(
        file="test/test_tree_3d_euler.jl",
        elixir="examples/tree_3d_dgsem/elixir_euler_ec.jl",
        ndims=3, polydeg=3, level=3, xmin=[-2.0] * 3, xmax=[2.0] * 3,
        ic="weak_blast_wave", source="none", vi="fluxdiff", volume_flux="chandrashekar",
        surface_flux="chandrashekar", cfl=1.3, tspan=[0.0, 0.4]),
    "TreeMesh3D Euler: elixir_euler_ec.jl with flux_shima_etal": dict(
        file="test/test_tree_3d_euler.jl",
        elixir="examples/tree_3d_dgsem/elixir_euler_ec.jl",
        ndims=3, polydeg=3, level=3, xmin=[-2.0] * 3, xmax=[2.0] * 3,
        ic="weak_blast_wave", source="none", vi="fluxdiff", volume_flux="shima_etal",
        surface_flux="shima_etal", cfl=1.3, tspan=[0.0, 0.4]),
    "TreeMesh3D Euler: elixir_euler_ec.jl with initial_condition=initial_condition_constant": dict(
        file="test/test_tree_3d_euler.jl",
        elixir="examples/tree_3d_dgsem/elixir_euler_ec.jl",
        ndims=3, polydeg=3, level=3, xmin=[-2.0] * 3, xmax=[2.0] * 3,
        ic="constant", source="none", vi="fluxdiff", volume_flux="ranocha",
        surface_flux="ranocha", cfl=1.3, tspan=[0.0, 0.4]),
    "TreeMesh3D Euler: elixir_euler_shockcapturing.jl": dict(
        file="test/test_tree_3d_euler.jl",
        elixir="examples/tree_3d_dgsem/elixir_euler_shockcapturing.jl",
        ndims=3, polydeg=3, level=3, xmin=[-2.0] * 3, xmax=[2.0] * 3,
        ic="weak_blast_wave", source="none", vi="hg", volume_flux="ranocha",
        surface_flux="ranocha", alpha_max=0.5, alpha_min=0.001, alpha_smooth=True,
        cfl=1.4, tspan=[0.0, 0.4]),
    "TreeMesh3D Euler: elixir_euler_density_pulse.jl": dict(
        file="test/test_tree_3d_euler.jl",
        elixir="examples/tree_3d_dgsem/elixir_euler_density_pulse.jl",
        ndims=3, polydeg=3, level=3, xmin=[-2.0] * 3, xmax=[2.0] * 3,
        ic="density_pulse", source="none", vi="fluxdiff", volume_flux="ranocha",
        surface_flux="ranocha", cfl=1.1, tspan=[0.0, 0.4]),
    "TreeMesh3D Euler: elixir_euler_mortar.jl": dict(
        file="test/test_tree_3d_euler.jl",
        elixir="examples/tree_3d_dgsem/elixir_euler_mortar.jl",
        ndims=3, polydeg=3, level=2, xmin=[0.0] * 3, xmax=[2.0] * 3,
        refinement_patches=[dict(type="box", coordinates_min=[0.5] * 3,
                                 coordinates_max=[1.5] * 3)],
        ic="convergence_test", source="convergence_test", vi="weak",
        volume_flux="central", surface_flux="llf_naive", cfl=0.6, tspan=[0.0, 1.0]),
    "TreeMesh3D Euler: elixir_euler_ec.jl": dict(
        file="test/test_tree_3d_euler.jl",
        elixir="examples/tree_3d_dgsem/elixir_euler_ec.jl",
        ndims=3, polydeg=3, level=3, xmin=[-2.0] * 3, xmax=[2.0] * 3,
        ic="weak_blast_wave", source="none", vi="fluxdiff", volume_flux="ranocha",
        surface_flux="ranocha", cfl=1.3, tspan=[0.0, 0.4]),
}

# Curvilinear 2D meshes (examples/structured_2d_dgsem, examples/p4est_2d_dgsem).
# mesh: structured (cells) | p4est (trees, level); mapping: the elixir's
# mapping or faces by name (restated in tests/_curved_cases.py).
CURVED_CASES = {
    "StructuredMesh2D: elixir_euler_source_terms.jl": dict(
        file="test/test_structured_2d.jl",
        elixir="examples/structured_2d_dgsem/elixir_euler_source_terms.jl",
        mesh="structured", cells=[16, 16], mapping="square_0_2", polydeg=3,
        ic="convergence_test", source="convergence_test", vi="weak",
        volume_flux="central", surface_flux="llf_naive", cfl=1.0, tspan=[0.0, 2.0]),
    "StructuredMesh2D: elixir_euler_source_terms_parallelogram.jl": dict(
        file="test/test_structured_2d.jl",
        elixir="examples/structured_2d_dgsem/elixir_euler_source_terms_parallelogram.jl",
        mesh="structured", cells=[16, 16], mapping="parallelogram", polydeg=3,
        ic="convergence_test", source="convergence_test", vi="weak",
        volume_flux="central", surface_flux="llf_naive", cfl=0.5, tspan=[0.0, 2.0]),
    "StructuredMesh2D: elixir_euler_source_terms_waving_flag.jl": dict(
        file="test/test_structured_2d.jl",
        elixir="examples/structured_2d_dgsem/elixir_euler_source_terms_waving_flag.jl",
        mesh="structured", cells=[16, 16], mapping="waving_flag", polydeg=3,
        ic="convergence_test", source="convergence_test", vi="weak",
        volume_flux="central", surface_flux="llf_naive", cfl=0.8, tspan=[0.0, 2.0]),
    "StructuredMesh2D: elixir_euler_source_terms_nonperiodic.jl": dict(
        file="test/test_structured_2d.jl",
        elixir="examples/structured_2d_dgsem/elixir_euler_source_terms_nonperiodic.jl",
        mesh="structured", cells=[16, 16], mapping="square_0_2", polydeg=3,
        ic="convergence_test", source="convergence_test", vi="weak",
        volume_flux="central", surface_flux="llf_naive", cfl=1.0, tspan=[0.0, 2.0],
        boundary="dirichlet"),
    "StructuredMesh2D: elixir_euler_free_stream.jl": dict(
        file="test/test_structured_2d.jl",
        elixir="examples/structured_2d_dgsem/elixir_euler_free_stream.jl",
        mesh="structured", cells=[16, 16], mapping="warped_square_0_3", polydeg=3,
        ic="constant", source="none", vi="weak",
        volume_flux="central", surface_flux="llf_naive", cfl=2.0, tspan=[0.0, 2.0]),
    "StructuredMesh2D: elixir_euler_ec.jl": dict(
        file="test/test_structured_2d.jl",
        elixir="examples/structured_2d_dgsem/elixir_euler_ec.jl",
        mesh="structured", cells=[16, 16], mapping="warped_square_0_3", polydeg=4,
        ic="weak_blast_wave", source="none", vi="fluxdiff",
        volume_flux="ranocha", surface_flux="ranocha", cfl=1.0, tspan=[0.0, 2.0]),
    # shock capturing on curvilinear meshes (oracle)
    "P4estMesh2D: elixir_euler_shockcapturing_ec.jl": dict(
        file="test/test_p4est_2d.jl",
        elixir="examples/p4est_2d_dgsem/elixir_euler_shockcapturing_ec.jl",
        mesh="p4est", trees=[4, 4], level=2, mapping="square_m1_1", polydeg=4,
        ic="weak_blast_wave", source="none", vi="hg", volume_flux="ranocha",
        volume_flux_fv="ranocha", surface_flux="ranocha", alpha_max=1.0, alpha_min=0.001,
        alpha_smooth=True, cfl=1.0, tspan=[0.0, 2.0]),
    "P4estMesh2D: elixir_euler_shockcapturing_ec.jl (flux_chandrashekar)": dict(
        file="test/test_p4est_2d.jl",
        elixir="examples/p4est_2d_dgsem/elixir_euler_shockcapturing_ec.jl",
        mesh="p4est", trees=[4, 4], level=2, mapping="square_m1_1", polydeg=4,
        ic="weak_blast_wave", source="none", vi="hg", volume_flux="chandrashekar",
        volume_flux_fv="ranocha", surface_flux="ranocha", alpha_max=1.0, alpha_min=0.001,
        alpha_smooth=True, cfl=1.0, tspan=[0.0, 2.0]),
    "StructuredMesh2D: elixir_euler_sedov.jl": dict(
        file="test/test_structured_2d.jl",
        elixir="examples/structured_2d_dgsem/elixir_euler_sedov.jl",
        mesh="structured", cells=[16, 16], mapping="sedov_warp", polydeg=4,
        ic="sedov_blast_wave", source="none", vi="hg", volume_flux="ranocha",
        volume_flux_fv="llf_naive", surface_flux="llf_naive", alpha_max=1.0, alpha_min=0.001,
        alpha_smooth=True, cfl=0.5, tspan=[0.0, 12.5]),
    # 3D
    "StructuredMesh3D: elixir_euler_sedov.jl": dict(
        file="test/test_structured_3d.jl",
        elixir="examples/structured_3d_dgsem/elixir_euler_sedov.jl",
        mesh="structured", ndims=3, cells=[4, 4, 4], mapping="sedov_warp_3d", polydeg=3,
        ic="medium_sedov_3d", source="none", vi="hg", volume_flux="ranocha",
        volume_flux_fv="llf_naive", surface_flux="llf_naive", alpha_max=1.0, alpha_min=0.001,
        alpha_smooth=True, cfl=0.5, tspan=[0.0, 12.5]),
    "StructuredMesh3D: elixir_euler_source_terms.jl": dict(
        file="test/test_structured_3d.jl",
        elixir="examples/structured_3d_dgsem/elixir_euler_source_terms.jl",
        mesh="structured", ndims=3, cells=[4, 4, 4], mapping="cube_0_2_faces", polydeg=3,
        ic="convergence_test", source="convergence_test", vi="weak",
        volume_flux="central", surface_flux="llf_naive", cfl=0.6, tspan=[0.0, 5.0]),
    "StructuredMesh3D: elixir_euler_free_stream.jl": dict(
        file="test/test_structured_3d.jl",
        elixir="examples/structured_3d_dgsem/elixir_euler_free_stream.jl",
        mesh="structured", ndims=3, cells=[4, 4, 4], mapping="warped_cube_0_3", polydeg=3,
        ic="constant", source="none", vi="weak",
        volume_flux="central", surface_flux="llf_naive", cfl=1.3, tspan=[0.0, 1.0]),
    "StructuredMesh3D: elixir_euler_ec.jl": dict(
        file="test/test_structured_3d.jl",
        elixir="examples/structured_3d_dgsem/elixir_euler_ec.jl",
        mesh="structured", ndims=3, cells=[4, 4, 4], mapping="warped_cube_0_3", polydeg=5,
        gamma=5.0 / 3.0, ic="weak_blast_wave", source="none", vi="fluxdiff",
        volume_flux="ranocha", surface_flux="ranocha", cfl=1.0, tspan=[0.0, 2.0]),
    "StructuredMesh3D: elixir_euler_source_terms_nonperiodic_curved.jl": dict(
        file="test/test_structured_3d.jl",
        elixir="examples/structured_3d_dgsem/elixir_euler_source_terms_nonperiodic_curved.jl",
        mesh="structured", ndims=3, cells=[4, 4, 4], mapping="warped_cube_nonperiodic", polydeg=3,
        ic="convergence_test", source="convergence_test", vi="weak",
        volume_flux="central", surface_flux="llf_naive", cfl=0.6, tspan=[0.0, 5.0],
        boundary="dirichlet"),
    "CUDA 2D: elixir_euler_source_terms.jl native": dict(
        file="test/test_cuda_2d.jl",
        elixir="examples/p4est_2d_dgsem/elixir_euler_source_terms.jl",
        mesh="p4est", trees=[16, 16], level=0, mapping="square_0_2", polydeg=3,
        ic="convergence_test", source="convergence_test", vi="weak",
        volume_flux="central", surface_flux="llf_naive", cfl=1.0, tspan=[0.0, 2.0]),
    # the reference's own Float32 run on a GPU (storage_type = CuArray)
    "CUDA 2D: elixir_euler_source_terms.jl Float32 / CUDA": dict(
        file="test/test_cuda_2d.jl",
        elixir="examples/p4est_2d_dgsem/elixir_euler_source_terms.jl",
        mesh="p4est", trees=[16, 16], level=0, mapping="square_0_2", polydeg=3,
        ic="convergence_test", source="convergence_test", vi="weak",
        volume_flux="central", surface_flux="llf_naive", cfl=1.0, tspan=[0.0, 2.0],
        float32=True),
}

_NUM = r"[-+]?\d+(?:\.\d*)?(?:[eE][-+]?\d+)?"


def _testitem_body(text: str, name: str) -> tuple[str, int]:
    key = '@testitem "' + name + '"'
    start = text.find(key)
    if start < 0:
        raise KeyError(name)
    end = text.find("@testitem", start + len(key))
    line = text.count("\n", 0, start) + 1
    return text[start:end if end > 0 else len(text)], line


def _vector(body: str, key: str) -> list[float]:
    m = re.search(r"\b" + key + r"\s*=\s*(?:Float32)?\[([^\]]*)\]", body)
    if not m:
        raise KeyError(key)
    return [float(x) for x in re.findall(_NUM, m.group(1))]


def main(root: str) -> None:
    out = {}
    for name, case in CASES.items():
        text = open(os.path.join(root, case["file"]), encoding="utf-8").read()
        body, line = _testitem_body(text, name)
        entry = dict(case)
        entry["source_line"] = f"{case['file']}:{line}"
        entry["l2"] = _vector(body, "l2")
        entry["linf"] = _vector(body, "linf")
        m = re.search(r"tspan\s*=\s*\((" + _NUM + r"),\s*(" + _NUM + r")\)", body)
        if m:
            entry["tspan"] = [float(m.group(1)), float(m.group(2))]
        m = re.search(r"maxiters\s*=\s*(\d+)", body)
        if m:
            entry["maxiters"] = int(m.group(1))
        out[name] = entry
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "trixi_goldens.json")
    with open(dst, "w", encoding="utf-8") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    print(f"wrote {len(out)} goldens to {dst}")
    curved = {}
    for name, case in CURVED_CASES.items():
        text = open(os.path.join(root, case["file"]), encoding="utf-8").read()
        body, line = _testitem_body(text, name)
        entry = dict(case)
        entry["source_line"] = f"{case['file']}:{line}"
        entry["l2"] = _vector(body, "l2")
        entry["linf"] = _vector(body, "linf")
        m = re.search(r"tspan\s*=\s*\((" + _NUM + r")f?0?,\s*(" + _NUM + r")\)", body)
        if m:
            entry["tspan"] = [float(m.group(1)), float(m.group(2))]
        m = re.search(r"atol\s*=\s*(" + _NUM + r")", body)
        if m:
            entry["atol"] = float(m.group(1))
        curved[name] = entry
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "curved_goldens.json")
    with open(dst, "w", encoding="utf-8") as f:
        json.dump(curved, f, indent=1, sort_keys=True)
    print(f"wrote {len(curved)} curvilinear goldens to {dst}")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: extract_goldens.py <path of the Trixi.jl source tree>")
    main(sys.argv[1])
