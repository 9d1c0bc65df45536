"""Curvilinear 2D golden cases: meshes and mappings of the elixirs named in
tests/golden/curved_goldens.json, restated from
examples/structured_2d_dgsem/elixir_euler_{source_terms,source_terms_parallelogram,
source_terms_waving_flag,free_stream,ec}.jl and
examples/p4est_2d_dgsem/elixir_euler_source_terms.jl."""
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def load_curved_goldens():
    with open(os.path.join(HERE, "golden", "curved_goldens.json"), encoding="utf-8") as f:
        return json.load(f)


def _warped_square_0_3(xi_, eta_):
    # elixir_euler_free_stream.jl / elixir_euler_ec.jl: a warped [0, 3]^2
    xi = 1.5 * xi_ + 1.5
    eta = 1.5 * eta_ + 1.5
    y = eta + 3 / 8 * (np.cos(1.5 * np.pi * (2 * xi - 3) / 3) *
                       np.cos(0.5 * np.pi * (2 * eta - 3) / 3))
    x = xi + 3 / 8 * (np.cos(0.5 * np.pi * (2 * xi - 3) / 3) *
                      np.cos(2 * np.pi * (2 * y - 3) / 3))
    return x, y


def _parallelogram(xi, eta):
    # elixir_euler_source_terms_parallelogram.jl
    return xi + eta, eta


WAVING_FLAG_FACES = (
    # elixir_euler_source_terms_waving_flag.jl
    lambda s: (-1.0, s - 1.0),
    lambda s: (1.0, s + 1.0),
    lambda s: (s, -1.0 + np.sin(0.5 * np.pi * s)),
    lambda s: (s, 1.0 + np.sin(0.5 * np.pi * s)),
)


CUBE_0_2_FACES = (
    # elixir_euler_source_terms.jl (structured_3d_dgsem): the faces of [0, 2]^3
    lambda s, t: (0.0, s + 1.0, t + 1.0), lambda s, t: (2.0, s + 1.0, t + 1.0),
    lambda s, t: (s + 1.0, 0.0, t + 1.0), lambda s, t: (s + 1.0, 2.0, t + 1.0),
    lambda s, t: (s + 1.0, t + 1.0, 0.0), lambda s, t: (s + 1.0, t + 1.0, 2.0),
)


def _warp3(xi, eta, zeta, amp):
    y = eta + amp * (np.cos(1.5 * np.pi * (2 * xi - 3) / 3) * np.cos(0.5 * np.pi * (2 * eta - 3) / 3) *
                     np.cos(0.5 * np.pi * (2 * zeta - 3) / 3))
    x = xi + amp * (np.cos(0.5 * np.pi * (2 * xi - 3) / 3) * np.cos(2 * np.pi * (2 * y - 3) / 3) *
                    np.cos(0.5 * np.pi * (2 * zeta - 3) / 3))
    z = zeta + amp * (np.cos(0.5 * np.pi * (2 * x - 3) / 3) * np.cos(np.pi * (2 * y - 3) / 3) *
                      np.cos(0.5 * np.pi * (2 * zeta - 3) / 3))
    return x, y, z


def _warped_cube_0_3(xi_, eta_, zeta_):
    # elixir_euler_free_stream.jl / elixir_euler_ec.jl (structured_3d_dgsem)
    return _warp3(1.5 * xi_ + 1.5, 1.5 * eta_ + 1.5, 1.5 * zeta_ + 1.5, 3 / 8)


def _warped_cube_nonperiodic(xi, eta, zeta):
    # elixir_euler_source_terms_nonperiodic_curved.jl (structured_3d_dgsem)
    x, y, z = _warp3(xi, eta, zeta, 1 / 6)
    return x + 1, y + 1, z + 1


def _sedov_warp_3d(xi, eta, zeta):
    # elixir_euler_sedov.jl (structured_3d_dgsem)
    y = eta + 0.125 * (np.cos(1.5 * np.pi * xi) * np.cos(0.5 * np.pi * eta) *
                       np.cos(0.5 * np.pi * zeta))
    x = xi + 0.125 * (np.cos(0.5 * np.pi * xi) * np.cos(2 * np.pi * y) * np.cos(0.5 * np.pi * zeta))
    z = zeta + 0.125 * (np.cos(0.5 * np.pi * x) * np.cos(np.pi * y) * np.cos(0.5 * np.pi * zeta))
    return x, y, z


def _sedov_warp(xi, eta):
    # elixir_euler_sedov.jl (structured_2d_dgsem)
    y = eta + 0.125 * (np.cos(1.5 * np.pi * xi) * np.cos(0.5 * np.pi * eta))
    x = xi + 0.125 * (np.cos(0.5 * np.pi * xi) * np.cos(2 * np.pi * y))
    return x, y


def mapping_kwargs(name):
    if name == "square_m1_1":
        return dict(coordinates_min=(-1.0, -1.0), coordinates_max=(1.0, 1.0))
    if name == "sedov_warp":
        return dict(mapping=_sedov_warp)
    if name == "sedov_warp_3d":
        return dict(mapping=_sedov_warp_3d)
    if name == "cube_0_2_faces":
        return dict(faces=CUBE_0_2_FACES)
    if name == "warped_cube_0_3":
        return dict(mapping=_warped_cube_0_3)
    if name == "warped_cube_nonperiodic":
        return dict(mapping=_warped_cube_nonperiodic)
    if name == "square_0_2":
        return dict(coordinates_min=(0.0, 0.0), coordinates_max=(2.0, 2.0))
    if name == "parallelogram":
        return dict(mapping=_parallelogram)
    if name == "waving_flag":
        return dict(faces=WAVING_FLAG_FACES)
    if name == "warped_square_0_3":
        return dict(mapping=_warped_square_0_3)
    raise KeyError(name)


def curved_mesh(c, cells=None):
    """The mesh of a case (optionally with another number of cells per direction)."""
    from trixi_gb300.curved_mesh import P4estMesh, StructuredMesh, StructuredMesh3D
    kw = mapping_kwargs(c["mapping"])
    kw["periodicity"] = c.get("boundary") is None
    if c.get("ndims", 2) == 3:
        return StructuredMesh3D(tuple(cells or c["cells"]), **kw)
    if c["mesh"] == "structured":
        return StructuredMesh(tuple(cells or c["cells"]), **kw)
    return P4estMesh(tuple(cells or c["trees"]), polydeg=c["polydeg"],
                     initial_refinement_level=c.get("level", 0), **kw)


def curved_oracle(O, c, mesh):
    from trixi_gb300.basis import LobattoLegendreBasis
    vi = dict(weak=O.VI_WEAK, fluxdiff=O.VI_FLUXDIFF, hg=O.VI_SHOCKCAPTURING_HG)[c["vi"]]
    fl = dict(central=O.FLUX_CENTRAL, ranocha=O.FLUX_RANOCHA, shima_etal=O.FLUX_SHIMA_ETAL,
              llf=O.FLUX_LAX_FRIEDRICHS, llf_naive=O.FLUX_LAX_FRIEDRICHS_NAIVE,
              chandrashekar=O.FLUX_CHANDRASHEKAR)
    src = O.SRC_CONVERGENCE_TEST if c.get("source") == "convergence_test" else O.SRC_NONE
    X = mesh.node_coordinates(LobattoLegendreBasis(c["polydeg"]))
    cls = O.CurvedOracle3D if c.get("ndims", 2) == 3 else O.CurvedOracle
    orc = cls(c["polydeg"], X, mesh.neighbors(), c.get("gamma", 1.4), vi, fl[c["volume_flux"]],
              fl[c["surface_flux"]], src)
    if c["vi"] == "hg":
        orc.set_hg(c["alpha_max"], c["alpha_min"], c["alpha_smooth"], fl[c["volume_flux_fv"]])
    if c.get("boundary") == "dirichlet":
        orc.set_dirichlet(dict(convergence_test=O.IC_CONVERGENCE_TEST,
                               weak_blast_wave=O.IC_WEAK_BLAST_WAVE,
                               constant=O.IC_CONSTANT)[c["ic"]])
    return orc
