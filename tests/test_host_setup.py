"""Host-side setup of the GPU path (basis, TreeMesh containers, initial conditions,
error norms) against the oracle's independent restatement.  CPU only."""
import numpy as np
import pytest

import trixi_gb300 as T
from oracle import oracle as O


@pytest.mark.parametrize("polydeg", [1, 2, 3, 4, 5, 7])
def test_basis_matches_oracle(polydeg):
    b = T.LobattoLegendreBasis(polydeg)
    orc = O.Oracle(2, polydeg, 1, [0, 0], [1, 1])
    ob = orc.basis()
    for name in ("nodes", "weights", "inverse_weights"):
        np.testing.assert_allclose(getattr(b, name), ob[name], rtol=0, atol=1e-15)
    for name in ("derivative_matrix", "derivative_hat", "derivative_split",
                 "inverse_vandermonde_legendre"):
        np.testing.assert_allclose(getattr(b, name), ob[name], rtol=0, atol=2e-13)


def test_basis_sbp_properties():
    # Dsplit has a zero diagonal (dg_2d.jl:235-239); Dhat = -M^-1 D^T M
    for p in range(1, 8):
        b = T.LobattoLegendreBasis(p)
        assert np.max(np.abs(np.diag(b.derivative_split))) < 1e-12
        M = np.diag(b.weights)
        np.testing.assert_allclose(b.derivative_hat, -np.linalg.inv(M) @ b.derivative_matrix.T @ M,
                                   atol=1e-12)
        assert abs(b.weights.sum() - 2) < 1e-14


@pytest.mark.parametrize("ndims,level", [(2, 1), (2, 3), (3, 1), (3, 2)])
def test_treemesh_containers_match_oracle(ndims, level):
    xmin, xmax = [-1.0] * ndims, [3.0] * ndims
    mesh = T.TreeMesh(xmin, xmax, initial_refinement_level=level)
    eq = T.CompressibleEulerEquations2D(1.4) if ndims == 2 else T.CompressibleEulerEquations3D(1.4)
    semi = T.SemidiscretizationHyperbolic(mesh, eq, T.initial_condition_convergence_test,
                                          T.DGSEM(polydeg=3))
    orc = O.Oracle(ndims, 3, level, xmin, xmax)
    m = orc.mesh()
    np.testing.assert_array_equal(semi.neighbor_ids, m["neighbor_ids"])
    np.testing.assert_array_equal(semi.orientations, m["orientations"])
    np.testing.assert_array_equal(semi.inverse_jacobian, m["inverse_jacobian"])
    np.testing.assert_allclose(semi.node_coordinates, m["node_coordinates"], rtol=0, atol=1e-15)


def test_treemesh_morton_order_2d():
    # depth-first leaves with x fastest: the first four elements form the
    # lower-left 2x2 block (abstract_tree.jl:122-130)
    mesh = T.TreeMesh((0, 0), (4, 4), initial_refinement_level=2)
    c = mesh.cell_centers()
    np.testing.assert_allclose(c[:4], [[0.5, 0.5], [1.5, 0.5], [0.5, 1.5], [1.5, 1.5]])
    np.testing.assert_allclose(c[4], [2.5, 0.5])


@pytest.mark.parametrize("ndims,ic,oic", [
    (2, "convergence_test", O.IC_CONVERGENCE_TEST), (3, "convergence_test", O.IC_CONVERGENCE_TEST),
    (2, "weak_blast_wave", O.IC_WEAK_BLAST_WAVE), (3, "weak_blast_wave", O.IC_WEAK_BLAST_WAVE),
    (2, "khi", O.IC_KELVIN_HELMHOLTZ), (2, "vortex", O.IC_ISENTROPIC_VORTEX),
    (3, "tgv", O.IC_TAYLOR_GREEN), (2, "constant", O.IC_CONSTANT), (3, "constant", O.IC_CONSTANT),
    (2, "gauss", O.IC_GAUSSIAN_BLAST), (2, "blast", O.IC_BLAST_WAVE),
    (3, "pulse", O.IC_DENSITY_PULSE), (2, "vortex_advected", O.IC_ISENTROPIC_VORTEX_ADVECTED),
    (2, "sedov", O.IC_SEDOV_BLAST_WAVE)])
def test_initial_conditions_match_oracle(ndims, ic, oic):
    funcs = dict(convergence_test=(T.initial_condition_convergence_test, None),
                 weak_blast_wave=(T.initial_condition_weak_blast_wave, None),
                 khi=(T.initial_condition_kelvin_helmholtz_instability, None),
                 vortex=(T.initial_condition_isentropic_vortex(1.0, 5.0), [1.0, 5.0]),
                 tgv=(T.initial_condition_taylor_green_vortex(0.1), [0.1]),
                 constant=(T.initial_condition_constant, None),
                 gauss=(T.initial_condition_gaussian_blast(1e-5, 1.0, 0.25), [1e-5, 1.0, 0.25]),
                 blast=(T.initial_condition_blast_wave, None),
                 pulse=(T.initial_condition_density_pulse, None),
                 sedov=(T.initial_condition_sedov_blast_wave, None),
                 vortex_advected=(T.initial_condition_isentropic_vortex_advected(25.0, 5.0),
                                  [25.0, 5.0]))
    f, par = funcs[ic]
    xmin, xmax = [-1.5] * ndims, [1.5] * ndims
    eq = T.CompressibleEulerEquations2D(1.4) if ndims == 2 else T.CompressibleEulerEquations3D(1.4)
    semi = T.SemidiscretizationHyperbolic(T.TreeMesh(xmin, xmax, initial_refinement_level=2), eq, f,
                                          T.DGSEM(polydeg=3))
    orc = O.Oracle(ndims, 3, 2, xmin, xmax)
    t = 13.7 if ic == "vortex_advected" else 0.3  # the advected vortex wraps around
    np.testing.assert_allclose(semi.compute_coefficients(t), orc.initial_condition(oic, par, t),
                               rtol=1e-13, atol=1e-13)


def test_error_norms_match_oracle():
    eq = T.CompressibleEulerEquations3D(1.4)
    semi = T.SemidiscretizationHyperbolic(T.TreeMesh((0,) * 3, (2,) * 3, initial_refinement_level=2),
                                          eq, T.initial_condition_convergence_test, T.DGSEM(polydeg=3))
    orc = O.Oracle(3, 3, 2, [0] * 3, [2] * 3)
    rng = np.random.default_rng(1)
    u = semi.compute_coefficients(0.0) * (1 + 1e-3 * rng.standard_normal(semi.u_shape))
    l2, linf = T.calc_error_norms(u, 0.25, semi)
    ol2, olinf = orc.error_norms(u, 0.25, O.IC_CONVERGENCE_TEST)
    np.testing.assert_allclose(l2, ol2, rtol=1e-12)
    np.testing.assert_allclose(linf, olinf, rtol=1e-12)


@pytest.mark.parametrize("ndims,level", [(2, 2), (3, 1)])
def test_nonperiodic_treemesh_interfaces_match_oracle(ndims, level):
    # periodicity = false: faces at the domain edge have no interface
    xmin, xmax = [0.0] * ndims, [2.0] * ndims
    mesh = T.TreeMesh(xmin, xmax, initial_refinement_level=level, periodicity=False)
    eq = T.CompressibleEulerEquations2D(1.4) if ndims == 2 else T.CompressibleEulerEquations3D(1.4)
    semi = T.SemidiscretizationHyperbolic(mesh, eq, T.initial_condition_convergence_test,
                                          T.DGSEM(polydeg=3),
                                          boundary_conditions=T.boundary_condition_slip_wall)
    orc = O.Oracle(ndims, 3, level, xmin, xmax)
    orc.set_boundaries([O.BC_SLIP_WALL] * (2 * ndims))
    m = orc.mesh()
    np.testing.assert_array_equal(semi.neighbor_ids, m["neighbor_ids"])
    np.testing.assert_array_equal(semi.orientations, m["orientations"])
    M = 1 << level
    assert len(semi.neighbor_ids) == ndims * (M - 1) * M ** (ndims - 1)


def test_boundary_conditions_must_match_periodicity():
    eq = T.CompressibleEulerEquations2D(1.4)
    with pytest.raises(ValueError):
        T.SemidiscretizationHyperbolic(T.TreeMesh((0, 0), (1, 1), initial_refinement_level=1),
                                       eq, T.initial_condition_convergence_test, T.DGSEM(polydeg=3),
                                       boundary_conditions=T.boundary_condition_slip_wall)
    with pytest.raises(ValueError):
        T.SemidiscretizationHyperbolic(
            T.TreeMesh((0, 0), (1, 1), initial_refinement_level=1, periodicity=(True, False)),
            eq, T.initial_condition_convergence_test, T.DGSEM(polydeg=3),
            boundary_conditions=T.boundary_condition_slip_wall)


@pytest.mark.parametrize("polydeg", [1, 2, 3, 4, 5, 7])
def test_mortar_matrices_match_oracle(polydeg):
    m = T.MortarL2(T.LobattoLegendreBasis(polydeg))
    orc = O.Oracle(2, polydeg, 1, [0, 0], [1, 1])
    for mine, ref in zip((m.forward_upper, m.forward_lower, m.reverse_upper, m.reverse_lower),
                         orc.mortar_matrices()):
        np.testing.assert_allclose(mine, ref, rtol=0, atol=1e-14)
    # interpolation reproduces constants; the two reverse projections of a
    # constant flux add up to it
    for F in (m.forward_upper, m.forward_lower):
        np.testing.assert_allclose(F.sum(axis=1), 1.0, atol=1e-14)
    np.testing.assert_allclose((m.reverse_upper + m.reverse_lower).sum(axis=1), 1.0, atol=1e-14)


PATCH_CASES = [
    (2, 4, [-10.0] * 2, [10.0] * 2, [dict(type="box", coordinates_min=(0.0, -10.0),
                                          coordinates_max=(10.0, 10.0))]),
    (2, 3, [-32.0] * 2, [32.0] * 2, [dict(type="box", coordinates_min=(-40.0, -5.0),
                                          coordinates_max=(40.0, 5.0))] * 2),
    (2, 3, [-1.0] * 2, [1.0] * 2, [dict(type="sphere", center=(0.1, 0.2), radius=0.5),
                                   dict(type="sphere", center=(0.1, 0.2), radius=0.2)]),
    (3, 2, [0.0] * 3, [2.0] * 3, [dict(type="box", coordinates_min=(0.5,) * 3,
                                       coordinates_max=(1.5,) * 3)]),
    (3, 2, [-1.0] * 3, [1.0] * 3, [dict(type="sphere", center=(0.3, 0.0, 0.0), radius=0.4)] * 3),
]


@pytest.mark.parametrize("ndims,level,xmin,xmax,patches", PATCH_CASES)
def test_refined_treemesh_matches_oracle(ndims, level, xmin, xmax, patches):
    # refine_box!/refine_sphere! with 2:1 rebalancing, leaf order, interfaces,
    # mortars and per-element geometry (abstract_tree.jl, containers_{2,3}d.jl)
    mesh = T.TreeMesh(xmin, xmax, initial_refinement_level=level, refinement_patches=patches)
    eq = T.CompressibleEulerEquations2D(1.4) if ndims == 2 else T.CompressibleEulerEquations3D(1.4)
    semi = T.SemidiscretizationHyperbolic(mesh, eq, T.initial_condition_convergence_test,
                                          T.DGSEM(polydeg=3))
    orc = O.Oracle(ndims, 3, level, xmin, xmax)
    orc.set_refinement(patches)
    om = orc.mesh()
    assert semi.nelements == orc.nelements and not mesh.is_uniform
    np.testing.assert_array_equal(semi.neighbor_ids, om["neighbor_ids"])
    np.testing.assert_array_equal(semi.orientations, om["orientations"])
    ids, ls, orient = orc.mortars()
    assert ids.shape[0] > 0
    np.testing.assert_array_equal(semi.mortar_neighbor_ids, ids)
    np.testing.assert_array_equal(semi.mortar_large_sides, ls)
    np.testing.assert_array_equal(semi.mortar_orientations, orient)
    np.testing.assert_allclose(semi.inverse_jacobian, om["inverse_jacobian"], rtol=1e-15)
    np.testing.assert_allclose(semi.node_coordinates, om["node_coordinates"], rtol=0, atol=1e-13)
    # every element face is covered exactly once by an interface side, a mortar side
    # or (periodic mesh) nothing else
    E, D = semi.nelements, ndims
    cover = np.zeros((E, 2 * D), dtype=int)
    for (l, r), o in zip(semi.neighbor_ids, semi.orientations):
        cover[l - 1, 2 * (o - 1) + 1] += 1
        cover[r - 1, 2 * (o - 1)] += 1
    ns = 1 << (D - 1)
    for row, side, o in zip(ids, ls, orient):
        dl = 2 * (o - 1) + (1 if side == 1 else 0)
        for q in range(ns):
            cover[row[q] - 1, dl ^ 1] += 1
        cover[row[ns] - 1, dl] += 1
    assert np.all(cover == 1)


def test_refined_mesh_config_carries_mortars():
    from trixi_gb300.semidiscretization import make_config
    patches = [dict(type="box", coordinates_min=(0.5,) * 3, coordinates_max=(1.5,) * 3)]
    mesh = T.TreeMesh([0.0] * 3, [2.0] * 3, initial_refinement_level=2, refinement_patches=patches)
    semi = T.SemidiscretizationHyperbolic(mesh, T.CompressibleEulerEquations3D(1.4),
                                          T.initial_condition_convergence_test, T.DGSEM(polydeg=3),
                                          source_terms=T.source_terms_convergence_test)
    cfg, keep = make_config(semi)
    assert cfg.nmortars == 24 and cfg.ninterfaces == 300 and cfg.nelements == 120
    ids = np.ctypeslib.as_array(cfg.mortar_neighbor_ids, shape=(24 * 5,))
    np.testing.assert_array_equal(ids.reshape(24, 5), semi.mortar_neighbor_ids)
    n = 4
    fu = np.ctypeslib.as_array(cfg.mortar_forward_upper, shape=(n * n,)).reshape(n, n, order="F")
    np.testing.assert_array_equal(fu, semi.solver.mortar.forward_upper)
    # uniform meshes pass no mortars
    semi_u = T.SemidiscretizationHyperbolic(T.TreeMesh([0.0] * 2, [2.0] * 2, 2),
                                            T.CompressibleEulerEquations2D(1.4),
                                            T.initial_condition_convergence_test, T.DGSEM(polydeg=3))
    cfg_u, _ = make_config(semi_u)
    assert cfg_u.nmortars == 0


def test_refinement_patch_validation():
    with pytest.raises(ValueError):
        T.TreeMesh([0.0] * 2, [1.0] * 2, 2, refinement_patches=[dict(type="cone")])
    with pytest.raises(ValueError):
        T.TreeMesh([0.0] * 2, [1.0] * 2, 2,
                   refinement_patches=[dict(type="box", coordinates_min=(0.5, 0.5),
                                            coordinates_max=(0.2, 0.9))])
    m = T.TreeMesh([0.0] * 2, [1.0] * 2, 2,
                   refinement_patches=[dict(type="box", coordinates_min=(5.0, 5.0),
                                            coordinates_max=(6.0, 6.0))])
    assert m.nelements == 16 and m.is_uniform and m.element_length() == 0.25
