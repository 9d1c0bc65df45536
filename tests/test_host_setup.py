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
    (2, "gauss", O.IC_GAUSSIAN_BLAST)])
def test_initial_conditions_match_oracle(ndims, ic, oic):
    funcs = dict(convergence_test=(T.initial_condition_convergence_test, None),
                 weak_blast_wave=(T.initial_condition_weak_blast_wave, None),
                 khi=(T.initial_condition_kelvin_helmholtz_instability, None),
                 vortex=(T.initial_condition_isentropic_vortex(1.0, 5.0), [1.0, 5.0]),
                 tgv=(T.initial_condition_taylor_green_vortex(0.1), [0.1]),
                 constant=(T.initial_condition_constant, None),
                 gauss=(T.initial_condition_gaussian_blast(1e-5, 1.0, 0.25), [1e-5, 1.0, 0.25]))
    f, par = funcs[ic]
    xmin, xmax = [-1.5] * ndims, [1.5] * ndims
    eq = T.CompressibleEulerEquations2D(1.4) if ndims == 2 else T.CompressibleEulerEquations3D(1.4)
    semi = T.SemidiscretizationHyperbolic(T.TreeMesh(xmin, xmax, initial_refinement_level=2), eq, f,
                                          T.DGSEM(polydeg=3))
    orc = O.Oracle(ndims, 3, 2, xmin, xmax)
    np.testing.assert_allclose(semi.compute_coefficients(0.3), orc.initial_condition(oic, par, 0.3),
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
