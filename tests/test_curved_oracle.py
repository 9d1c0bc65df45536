"""Curvilinear 2D meshes on the CPU: the oracle against the goldens of Trixi.jl's
StructuredMesh and P4estMesh Euler tests, and the host mesh setup against the
oracle's metric terms."""
import numpy as np
import pytest

from _curved_cases import curved_mesh, curved_oracle, load_curved_goldens

GOLDENS = load_curved_goldens()
FP64_GOLDENS = sorted(k for k, v in GOLDENS.items() if not v.get("float32"))


def test_3d_host_metric_free_stream(oracle_mod):
    # the curl-form metric of the oracle on the warped 3D cube satisfies the
    # discrete metric identities: rhs(constant state) = 0 to round-off
    O = oracle_mod
    c = GOLDENS["StructuredMesh3D: elixir_euler_free_stream.jl"]
    orc = curved_oracle(O, c, curved_mesh(c, cells=(3, 2, 2)))
    u = orc.initial_condition(O.IC_CONSTANT)
    du = orc.rhs(u)
    assert np.max(np.abs(du)) < 1e-13 * np.max(np.abs(u)) * np.max(np.abs(orc.metric()[1]))


def _ic(O, name):
    return dict(constant=O.IC_CONSTANT, convergence_test=O.IC_CONVERGENCE_TEST,
                weak_blast_wave=O.IC_WEAK_BLAST_WAVE, sedov_blast_wave=O.IC_SEDOV_BLAST_WAVE,
                medium_sedov_3d=O.IC_MEDIUM_SEDOV_3D)[name]


@pytest.mark.parametrize("name", FP64_GOLDENS)
def test_curved_oracle_reproduces_trixi_golden(oracle_mod, name):
    O = oracle_mod
    c = GOLDENS[name]
    orc = curved_oracle(O, c, curved_mesh(c))
    ic = _ic(O, c["ic"])
    u0 = orc.initial_condition(ic, c["tspan"][0])
    u, t, _ = orc.solve(u0, c["tspan"][0], c["tspan"][1], c["cfl"])
    assert t == pytest.approx(c["tspan"][1], rel=1e-14)
    l2, linf = orc.error_norms(u, t, ic)
    if c["ic"] == "constant":
        # free-stream preservation on a warped mesh: round-off goldens, compared
        # with the test's own absolute tolerance
        np.testing.assert_allclose(l2, c["l2"], rtol=0, atol=c.get("atol", 7e-13))
        np.testing.assert_allclose(linf, c["linf"], rtol=0, atol=c.get("atol", 7e-13))
        return
    np.testing.assert_allclose(l2, c["l2"], rtol=1e-8, atol=0)
    np.testing.assert_allclose(linf, c["linf"], rtol=1e-7, atol=0)


def test_host_metric_terms_match_oracle(oracle_mod):
    from trixi_gb300.basis import LobattoLegendreBasis
    from trixi_gb300.curved_mesh import metric_terms
    c = GOLDENS["StructuredMesh2D: elixir_euler_ec.jl"]
    mesh = curved_mesh(c, cells=(8, 6))
    b = LobattoLegendreBasis(c["polydeg"])
    X = mesh.node_coordinates(b)
    orc = curved_oracle(oracle_mod, c, mesh)
    Ja, ij = orc.metric()
    Ja2, ij2 = metric_terms(X, b)
    np.testing.assert_allclose(Ja2, Ja, rtol=0, atol=1e-13)
    np.testing.assert_allclose(ij2, ij, rtol=1e-13)


def test_p4est_refined_trees_cover_the_structured_mesh():
    # a 4x4 brick refined twice and a 16x16 StructuredMesh of the same mapping
    # hold the same elements (the mapping is affine, so interpolation is exact)
    from trixi_gb300.basis import LobattoLegendreBasis
    from trixi_gb300.curved_mesh import P4estMesh, StructuredMesh
    b = LobattoLegendreBasis(3)
    kw = dict(coordinates_min=(0.0, 0.0), coordinates_max=(2.0, 2.0))
    s = StructuredMesh((16, 16), **kw).node_coordinates(b)
    p4 = P4estMesh((4, 4), polydeg=3, initial_refinement_level=2, **kw)
    p = p4.node_coordinates(b)
    key = lambda X: np.lexsort((np.round(X[:, 0, 0, 0], 9), np.round(X[:, 0, 0, 1], 9)))
    np.testing.assert_allclose(p[key(p)], s[key(s)], rtol=0, atol=1e-14)
    # Morton order inside the first tree: (0,0), (1,0), (0,1), (1,1), ...
    np.testing.assert_array_equal(p4.cells[:4], [[0, 0], [1, 0], [0, 1], [1, 1]])


def test_p4est_curved_interpolation_converges():
    # element nodes interpolated from the tree nodes approach the mapping as the
    # mesh polydeg grows (calc_node_coordinates!, dgsem_p4est/containers_2d.jl:41-89)
    from trixi_gb300.basis import LobattoLegendreBasis
    from trixi_gb300.curved_mesh import P4estMesh
    from _curved_cases import _warped_square_0_3
    b = LobattoLegendreBasis(3)
    errs = []
    for pd in (3, 5, 7):
        m = P4estMesh((2, 2), polydeg=pd, mapping=_warped_square_0_3, initial_refinement_level=2)
        b2 = LobattoLegendreBasis(max(pd, 3))
        X = m.node_coordinates(b2)
        mx, my = m.grid
        xi = -1 + (m.cells[:, 0, None, None] + 0.5 * (b2.nodes[None, None, :] + 1)) * 2 / mx
        eta = -1 + (m.cells[:, 1, None, None] + 0.5 * (b2.nodes[None, :, None] + 1)) * 2 / my
        xe, ye = _warped_square_0_3(*np.broadcast_arrays(xi, eta))
        errs.append(max(np.abs(X[..., 0] - xe).max(), np.abs(X[..., 1] - ye).max()))
    assert errs[0] > errs[1] > errs[2]
    assert errs[2] < errs[0] / 5


def test_curved_mesh_rejects_unsupported():
    from trixi_gb300.curved_mesh import P4estMesh, StructuredMesh
    nb = StructuredMesh((4, 3), (0.0, 0.0), (1.0, 1.0), periodicity=(False, True)).neighbors()
    assert (nb[:, 0] == -1).sum() == 3 and (nb[:, 1] == -1).sum() == 3 and nb[:, 2:].min() >= 0
    with pytest.raises(ValueError):
        P4estMesh((2, 2), polydeg=3)
    with pytest.raises(ValueError):
        P4estMesh((2, 2), polydeg=3, coordinates_min=(0.0, 0.0), coordinates_max=(1.0, 1.0),
                  initial_refinement_level=-1)


@pytest.mark.parametrize("level", [0, 2])
def test_p4est_warped_free_stream_rhs_vanishes(oracle_mod, level):
    # free-stream preservation on a refined, warped P4estMesh: the element nodes
    # are interpolated from the tree nodes, and the cross-product metric of the
    # interpolant satisfies the discrete metric identities, so rhs(constant) = 0
    # to round-off for the split form with flux_ranocha as well as the weak form
    O = oracle_mod
    from trixi_gb300.basis import LobattoLegendreBasis
    from trixi_gb300.curved_mesh import P4estMesh
    from _curved_cases import _warped_square_0_3
    m = P4estMesh((6, 4), polydeg=3, mapping=_warped_square_0_3, initial_refinement_level=level)
    X = m.node_coordinates(LobattoLegendreBasis(3))
    for vi, vf, sf in ((O.VI_WEAK, O.FLUX_CENTRAL, O.FLUX_LAX_FRIEDRICHS),
                       (O.VI_FLUXDIFF, O.FLUX_RANOCHA, O.FLUX_RANOCHA)):
        orc = O.CurvedOracle(3, X, m.neighbors(), 1.4, vi, vf, sf, O.SRC_NONE)
        u = orc.initial_condition(O.IC_CONSTANT)
        du = orc.rhs(u)
        assert np.max(np.abs(du)) < 1e-13 * np.max(np.abs(u)) * np.max(np.abs(orc.metric()[1]))


def test_curved_config_carries_metric_and_boundaries():
    # the tg_config of a curvilinear semidiscretization: mesh type, per-node
    # inverse Jacobian and contravariant vectors, interfaces only where a
    # neighbour exists, Dirichlet codes on the non-periodic edges
    import trixi_gb300 as T
    from trixi_gb300 import _lib
    from trixi_gb300.semidiscretization import make_config
    eq = T.CompressibleEulerEquations2D(1.4)
    solver = T.DGSEM(polydeg=3, surface_flux=T.flux_lax_friedrichs)
    for per, nif, codes in ((True, 2 * 12 * 10, [0, 0, 0, 0]),
                            ((False, True), 11 * 10 + 12 * 10, [1, 1, 0, 0])):
        mesh = T.StructuredMesh((12, 10), (0.0, 0.0), (1.0, 2.0), periodicity=per)
        bcs = (T.boundary_condition_periodic if per is True else
               dict(x_neg=T.BoundaryConditionDirichlet(T.initial_condition_convergence_test),
                    x_pos=T.BoundaryConditionDirichlet(T.initial_condition_convergence_test),
                    y_neg=T.boundary_condition_periodic, y_pos=T.boundary_condition_periodic))
        semi = T.SemidiscretizationHyperbolic(mesh, eq, T.initial_condition_convergence_test,
                                              solver, boundary_conditions=bcs)
        cfg, keep = make_config(semi, "mixed")
        assert cfg.mesh_type == _lib.TG_MESH_CURVED
        assert cfg.ninterfaces == nif
        assert list(cfg.boundary_conditions)[:4] == codes
        assert semi.inverse_jacobian.shape == (120, 4, 4)
        assert semi.contravariant_vectors.shape == (120, 4, 4, 2, 2)
        # affine map: Ja^1 = (dy/deta, 0) = (1/10 * 2 / 2, 0) per unit reference length
        np.testing.assert_allclose(semi.contravariant_vectors[..., 0, 0], 2.0 / 10 / 2, rtol=1e-13)
        np.testing.assert_allclose(semi.inverse_jacobian, 1.0 / ((1.0 / 12 / 2) * (2.0 / 10 / 2)),
                                   rtol=1e-12)


def test_host_metric_terms_3d_match_oracle(oracle_mod):
    # numpy curl-form metric (the host side a 3D curvilinear context would
    # pass) against the oracle's, on the warped cube
    from trixi_gb300.basis import LobattoLegendreBasis
    from trixi_gb300.curved_mesh import metric_terms_3d
    c = GOLDENS["StructuredMesh3D: elixir_euler_free_stream.jl"]
    mesh = curved_mesh(c, cells=(3, 2, 2))
    X = mesh.node_coordinates(LobattoLegendreBasis(c["polydeg"]))
    Ja, ij = curved_oracle(oracle_mod, c, mesh).metric()
    Ja2, ij2 = metric_terms_3d(X, LobattoLegendreBasis(c["polydeg"]))
    np.testing.assert_allclose(Ja2, Ja, rtol=0, atol=1e-13 * np.abs(Ja).max())
    np.testing.assert_allclose(ij2, ij, rtol=1e-12)


def test_amr_rejects_curvilinear_meshes():
    import trixi_gb300 as T
    semi = T.SemidiscretizationHyperbolic(
        T.StructuredMesh((4, 4), (0.0, 0.0), (1.0, 1.0)), T.CompressibleEulerEquations2D(1.4),
        T.initial_condition_constant, T.DGSEM(polydeg=3, surface_flux=T.flux_lax_friedrichs))
    with pytest.raises(NotImplementedError):
        T.AMRCallback(semi, None, interval=5)


def test_curved3_config_carries_metric_and_interfaces():
    import trixi_gb300 as T
    from trixi_gb300 import _lib
    from trixi_gb300.semidiscretization import make_config
    eq = T.CompressibleEulerEquations3D(1.4)
    solver = T.DGSEM(polydeg=3, surface_flux=T.flux_lax_friedrichs)
    mesh = T.StructuredMesh((3, 2, 2), (0.0, 0.0, 0.0), (3.0, 2.0, 1.0))
    assert isinstance(mesh, T.curved_mesh.StructuredMesh3D)
    semi = T.SemidiscretizationHyperbolic(mesh, eq, T.initial_condition_convergence_test, solver)
    cfg, keep = make_config(semi, "fp64")
    assert cfg.mesh_type == _lib.TG_MESH_CURVED and cfg.ndims == 3
    assert cfg.ninterfaces == 3 * 12
    assert semi.contravariant_vectors.shape == (12, 4, 4, 4, 3, 3)
    # affine box: Ja^1 = (dy/deta dz/dzeta, 0, 0) with cell sizes 1, 1, 0.5
    np.testing.assert_allclose(semi.contravariant_vectors[..., 0, 0], 0.5 * 0.25, rtol=1e-13)
    np.testing.assert_allclose(semi.inverse_jacobian, 1.0 / (0.5 * 0.5 * 0.25), rtol=1e-12)
