"""Curvilinear meshes (2D StructuredMesh and P4estMesh bricks, 3D StructuredMesh) on
the GPU against the oracle and the goldens of Trixi.jl's StructuredMesh / P4estMesh
Euler tests."""
import numpy as np
import pytest

import trixi_gb300 as T
from _curved_cases import curved_mesh, curved_oracle, load_curved_goldens
from _gpu_cases import FLUX, perturbed_state, rel_err
from oracle import oracle as O

pytestmark = pytest.mark.gpu

GOLDENS = load_curved_goldens()
# the 2D goldens (the 3D ones below), shock capturing included
FP64_GOLDENS = sorted(k for k, v in GOLDENS.items()
                      if not v.get("float32") and v.get("ndims", 2) == 2)


def build(c, precision="fp64", cells=None):
    eq = (T.CompressibleEulerEquations3D if c.get("ndims", 2) == 3
          else T.CompressibleEulerEquations2D)(c.get("gamma", 1.4))
    basis = T.LobattoLegendreBasis(c["polydeg"])
    sflux = FLUX[c["surface_flux"]][0]
    if c["vi"] == "weak":
        vi = T.VolumeIntegralWeakForm()
    elif c["vi"] == "fluxdiff":
        vi = T.VolumeIntegralFluxDifferencing(FLUX[c["volume_flux"]][0])
    else:
        ind = T.IndicatorHennemannGassner(eq, basis, alpha_max=c["alpha_max"],
                                          alpha_min=c["alpha_min"], alpha_smooth=c["alpha_smooth"],
                                          variable=T.density_pressure)
        vi = T.VolumeIntegralShockCapturingHG(ind, volume_flux_dg=FLUX[c["volume_flux"]][0],
                                              volume_flux_fv=FLUX[c["volume_flux_fv"]][0])
    solver = T.DGSEM(basis, sflux, vi)
    mesh = curved_mesh(c, cells)
    ic = {"convergence_test": T.initial_condition_convergence_test,
          "weak_blast_wave": T.initial_condition_weak_blast_wave,
          "sedov_blast_wave": T.initial_condition_sedov_blast_wave,
          "medium_sedov_3d": T.initial_condition_medium_sedov_blast_wave,
          "constant": T.initial_condition_constant}[c["ic"]]
    src = T.source_terms_convergence_test if c.get("source") == "convergence_test" else None
    bcs = (T.BoundaryConditionDirichlet(ic) if c.get("boundary") == "dirichlet"
           else T.boundary_condition_periodic)
    semi = T.SemidiscretizationHyperbolic(mesh, eq, ic, solver, source_terms=src,
                                          boundary_conditions=bcs, precision=precision)
    return semi, curved_oracle(O, c, mesh)


def _case(name, **over):
    return dict(GOLDENS[name], **over)


PAR = "StructuredMesh2D: elixir_euler_source_terms_parallelogram.jl"
FLAG = "StructuredMesh2D: elixir_euler_source_terms_waving_flag.jl"
EC = "StructuredMesh2D: elixir_euler_ec.jl"
P4 = "CUDA 2D: elixir_euler_source_terms.jl native"
P4SC = "P4estMesh2D: elixir_euler_shockcapturing_ec.jl"
P4SC_CH = "P4estMesh2D: elixir_euler_shockcapturing_ec.jl (flux_chandrashekar)"
SEDOV = "StructuredMesh2D: elixir_euler_sedov.jl"
HG_FLAG = dict(vi="hg", volume_flux="ranocha", surface_flux="llf", volume_flux_fv="llf",
               alpha_max=0.5, alpha_min=0.001, alpha_smooth=True)
RHS_CASES = [
    _case(PAR),
    _case(FLAG),
    _case(EC),                                               # FD ranocha / ranocha, N = 5
    _case(EC, polydeg=3, volume_flux="shima_etal", surface_flux="llf"),
    _case(EC, polydeg=2, volume_flux="chandrashekar", surface_flux="llf_naive"),
    _case(EC, polydeg=3, volume_flux="central", surface_flux="central"),
    _case(FLAG, vi="fluxdiff", volume_flux="ranocha", surface_flux="llf"),
    _case(P4, mesh="p4est", trees=[6, 4], level=1, mapping="warped_square_0_3"),
    # Dirichlet faces on a curved boundary
    _case(FLAG, boundary="dirichlet"),
    _case(FLAG, boundary="dirichlet", vi="fluxdiff", volume_flux="ranocha", surface_flux="llf"),
    # shock capturing: the P4estMesh EC elixirs (ranocha / chandrashekar, FV
    # ranocha), Sedov on the warped square (FV llf_naive), a smooth state with
    # Dirichlet faces and an unsmoothed indicator
    _case(P4SC, trees=[4, 4], level=1),
    _case(P4SC_CH, trees=[3, 4], level=1),
    _case(SEDOV),
    _case(SEDOV, polydeg=3, alpha_smooth=False, volume_flux="shima_etal"),
    _case(FLAG, boundary="dirichlet", **HG_FLAG),
    # a subcell flux other than the surface flux (the run-time flux instances)
    _case(FLAG, boundary="dirichlet", **dict(HG_FLAG, volume_flux_fv="llf_naive")),
]


def _id(c):
    return (f"{c['mesh']}-{c['mapping']}-{c['vi']}-{c['volume_flux']}-{c['surface_flux']}"
            + (f"-fv_{c['volume_flux_fv']}" if c["vi"] == "hg" else "")
            + f"-p{c['polydeg']}" + ("-dirichlet" if c.get("boundary") else ""))


@pytest.mark.parametrize("c", RHS_CASES, ids=_id)
def test_curved_rhs_fp64_matches_oracle(c):
    semi, orc = build(c, cells=(12, 10) if c["mesh"] == "structured" else None)
    u = perturbed_state(semi, seed=5)
    np.testing.assert_array_less(rel_err(semi.device_context.rhs_host(u, 0.37), orc.rhs(u, 0.37)),
                                 1e-12)


@pytest.mark.parametrize("c", RHS_CASES, ids=_id)
def test_curved_rhs_mixed_close_to_oracle(c):
    # float-float state, FP32 deviation fluxes: the perturbed state's node
    # deviations are ~1e-2 of the state, FP32 rounds them to ~1e-9 relative and
    # the derivative operator amplifies that by |D| ~ N^2
    semi, orc = build(c, precision="mixed", cells=(12, 10) if c["mesh"] == "structured" else None)
    u = perturbed_state(semi, seed=5)
    assert rel_err(semi.device_context.rhs_host(u, 0.37), orc.rhs(u, 0.37)) < 2e-4


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_curved_max_dt_and_integrals(precision):
    c = _case(FLAG)
    semi, orc = build(c, precision, cells=(12, 10))
    u = perturbed_state(semi, seed=2)
    ctx = semi.device_context
    ctx.upload(u)
    tol = 1e-13 if precision == "fp64" else 1e-6
    assert ctx.max_dt() == pytest.approx(orc.max_dt(u), rel=tol)
    tot = ctx.integrals()
    w = semi.solver.basis.weights
    J = 1.0 / semi.inverse_jacobian
    ref = np.einsum("j,i,eji,ejiv->v", w, w, J, u)
    np.testing.assert_allclose(tot[:4], ref, rtol=1e-12 if precision == "fp64" else 1e-12)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_curved_time_steps_match_oracle(precision):
    c = _case(FLAG)
    semi, orc = build(c, precision, cells=(12, 10))
    u0 = semi.compute_coefficients(0.0)
    ctx = semi.device_context
    ctx.upload(u0)
    t, n = ctx.step(8, c["cfl"], 10.0, 0.0)
    u_orc, t_orc, n_orc = orc.solve(u0, 0.0, 10.0, c["cfl"], max_steps=8)
    assert n == n_orc == 8
    assert t == pytest.approx(t_orc, rel=1e-12 if precision == "fp64" else 1e-6)
    tol = 1e-12 if precision == "fp64" else 1e-7
    assert rel_err(ctx.download(), u_orc) < tol


def _golden_run(c, precision="fp64"):
    semi, _ = build(c, precision)
    ode = T.semidiscretize(semi, c["tspan"])
    ana = T.AnalysisCallback(semi)
    sol = T.solve(ode, T.CarpenterKennedy2N54(williamson_condition=False), dt=1.0,
                  callback=T.CallbackSet(T.StepsizeCallback(cfl=c["cfl"]), ana))
    return sol, ana


@pytest.mark.parametrize("name", FP64_GOLDENS)
def test_curved_gpu_fp64_reproduces_trixi_goldens(name):
    c = dict(GOLDENS[name])
    sol, ana = _golden_run(c)
    assert sol.t[-1] == pytest.approx(c["tspan"][1], rel=1e-14)
    if c["ic"] == "constant":
        atol = c.get("atol", 7e-13)
        np.testing.assert_allclose(ana.l2, c["l2"], rtol=0, atol=atol)
        np.testing.assert_allclose(ana.linf, c["linf"], rtol=0, atol=atol)
        return
    np.testing.assert_allclose(ana.l2, c["l2"], rtol=1e-8)
    np.testing.assert_allclose(ana.linf, c["linf"], rtol=1e-7)


@pytest.mark.parametrize("name", [PAR, FLAG, P4, "StructuredMesh2D: elixir_euler_source_terms.jl",
                                  "StructuredMesh2D: elixir_euler_source_terms_nonperiodic.jl"])
def test_curved_mixed_error_within_1p1x_of_fp64_golden(name):
    c = dict(GOLDENS[name])
    _, ana = _golden_run(c, "mixed")
    assert np.all(ana.l2 <= 1.1 * np.asarray(c["l2"]))
    assert np.all(ana.l2 >= 0.9 * np.asarray(c["l2"]))


def test_curved_mixed_free_stream():
    # the deviation form carries no reference flux: a free stream on the warped
    # mesh stays constant to round-off in mixed precision too
    c = dict(GOLDENS["StructuredMesh2D: elixir_euler_free_stream.jl"])
    _, ana = _golden_run(c, "mixed")
    assert np.all(ana.l2 < 1e-11) and np.all(ana.linf < 1e-10)


def test_curved_mixed_beats_reference_float32_gpu_run():
    # the reference's own Float32 run of this P4estMesh elixir on a GPU
    # (test_cuda_2d.jl) against the mixed path: float-float state and deviation
    # fluxes keep the FP64 discretization error
    c32 = GOLDENS["CUDA 2D: elixir_euler_source_terms.jl Float32 / CUDA"]
    c64 = GOLDENS[P4]
    _, ana = _golden_run(dict(c64), "mixed")
    assert np.all(ana.l2 < np.asarray(c32["l2"]))
    np.testing.assert_allclose(ana.l2, c64["l2"], rtol=1e-3)


HG_CASES = [c for c in RHS_CASES if c["vi"] == "hg"]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("c", HG_CASES, ids=_id)
def test_curved_hg_alpha_matches_oracle(c, precision):
    # IndicatorHennemannGassner on density_pressure with apply_smoothing! over
    # the curvilinear face neighbours; mixed: FP32 indicator on the state's
    # FP32 value (the logistic's slope turns its rounding into up to ~1e-3 of
    # alpha_max near the threshold)
    semi, orc = build(c, precision, cells=(12, 10) if c["mesh"] == "structured" else None)
    u = perturbed_state(semi, seed=5)
    ctx = semi.device_context
    ctx.upload(u)
    a_gpu, a_orc = ctx.alpha(), orc.alpha(u)
    assert np.any(a_orc > 0)
    tol = 1e-12 if precision == "fp64" else 1e-2 * c["alpha_max"]
    assert np.max(np.abs(a_gpu - a_orc)) < tol


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_curved_hg_time_steps_match_oracle(precision):
    c = _case(SEDOV)
    semi, orc = build(c, precision, cells=(12, 10))
    u0 = semi.compute_coefficients(0.0)
    ctx = semi.device_context
    ctx.upload(u0)
    t, n = ctx.step(8, c["cfl"], 10.0, 0.0)
    u_orc, t_orc, n_orc = orc.solve(u0, 0.0, 10.0, c["cfl"], max_steps=8)
    assert n == n_orc == 8
    assert t == pytest.approx(t_orc, rel=1e-12 if precision == "fp64" else 1e-5)
    assert rel_err(ctx.download(), u_orc) < (1e-12 if precision == "fp64" else 1e-5)


@pytest.mark.parametrize("name", [P4SC, SEDOV])
def test_curved_hg_mixed_golden(name):
    # shock capturing in mixed precision stays on the FP64 elixir's golden
    c = dict(GOLDENS[name])
    _, ana = _golden_run(c, "mixed")
    np.testing.assert_allclose(ana.l2, c["l2"], rtol=1e-3)


def test_curved_unsupported_options_fail_loudly():
    c = _case(EC)
    eq = T.CompressibleEulerEquations2D(1.4)
    basis = T.LobattoLegendreBasis(3)
    semi = T.SemidiscretizationHyperbolic(curved_mesh(c, (4, 4)), eq, T.initial_condition_constant,
                                          T.DGSEM(basis, T.flux_hllc))
    with pytest.raises(T.TrixiGB300Error):
        semi.device_context
    # slip walls are not built for curvilinear meshes
    semi = T.SemidiscretizationHyperbolic(curved_mesh(dict(c, boundary="dirichlet"), (4, 4)), eq,
                                          T.initial_condition_constant,
                                          T.DGSEM(basis, T.flux_lax_friedrichs),
                                          boundary_conditions=T.boundary_condition_slip_wall)
    with pytest.raises(T.TrixiGB300Error):
        semi.device_context


def test_curved_mixed_ec_golden():
    # flux_ranocha as volume and surface flux (the one-pass deviation form along
    # the normal) on the warped mesh, polydeg 4: the mixed run stays on the
    # golden of the FP64 elixir
    c = dict(GOLDENS[EC])
    _, ana = _golden_run(c, "mixed")
    np.testing.assert_allclose(ana.l2, c["l2"], rtol=1e-4)
    np.testing.assert_allclose(ana.linf, c["linf"], rtol=1e-3)



# ---- 3D curvilinear meshes (FP64) -------------------------------------------------
FREE3 = "StructuredMesh3D: elixir_euler_free_stream.jl"
EC3 = "StructuredMesh3D: elixir_euler_ec.jl"
NONP3 = "StructuredMesh3D: elixir_euler_source_terms_nonperiodic_curved.jl"
SRC3 = "StructuredMesh3D: elixir_euler_source_terms.jl"
# the 3D path runs the weak form and flux differencing at polydeg 3 and 5: every
# StructuredMesh3D golden (EC3 is flux_ranocha flux differencing at polydeg 5)
SEDOV3 = "StructuredMesh3D: elixir_euler_sedov.jl"
GOLDENS_3D = sorted(k for k, v in GOLDENS.items()
                    if v.get("ndims", 2) == 3 and v["polydeg"] in (3, 5))
RHS_CASES_3D = [
    (_case(FREE3, ic="convergence_test", source="convergence_test"), (4, 4, 4)),
    (_case(FREE3, ic="convergence_test", source="convergence_test", surface_flux="llf"), (4, 4, 4)),
    (_case(NONP3), (3, 2, 2)),                                  # Dirichlet faces
    (_case(FREE3, polydeg=5, ic="convergence_test", source="convergence_test"), (4, 4, 4)),
    # flux differencing: the EC elixir (ranocha / ranocha, polydeg 5, gamma 5/3)
    # and each two-point volume flux at polydeg 3
    (_case(EC3), (4, 4, 4)),
    (_case(EC3, polydeg=3, volume_flux="shima_etal", surface_flux="llf"), (4, 4, 4)),
    (_case(EC3, polydeg=3, volume_flux="chandrashekar", surface_flux="llf_naive"), (4, 4, 4)),
    (_case(EC3, polydeg=3, volume_flux="central", surface_flux="central"), (4, 4, 4)),
    (_case(NONP3, vi="fluxdiff", volume_flux="ranocha", surface_flux="llf"), (3, 2, 2)),
    # shock capturing: the Sedov elixir (ranocha / naive LLF FV) and another
    # flux set without smoothing
    (_case(SEDOV3), (4, 4, 4)),
    (_case(SEDOV3, volume_flux="shima_etal", surface_flux="llf", volume_flux_fv="llf",
           alpha_smooth=False), (3, 4, 2)),
]


@pytest.mark.parametrize("c,cells", RHS_CASES_3D, ids=lambda x: _id(x) if isinstance(x, dict) else "")
def test_curved3_rhs_fp64_matches_oracle(c, cells):
    # (the warped cube folds on meshes coarser than 4^3: cells keeps it valid)
    semi, orc = build(c, cells=cells)
    u = perturbed_state(semi, seed=7)
    np.testing.assert_array_less(rel_err(semi.device_context.rhs_host(u, 0.29), orc.rhs(u, 0.29)),
                                 1e-12)


def test_curved3_max_dt_integrals_and_steps():
    c = _case(NONP3)
    semi, orc = build(c, cells=(3, 2, 2))
    u0 = semi.compute_coefficients(0.0)
    ctx = semi.device_context
    ctx.upload(u0)
    assert ctx.max_dt() == pytest.approx(orc.max_dt(u0), rel=1e-13)
    w = semi.solver.basis.weights
    ref = np.einsum("k,j,i,ekji,ekjiv->v", w, w, w, 1.0 / semi.inverse_jacobian, u0)
    np.testing.assert_allclose(ctx.integrals()[:5], ref, rtol=1e-12)
    t, n = ctx.step(5, c["cfl"], 10.0, 0.0)
    u_orc, t_orc, n_orc = orc.solve(u0, 0.0, 10.0, c["cfl"], max_steps=5)
    assert n == n_orc == 5 and t == pytest.approx(t_orc, rel=1e-12)
    assert rel_err(ctx.download(), u_orc) < 1e-12


@pytest.mark.parametrize("name", GOLDENS_3D)
def test_curved3_gpu_fp64_reproduces_trixi_goldens(name):
    c = dict(GOLDENS[name])
    sol, ana = _golden_run(c)
    assert sol.t[-1] == pytest.approx(c["tspan"][1], rel=1e-14)
    if c["ic"] == "constant":
        np.testing.assert_allclose(ana.l2, c["l2"], rtol=0, atol=7e-13)
        return
    np.testing.assert_allclose(ana.l2, c["l2"], rtol=1e-8)
    np.testing.assert_allclose(ana.linf, c["linf"], rtol=1e-7)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_curved3_hg_alpha_and_steps_match_oracle(precision):
    c = _case(SEDOV3)
    semi, orc = build(c, precision, cells=(4, 4, 4))
    u0 = semi.compute_coefficients(0.0)
    ctx = semi.device_context
    ctx.upload(u0)
    a_orc = orc.alpha(u0)
    assert np.max(a_orc) > 0
    tol = 1e-12 if precision == "fp64" else 1e-2 * c["alpha_max"]
    assert np.max(np.abs(ctx.alpha() - a_orc)) < tol
    t, n = ctx.step(5, c["cfl"], 10.0, 0.0)
    u_orc, t_orc, n_orc = orc.solve(u0, 0.0, 10.0, c["cfl"], max_steps=5)
    assert n == n_orc == 5
    assert t == pytest.approx(t_orc, rel=1e-12 if precision == "fp64" else 1e-5)
    assert rel_err(ctx.download(), u_orc) < (1e-12 if precision == "fp64" else 1e-5)


def test_curved3_hg_mixed_golden():
    c = dict(GOLDENS[SEDOV3])
    _, ana = _golden_run(c, "mixed")
    np.testing.assert_allclose(ana.l2, c["l2"], rtol=1e-3)


def test_curved3_fd_steps_match_oracle():
    # five CK2N54 steps of the EC elixir through the fused stage kernel, with
    # the CFL reduction inside it
    c = _case(EC3)
    semi, orc = build(c, cells=(4, 4, 4))
    u0 = semi.compute_coefficients(0.0)
    ctx = semi.device_context
    ctx.upload(u0)
    t, n = ctx.step(5, c["cfl"], 10.0, 0.0)
    u_orc, t_orc, n_orc = orc.solve(u0, 0.0, 10.0, c["cfl"], max_steps=5)
    assert n == n_orc == 5 and t == pytest.approx(t_orc, rel=1e-12)
    assert rel_err(ctx.download(), u_orc) < 1e-12


def test_curved3_other_degrees_are_rejected():
    for precision in ("fp64", "mixed"):
        semi, _ = build(_case(EC3, polydeg=4), precision, cells=(2, 2, 2))
        with pytest.raises(T.TrixiGB300Error):
            semi.device_context


# ---- 3D curvilinear meshes, mixed precision ---------------------------------------
@pytest.mark.parametrize("c,cells", RHS_CASES_3D, ids=lambda x: _id(x) if isinstance(x, dict) else "")
def test_curved3_rhs_mixed_close_to_oracle(c, cells):
    # float-float state, FP32 deviation fluxes along the contravariant vectors
    semi, orc = build(c, "mixed", cells=cells)
    u = perturbed_state(semi, seed=7)
    assert rel_err(semi.device_context.rhs_host(u, 0.29), orc.rhs(u, 0.29)) < 2e-4


def test_curved3_mixed_max_dt_integrals_and_steps():
    c = _case(NONP3)
    semi, orc = build(c, "mixed", cells=(3, 2, 2))
    u0 = semi.compute_coefficients(0.0)
    ctx = semi.device_context
    ctx.upload(u0)
    assert ctx.max_dt() == pytest.approx(orc.max_dt(u0), rel=1e-6)
    w = semi.solver.basis.weights
    ref = np.einsum("k,j,i,ekji,ekjiv->v", w, w, w, 1.0 / semi.inverse_jacobian, u0)
    np.testing.assert_allclose(ctx.integrals()[:5], ref, rtol=1e-12)
    t, n = ctx.step(5, c["cfl"], 10.0, 0.0)
    u_orc, t_orc, n_orc = orc.solve(u0, 0.0, 10.0, c["cfl"], max_steps=5)
    assert n == n_orc == 5 and t == pytest.approx(t_orc, rel=1e-6)
    assert rel_err(ctx.download(), u_orc) < 1e-7


@pytest.mark.parametrize("name", [SRC3, NONP3])
def test_curved3_mixed_error_within_1p1x_of_fp64_golden(name):
    c = dict(GOLDENS[name])
    _, ana = _golden_run(c, "mixed")
    assert np.all(ana.l2 <= 1.1 * np.asarray(c["l2"]))
    assert np.all(ana.l2 >= 0.9 * np.asarray(c["l2"]))


def test_curved3_mixed_free_stream_and_ec_golden():
    # the deviation form carries no reference flux: the warped cube keeps a
    # free stream to round-off; the EC elixir stays on the FP64 golden
    _, ana = _golden_run(dict(GOLDENS[FREE3]), "mixed")
    assert np.all(ana.l2 < 1e-11) and np.all(ana.linf < 1e-10)
    c = dict(GOLDENS[EC3])
    _, ana = _golden_run(c, "mixed")
    np.testing.assert_allclose(ana.l2, c["l2"], rtol=1e-4)
    np.testing.assert_allclose(ana.linf, c["linf"], rtol=1e-3)
