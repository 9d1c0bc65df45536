"""GPU (sm_103a) parity of the fused DGSEM kernels against the oracle.

FP64 path: rhs!, the HG blending factors, the CFL step and whole time
integrations must match the oracle's restatement of Trixi to 1e-12 relative
(normwise per variable); conservation and free-stream preservation hold to
round-off.  Mixed path: FP32 bulk arithmetic, FP64 accumulation; its error
against the exact solution must stay within 1.1x of the FP64 path's error.
Every call goes through the C ABI (libtrixi_gb300.so).
"""
import numpy as np
import pytest

from _cases import load_goldens
from _gpu_cases import build, perturbed_state, rel_err
import trixi_gb300 as T

pytestmark = pytest.mark.gpu

RHS_CASES = [
    dict(ndims=2, polydeg=3, level=3, xmin=[0, 0], xmax=[2, 2], vi="weak", surface_flux="llf",
         ic="convergence_test", source="convergence_test"),
    dict(ndims=2, polydeg=3, level=3, xmin=[-1, -1], xmax=[1, 1], vi="fluxdiff",
         volume_flux="ranocha", surface_flux="llf_naive", ic="kelvin_helmholtz"),
    dict(ndims=2, polydeg=2, level=3, xmin=[-10, -10], xmax=[10, 10], vi="weak",
         surface_flux="llf_naive", ic="isentropic_vortex", ic_params=[1.0, 5.0]),
    dict(ndims=2, polydeg=4, level=2, xmin=[-2, -2], xmax=[2, 2], vi="fluxdiff",
         volume_flux="shima_etal", surface_flux="ranocha", ic="weak_blast_wave"),
    dict(ndims=2, polydeg=3, level=4, xmin=[-1, -1], xmax=[1, 1], vi="hg", volume_flux="ranocha",
         surface_flux="llf", ic="kelvin_helmholtz", alpha_max=0.002, alpha_min=0.0001),
    dict(ndims=2, polydeg=3, level=4, xmin=[-2, -2], xmax=[2, 2], vi="hg",
         volume_flux="shima_etal", surface_flux="llf_naive", ic="weak_blast_wave"),
    dict(ndims=3, polydeg=3, level=2, xmin=[0] * 3, xmax=[2] * 3, vi="fluxdiff",
         volume_flux="ranocha", surface_flux="llf", ic="convergence_test", source="convergence_test"),
    dict(ndims=3, polydeg=3, level=2, xmin=[0] * 3, xmax=[2] * 3, vi="weak", surface_flux="llf_naive",
         ic="convergence_test", source="convergence_test"),
    dict(ndims=3, polydeg=2, level=2, xmin=[-3.14159] * 3, xmax=[3.14159] * 3, vi="fluxdiff",
         volume_flux="ranocha", surface_flux="llf_naive", ic="taylor_green"),
    dict(ndims=3, polydeg=4, level=1, xmin=[-2] * 3, xmax=[2] * 3, vi="fluxdiff",
         volume_flux="central", surface_flux="ranocha", ic="weak_blast_wave"),
    dict(ndims=3, polydeg=3, level=2, xmin=[-2] * 3, xmax=[2] * 3, vi="hg", volume_flux="ranocha",
         surface_flux="llf_naive", ic="weak_blast_wave"),
]


def _id(c):
    return f"{c['ndims']}d-p{c['polydeg']}-{c['vi']}-{c.get('volume_flux', '')}-{c['surface_flux']}-{c['ic']}"


@pytest.mark.parametrize("c", RHS_CASES, ids=[_id(c) for c in RHS_CASES])
def test_rhs_fp64_matches_oracle(c):
    semi, orc = build(c)
    u = perturbed_state(semi, seed=3)
    du_gpu = semi.device_context.rhs_host(u, 0.37)
    du_orc = orc.rhs(u, 0.37)
    assert rel_err(du_gpu, du_orc) < 1e-12


@pytest.mark.parametrize("c", [c for c in RHS_CASES if c["vi"] == "hg"], ids=lambda c: _id(c))
def test_hg_alpha_fp64_matches_oracle(c):
    semi, orc = build(c)
    u = perturbed_state(semi, seed=5, amp=0.05)
    ctx = semi.device_context
    ctx.upload(u)
    a_gpu = ctx.alpha()
    a_orc = orc.alpha(u)
    assert np.max(np.abs(a_gpu - a_orc)) < 1e-12
    assert np.any(a_orc > 0)  # the case exercises the blending


@pytest.mark.parametrize("c", RHS_CASES[:7], ids=lambda c: _id(c))
def test_rhs_mixed_close_to_oracle(c):
    semi, orc = build(c, precision="mixed")
    u = perturbed_state(semi, seed=3)
    du_gpu = semi.device_context.rhs_host(u, 0.37)
    du_orc = orc.rhs(u, 0.37)
    assert rel_err(du_gpu, du_orc) < 2e-4


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("c", [RHS_CASES[1], RHS_CASES[4], RHS_CASES[8]], ids=lambda c: _id(c))
def test_conservation_to_roundoff(c, precision):
    # sum over the domain of w J du vanishes for periodic meshes without sources
    semi, _ = build(c, precision=precision)
    u = perturbed_state(semi, seed=7)
    du = semi.device_context.rhs_host(u, 0.0)
    b = semi.solver.basis
    D = semi.equations.ndims
    W = np.einsum("j,i->ji", b.weights, b.weights) if D == 2 else \
        np.einsum("k,j,i->kji", b.weights, b.weights, b.weights)
    J = (1.0 / semi.inverse_jacobian) ** D
    nv = du.shape[-1]
    wj = (J[:, None] * W.reshape(1, -1)).reshape(-1, 1)
    tot = np.sum(du.reshape(-1, nv) * wj, axis=0)
    scale = np.sum(np.abs(du.reshape(-1, nv)) * wj, axis=0)
    tol = 1e-13 if precision == "fp64" else 1e-6
    assert np.all(np.abs(tot) <= tol * scale)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("ndims,vi", [(2, "weak"), (2, "fluxdiff"), (3, "fluxdiff"), (2, "hg")])
def test_free_stream_preservation(ndims, vi, precision):
    c = dict(ndims=ndims, polydeg=3, level=2, xmin=[-1] * ndims, xmax=[1] * ndims, vi=vi,
             volume_flux="ranocha", surface_flux="llf", ic="constant")
    semi, _ = build(c, precision=precision)
    u = semi.compute_coefficients(0.0)
    du = semi.device_context.rhs_host(u, 0.0)
    assert np.max(np.abs(du)) < (1e-12 if precision == "fp64" else 1e-4)


def test_rhs_is_deterministic():
    semi, _ = build(RHS_CASES[6])
    u = perturbed_state(semi)
    a = semi.device_context.rhs_host(u, 0.1)
    b = semi.device_context.rhs_host(u, 0.1)
    assert np.array_equal(a, b)


@pytest.mark.parametrize("c", [RHS_CASES[0], RHS_CASES[4], RHS_CASES[6]], ids=lambda c: _id(c))
def test_max_dt_and_integrals_match_oracle(c):
    semi, orc = build(c)
    u = perturbed_state(semi, seed=11)
    ctx = semi.device_context
    ctx.upload(u)
    assert ctx.max_dt() == pytest.approx(orc.max_dt(u), rel=1e-14)
    np.testing.assert_allclose(ctx.integrals(), orc.integrals(u), rtol=1e-12)


@pytest.mark.parametrize("c", [RHS_CASES[0], RHS_CASES[4], RHS_CASES[6], RHS_CASES[10]],
                         ids=lambda c: _id(c))
def test_time_steps_fp64_match_oracle(c):
    semi, orc = build(c)
    u0 = perturbed_state(semi, seed=13, amp=1e-3)
    ctx = semi.device_context
    ctx.upload(u0)
    t, n = ctx.step(6, 0.9, 10.0, 0.0)
    u_gpu = ctx.download()
    u_orc, t_orc, n_orc = orc.solve(u0, 0.0, 10.0, 0.9, max_steps=6)
    assert n == n_orc == 6
    assert t == pytest.approx(t_orc, rel=1e-13)
    assert rel_err(u_gpu, u_orc) < 1e-12


def test_rk_stage_matches_oracle():
    c = RHS_CASES[6]
    semi, orc = build(c)
    u = perturbed_state(semi, seed=17)
    ctx = semi.device_context
    ctx.upload(u)
    u_o = u.copy()
    ut_o = np.zeros_like(u)
    for s in range(5):
        ctx.rk_stage(s, 0.2, 1e-3)
        orc.rk_stage(u_o, ut_o, s, 0.2, 1e-3)
    assert rel_err(ctx.download(), u_o) < 1e-13


GOLDENS = load_goldens()
# AMR goldens: test_gpu_amr.py; constant initial conditions (free stream): below
GOLDEN_NAMES = sorted(k for k in GOLDENS if "amr" not in GOLDENS[k]
                      and GOLDENS[k]["ic"] != "constant")
FREE_STREAM_GOLDENS = sorted(k for k in GOLDENS if GOLDENS[k]["ic"] == "constant")


def _golden_run(c):
    semi, _ = build(c)
    ode = T.semidiscretize(semi, c["tspan"])
    ana = T.AnalysisCallback(semi)
    sol = T.solve(ode, T.CarpenterKennedy2N54(williamson_condition=False), dt=1.0,
                  maxiters=c.get("maxiters", 10 ** 12),
                  callback=T.CallbackSet(T.StepsizeCallback(cfl=c["cfl"]), ana))
    return sol, ana


@pytest.mark.parametrize("name", GOLDEN_NAMES)
def test_gpu_fp64_reproduces_trixi_goldens(name):
    c = dict(GOLDENS[name])
    sol, ana = _golden_run(c)
    if "maxiters" in c:
        assert sol.nsteps == c["maxiters"]
    else:
        assert sol.t[-1] == pytest.approx(c["tspan"][1], rel=1e-14)
    np.testing.assert_allclose(ana.l2, c["l2"], rtol=1e-8)
    np.testing.assert_allclose(ana.linf, c["linf"], rtol=1e-7)


@pytest.mark.parametrize("name", FREE_STREAM_GOLDENS)
def test_gpu_free_stream_goldens(name):
    # the goldens are round-off (~1e-16): compare absolutely
    _, ana = _golden_run(dict(GOLDENS[name]))
    assert np.all(ana.l2 < 1e-14) and np.all(ana.linf < 1e-13)
    assert np.allclose(ana.l2, GOLDENS[name]["l2"], atol=5e-15, rtol=0)


# every golden with a smooth exact solution (errors against it measure accuracy)
@pytest.mark.parametrize("name", ["TreeMesh3D Euler: elixir_euler_source_terms.jl",
                                  "TreeMesh3D Euler: elixir_euler_source_terms.jl with split_form",
                                  "TreeMesh2D Euler: elixir_euler_source_terms.jl",
                                  "TreeMesh2D Euler: elixir_euler_source_terms_nonperiodic.jl",
                                  "TreeMesh2D Euler: elixir_euler_density_wave.jl",
                                  "TreeMesh3D Euler: elixir_euler_density_pulse.jl",
                                  "TreeMesh2D Euler: elixir_euler_vortex.jl"])
def test_mixed_precision_error_within_1p1x_of_fp64(name):
    c = dict(GOLDENS[name])
    errs = {}
    for prec in ("fp64", "mixed"):
        semi, _ = build(c, precision=prec)
        ana = T.AnalysisCallback(semi)
        T.solve(T.semidiscretize(semi, c["tspan"]), T.CarpenterKennedy2N54(), dt=1.0,
                callback=T.CallbackSet(T.StepsizeCallback(cfl=c["cfl"]), ana))
        errs[prec] = ana.l2
    assert errs["mixed"][0] <= 1.1 * errs["fp64"][0]


def test_status_flags_nonphysical_state():
    # failure detection: a negative density planted in the host input is
    # reported through the status word after one step, without faulting
    semi, _ = build(RHS_CASES[0])
    u = semi.compute_coefficients(0.0)
    u[3, 1, 1, 0] = -1.0
    ctx = semi.device_context
    ctx.upload(u)
    ctx.step(1, 0.5, 10.0, 0.0)
    assert ctx.status() != 0
    assert ctx.status() == 0  # reading clears it


def test_rhs_with_device_pointers():
    torch = pytest.importorskip("torch")
    semi, orc = build(RHS_CASES[6])
    u = perturbed_state(semi, seed=19)
    ud = torch.from_numpy(u).cuda()
    dud = torch.empty_like(ud)
    semi.rhs(dud, ud, 0.4)
    semi.device_context.synchronize()
    assert rel_err(dud.cpu().numpy(), orc.rhs(u, 0.4)) < 1e-12


@pytest.mark.parametrize("c", [RHS_CASES[0], RHS_CASES[4], RHS_CASES[6]], ids=lambda c: _id(c))
def test_entropy_timederivative_matches_oracle(c):
    semi, orc = build(c)
    u = perturbed_state(semi, seed=29)
    ctx = semi.device_context
    ctx.upload(u)
    ref = orc.entropy_timederivative(u, 0.3)
    got = ctx.entropy_timederivative(0.3)
    scale = abs(orc.integrals(u)[-2])  # total entropy, for the absolute tolerance
    assert abs(got - ref) <= 1e-12 * scale + 1e-10 * abs(ref)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("mixed", 1e-3)])
@pytest.mark.parametrize("ndims", [2, 3])
def test_entropy_conservative_scheme_produces_no_entropy(ndims, precision, tol):
    # flux_ranocha as volume and surface flux is entropy conservative on a
    # periodic mesh (elixir_euler_ec.jl): d/dt of the total entropy vanishes up
    # to rounding, while the LLF surface flux dissipates at the jumps.
    c = dict(ndims=ndims, polydeg=3, level=3 if ndims == 2 else 2, xmin=[-2.0] * ndims,
             xmax=[2.0] * ndims, vi="fluxdiff", volume_flux="ranocha", surface_flux="ranocha",
             ic="weak_blast_wave")
    semi, _ = build(c, precision=precision)
    semi_llf, _ = build(dict(c, surface_flux="llf"), precision=precision)
    u = perturbed_state(semi, seed=31, amp=0.02)  # opens jumps at the interfaces
    semi.device_context.upload(u)
    semi_llf.device_context.upload(u)
    ds = semi.device_context.entropy_timederivative(0.0)
    ds_llf = semi_llf.device_context.entropy_timederivative(0.0)
    assert ds_llf < 0
    assert abs(ds) <= tol * abs(ds_llf), (ds, ds_llf)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_autotune_keeps_state_and_steps_like_a_fixed_choice(precision):
    c = RHS_CASES[6]  # 3D, polydeg 3: kernels built for 2, 4 and 8 elements per block
    semi, _ = build(c, precision=precision)
    ctx = semi.device_context
    ctx.upload(perturbed_state(semi, seed=41))
    before = ctx.download()
    epb, ms = ctx.autotune(iters=3)
    assert epb in (2, 4, 8) and ms > 0 and ctx.elements_per_block() == epb
    np.testing.assert_array_equal(ctx.download(), before)
    ctx.step(3, 0.6, 10.0, 0.0)
    ref, _ = build(c, precision=precision, elements_per_block=epb)
    rctx = ref.device_context
    rctx.upload(perturbed_state(ref, seed=41))
    rctx.step(3, 0.6, 10.0, 0.0)
    np.testing.assert_array_equal(ctx.download(), rctx.download())


def test_mixed_pinned_and_pageable_transfers_agree():
    # page-locked buffers are converted in place by the device (no staging
    # copy); the result must be the same bits as through pageable memory
    torch = pytest.importorskip("torch")
    c = RHS_CASES[6]
    semi, _ = build(c, precision="mixed")
    ctx = semi.device_context
    u = perturbed_state(semi, seed=43)
    ctx.upload(u)
    ref = ctx.download()
    ctx.step(2, 0.6, 10.0, 0.0)
    ref_stepped = ctx.download()
    pin_in = torch.from_numpy(np.ascontiguousarray(u).reshape(-1)).pin_memory()
    pin_out = torch.empty_like(pin_in).pin_memory()
    ctx.upload(pin_in.data_ptr())
    ctx.download(pin_out.data_ptr())
    np.testing.assert_array_equal(pin_out.numpy().reshape(ref.shape), ref)
    ctx.step(2, 0.6, 10.0, 0.0)
    ctx.download(pin_out.data_ptr())
    np.testing.assert_array_equal(pin_out.numpy().reshape(ref.shape), ref_stepped)



BOUNDARY_CASES = [
    dict(ndims=2, polydeg=3, level=3, xmin=[0, 0], xmax=[2, 2], vi="weak", surface_flux="llf_naive",
         ic="convergence_test", source="convergence_test", boundary="dirichlet"),
    dict(ndims=2, polydeg=3, level=3, xmin=[-2, -2], xmax=[2, 2], vi="fluxdiff",
         volume_flux="ranocha", surface_flux="ranocha", ic="weak_blast_wave", boundary="slip_wall"),
    dict(ndims=2, polydeg=3, level=3, xmin=[-2, -2], xmax=[2, 2], vi="hg", volume_flux="ranocha",
         surface_flux="llf", ic="weak_blast_wave", boundary="slip_wall"),
    dict(ndims=2, polydeg=3, level=3, xmin=[-2, -2], xmax=[2, 2], vi="fluxdiff",
         volume_flux="ranocha", surface_flux="llf", ic="weak_blast_wave", boundary="dirichlet"),
    dict(ndims=3, polydeg=3, level=2, xmin=[0] * 3, xmax=[2] * 3, vi="fluxdiff",
         volume_flux="ranocha", surface_flux="llf", ic="convergence_test",
         source="convergence_test", boundary="dirichlet"),
    dict(ndims=3, polydeg=2, level=2, xmin=[-2] * 3, xmax=[2] * 3, vi="fluxdiff",
         volume_flux="ranocha", surface_flux="llf_naive", ic="weak_blast_wave", boundary="slip_wall"),
]


def _bid(c):
    return f"{c['ndims']}d-p{c['polydeg']}-{c['vi']}-{c['surface_flux']}-{c['boundary']}"


@pytest.mark.parametrize("c", BOUNDARY_CASES, ids=_bid)
def test_nonperiodic_rhs_fp64_matches_oracle(c):
    semi, orc = build(c)
    u = perturbed_state(semi, seed=47)
    np.testing.assert_array_less(rel_err(semi.device_context.rhs_host(u, 0.41), orc.rhs(u, 0.41)), 1e-12)


@pytest.mark.parametrize("c", BOUNDARY_CASES, ids=_bid)
def test_nonperiodic_rhs_mixed_close_to_oracle(c):
    semi, orc = build(c, precision="mixed")
    u = perturbed_state(semi, seed=47)
    assert rel_err(semi.device_context.rhs_host(u, 0.41), orc.rhs(u, 0.41)) < 2e-4


@pytest.mark.parametrize("c", BOUNDARY_CASES[:2], ids=_bid)
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_nonperiodic_steps_match_oracle(c, precision):
    semi, orc = build(c, precision=precision)
    u0 = semi.compute_coefficients(0.0)
    ctx = semi.device_context
    ctx.upload(u0)
    t, n = ctx.step(6, 0.5, 10.0, 0.0)
    ref, t_ref, n_ref = orc.solve(u0, 0.0, 10.0, 0.5, max_steps=6)
    assert n == n_ref == 6
    tol = 1e-12 if precision == "fp64" else 1e-5
    assert abs(t - t_ref) <= tol * t_ref
    assert rel_err(ctx.download(), ref) < tol


# the edges of the compiled polynomial degrees (2D polydeg 1..5, 3D 1..4)
EDGE_CASES = [
    dict(ndims=2, polydeg=1, level=3, xmin=[0, 0], xmax=[2, 2], vi="weak", surface_flux="llf",
         ic="convergence_test", source="convergence_test"),
    dict(ndims=2, polydeg=5, level=2, xmin=[-1, -1], xmax=[1, 1], vi="fluxdiff",
         volume_flux="ranocha", surface_flux="llf", ic="kelvin_helmholtz"),
    dict(ndims=2, polydeg=5, level=3, xmin=[-2, -2], xmax=[2, 2], vi="hg", volume_flux="shima_etal",
         surface_flux="llf_naive", ic="weak_blast_wave"),
    dict(ndims=3, polydeg=1, level=2, xmin=[0] * 3, xmax=[2] * 3, vi="fluxdiff",
         volume_flux="ranocha", surface_flux="llf", ic="convergence_test", source="convergence_test"),
    dict(ndims=3, polydeg=4, level=1, xmin=[0] * 3, xmax=[2] * 3, vi="weak", surface_flux="llf",
         ic="convergence_test", source="convergence_test"),
]


@pytest.mark.parametrize("c", EDGE_CASES, ids=[_id(c) for c in EDGE_CASES])
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("mixed", 2e-4)])
def test_rhs_edge_polydeg_matches_oracle(c, precision, tol):
    semi, orc = build(c, precision=precision)
    u = perturbed_state(semi, seed=53)
    assert rel_err(semi.device_context.rhs_host(u, 0.29), orc.rhs(u, 0.29)) < tol


# flux_hllc, flux_hlle (surface and FV subcell fluxes) and flux_chandrashekar
# (volume and surface flux), compressible_euler_{2,3}d.jl
MORE_FLUX_CASES = [
    dict(ndims=2, polydeg=3, level=3, xmin=[-10, -10], xmax=[10, 10], vi="weak",
         surface_flux="hllc", ic="isentropic_vortex_advected", ic_params=[25.0, 5.0]),
    dict(ndims=3, polydeg=3, level=2, xmin=[0] * 3, xmax=[2] * 3, vi="weak", surface_flux="hllc",
         ic="convergence_test", source="convergence_test"),
    dict(ndims=2, polydeg=3, level=4, xmin=[-2, -2], xmax=[2, 2], vi="hg", volume_flux="ranocha",
         surface_flux="hllc", ic="weak_blast_wave"),
    dict(ndims=3, polydeg=3, level=2, xmin=[-2] * 3, xmax=[2] * 3, vi="fluxdiff",
         volume_flux="ranocha", surface_flux="hllc", ic="weak_blast_wave"),
    dict(ndims=2, polydeg=3, level=3, xmin=[-10, -10], xmax=[10, 10], vi="weak",
         surface_flux="hllc", ic="isentropic_vortex_advected", ic_params=[25.0, 5.0],
         refinement_patches=[dict(type="box", coordinates_min=[0.0, -10.0],
                                  coordinates_max=[10.0, 10.0])]),
    # flux_chandrashekar volume flux, flux_hlle surface / FV flux
    dict(ndims=2, polydeg=3, level=3, xmin=[-1, -1], xmax=[1, 1], vi="fluxdiff",
         volume_flux="chandrashekar", surface_flux="hlle", ic="kelvin_helmholtz"),
    dict(ndims=3, polydeg=3, level=2, xmin=[0] * 3, xmax=[2] * 3, vi="fluxdiff",
         volume_flux="chandrashekar", surface_flux="chandrashekar", ic="convergence_test",
         source="convergence_test"),
    dict(ndims=2, polydeg=3, level=4, xmin=[-2, -2], xmax=[2, 2], vi="hg",
         volume_flux="chandrashekar", surface_flux="hlle", ic="weak_blast_wave"),
    dict(ndims=3, polydeg=2, level=2, xmin=[-2] * 3, xmax=[2] * 3, vi="weak", surface_flux="hlle",
         ic="weak_blast_wave", refinement_patches=[dict(type="box", coordinates_min=[-1.0] * 3,
                                                        coordinates_max=[1.0] * 3)]),
]


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("mixed", 2e-4)])
@pytest.mark.parametrize("c", MORE_FLUX_CASES,
                         ids=[_id(c) + ("-mortar" if c.get("refinement_patches") else "")
                              for c in MORE_FLUX_CASES])
def test_rhs_more_fluxes_match_oracle(c, precision, tol):
    semi, orc = build(c, precision=precision)
    u = perturbed_state(semi, seed=13, amp=0.05)
    du_gpu = semi.device_context.rhs_host(u, 0.41)
    du_orc = orc.rhs(u, 0.41)
    assert rel_err(du_gpu, du_orc) < tol


# shock capturing whose subcell (FV) flux is not the surface flux: the kernels
# compiled for a fixed surface flux serve only contexts whose subcell flux is
# that flux, so these run the instances that dispatch the fluxes at run time
FV_FLUX_CASES = [
    dict(ndims=2, polydeg=3, level=4, xmin=[-1, -1], xmax=[1, 1], vi="hg", volume_flux="ranocha",
         surface_flux="llf", fv_flux="llf_naive", ic="kelvin_helmholtz", alpha_max=0.5,
         alpha_min=0.0001),
    dict(ndims=2, polydeg=3, level=4, xmin=[-2, -2], xmax=[2, 2], vi="hg", volume_flux="ranocha",
         surface_flux="hllc", fv_flux="llf", ic="weak_blast_wave"),
    dict(ndims=3, polydeg=3, level=2, xmin=[-2] * 3, xmax=[2] * 3, vi="hg", volume_flux="ranocha",
         surface_flux="llf", fv_flux="hlle", ic="weak_blast_wave"),
]


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("mixed", 2e-4)])
@pytest.mark.parametrize("c", FV_FLUX_CASES, ids=[_id(c) + "-fv_" + c["fv_flux"] for c in FV_FLUX_CASES])
def test_rhs_subcell_flux_other_than_surface_flux(c, precision, tol):
    semi, orc = build(c, precision=precision)
    u = perturbed_state(semi, seed=17, amp=0.05)
    ctx = semi.device_context
    ctx.upload(u)
    assert np.any(ctx.alpha() > 0)  # the subcell fluxes take part
    du_gpu = ctx.rhs_host(u, 0.23)
    du_orc = orc.rhs(u, 0.23)
    assert rel_err(du_gpu, du_orc) < tol


def test_hllc_is_not_a_volume_flux():
    c = dict(ndims=2, polydeg=3, level=2, xmin=[-1, -1], xmax=[1, 1], vi="fluxdiff",
             volume_flux="hllc", surface_flux="llf", ic="weak_blast_wave")
    semi, _ = build(c)
    with pytest.raises(T.TrixiGB300Error):
        semi.device_context


# 3D mixed contexts with 2 elements per block (the default at polydeg 3
# without shock capturing) run the persistent kernel
# (bulk copies of the next element block while the current one computes); its
# phases are the per-block kernel's (4 elements per block), so both give the
# same bits
PERSISTENT_3D_CASES = [
    RHS_CASES[6], RHS_CASES[7], BOUNDARY_CASES[4],
    # faces of a given flux: slip walls, and mortars of a refined box
    dict(ndims=3, polydeg=3, level=2, xmin=[-2] * 3, xmax=[2] * 3, vi="fluxdiff",
         volume_flux="ranocha", surface_flux="llf", ic="weak_blast_wave", boundary="slip_wall"),
    dict(ndims=3, polydeg=3, level=2, xmin=[0] * 3, xmax=[2] * 3, vi="fluxdiff",
         volume_flux="ranocha", surface_flux="llf", ic="convergence_test", source="convergence_test",
         refinement_patches=[dict(type="box", coordinates_min=[0.5] * 3, coordinates_max=[1.5] * 3)]),
]


@pytest.mark.parametrize("c", PERSISTENT_3D_CASES,
                         ids=[_id(c) + ("-" + c["boundary"] if c.get("boundary") else "")
                              + ("-mortar" if c.get("refinement_patches") else "")
                              for c in PERSISTENT_3D_CASES])
def test_3d_persistent_kernel_equals_per_block_kernel(c):
    u0 = None
    out = {}
    for epb in (2, 4):
        semi, orc = build(c, precision="mixed", elements_per_block=epb)
        ctx = semi.device_context
        if u0 is None:
            u0 = perturbed_state(semi, seed=29)
        du = ctx.rhs_host(u0, 0.31)
        ctx.upload(u0)
        t, n = ctx.step(3, 0.6, 10.0, 0.0)
        out[epb] = (du, ctx.download(), t)
    assert ctx.elements_per_block() == 4
    np.testing.assert_array_equal(out[2][0], out[4][0])
    np.testing.assert_array_equal(out[2][1], out[4][1])
    assert out[2][2] == out[4][2]
    default, _ = build(c, precision="mixed")
    assert default.device_context.elements_per_block() == 2
    assert rel_err(out[2][0], orc.rhs(u0, 0.31)) < 2e-4
