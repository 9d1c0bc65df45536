"""AMR on the GPU (AMRCallback + ControllerThreeLevel on a TreeMesh).

The controller's indicator (tg_amr_indicator, FP64 for both precisions) and
the device solution transfer (tg_adapt_state) must match the oracle's
restatement of amr.jl / amr_dg2d.jl / amr_dg3d.jl, and a whole adaptive run
must reproduce Trixi's elixir_euler_blast_wave_amr.jl golden.
"""
import numpy as np
import pytest

from _cases import ic_id, load_goldens
from _gpu_cases import amr_callback, build
from oracle import oracle as O
import trixi_gb300 as T

pytestmark = pytest.mark.gpu

GOLDENS = load_goldens()
AMR_GOLDENS = sorted(k for k in GOLDENS if GOLDENS[k].get("amr"))


def _case(ndims, level, patches=()):
    return dict(ndims=ndims, polydeg=3, level=level, xmin=[-2.0] * ndims, xmax=[2.0] * ndims,
                vi="hg", volume_flux="ranocha", surface_flux="llf_naive", ic="weak_blast_wave",
                alpha_max=0.5, alpha_min=0.001, refinement_patches=list(patches))


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("mixed", 1e-10)])
@pytest.mark.parametrize("ndims", [2, 3])
def test_amr_indicator_matches_oracle(ndims, precision, tol):
    patch = dict(type="box", coordinates_min=[-1.0] * ndims, coordinates_max=[0.0] * ndims)
    semi, orc = build(_case(ndims, 4 if ndims == 2 else 2, [patch]), precision=precision)
    u = semi.compute_coefficients(0.0)
    ctx = semi.device_context
    ctx.upload(u)
    for amax, amin, smooth in [(0.5, 0.001, True), (0.2, 0.01, False)]:
        a_gpu = ctx.amr_indicator(amax, amin, smooth)
        o2 = O.Oracle(ndims, 3, 4 if ndims == 2 else 2,
                      [-2.0] * ndims, [2.0] * ndims, volume_integral=O.VI_SHOCKCAPTURING_HG,
                      alpha_max=amax, alpha_min=amin, alpha_smooth=smooth)
        o2.set_refinement([patch])
        a_orc = o2.alpha(u)
        assert np.any(a_orc > 0)
        assert np.max(np.abs(a_gpu - a_orc)) < tol
    # the indicator on density (the KHI AMR elixir's): against the oracle's controller
    o3 = O.Oracle(ndims, 3, 4 if ndims == 2 else 2, [-2.0] * ndims, [2.0] * ndims)
    o3.set_refinement([patch])
    o3.set_amr(alpha_max=1.0, alpha_min=0.0001, alpha_smooth=False, variable="density",
               base_level=1, med_level=0, med_threshold=0.0003, max_level=6, max_threshold=0.003)
    ind = T.IndicatorHennemannGassner(semi, alpha_max=1.0, alpha_min=0.0001, alpha_smooth=False,
                                      variable=T.density)
    ctrl = T.ControllerThreeLevel(semi, ind, base_level=1, med_level=0, med_threshold=0.0003,
                                  max_level=6, max_threshold=0.003)
    np.testing.assert_array_equal(ctrl(semi), o3.amr_lambda(u))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("ndims,level", [(2, 4), (3, 2)])
def test_adapt_state_matches_oracle(ndims, level, precision):
    rng = np.random.default_rng(5 + ndims)
    semi, orc = build(_case(ndims, level), precision=precision)
    u = semi.compute_coefficients(0.0)
    u = u * (1 + 0.01 * rng.uniform(-1, 1, u.shape))
    semi.device_context.upload(u)
    for step in range(5):
        lam = rng.choice([-1, 0, 1], size=semi.nelements, p=[0.5, 0.3, 0.2]).astype(np.int8)
        u_prev = semi.device_context.download()
        changed = semi.adapt(lam)
        ochanged, u_orc = orc.adapt_with(u_prev, lam)
        assert changed == ochanged
        if not changed:
            continue
        assert semi.nelements == orc.nelements
        np.testing.assert_array_equal(semi.mesh.element_levels(), orc.element_levels())
        u_gpu = semi.device_context.download()
        scale = np.abs(u_orc).max()
        assert np.max(np.abs(u_gpu - u_orc)) <= 1e-13 * scale
    # the adapted context runs: rhs on the adapted mesh against the oracle
    du = semi.device_context.rhs_host(u_orc, 0.1)
    du_orc = orc.rhs(u_orc, 0.1)
    err = np.max(np.abs(du - du_orc)) / np.abs(du_orc).max()
    assert err < (1e-12 if precision == "fp64" else 2e-4)


def _amr_run(name, precision):
    c = dict(GOLDENS[name])
    semi, _ = build(c, precision=precision)
    cb_amr = amr_callback(semi, c)
    ana = T.AnalysisCallback(semi)
    sol = T.solve(T.semidiscretize(semi, tuple(c["tspan"])), T.CarpenterKennedy2N54(), dt=1.0,
                  maxiters=c.get("maxiters", 10 ** 12),
                  callback=T.CallbackSet(ana, cb_amr, T.StepsizeCallback(cfl=c["cfl"])))
    return semi, sol, ana, cb_amr


@pytest.mark.parametrize("name", AMR_GOLDENS)
def test_gpu_fp64_reproduces_amr_goldens(name):
    c = GOLDENS[name]
    semi, sol, ana, cb = _amr_run(name, "fp64")
    np.testing.assert_allclose(ana.l2, c["l2"], rtol=1e-8)
    np.testing.assert_allclose(ana.linf, c["linf"], rtol=1e-7)
    # the same adaptive history as the oracle: steps, passes and final mesh
    from _cases import oracle_from_case
    orc = oracle_from_case(O, c)
    _, t, n = orc.solve_amr(ic_id(O, c["ic"]), c.get("ic_params"), c["tspan"][0],
                            c["tspan"][1], c["cfl"], max_steps=c.get("maxiters", 10 ** 9))
    assert sol.nsteps == n and sol.t[-1] == pytest.approx(t, rel=1e-14)
    k = c["amr"]["interval"]
    # at least one pass on the initial condition (more while it keeps changing
    # the mesh), then one after every `interval` steps unless the final time
    # was reached
    finished = t >= c["tspan"][1]
    assert cb.passes >= 1 + (n - 1) // k + (0 if finished or n % k else 1)
    np.testing.assert_array_equal(semi.mesh.element_levels(), orc.element_levels())


@pytest.mark.parametrize("name", AMR_GOLDENS)
def test_mixed_amr_goldens_within_1p1x_of_fp64(name):
    _, _, ana64, _ = _amr_run(name, "fp64")
    semi, _, ana, _ = _amr_run(name, "mixed")
    assert ana.l2[0] <= 1.1 * ana64.l2[0]
    assert semi.nelements > 0


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_indicator_max_matches_host(precision):
    # IndicatorMax(semi; variable) (indicators_3d.jl:239-259) on the device
    c = dict(ndims=3, polydeg=3, level=2, xmin=[-5.0] * 3, xmax=[5.0] * 3, vi="weak",
             surface_flux="llf_naive", ic="density_pulse")
    semi, _ = build(c, precision=precision)
    u = semi.compute_coefficients(0.0)
    ctx = semi.device_context
    ctx.upload(u)
    # float-float states hold ~48 bits: the mixed context's maxima agree to ~1e-14
    rtol = 1e-15 if precision == "fp64" else 1e-14
    rho_max = u[..., 0].reshape(semi.nelements, -1).max(axis=1)
    np.testing.assert_allclose(ctx.amr_indicator_max(1), rho_max, rtol=rtol, atol=0)
    dp = T.density_pressure(u, semi.equations).reshape(semi.nelements, -1).max(axis=1)
    np.testing.assert_allclose(ctx.amr_indicator_max(0), dp, rtol=1e-13, atol=0)
