"""Batched ensemble (tg_ensemble_*): uneven 2D vortex instances advanced by one
persistent launch per stage must give each instance the same states, times and
step counts as stepping that instance alone through its own context."""
import numpy as np
import pytest

import trixi_gb300 as T

pytestmark = pytest.mark.gpu


def vortex_semi(level, polydeg, eps, precision="mixed", surface_flux=None, volume_integral=None):
    eq = T.CompressibleEulerEquations2D(1.4)
    solver = T.DGSEM(polydeg=polydeg, surface_flux=surface_flux or T.flux_lax_friedrichs,
                     volume_integral=volume_integral or T.VolumeIntegralWeakForm())
    mesh = T.TreeMesh((-10.0, -10.0), (10.0, 10.0), initial_refinement_level=level)
    ic = T.initial_condition_isentropic_vortex(1.0, eps)
    return T.SemidiscretizationHyperbolic(mesh, eq, ic, solver, precision=precision)


SPECS = [(2, 2), (3, 3), (2, 4), (3, 4), (4, 3), (2, 2), (4, 2)]


def make_semis(seed=20261204, **kw):
    rng = np.random.default_rng(seed)
    return [vortex_semi(level, p, float(rng.uniform(1.0, 5.0)), **kw) for level, p in SPECS]


def solo_run(semi, t_end, max_steps, cfl=1.0):
    c = semi.device_context
    c.upload(semi.compute_coefficients(0.0))
    t, n = c.step(max_steps, cfl, t_end, 0.0)
    return c.download(), t, n


@pytest.mark.parametrize("tpb", [120, 240])
def test_ensemble_matches_single_instances(tpb):
    semis = make_semis()
    ens = T.Ensemble(semis, threads_per_block=tpb)
    assert ens.threads_per_block == tpb
    ens.upload_initial()
    t, steps = ens.step(10 ** 6, 1.0, 1.5)
    assert np.all(t == 1.5)
    for i, s in enumerate(make_semis()):
        u_ref, t_ref, n_ref = solo_run(s, 1.5, 10 ** 6)
        assert steps[i] == n_ref and t[i] == t_ref
        u = ens.download(i)
        scale = np.max(np.abs(u_ref))
        assert np.max(np.abs(u - u_ref)) <= 1e-12 * scale, i
    # uneven instances take different numbers of steps
    assert len(set(steps.tolist())) > 1


def test_ensemble_max_steps_and_restart():
    semis = make_semis(seed=7)
    ens = T.Ensemble(semis)
    ens.upload_initial()
    t1, s1 = ens.step(3, 1.0, 100.0)
    assert np.all(s1 == 3) and np.all(t1 > 0)
    t2, s2 = ens.step(4, 1.0, 100.0)
    assert np.all(s2 == 4) and np.all(t2 > t1)
    for i, s in enumerate(make_semis(seed=7)):
        u_ref, t_ref, n_ref = solo_run(s, 100.0, 7)
        assert n_ref == 7 and abs(t2[i] - t_ref) <= 1e-14 * t_ref
        assert np.max(np.abs(ens.download(i) - u_ref)) <= 1e-12 * np.max(np.abs(u_ref))


def test_ensemble_close_to_fp64():
    semis = make_semis(seed=3)
    ens = T.Ensemble(semis)
    ens.upload_initial()
    t, _ = ens.step(10 ** 6, 1.0, 1.0)
    for i, s in enumerate(make_semis(seed=3, precision="fp64")):
        u64, t64, _ = solo_run(s, 1.0, 10 ** 6)
        assert t64 == t[i] == 1.0
        u = ens.download(i)
        assert np.max(np.abs(u - u64)) <= 1e-6 * np.max(np.abs(u64)), i


def test_ensemble_autotune_keeps_states():
    semis = make_semis(seed=11)
    ens = T.Ensemble(semis)
    ens.upload_initial()
    ens.step(2, 1.0, 100.0)
    before = [ens.download(i) for i in range(len(ens))]
    tpb, ms = ens.autotune(iters=5)
    assert tpb in (120, 240) and ms > 0 and ens.threads_per_block == tpb
    for i in range(len(ens)):
        assert np.array_equal(ens.download(i), before[i])
    t, s = ens.step(3, 1.0, 100.0)
    assert np.all(s == 3)
    for i, sm in enumerate(make_semis(seed=11)):
        u_ref, _, _ = solo_run(sm, 100.0, 5)
        assert np.max(np.abs(ens.download(i) - u_ref)) <= 1e-12 * np.max(np.abs(u_ref))


def test_ensemble_flux_differencing():
    semis = make_semis(seed=5, volume_integral=T.VolumeIntegralFluxDifferencing(T.flux_ranocha),
                       surface_flux=T.flux_ranocha)
    ens = T.Ensemble(semis)
    ens.upload_initial()
    t, steps = ens.step(6, 1.0, 100.0)
    for i, s in enumerate(make_semis(seed=5,
                                     volume_integral=T.VolumeIntegralFluxDifferencing(T.flux_ranocha),
                                     surface_flux=T.flux_ranocha)):
        u_ref, _, _ = solo_run(s, 100.0, 6)
        assert np.max(np.abs(ens.download(i) - u_ref)) <= 1e-12 * np.max(np.abs(u_ref))


def test_ensemble_rejects_unsupported():
    with pytest.raises(T.TrixiGB300Error):
        T.Ensemble([vortex_semi(2, 3, 5.0), vortex_semi(2, 5, 5.0)])  # polydeg 5
    with pytest.raises(T.TrixiGB300Error):
        T.Ensemble([vortex_semi(2, 3, 5.0), vortex_semi(2, 3, 5.0, surface_flux=T.flux_ranocha)])
    with pytest.raises(T.TrixiGB300Error):
        T.Ensemble([vortex_semi(2, 3, 5.0)], threads_per_block=128)


def test_ensemble_mixed_error_within_1p1x_of_fp64():
    # the 1.1x target on L2(rho) at t = 20 (the vortex is back at its start), for
    # instances of the C5a kind up to 32^2 elements: there the FP64 error
    # (1e-6 .. 1e-3) is far above the mixed path's rounding floor (~1e-8, see
    # the design notes for the 128^2 polydeg-4 instances, where it is not)
    specs = [(3, 2, 4.1), (4, 2, 2.3), (3, 3, 1.7), (4, 3, 3.6), (5, 3, 4.8), (4, 4, 2.9),
             (5, 4, 1.2)]
    semis = [vortex_semi(lv, p, eps) for lv, p, eps in specs]
    ens = T.Ensemble(semis)
    ens.upload_initial()
    t, _ = ens.step(10 ** 7, 1.0, 20.0)
    assert np.allclose(t, 20.0, rtol=1e-13)
    for i, ((lv, p, eps), semi) in enumerate(zip(specs, semis)):
        l2m = T.calc_error_norms(ens.download(i), 20.0, semi)[0][0]
        ref = vortex_semi(lv, p, eps, precision="fp64")
        u, tt, _ = solo_run(ref, 20.0, 10 ** 7)
        l2f = T.calc_error_norms(u, tt, ref)[0][0]
        assert l2m <= 1.1 * l2f, (lv, p, eps, l2m, l2f)
