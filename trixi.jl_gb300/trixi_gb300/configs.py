"""Runs of the benchmark configurations on the GB300 path, FP64 beside mixed.

    python -m trixi_gb300.configs --only c1,c3 --out results.json

  c1   2D isentropic vortex, 16^2 elements, polydeg 3, weak form, LLF, CFL 1, t = 20
       (examples/tree_2d_dgsem/elixir_euler_vortex.jl with p = 1): L2/Linf against
       the exact solution (the vortex is back at its start at t = 20).
  c3   2D Kelvin-Helmholtz instability, 256^2, polydeg 3, HG shock capturing on
       rho*p (alpha_max 0.002, alpha_min 1e-4), flux_ranocha / LLF, CFL 1.3,
       t = 3 (elixir_euler_kelvin_helmholtz_instability.jl): density error of
       FP64 and mixed against a 512^2 run, sampled on a uniform grid.
  c4   learned indicator: pairs harvested every 10 steps from the c3 run and a
       Gaussian blast (128^2), trained on the GPU, deployed at 512^2 with HG as
       fallback; alpha MAE, fallbacks, positivity and the L2 density
       difference to the plain-HG run, throughput against FP64 + HG.
  c5a  64 uneven vortices (8^2..128^2, polydeg 2..4, eps ~ U[1, 5], seed
       20261204) in one ensemble to t = 20, against FP64 instance by instance.
  c5b  3D Taylor-Green vortex, Ma 0.1, polydeg 3, flux_ranocha volume flux,
       naive LLF, CFL 1.4 (elixir_euler_taylor_green_vortex.jl): kinetic
       energy history of mixed against FP64 (32^3 to t = 20; 64^3 mixed to
       t = 20 and FP64 to t = 2); c5b_64: both to t = 20 at 64^3.
  c6   AMR: the medium blast wave of elixir_euler_blast_wave_amr.jl at initial
       level 8 (ControllerThreeLevel on HG, base 6, max 8, interval 5) to
       t = 0.5, FP64 and mixed: time stepping vs in AMR passes; and the elixir's
       own size (level 6, base 4, t = 1) in FP64.
  c7   mortars: 3D MMS 32^3 with the central box refined once, against the
       uniform 32^3 mesh, FP64 and mixed.
  c8   curvilinear meshes: the waving-flag StructuredMesh MMS (weak form) and a
       warped P4estMesh weak blast wave (flux differencing) at 512^2, the Sedov
       blast with shock capturing on a warped StructuredMesh at 512^2 and the
       3D warped-cube EC elixir at 32^3, FP64 and mixed.

The 3D manufactured solution at 32^3 is the headline case of bench.py.
Throughput is DOF-updates per second per RK stage (ndofs x 5 stages x steps /
seconds), with the device synchronised around each timed call.
"""
from __future__ import annotations

import argparse
import json
import math
import time

import numpy as np

import trixi_gb300 as T
from .learned import ShockIndicatorMLP


# ---------------------------------------------------------------------------
# helpers
def solve_timed(semi, t_end, cfl, max_steps=10 ** 9, u0=None):
    c = semi.device_context
    c.upload(semi.compute_coefficients(0.0) if u0 is None else u0)
    c.synchronize()
    t0 = time.perf_counter()
    t, n = c.step(max_steps, cfl, t_end, 0.0)
    c.synchronize()
    secs = time.perf_counter() - t0
    return c.download(), t, n, secs


def rate(ndofs, steps, secs):
    return float(ndofs) * 5 * steps / secs if secs > 0 else float("nan")


def lagrange(nodes, x):
    """Lagrange basis of `nodes` at points x: (len(x), n)."""
    n = len(nodes)
    out = np.ones((len(x), n))
    for i in range(n):
        for k in range(n):
            if k != i:
                out[:, i] *= (x - nodes[k]) / (nodes[i] - nodes[k])
    return out


def sample2d(semi, u, npts, var=0, chunk=1 << 17):
    """Values of variable `var` of a 2D DG solution at the centres of an
    npts x npts grid over the domain (row-major in y)."""
    xc = semi.node_coordinates  # (E, j, i, 2)
    lo = xc.reshape(-1, 2).min(axis=0)
    hi = xc.reshape(-1, 2).max(axis=0)
    cen = xc.mean(axis=(1, 2))
    dx = (hi - lo) / np.round((hi - lo) / (xc[0, 0, -1, 0] - xc[0, 0, 0, 0]))
    nel = np.round((hi - lo) / dx).astype(int)
    ij = np.floor((cen - lo) / dx).astype(int)
    lookup = np.empty((nel[1], nel[0]), dtype=np.int64)
    lookup[ij[:, 1], ij[:, 0]] = np.arange(len(cen))
    nodes = np.asarray(semi.solver.basis.nodes)
    g = lo[None, :] + (np.arange(npts)[:, None] + 0.5) * (hi - lo)[None, :] / npts
    X, Y = np.meshgrid(g[:, 0], g[:, 1])
    P = np.stack([X.ravel(), Y.ravel()], axis=1)
    out = np.empty(len(P))
    for s in range(0, len(P), chunk):
        p = P[s:s + chunk]
        k = np.clip(np.floor((p - lo) / dx).astype(int), 0, nel - 1)
        e = lookup[k[:, 1], k[:, 0]]
        loc = 2 * (p - (lo + k * dx)) / dx - 1
        lx, ly = lagrange(nodes, loc[:, 0]), lagrange(nodes, loc[:, 1])
        out[s:s + chunk] = np.einsum("mji,mi,mj->m", u[e, :, :, var], lx, ly)
    return out


def vortex_semi(level, polydeg, eps, precision, surface_flux=None):
    eq = T.CompressibleEulerEquations2D(1.4)
    solver = T.DGSEM(polydeg=polydeg, surface_flux=surface_flux or T.flux_lax_friedrichs,
                     volume_integral=T.VolumeIntegralWeakForm())
    mesh = T.TreeMesh((-10.0, -10.0), (10.0, 10.0), initial_refinement_level=level)
    ic = T.initial_condition_isentropic_vortex(1.0, eps)
    return T.SemidiscretizationHyperbolic(mesh, eq, ic, solver, precision=precision)


def khi_semi(level, precision, elements_per_block=0):
    eq = T.CompressibleEulerEquations2D(1.4)
    basis = T.LobattoLegendreBasis(3)
    ind = T.IndicatorHennemannGassner(eq, basis, alpha_max=0.002, alpha_min=0.0001,
                                      alpha_smooth=True, variable=T.density_pressure)
    vi = T.VolumeIntegralShockCapturingHG(ind, volume_flux_dg=T.flux_ranocha,
                                          volume_flux_fv=T.flux_lax_friedrichs)
    solver = T.DGSEM(basis, T.flux_lax_friedrichs, vi)
    mesh = T.TreeMesh((-1.0, -1.0), (1.0, 1.0), initial_refinement_level=level)
    return T.SemidiscretizationHyperbolic(mesh, eq, T.initial_condition_kelvin_helmholtz_instability,
                                          solver, precision=precision,
                                          elements_per_block=elements_per_block)


def blast_semi(level, precision):
    eq = T.CompressibleEulerEquations2D(1.4)
    basis = T.LobattoLegendreBasis(3)
    ind = T.IndicatorHennemannGassner(eq, basis, alpha_max=0.5, alpha_min=0.001,
                                      alpha_smooth=True, variable=T.density_pressure)
    vi = T.VolumeIntegralShockCapturingHG(ind, volume_flux_dg=T.flux_ranocha,
                                          volume_flux_fv=T.flux_lax_friedrichs)
    solver = T.DGSEM(basis, T.flux_lax_friedrichs, vi)
    mesh = T.TreeMesh((-1.5, -1.5), (1.5, 1.5), initial_refinement_level=level)
    ic = T.initial_condition_gaussian_blast(1e-5, 1.0, 0.25)
    return T.SemidiscretizationHyperbolic(mesh, eq, ic, solver, precision=precision)


def tgv_semi(level, precision):
    eq = T.CompressibleEulerEquations3D(1.4)
    solver = T.DGSEM(polydeg=3, surface_flux=T.FluxLaxFriedrichs(T.max_abs_speed_naive),
                     volume_integral=T.VolumeIntegralFluxDifferencing(T.flux_ranocha))
    mesh = T.TreeMesh((-math.pi,) * 3, (math.pi,) * 3, initial_refinement_level=level)
    return T.SemidiscretizationHyperbolic(mesh, eq, T.initial_condition_taylor_green_vortex(0.1),
                                          solver, precision=precision)


# ---------------------------------------------------------------------------
def c1():
    out = {}
    for prec in ("fp64", "mixed"):
        semi = vortex_semi(4, 3, 5.0, prec)
        u, t, n, secs = solve_timed(semi, 20.0, 1.0)
        l2, linf = T.calc_error_norms(u, t, semi)
        out[prec] = dict(l2=l2.tolist(), linf=linf.tolist(), t=t, steps=n, secs=secs,
                         rate=rate(semi.ndofs, n, secs))
    out["l2_rho_ratio"] = out["mixed"]["l2"][0] / out["fp64"]["l2"][0]
    out["linf_rho_ratio"] = out["mixed"]["linf"][0] / out["fp64"]["linf"][0]
    out["speedup"] = out["mixed"]["rate"] / out["fp64"]["rate"]
    return out


def c3(npts=1024):
    out = {}
    sol = {}
    for prec, level in (("fp64", 8), ("mixed", 8), ("mixed_512", 9)):
        semi = khi_semi(level, "mixed" if prec == "mixed_512" else prec)
        u, t, n, secs = solve_timed(semi, 3.0, 1.3)
        sol[prec] = sample2d(semi, u, npts)
        out[prec] = dict(t=t, steps=n, secs=secs, rate=rate(semi.ndofs, n, secs))
        del semi
    truth = sol["mixed_512"]

    def rms(a):
        return float(np.sqrt(np.mean(a * a)))

    for prec in ("fp64", "mixed"):
        out[prec]["l2_rho_vs_512"] = rms(sol[prec] - truth)
        out[prec]["linf_rho_vs_512"] = float(np.max(np.abs(sol[prec] - truth)))
    out["l2_rho_ratio"] = out["mixed"]["l2_rho_vs_512"] / out["fp64"]["l2_rho_vs_512"]
    out["l2_rho_mixed_vs_fp64"] = rms(sol["mixed"] - sol["fp64"])
    out["speedup"] = out["mixed"]["rate"] / out["fp64"]["rate"]
    out["sample_grid"] = npts
    return out


def _clip_alpha(a, alpha_min, alpha_max):
    a = np.where(a < alpha_min, 0.0, a)
    a = np.where(a > 1 - alpha_min, 1.0, a)
    return np.minimum(alpha_max, a)


def harvest_and_train(net, every=10, khi_level=8, khi_t_end=3.0, khi_stride=16,
                      blast_level=7, blast_t_end=0.3, blast_stride=4, train_steps=4000,
                      batch=4096, lr=2e-3):
    """Training set and training of the learned indicator: (modes, sqrt E) pairs of
    every `*_stride`-th element, harvested every `every` steps from the KHI run
    (256^2, t = 3, CFL 1.3) and the Gaussian blast (128^2, t = 0.3, CFL 1), both
    mixed precision with the plain HG indicator; then Adam on the GPU: 50 and
    `train_steps` steps at `lr`, and `train_steps` / 4 at lr / 10 (training is
    reproducible bit for bit).  Returns the statistics of both phases."""
    out = {}
    t_start = time.perf_counter()
    for name, semi, t_end, stride in (
            (f"khi_{2 ** khi_level}", khi_semi(khi_level, "mixed"), khi_t_end, khi_stride),
            (f"blast_{2 ** blast_level}", blast_semi(blast_level, "mixed"), blast_t_end,
             blast_stride)):
        c = semi.device_context
        c.upload(semi.compute_coefficients(0.0))
        t, steps, k = 0.0, 0, 0
        cfl = 1.3 if name.startswith("khi") else 1.0
        while True:
            t, n = c.step(every, cfl, t_end, t)
            steps += n
            net.harvest(semi, stride=stride, phase=k % stride)
            k += 1
            if n < every or t >= t_end:
                break
        out[f"harvest_{name}"] = dict(t=t, steps=steps, pairs_total=net.count, stride=stride)
        del semi
    out["harvest_secs"] = time.perf_counter() - t_start
    t0 = time.perf_counter()
    first = net.train(50, batch=batch, lr=lr)
    net.train(train_steps, batch=batch, lr=lr)
    # a last quarter at a tenth of the rate settles the weights
    last = net.train(train_steps // 4, batch=batch, lr=0.1 * lr)
    out["train"] = dict(pairs=net.count, steps=50 + train_steps + train_steps // 4,
                        loss_first=first, loss_last=last, secs=time.perf_counter() - t0)
    x, y = net.dataset()
    held = np.arange(len(y)) % 10 == 0
    pred = np.maximum(net.predict(x[held]), 0.0)  # as deployed: sqrt E >= 0
    yh, yt = y[held], y[~held]
    tr = out["train"]
    # the objective (mean squared error of sqrt E) against the best constant, its mean
    tr["heldout_rmse_sqrtE"] = float(np.sqrt(np.mean((pred - yh) ** 2)))
    tr["heldout_rmse_const"] = float(np.sqrt(np.mean((np.mean(yt) - yh) ** 2)))
    tr["heldout_mae_sqrtE"] = float(np.mean(np.abs(pred - yh)))
    tr["heldout_mae_const"] = float(np.mean(np.abs(np.median(yt) - yh)))
    # the decision that matters: alpha switched on (E above the HG threshold)
    sqrt_thr = math.sqrt(0.5 * 10 ** (-1.8 * (net.polydeg + 1) ** 0.25))
    tr["heldout_on_off_agreement"] = float(np.mean((pred > sqrt_thr) == (yh > sqrt_thr)))
    tr["heldout_fraction_on"] = float(np.mean(yh > sqrt_thr))
    return out


def c4(harvest_every=10, train_steps=4000, deploy_level=9, fp64_steps=200):
    """Learned indicator: harvest, train, deploy against HG."""
    net = ShockIndicatorMLP(2, 3, seed=3)
    out = harvest_and_train(net, every=harvest_every, train_steps=train_steps)

    # deployment at 512^2: mixed + learned vs mixed + HG (same states), FP64 + HG throughput
    thr = 0.5 * 10 ** (-1.8 * 4 ** 0.25)
    s_par = math.log((1 - 0.0001) / 0.0001)
    res = {}
    mae = []
    for name in ("hg", "learned"):
        semi = khi_semi(deploy_level, "mixed")
        c = semi.device_context
        c.upload(semi.compute_coefficients(0.0))
        if name == "learned":
            net.deploy(semi, band=0.01)
        c.synchronize()
        t, steps, secs = 0.0, 0, 0.0
        for t_stop in (0.5, 1.0, 1.5, 2.0, 2.5, 3.0):
            t0 = time.perf_counter()
            t, n = c.step(10 ** 9, 1.3, t_stop, t)
            c.synchronize()
            secs += time.perf_counter() - t0
            steps += n
            if name == "learned":
                p, hg, flag, counts = net.last(semi.nelements)
                a_net = _clip_alpha(1 / (1 + np.exp(-s_par / thr * (np.maximum(p, 0) ** 2 - thr))),
                                    0.0001, 0.002)
                a_hg = _clip_alpha(hg, 0.0001, 0.002)
                a_used = np.where(flag != 0, a_hg, a_net)
                mae.append(dict(t=t, mae_used=float(np.mean(np.abs(a_used - a_hg))),
                                mae_network=float(np.mean(np.abs(a_net - a_hg))),
                                fallback_fraction=float(np.mean(flag != 0)),
                                active_hg=float(np.mean(a_hg > 0))))
        res[name] = c.download()
        out[f"deploy_{name}"] = dict(t=t, steps=steps, secs=secs, rate=rate(semi.ndofs, steps, secs),
                                     status=c.status())
        if name == "learned":
            _, _, _, counts = net.last(semi.nelements)
            out["deploy_learned"]["evaluated"] = int(counts[0])
            out["deploy_learned"]["band_fallbacks"] = int(counts[1])
            out["deploy_learned"]["positivity_fallbacks"] = int(counts[2])
            ShockIndicatorMLP.undeploy(semi)
        del semi
    out["alpha_mae"] = mae
    rho_hg, rho_ml = res["hg"][..., 0], res["learned"][..., 0]
    out["l2_rho_learned_vs_hg"] = float(np.sqrt(np.mean((rho_ml - rho_hg) ** 2)))
    out["l2_rho_learned_vs_hg_rel"] = out["l2_rho_learned_vs_hg"] / float(np.sqrt(np.mean(rho_hg ** 2)))
    semi = khi_semi(deploy_level, "fp64")
    _, t, n, secs = solve_timed(semi, 10.0, 1.3, max_steps=fp64_steps)
    out["fp64_hg"] = dict(steps=n, secs=secs, rate=rate(semi.ndofs, n, secs))
    out["speedup_learned_vs_fp64"] = out["deploy_learned"]["rate"] / out["fp64_hg"]["rate"]
    out["speedup_hg_mixed_vs_fp64"] = out["deploy_hg"]["rate"] / out["fp64_hg"]["rate"]
    return out


def c5a(n=64, seed=20261204, t_end=20.0):
    specs = c5a_specs(n, seed)
    out = dict(specs=specs)
    semis = [vortex_semi(lv, p, eps, "mixed") for lv, p, eps in specs]
    ens = T.Ensemble(semis)
    ens.upload_initial()
    tpb, ms = ens.autotune(iters=20)
    out["autotune"] = dict(threads_per_block=tpb, ms_per_stage=ms)
    t0 = time.perf_counter()
    t, steps = ens.step(10 ** 9, 1.0, t_end)
    secs = time.perf_counter() - t0
    dof_updates = sum(s.ndofs * 5 * int(k) for s, k in zip(semis, steps))
    out["ensemble"] = dict(secs=secs, rate=dof_updates / secs, steps=steps.tolist(),
                           ndofs=sum(s.ndofs for s in semis))
    l2m = [T.calc_error_norms(ens.download(i), t[i], s)[0][0] for i, s in enumerate(semis)]
    ens.close()
    del ens
    # one context at a time: mixed and FP64
    for prec in ("mixed", "fp64"):
        secs, upd, l2 = 0.0, 0, []
        for lv, p, eps in specs:
            semi = vortex_semi(lv, p, eps, prec)
            u, tt, k, s = solve_timed(semi, t_end, 1.0)
            secs += s
            upd += semi.ndofs * 5 * k
            l2.append(T.calc_error_norms(u, tt, semi)[0][0])
            del semi
        out[f"sequential_{prec}"] = dict(secs=secs, rate=upd / secs)
        if prec == "fp64":
            l2f = l2
    ratio = np.asarray(l2m) / np.asarray(l2f)
    out["l2_rho_mixed"] = [float(v) for v in l2m]
    out["l2_rho_fp64"] = [float(v) for v in l2f]
    out["l2_rho_ratio_max"] = float(ratio.max())
    out["l2_rho_ratio_median"] = float(np.median(ratio))
    out["speedup_vs_fp64"] = out["ensemble"]["rate"] / out["sequential_fp64"]["rate"]
    out["speedup_vs_sequential_mixed"] = out["ensemble"]["rate"] / out["sequential_mixed"]["rate"]
    return out


def _ke_history(semi, t_end, dt_out, cfl=1.4, perturb=0.0):
    c = semi.device_context
    u0 = semi.compute_coefficients(0.0)
    if perturb:
        u0 = u0 * (1.0 + perturb * np.random.default_rng(1).uniform(-1, 1, size=u0.shape))
    c.upload(u0)
    hist = [(0.0, float(c.integrals()[-1]))]
    t, steps, secs = 0.0, 0, 0.0
    while t < t_end:
        t0 = time.perf_counter()
        t, n = c.step(10 ** 9, cfl, min(t_end, t + dt_out), t)
        c.synchronize()
        secs += time.perf_counter() - t0
        steps += n
        hist.append((t, float(c.integrals()[-1])))
    return hist, steps, secs


def c5b(levels=((5, 20.0, 20.0), (6, 20.0, 2.0)), dt_out=0.25, control_level=5):
    """levels: (refinement level, mixed t_end, FP64 t_end).  At control_level
    an FP64 run from the initial state perturbed by 1e-13 (relative) shows how
    far two FP64 runs drift apart through the turbulent phase alone."""
    out = {}
    for level, t_mixed, t_fp64 in levels:
        r = {}
        runs = [("mixed", t_mixed, 0.0), ("fp64", t_fp64, 0.0)]
        if level == control_level:
            runs.append(("fp64_perturbed", t_fp64, 1e-13))
        for name, t_end, eps in runs:
            semi = tgv_semi(level, "mixed" if name == "mixed" else "fp64")
            hist, steps, secs = _ke_history(semi, t_end, dt_out, perturb=eps)
            r[name] = dict(ke=hist, steps=steps, secs=secs, rate=rate(semi.ndofs, steps, secs))
            del semi

        def rel_diffs(a, b):
            ka = {round(t, 9): k for t, k in r[a]["ke"]}
            return [abs(ka[round(t, 9)] - k) / k for t, k in r[b]["ke"] if round(t, 9) in ka]

        diffs = rel_diffs("mixed", "fp64")
        r["ke_rel_diff_max"] = float(max(diffs))
        r["ke_rel_diff_final_common"] = float(diffs[-1])
        if "fp64_perturbed" in r:
            ctrl = rel_diffs("fp64_perturbed", "fp64")
            r["control_ke_rel_diff_max"] = float(max(ctrl))
            r["control_ke_rel_diff_final"] = float(ctrl[-1])
        r["speedup"] = r["mixed"]["rate"] / r["fp64"]["rate"]
        out[f"{2 ** level}^3"] = r
    return out


def c5a_specs(n=64, seed=20261204):
    rng = np.random.default_rng(seed)
    return [(int(rng.integers(3, 8)), int(rng.integers(2, 5)), float(rng.uniform(1.0, 5.0)))
            for _ in range(n)]


# Short runs of single kernels (for profiling a handful of launches).
def learned_steps(steps=4, level=9):
    """KHI 512^2 (the bench mesh), mixed precision, a 16-64-64-1 network with its
    initial weights deployed as the shock indicator, `steps` steps."""
    semi = khi_semi(level, "mixed")
    net = ShockIndicatorMLP(2, 3, seed=3)
    c = semi.device_context
    c.upload(semi.compute_coefficients(0.0))
    net.deploy(semi, band=0.01)
    t, n = c.step(steps, 1.3, 10.0, 0.0)
    c.synchronize()
    return dict(steps=n, t=t, status=c.status())


def mms_steps(steps=3, level=5):
    """3D manufactured solution at 32^3 (the mms3d bench mesh), flux differencing
    with flux_ranocha, mixed precision, `steps` steps."""
    eq = T.CompressibleEulerEquations3D(1.4)
    solver = T.DGSEM(polydeg=3, surface_flux=T.flux_lax_friedrichs,
                     volume_integral=T.VolumeIntegralFluxDifferencing(T.flux_ranocha))
    mesh = T.TreeMesh((0.0,) * 3, (2.0,) * 3, initial_refinement_level=level)
    semi = T.SemidiscretizationHyperbolic(mesh, eq, T.initial_condition_convergence_test, solver,
                                          source_terms=T.source_terms_convergence_test,
                                          precision="mixed")
    c = semi.device_context
    c.upload(semi.compute_coefficients(0.0))
    t, n = c.step(steps, 0.6, 10.0, 0.0)
    c.synchronize()
    return dict(steps=n, t=t, status=c.status())


def ensemble_steps(steps=3):
    """The 64-vortex ensemble of c5a, `steps` steps."""
    ens = T.Ensemble([vortex_semi(lv, p, eps, "mixed") for lv, p, eps in c5a_specs()])
    ens.upload_initial()
    t, n = ens.step(steps, 1.0, 20.0)
    return dict(steps=n.tolist())


# ---------------------------------------------------------------------------
# c6: AMR (elixir_euler_blast_wave_amr.jl scaled up)
def amr_blast_semi(level, precision):
    eq = T.CompressibleEulerEquations2D(1.4)
    basis = T.LobattoLegendreBasis(3)
    llf = T.FluxLaxFriedrichs(T.max_abs_speed_naive)
    ind = T.IndicatorHennemannGassner(eq, basis, alpha_max=0.5, alpha_min=0.001,
                                      alpha_smooth=True, variable=T.density_pressure)
    vi = T.VolumeIntegralShockCapturingHG(ind, volume_flux_dg=T.flux_ranocha, volume_flux_fv=llf)
    mesh = T.TreeMesh((-2.0, -2.0), (2.0, 2.0), initial_refinement_level=level)
    return T.SemidiscretizationHyperbolic(mesh, eq, T.initial_condition_blast_wave,
                                          T.DGSEM(basis, llf, vi), precision=precision)


def amr_run(level, base_level, max_level, t_end, precision, cfl=0.9, interval=5):
    """solve() with AMRCallback, stepping and AMR passes timed apart."""
    semi = amr_blast_semi(level, precision)
    ind = T.IndicatorHennemannGassner(semi, alpha_max=0.5, alpha_min=0.001, alpha_smooth=True,
                                      variable=T.density_pressure)
    ctrl = T.ControllerThreeLevel(semi, ind, base_level=base_level, max_level=max_level,
                                  max_threshold=0.01)
    amr = T.AMRCallback(semi, ctrl, interval=interval, adapt_initial_condition=True,
                        adapt_initial_condition_only_refine=True)
    wall0 = time.perf_counter()
    semi.device_context.upload(semi.compute_coefficients(0.0))
    amr.initialize(semi, 0.0)
    t, steps, dof_updates, step_secs, elements = 0.0, 0, 0, 0.0, []
    while True:
        c = semi.device_context
        c.synchronize()
        tic = time.perf_counter()
        t, n = c.step(interval, cfl, t_end, t)
        c.synchronize()
        step_secs += time.perf_counter() - tic
        steps += n
        dof_updates += semi.ndofs * 5 * n
        elements.append(semi.nelements)
        if t >= t_end or n < interval:
            break
        amr(semi)
    wall = time.perf_counter() - wall0
    u = semi.device_context.download()
    l2, linf = T.calc_error_norms(u, t, semi)
    return dict(t=t, steps=steps, passes=amr.passes, wall_secs=wall, step_secs=step_secs,
                amr_indicator_secs=amr.seconds["indicator"], amr_adapt_secs=amr.seconds["adapt"],
                rate_while_stepping=dof_updates / step_secs, rate_overall=dof_updates / wall,
                elements_min=int(min(elements)), elements_max=int(max(elements)),
                elements_final=int(semi.nelements), l2=l2.tolist(), linf=linf.tolist())


def c6(level=8, base_level=6, max_level=8, t_end=0.5):
    """AMR blast wave at 8x the elixir's resolution (initial level 8, base 6, max 8)
    in FP64 and mixed precision: time in steps and in AMR passes, DOF-updates/s."""
    out = {}
    for prec in ("fp64", "mixed"):
        out[prec] = amr_run(level, base_level, max_level, t_end, prec)
    out["elixir_size_fp64"] = amr_run(6, 4, 6, 1.0, "fp64")
    out["l2_rho_mixed_over_fp64"] = out["mixed"]["l2"][0] / out["fp64"]["l2"][0]
    return out


# ---------------------------------------------------------------------------
# c7: throughput on a mesh with mortars
def c7(steps=40):
    """3D MMS (polydeg 3, flux_ranocha, LLF, CFL 0.6) on 32^3 elements and on the
    same mesh with the central box (0.5, 1.5)^3 refined once (61,440 elements,
    4,096 mortars... counted below), FP64 and mixed: DOF-updates/s per stage."""
    out = {}
    for prec in ("mixed", "fp64"):
        for name, patches in (("uniform", ()),
                              ("refined", (dict(type="box", coordinates_min=(0.5,) * 3,
                                                coordinates_max=(1.5,) * 3),))):
            eq = T.CompressibleEulerEquations3D(1.4)
            solver = T.DGSEM(polydeg=3, surface_flux=T.flux_lax_friedrichs,
                             volume_integral=T.VolumeIntegralFluxDifferencing(T.flux_ranocha))
            mesh = T.TreeMesh((0.0,) * 3, (2.0,) * 3, initial_refinement_level=5,
                              refinement_patches=patches)
            semi = T.SemidiscretizationHyperbolic(mesh, eq, T.initial_condition_convergence_test,
                                                  solver, source_terms=T.source_terms_convergence_test,
                                                  precision=prec)
            solve_timed(semi, 10.0, 0.6, max_steps=3)  # warm-up (graphs, caches)
            _, t, n, secs = solve_timed(semi, 10.0, 0.6, max_steps=steps)
            out[f"{prec}_{name}"] = dict(elements=semi.nelements,
                                         mortars=int(semi.mortar_neighbor_ids.shape[0]),
                                         steps=n, secs=secs, rate=rate(semi.ndofs, n, secs))
    for prec in ("mixed", "fp64"):
        out[f"{prec}_refined_over_uniform_rate"] = (out[f"{prec}_refined"]["rate"] /
                                                    out[f"{prec}_uniform"]["rate"])
    return out


def _waving_flag_faces():
    # examples/structured_2d_dgsem/elixir_euler_source_terms_waving_flag.jl
    return (lambda s: (-1.0, s - 1.0), lambda s: (1.0, s + 1.0),
            lambda s: (s, -1.0 + np.sin(0.5 * np.pi * s)),
            lambda s: (s, 1.0 + np.sin(0.5 * np.pi * s)))


def _warped_square(xi_, eta_):
    # examples/structured_2d_dgsem/elixir_euler_free_stream.jl / elixir_euler_ec.jl
    xi = 1.5 * xi_ + 1.5
    eta = 1.5 * eta_ + 1.5
    y = eta + 3 / 8 * (np.cos(1.5 * np.pi * (2 * xi - 3) / 3) * np.cos(0.5 * np.pi * (2 * eta - 3) / 3))
    x = xi + 3 / 8 * (np.cos(0.5 * np.pi * (2 * xi - 3) / 3) * np.cos(2 * np.pi * (2 * y - 3) / 3))
    return x, y


def _warped_cube(xi_, eta_, zeta_):
    # examples/structured_3d_dgsem/elixir_euler_ec.jl / elixir_euler_free_stream.jl
    xi, eta, zeta = 1.5 * xi_ + 1.5, 1.5 * eta_ + 1.5, 1.5 * zeta_ + 1.5
    y = eta + 3 / 8 * (np.cos(1.5 * np.pi * (2 * xi - 3) / 3) * np.cos(0.5 * np.pi * (2 * eta - 3) / 3) *
                       np.cos(0.5 * np.pi * (2 * zeta - 3) / 3))
    x = xi + 3 / 8 * (np.cos(0.5 * np.pi * (2 * xi - 3) / 3) * np.cos(2 * np.pi * (2 * y - 3) / 3) *
                      np.cos(0.5 * np.pi * (2 * zeta - 3) / 3))
    z = zeta + 3 / 8 * (np.cos(0.5 * np.pi * (2 * x - 3) / 3) * np.cos(np.pi * (2 * y - 3) / 3) *
                        np.cos(0.5 * np.pi * (2 * zeta - 3) / 3))
    return x, y, z


def _sedov_warp(xi, eta):
    # examples/structured_2d_dgsem/elixir_euler_sedov.jl
    y = eta + 0.125 * (np.cos(1.5 * np.pi * xi) * np.cos(0.5 * np.pi * eta))
    x = xi + 0.125 * (np.cos(0.5 * np.pi * xi) * np.cos(2 * np.pi * y))
    return x, y


def curved3_semi(cells, precision):
    """The EC elixir of the 3D StructuredMesh examples at cells^3, polydeg 3:
    weak blast wave (gamma 5/3) on the warped cube, flux_ranocha volume and
    surface flux."""
    eq = T.CompressibleEulerEquations3D(5.0 / 3.0)
    solver = T.DGSEM(polydeg=3, surface_flux=T.flux_ranocha,
                     volume_integral=T.VolumeIntegralFluxDifferencing(T.flux_ranocha))
    mesh = T.StructuredMesh((cells,) * 3, mapping=_warped_cube)
    return T.SemidiscretizationHyperbolic(mesh, eq, T.initial_condition_weak_blast_wave, solver,
                                          precision=precision)


def sedov_semi(cells, precision):
    """The Sedov blast of the 2D StructuredMesh examples at cells^2, polydeg 3:
    shock capturing (HG on rho*p, alpha_max 1, flux_ranocha / naive LLF FV)
    on the warped square, naive LLF surface flux."""
    eq = T.CompressibleEulerEquations2D(1.4)
    basis = T.LobattoLegendreBasis(3)
    llf = T.FluxLaxFriedrichs(T.max_abs_speed_naive)
    ind = T.IndicatorHennemannGassner(eq, basis, alpha_max=1.0, alpha_min=0.001,
                                      alpha_smooth=True, variable=T.density_pressure)
    vi = T.VolumeIntegralShockCapturingHG(ind, volume_flux_dg=T.flux_ranocha, volume_flux_fv=llf)
    mesh = T.StructuredMesh((cells, cells), mapping=_sedov_warp)
    return T.SemidiscretizationHyperbolic(mesh, eq, T.initial_condition_sedov_blast_wave,
                                          T.DGSEM(basis, llf, vi), precision=precision)


def c8(cells=512, steps=30, t_end=0.25, cells3=32):
    """Curvilinear 2D meshes: (a) the waving-flag StructuredMesh MMS at cells^2,
    polydeg 3, weak form, naive LLF, CFL 0.8 (L2 density error at t_end of both
    paths); (b) the weak blast wave on the warped square as a P4estMesh of
    16 x 16 trees refined to cells^2, polydeg 3, flux_ranocha volume and surface
    flux, CFL 1.0.  DOF-updates/s per stage, FP64 and mixed."""
    out = {}
    eq = T.CompressibleEulerEquations2D(1.4)
    level = int(round(math.log2(cells // 16)))
    for name in ("flag_weak", "p4est_fd_ranocha"):
        for prec in ("mixed", "fp64"):
            if name == "flag_weak":
                solver = T.DGSEM(polydeg=3, surface_flux=T.FluxLaxFriedrichs(T.max_abs_speed_naive))
                mesh = T.StructuredMesh((cells, cells), faces=_waving_flag_faces())
                semi = T.SemidiscretizationHyperbolic(
                    mesh, eq, T.initial_condition_convergence_test, solver,
                    source_terms=T.source_terms_convergence_test, precision=prec)
                cfl = 0.8
            else:
                solver = T.DGSEM(polydeg=3, surface_flux=T.flux_ranocha,
                                 volume_integral=T.VolumeIntegralFluxDifferencing(T.flux_ranocha))
                mesh = T.P4estMesh((16, 16), polydeg=3, mapping=_warped_square,
                                   initial_refinement_level=level)
                semi = T.SemidiscretizationHyperbolic(mesh, eq, T.initial_condition_weak_blast_wave,
                                                      solver, precision=prec)
                cfl = 1.0
            solve_timed(semi, 10.0, cfl, max_steps=3)  # warm-up
            n_steps = steps if prec == "mixed" else max(3, steps // 3)
            _, t, n, secs = solve_timed(semi, 10.0, cfl, max_steps=n_steps)
            r = dict(elements=semi.nelements, steps=n, secs=secs, rate=rate(semi.ndofs, n, secs))
            if name == "flag_weak":
                u, tt, _, _ = solve_timed(semi, t_end, cfl)
                l2, linf = T.calc_error_norms(u, tt, semi)
                r.update(l2_rho=float(l2[0]), linf_rho=float(linf[0]), t=tt)
            out[f"{name}_{prec}"] = r
        out[f"{name}_speedup"] = out[f"{name}_mixed"]["rate"] / out[f"{name}_fp64"]["rate"]
    out["flag_l2_rho_mixed_over_fp64"] = (out["flag_weak_mixed"]["l2_rho"] /
                                          out["flag_weak_fp64"]["l2_rho"])
    # (c) 3D: the warped-cube EC elixir at cells3^3; (d) shock capturing: the
    # Sedov blast on the warped square at cells^2
    for name, make, cfl in (("cube3d_fd_ranocha", lambda p: curved3_semi(cells3, p), 1.0),
                            ("sedov_hg", lambda p: sedov_semi(cells, p), 0.5)):
        for prec in ("mixed", "fp64"):
            semi = make(prec)
            solve_timed(semi, 10.0, cfl, max_steps=3)  # warm-up
            n_steps = steps if prec == "mixed" else max(3, steps // 3)
            _, t, n, secs = solve_timed(semi, 10.0, cfl, max_steps=n_steps)
            out[f"{name}_{prec}"] = dict(elements=semi.nelements, steps=n, secs=secs,
                                         rate=rate(semi.ndofs, n, secs))
            del semi
        out[f"{name}_speedup"] = out[f"{name}_mixed"]["rate"] / out[f"{name}_fp64"]["rate"]
    return out


def mortar_steps(steps=4):
    """c7's refined mesh (3D MMS 32^3 with the central box refined once, 61,440
    elements, 1,536 mortars), mixed precision, `steps` steps."""
    eq = T.CompressibleEulerEquations3D(1.4)
    solver = T.DGSEM(polydeg=3, surface_flux=T.flux_lax_friedrichs,
                     volume_integral=T.VolumeIntegralFluxDifferencing(T.flux_ranocha))
    mesh = T.TreeMesh((0.0,) * 3, (2.0,) * 3, initial_refinement_level=5,
                      refinement_patches=(dict(type="box", coordinates_min=(0.5,) * 3,
                                               coordinates_max=(1.5,) * 3),))
    semi = T.SemidiscretizationHyperbolic(mesh, eq, T.initial_condition_convergence_test, solver,
                                          source_terms=T.source_terms_convergence_test,
                                          precision="mixed")
    _, t, n, secs = solve_timed(semi, 10.0, 0.6, max_steps=steps)
    return dict(steps=n, t=t)


def curved_steps(steps=3, cells=512):
    """c8's waving-flag StructuredMesh MMS (cells^2, polydeg 3, weak form, naive
    LLF, CFL 0.8), mixed precision, `steps` steps."""
    eq = T.CompressibleEulerEquations2D(1.4)
    solver = T.DGSEM(polydeg=3, surface_flux=T.FluxLaxFriedrichs(T.max_abs_speed_naive))
    mesh = T.StructuredMesh((cells, cells), faces=_waving_flag_faces())
    semi = T.SemidiscretizationHyperbolic(mesh, eq, T.initial_condition_convergence_test, solver,
                                          source_terms=T.source_terms_convergence_test,
                                          precision="mixed")
    _, t, n, secs = solve_timed(semi, 10.0, 0.8, max_steps=steps)
    return dict(steps=n, t=t)


def curved3_steps(steps=3, cells=32):
    """c8's 3D warped-cube EC case (cells^3, polydeg 3, flux_ranocha), mixed
    precision, `steps` steps."""
    semi = curved3_semi(cells, "mixed")
    _, t, n, secs = solve_timed(semi, 10.0, 1.0, max_steps=steps)
    return dict(steps=n, t=t)


def c5b_64():
    """C5b at its full size: 64^3, mixed and FP64 both to t = 20."""
    return c5b(levels=((6, 20.0, 20.0),), control_level=None)


def c5b_64_control(eps=1e-9, dt_out=0.25):
    """How far two mixed runs at 64^3 drift apart through the turbulent phase when
    one starts from the initial state perturbed by eps (relative): the growth of
    a perturbation of the size of the mixed path's early difference to FP64."""
    r = {}
    for name, e in (("mixed", 0.0), ("mixed_perturbed", eps)):
        semi = tgv_semi(6, "mixed")
        hist, steps, secs = _ke_history(semi, 20.0, dt_out, perturb=e)
        r[name] = dict(ke=hist, steps=steps, secs=secs)
        del semi
    ka = {round(t, 9): k for t, k in r["mixed_perturbed"]["ke"]}
    diffs = [(t, abs(ka[round(t, 9)] - k) / k) for t, k in r["mixed"]["ke"] if round(t, 9) in ka]
    r["ke_rel_diff"] = diffs
    r["ke_rel_diff_max"] = float(max(d for _, d in diffs))
    r["ke_rel_diff_final"] = float(diffs[-1][1])
    return r


RUNS = dict(c1=c1, c3=c3, c4=c4, c5a=c5a, c5b=c5b, c5b_64=c5b_64, c5b_64_control=c5b_64_control,
            c6=c6, c7=c7, c8=c8)
SHORT_RUNS = dict(learned_steps=learned_steps, mms_steps=mms_steps, ensemble_steps=ensemble_steps,
                  mortar_steps=mortar_steps, curved_steps=curved_steps,
                  curved3_steps=curved3_steps)


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--only", default=",".join(RUNS),
                    help="comma-separated subset of " + ",".join(list(RUNS) + list(SHORT_RUNS)))
    ap.add_argument("--out", default=None, help="write the results as JSON here")
    args = ap.parse_args(argv)
    results = {}
    for name in args.only.split(","):
        t0 = time.perf_counter()
        results[name] = {**RUNS, **SHORT_RUNS}[name]()
        results[name]["wall_secs"] = time.perf_counter() - t0
        brief = {k: v for k, v in results[name].items() if not isinstance(v, (list, dict))}
        print(name, json.dumps(brief), flush=True)
        if args.out:
            with open(args.out, "w") as f:
                json.dump(results, f, indent=1)
    return results


if __name__ == "__main__":
    main()
