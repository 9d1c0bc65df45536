"""Time integration on the device: CarpenterKennedy2N54 driven by a StepsizeCallback.

Mirrors Trixi's SimpleIntegrator2N (src/time_integration/methods_2N.jl:95-168)
with the StepsizeCallback (src/callbacks_step/stepsize.jl:66-126): each step
is a CUDA graph of five fused stage kernels, and t, dt and the CFL reduction
stay on the device (tg_step).  solve() returns the final state on the host.
"""
from __future__ import annotations

import time

import numpy as np

from .analysis import calc_error_norms
from .amr import AMRCallback


class CarpenterKennedy2N54:
    """methods_2N.jl:24-48 (OrdinaryDiffEq's CarpenterKennedy2N54(williamson_condition=false)
    is the same scheme)."""
    a = (0.0, 567301805773.0 / 1357537059087.0, 2404267990393.0 / 2016746695238.0,
         3550918686646.0 / 2091501179385.0, 1275806237668.0 / 842570457699.0)
    b = (1432997174477.0 / 9575080441755.0, 5161836677717.0 / 13612068292357.0,
         1720146321549.0 / 2090206949498.0, 3134564353537.0 / 4481467310338.0,
         2277821191437.0 / 14882151754819.0)
    c = (0.0, 1432997174477.0 / 9575080441755.0, 2526269341429.0 / 6820363962896.0,
         2006345519317.0 / 3224310063776.0, 2802321613138.0 / 2924317926251.0)

    def __init__(self, williamson_condition=False):
        self.williamson_condition = williamson_condition


class StepsizeCallback:
    def __init__(self, cfl=1.0, interval=1):
        if interval != 1:
            raise NotImplementedError("StepsizeCallback: interval must be 1 on the GPU path")
        self.cfl = float(cfl)


class AnalysisCallback:
    """Computes the final L2/Linf errors (cons2cons vs the initial condition at
    t): on the device from the context state where the initial condition runs
    there (TreeMesh), else on the host from u."""

    def __init__(self, semi, interval=100, **kwargs):
        self.semi, self.interval = semi, interval
        self.l2 = self.linf = None

    def finalize(self, u, t):
        if not getattr(self.semi, "curved", False):
            try:
                self.l2, self.linf = calc_error_norms(None, t, self.semi)
                return self.l2, self.linf
            except NotImplementedError:
                pass
        self.l2, self.linf = calc_error_norms(u, t, self.semi)
        return self.l2, self.linf


class SummaryCallback:
    pass


class AliveCallback:
    def __init__(self, *args, **kwargs):
        pass


class CallbackSet:
    def __init__(self, *callbacks):
        self.callbacks = [c for c in callbacks if c is not None]

    def find(self, cls):
        for c in self.callbacks:
            if isinstance(c, cls):
                return c
        return None


def ode_default_options():
    return dict(save_everystep=False)


class ODESolution:
    def __init__(self, u, t, nsteps, wall):
        self.u = u
        self.t = t
        self.nsteps = nsteps
        self.wall_time = wall
        self.stats = dict(naccept=nsteps)


def solve(ode, alg, dt=None, callback=None, save_everystep=False, maxiters=10**12, **kwargs):
    """solve(ode, CarpenterKennedy2N54(); dt, callback): steps to tspan[1] on the device."""
    if not isinstance(alg, CarpenterKennedy2N54):
        raise NotImplementedError("only CarpenterKennedy2N54 is on the GPU path")
    semi = ode.p
    ctx = semi.device_context
    cbs = callback if isinstance(callback, CallbackSet) else CallbackSet(
        *(callback if isinstance(callback, (list, tuple)) else [callback] if callback else []))
    ctx.upload(ode.u0)
    t0, t_end = ode.tspan
    stepsize = cbs.find(StepsizeCallback)
    amr = cbs.find(AMRCallback)
    tic = time.perf_counter()
    if amr is not None:
        if stepsize is None:
            raise NotImplementedError("AMR on the GPU path needs a StepsizeCallback")
        # AMRCallback before StepsizeCallback: the initial mesh is adapted
        # first, and after every `interval` accepted steps the mesh is adapted
        # and the next step size computed from the adapted state
        amr.initialize(semi, t0)
        t, nsteps = t0, 0
        chunk = amr.interval if amr.interval > 0 else maxiters
        while nsteps < maxiters:
            t, n = semi.device_context.step(min(chunk, maxiters - nsteps), stepsize.cfl, t_end, t)
            nsteps += n
            if t >= t_end or n < chunk or amr.interval == 0:
                break
            amr(semi)
        ctx = semi.device_context
    elif stepsize is not None:
        t, nsteps = ctx.step(maxiters, stepsize.cfl, t_end, t0)
    else:
        if dt is None:
            raise ValueError("fixed-step solve needs dt")
        t, nsteps = t0, 0
        while t < t_end and nsteps < maxiters:
            h = min(dt, t_end - t)
            for s in range(5):
                ctx.rk_stage(s, t, h)
            t += h
            nsteps += 1
    u = ctx.download()
    wall = time.perf_counter() - tic
    sol = ODESolution([ode.u0, u], [t0, t], nsteps, wall)
    ana = cbs.find(AnalysisCallback)
    if ana is not None:
        ana.finalize(u, t)
    return sol
