"""Adaptive mesh refinement on a TreeMesh: AMRCallback with ControllerThreeLevel.

Mirrors src/callbacks_step/amr.jl: the controller turns an indicator into a
value per element (+1 refine, -1 coarsen, 0 keep; amr.jl:1116-1168); the
callback adapts the tree (refine! with 2:1 rebalancing, then coarsen!;
amr.jl:244-392) every `interval` accepted steps and once, or repeatedly, on
the initial condition (amr.jl:143-181).  The indicator is evaluated and the
solution transferred on the device (tg_amr_indicator, tg_adapt_state); the
tree lives on the host.
"""
from __future__ import annotations

import time

import numpy as np

from .equations import density
from .solvers import IndicatorHennemannGassner, IndicatorMax


class ControllerThreeLevel:
    """ControllerThreeLevel(semi, indicator; base_level, med_level, med_threshold,
    max_level, max_threshold), amr.jl:984-1010: target level max_level where the
    indicator exceeds max_threshold, med_level (if > 0, else the current level)
    where it exceeds med_threshold, base_level elsewhere."""

    def __init__(self, semi, indicator, base_level=1, med_level=None, med_threshold=0.0,
                 max_level=None, max_threshold=1.0):
        if not isinstance(indicator, (IndicatorHennemannGassner, IndicatorMax)):
            raise NotImplementedError("ControllerThreeLevel: IndicatorHennemannGassner or "
                                      "IndicatorMax on the GPU path")
        self.indicator = indicator
        self.base_level = int(base_level)
        self.med_level = self.base_level if med_level is None else int(med_level)
        self.max_level = self.base_level if max_level is None else int(max_level)
        self.med_threshold = float(med_threshold)
        self.max_threshold = float(max_threshold)

    def indicator_values(self, semi):
        ind = self.indicator
        variable = 1 if ind.variable is density else 0
        if isinstance(ind, IndicatorMax):
            return semi.device_context.amr_indicator_max(variable)
        return semi.device_context.amr_indicator(ind.alpha_max, ind.alpha_min, ind.alpha_smooth,
                                                 variable)

    def __call__(self, semi):
        alpha = self.indicator_values(semi)
        current = semi.mesh.element_levels()
        target = np.where(alpha > self.max_threshold, self.max_level,
                          np.where(alpha > self.med_threshold,
                                   self.med_level if self.med_level > 0 else current,
                                   self.base_level))
        return np.sign(target - current).astype(np.int8)


class AMRCallback:
    """AMRCallback(semi, controller; interval, adapt_initial_condition,
    adapt_initial_condition_only_refine), amr.jl:33-76."""

    def __init__(self, semi, controller, interval, adapt_initial_condition=True,
                 adapt_initial_condition_only_refine=True):
        if not (isinstance(interval, (int, np.integer)) and interval >= 0):
            raise ValueError("`interval` must be a non-negative integer")
        if getattr(semi.mesh, "curved", False):
            raise NotImplementedError("AMR runs on TreeMeshes; curvilinear meshes are not adapted")
        self.controller = controller
        self.interval = int(interval)
        self.adapt_initial_condition = bool(adapt_initial_condition)
        self.adapt_initial_condition_only_refine = bool(adapt_initial_condition_only_refine)
        self.passes = 0
        self.seconds = dict(indicator=0.0, adapt=0.0)  # wall time of the passes

    def __call__(self, semi, only_refine=False, only_coarsen=False):
        """One AMR pass on the device state of semi; returns whether the mesh changed."""
        tic = time.perf_counter()
        lam = self.controller(semi)
        toc = time.perf_counter()
        changed = semi.adapt(lam, only_refine=only_refine, only_coarsen=only_coarsen)
        self.seconds["indicator"] += toc - tic
        self.seconds["adapt"] += time.perf_counter() - toc
        self.passes += 1
        return changed

    def initialize(self, semi, t0):
        """The initial-condition adaptation of initialize! (amr.jl:143-181): while
        the mesh changes, the initial condition is evaluated afresh on it."""
        if not self.adapt_initial_condition:
            return
        only_refine = self.adapt_initial_condition_only_refine
        changed = self(semi, only_refine=only_refine)
        iterations = 1
        while changed:
            semi.device_context.upload(semi.compute_coefficients(t0))
            changed = self(semi, only_refine=only_refine)
            iterations += 1
            if iterations > max(10, self.controller.max_level):
                break
