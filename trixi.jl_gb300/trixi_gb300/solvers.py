"""DGSEM solver description (host side): src/solvers/dg.jl, src/solvers/dgsem/dgsem.jl,
src/solvers/dgsem/indicators.jl."""
from __future__ import annotations

from . import _lib
from .basis import LobattoLegendreBasis, MortarL2
from .equations import density, density_pressure, flux_central, flux_lax_friedrichs


class VolumeIntegralWeakForm:
    """dg.jl:105."""
    code = _lib.TG_VOLUME_WEAK_FORM

    def __repr__(self):
        return "VolumeIntegralWeakForm()"


class VolumeIntegralFluxDifferencing:
    """dg.jl:135-141."""
    code = _lib.TG_VOLUME_FLUX_DIFFERENCING

    def __init__(self, volume_flux):
        self.volume_flux = volume_flux

    def __repr__(self):
        return f"VolumeIntegralFluxDifferencing({self.volume_flux!r})"


class IndicatorHennemannGassner:
    """IndicatorHennemannGassner(equations, basis; alpha_max, alpha_min, alpha_smooth,
    variable), indicators.jl:50-72.  Only variable = density_pressure is on the GPU path."""

    def __init__(self, equations, basis=None, alpha_max=0.5, alpha_min=0.001, alpha_smooth=True,
                 variable=density_pressure):
        if variable is not density_pressure and variable is not density:
            raise NotImplementedError("IndicatorHennemannGassner: variable density_pressure or density")
        if basis is None and hasattr(equations, "solver"):
            # IndicatorHennemannGassner(semi; ...), indicators.jl:74-83
            equations, basis = equations.equations, equations.solver.basis
        self.equations, self.basis = equations, basis
        self.alpha_max, self.alpha_min = float(alpha_max), float(alpha_min)
        self.alpha_smooth = bool(alpha_smooth)
        self.variable = variable


class IndicatorMax:
    """IndicatorMax(semi; variable), indicators.jl: the maximum of `variable`
    (density or density_pressure on the GPU path) over the nodes of each element;
    an AMR indicator (indicators_3d.jl:239-259)."""

    def __init__(self, semi, variable=density):
        if variable is not density and variable is not density_pressure:
            raise NotImplementedError("IndicatorMax: variable density or density_pressure")
        self.variable = variable


class VolumeIntegralShockCapturingHG:
    """VolumeIntegralShockCapturingHG(indicator; volume_flux_dg, volume_flux_fv), dg.jl:208-221."""
    code = _lib.TG_VOLUME_SHOCK_CAPTURING_HG

    def __init__(self, indicator, volume_flux_dg=flux_central, volume_flux_fv=flux_lax_friedrichs):
        if indicator.variable is not density_pressure:
            raise NotImplementedError("shock capturing: the indicator variable is density_pressure")
        self.indicator = indicator
        self.volume_flux_dg = volume_flux_dg
        self.volume_flux_fv = volume_flux_fv

    @property
    def volume_flux(self):
        return self.volume_flux_dg


class DGSEM:
    """DGSEM(; polydeg, surface_flux, volume_integral) or DGSEM(basis, surface_flux,
    volume_integral), dgsem.jl:25, 65-73."""

    def __init__(self, basis=None, surface_flux=flux_central, volume_integral=None, *,
                 polydeg=None):
        if basis is None:
            if polydeg is None:
                raise TypeError("DGSEM needs polydeg or a basis")
            basis = LobattoLegendreBasis(polydeg)
        elif isinstance(basis, int):
            basis = LobattoLegendreBasis(basis)
        self.basis = basis
        self.mortar = MortarL2(basis)  # dg.mortar (dgsem.jl:25-35)
        self.surface_flux = surface_flux
        self.volume_integral = volume_integral if volume_integral is not None else VolumeIntegralWeakForm()

    @property
    def polydeg(self):
        return self.basis.polydeg

    def nnodes(self):
        return self.basis.nnodes()

    def __repr__(self):
        return (f"DGSEM(polydeg={self.polydeg}, surface_flux={self.surface_flux!r}, "
                f"volume_integral={self.volume_integral!r})")
