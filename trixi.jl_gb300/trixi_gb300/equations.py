"""Compressible Euler equations, numerical fluxes, initial conditions, sources.

Host-side mirror of src/equations/compressible_euler_{2,3}d.jl and
src/equations/numerical_fluxes.jl.  Fluxes and source terms are markers that
select the device implementation; initial conditions are vectorised numpy
functions of node coordinates x[..., ndims] (evaluated once, at setup).
"""
from __future__ import annotations

import math

import numpy as np

from . import _lib


class CompressibleEulerEquations2D:
    ndims = 2
    nvariables = 4

    def __init__(self, gamma: float):
        self.gamma = float(gamma)
        self.inv_gamma_minus_one = 1.0 / (self.gamma - 1.0)

    def __repr__(self):
        return f"CompressibleEulerEquations2D(gamma={self.gamma})"


class CompressibleEulerEquations3D(CompressibleEulerEquations2D):
    ndims = 3
    nvariables = 5

    def __repr__(self):
        return f"CompressibleEulerEquations3D(gamma={self.gamma})"


# ---------------------------------------------------------------------------
# numerical fluxes (markers)
# ---------------------------------------------------------------------------
class _Flux:
    def __init__(self, name: str, code: int):
        self.name, self.code = name, code

    def __repr__(self):
        return self.name


flux_central = _Flux("flux_central", _lib.TG_FLUX_CENTRAL)
flux_ranocha = _Flux("flux_ranocha", _lib.TG_FLUX_RANOCHA)
flux_shima_etal = _Flux("flux_shima_etal", _lib.TG_FLUX_SHIMA_ETAL)
# flux_hllc, compressible_euler_2d.jl:1720-1816 (a surface flux)
flux_hllc = _Flux("flux_hllc", _lib.TG_FLUX_HLLC)
# flux_chandrashekar, compressible_euler_2d.jl, 3d.jl:640-692
flux_chandrashekar = _Flux("flux_chandrashekar", _lib.TG_FLUX_CHANDRASHEKAR)
# flux_hlle = FluxHLL(min_max_speed_einfeldt), numerical_fluxes.jl:422-457 (a surface flux)
flux_hlle = _Flux("flux_hlle", _lib.TG_FLUX_HLLE)


class _MaxAbsSpeed:
    def __init__(self, name):
        self.name = name

    def __repr__(self):
        return self.name


max_abs_speed = _MaxAbsSpeed("max_abs_speed")
max_abs_speed_naive = _MaxAbsSpeed("max_abs_speed_naive")


def FluxLaxFriedrichs(max_abs_speed_fn=max_abs_speed):
    """FluxLaxFriedrichs(max_abs_speed), numerical_fluxes.jl:222-253."""
    if max_abs_speed_fn is max_abs_speed_naive:
        return _Flux("FluxLaxFriedrichs(max_abs_speed_naive)", _lib.TG_FLUX_LAX_FRIEDRICHS_NAIVE)
    if max_abs_speed_fn is max_abs_speed:
        return _Flux("FluxLaxFriedrichs(max_abs_speed)", _lib.TG_FLUX_LAX_FRIEDRICHS)
    raise NotImplementedError(f"wave speed estimate {max_abs_speed_fn!r}")


flux_lax_friedrichs = FluxLaxFriedrichs()


# ---------------------------------------------------------------------------
# source terms (markers evaluated on the device)
# ---------------------------------------------------------------------------
class _Source:
    def __init__(self, name, code):
        self.name, self.code = name, code

    def __repr__(self):
        return self.name


source_terms_convergence_test = _Source("source_terms_convergence_test",
                                        _lib.TG_SOURCE_CONVERGENCE_TEST)


# ---------------------------------------------------------------------------
# variable conversions
# ---------------------------------------------------------------------------
def prim2cons(prim, equations):
    """prim2cons, compressible_euler_2d.jl / 3d.jl."""
    D = equations.ndims
    rho = prim[..., 0]
    u = np.empty_like(prim)
    u[..., 0] = rho
    ke = np.zeros_like(rho)
    for d in range(D):
        u[..., 1 + d] = rho * prim[..., 1 + d]
        ke = ke + u[..., 1 + d] * prim[..., 1 + d]
    u[..., D + 1] = prim[..., D + 1] * equations.inv_gamma_minus_one + 0.5 * ke
    return u


def cons2prim(u, equations):
    D = equations.ndims
    w = np.empty_like(u)
    w[..., 0] = u[..., 0]
    ke = np.zeros_like(u[..., 0])
    for d in range(D):
        w[..., 1 + d] = u[..., 1 + d] / u[..., 0]
        ke = ke + u[..., 1 + d] * w[..., 1 + d]
    w[..., D + 1] = (equations.gamma - 1) * (u[..., D + 1] - 0.5 * ke)
    return w


# ---------------------------------------------------------------------------
# initial conditions: f(x[..., D], t, equations) -> u[..., NV]
# ---------------------------------------------------------------------------
def initial_condition_constant(x, t, equations):
    """compressible_euler_2d.jl:71-78, 3d.jl:78-86."""
    shape = x.shape[:-1]
    if equations.ndims == 2:
        vals = (1.0, 0.1, -0.2, 10.0)
    else:
        vals = (1.0, 0.1, -0.2, 0.7, 10.0)
    return np.broadcast_to(np.array(vals), shape + (len(vals),)).copy()


def initial_condition_convergence_test(x, t, equations):
    """compressible_euler_2d.jl:87-104, 3d.jl:93-110."""
    c, A = 2.0, 0.1
    omega = 2 * math.pi * 0.5
    s = x[..., 0] + x[..., 1]
    if equations.ndims == 3:
        s = s + x[..., 2]
    ini = c + A * np.sin(omega * (s - t))
    u = np.empty(x.shape[:-1] + (equations.nvariables,))
    for v in range(equations.nvariables - 1):
        u[..., v] = ini
    u[..., -1] = ini * ini
    return u


def initial_condition_isentropic_vortex_advected(p_inf=25.0, amplitude=5.0):
    """examples/tree_2d_dgsem/elixir_euler_vortex_mortar.jl:18-64: the vortex of
    initial_condition_isentropic_vortex advected with the base flow (1, 1) and
    wrapped to the nearest periodic image on [-10, 10]^2 (exact at every t)."""

    def ic(x, t, equations):
        g = equations.gamma
        rho0, p0 = 1.0, float(p_inf)
        rt = p0 / rho0
        c0 = x[..., 0] - t
        c1 = x[..., 1] - t
        c0 = c0 - 20.0 * np.round(c0 / 20.0)  # round half to even, as Julia's round
        c1 = c1 - 20.0 * np.round(c1 / 20.0)
        a0, a1 = -c1, c0
        r2 = a0 * a0 + a1 * a1
        du = amplitude / (2 * math.pi) * np.exp(0.5 * (1 - r2))
        dtemp = -(g - 1) / (2 * g * rt) * du * du
        prim = np.empty(x.shape[:-1] + (4,))
        prim[..., 0] = rho0 * (1 + dtemp) ** (1 / (g - 1))
        prim[..., 1] = 1.0 + du * a0
        prim[..., 2] = 1.0 + du * a1
        prim[..., 3] = p0 * (1 + dtemp) ** (g / (g - 1))
        return prim2cons(prim, equations)

    ic.__name__ = "initial_condition_isentropic_vortex_advected"
    ic.params = (float(p_inf), float(amplitude))
    return ic


def initial_condition_density_wave(x, t, equations):
    """initial_condition_density_wave, compressible_euler_2d.jl:161-171: a density
    sine wave advected with velocity (0.1, 0.2) at pressure 20 (exact at every t)."""
    if equations.ndims != 2:
        raise NotImplementedError("initial_condition_density_wave is 2D")
    v1, v2 = 0.1, 0.2
    a = 2 * (x[..., 0] + x[..., 1] - t * (v1 + v2))
    rho = 1 + 0.98 * _sinpi(a)
    u = np.empty(x.shape[:-1] + (4,))
    u[..., 0] = rho
    u[..., 1] = rho * v1
    u[..., 2] = rho * v2
    u[..., 3] = 20 / (equations.gamma - 1) + 0.5 * rho * (v1 ** 2 + v2 ** 2)
    return u


def initial_condition_sedov_blast_wave(x, t, equations):
    """examples/tree_2d_dgsem/elixir_euler_sedov_blast_wave.jl:11-32: energy 1 in a
    disc of radius 0.21875 at rest in a background at p = 1e-5."""
    if equations.ndims != 2:
        raise NotImplementedError("initial_condition_sedov_blast_wave is the 2D elixir's")
    r = np.sqrt(x[..., 0] ** 2 + x[..., 1] ** 2)
    r0, E = 0.21875, 1.0
    p_inner = 3 * (equations.gamma - 1) * E / (3 * math.pi * r0 ** 2)
    prim = np.zeros(x.shape[:-1] + (4,))
    prim[..., 0] = 1.0
    prim[..., 3] = np.where(r > r0, 1.0e-5, p_inner)
    return prim2cons(prim, equations)


def initial_condition_medium_sedov_blast_wave(x, t, equations):
    """initial_condition_medium_sedov_blast_wave of
    examples/structured_3d_dgsem/elixir_euler_sedov.jl: energy 1 in a ball of
    radius 0.21875 at rest in a background at p = 1e-3."""
    if equations.ndims != 3:
        raise NotImplementedError("initial_condition_medium_sedov_blast_wave is the 3D elixir's")
    r = np.sqrt(x[..., 0] ** 2 + x[..., 1] ** 2 + x[..., 2] ** 2)
    r0, E = 0.21875, 1.0
    p_inner = 3 * (equations.gamma - 1) * E / (4 * math.pi * r0 ** 2)
    prim = np.zeros(x.shape[:-1] + (5,))
    prim[..., 0] = 1.0
    prim[..., 4] = np.where(r > r0, 1.0e-3, p_inner)
    return prim2cons(prim, equations)


def initial_condition_density_pulse(x, t, equations):
    """examples/tree_3d_dgsem/elixir_euler_amr.jl:9-25: a Gaussian density pulse
    at rest pressure 1 moving with velocity (1, 1, 1)."""
    if equations.ndims != 3:
        raise NotImplementedError("initial_condition_density_pulse is the 3D elixir's")
    g = equations.gamma
    rho = 1 + np.exp(-(x[..., 0] ** 2 + x[..., 1] ** 2 + x[..., 2] ** 2)) / 2
    u = np.empty(x.shape[:-1] + (5,))
    u[..., 0] = rho
    u[..., 1] = rho
    u[..., 2] = rho
    u[..., 3] = rho
    u[..., 4] = 1 / (g - 1) + 1 / 2 * rho * 3
    return u


def initial_condition_blast_wave(x, t, equations):
    """The medium blast wave of examples/tree_2d_dgsem/elixir_euler_blast_wave_amr.jl:18-34
    (Hennemann & Gassner 2020, sec. 6.3): the weak blast wave's inner state in a
    background at p = 1e-3."""
    if equations.ndims != 2:
        raise NotImplementedError("initial_condition_blast_wave is the 2D elixir's")
    r = np.sqrt(x[..., 0] ** 2 + x[..., 1] ** 2)
    phi = np.arctan2(x[..., 1], x[..., 0])
    out = r > 0.5
    prim = np.empty(x.shape[:-1] + (4,))
    prim[..., 0] = np.where(out, 1.0, 1.1691)
    prim[..., 1] = np.where(out, 0.0, 0.1882 * np.cos(phi))
    prim[..., 2] = np.where(out, 0.0, 0.1882 * np.sin(phi))
    prim[..., 3] = np.where(out, 1.0e-3, 1.245)
    return prim2cons(prim, equations)


def initial_condition_weak_blast_wave(x, t, equations):
    """compressible_euler_2d.jl:245-264, 3d.jl:241-263."""
    D = equations.ndims
    prim = np.empty(x.shape[:-1] + (D + 2,))
    if D == 2:
        r = np.sqrt(x[..., 0] ** 2 + x[..., 1] ** 2)
        phi = np.arctan2(x[..., 1], x[..., 0])
        out = r > 0.5
        prim[..., 0] = np.where(out, 1.0, 1.1691)
        prim[..., 1] = np.where(out, 0.0, 0.1882 * np.cos(phi))
        prim[..., 2] = np.where(out, 0.0, 0.1882 * np.sin(phi))
        prim[..., 3] = np.where(out, 1.0, 1.245)
    else:
        r = np.sqrt(x[..., 0] ** 2 + x[..., 1] ** 2 + x[..., 2] ** 2)
        phi = np.arctan2(x[..., 1], x[..., 0])
        with np.errstate(invalid="ignore", divide="ignore"):
            theta = np.where(r == 0, 0.0, np.arccos(np.where(r == 0, 1.0, x[..., 2] / np.where(r == 0, 1.0, r))))
        out = r > 0.5
        prim[..., 0] = np.where(out, 1.0, 1.1691)
        prim[..., 1] = np.where(out, 0.0, 0.1882 * np.cos(phi) * np.sin(theta))
        prim[..., 2] = np.where(out, 0.0, 0.1882 * np.sin(phi) * np.sin(theta))
        prim[..., 3] = np.where(out, 0.0, 0.1882 * np.cos(theta))
        prim[..., 4] = np.where(out, 1.0, 1.245)
    return prim2cons(prim, equations)


def _sinpi(a):
    r = np.fmod(a, 2.0)
    r = np.where(r > 1, r - 2, r)
    r = np.where(r < -1, r + 2, r)
    return np.where((r == 0) | (r == 1) | (r == -1), 0.0, np.sin(math.pi * r))


def initial_condition_kelvin_helmholtz_instability(x, t, equations):
    """examples/tree_2d_dgsem/elixir_euler_kelvin_helmholtz_instability.jl:18-31."""
    slope = 15.0
    B = np.tanh(slope * x[..., 1] + 7.5) - np.tanh(slope * x[..., 1] - 7.5)
    prim = np.empty(x.shape[:-1] + (4,))
    prim[..., 0] = 0.5 + 0.75 * B
    prim[..., 1] = 0.5 * (B - 1)
    prim[..., 2] = 0.1 * _sinpi(2 * x[..., 0])
    prim[..., 3] = 1.0
    return prim2cons(prim, equations)


def initial_condition_isentropic_vortex(p_inf=25.0, amplitude=5.0):
    """examples/tree_2d_dgsem/elixir_euler_vortex.jl:18-52 (rho=1, v=(1,1), radius 1),
    with the background pressure and the vortex strength as parameters."""

    def ic(x, t, equations):
        g = equations.gamma
        rho0, p0 = 1.0, float(p_inf)
        rt = p0 / rho0
        c0, c1 = -x[..., 1], x[..., 0]
        r2 = c0 * c0 + c1 * c1
        du = amplitude / (2 * math.pi) * np.exp(0.5 * (1 - r2))
        dtemp = -(g - 1) / (2 * g * rt) * du * du
        prim = np.empty(x.shape[:-1] + (4,))
        prim[..., 0] = rho0 * (1 + dtemp) ** (1 / (g - 1))
        prim[..., 1] = 1.0 + du * c0
        prim[..., 2] = 1.0 + du * c1
        prim[..., 3] = p0 * (1 + dtemp) ** (g / (g - 1))
        return prim2cons(prim, equations)

    ic.__name__ = "initial_condition_isentropic_vortex"
    ic.params = (float(p_inf), float(amplitude))
    return ic


def initial_condition_taylor_green_vortex(Ms=0.1):
    """examples/tree_3d_dgsem/elixir_euler_taylor_green_vortex.jl:14-30."""

    def ic(x, t, equations):
        A, rho = 1.0, 1.0
        X, Y, Z = x[..., 0], x[..., 1], x[..., 2]
        prim = np.empty(x.shape[:-1] + (5,))
        prim[..., 0] = rho
        prim[..., 1] = A * np.sin(X) * np.cos(Y) * np.cos(Z)
        prim[..., 2] = -A * np.cos(X) * np.sin(Y) * np.cos(Z)
        prim[..., 3] = 0.0
        p = (A / Ms) ** 2 * rho / equations.gamma
        p = p + 1.0 / 16.0 * A * A * rho * (np.cos(2 * X) * np.cos(2 * Z) + 2 * np.cos(2 * Y) +
                                            2 * np.cos(2 * X) + np.cos(2 * Y) * np.cos(2 * Z))
        prim[..., 4] = p
        return prim2cons(prim, equations)

    ic.__name__ = "initial_condition_taylor_green_vortex"
    ic.params = (float(Ms),)
    return ic


def initial_condition_gaussian_blast(p_background=1e-5, energy=1.0, width=0.25):
    """Gaussian energy deposit at the origin: rho = 1, v = 0,
    p = p_bg + (gamma - 1) E exp(-r^2 / w^2) / (pi w^2)^(d/2) (total energy E)."""

    def ic(x, t, equations):
        D = equations.ndims
        r2 = np.sum(x ** 2, axis=-1)
        norm = (math.pi * width * width) ** (D / 2)
        prim = np.zeros(x.shape[:-1] + (D + 2,))
        prim[..., 0] = 1.0
        prim[..., D + 1] = p_background + (equations.gamma - 1) * energy * np.exp(-r2 / width ** 2) / norm
        return prim2cons(prim, equations)

    ic.__name__ = "initial_condition_gaussian_blast"
    ic.params = (float(p_background), float(energy), float(width))
    return ic


def density(u, equations):
    """density, compressible_euler_2d.jl (the first conserved variable)."""
    return u[..., 0]


def density_pressure(u, equations):
    """density_pressure, compressible_euler_2d.jl:2205-2210."""
    D = equations.ndims
    m2 = sum(u[..., 1 + d] ** 2 for d in range(D))
    return (equations.gamma - 1) * (u[..., 0] * u[..., D + 1] - 0.5 * m2)
