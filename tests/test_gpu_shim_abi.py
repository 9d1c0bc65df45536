"""The C ABI called the way the Julia drop-in calls it: tests/c/shim_driver.c,
plain C linked against libtrixi_gb300 only, builds the tg_config from Trixi's
own arrays (1-based Int64 neighbor_ids, column-major basis matrices), keeps the
integrator's vectors in library-owned device memory, evaluates rhs! with tg_rhs
on them and steps CarpenterKennedy2N54 in OrdinaryDiffEq's broadcast form
through tg_lincomb.  Its results are compared with the oracle."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from _gpu_cases import build
from trixi_gb300 import _lib
from trixi_gb300.time_integration import CarpenterKennedy2N54

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "c", "shim_driver.c")

CASES = {
    "2d_fd_ranocha_mms": dict(ndims=2, polydeg=3, level=3, xmin=[0.0, 0.0], xmax=[2.0, 2.0],
                              vi="fluxdiff", volume_flux="ranocha", surface_flux="llf",
                              ic="convergence_test", source="convergence_test"),
    "2d_hg_khi": dict(ndims=2, polydeg=3, level=4, xmin=[-1.0, -1.0], xmax=[1.0, 1.0], vi="hg",
                      volume_flux="ranocha", surface_flux="llf", ic="kelvin_helmholtz",
                      alpha_max=0.002, alpha_min=0.0001),
    "3d_hg_blast": dict(ndims=3, polydeg=3, level=2, xmin=[-2.0] * 3, xmax=[2.0] * 3, vi="hg",
                        volume_flux="ranocha", surface_flux="llf", ic="weak_blast_wave"),
}


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    libdir = os.path.dirname(_lib.LIB_PATH)
    exe = str(tmp_path_factory.mktemp("shim") / "shim_driver")
    subprocess.run([cc, "-O2", "-std=c99", "-I", os.path.join(ROOT, "include"), SRC, "-o", exe,
                    "-L", libdir, "-ltrixi_gb300", "-Wl,-rpath," + libdir], check=True)
    return exe


def _write_input(path, semi, precision_code, u0, t0, dt, nsteps):
    """The driver's input: the arrays a Julia caller hands over, in Trixi's
    layouts (semi.neighbor_ids is [2, I] column-major and 1-based)."""
    dg, eq = semi.solver, semi.equations
    vi = dg.volume_integral
    b = dg.basis
    hg = hasattr(vi, "indicator")
    ck = CarpenterKennedy2N54
    hdr = np.array([eq.ndims, b.polydeg, semi.nelements, semi.neighbor_ids.shape[0], vi.code,
                    vi.volume_flux_dg.code if hg else getattr(getattr(vi, "volume_flux", None),
                                                               "code", 0),
                    dg.surface_flux.code, vi.volume_flux_fv.code if hg else dg.surface_flux.code,
                    int(vi.indicator.alpha_smooth) if hg else 1,
                    semi.source_terms.code if semi.source_terms is not None else 0,
                    precision_code, nsteps], dtype=np.int64)
    hd = np.array([eq.gamma, vi.indicator.alpha_max if hg else 0.5,
                   vi.indicator.alpha_min if hg else 0.001, t0, dt])
    colmajor = [np.asfortranarray(m).ravel(order="F") for m in
                (b.derivative_hat, b.derivative_split, b.inverse_vandermonde_legendre)]
    with open(path, "wb") as f:
        for a in ([hdr, hd, -np.asarray(ck.a), np.asarray(ck.b), np.asarray(ck.c),
                   np.asarray(b.nodes), np.asarray(b.weights), np.asarray(b.inverse_weights)] +
                  colmajor +
                  [np.ascontiguousarray(semi.neighbor_ids, dtype=np.int64),
                   np.ascontiguousarray(semi.orientations, dtype=np.int64),
                   np.asarray(semi.inverse_jacobian), np.asarray(semi.node_coordinates),
                   np.ascontiguousarray(u0, dtype=np.float64)]):
            f.write(np.ascontiguousarray(a).tobytes())


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("name", sorted(CASES))
def test_shim_calling_convention_matches_the_oracle(driver, tmp_path, name, precision):
    semi, orc = build(CASES[name], precision=precision)
    u0 = semi.compute_coefficients(0.0)
    t0, nsteps = 0.0, 3
    dt = 0.5 * orc.max_dt(u0)
    inp, out = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    _write_input(inp, semi, 0 if precision == "fp64" else 1, u0, t0, dt, nsteps)
    subprocess.run([driver, inp, out], check=True)
    res = np.fromfile(out, dtype=np.float64)
    nv = u0.size
    du, u_end, max_dt = res[:nv].reshape(u0.shape), res[nv:2 * nv].reshape(u0.shape), res[-1]

    du_ref = orc.rhs(u0, t0)
    u_ref = np.array(u0, copy=True)
    u_tmp = np.zeros_like(u_ref)
    t = t0
    for _ in range(nsteps):
        for s in range(5):
            orc.rk_stage(u_ref, u_tmp, s, t, dt)
        t += dt
    # FP64: Trixi's rhs! to 1e-12; the OrdinaryDiffEq form of the 2N stage
    # (tmp = A tmp + dt du) differs from Trixi's (u_tmp = du - a u_tmp) by
    # rounding only.  Mixed: FP32 flux arithmetic on a float-float state.
    # Mixed states are compared relative to the whole state's magnitude: FP32
    # rounding scales with |u|, not with a variable that starts at zero.
    tol_du, tol_u = (1e-12, 1e-12) if precision == "fp64" else (2e-4, 5e-5)
    for v in range(u0.shape[-1]):
        scale = np.max(np.abs(du_ref[..., v])) + 1e-300
        assert np.max(np.abs(du[..., v] - du_ref[..., v])) <= tol_du * scale, v
        uscale = np.max(np.abs(u_ref[..., v] if precision == "fp64" else u_ref)) + 1e-300
        assert np.max(np.abs(u_end[..., v] - u_ref[..., v])) <= tol_u * uscale, v
    assert max_dt == pytest.approx(orc.max_dt(u_ref), rel=1e-4 if precision == "mixed" else 1e-13)
