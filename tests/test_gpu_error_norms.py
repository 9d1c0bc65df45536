"""calc_error_norms on the device (tg_error_norms) against the oracle and the
host restatement: the (2N+1)-node analyzer, the device initial conditions as
exact solutions, FP64 and float-float states, 2D and 3D."""
import numpy as np
import pytest

import trixi_gb300 as T
from _gpu_cases import IC, build, perturbed_state
from trixi_gb300.time_integration import AnalysisCallback

pytestmark = pytest.mark.gpu

CASES = [
    dict(ndims=2, polydeg=3, level=4, xmin=[0.0, 0.0], xmax=[2.0, 2.0], vi="weak",
         surface_flux="llf", ic="convergence_test", source="convergence_test"),
    dict(ndims=2, polydeg=4, level=3, xmin=[-10.0, -10.0], xmax=[10.0, 10.0], vi="weak",
         surface_flux="llf", ic="isentropic_vortex", ic_params=[1.0, 5.0]),
    dict(ndims=2, polydeg=3, level=5, xmin=[-1.0, -1.0], xmax=[1.0, 1.0], vi="hg",
         volume_flux="ranocha", surface_flux="llf", ic="kelvin_helmholtz"),
    dict(ndims=3, polydeg=3, level=2, xmin=[0.0] * 3, xmax=[2.0] * 3, vi="fluxdiff",
         volume_flux="ranocha", surface_flux="llf", ic="convergence_test",
         source="convergence_test"),
    dict(ndims=3, polydeg=2, level=2, xmin=[-np.pi] * 3, xmax=[np.pi] * 3, vi="fluxdiff",
         volume_flux="ranocha", surface_flux="llf", ic="taylor_green", ic_params=[0.1]),
]


def _close(gpu, ref, u):
    # FP64 on both sides: the norms agree to round-off of the interpolated
    # state (the errors are differences of numbers of the state's size)
    return np.all(np.abs(gpu - ref) <= 1e-12 * np.abs(ref) + 1e-14 * np.max(np.abs(u)))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("c", CASES, ids=lambda c: f"{c['ndims']}d-p{c['polydeg']}-{c['ic']}")
@pytest.mark.parametrize("perturb", [0.0, 1e-2])
def test_error_norms_on_the_device_match_the_oracle(c, precision, perturb):
    semi, orc = build(c, precision=precision)
    u = perturbed_state(semi, seed=4, amp=perturb) if perturb else semi.compute_coefficients(0.0)
    ctx = semi.device_context
    ctx.upload(u)
    t = 0.3
    l2, linf = ctx.error_norms(t)
    u_dev = ctx.download()  # the state as the device holds it (float-float for mixed)
    l2_ref, linf_ref = orc.error_norms(u_dev, t, IC[c["ic"]][1], c.get("ic_params"))
    assert _close(l2, l2_ref, u_dev) and _close(linf, linf_ref, u_dev), (l2, l2_ref, linf, linf_ref)
    # and the host restatement of calc_error_norms
    l2_h, linf_h = T.calc_error_norms(u_dev, t, semi)
    assert _close(l2, l2_h, u_dev) and _close(linf, linf_h, u_dev)


def test_error_norms_are_deterministic_and_need_no_download():
    c = CASES[3]
    semi, _ = build(c)
    ctx = semi.device_context
    ctx.upload(perturbed_state(semi, seed=2, amp=1e-3))
    a = ctx.error_norms(0.1)
    b = ctx.error_norms(0.1)
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])
    # the AnalysisCallback takes the device path on a TreeMesh
    ana = AnalysisCallback(semi)
    l2, linf = ana.finalize(None, 0.1)
    np.testing.assert_array_equal(l2, a[0])


def test_error_norms_reject_an_exact_solution_off_the_device():
    semi, _ = build(CASES[0])
    ctx = semi.device_context
    ctx.upload(semi.compute_coefficients(0.0))

    def initial_condition_custom(x, t, eq):
        return x

    with pytest.raises(NotImplementedError):
        ctx.error_norms(0.0, exact=initial_condition_custom)
