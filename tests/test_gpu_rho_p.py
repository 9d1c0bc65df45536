"""The indicator input kept on the device between stages: in mixed 2D
shock-capturing contexts each stage kernel (and an upload) writes rho*p of the
new state per node, and the next stage's indicator (HG or the learned network)
reads those values instead of the whole state.  The blending factors so
obtained equal the ones computed from the state itself, through a step, an
upload and a state handed out for writing."""
import numpy as np
import pytest

from _gpu_cases import build
from trixi_gb300.learned import ShockIndicatorMLP

pytestmark = pytest.mark.gpu

KHI = dict(ndims=2, polydeg=3, level=5, xmin=[-1.0, -1.0], xmax=[1.0, 1.0], vi="hg",
           volume_flux="ranocha", surface_flux="llf", ic="kelvin_helmholtz",
           alpha_max=0.002, alpha_min=0.0001)
BLAST = dict(ndims=2, polydeg=3, level=5, xmin=[-1.5, -1.5], xmax=[1.5, 1.5], vi="hg",
             volume_flux="ranocha", surface_flux="llf", ic="gaussian_blast",
             ic_params=[1e-5, 1.0, 0.25], alpha_max=0.5, alpha_min=0.001)


def _state_path_alpha(case, u, net=None):
    """Blending factors of state u from a fresh context, evaluated on an FP64
    device copy of u (tg_alpha with a state argument: the indicator reads that
    state, never the stored rho*p)."""
    torch = pytest.importorskip("torch")
    semi, _ = build(case, precision="mixed")
    ctx = semi.device_context
    ctx.upload(u)
    if net is not None:
        net.deploy(semi, band=0.01)
    u_dev = torch.from_numpy(np.ascontiguousarray(u).reshape(-1)).cuda()
    a = ctx.alpha(u_dev)
    torch.cuda.synchronize()
    return a


@pytest.mark.parametrize("case", [KHI, BLAST], ids=["khi", "blast"])
@pytest.mark.parametrize("learned", [False, True], ids=["hg", "learned"])
def test_indicator_from_stage_rho_p_matches_state_path(case, learned):
    semi, _ = build(case, precision="mixed")
    ctx = semi.device_context
    ctx.upload(semi.compute_coefficients(0.0))
    net = ShockIndicatorMLP(2, 3, seed=3) if learned else None
    if net is not None:
        net.deploy(semi, band=0.01)
    t, n = ctx.step(6, 1.0, 10.0, 0.0)
    assert n == 6
    a_rp = ctx.alpha()  # the last stage kernel's rho*p
    p_rp = net.last(semi.nelements)[0] if learned else None
    u = ctx.download()  # float-float -> FP64 is exact, and back
    a_state = _state_path_alpha(case, u, net)
    np.testing.assert_allclose(a_rp, a_state, rtol=0, atol=1e-6 * case["alpha_max"])
    if learned:
        # the network's own output (an untrained network may switch nothing on)
        p_state = net.last(semi.nelements)[0]
        np.testing.assert_allclose(p_rp, p_state, rtol=1e-6, atol=1e-7)
    else:
        # the same kernels' arithmetic on the same values
        assert np.max(a_state) > 0
        np.testing.assert_array_equal(a_rp, a_state)


def test_steps_after_upload_and_state_pointer_match_fresh_runs():
    # an upload, or a state pointer handed out (the caller may write through
    # it), makes the stored rho*p stale: the next step recomputes it, so the
    # trajectory equals a fresh context's
    semi, _ = build(BLAST, precision="mixed")
    ctx = semi.device_context
    u0 = semi.compute_coefficients(0.0)
    ctx.upload(u0)
    ctx.step(3, 1.0, 10.0, 0.0)
    ctx.upload(u0)  # back to the start: rho*p of the stepped state is stale now
    t, _ = ctx.step(3, 1.0, 10.0, 0.0)
    ctx.state_ptr()
    t, _ = ctx.step(2, 1.0, 10.0, t)
    u_a = ctx.download()
    semi2, _ = build(BLAST, precision="mixed")
    ctx2 = semi2.device_context
    ctx2.upload(u0)
    t2, _ = ctx2.step(5, 1.0, 10.0, 0.0)
    assert t == t2
    np.testing.assert_array_equal(u_a, ctx2.download())
