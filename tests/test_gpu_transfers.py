"""Host transfers that overlap the stepping (tg_prefetch_state,
tg_load_prefetched, tg_fetch_state on the context's copy streams): a pipelined
sequence -- the next input arriving and the previous result leaving while a
step computes -- gives the same states, bit for bit, as synchronous uploads,
steps and downloads."""
import numpy as np
import pytest

import trixi_gb300 as T
from _gpu_cases import build, perturbed_state

pytestmark = pytest.mark.gpu

KHI = dict(ndims=2, polydeg=3, level=4, xmin=[-1.0, -1.0], xmax=[1.0, 1.0], vi="hg",
           volume_flux="ranocha", surface_flux="llf", ic="kelvin_helmholtz",
           alpha_max=0.002, alpha_min=0.0001)
MMS3 = dict(ndims=3, polydeg=3, level=2, xmin=[0.0] * 3, xmax=[2.0] * 3, vi="fluxdiff",
            volume_flux="ranocha", surface_flux="llf", ic="convergence_test",
            source="convergence_test")


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("case", [KHI, MMS3], ids=["khi2d", "mms3d"])
def test_pipelined_transfers_match_synchronous(case, precision):
    torch = pytest.importorskip("torch")
    semi, _ = build(case, precision=precision)
    ctx = semi.device_context
    inputs = [perturbed_state(semi, seed=s, amp=0.01) for s in (1, 2, 3, 4)]
    ref, ref_t = [], []
    for u in inputs:
        ctx.upload(u)
        t, _ = ctx.step(2, 0.5, 10.0, 0.0)
        ref.append(ctx.download())
        ref_t.append(t)
    hin = [torch.from_numpy(np.ascontiguousarray(u).reshape(-1)).pin_memory() for u in inputs]
    hout = [torch.empty_like(hin[0]).pin_memory() for _ in inputs]
    n = len(inputs)
    ctx.prefetch(0, hin[0].data_ptr())
    for k in range(n):
        ctx.load_prefetched(k % 2)
        if k + 1 < n:
            ctx.prefetch((k + 1) % 2, hin[k + 1].data_ptr())
        if k % 2:
            ctx.step(2, 0.5, 10.0, 0.0)
        else:
            ctx.step_enqueue(2, 0.5, 10.0, 0.0)  # no host wait
        ctx.fetch(k % 2, hout[k].data_ptr())  # slot reuse waits for its previous copy
    for slot in (0, 1):
        ctx.transfer_wait(slot, 1)
    t, steps, finished = ctx.clock_read()
    assert steps == 2 and not finished and t == ref_t[-1]
    for k in range(n):
        np.testing.assert_array_equal(hout[k].numpy().reshape(semi.u_shape), ref[k])


def test_transfer_misuse_fails_loudly():
    semi, _ = build(KHI, precision="mixed")
    ctx = semi.device_context
    ctx.upload(semi.compute_coefficients(0.0))
    with pytest.raises(T.TrixiGB300Error):
        ctx.load_prefetched(0)  # nothing prefetched
    u = np.ascontiguousarray(semi.compute_coefficients(0.0))
    with pytest.raises(T.TrixiGB300Error):
        ctx.prefetch(2, u)  # slots are 0 and 1
    ctx.prefetch(1, u)
    ctx.transfer_wait(1, 0)
    ctx.load_prefetched(1)
    with pytest.raises(T.TrixiGB300Error):
        ctx.load_prefetched(1)  # consumed
    ctx.transfer_join()
    ctx.synchronize()
