"""Learned shock indicator on the GPU: gradients of the hand-written
forward/backward kernels against the FP64 oracle, training on (modes, sqrt E)
pairs harvested from the method's own runs, what the trained network gains
over a network-free predictor, and deployment in place of the HG indicator
with HG as fallback and judge."""
import numpy as np
import pytest

import trixi_gb300 as T
from _gpu_cases import build
from oracle import mlp_oracle as MO
from trixi_gb300.learned import ShockIndicatorMLP

pytestmark = pytest.mark.gpu

KHI = dict(ndims=2, polydeg=3, level=5, xmin=[-1.0, -1.0], xmax=[1.0, 1.0], vi="hg",
           volume_flux="ranocha", surface_flux="llf", ic="kelvin_helmholtz",
           alpha_max=0.002, alpha_min=0.0001)
BLAST = dict(ndims=2, polydeg=3, level=5, xmin=[-1.5, -1.5], xmax=[1.5, 1.5], vi="hg",
             volume_flux="ranocha", surface_flux="llf", ic="gaussian_blast",
             ic_params=[1e-5, 1.0, 0.25], alpha_max=0.5, alpha_min=0.001)


@pytest.mark.parametrize("ndims", [2, 3])
def test_mlp_gradient_matches_oracle(ndims):
    net = ShockIndicatorMLP(ndims, 3, seed=11)
    rng = np.random.default_rng(5)
    n_in, H = net.n_inputs, net.hidden
    x = rng.standard_normal((300, n_in)).astype(np.float32)
    x /= np.linalg.norm(x, axis=1, keepdims=True)
    y = np.abs(0.05 * rng.standard_normal(300)).astype(np.float32)
    w = net.params
    g_gpu, loss_gpu = net.gradient(x, y)
    loss_ref, g_ref = MO.loss_and_grad(w, x.astype(np.float64), y.astype(np.float64), n_in, H)
    assert loss_gpu == pytest.approx(loss_ref, rel=1e-5)
    assert np.linalg.norm(g_gpu - g_ref) <= 1e-4 * np.linalg.norm(g_ref)
    # predictions of the tensor-core kernel (BF16 MMAs on hi/lo splits of the
    # FP32 layer inputs, FP32 accumulation) against the oracle of that
    # evaluation, and against the exact network
    p_gpu = net.predict(x)
    p_split, _ = MO.forward(MO.to_bf16(w), x.astype(np.float64), n_in, H, split_inputs=True)
    np.testing.assert_allclose(p_gpu, p_split, rtol=3e-5, atol=3e-6)
    p_ref, _ = MO.forward(MO.to_bf16(w), x.astype(np.float64), n_in, H)
    np.testing.assert_allclose(p_gpu, p_ref, rtol=1e-4, atol=1e-5)


def _run_and_harvest(net, case, t_end, every=10, stride=1, precision="mixed"):
    semi, _ = build(case, precision=precision)
    ctx = semi.device_context
    ctx.upload(semi.compute_coefficients(0.0))
    t, steps = 0.0, 0
    while t < t_end:
        t, n = ctx.step(every, 1.0, t_end, t)
        steps += n
        net.harvest(semi, stride=stride, phase=steps % stride)
        if n < every:
            break
    return semi, t


@pytest.fixture(scope="module")
def trained():
    net = ShockIndicatorMLP(2, 3, seed=3)
    _run_and_harvest(net, KHI, 3.0)
    _run_and_harvest(net, BLAST, 0.3)
    x, y = net.dataset()
    first = net.train(50, batch=2048, lr=2e-3)
    last = net.train(3000, batch=2048, lr=2e-3)
    return net, x, y, first, last


def test_training_reduces_loss_and_beats_a_network_free_predictor(trained):
    net, x, y, first, last = trained
    assert len(y) > 50_000
    assert last < 0.2 * first
    held = np.arange(len(y)) % 10 == 0  # rows held out of training
    pred = net.predict(x[held])
    mae_net = np.mean(np.abs(pred - y[held]))
    mae_const = np.mean(np.abs(np.median(y[~held]) - y[held]))  # best constant guess
    assert mae_net < 0.25 * mae_const
    # the decision that matters: alpha switched on (E above the HG threshold)
    thr = np.sqrt(0.5 * 10 ** (-1.8 * 4 ** 0.25))
    agree = np.mean((pred > thr) == (y[held] > thr))
    assert agree > 0.97


def test_learned_indicator_deployed_with_hg_fallback(trained):
    net = trained[0]
    semi_hg, _ = build(KHI, precision="mixed")
    semi_ml, _ = build(KHI, precision="mixed")
    u0 = semi_hg.compute_coefficients(0.0)
    res = {}
    for name, semi in (("hg", semi_hg), ("ml", semi_ml)):
        ctx = semi.device_context
        ctx.upload(u0)
        if name == "ml":
            net.deploy(semi, band=0.01)
        t, n = ctx.step(10**6, 1.0, 0.5, 0.0)
        assert t == pytest.approx(0.5)
        res[name] = ctx.download()
    pred, hg, flag, counts = net.last(semi_ml.nelements)
    assert counts[0] > 0 and counts[2] == 0  # no positivity fallbacks in KHI
    # the deployed run stays close to the HG run
    rho_hg, rho_ml = res["hg"][..., 0], res["ml"][..., 0]
    assert np.sqrt(np.mean((rho_ml - rho_hg) ** 2)) < 1e-3 * np.sqrt(np.mean(rho_hg ** 2))
    ShockIndicatorMLP.undeploy(semi_ml)


def test_deployed_predictions_equal_the_inference_kernel(trained):
    # deployment and predict() run the same tensor-core kernel: the same bits
    net = trained[0]
    semi, _ = build(KHI, precision="mixed")
    ctx = semi.device_context
    ctx.upload(semi.compute_coefficients(0.0))
    net.deploy(semi, band=0.01)
    ctx.step(40, 1.0, 10.0, 0.0)
    ctx.alpha()  # evaluates the indicator on the current state
    pred, hg, flag, _ = net.last(semi.nelements)
    n0 = net.count
    net.harvest(semi)
    x, y = net.dataset()
    x = x[n0:]
    np.testing.assert_array_equal(net.predict(x), pred)
    sqrt_thr = np.sqrt(0.5 * 10 ** (-1.8 * 4 ** 0.25))
    np.testing.assert_array_equal(flag == 1, np.abs(pred - sqrt_thr) < 0.01)
    ShockIndicatorMLP.undeploy(semi)


def test_3d_deployment_uses_the_network_and_the_hg_fallback():
    # 3D networks (64-128-128-1) deploy through the features / inference /
    # alpha kernels: the per-element predictions are the network's on the
    # current state, and elements in the band around sqrt(T) take HG
    case = dict(ndims=3, polydeg=3, level=2, xmin=[-2.0] * 3, xmax=[2.0] * 3, vi="hg",
                volume_flux="ranocha", surface_flux="llf", ic="weak_blast_wave",
                alpha_max=0.5, alpha_min=0.001)
    net = ShockIndicatorMLP(3, 3, seed=21)
    semi, _ = build(case, precision="mixed")
    ctx = semi.device_context
    ctx.upload(semi.compute_coefficients(0.0))
    net.deploy(semi, band=0.05)
    t, n = ctx.step(3, 0.5, 10.0, 0.0)
    assert n == 3 and ctx.status() == 0
    ctx.alpha()
    pred, hg, flag, counts = net.last(semi.nelements)
    n0 = net.count
    net.harvest(semi)
    x, _ = net.dataset()
    np.testing.assert_array_equal(net.predict(x[n0:]), pred)  # the same tensor-core kernel
    sqrt_thr = np.sqrt(0.5 * 10 ** (-1.8 * 4 ** 0.25))
    np.testing.assert_array_equal(flag == 1, np.abs(pred - sqrt_thr) < 0.05)
    ShockIndicatorMLP.undeploy(semi)


def test_tensor_core_network_matches_the_oracle_on_the_training_set(trained):
    # the trained network on its own harvested rows: the tcgen05 kernel against
    # the FP64 oracle of the same evaluation (hi/lo BF16 layer inputs)
    net, x, y = trained[:3]
    rows = x[::7][:20000]
    p_ref, _ = MO.forward(MO.to_bf16(net.params), rows.astype(np.float64), net.n_inputs,
                          net.hidden, split_inputs=True)
    np.testing.assert_allclose(net.predict(rows), p_ref, rtol=3e-5, atol=3e-6)


def test_training_is_reproducible_bit_for_bit():
    # gradient partial sums are reduced in a fixed order: two networks with the
    # same seed, trained on the same harvested rows, end with the same weights
    nets = [ShockIndicatorMLP(2, 3, seed=9) for _ in range(2)]
    semi, _ = build(KHI, precision="mixed")
    ctx = semi.device_context
    ctx.upload(semi.compute_coefficients(0.0))
    t = 0.0
    for _ in range(5):
        t, _n = ctx.step(20, 1.0, 3.0, t)
        for net in nets:
            net.harvest(semi, stride=3, phase=1)
    losses = [net.train(200, batch=1000, lr=2e-3) for net in nets]
    assert losses[0] == losses[1]
    np.testing.assert_array_equal(nets[0].params, nets[1].params)
    g0, l0 = nets[0].gradient(*nets[0].dataset())
    g1, l1 = nets[0].gradient(*nets[0].dataset())
    np.testing.assert_array_equal(g0, g1)
    assert l0 == l1
