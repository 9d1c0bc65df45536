"""The MLP oracle's analytic gradient against central finite differences (CPU)."""
import numpy as np

from oracle import mlp_oracle as M


def test_mlp_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(3)
    n_in, H = 16, 8
    npar = H * n_in + 3 * H + H * H + 1
    w = rng.standard_normal(npar).astype(np.float32) * 0.3
    w = M.to_bf16(w)  # exactly representable: rounding is the identity
    x = rng.standard_normal((40, n_in))
    y = rng.standard_normal(40)
    loss, g = M.loss_and_grad(w.astype(np.float32), x, y, n_in, H)
    eps = 1e-6
    for k in rng.choice(npar, 25, replace=False):
        wp = w.copy(); wp[k] += eps
        wm = w.copy(); wm[k] -= eps
        fp = np.mean((M.forward(wp, x, n_in, H)[0] - y) ** 2)
        fm = np.mean((M.forward(wm, x, n_in, H)[0] - y) ** 2)
        assert abs((fp - fm) / (2 * eps) - g[k]) <= 1e-6 * max(1.0, abs(g[k]))


def test_bf16_rounding_is_nearest_even():
    v = np.array([1.0, 1.00390625, 1.005859375, -3.3e-3], dtype=np.float32)
    r = M.to_bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0  # tie to even
    assert r[2] == 1.0078125
    assert abs(r[3] - v[3]) <= abs(v[3]) * 2 ** -8


def test_split_bf16_inputs_represent_float32_to_2_pow_minus_16():
    # the tensor-core kernel feeds each FP32 layer input as BF16 hi + lo: the
    # pair carries 16 significant bits, and the network it evaluates stays
    # within that of the exact one
    rng = np.random.default_rng(4)
    v = rng.standard_normal(10000).astype(np.float32) * 10.0 ** rng.uniform(-4, 1, 10000)
    assert np.max(np.abs(M.split_bf16(v) - v) / np.abs(v)) <= 2.0 ** -16
    n_in, H = 16, 64
    npar = H * n_in + 3 * H + H * H + 1
    w = M.to_bf16(rng.standard_normal(npar).astype(np.float32) * 0.2)
    x = rng.standard_normal((200, n_in))
    x /= np.linalg.norm(x, axis=1, keepdims=True)
    p_exact = M.forward(w, x, n_in, H)[0]
    p_split = M.forward(w, x, n_in, H, split_inputs=True)[0]
    assert np.max(np.abs(p_split - p_exact)) <= 2.0 ** -13 * np.max(np.abs(p_exact))
