"""TEST INFRASTRUCTURE ONLY -- FP64 oracle of the learned indicator's MLP.

Forward pass, mean-squared-error loss and its gradient for the network
n_in -> H -> H -> 1 (ReLU) with the parameter layout of libtrixi_gb300
(W1[H][n_in], b1[H], W2[H][H], b2[H], w3[H], b3), evaluated in float64 with
the weights rounded to bfloat16 (round to nearest even) as the GPU kernels
use them; layer inputs and accumulation are exact.  With ``split_inputs``
the inputs of the two hidden layers (the features and the first hidden
layer's activations) are replaced by the sum of their BF16 hi and lo parts,
hi = bf16(x), lo = bf16(x - hi) of the float32 value, which is what the
tensor-core inference kernel feeds its MMAs.  Used to check the GPU
forward/backward kernels.
"""
import numpy as np


def to_bf16(w):
    """Round float32 values to bfloat16 (nearest even), returned as float64."""
    b = np.ascontiguousarray(w, dtype=np.float32).view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(w, n_in, H):
    w = np.asarray(w, dtype=np.float64)
    o = 0
    W1 = w[o:o + H * n_in].reshape(H, n_in); o += H * n_in
    b1 = w[o:o + H]; o += H
    W2 = w[o:o + H * H].reshape(H, H); o += H * H
    b2 = w[o:o + H]; o += H
    w3 = w[o:o + H]; o += H
    b3 = w[o]
    return W1, b1, W2, b2, w3, b3


def split_bf16(x):
    """hi + lo with hi = bf16(x), lo = bf16(x - hi), of the float32 values of x."""
    x32 = np.asarray(x, dtype=np.float32)
    hi = to_bf16(x32)
    lo = to_bf16((x32.astype(np.float64) - hi).astype(np.float32))
    return hi + lo


def forward(w, x, n_in, H, split_inputs=False):
    """Network output and the layer inputs/activations (x as used, h1, h2)."""
    W1, b1, W2, b2, w3, b3 = unpack(w, n_in, H)
    x = split_bf16(x) if split_inputs else np.asarray(x, dtype=np.float64)
    z1 = x @ W1.T + b1
    h1 = np.maximum(z1, 0)
    if split_inputs:
        h1 = split_bf16(h1)
    z2 = h1 @ W2.T + b2
    h2 = np.maximum(z2, 0)
    return h2 @ w3 + b3, (x, h1, h2)


def loss_and_grad(w32, x, y, n_in, H):
    """MSE and its gradient with respect to the (bf16-rounded) parameters."""
    w = to_bf16(w32)
    y = np.asarray(y, dtype=np.float64)
    W1, b1, W2, b2, w3, b3 = unpack(w, n_in, H)
    out, (xu, h1, h2) = forward(w, x, n_in, H)
    n = len(y)
    r = out - y
    loss = np.mean(r ** 2)
    dout = 2 * r / n
    gw3 = h2.T @ dout
    gb3 = dout.sum()
    dz2 = np.outer(dout, w3) * (h2 > 0)
    gW2 = dz2.T @ h1
    gb2 = dz2.sum(0)
    dh1 = dz2 @ W2
    dz1 = dh1 * (h1 > 0)
    gW1 = dz1.T @ xu
    gb1 = dz1.sum(0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gw3, [gb3]])
    return loss, g
