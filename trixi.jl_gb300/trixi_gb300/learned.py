"""Learned shock indicator (host side): the MLP that predicts the
Hennemann-Gassner smoothness indicator, its harvesting, training on the GPU and
deployment with the HG indicator as fallback and judge
(libtrixi_gb300 tg_mlp_* entry points)."""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib


def _fp(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class ShockIndicatorMLP:
    """MLP n^d -> H -> H -> 1 (ReLU, BF16 weights, FP32 accumulation) predicting
    sqrt of the HG energy indicator from modal coefficients of density*pressure
    normalised to unit energy.  2D polydeg 3: 16 -> 64 -> 64 -> 1; 3D: 64 -> 128 -> 128 -> 1."""

    def __init__(self, ndims: int, polydeg: int, hidden: int = 0, seed: int = 1):
        self.lib = _lib.load()
        h = ctypes.c_void_p()
        _lib.check(self.lib.tg_mlp_create(ndims, polydeg, hidden, seed, ctypes.byref(h)))
        self.h = h
        self.ndims, self.polydeg = ndims, polydeg
        self.n_inputs = (polydeg + 1) ** ndims
        self.hidden = hidden or (64 if ndims == 2 else 128)
        n = ctypes.c_int64()
        _lib.check(self.lib.tg_mlp_nparams(self.h, ctypes.byref(n)))
        self.nparams = n.value
        self.count = 0

    def close(self):
        if getattr(self, "h", None):
            self.lib.tg_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        _lib.check(rc)

    @property
    def params(self) -> np.ndarray:
        w = np.zeros(self.nparams, dtype=np.float32)
        self._check(self.lib.tg_mlp_get_params(self.h, _fp(w)))
        return w

    @params.setter
    def params(self, w):
        w = np.ascontiguousarray(w, dtype=np.float32)
        assert w.size == self.nparams
        self._check(self.lib.tg_mlp_set_params(self.h, _fp(w)))

    def harvest(self, semi, stride: int = 1, phase: int = 0) -> int:
        """Append (features, sqrt E) of every stride-th element of the semi's
        current device state to the training set; returns the set's size."""
        tot = ctypes.c_int64()
        self._check(self.lib.tg_mlp_harvest(self.h, semi.device_context.h, stride, phase,
                                            ctypes.byref(tot)))
        self.count = tot.value
        return self.count

    def dataset(self):
        x = np.zeros((self.count, self.n_inputs), dtype=np.float32)
        y = np.zeros(self.count, dtype=np.float32)
        self._check(self.lib.tg_mlp_dataset(self.h, _fp(x), _fp(y)))
        return x, y

    def train(self, steps: int, batch: int = 4096, lr: float = 1e-3, holdout: int = 10,
              seed: int = 7) -> float:
        loss = ctypes.c_float()
        self._check(self.lib.tg_mlp_train(self.h, steps, batch, lr, holdout, seed,
                                          ctypes.byref(loss)))
        return loss.value

    def gradient(self, x, y):
        x = np.ascontiguousarray(x, dtype=np.float32)
        y = np.ascontiguousarray(y, dtype=np.float32)
        g = np.zeros(self.nparams, dtype=np.float32)
        loss = ctypes.c_float()
        self._check(self.lib.tg_mlp_gradient(self.h, _fp(x), _fp(y), len(y), _fp(g),
                                             ctypes.byref(loss)))
        return g, loss.value

    def predict(self, x) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float32)
        p = np.zeros(len(x), dtype=np.float32)
        self._check(self.lib.tg_mlp_predict(self.h, _fp(x), len(x), _fp(p)))
        return p

    def deploy(self, semi, band: float = 0.01):
        """Use the network as semi's shock indicator (HG fallback where the
        predicted sqrt(E) is within `band` of sqrt(threshold), and for
        non-positive rho*p)."""
        self._check(self.lib.tg_ctx_set_learned_indicator(semi.device_context.h, self.h, band))

    @staticmethod
    def undeploy(semi):
        _lib.check(_lib.load().tg_ctx_set_learned_indicator(semi.device_context.h, None, 0.0))

    def last(self, nelements: int):
        """Per element: predicted sqrt(E), HG logistic, fallback flag; and the
        running counts (evaluated, band fallbacks, positivity fallbacks)."""
        pred = np.zeros(nelements, dtype=np.float32)
        hg = np.zeros(nelements, dtype=np.float32)
        flag = np.zeros(nelements, dtype=np.int32)
        counts = np.zeros(3, dtype=np.uint64)
        self._check(self.lib.tg_mlp_last(self.h, _fp(pred), _fp(hg), _fp(flag), _fp(counts)))
        return pred, hg, flag, counts
