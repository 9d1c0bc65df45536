"""Batched ensembles of 2D semidiscretizations (C ABI ``tg_ensemble_*``).

Many independent ``SemidiscretizationHyperbolic`` instances of uneven mesh
sizes and polynomial degrees (2D, polydeg 2..4, mixed precision, one solver
type) advanced together: each 2N stage of all instances is one persistent
kernel launch and each step one CUDA graph, while every instance keeps its own
time, step size (StepsizeCallback) and state, exactly as if it were solved on
its own (``semidiscretize`` + ``solve`` per elixir in the reference,
src/semidiscretization/semidiscretization.jl:129-151,
src/time_integration/methods_2N.jl:95-168).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .semidiscretization import DeviceContext, make_config


class Ensemble:
    def __init__(self, semis, threads_per_block=0, device=0):
        semis = list(semis)
        if not semis:
            raise ValueError("an ensemble needs at least one semidiscretization")
        lib = _lib.load()
        self.lib = lib
        self.semis = semis
        n = len(semis)
        cfgs = (_lib.tg_config * n)()
        keep = []
        for i, s in enumerate(semis):
            cfg, k = make_config(s, "mixed", device)
            cfgs[i] = cfg
            keep.append(k)
        h = ctypes.c_void_p()
        rc = lib.tg_ensemble_create(cfgs, n, int(threads_per_block), ctypes.byref(h))
        if rc != _lib.TG_OK:
            raise _lib.TrixiGB300Error(rc, self._error(None))
        self.h = h
        self.contexts = []
        for i, s in enumerate(semis):
            p = ctypes.c_void_p()
            self._check(lib.tg_ensemble_context(h, i, ctypes.byref(p)))
            self.contexts.append(DeviceContext(s, "mixed", _handle=p.value))
        self.t = np.zeros(n)

    def _error(self, h):
        buf = ctypes.create_string_buffer(1024)
        self.lib.tg_ensemble_last_error(h, buf, len(buf))
        return buf.value.decode(errors="replace")

    def _check(self, rc):
        if rc != _lib.TG_OK:
            raise _lib.TrixiGB300Error(rc, self._error(self.h))

    def __len__(self):
        return len(self.semis)

    def close(self):
        if getattr(self, "h", None):
            for c in self.contexts:
                c.h = None  # owned by the ensemble
            self.lib.tg_ensemble_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def threads_per_block(self) -> int:
        return self.lib.tg_ensemble_threads_per_block(self.h)

    def upload(self, i, u, t=0.0):
        """State of instance i (Trixi layout, FP64) at time t."""
        self.contexts[i].upload(u)
        self.t[i] = t

    def upload_initial(self):
        """compute_coefficients(0) of every instance."""
        for i, s in enumerate(self.semis):
            self.upload(i, s.compute_coefficients(0.0), 0.0)

    def download(self, i, out=None):
        return self.contexts[i].download(out)

    def step(self, max_steps, cfl, t_end):
        """Advance every instance with its own CFL step size until t_end or
        max_steps steps; returns (times, steps) per instance."""
        t = np.ascontiguousarray(self.t, dtype=np.float64)
        steps = np.zeros(len(self), dtype=np.int64)
        self._check(self.lib.tg_ensemble_step(
            self.h, int(max_steps), float(cfl), float(t_end),
            t.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
            steps.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))))
        self.t = t
        return t.copy(), steps

    def autotune(self, iters=20):
        """Time every block size of the ensemble kernel on the current states
        and keep the fastest; returns (threads_per_block, ms per stage)."""
        tpb = ctypes.c_int32()
        ms = ctypes.c_double()
        self._check(self.lib.tg_ensemble_autotune(self.h, int(iters), ctypes.byref(tpb),
                                                  ctypes.byref(ms)))
        return tpb.value, ms.value

    @property
    def ndofs(self) -> int:
        return sum(s.ndofs for s in self.semis)
