"""tg_integrals_noalloc: the integrals entry point for callers that cannot
allocate device memory (and so cannot create a context).  It must give what
tg_integrals gives for the same state, call after call, while its scratch
lives in the library's static device memory.  Kept in a file that pytest
collects last, so a failure here cannot hide the other tests' results."""
import ctypes

import numpy as np
import pytest

from _gpu_cases import build, perturbed_state
from trixi_gb300 import _lib

pytestmark = pytest.mark.gpu


def _call(lib, semi, u_dev, invj_dev, out_dev, nelements=None):
    b = semi.solver.basis
    w = np.ascontiguousarray(b.weights, dtype=np.float64)
    return lib.tg_integrals_noalloc(
        semi.equations.ndims, b.polydeg, semi.nelements if nelements is None else nelements,
        semi.equations.gamma, w.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
        u_dev.data_ptr(), invj_dev.data_ptr(), out_dev.data_ptr(), None)


@pytest.mark.parametrize("ndims", [2, 3])
def test_integrals_noalloc_matches_context_integrals(ndims):
    torch = pytest.importorskip("torch")
    c = dict(ndims=ndims, polydeg=3, level=3 if ndims == 3 else 5, xmin=[-1.0] * ndims,
             xmax=[1.0] * ndims, vi="fluxdiff", volume_flux="ranocha", surface_flux="llf",
             ic="weak_blast_wave")
    semi, _ = build(c)
    u = perturbed_state(semi, seed=23)
    ctx = semi.device_context
    ctx.upload(u)
    expected = ctx.integrals()
    lib = _lib.load()
    u_dev = torch.from_numpy(u).cuda()
    invj_dev = torch.from_numpy(semi.inverse_jacobian).cuda()
    for _ in range(2):  # the shared scratch keeps the previous call's contents
        out_dev = torch.full((semi.equations.nvariables + 2,), float("nan"), dtype=torch.float64,
                             device="cuda")
        assert _call(lib, semi, u_dev, invj_dev, out_dev) == 0
        torch.cuda.synchronize()
        # same integrals summed in another order: relative 1e-12, plus round-off
        # relative to the largest integral for totals that cancel to ~0
        np.testing.assert_allclose(out_dev.cpu().numpy(), expected, rtol=1e-12,
                                   atol=1e-14 * np.max(np.abs(expected)))


def test_integrals_noalloc_rejects_meshes_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    c = dict(ndims=2, polydeg=3, level=2, xmin=[-1.0] * 2, xmax=[1.0] * 2, vi="weak",
             surface_flux="llf", ic="constant")
    semi, _ = build(c)
    lib = _lib.load()
    t = torch.zeros(1, dtype=torch.float64, device="cuda")
    rc = _call(lib, semi, t, t, t, nelements=4_194_304 + 1)
    assert rc == _lib.TG_ERR_INVALID_ARGUMENT  # before any launch
    assert "static scratch limit" in _lib.last_error()
