"""Error norms of the AnalysisCallback (host, FP64), analysis_dg2d.jl:95-139 / analysis_dg3d.jl:123."""
from __future__ import annotations

import numpy as np

from .basis import LobattoLegendreAnalyzer


def calc_error_norms(u, t, semi, analyzer: LobattoLegendreAnalyzer | None = None,
                     exact=None, chunk=4096):
    """L2 and Linf errors of the conservative variables against the initial
    condition at time t (or `exact`), on the (2N+1)-node analyzer.  u is None:
    the device context's state, evaluated on the device (tg_error_norms, no
    download); otherwise a host array, evaluated here in numpy."""
    if u is None:
        return semi.device_context.error_norms(t, exact=exact, analyzer=analyzer)
    if analyzer is None:
        analyzer = LobattoLegendreAnalyzer(semi.solver.basis)
    exact = exact or semi.initial_condition
    eq = semi.equations
    D = eq.ndims
    V = analyzer.vandermonde
    w = analyzer.weights
    u = np.asarray(u).reshape(semi.u_shape)
    X = semi.node_coordinates
    E = semi.nelements
    l2 = np.zeros(eq.nvariables)
    linf = np.zeros(eq.nvariables)
    if D == 2:
        W = np.einsum("j,i->ji", w, w)
    else:
        W = np.einsum("k,j,i->kji", w, w, w)
    curved = getattr(semi, "curved", False)
    vol = 0.0 if curved else semi.mesh.length_level_0 ** D
    for s in range(0, E, chunk):
        ue = u[s:s + chunk]
        xe = X[s:s + chunk]
        if D == 2:
            ua = np.einsum("aj,bi,ejiv->eabv", V, V, ue, optimize=True)
            xa = np.einsum("aj,bi,ejid->eabd", V, V, xe, optimize=True)
        else:
            ua = np.einsum("ak,bj,ci,ekjiv->eabcv", V, V, V, ue, optimize=True)
            xa = np.einsum("ak,bj,ci,ekjid->eabcd", V, V, V, xe, optimize=True)
        ue_exact = exact(xa, t, eq)
        diff = ue_exact - ua
        if curved:
            # |J| interpolated to the analyzer nodes (analysis_dg2d.jl:141-197, 3D analogue)
            if D == 2:
                ja = np.abs(np.einsum("aj,bi,eji->eab", V, V,
                                      1.0 / semi.inverse_jacobian[s:s + chunk], optimize=True))
            else:
                ja = np.abs(np.einsum("ak,bj,ci,ekji->eabc", V, V, V,
                                      1.0 / semi.inverse_jacobian[s:s + chunk], optimize=True))
            wj = W[None] * ja
            l2 += np.sum(diff ** 2 * wj[..., None], axis=tuple(range(D + 1)))
            vol += wj.sum()
        else:
            vj = (1.0 / semi.inverse_jacobian[s:s + chunk]) ** D
            wshape = (-1,) + (1,) * D + (1,)
            l2 += np.sum(diff ** 2 * W[None, ..., None] * vj.reshape(wshape),
                         axis=tuple(range(D + 1)))
        linf = np.maximum(linf, np.max(np.abs(diff), axis=tuple(range(D + 1))))
    return np.sqrt(l2 / vol), linf
