"""LobattoLegendreBasis on the host (setup only; the device receives its matrices).

Follows src/solvers/dgsem/basis_lobatto_legendre.jl: nodes/weights by
Newton iteration on the Legendre polynomial (Kopriva alg. 25), barycentric
weights, the derivative matrix D (alg. 37), D_split = 2D - M^{-1}B,
D_hat = -M^{-1} D^T M and the inverse of the normalised Legendre Vandermonde
matrix; plus the (2N+1)-node analyzer used for error norms.
"""
from __future__ import annotations

import math

import numpy as np

_EPS = np.finfo(np.float64).eps


def _q_and_l(N: int, x: float):
    # calc_q_and_l, basis_lobatto_legendre.jl:643-665
    L_Nm2, L_Nm1, Ld_Nm2, Ld_Nm1 = 1.0, x, 0.0, 1.0
    L = x
    for i in range(2, N + 1):
        L = ((2 * i - 1) * x * L_Nm1 - (i - 1) * L_Nm2) / i
        Ld = Ld_Nm2 + (2 * i - 1) * L_Nm1
        L_Nm2, L_Nm1, Ld_Nm2, Ld_Nm1 = L_Nm1, L, Ld_Nm1, Ld
    q = (2.0 * N + 1) / (N + 1) * (x * L - L_Nm2)
    qder = (2.0 * N + 1) * L
    return q, qder, L


def gauss_lobatto_nodes_weights(n_nodes: int):
    """basis_lobatto_legendre.jl:570-640."""
    nodes = np.zeros(n_nodes)
    weights = np.zeros(n_nodes)
    if n_nodes == 1:
        weights[0] = 2.0
        return nodes, weights
    N = n_nodes - 1
    tol = 2 * _EPS
    nodes[0], nodes[-1] = -1.0, 1.0
    weights[0] = 2.0 / (N * (N + 1))
    weights[-1] = weights[0]
    if N > 1:
        cont1 = math.pi / N
        cont2 = 3.0 / (8 * N * math.pi)
        for i in range(1, (N + 1) // 2):
            x = -math.cos(cont1 * (i + 0.25) - cont2 / (i + 0.25))
            for _ in range(21):
                q, qder, _L = _q_and_l(N, x)
                dx = -q / qder
                x += dx
                if abs(dx) < tol * abs(x):
                    break
            _, _, L = _q_and_l(N, x)
            nodes[i] = x
            weights[i] = weights[0] / L ** 2
            nodes[N - i] = -x
            weights[N - i] = weights[i]
    if n_nodes % 2 == 1:
        _, _, L = _q_and_l(N, 0.0)
        nodes[N // 2] = 0.0
        weights[N // 2] = weights[0] / L ** 2
    return nodes, weights


def barycentric_weights(x):
    n = len(x)
    w = np.ones(n)
    for j in range(1, n):
        for k in range(j):
            w[k] *= x[k] - x[j]
            w[j] *= x[j] - x[k]
    return 1.0 / w


def polynomial_interpolation_matrix(x_in, x_out):
    """basis_lobatto_legendre.jl:471-498 (rows: output nodes)."""
    wb = barycentric_weights(x_in)
    V = np.zeros((len(x_out), len(x_in)))
    for k, xo in enumerate(x_out):
        match = False
        for j, xi in enumerate(x_in):
            if xo == xi or abs(xo - xi) <= math.sqrt(_EPS) * max(abs(xo), abs(xi)):
                V[k, j] = 1.0
                match = True
        if not match:
            t = wb / (xo - x_in)
            V[k, :] = t / t.sum()
    return V


def _legendre_normalised(N: int, x: float) -> float:
    if N == 0:
        p = 1.0
    elif N == 1:
        p = x
    else:
        p2, p1, p = 1.0, x, 0.0
        for i in range(2, N + 1):
            p = ((2 * i - 1) * x * p1 - (i - 1) * p2) / i
            p2, p1 = p1, p
    return p * math.sqrt(N + 0.5)


def _legendre_and_derivative(N: int, x: float):
    """legendre_polynomial_and_derivative, basis_lobatto_legendre.jl:677-706."""
    if N == 0:
        p, dp = 1.0, 0.0
    elif N == 1:
        p, dp = x, 1.0
    else:
        p2, p1, d2, d1 = 1.0, x, 0.0, 1.0
        p = dp = 0.0
        for i in range(2, N + 1):
            p = ((2 * i - 1) * x * p1 - (i - 1) * p2) / i
            dp = d2 + (2 * i - 1) * p1
            p2, p1, d2, d1 = p1, p, d1, dp
    return p * math.sqrt(N + 0.5), dp * math.sqrt(N + 0.5)


def gauss_nodes_weights(n_nodes: int):
    """Legendre-Gauss nodes and weights, basis_gauss_legendre.jl:149-205
    (Newton iteration on P_{N+1} from -cos(pi (2i+1) / (2N+2)))."""
    nodes = np.ones(n_nodes)
    weights = np.zeros(n_nodes)
    N = n_nodes - 1
    if N == 0:
        return np.zeros(1), np.full(1, 2.0)
    if N == 1:
        x = math.sqrt(1.0 / 3)
        return np.array([-x, x]), np.ones(2)
    tol = 2 * _EPS
    for i in range((N + 1) // 2):
        x = -math.cos(math.pi * (2 * i + 1) / (2 * N + 2))
        for _ in range(21):
            p, dp = _legendre_and_derivative(N + 1, x)
            dx = -p / dp
            x += dx
            if abs(dx) < tol * abs(x):
                break
        _, dp = _legendre_and_derivative(N + 1, x)
        nodes[i], nodes[N - i] = x, -x
        weights[i] = weights[N - i] = (2 * N + 3) / ((1 - x * x) * dp * dp)
    if n_nodes % 2 == 1:
        _, dp = _legendre_and_derivative(N + 1, 0.0)
        nodes[N // 2] = 0.0
        weights[N // 2] = (2 * N + 3) / (dp * dp)
    return nodes, weights


def lagrange_interpolating_polynomials(x: float, nodes, wbary):
    """basis_lobatto_legendre.jl:533-557."""
    p = np.zeros(len(nodes))
    ex = float(np.spacing(abs(x)))
    for i, xi in enumerate(nodes):
        if x == xi or abs(x - xi) <= ex * max(abs(x), abs(xi)):
            p[i] = 1.0
            return p
    p = wbary / (x - np.asarray(nodes))
    return p / p.sum()


class MortarL2:
    """LobattoLegendreMortarL2 = MortarL2(basis), basis_lobatto_legendre.jl:159-205
    with l2projection.jl:26-115: forward_{upper,lower} interpolate a face trace
    to the upper/lower half of the face, reverse_{upper,lower} project fluxes on
    the halves back with a Gauss-quadrature L2 projection."""

    def __init__(self, basis):
        n = basis.nnodes()
        nodes = basis.nodes
        wb = barycentric_weights(nodes)
        fwd = []
        for shift in (1.0, -1.0):
            F = np.zeros((n, n))
            for j in range(n):
                F[j, :] = lagrange_interpolating_polynomials(0.5 * (nodes[j] + shift), nodes, wb)
            fwd.append(F)
        self.forward_upper, self.forward_lower = fwd
        gn, gw = gauss_nodes_weights(n)
        gwb = barycentric_weights(gn)
        g2l = polynomial_interpolation_matrix(gn, nodes)
        l2g = polynomial_interpolation_matrix(nodes, gn)
        rev = []
        for shift in (1.0, -1.0):
            op = np.zeros((n, n))
            for j in range(n):
                p = lagrange_interpolating_polynomials(0.5 * (gn[j] + shift), gn, gwb)
                op[:, j] = 0.5 * p * gw[j] / gw
            rev.append(g2l @ op @ l2g)
        self.reverse_upper, self.reverse_lower = rev

    def __repr__(self):
        return f"LobattoLegendreMortarL2{{Float64}}(polydeg={self.forward_upper.shape[0] - 1})"


class LobattoLegendreBasis:
    """LobattoLegendreBasis(polydeg), basis_lobatto_legendre.jl:54-85."""

    def __init__(self, polydeg: int):
        if polydeg < 1:
            raise ValueError("polydeg must be >= 1")
        self.polydeg = polydeg
        n = polydeg + 1
        self.nodes, self.weights = gauss_lobatto_nodes_weights(n)
        self.inverse_weights = 1.0 / self.weights
        V = np.array([[_legendre_normalised(m, x) for m in range(n)] for x in self.nodes])
        self.inverse_vandermonde_legendre = np.linalg.inv(V)
        wb = barycentric_weights(self.nodes)
        D = np.zeros((n, n))
        for i in range(n):
            for j in range(n):
                if i != j:
                    D[i, j] = (wb[j] / wb[i]) * 1.0 / (self.nodes[i] - self.nodes[j])
                    D[i, i] -= D[i, j]
        self.derivative_matrix = D
        Ds = 2.0 * D
        Ds[0, 0] += 1.0 / self.weights[0]
        Ds[-1, -1] -= 1.0 / self.weights[-1]
        self.derivative_split = Ds
        Dh = D.T.copy()
        for m in range(n):
            for j in range(n):
                Dh[j, m] *= -self.weights[m] / self.weights[j]
        self.derivative_hat = Dh

    def nnodes(self) -> int:
        return self.polydeg + 1

    def __repr__(self):
        return f"LobattoLegendreBasis{{Float64}}(polydeg={self.polydeg})"


class LobattoLegendreAnalyzer:
    """SolutionAnalyzer(basis; analysis_polydeg = 2 polydeg), basis_lobatto_legendre.jl:274-290."""

    def __init__(self, basis: LobattoLegendreBasis, analysis_polydeg: int | None = None):
        apd = 2 * basis.polydeg if analysis_polydeg is None else analysis_polydeg
        self.nodes, self.weights = gauss_lobatto_nodes_weights(apd + 1)
        self.vandermonde = polynomial_interpolation_matrix(basis.nodes, self.nodes)
