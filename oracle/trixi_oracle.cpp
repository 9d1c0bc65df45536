// TEST INFRASTRUCTURE ONLY -- the oracle.
//
// A CPU, FP64 restatement of Trixi.jl's DGSEM semidiscretization of the
// compressible Euler equations on a uniformly refined, periodic TreeMesh
// (2D and 3D), together with Trixi's own 2N low-storage Runge-Kutta driver,
// the CFL step-size rule and the error norms of its AnalysisCallback.
//
// Only the test suite, the smoke check and the CPU-baseline leg of the
// benchmark load this library.  It is never part of the product path.
//
// Each function names the reference file:line it restates (paths relative to
// the Trixi.jl source tree).  Parity of this restatement is pinned against the
// L2/Linf goldens that Trixi's own regression tests hold for the TreeMesh
// Euler elixirs (test/test_tree_2d_euler.jl, test/test_tree_3d_euler.jl).
//
// Layout conventions follow Trixi exactly:
//   u[v, i, j, (k), element]    (column-major; variables fastest)
//   node_coordinates[d, i, j, (k), element]
//   neighbor_ids[2, interface]  (1-based element ids), orientations[interface]
// Matrices are stored row-major here: M[a*n + b] = M[a, b] (0-based a, b).

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <unordered_map>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace orc {

enum VolumeIntegral { VI_WEAK = 0, VI_FLUXDIFF = 1, VI_SHOCKCAPTURING_HG = 2 };
enum Flux {
  FLUX_CENTRAL = 0,
  FLUX_RANOCHA = 1,
  FLUX_SHIMA_ETAL = 2,
  FLUX_LAX_FRIEDRICHS = 3,        // FluxLaxFriedrichs(max_abs_speed)
  FLUX_LAX_FRIEDRICHS_NAIVE = 4,  // FluxLaxFriedrichs(max_abs_speed_naive)
  FLUX_HLLC = 5,                  // flux_hllc
  FLUX_CHANDRASHEKAR = 6,         // flux_chandrashekar
  FLUX_HLLE = 7,                  // flux_hlle = FluxHLL(min_max_speed_einfeldt)
};
enum Source { SRC_NONE = 0, SRC_CONVERGENCE_TEST = 1 };
enum Boundary { BC_PERIODIC = 0, BC_DIRICHLET = 1, BC_SLIP_WALL = 2 };
enum InitialCondition {
  IC_CONSTANT = 0,
  IC_CONVERGENCE_TEST = 1,
  IC_ISENTROPIC_VORTEX = 2,
  IC_WEAK_BLAST_WAVE = 3,
  IC_KELVIN_HELMHOLTZ = 4,
  IC_TAYLOR_GREEN = 5,
  IC_GAUSSIAN_BLAST = 6,
  IC_ISENTROPIC_VORTEX_ADVECTED = 7,
  IC_BLAST_WAVE = 8,
  IC_DENSITY_PULSE = 9,
  IC_SEDOV_BLAST_WAVE = 10,
  IC_DENSITY_WAVE = 11,
  IC_MEDIUM_SEDOV_3D = 12,
};

// ---------------------------------------------------------------------------
// LGL basis: src/solvers/dgsem/basis_lobatto_legendre.jl
// ---------------------------------------------------------------------------

// calc_q_and_l, basis_lobatto_legendre.jl:643-665 (Kopriva alg. 24)
static void calc_q_and_l(int N, double x, double& q, double& qder, double& L) {
  double L_Nm2 = 1.0, L_Nm1 = x, Lder_Nm2 = 0.0, Lder_Nm1 = 1.0;
  L = x;
  for (int i = 2; i <= N; ++i) {
    L = ((2 * i - 1) * x * L_Nm1 - (i - 1) * L_Nm2) / i;
    double Lder = Lder_Nm2 + (2 * i - 1) * L_Nm1;
    L_Nm2 = L_Nm1;
    L_Nm1 = L;
    Lder_Nm2 = Lder_Nm1;
    Lder_Nm1 = Lder;
  }
  q = (2.0 * N + 1) / (N + 1) * (x * L - L_Nm2);
  qder = (2.0 * N + 1) * L;
}

// gauss_lobatto_nodes_weights, basis_lobatto_legendre.jl:570-640 (Kopriva alg. 25)
static void lgl_nodes_weights(int n_nodes, std::vector<double>& nodes,
                              std::vector<double>& weights) {
  nodes.assign(n_nodes, 0.0);
  weights.assign(n_nodes, 0.0);
  if (n_nodes == 1) {
    nodes[0] = 0;
    weights[0] = 2;
    return;
  }
  const int N = n_nodes - 1;
  const double tol = 2 * 2.220446049250313e-16;
  nodes[0] = -1;
  nodes[N] = 1;
  weights[0] = 2.0 / (N * (N + 1));
  weights[N] = weights[0];
  if (N > 1) {
    const double cont1 = M_PI / N;
    const double cont2 = 3.0 / (8 * N * M_PI);
    for (int i = 1; i <= (N + 1) / 2 - 1; ++i) {
      nodes[i] = -std::cos(cont1 * (i + 0.25) - cont2 / (i + 0.25));
      for (int k = 0; k <= 20; ++k) {
        double q, qder, L;
        calc_q_and_l(N, nodes[i], q, qder, L);
        double dx = -q / qder;
        nodes[i] += dx;
        if (std::fabs(dx) < tol * std::fabs(nodes[i])) break;
      }
      double q, qder, L;
      calc_q_and_l(N, nodes[i], q, qder, L);
      weights[i] = weights[0] / (L * L);
      nodes[N - i] = -nodes[i];
      weights[N - i] = weights[i];
    }
  }
  if (n_nodes % 2 == 1) {
    double q, qder, L;
    calc_q_and_l(N, 0.0, q, qder, L);
    nodes[N / 2] = 0;
    weights[N / 2] = weights[0] / (L * L);
  }
}

// barycentric_weights, basis_lobatto_legendre.jl:518-531
static std::vector<double> barycentric_weights(const std::vector<double>& x) {
  const int n = (int)x.size();
  std::vector<double> w(n, 1.0);
  for (int j = 1; j < n; ++j)
    for (int k = 0; k < j; ++k) {
      w[k] *= x[k] - x[j];
      w[j] *= x[j] - x[k];
    }
  for (int j = 0; j < n; ++j) w[j] = 1.0 / w[j];
  return w;
}

// polynomial_interpolation_matrix!, basis_lobatto_legendre.jl:471-498 (Kopriva alg. 32)
static std::vector<double> interpolation_matrix(const std::vector<double>& xin,
                                                const std::vector<double>& xout) {
  const int nin = (int)xin.size(), nout = (int)xout.size();
  std::vector<double> wb = barycentric_weights(xin);
  std::vector<double> V(nout * nin, 0.0);
  const double rt = 1.4901161193847656e-08;  // sqrt(eps), Julia isapprox default
  for (int k = 0; k < nout; ++k) {
    bool match = false;
    for (int j = 0; j < nin; ++j) {
      double a = xout[k], b = xin[j];
      if (a == b || std::fabs(a - b) <= rt * std::max(std::fabs(a), std::fabs(b))) {
        match = true;
        V[k * nin + j] = 1;
      }
    }
    if (!match) {
      double s = 0;
      for (int j = 0; j < nin; ++j) {
        double t = wb[j] / (xout[k] - xin[j]);
        V[k * nin + j] = t;
        s += t;
      }
      for (int j = 0; j < nin; ++j) V[k * nin + j] /= s;
    }
  }
  return V;
}

// legendre_polynomial_and_derivative, basis_lobatto_legendre.jl:677-706 (normalised)
static double legendre_normalised(int N, double x) {
  double poly;
  if (N == 0) {
    poly = 1;
  } else if (N == 1) {
    poly = x;
  } else {
    double p2 = 1, p1 = x;
    poly = 0;
    for (int i = 2; i <= N; ++i) {
      poly = ((2 * i - 1) * x * p1 - (i - 1) * p2) / i;
      p2 = p1;
      p1 = poly;
    }
  }
  return poly * std::sqrt(N + 0.5);
}

// Gauss-Jordan inverse with partial pivoting (Trixi calls LAPACK `inv`,
// basis_lobatto_legendre.jl:721).
static std::vector<double> invert(std::vector<double> A, int n) {
  std::vector<double> B(n * n, 0.0);
  for (int i = 0; i < n; ++i) B[i * n + i] = 1;
  for (int c = 0; c < n; ++c) {
    int p = c;
    for (int r = c + 1; r < n; ++r)
      if (std::fabs(A[r * n + c]) > std::fabs(A[p * n + c])) p = r;
    if (p != c)
      for (int k = 0; k < n; ++k) {
        std::swap(A[c * n + k], A[p * n + k]);
        std::swap(B[c * n + k], B[p * n + k]);
      }
    double piv = A[c * n + c];
    for (int k = 0; k < n; ++k) {
      A[c * n + k] /= piv;
      B[c * n + k] /= piv;
    }
    for (int r = 0; r < n; ++r) {
      if (r == c) continue;
      double f = A[r * n + c];
      if (f == 0) continue;
      for (int k = 0; k < n; ++k) {
        A[r * n + k] -= f * A[c * n + k];
        B[r * n + k] -= f * B[c * n + k];
      }
    }
  }
  return B;
}

// legendre_polynomial_and_derivative, basis_lobatto_legendre.jl:677-706
// (normalised by sqrt(N + 1/2))
static void legendre_and_derivative(int N, double x, double& poly, double& deriv) {
  if (N == 0) {
    poly = 1;
    deriv = 0;
  } else if (N == 1) {
    poly = x;
    deriv = 1;
  } else {
    double p2 = 1, p1 = x, d2 = 0, d1 = 1;
    poly = deriv = 0;
    for (int i = 2; i <= N; ++i) {
      poly = ((2 * i - 1) * x * p1 - (i - 1) * p2) / i;
      deriv = d2 + (2 * i - 1) * p1;
      p2 = p1;
      p1 = poly;
      d2 = d1;
      d1 = deriv;
    }
  }
  poly *= std::sqrt(N + 0.5);
  deriv *= std::sqrt(N + 0.5);
}

// gauss_nodes_weights, basis_gauss_legendre.jl:149-205 (Kopriva alg. 23):
// Newton iteration from -cos(pi (2i+1)/(2N+2)), symmetric completion.
static void gauss_nodes_weights(int n_nodes, std::vector<double>& nodes,
                                std::vector<double>& weights) {
  nodes.assign(n_nodes, 1.0);
  weights.assign(n_nodes, 0.0);
  const int N = n_nodes - 1;
  if (N == 0) {
    nodes[0] = 0;
    weights[0] = 2;
    return;
  }
  if (N == 1) {
    nodes[0] = -std::sqrt(1.0 / 3);
    nodes[1] = -nodes[0];
    weights[0] = weights[1] = 1;
    return;
  }
  const double tol = 2 * 2.220446049250313e-16;
  for (int i = 0; i <= (N + 1) / 2 - 1; ++i) {
    double x = -std::cos(M_PI * (2 * i + 1) / (2.0 * N + 2));
    for (int k = 0; k <= 20; ++k) {
      double p, dp;
      legendre_and_derivative(N + 1, x, p, dp);
      const double dx = -p / dp;
      x += dx;
      if (std::fabs(dx) < tol * std::fabs(x)) break;
    }
    double p, dp;
    legendre_and_derivative(N + 1, x, p, dp);
    nodes[i] = x;
    weights[i] = (2 * N + 3) / ((1 - x * x) * dp * dp);
    nodes[N - i] = -x;
    weights[N - i] = weights[i];
  }
  if (n_nodes % 2 == 1) {
    double p, dp;
    legendre_and_derivative(N + 1, 0.0, p, dp);
    nodes[N / 2] = 0;
    weights[N / 2] = (2 * N + 3) / (dp * dp);
  }
}

// lagrange_interpolating_polynomials, basis_lobatto_legendre.jl:533-557
static std::vector<double> lagrange_polys(double x, const std::vector<double>& nodes,
                                          const std::vector<double>& wbary) {
  const int n = (int)nodes.size();
  std::vector<double> p(n, 0.0);
  const double ex = std::nextafter(std::fabs(x), INFINITY) - std::fabs(x);  // eps(x)
  for (int i = 0; i < n; ++i)
    if (x == nodes[i] || std::fabs(x - nodes[i]) <= ex * std::max(std::fabs(x), std::fabs(nodes[i]))) {
      p[i] = 1;
      return p;
    }
  double total = 0;
  for (int i = 0; i < n; ++i) {
    p[i] = wbary[i] / (x - nodes[i]);
    total += p[i];
  }
  for (int i = 0; i < n; ++i) p[i] /= total;
  return p;
}

static std::vector<double> matmul(const std::vector<double>& A, const std::vector<double>& B,
                                  int n) {
  std::vector<double> C(n * n, 0.0);
  for (int i = 0; i < n; ++i)
    for (int k = 0; k < n; ++k)
      for (int j = 0; j < n; ++j) C[i * n + j] += A[i * n + k] * B[k * n + j];
  return C;
}

struct Basis {
  int n = 0;
  std::vector<double> nodes, weights, inv_weights;
  std::vector<double> D, Dhat, Dsplit, Vinv;  // n x n, row-major
  // analyzer (AnalysisCallback default analysis_polydeg = 2*polydeg,
  // basis_lobatto_legendre.jl:274-290)
  int na = 0;
  std::vector<double> anodes, aweights, avand;  // avand: na x n
  // MortarL2(basis), basis_lobatto_legendre.jl:159-205: forward (interpolation
  // to the lower/upper half) and reverse (Gauss-quadrature L2 projection back)
  std::vector<double> fwd[2], rev[2];  // [0]: lower, [1]: upper; n x n
};

// calc_forward_{upper,lower}, calc_reverse_{upper,lower}(::Val{:gauss}),
// l2projection.jl:26-115
static void make_mortar(Basis& b) {
  const int n = b.n;
  std::vector<double> wb = barycentric_weights(b.nodes);
  for (int h = 0; h < 2; ++h) {
    const double shift = h ? 1.0 : -1.0;
    b.fwd[h].assign(n * n, 0.0);
    for (int j = 0; j < n; ++j) {
      std::vector<double> p = lagrange_polys(0.5 * (b.nodes[j] + shift), b.nodes, wb);
      for (int i = 0; i < n; ++i) b.fwd[h][j * n + i] = p[i];
    }
  }
  std::vector<double> gn, gw;
  gauss_nodes_weights(n, gn, gw);
  std::vector<double> gwb = barycentric_weights(gn);
  std::vector<double> g2l = interpolation_matrix(gn, b.nodes);
  std::vector<double> l2g = interpolation_matrix(b.nodes, gn);
  for (int h = 0; h < 2; ++h) {
    const double shift = h ? 1.0 : -1.0;
    std::vector<double> op(n * n, 0.0);
    for (int j = 0; j < n; ++j) {
      std::vector<double> p = lagrange_polys(0.5 * (gn[j] + shift), gn, gwb);
      for (int i = 0; i < n; ++i) op[i * n + j] = 0.5 * p[i] * gw[j] / gw[i];
    }
    b.rev[h] = matmul(matmul(g2l, op, n), l2g, n);
  }
}

// LobattoLegendreBasis(RealT, polydeg), basis_lobatto_legendre.jl:54-85
static Basis make_basis(int polydeg) {
  Basis b;
  b.n = polydeg + 1;
  const int n = b.n;
  lgl_nodes_weights(n, b.nodes, b.weights);
  b.inv_weights.resize(n);
  for (int i = 0; i < n; ++i) b.inv_weights[i] = 1.0 / b.weights[i];
  // vandermonde_legendre + inv, basis_lobatto_legendre.jl:709-724
  std::vector<double> V(n * n);
  for (int i = 0; i < n; ++i)
    for (int m = 0; m < n; ++m) V[i * n + m] = legendre_normalised(m, b.nodes[i]);
  b.Vinv = invert(V, n);
  // polynomial_derivative_matrix, basis_lobatto_legendre.jl:427-440 (Kopriva alg. 37)
  std::vector<double> wb = barycentric_weights(b.nodes);
  b.D.assign(n * n, 0.0);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j)
      if (j != i) {
        b.D[i * n + j] = (wb[j] / wb[i]) * 1.0 / (b.nodes[i] - b.nodes[j]);
        b.D[i * n + i] -= b.D[i * n + j];
      }
  // calc_Dsplit, basis_lobatto_legendre.jl:414-424
  b.Dsplit.resize(n * n);
  for (int k = 0; k < n * n; ++k) b.Dsplit[k] = 2 * b.D[k];
  b.Dsplit[0] += 1.0 / b.weights[0];
  b.Dsplit[n * n - 1] -= 1.0 / b.weights[n - 1];
  // calc_Dhat, basis_lobatto_legendre.jl:399-409
  b.Dhat.resize(n * n);
  for (int j = 0; j < n; ++j)
    for (int m = 0; m < n; ++m) b.Dhat[j * n + m] = b.D[m * n + j];
  for (int m = 0; m < n; ++m)
    for (int j = 0; j < n; ++j) b.Dhat[j * n + m] *= -b.weights[m] / b.weights[j];
  // analyzer
  b.na = 2 * polydeg + 1;
  lgl_nodes_weights(b.na, b.anodes, b.aweights);
  b.avand = interpolation_matrix(b.nodes, b.anodes);
  make_mortar(b);
  return b;
}

// ---------------------------------------------------------------------------
// Euler physics: src/equations/compressible_euler_{2,3}d.jl,
// src/equations/numerical_fluxes.jl, src/auxiliary/math.jl
// ---------------------------------------------------------------------------

struct Eq {
  int D = 2;
  int NV = 4;
  double gamma = 1.4;
  double inv_gamma_minus_one = 2.5;
};

// cons2prim, compressible_euler_2d.jl:2038-2046 / 3d analogue
static inline void cons2prim(const Eq& eq, const double* u, double* prim) {
  const double rho = u[0];
  double ke = 0;
  for (int d = 0; d < eq.D; ++d) {
    prim[1 + d] = u[1 + d] / rho;
    ke += u[1 + d] * prim[1 + d];
  }
  prim[0] = rho;
  prim[eq.NV - 1] = (eq.gamma - 1) * (u[eq.NV - 1] - 0.5 * ke);
}

// flux(u, orientation), compressible_euler_2d.jl:415-432, 3d.jl:420-447
static inline void flux_phys(const Eq& eq, const double* u, int o, double* f) {
  double prim[5];
  cons2prim(eq, u, prim);
  const double p = prim[eq.NV - 1];
  const double rvo = u[1 + o];
  f[0] = rvo;
  for (int d = 0; d < eq.D; ++d) f[1 + d] = rvo * prim[1 + d];
  f[1 + o] += p;
  f[eq.NV - 1] = (u[eq.NV - 1] + p) * prim[1 + o];
}

// ln_mean / inv_ln_mean, math.jl:198-210, 238-250
static inline double ln_mean(double x, double y) {
  const double f2 = (x * (x - 2 * y) + y * y) / (x * (x + 2 * y) + y * y);
  if (f2 < 1.0e-4)
    return (x + y) / (2 + f2 * (2.0 / 3 + f2 * (2.0 / 5 + f2 * (2.0 / 7))));
  return (y - x) / std::log(y / x);
}
static inline double inv_ln_mean(double x, double y) {
  const double f2 = (x * (x - 2 * y) + y * y) / (x * (x + 2 * y) + y * y);
  if (f2 < 1.0e-4)
    return (2 + f2 * (2.0 / 3 + f2 * (2.0 / 5 + f2 * (2.0 / 7)))) / (x + y);
  return std::log(y / x) / (y - x);
}

// flux_ranocha, compressible_euler_2d.jl:686-722, 3d.jl:746-792
static inline void flux_ranocha(const Eq& eq, const double* ul, const double* ur, int o,
                                double* f) {
  double pl[5], pr[5];
  cons2prim(eq, ul, pl);
  cons2prim(eq, ur, pr);
  const int P = eq.NV - 1;
  const double rho_mean = ln_mean(pl[0], pr[0]);
  const double inv_rho_p_mean = pl[P] * pr[P] * inv_ln_mean(pl[0] * pr[P], pr[0] * pl[P]);
  double vavg[3] = {0, 0, 0}, vsq = 0;
  for (int d = 0; d < eq.D; ++d) {
    vavg[d] = 0.5 * (pl[1 + d] + pr[1 + d]);
    vsq += pl[1 + d] * pr[1 + d];
  }
  vsq *= 0.5;
  const double p_avg = 0.5 * (pl[P] + pr[P]);
  const double f1 = rho_mean * vavg[o];
  f[0] = f1;
  for (int d = 0; d < eq.D; ++d) f[1 + d] = f1 * vavg[d];
  f[1 + o] += p_avg;
  f[P] = f1 * (vsq + inv_rho_p_mean * eq.inv_gamma_minus_one) +
         0.5 * (pl[P] * pr[1 + o] + pr[P] * pl[1 + o]);
}

// flux_chandrashekar, compressible_euler_2d.jl (orientation method), 3d.jl:640-692
static inline void flux_chandrashekar(const Eq& eq, const double* ul, const double* ur, int o,
                                      double* f) {
  double pl[5], pr[5];
  cons2prim(eq, ul, pl);
  cons2prim(eq, ur, pr);
  const int P = eq.NV - 1;
  const double beta_ll = 0.5 * pl[0] / pl[P], beta_rr = 0.5 * pr[0] / pr[P];
  double kin_ll = 0, kin_rr = 0, vavg[3] = {0, 0, 0};
  for (int d = 0; d < eq.D; ++d) {
    kin_ll += pl[1 + d] * pl[1 + d];
    kin_rr += pr[1 + d] * pr[1 + d];
    vavg[d] = 0.5 * (pl[1 + d] + pr[1 + d]);
  }
  kin_ll *= 0.5;
  kin_rr *= 0.5;
  const double rho_avg = 0.5 * (pl[0] + pr[0]);
  const double rho_mean = ln_mean(pl[0], pr[0]);
  const double beta_mean = ln_mean(beta_ll, beta_rr);
  const double beta_avg = 0.5 * (beta_ll + beta_rr);
  const double p_mean = 0.5 * rho_avg / beta_avg;
  const double velocity_square_avg = kin_ll + kin_rr;
  const double f1 = rho_mean * vavg[o];
  f[0] = f1;
  for (int d = 0; d < eq.D; ++d) f[1 + d] = f1 * vavg[d];
  f[1 + o] += p_mean;
  double e = f1 * 0.5 * (1 / (eq.gamma - 1) / beta_mean - velocity_square_avg);
  for (int d = 0; d < eq.D; ++d) e += f[1 + d] * vavg[d];
  f[P] = e;
}

// flux_hlle = FluxHLL(min_max_speed_einfeldt): numerical_fluxes.jl:422-457,
// min_max_speed_einfeldt compressible_euler_2d.jl:1925-1963 (3d analogue)
static inline void flux_hlle(const Eq& eq, const double* ul, const double* ur, int o, double* F) {
  double pl[5], pr[5];
  cons2prim(eq, ul, pl);
  cons2prim(eq, ur, pr);
  const int P = eq.NV - 1;
  const double g = eq.gamma;
  const double Hl = (ul[P] + pl[P]) / pl[0], Hr = (ur[P] + pr[P]) / pr[0];
  const double cl = std::sqrt(g * pl[P] / pl[0]), cr = std::sqrt(g * pr[P] / pr[0]);
  const double sl = std::sqrt(pl[0]), sr = std::sqrt(pr[0]);
  const double inv = 1 / (sl + sr);
  double vroe[3] = {0, 0, 0}, vroe2 = 0;
  for (int d = 0; d < eq.D; ++d) {
    vroe[d] = (sl * pl[1 + d] + sr * pr[1 + d]) * inv;
    vroe2 += vroe[d] * vroe[d];
  }
  const double H_roe = (sl * Hl + sr * Hr) * inv;
  const double c_roe = std::sqrt((g - 1) * (H_roe - 0.5 * vroe2));
  const double beta = std::sqrt(0.5 * (g - 1) / g);
  const double lmin = std::min({vroe[o] - c_roe, pl[1 + o] - beta * cl, 0.0});
  const double lmax = std::max({vroe[o] + c_roe, pr[1 + o] + beta * cr, 0.0});
  double fl[5], fr[5];
  flux_phys(eq, ul, o, fl);
  flux_phys(eq, ur, o, fr);
  if (lmin >= 0 && lmax >= 0) {
    for (int v = 0; v < eq.NV; ++v) F[v] = fl[v];
  } else if (lmax <= 0 && lmin <= 0) {
    for (int v = 0; v < eq.NV; ++v) F[v] = fr[v];
  } else {
    const double id = 1 / (lmax - lmin);
    const double fac_ll = lmax * id, fac_rr = lmin * id, fac_diss = lmin * lmax * id;
    for (int v = 0; v < eq.NV; ++v) F[v] = fac_ll * fl[v] - fac_rr * fr[v] + fac_diss * (ur[v] - ul[v]);
  }
}

// flux_shima_etal, compressible_euler_2d.jl:466-495, 3d analogue
static inline void flux_shima(const Eq& eq, const double* ul, const double* ur, int o,
                              double* f) {
  double pl[5], pr[5];
  cons2prim(eq, ul, pl);
  cons2prim(eq, ur, pr);
  const int P = eq.NV - 1;
  const double rho_avg = 0.5 * (pl[0] + pr[0]);
  double vavg[3] = {0, 0, 0}, kin = 0;
  for (int d = 0; d < eq.D; ++d) {
    vavg[d] = 0.5 * (pl[1 + d] + pr[1 + d]);
    kin += pl[1 + d] * pr[1 + d];
  }
  kin *= 0.5;
  const double p_avg = 0.5 * (pl[P] + pr[P]);
  const double pv_avg = 0.5 * (pl[P] * pr[1 + o] + pr[P] * pl[1 + o]);
  const double f1 = rho_avg * vavg[o];
  f[0] = f1;
  for (int d = 0; d < eq.D; ++d) f[1 + d] = f1 * vavg[d];
  f[1 + o] += p_avg;
  f[P] = p_avg * vavg[o] * eq.inv_gamma_minus_one + f1 * kin + pv_avg;
}

// flux_central, numerical_fluxes.jl:17-25
static inline void flux_central(const Eq& eq, const double* ul, const double* ur, int o,
                                double* f) {
  double fl[5], fr[5];
  flux_phys(eq, ul, o, fl);
  flux_phys(eq, ur, o, fr);
  for (int v = 0; v < eq.NV; ++v) f[v] = 0.5 * (fl[v] + fr[v]);
}

// max_abs_speed / max_abs_speed_naive, compressible_euler_2d.jl:1423-1482
static inline double max_abs_speed(const Eq& eq, const double* ul, const double* ur, int o,
                                   bool naive) {
  double pl[5], pr[5];
  cons2prim(eq, ul, pl);
  cons2prim(eq, ur, pr);
  const int P = eq.NV - 1;
  const double vl = pl[1 + o], vr = pr[1 + o];
  const double cl = std::sqrt(eq.gamma * pl[P] / pl[0]);
  const double cr = std::sqrt(eq.gamma * pr[P] / pr[0]);
  if (naive) return std::max(std::fabs(vl), std::fabs(vr)) + std::max(cl, cr);
  return std::max(std::fabs(vl) + cl, std::fabs(vr) + cr);
}

// FluxLaxFriedrichs = flux_central + DissipationLocalLaxFriedrichs,
// numerical_fluxes.jl:32-45, 166-178, 222-253
static inline void flux_llf(const Eq& eq, const double* ul, const double* ur, int o,
                            bool naive, double* f) {
  flux_central(eq, ul, ur, o, f);
  const double lam = max_abs_speed(eq, ul, ur, o, naive);
  for (int v = 0; v < eq.NV; ++v) f[v] = f[v] + (-0.5 * lam * (ur[v] - ul[v]));
}

// flux_hllc, compressible_euler_2d.jl:1720-1816, 3d.jl:1423-1541 (Toro's HLLC
// with Roe-average and Einfeldt-type bounds on the signal speeds)
static inline void flux_hllc(const Eq& eq, const double* ul, const double* ur, int o, double* F) {
  const int D = eq.D, NV = eq.NV;
  const double g = eq.gamma;
  double vl[3] = {0, 0, 0}, vr[3] = {0, 0, 0}, v2l = 0, v2r = 0;
  for (int d = 0; d < D; ++d) {
    vl[d] = ul[1 + d] / ul[0];
    vr[d] = ur[1 + d] / ur[0];
    v2l += vl[d] * vl[d];
    v2r += vr[d] * vr[d];
  }
  const double rl = ul[0], rr = ur[0];
  const double el = ul[NV - 1] / rl, er = ur[NV - 1] / rr;
  const double pl = (g - 1) * (ul[NV - 1] - 0.5 * rl * v2l);
  const double pr = (g - 1) * (ur[NV - 1] - 0.5 * rr * v2r);
  const double cl = std::sqrt(g * pl / rl), cr = std::sqrt(g * pr / rr);
  double fl[5], fr[5];
  flux_phys(eq, ul, o, fl);
  flux_phys(eq, ur, o, fr);
  const double sl = std::sqrt(rl), sr = std::sqrt(rr), ss = sl + sr;
  const double vel_L = vl[o], vel_R = vr[o];
  const double vel_roe = (sl * vel_L + sr * vel_R) / ss;
  double vroe2 = 0;
  for (int d = 0; d < D; ++d) {
    const double vroe = sl * vl[d] + sr * vr[d];
    vroe2 += vroe * vroe;
  }
  const double vel_roe_mag = vroe2 / (ss * ss);
  const double Hl = (ul[NV - 1] + pl) / rl, Hr = (ur[NV - 1] + pr) / rr;
  const double H_roe = (sl * Hl + sr * Hr) / ss;
  const double c_roe = std::sqrt((g - 1) * (H_roe - 0.5 * vel_roe_mag));
  const double Ssl = std::min(vel_L - cl, vel_roe - c_roe);
  const double Ssr = std::max(vel_R + cr, vel_roe + c_roe);
  const double sMu_L = Ssl - vel_L, sMu_R = Ssr - vel_R;
  if (Ssl >= 0) {
    for (int v = 0; v < NV; ++v) F[v] = fl[v];
    return;
  }
  if (Ssr <= 0) {
    for (int v = 0; v < NV; ++v) F[v] = fr[v];
    return;
  }
  const double SStar =
      (pr - pl + rl * vel_L * sMu_L - rr * vel_R * sMu_R) / (rl * sMu_L - rr * sMu_R);
  const bool left = Ssl <= 0 && 0 <= SStar;
  const double* u = left ? ul : ur;
  const double* f = left ? fl : fr;
  const double* vv = left ? vl : vr;
  const double S = left ? Ssl : Ssr, sMu = left ? sMu_L : sMu_R, rho = left ? rl : rr;
  const double vel = left ? vel_L : vel_R, e = left ? el : er, p = left ? pl : pr;
  const double densStar = rho * sMu / (S - SStar);
  const double enerStar = e + (SStar - vel) * (SStar + p / (rho * sMu));
  double UStar[5];
  UStar[0] = densStar;
  for (int d = 0; d < D; ++d) UStar[1 + d] = densStar * (d == o ? SStar : vv[d]);
  UStar[NV - 1] = densStar * enerStar;
  for (int v = 0; v < NV; ++v) F[v] = f[v] + S * (UStar[v] - u[v]);
}

static inline void two_point_flux(const Eq& eq, int kind, const double* ul, const double* ur,
                                  int o, double* f) {
  switch (kind) {
    case FLUX_CENTRAL: flux_central(eq, ul, ur, o, f); break;
    case FLUX_RANOCHA: flux_ranocha(eq, ul, ur, o, f); break;
    case FLUX_SHIMA_ETAL: flux_shima(eq, ul, ur, o, f); break;
    case FLUX_LAX_FRIEDRICHS: flux_llf(eq, ul, ur, o, false, f); break;
    case FLUX_LAX_FRIEDRICHS_NAIVE: flux_llf(eq, ul, ur, o, true, f); break;
    case FLUX_HLLC: flux_hllc(eq, ul, ur, o, f); break;
    case FLUX_CHANDRASHEKAR: flux_chandrashekar(eq, ul, ur, o, f); break;
    case FLUX_HLLE: flux_hlle(eq, ul, ur, o, f); break;
    default: for (int v = 0; v < eq.NV; ++v) f[v] = NAN;
  }
}

// max_abs_speeds, compressible_euler_2d.jl:2025-2030
static inline void max_abs_speeds(const Eq& eq, const double* u, double* lam) {
  double prim[5];
  cons2prim(eq, u, prim);
  const double c = std::sqrt(eq.gamma * prim[eq.NV - 1] / prim[0]);
  for (int d = 0; d < eq.D; ++d) lam[d] = std::fabs(prim[1 + d]) + c;
}

// density_pressure, compressible_euler_2d.jl:2205-2210, 3d analogue
static inline double density_pressure(const Eq& eq, const double* u) {
  double m2 = 0;
  for (int d = 0; d < eq.D; ++d) m2 += u[1 + d] * u[1 + d];
  return (eq.gamma - 1) * (u[0] * u[eq.NV - 1] - 0.5 * m2);
}

// source_terms_convergence_test, compressible_euler_2d.jl:116-145, 3d.jl:127-150
static inline void source_convergence(const Eq& eq, const double* x, double t, double* s) {
  const double c = 2, A = 0.1, omega = 2 * M_PI * 0.5;
  const double g = eq.gamma;
  // Julia evaluates x1 + x2 (+ x3) - t left to right
  double arg = x[0] + x[1];
  if (eq.D == 3) arg += x[2];
  arg = omega * (arg - t);
  const double si = std::sin(arg), co = std::cos(arg);
  const double rho = c + A * si;
  const double rho_x = omega * A * co;
  if (eq.D == 2) {
    const double tmp = (2 * rho - 1) * (g - 1);
    s[0] = rho_x;
    s[1] = rho_x * (1 + tmp);
    s[2] = s[1];
    s[3] = 2 * rho_x * (rho + tmp);
  } else {
    const double tmp = (2 * rho - 1.5) * (g - 1);
    s[0] = 2 * rho_x;
    s[1] = rho_x * (2 + tmp);
    s[2] = s[1];
    s[3] = s[1];
    s[4] = rho_x * (4 * rho + 3 * tmp);
  }
}

// sin(pi a) with the argument reduced to [-1, 1] first, so that integer
// arguments give an exact zero (Julia's sinpi has the same property).
static inline double sinpi(double a) {
  double r = std::fmod(a, 2.0);
  if (r > 1) r -= 2;
  if (r < -1) r += 2;
  if (r == 0 || r == 1 || r == -1) return 0.0;
  return std::sin(M_PI * r);
}

static inline void prim2cons(const Eq& eq, const double* prim, double* u) {
  u[0] = prim[0];
  double ke = 0;
  for (int d = 0; d < eq.D; ++d) {
    u[1 + d] = prim[0] * prim[1 + d];
    ke += u[1 + d] * prim[1 + d];
  }
  u[eq.NV - 1] = prim[eq.NV - 1] * eq.inv_gamma_minus_one + 0.5 * ke;
}

// Initial conditions.  params[] carries the free constants of the configurable
// ones (see each case).
static void initial_condition(const Eq& eq, int ic, const double* par, const double* x,
                              double t, double* u) {
  double prim[5];
  const int P = eq.NV - 1;
  switch (ic) {
    case IC_CONSTANT: {
      // initial_condition_constant, compressible_euler_2d.jl:71-78 / 3d.jl:71-79
      if (eq.D == 2) {
        u[0] = 1; u[1] = 0.1; u[2] = -0.2; u[3] = 10;
      } else {
        u[0] = 1; u[1] = 0.1; u[2] = -0.2; u[3] = 0.7; u[4] = 10;
      }
      return;
    }
    case IC_CONVERGENCE_TEST: {
      // initial_condition_convergence_test, compressible_euler_2d.jl:87-104, 3d.jl:93-110
      const double c = 2, A = 0.1, omega = 2 * M_PI * 0.5;
      double arg = x[0] + x[1];
      if (eq.D == 3) arg += x[2];
      const double ini = c + A * std::sin(omega * (arg - t));
      for (int v = 0; v < P; ++v) u[v] = ini;
      u[P] = ini * ini;
      return;
    }
    case IC_ISENTROPIC_VORTEX: {
      // examples/tree_2d_dgsem/elixir_euler_vortex.jl:18-52; par = {p_inf, amplitude}
      const double p0 = par ? par[0] : 25.0;
      const double amp = par ? par[1] : 5.0;
      double rho = 1, v1 = 1, v2 = 1, p = p0;
      const double rt = p / rho;
      double c0 = x[0], c1 = x[1];
      double cent0 = -c1, cent1 = c0;
      const double r2 = cent0 * cent0 + cent1 * cent1;
      const double du = amp / (2 * M_PI) * std::exp(0.5 * (1 - r2));
      const double dtemp = -(eq.gamma - 1) / (2 * eq.gamma * rt) * du * du;
      rho = rho * std::pow(1 + dtemp, 1 / (eq.gamma - 1));
      v1 = v1 + du * cent0;
      v2 = v2 + du * cent1;
      p = p * std::pow(1 + dtemp, eq.gamma / (eq.gamma - 1));
      prim[0] = rho; prim[1] = v1; prim[2] = v2; prim[3] = p;
      prim2cons(eq, prim, u);
      return;
    }
    case IC_ISENTROPIC_VORTEX_ADVECTED: {
      // examples/tree_2d_dgsem/elixir_euler_vortex_mortar.jl:18-64: the vortex
      // of elixir_euler_vortex.jl advected with the base flow (1, 1) and
      // wrapped to the nearest periodic image on [-10, 10]^2;
      // par = {p_inf, amplitude}
      const double p0 = par ? par[0] : 25.0;
      const double amp = par ? par[1] : 5.0;
      double rho = 1, v1 = 1, v2 = 1, p = p0;
      const double rt = p / rho;
      double c0 = x[0] - v1 * t, c1 = x[1] - v2 * t;
      c0 = c0 - 20.0 * std::nearbyint(c0 / 20.0);  // round-half-even, as Julia's round
      c1 = c1 - 20.0 * std::nearbyint(c1 / 20.0);
      const double cent0 = -c1, cent1 = c0;
      const double r2 = cent0 * cent0 + cent1 * cent1;
      const double du = amp / (2 * M_PI) * std::exp(0.5 * (1 - r2));
      const double dtemp = -(eq.gamma - 1) / (2 * eq.gamma * rt) * du * du;
      rho = rho * std::pow(1 + dtemp, 1 / (eq.gamma - 1));
      v1 = v1 + du * cent0;
      v2 = v2 + du * cent1;
      p = p * std::pow(1 + dtemp, eq.gamma / (eq.gamma - 1));
      prim[0] = rho; prim[1] = v1; prim[2] = v2; prim[3] = p;
      prim2cons(eq, prim, u);
      return;
    }
    case IC_DENSITY_WAVE: {
      // initial_condition_density_wave, compressible_euler_2d.jl:161-171 (2D)
      const double v1 = 0.1, v2 = 0.2;
      const double rho = 1 + 0.98 * sinpi(2 * (x[0] + x[1] - t * (v1 + v2)));
      u[0] = rho;
      u[1] = rho * v1;
      u[2] = rho * v2;
      u[3] = 20 / (eq.gamma - 1) + 0.5 * rho * (v1 * v1 + v2 * v2);
      return;
    }
    case IC_SEDOV_BLAST_WAVE: {
      // examples/tree_2d_dgsem/elixir_euler_sedov_blast_wave.jl:11-32 (2D)
      const double r = std::sqrt(x[0] * x[0] + x[1] * x[1]);
      const double r0 = 0.21875;
      const double E = 1;
      const double p_inner = 3 * (eq.gamma - 1) * E / (3 * M_PI * r0 * r0);
      prim[0] = 1;
      prim[1] = 0;
      prim[2] = 0;
      prim[3] = r > r0 ? 1.0e-5 : p_inner;
      prim2cons(eq, prim, u);
      return;
    }
    case IC_MEDIUM_SEDOV_3D: {
      // initial_condition_medium_sedov_blast_wave of
      // examples/structured_3d_dgsem/elixir_euler_sedov.jl (3D)
      const double r = std::sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
      const double r0 = 0.21875;
      const double E = 1;
      const double p_inner = 3 * (eq.gamma - 1) * E / (4 * M_PI * r0 * r0);
      prim[0] = 1;
      prim[1] = 0;
      prim[2] = 0;
      prim[3] = 0;
      prim[4] = r > r0 ? 1.0e-3 : p_inner;
      prim2cons(eq, prim, u);
      return;
    }
    case IC_DENSITY_PULSE: {
      // examples/tree_3d_dgsem/elixir_euler_amr.jl:9-25 (3D; conservative state given directly)
      const double rho = 1 + std::exp(-(x[0] * x[0] + x[1] * x[1] + x[2] * x[2])) / 2;
      u[0] = rho;
      u[1] = rho;
      u[2] = rho;
      u[3] = rho;
      u[4] = 1 / (eq.gamma - 1) + 1.0 / 2 * rho * 3;
      return;
    }
    case IC_BLAST_WAVE: {
      // the medium blast wave of examples/tree_2d_dgsem/elixir_euler_blast_wave_amr.jl:18-34
      // (Hennemann & Gassner 2020, sec. 6.3): the weak blast wave's inner state
      // in a background at p = 1e-3
      const double r = std::sqrt(x[0] * x[0] + x[1] * x[1]);
      const double phi = std::atan2(x[1], x[0]);
      const double sp = std::sin(phi), cp = std::cos(phi);
      const bool out = r > 0.5;
      prim[0] = out ? 1.0 : 1.1691;
      prim[1] = out ? 0.0 : 0.1882 * cp;
      prim[2] = out ? 0.0 : 0.1882 * sp;
      prim[3] = out ? 1.0e-3 : 1.245;
      prim2cons(eq, prim, u);
      return;
    }
    case IC_WEAK_BLAST_WAVE: {
      // initial_condition_weak_blast_wave, compressible_euler_2d.jl:245-264, 3d.jl:241-263
      if (eq.D == 2) {
        const double r = std::sqrt(x[0] * x[0] + x[1] * x[1]);
        const double phi = std::atan2(x[1], x[0]);
        const double s = std::sin(phi), c = std::cos(phi);
        const bool out = r > 0.5;
        prim[0] = out ? 1.0 : 1.1691;
        prim[1] = out ? 0.0 : 0.1882 * c;
        prim[2] = out ? 0.0 : 0.1882 * s;
        prim[3] = out ? 1.0 : 1.245;
      } else {
        const double r = std::sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
        const double phi = std::atan2(x[1], x[0]);
        const double theta = r == 0 ? 0.0 : std::acos(x[2] / r);
        const bool out = r > 0.5;
        prim[0] = out ? 1.0 : 1.1691;
        prim[1] = out ? 0.0 : 0.1882 * std::cos(phi) * std::sin(theta);
        prim[2] = out ? 0.0 : 0.1882 * std::sin(phi) * std::sin(theta);
        prim[3] = out ? 0.0 : 0.1882 * std::cos(theta);
        prim[4] = out ? 1.0 : 1.245;
      }
      prim2cons(eq, prim, u);
      return;
    }
    case IC_KELVIN_HELMHOLTZ: {
      // examples/tree_2d_dgsem/elixir_euler_kelvin_helmholtz_instability.jl:18-31
      const double slope = 15;
      const double B = std::tanh(slope * x[1] + 7.5) - std::tanh(slope * x[1] - 7.5);
      prim[0] = 0.5 + 0.75 * B;
      prim[1] = 0.5 * (B - 1);
      prim[2] = 0.1 * sinpi(2 * x[0]);
      prim[3] = 1;
      prim2cons(eq, prim, u);
      return;
    }
    case IC_TAYLOR_GREEN: {
      // examples/tree_3d_dgsem/elixir_euler_taylor_green_vortex.jl:14-30; par = {Ms}
      const double A = 1.0, Ms = par ? par[0] : 0.1, rho = 1.0;
      prim[0] = rho;
      prim[1] = A * std::sin(x[0]) * std::cos(x[1]) * std::cos(x[2]);
      prim[2] = -A * std::cos(x[0]) * std::sin(x[1]) * std::cos(x[2]);
      prim[3] = 0.0;
      double p = (A / Ms) * (A / Ms) * rho / eq.gamma;
      p = p + 1.0 / 16.0 * A * A * rho *
                  (std::cos(2 * x[0]) * std::cos(2 * x[2]) + 2 * std::cos(2 * x[1]) +
                   2 * std::cos(2 * x[0]) + std::cos(2 * x[1]) * std::cos(2 * x[2]));
      prim[4] = p;
      prim2cons(eq, prim, u);
      return;
    }
    case IC_GAUSSIAN_BLAST: {
      // Gaussian energy deposit (no reference elixir): rho = 1, p = p_bg +
      // (gamma-1) * E * exp(-r^2/w^2) / (pi w^2); par = {p_bg, E, w}
      const double pbg = par ? par[0] : 1e-5, E = par ? par[1] : 1.0, w = par ? par[2] : 0.25;
      double r2 = 0;
      for (int d = 0; d < eq.D; ++d) r2 += x[d] * x[d];
      double norm = eq.D == 2 ? M_PI * w * w : std::pow(M_PI * w * w, 1.5);
      prim[0] = 1;
      for (int d = 0; d < eq.D; ++d) prim[1 + d] = 0;
      prim[P] = pbg + (eq.gamma - 1) * E * std::exp(-r2 / (w * w)) / norm;
      prim2cons(eq, prim, u);
      return;
    }
    default:
      for (int v = 0; v < eq.NV; ++v) u[v] = NAN;
  }
}

// ---------------------------------------------------------------------------
// Mesh: TreeMesh with an initial uniform refinement and optional refinement
// patches, periodic or not (periodicity = false: faces at the domain edge are
// boundaries).
//   tree_mesh.jl:128-215 (TreeMesh, initialize!),
//   abstract_tree.jl:35-47 (has_neighbor, has_coarse_neighbor), 122-130
//   (_child_signs), 317-402 (refine_unbalanced!, refine!), 405-447
//   (refine_box!, refine_sphere!), 453-489 (rebalance!), 668-674
//   (child_coordinates);
//   containers_2d.jl:85-127 (elements), 193-284 (interfaces), 660-810
//   (mortars); containers_3d.jl:87, 229, 652-790.
// Cells live in a map keyed by (level, integer position); a same-level
// neighbour exists iff that key is present (periodic wrap from the root),
// which is what Trixi's neighbour links record.  Leaves are enumerated in
// depth-first order with children in _child_signs order, the order in which
// Trixi stores its cells (children are inserted right behind the parent).
// ---------------------------------------------------------------------------

struct Patch {
  int kind;       // 0: box (a = coordinates_min, b = coordinates_max); 1: sphere (a = center, r)
  double a[3], b[3], r;
};

struct Tree {
  struct Cell {
    int level;
    int64_t ix[3];
    double c[3];
    int64_t child0;  // index of the first child, -1 for a leaf
  };
  int D = 2;
  bool periodic = true;
  double length0 = 0;
  std::vector<Cell> cells;
  std::unordered_map<uint64_t, int64_t> index;

  static uint64_t key(int level, const int64_t* ix) {
    return ((uint64_t)level << 60) | (uint64_t)ix[0] | ((uint64_t)ix[1] << 20) |
           ((uint64_t)ix[2] << 40);
  }
  int64_t find(int level, const int64_t* ix) const {
    auto it = index.find(key(level, ix));
    return it == index.end() ? -1 : it->second;
  }
  int64_t add(int level, const int64_t* ix, const double* c) {
    Cell cl;
    cl.level = level;
    for (int d = 0; d < 3; ++d) {
      cl.ix[d] = ix[d];
      cl.c[d] = c[d];
    }
    cl.child0 = -1;
    cells.push_back(cl);
    index[key(level, ix)] = (int64_t)cells.size() - 1;
    return (int64_t)cells.size() - 1;
  }
  double length(int level) const { return length0 / (double)(1LL << level); }
  // same-level neighbour in direction dir (0:-x, 1:+x, 2:-y, ...), -1 if none
  int64_t neighbour(int64_t cell, int dir) const {
    const Cell& c = cells[cell];
    int64_t ix[3] = {c.ix[0], c.ix[1], c.ix[2]};
    const int d = dir / 2;
    const int64_t M = 1LL << c.level;
    ix[d] += (dir & 1) ? 1 : -1;
    if (ix[d] < 0 || ix[d] >= M) {
      if (!periodic) return -1;
      ix[d] = (ix[d] + M) % M;
    }
    return find(c.level, ix);
  }
  int64_t parent(int64_t cell) const {
    const Cell& c = cells[cell];
    if (c.level == 0) return -1;
    int64_t ix[3] = {c.ix[0] >> 1, c.ix[1] >> 1, c.ix[2] >> 1};
    return find(c.level - 1, ix);
  }
  bool leaf(int64_t cell) const { return cells[cell].child0 < 0; }
  // init_child! with child_coordinates: centre + sign * (parent length / 2) / 2
  void refine_cell(int64_t cell) {
    const int nch = 1 << D;
    const double child_len = length(cells[cell].level) / 2;
    int64_t first = -1;
    for (int ch = 0; ch < nch; ++ch) {
      const Cell p = cells[cell];
      int64_t ix[3] = {0, 0, 0};
      double c[3] = {0, 0, 0};
      for (int d = 0; d < D; ++d) {
        const int bit = (ch >> d) & 1;
        ix[d] = 2 * p.ix[d] + bit;
        c[d] = p.c[d] + (bit ? 1.0 : -1.0) * child_len / 2;
      }
      const int64_t id = add(p.level + 1, ix, c);
      if (ch == 0) first = id;
    }
    cells[cell].child0 = first;
  }
  int64_t child(int64_t cell, int ch) const { return cells[cell].child0 + ch; }
  void refine_unbalanced(std::vector<int64_t> ids) {
    std::sort(ids.begin(), ids.end());
    ids.erase(std::unique(ids.begin(), ids.end()), ids.end());
    for (int64_t id : ids) refine_cell(id);
  }
  // refine!(t, cell_ids): refine, then rebalance! until the 2:1 rule holds
  // across faces (Cartesian neighbours only)
  void refine(const std::vector<int64_t>& ids) {
    std::vector<int64_t> refined(ids);
    refine_unbalanced(refined);
    while (!refined.empty()) {
      std::vector<int64_t> to_refine;
      for (int64_t cell : refined)
        for (int dir = 0; dir < 2 * D; ++dir) {
          if (neighbour(cell, dir) >= 0) continue;
          const int64_t p = parent(cell);
          if (p < 0) continue;
          const int64_t pn = neighbour(p, dir);
          if (pn < 0) continue;
          to_refine.push_back(pn);
        }
      std::sort(to_refine.begin(), to_refine.end());
      to_refine.erase(std::unique(to_refine.begin(), to_refine.end()), to_refine.end());
      refine_unbalanced(to_refine);
      refined.swap(to_refine);
    }
  }
  // coarsen!(t, cell_ids), abstract_tree.jl:516-618: parents (all children
  // leaves) from the highest level down; a parent is kept when a child has a
  // same-level neighbour with children across a face that is not shared with
  // a sibling (the 2:1 rule).  Returns the parents that were coarsened.
  std::vector<int64_t> coarsen(std::vector<int64_t> ids) {
    std::stable_sort(ids.begin(), ids.end(),
                     [&](int64_t a, int64_t b) { return cells[a].level < cells[b].level; });
    std::vector<int64_t> done;
    while (!ids.empty()) {
      const int64_t cell = ids.back();
      ids.pop_back();
      bool skip = false;
      for (int ch = 0; ch < (1 << D) && !skip; ++ch) {
        const int64_t c = child(cell, ch);
        for (int dir = 0; dir < 2 * D; ++dir) {
          const int bit = (ch >> (dir / 2)) & 1;
          if (bit != (dir & 1)) continue;  // the neighbour there is a sibling
          const int64_t nb = neighbour(c, dir);
          if (nb >= 0 && !leaf(nb)) {
            skip = true;
            break;
          }
        }
      }
      if (skip) continue;
      for (int ch = 0; ch < (1 << D); ++ch) {
        const Cell& c = cells[child(cell, ch)];
        index.erase(key(c.level, c.ix));
      }
      cells[cell].child0 = -1;
      done.push_back(cell);
    }
    return done;
  }
  void leaves(int64_t cell, std::vector<int64_t>& out) const {
    if (leaf(cell)) {
      out.push_back(cell);
      return;
    }
    for (int ch = 0; ch < (1 << D); ++ch) leaves(child(cell, ch), out);
  }
  std::vector<int64_t> leaves() const {
    std::vector<int64_t> out;
    leaves(0, out);
    return out;
  }
};

struct Mesh {
  int D = 2, level = 0;
  int64_t nelem = 0, nif = 0, nmortar = 0;
  std::vector<int> elevel;               // [E] tree level
  std::vector<double> center;            // [D, E]
  std::vector<double> inverse_jacobian;  // [E]
  std::vector<double> node_coords;       // [D, n^D, E]
  std::vector<int64_t> if_left, if_right;  // 0-based
  std::vector<int> if_orient;               // 0-based orientation
  // mortars: [2^(D-1) small elements (lower(_left), ...), large], 0-based;
  // large side 0 = large element on the negative side (Trixi large_sides 1)
  std::vector<int64_t> mo_ids;
  std::vector<int> mo_large_side, mo_orient;
  // [E, 2D] across face (0:-x,1:+x,2:-y,...): a conforming neighbour (>= 0),
  // -1 for a domain boundary, -2 - m for a face of mortar m
  std::vector<int64_t> nbr;
  double length0 = 0;
  double xmin[3] = {0, 0, 0};
  std::vector<Patch> patches;
  Tree tree;
  std::vector<int64_t> leaf_cells;  // [E] tree cell of each element
};

static Mesh mesh_from_tree(const Tree& t, int level, const double* xmin, const Basis& b);

static Mesh make_mesh(int D, int level, const double* xmin, const double* xmax, const Basis& b,
                      bool periodic = true, const std::vector<Patch>& patches = {}) {
  Tree t;
  t.D = D;
  t.periodic = periodic;
  double c0[3] = {0, 0, 0};
  for (int d = 0; d < D; ++d) c0[d] = (xmin[d] + xmax[d]) / 2;
  t.length0 = xmax[0] - xmin[0];
  const int64_t root_ix[3] = {0, 0, 0};
  t.add(0, root_ix, c0);
  // refine_uniformly!: refine! of all leaves, level by level
  for (int l = 0; l < level; ++l) t.refine(t.leaves());
  // refinement patches (each one refine! of the leaves inside)
  for (const Patch& p : patches) {
    std::vector<int64_t> sel;
    for (int64_t cell : t.leaves()) {
      const double* c = t.cells[cell].c;
      bool in = true;
      if (p.kind == 0) {
        for (int d = 0; d < D; ++d) in = in && p.a[d] < c[d] && p.b[d] > c[d];
      } else {
        double r2 = 0;
        for (int d = 0; d < D; ++d) r2 += (c[d] - p.a[d]) * (c[d] - p.a[d]);
        in = r2 < p.r * p.r;
      }
      if (in) sel.push_back(cell);
    }
    if (!sel.empty()) t.refine(sel);
  }
  Mesh out = mesh_from_tree(t, level, xmin, b);
  out.patches = patches;
  return out;
}

// The elements, interfaces and mortars of the leaves of a tree
// (init_elements!, init_interfaces!, init_mortars!).
static Mesh mesh_from_tree(const Tree& t, int level, const double* xmin, const Basis& b) {
  Mesh m;
  const int D = t.D;
  m.D = D;
  m.level = level;
  m.tree = t;
  for (int d = 0; d < D; ++d) m.xmin[d] = xmin[d];
  m.length0 = t.length0;
  const std::vector<int64_t> leaves = t.leaves();
  m.leaf_cells = leaves;
  m.nelem = (int64_t)leaves.size();
  std::unordered_map<int64_t, int64_t> c2e;
  for (int64_t e = 0; e < m.nelem; ++e) c2e[leaves[e]] = e;
  const int n = b.n;
  int nn = 1;
  for (int d = 0; d < D; ++d) nn *= n;
  // init_elements!: reference_length = integrate(one, basis), node coordinates
  double reference_length = 0;
  for (int i = 0; i < n; ++i) reference_length += 1.0 * b.weights[i];
  const double reference_offset = (b.nodes[0] + b.nodes[n - 1]) / 2;
  m.elevel.resize(m.nelem);
  m.center.resize((size_t)D * m.nelem);
  m.inverse_jacobian.resize(m.nelem);
  m.node_coords.resize((size_t)D * nn * m.nelem);
  for (int64_t e = 0; e < m.nelem; ++e) {
    const Tree::Cell& c = t.cells[leaves[e]];
    m.elevel[e] = c.level;
    const double jac = t.length(c.level) / reference_length;
    m.inverse_jacobian[e] = 1.0 / jac;
    for (int d = 0; d < D; ++d) m.center[e * D + d] = c.c[d];
    for (int node = 0; node < nn; ++node) {
      int idx[3] = {node % n, (node / n) % n, node / (n * n)};
      for (int d = 0; d < D; ++d)
        m.node_coords[((size_t)e * nn + node) * D + d] = c.c[d] + jac * (b.nodes[idx[d]] - reference_offset);
    }
  }
  m.nbr.assign((size_t)m.nelem * 2 * D, -1);
  // init_interfaces!: per element, positive directions, same-level leaf neighbour
  for (int64_t e = 0; e < m.nelem; ++e)
    for (int d = 0; d < D; ++d) {
      const int64_t nc = t.neighbour(leaves[e], 2 * d + 1);
      if (nc < 0 || !t.leaf(nc)) continue;
      const int64_t r = c2e[nc];
      m.if_left.push_back(e);
      m.if_right.push_back(r);
      m.if_orient.push_back(d);
      m.nbr[e * 2 * D + 2 * d + 1] = r;
      m.nbr[r * 2 * D + 2 * d] = e;
    }
  m.nif = (int64_t)m.if_left.size();
  // init_mortars!: per element (the large one), all directions, neighbour
  // refined; the small elements are the neighbour's children facing it, in
  // child order
  const int ns = 1 << (D - 1);
  for (int64_t e = 0; e < m.nelem; ++e)
    for (int dir = 0; dir < 2 * D; ++dir) {
      const int64_t nc = t.neighbour(leaves[e], dir);
      if (nc < 0 || t.leaf(nc)) continue;
      const int d = dir / 2;
      const int want = (dir & 1) ? 0 : 1;  // children on the side facing e
      const int64_t k = (int64_t)m.mo_large_side.size();
      for (int ch = 0; ch < (1 << D); ++ch) {
        if (((ch >> d) & 1) != want) continue;
        const int64_t sc = t.child(nc, ch);
        if (!t.leaf(sc)) {
          std::fprintf(stderr, "oracle: unbalanced tree at a mortar\n");
          std::abort();
        }
        const int64_t se = c2e[sc];
        m.mo_ids.push_back(se);
        m.nbr[se * 2 * D + (dir ^ 1)] = -2 - k;
      }
      m.mo_ids.push_back(e);
      m.nbr[e * 2 * D + dir] = -2 - k;
      m.mo_large_side.push_back((dir & 1) ? 0 : 1);
      m.mo_orient.push_back(d);
    }
  m.nmortar = (int64_t)m.mo_large_side.size();
  (void)ns;
  return m;
}

// ---------------------------------------------------------------------------
// Solver
// ---------------------------------------------------------------------------

// AMRCallback + ControllerThreeLevel settings (callbacks_step/amr.jl)
struct AmrParams {
  double alpha_max = 0.5, alpha_min = 0.001;
  bool alpha_smooth = true;
  int base_level = 1, med_level = 1, max_level = 1;
  double med_threshold = 0.0, max_threshold = 1.0;
  int variable = 0;   // 0 density_pressure, 1 density
  int indicator = 0;  // 0 IndicatorHennemannGassner, 1 IndicatorMax
  int interval = 5;
  bool adapt_initial = true, initial_only_refine = true;
};

struct Solver {
  Eq eq;
  Basis b;
  Mesh m;
  int nn = 0;  // nodes per element
  int vi = VI_WEAK, vflux = FLUX_CENTRAL, sflux = FLUX_LAX_FRIEDRICHS,
      fvflux = FLUX_LAX_FRIEDRICHS;
  double alpha_max = 0.5, alpha_min = 0.001;
  bool alpha_smooth = true;
  int source = SRC_NONE;
  // boundary conditions per direction (0:-x, 1:+x, 2:-y, ...) of a
  // non-periodic mesh, and the initial condition that Dirichlet faces use
  bool periodic = true;
  int bc[6] = {0, 0, 0, 0, 0, 0};
  int bc_ic = 0;
  double bc_par[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  std::vector<double> alpha, alpha_tmp, sfv;  // sfv: [NV, n^(D-1), 2D, E]
  AmrParams amr;
  std::vector<double> u_state;  // state of the AMR entry points
  int64_t ndofs() const { return (int64_t)nn * m.nelem; }
};

static inline size_t uidx(const Solver& s, int64_t e, int node, int v) {
  return ((size_t)e * s.nn + node) * s.eq.NV + v;
}

// HG indicator: indicators.jl:114-148 + indicators_2d.jl:30-101, indicators_3d.jl:39-123
static void hg_alpha(const Solver& s, const double* u, double alpha_max, double alpha_min,
                     bool alpha_smooth, std::vector<double>& alpha, int variable = 0);

static void calc_alpha(Solver& s, const double* u) {
  hg_alpha(s, u, s.alpha_max, s.alpha_min, s.alpha_smooth, s.alpha);
}

// The HG indicator with the given parameters (IndicatorHennemannGassner, also
// as the AMR indicator of ControllerThreeLevel); variable 0 density_pressure,
// 1 density.
static void hg_alpha(const Solver& s, const double* u, double alpha_max, double alpha_min,
                     bool alpha_smooth, std::vector<double>& alpha, int variable) {
  const int n = s.b.n, D = s.eq.D, nn = s.nn;
  const double threshold = 0.5 * std::pow(10.0, -1.8 * std::pow((double)n, 0.25));
  const double o_0001 = 0.0001;
  const double parameter_s = std::log((1 - o_0001) / o_0001);
  alpha.assign(s.m.nelem, 0.0);
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < s.m.nelem; ++e) {
    double ind[512], t1[512], t2[512];
    for (int node = 0; node < nn; ++node)
      ind[node] = variable == 1 ? u[uidx(s, e, node, 0)] : density_pressure(s.eq, &u[uidx(s, e, node, 0)]);
    const double* V = s.b.Vinv.data();
    // multiply_scalar_dimensionwise!, interpolation.jl:207-234, 348-385
    double* in = ind;
    double* out = t1;
    for (int d = 0; d < D; ++d) {
      int stride = 1;
      for (int q = 0; q < d; ++q) stride *= n;
      for (int node = 0; node < nn; ++node) {
        const int i = (node / stride) % n;
        const int base = node - i * stride;
        double r = 0;
        for (int ii = 0; ii < n; ++ii) r += V[i * n + ii] * in[base + ii * stride];
        out[node] = r;
      }
      in = out;
      out = (out == t1) ? t2 : t1;
    }
    const double* modal = in;
    double e_clip2 = 0, e_clip1 = 0, e_tot = 0;
    for (int node = 0; node < nn; ++node) {
      int idx[3] = {node % n, (node / n) % n, node / (n * n)};
      int mx = 0;
      for (int d = 0; d < D; ++d) mx = std::max(mx, idx[d]);
      const double m2 = modal[node] * modal[node];
      if (mx <= n - 3) e_clip2 += m2;
      if (mx <= n - 2) e_clip1 += m2;
      e_tot += m2;
    }
    double f1 = e_tot != 0 ? (e_tot - e_clip1) / e_tot : 0.0;
    double f2 = e_clip1 != 0 ? (e_clip1 - e_clip2) / e_clip1 : 0.0;
    const double energy = std::max(f1, f2);
    double a = 1 / (1 + std::exp(-parameter_s / threshold * (energy - threshold)));
    if (a < alpha_min) a = 0;
    if (a > 1 - alpha_min) a = 1;
    alpha[e] = std::min(alpha_max, a);
  }
  if (alpha_smooth) {
    // apply_smoothing!, indicators_2d.jl:104-136
    const std::vector<double> alpha_tmp = alpha;
    for (int64_t f = 0; f < s.m.nif; ++f) {
      const int64_t l = s.m.if_left[f], r = s.m.if_right[f];
      alpha[l] = std::max({alpha_tmp[l], 0.5 * alpha_tmp[r], alpha[l]});
      alpha[r] = std::max({alpha_tmp[r], 0.5 * alpha_tmp[l], alpha[r]});
    }
    // L2 mortars: each small element with the large one (indicators_3d.jl:140-162)
    const int ns = 1 << (D - 1);
    for (int64_t k = 0; k < s.m.nmortar; ++k) {
      const int64_t* ids = &s.m.mo_ids[(size_t)k * (ns + 1)];
      const int64_t large = ids[ns];
      for (int q = 0; q < ns; ++q)
        alpha[ids[q]] = std::max({alpha_tmp[ids[q]], 0.5 * alpha_tmp[large], alpha[ids[q]]});
      for (int q = 0; q < ns; ++q)
        alpha[large] = std::max({alpha_tmp[large], 0.5 * alpha_tmp[ids[q]], alpha[large]});
    }
  }
}

// weak_form_kernel!, dg_2d.jl:195-221, dg_3d.jl:133-164
static void weak_form(const Solver& s, double* du, const double* u, int64_t e) {
  const int n = s.b.n, D = s.eq.D, NV = s.eq.NV;
  for (int node = 0; node < s.nn; ++node) {
    const double* un = &u[uidx(s, e, node, 0)];
    int idx[3] = {node % n, (node / n) % n, node / (n * n)};
    for (int d = 0; d < D; ++d) {
      double f[5];
      flux_phys(s.eq, un, d, f);
      int stride = 1;
      for (int q = 0; q < d; ++q) stride *= n;
      const int base = node - idx[d] * stride;
      for (int ii = 0; ii < n; ++ii) {
        const double fac = s.b.Dhat[ii * n + idx[d]];
        double* dt = &du[uidx(s, e, base + ii * stride, 0)];
        for (int v = 0; v < NV; ++v) dt[v] = dt[v] + fac * f[v];
      }
    }
  }
}

// flux_differencing_kernel!, dg_2d.jl:223-259, dg_3d.jl:166-214
static void flux_differencing(const Solver& s, double* du, const double* u, int64_t e,
                              double alpha) {
  const int n = s.b.n, D = s.eq.D, NV = s.eq.NV;
  for (int node = 0; node < s.nn; ++node) {
    const double* un = &u[uidx(s, e, node, 0)];
    int idx[3] = {node % n, (node / n) % n, node / (n * n)};
    for (int d = 0; d < D; ++d) {
      int stride = 1;
      for (int q = 0; q < d; ++q) stride *= n;
      const int i = idx[d];
      const int base = node - i * stride;
      for (int ii = i + 1; ii < n; ++ii) {
        const int pn = base + ii * stride;
        double f[5];
        two_point_flux(s.eq, s.vflux, un, &u[uidx(s, e, pn, 0)], d, f);
        const double f_i = alpha * s.b.Dsplit[i * n + ii];
        const double f_ii = alpha * s.b.Dsplit[ii * n + i];
        double* di = &du[uidx(s, e, node, 0)];
        double* dii = &du[uidx(s, e, pn, 0)];
        for (int v = 0; v < NV; ++v) {
          di[v] = di[v] + f_i * f[v];
          dii[v] = dii[v] + f_ii * f[v];
        }
      }
    }
  }
}

// fv_kernel! + calcflux_fv!, dg_2d.jl:407-464, dg_3d.jl:268-390
static void fv_volume(const Solver& s, double* du, const double* u, int64_t e, double alpha) {
  const int n = s.b.n, D = s.eq.D, NV = s.eq.NV;
  // fstar[d][v][node-position along d in 0..n][other node]: stored per node as
  // flux between (i-1, i) at slot i, zero at slots 0 and n.
  std::vector<double> fstar((size_t)D * (n + 1) * s.nn / n * NV, 0.0);
  const int nl = s.nn / n;  // lines per direction
  auto fidx = [&](int d, int slot, int line, int v) -> size_t {
    return (((size_t)d * (n + 1) + slot) * nl + line) * NV + v;
  };
  for (int d = 0; d < D; ++d) {
    int stride = 1;
    for (int q = 0; q < d; ++q) stride *= n;
    for (int node = 0; node < s.nn; ++node) {
      const int i = (node / stride) % n;
      if (i == 0) continue;
      const int base = node - i * stride;
      const int line = (base % stride) + (base / (stride * n)) * stride;
      double f[5];
      two_point_flux(s.eq, s.fvflux, &u[uidx(s, e, base + (i - 1) * stride, 0)],
                     &u[uidx(s, e, node, 0)], d, f);
      for (int v = 0; v < NV; ++v) fstar[fidx(d, i, line, v)] = f[v];
    }
  }
  for (int node = 0; node < s.nn; ++node) {
    double acc[5] = {0, 0, 0, 0, 0};
    for (int d = 0; d < D; ++d) {
      int stride = 1;
      for (int q = 0; q < d; ++q) stride *= n;
      const int i = (node / stride) % n;
      const int base = node - i * stride;
      const int line = (base % stride) + (base / (stride * n)) * stride;
      for (int v = 0; v < NV; ++v)
        acc[v] += s.b.inv_weights[i] * (fstar[fidx(d, i + 1, line, v)] - fstar[fidx(d, i, line, v)]);
    }
    double* dn = &du[uidx(s, e, node, 0)];
    for (int v = 0; v < NV; ++v) dn[v] += alpha * acc[v];
  }
}

// Boundary flux of one face node: BoundaryConditionDirichlet (equations.jl:164-182,
// u_inner left of the face on + faces) or boundary_condition_slip_wall on a
// TreeMesh (compressible_euler_2d.jl:322-393, 3d.jl:315-416): p* from the 1D
// pressure Riemann problem on the outward normal velocity, flux p* in the
// normal momentum and zero elsewhere.
static void boundary_flux(const Solver& s, int bc, const double* ui, int o, int side,
                          const double* x, double t, double* F) {
  const Eq& eq = s.eq;
  if (bc == BC_DIRICHLET) {
    double ub[5];
    initial_condition(eq, s.bc_ic, s.bc_par, x, t, ub);
    if (side)
      two_point_flux(eq, s.sflux, ui, ub, o, F);
    else
      two_point_flux(eq, s.sflux, ub, ui, o, F);
    return;
  }
  double w[5];
  cons2prim(eq, ui, w);
  const double rho = w[0], p = w[eq.NV - 1], g = eq.gamma;
  const double vn = side ? w[1 + o] : -w[1 + o];
  double p_star;
  if (vn <= 0) {
    const double c = std::sqrt(g * p / rho);
    const double base = 1 + 0.5 * (g - 1) * vn / c;
    p_star = base >= 0 ? p * std::pow(base, 2 * g * eq.inv_gamma_minus_one) : 0.0;
  } else {
    const double A = 2 / ((g + 1) * rho);
    const double B = p * (g - 1) / (g + 1);
    p_star = p + 0.5 * vn / A * (vn + std::sqrt(vn * vn + 4 * A * (p + B)));
  }
  for (int v = 0; v < eq.NV; ++v) F[v] = 0.0;
  F[1 + o] = p_star;
}

// rhs_hyperbolic!, dg_2d.jl:113-186
static void rhs(Solver& s, double* du, const double* u, double t) {
  const int n = s.b.n, D = s.eq.D, NV = s.eq.NV, nn = s.nn;
  const int64_t E = s.m.nelem;
  const int nf = nn / n;  // nodes per face
  // set_zero!
  std::memset(du, 0, sizeof(double) * (size_t)E * nn * NV);
  // calc_volume_integral!, calc_volume_integral.jl:180-191, 231-272
  if (s.vi == VI_SHOCKCAPTURING_HG) calc_alpha(s, u);
  const double atol = std::max(100 * 2.220446049250313e-16, std::pow(2.220446049250313e-16, 0.75));
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < E; ++e) {
    if (s.vi == VI_WEAK) {
      weak_form(s, du, u, e);
    } else if (s.vi == VI_FLUXDIFF) {
      flux_differencing(s, du, u, e, 1.0);
    } else {
      const double a = s.alpha[e];
      if (std::fabs(a) <= atol) {
        flux_differencing(s, du, u, e, 1.0);
      } else {
        flux_differencing(s, du, u, e, 1 - a);
        fv_volume(s, du, u, e, a);
      }
    }
  }
  // prolong2interfaces! + calc_interface_flux!, dg_2d.jl:515-541, 600-632
  s.sfv.resize((size_t)NV * nf * 2 * D * E);
  auto sidx = [&](int64_t e, int dir, int fn, int v) -> size_t {
    return (((size_t)e * 2 * D + dir) * nf + fn) * NV + v;
  };
#pragma omp parallel for schedule(static)
  for (int64_t f = 0; f < s.m.nif; ++f) {
    const int64_t l = s.m.if_left[f], r = s.m.if_right[f];
    const int o = s.m.if_orient[f];
    int stride = 1;
    for (int q = 0; q < o; ++q) stride *= n;
    for (int fn = 0; fn < nf; ++fn) {
      // face node fn enumerates the remaining indices in order
      const int lo = fn % stride, hi = fn / stride;
      const int base = lo + hi * stride * n;
      const double* ul = &u[uidx(s, l, base + (n - 1) * stride, 0)];
      const double* ur = &u[uidx(s, r, base, 0)];
      double F[5];
      two_point_flux(s.eq, s.sflux, ul, ur, o, F);
      for (int v = 0; v < NV; ++v) {
        s.sfv[sidx(l, 2 * o + 1, fn, v)] = F[v];
        s.sfv[sidx(r, 2 * o, fn, v)] = F[v];
      }
    }
  }
  // prolong2mortars! + calc_mortar_flux! + mortar_fluxes_to_elements!,
  // dg_2d.jl:899-1243, dg_3d.jl:770-1335: the large element's trace is
  // interpolated to each half (quarter) face, the surface flux is taken there
  // against the small element's trace, copied to the small element, and
  // L2-projected back to the large face.
  const int ns = 1 << (D - 1);
#pragma omp parallel for schedule(static)
  for (int64_t k = 0; k < s.m.nmortar; ++k) {
    const int o = s.m.mo_orient[k], ls = s.m.mo_large_side[k];
    const int64_t* ids = &s.m.mo_ids[(size_t)k * (ns + 1)];
    const int64_t large = ids[ns];
    const int dir_large = ls == 0 ? 2 * o + 1 : 2 * o;  // large face towards the small ones
    const int dir_small = dir_large ^ 1;
    int stride = 1;
    for (int q = 0; q < o; ++q) stride *= n;
    auto face_node = [&](int fn, int dir) {
      const int lo = fn % stride, hi = fn / stride;
      return lo + hi * stride * n + ((dir & 1) ? (n - 1) * stride : 0);
    };
    std::vector<double> ul((size_t)nf * NV), up((size_t)nf * NV), fs((size_t)ns * nf * NV);
    for (int fn = 0; fn < nf; ++fn)
      for (int v = 0; v < NV; ++v) ul[fn * NV + v] = u[uidx(s, large, face_node(fn, dir_large), v)];
    for (int q = 0; q < ns; ++q) {
      // u_lower / u_upper (2D) and u_{lower,upper}_{left,right} (3D): the
      // first face axis picks left/right, the second lower/upper
      const double* F1 = s.b.fwd[q & 1].data();
      const double* F2 = s.b.fwd[(q >> 1) & 1].data();
      for (int fn = 0; fn < nf; ++fn) {
        const int i = fn % n, j = fn / n;
        for (int v = 0; v < NV; ++v) {
          double r = 0;
          if (D == 2) {
            for (int a = 0; a < n; ++a) r += F1[i * n + a] * ul[a * NV + v];
          } else {
            for (int bb = 0; bb < n; ++bb)
              for (int a = 0; a < n; ++a) r += F1[i * n + a] * F2[j * n + bb] * ul[(a + bb * n) * NV + v];
          }
          up[fn * NV + v] = r;
        }
      }
      const int64_t small = ids[q];
      for (int fn = 0; fn < nf; ++fn) {
        const double* us = &u[uidx(s, small, face_node(fn, dir_small), 0)];
        double F[5];
        if (ls == 0)
          two_point_flux(s.eq, s.sflux, &up[fn * NV], us, o, F);
        else
          two_point_flux(s.eq, s.sflux, us, &up[fn * NV], o, F);
        for (int v = 0; v < NV; ++v) {
          fs[((size_t)q * nf + fn) * NV + v] = F[v];
          s.sfv[sidx(small, dir_small, fn, v)] = F[v];
        }
      }
    }
    for (int fn = 0; fn < nf; ++fn) {
      const int i = fn % n, j = fn / n;
      for (int v = 0; v < NV; ++v) {
        double r = 0;
        for (int q = 0; q < ns; ++q) {
          const double* R1 = s.b.rev[q & 1].data();
          const double* R2 = s.b.rev[(q >> 1) & 1].data();
          const double* f = &fs[(size_t)q * nf * NV];
          if (D == 2) {
            for (int a = 0; a < n; ++a) r += R1[i * n + a] * f[a * NV + v];
          } else {
            for (int bb = 0; bb < n; ++bb)
              for (int a = 0; a < n; ++a) r += R1[i * n + a] * R2[j * n + bb] * f[(a + bb * n) * NV + v];
          }
        }
        s.sfv[sidx(large, dir_large, fn, v)] = r;
      }
    }
  }
  // prolong2boundaries! + calc_boundary_flux!, dg_2d.jl:680-717, 795-860
  if (!s.periodic) {
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < E; ++e)
      for (int dir = 0; dir < 2 * D; ++dir) {
        if (s.m.nbr[e * 2 * D + dir] != -1) continue;
        const int o = dir / 2, side = dir % 2;
        int stride = 1;
        for (int q = 0; q < o; ++q) stride *= n;
        for (int fn = 0; fn < nf; ++fn) {
          const int lo = fn % stride, hi = fn / stride;
          const int node = lo + hi * stride * n + (side ? (n - 1) * stride : 0);
          double F[5];
          boundary_flux(s, s.bc[dir], &u[uidx(s, e, node, 0)], o, side,
                        &s.m.node_coords[((size_t)e * nn + node) * D], t, F);
          for (int v = 0; v < NV; ++v) s.sfv[sidx(e, dir, fn, v)] = F[v];
        }
      }
  }
  // calc_surface_integral!, dg_2d.jl:1245-1287; apply_jacobian!, dg_2d.jl:1345-1363;
  // calc_sources!, dg_2d.jl:1366-1386
  const double factor = s.b.inv_weights[0];
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < E; ++e) {
    for (int o = 0; o < D; ++o) {
      int stride = 1;
      for (int q = 0; q < o; ++q) stride *= n;
      for (int fn = 0; fn < nf; ++fn) {
        const int lo = fn % stride, hi = fn / stride;
        const int base = lo + hi * stride * n;
        double* dm = &du[uidx(s, e, base, 0)];
        double* dp = &du[uidx(s, e, base + (n - 1) * stride, 0)];
        for (int v = 0; v < NV; ++v) {
          dm[v] = dm[v] - s.sfv[sidx(e, 2 * o, fn, v)] * factor;
          dp[v] = dp[v] + s.sfv[sidx(e, 2 * o + 1, fn, v)] * factor;
        }
      }
    }
    const double fac = -s.m.inverse_jacobian[e];
    for (int node = 0; node < nn; ++node)
      for (int v = 0; v < NV; ++v) du[uidx(s, e, node, v)] *= fac;
    if (s.source == SRC_CONVERGENCE_TEST) {
      for (int node = 0; node < nn; ++node) {
        double src[5];
        source_convergence(s.eq, &s.m.node_coords[((size_t)e * nn + node) * D], t, src);
        for (int v = 0; v < NV; ++v) du[uidx(s, e, node, v)] += src[v];
      }
    }
  }
}

// max_dt, stepsize_dg2d.jl:8-30, stepsize_dg3d.jl:8-33
static double max_dt(const Solver& s, const double* u) {
  const int D = s.eq.D;
  double mss = 4.9406564584124654e-324;  // nextfloat(0.0)
  for (int64_t e = 0; e < s.m.nelem; ++e) {
    double ml[3] = {0, 0, 0};
    for (int node = 0; node < s.nn; ++node) {
      double lam[3];
      max_abs_speeds(s.eq, &u[uidx(s, e, node, 0)], lam);
      for (int d = 0; d < D; ++d) ml[d] = std::max(ml[d], lam[d]);
    }
    double sum = ml[0] + ml[1];
    if (D == 3) sum += ml[2];
    mss = std::max(mss, s.m.inverse_jacobian[e] * sum);
  }
  return 2 / (s.b.n * mss);
}

// CarpenterKennedy2N54, methods_2N.jl:24-48
static const double CK_A[5] = {0.0, 567301805773.0 / 1357537059087.0,
                                2404267990393.0 / 2016746695238.0,
                                3550918686646.0 / 2091501179385.0,
                                1275806237668.0 / 842570457699.0};
static const double CK_B[5] = {1432997174477.0 / 9575080441755.0,
                               5161836677717.0 / 13612068292357.0,
                               1720146321549.0 / 2090206949498.0,
                               3134564353537.0 / 4481467310338.0,
                               2277821191437.0 / 14882151754819.0};
static const double CK_C[5] = {0.0, 1432997174477.0 / 9575080441755.0,
                               2526269341429.0 / 6820363962896.0,
                               2006345519317.0 / 3224310063776.0,
                               2802321613138.0 / 2924317926251.0};

// One 2N stage update, methods_2N.jl:153-157
static void rk_update(int64_t ndof, double* u, double* u_tmp, const double* du, double a,
                      double b_dt) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < ndof; ++i) {
    u_tmp[i] = du[i] - u_tmp[i] * a;
    u[i] += u_tmp[i] * b_dt;
  }
}

// ---------------------------------------------------------------------------
// AMR: AMRCallback on a TreeMesh (callbacks_step/amr.jl:143-197, 244-392)
// with ControllerThreeLevel (amr.jl:984-1168) on the HG indicator, and the
// solution transfer of amr_dg2d.jl:85-485 / amr_dg3d.jl (LobattoLegendre
// AdaptorL2: the mortar matrices).
// ---------------------------------------------------------------------------


// ControllerThreeLevel: +1 refine, -1 coarsen, 0 keep
static std::vector<int> amr_controller(const Solver& s, const double* u, const AmrParams& ap) {
  std::vector<double> alpha;
  if (ap.indicator == 1) {
    // IndicatorMax, indicators_3d.jl:239-259
    alpha.assign(s.m.nelem, -INFINITY);
    for (int64_t e = 0; e < s.m.nelem; ++e)
      for (int node = 0; node < s.nn; ++node) {
        const double* un = &u[uidx(s, e, node, 0)];
        alpha[e] = std::max(alpha[e], ap.variable == 1 ? un[0] : density_pressure(s.eq, un));
      }
  } else {
    hg_alpha(s, u, ap.alpha_max, ap.alpha_min, ap.alpha_smooth, alpha, ap.variable);
  }
  std::vector<int> lambda(s.m.nelem, 0);
  for (int64_t e = 0; e < s.m.nelem; ++e) {
    const int cur = s.m.elevel[e];
    int target = cur;
    if (alpha[e] > ap.max_threshold)
      target = ap.max_level;
    else if (alpha[e] > ap.med_threshold) {
      if (ap.med_level > 0) target = ap.med_level;
    } else
      target = ap.base_level;
    lambda[e] = cur < target ? 1 : (cur > target ? -1 : 0);
  }
  return lambda;
}

// One AMR pass on the state u (resized in place): refine! (with rebalancing),
// then coarsen! of the parents whose children are all marked; refined
// elements get the tensor-product interpolation of their parent
// (refine_element!), coarsened ones the sum of the L2 projections of their
// children (coarsen_elements!).  Returns whether the mesh changed.
static bool amr_adapt_with(Solver& s, std::vector<double>& u, const std::vector<int>& lambda,
                           bool only_refine, bool only_coarsen);

static bool amr_adapt(Solver& s, std::vector<double>& u, const AmrParams& ap, bool only_refine,
                      bool only_coarsen) {
  return amr_adapt_with(s, u, amr_controller(s, u.data(), ap), only_refine, only_coarsen);
}

// The AMR pass for given controller values (+1 refine, -1 coarsen, 0 keep).
static bool amr_adapt_with(Solver& s, std::vector<double>& u, const std::vector<int>& lambda,
                           bool only_refine, bool only_coarsen) {
  const int D = s.eq.D, NV = s.eq.NV, n = s.b.n, nn = s.nn, nch = 1 << D;
  Tree& t = s.m.tree;
  const std::vector<int64_t> old_leaves = s.m.leaf_cells;
  std::unordered_map<int64_t, int64_t> old_elem;
  for (int64_t e = 0; e < (int64_t)old_leaves.size(); ++e) old_elem[old_leaves[e]] = e;
  std::vector<int64_t> to_refine, to_coarsen;
  for (int64_t e = 0; e < (int64_t)lambda.size(); ++e) {
    if (lambda[e] > 0) to_refine.push_back(old_leaves[e]);
    if (lambda[e] < 0) to_coarsen.push_back(old_leaves[e]);
  }
  bool changed = false;
  std::unordered_map<int64_t, int64_t> former_child0;  // first child of each coarsened parent
  if (!only_coarsen && !to_refine.empty()) {
    t.refine(to_refine);
    changed = true;
  }
  if (!only_refine && !to_coarsen.empty()) {
    std::unordered_map<int64_t, int> count;
    std::vector<int64_t> parents;
    for (int64_t cell : to_coarsen) {
      if (t.cells[cell].level == 0 || !t.leaf(cell)) continue;
      const int64_t p = t.parent(cell);
      if (++count[p] == nch) parents.push_back(p);
    }
    std::sort(parents.begin(), parents.end());  // cell order does not change the result
    for (int64_t p : parents) former_child0[p] = t.cells[p].child0;
    if (!t.coarsen(parents).empty()) changed = true;
  }
  if (!changed) return false;
  Mesh nm = mesh_from_tree(t, s.m.level, s.m.xmin, s.b);
  nm.patches = s.m.patches;
  std::vector<double> un((size_t)nm.nelem * nn * NV, 0.0);
  const std::vector<double>* F[2] = {&s.b.fwd[0], &s.b.fwd[1]};
  const std::vector<double>* R[2] = {&s.b.rev[0], &s.b.rev[1]};
  for (int64_t e = 0; e < nm.nelem; ++e) {
    const int64_t cell = nm.leaf_cells[e];
    double* dst = &un[(size_t)e * nn * NV];
    auto it = old_elem.find(cell);
    if (it != old_elem.end()) {
      std::memcpy(dst, &u[(size_t)it->second * nn * NV], sizeof(double) * nn * NV);
      continue;
    }
    const int64_t p = t.parent(cell);
    auto ip = p >= 0 ? old_elem.find(p) : old_elem.end();
    if (ip != old_elem.end()) {
      // child q of a refined element: forward_{lower,upper} per axis
      const int q = (int)(cell - t.cells[p].child0);
      const double* src = &u[(size_t)ip->second * nn * NV];
      for (int node = 0; node < nn; ++node) {
        const int i[3] = {node % n, (node / n) % n, node / (n * n)};
        for (int sn = 0; sn < nn; ++sn) {
          const int k[3] = {sn % n, (sn / n) % n, sn / (n * n)};
          double w = 1;
          for (int d = 0; d < D; ++d) w *= (*F[(q >> d) & 1])[i[d] * n + k[d]];
          for (int v = 0; v < NV; ++v) dst[node * NV + v] += w * src[sn * NV + v];
        }
      }
      continue;
    }
    // a coarsened parent: sum over its children of reverse_{lower,upper} per axis
    for (int q = 0; q < nch; ++q) {
      const int64_t c = former_child0.at(cell) + q;
      const double* src = &u[(size_t)old_elem.at(c) * nn * NV];
      for (int node = 0; node < nn; ++node) {
        const int i[3] = {node % n, (node / n) % n, node / (n * n)};
        for (int sn = 0; sn < nn; ++sn) {
          const int k[3] = {sn % n, (sn / n) % n, sn / (n * n)};
          double w = 1;
          for (int d = 0; d < D; ++d) w *= (*R[(q >> d) & 1])[i[d] * n + k[d]];
          for (int v = 0; v < NV; ++v) dst[node * NV + v] += w * src[sn * NV + v];
        }
      }
    }
  }
  s.m = std::move(nm);
  u.swap(un);
  return true;
}

// Julia isapprox(a, b) with default rtol = sqrt(eps)
static bool isapprox(double a, double b) {
  return a == b || (std::isfinite(a) && std::isfinite(b) &&
                    std::fabs(a - b) <= 1.4901161193847656e-08 * std::max(std::fabs(a), std::fabs(b)));
}

}  // namespace orc

using namespace orc;

extern "C" {

void* orc_create(int ndims, int polydeg, int level, const double* xmin, const double* xmax,
                 double gamma, int volume_integral, int volume_flux, int surface_flux,
                 int fv_flux, double alpha_max, double alpha_min, int alpha_smooth,
                 int source) {
  if (ndims < 2 || ndims > 3 || polydeg < 1 || polydeg > 7 || level < 0 || level > 10)
    return nullptr;
  Solver* s = new Solver();
  s->eq.D = ndims;
  s->eq.NV = ndims + 2;
  s->eq.gamma = gamma;
  s->eq.inv_gamma_minus_one = 1.0 / (gamma - 1);
  s->b = make_basis(polydeg);
  s->m = make_mesh(ndims, level, xmin, xmax, s->b);
  s->nn = 1;
  for (int d = 0; d < ndims; ++d) s->nn *= s->b.n;
  s->vi = volume_integral;
  s->vflux = volume_flux;
  s->sflux = surface_flux;
  s->fvflux = fv_flux;
  s->alpha_max = alpha_max;
  s->alpha_min = alpha_min;
  s->alpha_smooth = alpha_smooth != 0;
  s->source = source;
  return s;
}

void orc_destroy(void* h) { delete (Solver*)h; }

// periodicity = false with boundary conditions per direction (BC_DIRICHLET
// takes the values of initial condition `ic` with `params`, BC_SLIP_WALL);
// rebuilds the interfaces.  Returns 0, or -1 for an invalid code.
int orc_set_boundaries(void* h, const int* bc, int ic, const double* params) {
  Solver& s = *(Solver*)h;
  for (int dir = 0; dir < 2 * s.eq.D; ++dir)
    if (bc[dir] != BC_DIRICHLET && bc[dir] != BC_SLIP_WALL) return -1;
  double xmin[3], xmax[3];
  for (int d = 0; d < s.eq.D; ++d) {
    xmin[d] = s.m.xmin[d];
    xmax[d] = s.m.xmin[d] + s.m.length0;
  }
  s.m = make_mesh(s.eq.D, s.m.level, xmin, xmax, s.b, false, s.m.patches);
  s.periodic = false;
  for (int dir = 0; dir < 2 * s.eq.D; ++dir) s.bc[dir] = bc[dir];
  s.bc_ic = ic;
  for (int k = 0; k < 8; ++k) s.bc_par[k] = params ? params[k] : 0.0;
  return 0;
}

// Refinement patches applied after the initial refinement, in order
// (tree_mesh.jl:186-215): kinds[p] 0 = box, 1 = sphere; params[7 p ...] =
// coordinates_min[3], coordinates_max[3] (box) or center[3], -, -, -, radius
// (sphere).  Keeps the periodicity and the boundary conditions.  Returns 0,
// or -1 for an invalid patch.
int orc_set_refinement(void* h, int npatches, const int* kinds, const double* params) {
  Solver& s = *(Solver*)h;
  std::vector<Patch> patches;
  for (int k = 0; k < npatches; ++k) {
    if (kinds[k] != 0 && kinds[k] != 1) return -1;
    Patch p;
    p.kind = kinds[k];
    for (int d = 0; d < 3; ++d) {
      p.a[d] = params[7 * k + d];
      p.b[d] = params[7 * k + 3 + d];
    }
    p.r = params[7 * k + 6];
    patches.push_back(p);
  }
  double xmin[3], xmax[3];
  for (int d = 0; d < s.eq.D; ++d) {
    xmin[d] = s.m.xmin[d];
    xmax[d] = s.m.xmin[d] + s.m.length0;
  }
  s.m = make_mesh(s.eq.D, s.m.level, xmin, xmax, s.b, s.periodic, patches);
  return 0;
}

int64_t orc_nmortars(void* h) { return ((Solver*)h)->m.nmortar; }

// cache.mortars: neighbor_ids [2^(D-1) + 1, nmortars] (1-based; small ones
// first, the large one last), large_sides (1: large element on the negative
// side), orientations (1-based)
void orc_get_mortars(void* h, int64_t* neighbor_ids, int64_t* large_sides, int64_t* orientations) {
  const Solver& s = *(Solver*)h;
  const int ns1 = (1 << (s.eq.D - 1)) + 1;
  for (int64_t k = 0; k < s.m.nmortar; ++k) {
    for (int q = 0; q < ns1; ++q) neighbor_ids[k * ns1 + q] = s.m.mo_ids[k * ns1 + q] + 1;
    large_sides[k] = s.m.mo_large_side[k] + 1;
    orientations[k] = s.m.mo_orient[k] + 1;
  }
}

// dg.mortar (LobattoLegendreMortarL2): forward_upper, forward_lower,
// reverse_upper, reverse_lower, each n x n row-major
void orc_get_mortar_matrices(void* h, double* out) {
  const Solver& s = *(Solver*)h;
  const size_t nn = (size_t)s.b.n * s.b.n;
  std::memcpy(out, s.b.fwd[1].data(), sizeof(double) * nn);
  std::memcpy(out + nn, s.b.fwd[0].data(), sizeof(double) * nn);
  std::memcpy(out + 2 * nn, s.b.rev[1].data(), sizeof(double) * nn);
  std::memcpy(out + 3 * nn, s.b.rev[0].data(), sizeof(double) * nn);
}

void orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

int orc_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

int64_t orc_nelements(void* h) { return ((Solver*)h)->m.nelem; }
int64_t orc_ninterfaces(void* h) { return ((Solver*)h)->m.nif; }
int orc_nnodes(void* h) { return ((Solver*)h)->b.n; }
int64_t orc_ndofs(void* h) { return ((Solver*)h)->ndofs(); }

// Basis matrices are written column-major (Julia order) so that they compare
// directly with what a Julia host passes.
void orc_get_basis(void* h, double* nodes, double* weights, double* inv_weights, double* D,
                   double* Dhat, double* Dsplit, double* Vinv) {
  const Basis& b = ((Solver*)h)->b;
  const int n = b.n;
  for (int i = 0; i < n; ++i) {
    nodes[i] = b.nodes[i];
    weights[i] = b.weights[i];
    inv_weights[i] = b.inv_weights[i];
  }
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      D[i + j * n] = b.D[i * n + j];
      Dhat[i + j * n] = b.Dhat[i * n + j];
      Dsplit[i + j * n] = b.Dsplit[i * n + j];
      Vinv[i + j * n] = b.Vinv[i * n + j];
    }
}

// neighbor_ids[2, I] (1-based), orientations[I] (1-based), inverse_jacobian[E],
// node_coordinates[D, n^D, E]
void orc_get_mesh(void* h, int64_t* neighbor_ids, int64_t* orientations,
                  double* inverse_jacobian, double* node_coordinates) {
  const Solver& s = *(Solver*)h;
  for (int64_t f = 0; f < s.m.nif; ++f) {
    neighbor_ids[2 * f] = s.m.if_left[f] + 1;
    neighbor_ids[2 * f + 1] = s.m.if_right[f] + 1;
    orientations[f] = s.m.if_orient[f] + 1;
  }
  for (int64_t e = 0; e < s.m.nelem; ++e) inverse_jacobian[e] = s.m.inverse_jacobian[e];
  std::memcpy(node_coordinates, s.m.node_coords.data(), sizeof(double) * s.m.node_coords.size());
}

void orc_initial_condition(void* h, int ic, const double* params, double t, double* u) {
  const Solver& s = *(Solver*)h;
  const int D = s.eq.D;
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < s.m.nelem; ++e)
    for (int node = 0; node < s.nn; ++node)
      initial_condition(s.eq, ic, params, &s.m.node_coords[((size_t)e * s.nn + node) * D], t,
                        &u[uidx(s, e, node, 0)]);
}

void orc_rhs(void* h, double* du, const double* u, double t) { rhs(*(Solver*)h, du, u, t); }

void orc_alpha(void* h, const double* u, double* alpha) {
  Solver& s = *(Solver*)h;
  calc_alpha(s, u);
  std::memcpy(alpha, s.alpha.data(), sizeof(double) * s.m.nelem);
}

double orc_max_dt(void* h, const double* u) { return max_dt(*(Solver*)h, u); }

// One 2N stage: du = rhs(u, t_stage); u_tmp = du - a u_tmp; u += b dt u_tmp
void orc_rk_stage(void* h, double* u, double* u_tmp, double* du, int stage, double t,
                  double dt) {
  Solver& s = *(Solver*)h;
  rhs(s, du, u, t + dt * CK_C[stage]);
  rk_update(s.ndofs() * s.eq.NV, u, u_tmp, du, CK_A[stage], CK_B[stage] * dt);
}

// Trixi's SimpleIntegrator2N driven by a StepsizeCallback(cfl), methods_2N.jl:113-168,
// time_integration.jl:46-55, stepsize.jl:93-126.  Returns 0 on success, -1 on NaN dt.
int orc_solve(void* h, double* u, double t0, double t_end, double cfl, int64_t max_steps,
              double* t_out, int64_t* nsteps_out) {
  Solver& s = *(Solver*)h;
  const int64_t ndof = s.ndofs() * s.eq.NV;
  std::vector<double> du(ndof), u_tmp(ndof);
  double t = t0;
  double dt = cfl * max_dt(s, u);
  int64_t iter = 0;
  bool finalstep = false;
  while (!finalstep && iter < max_steps) {
    if (std::isnan(dt)) {
      *t_out = t;
      *nsteps_out = iter;
      return -1;
    }
    if (t + dt > t_end || isapprox(t + dt, t_end)) {
      dt = t_end - t;
      finalstep = true;
    }
    std::fill(u_tmp.begin(), u_tmp.end(), 0.0);
    for (int stage = 0; stage < 5; ++stage) {
      rhs(s, du.data(), u, t + dt * CK_C[stage]);
      rk_update(ndof, u, u_tmp.data(), du.data(), CK_A[stage], CK_B[stage] * dt);
    }
    iter += 1;
    t += dt;
    dt = cfl * max_dt(s, u);
  }
  *t_out = t;
  *nsteps_out = iter;
  return 0;
}

// AMR settings of the solver (AMRCallback + ControllerThreeLevel with an HG
// indicator); ints: interval, adapt_initial_condition,
// adapt_initial_condition_only_refine, alpha_smooth, base_level, med_level,
// max_level, indicator variable (0 density_pressure, 1 density), indicator
// (0 IndicatorHennemannGassner, 1 IndicatorMax); doubles:
// alpha_max, alpha_min, med_threshold, max_threshold.
void orc_set_amr(void* h, const int* ints, const double* dbls) {
  Solver& s = *(Solver*)h;
  AmrParams& a = s.amr;
  a.interval = ints[0];
  a.adapt_initial = ints[1] != 0;
  a.initial_only_refine = ints[2] != 0;
  a.alpha_smooth = ints[3] != 0;
  a.base_level = ints[4];
  a.med_level = ints[5];
  a.max_level = ints[6];
  a.variable = ints[7];
  a.indicator = ints[8];
  a.alpha_max = dbls[0];
  a.alpha_min = dbls[1];
  a.med_threshold = dbls[2];
  a.max_threshold = dbls[3];
}

// One AMR pass on u (nelements(h) elements); the adapted state is kept in
// the solver (orc_get_state).  Returns 1 if the mesh changed.
int orc_adapt(void* h, const double* u, int only_refine, int only_coarsen) {
  Solver& s = *(Solver*)h;
  s.u_state.assign(u, u + (size_t)s.ndofs() * s.eq.NV);
  return amr_adapt(s, s.u_state, s.amr, only_refine != 0, only_coarsen != 0) ? 1 : 0;
}

// The same pass with controller values given per element.
int orc_adapt_with(void* h, const double* u, const int* lambda, int only_refine, int only_coarsen) {
  Solver& s = *(Solver*)h;
  s.u_state.assign(u, u + (size_t)s.ndofs() * s.eq.NV);
  std::vector<int> lam(lambda, lambda + s.m.nelem);
  return amr_adapt_with(s, s.u_state, lam, only_refine != 0, only_coarsen != 0) ? 1 : 0;
}

// ControllerThreeLevel's values for u with the AMR settings of the solver.
void orc_amr_lambda(void* h, const double* u, int* lambda) {
  const Solver& s = *(Solver*)h;
  const std::vector<int> lam = amr_controller(s, u, s.amr);
  std::memcpy(lambda, lam.data(), sizeof(int) * lam.size());
}

void orc_get_state(void* h, double* u) {
  const Solver& s = *(Solver*)h;
  std::memcpy(u, s.u_state.data(), sizeof(double) * s.u_state.size());
}

void orc_element_levels(void* h, int* levels) {
  const Solver& s = *(Solver*)h;
  for (int64_t e = 0; e < s.m.nelem; ++e) levels[e] = s.m.elevel[e];
}

// solve() with the AMR callback: initial-condition adaptation (repeated with
// a fresh initial condition while the mesh changes, at most
// max(10, max_level) passes, amr.jl:143-181), then AMR after every
// `interval` accepted steps unless the final time is reached; the step size
// is recomputed from the adapted state (StepsizeCallback after AMRCallback).
// The final state stays in the solver (orc_get_state).
int orc_solve_amr(void* h, int ic, const double* params, double t0, double t_end, double cfl,
                  int64_t max_steps, double* t_out, int64_t* nsteps_out) {
  Solver& s = *(Solver*)h;
  const AmrParams& ap = s.amr;
  auto fresh = [&]() {
    s.u_state.assign((size_t)s.ndofs() * s.eq.NV, 0.0);
    orc_initial_condition(h, ic, params, t0, s.u_state.data());
  };
  fresh();
  if (ap.adapt_initial) {
    bool changed = amr_adapt(s, s.u_state, ap, ap.initial_only_refine, false);
    int iterations = 1;
    while (changed) {
      fresh();
      changed = amr_adapt(s, s.u_state, ap, ap.initial_only_refine, false);
      if (++iterations > std::max(10, ap.max_level)) break;
    }
  }
  double t = t0;
  std::vector<double> du, u_tmp;
  double dt = cfl * max_dt(s, s.u_state.data());
  int64_t iter = 0;
  bool finalstep = false;
  while (!finalstep && iter < max_steps) {
    if (std::isnan(dt)) {
      *t_out = t;
      *nsteps_out = iter;
      return -1;
    }
    if (t + dt > t_end || isapprox(t + dt, t_end)) {
      dt = t_end - t;
      finalstep = true;
    }
    const int64_t ndof = s.ndofs() * s.eq.NV;
    du.assign(ndof, 0.0);
    u_tmp.assign(ndof, 0.0);
    for (int stage = 0; stage < 5; ++stage) {
      rhs(s, du.data(), s.u_state.data(), t + dt * CK_C[stage]);
      rk_update(ndof, s.u_state.data(), u_tmp.data(), du.data(), CK_A[stage], CK_B[stage] * dt);
    }
    iter += 1;
    t += dt;
    if (ap.interval > 0 && iter % ap.interval == 0 && !finalstep)
      amr_adapt(s, s.u_state, ap, false, false);
    dt = cfl * max_dt(s, s.u_state.data());
  }
  *t_out = t;
  *nsteps_out = iter;
  return 0;
}

// calc_error_norms, analysis_dg2d.jl:95-139 (cons2cons errors against the
// initial condition evaluated at time t)
void orc_error_norms(void* h, const double* u, double t, int ic, const double* params,
                     double* l2, double* linf) {
  const Solver& s = *(Solver*)h;
  const int n = s.b.n, na = s.b.na, D = s.eq.D, NV = s.eq.NV;
  int nna = 1;
  for (int d = 0; d < D; ++d) nna *= na;
  double L2[5] = {0, 0, 0, 0, 0}, LI[5] = {0, 0, 0, 0, 0};
  std::vector<double> ua((size_t)nna * NV), xa((size_t)nna * D), tmp1, tmp2;
  for (int64_t e = 0; e < s.m.nelem; ++e) {
    // multiply_dimensionwise! applied to u and to the node coordinates
    auto interp = [&](const double* in, int nv, double* out) {
      // in: [nv, n^D] -> out [nv, na^D], x then y then z
      std::vector<double> cur(in, in + (size_t)nv * s.nn), nxt;
      int dims_in[3] = {n, n, n};
      for (int d = 0; d < D; ++d) {
        int shape_out[3] = {dims_in[0], dims_in[1], dims_in[2]};
        shape_out[d] = na;
        int tot = 1;
        for (int q = 0; q < D; ++q) tot *= shape_out[q];
        nxt.assign((size_t)tot * nv, 0.0);
        for (int o = 0; o < tot; ++o) {
          int ii[3] = {o % shape_out[0], (o / shape_out[0]) % shape_out[1],
                       o / (shape_out[0] * shape_out[1])};
          for (int v = 0; v < nv; ++v) {
            double r = 0;
            for (int k = 0; k < n; ++k) {
              int src[3] = {ii[0], ii[1], ii[2]};
              src[d] = k;
              const int si = src[0] + dims_in[0] * (src[1] + dims_in[1] * src[2]);
              r += s.b.avand[ii[d] * n + k] * cur[(size_t)si * nv + v];
            }
            nxt[(size_t)o * nv + v] = r;
          }
        }
        dims_in[d] = na;
        cur.swap(nxt);
      }
      std::memcpy(out, cur.data(), sizeof(double) * cur.size());
    };
    interp(&u[uidx(s, e, 0, 0)], NV, ua.data());
    interp(&s.m.node_coords[(size_t)e * s.nn * D], D, xa.data());
    double vj = 1.0 / s.m.inverse_jacobian[e];
    vj = D == 2 ? vj * vj : vj * vj * vj;
    double loc[5] = {0, 0, 0, 0, 0};
    for (int node = 0; node < nna; ++node) {
      int idx[3] = {node % na, (node / na) % na, node / (na * na)};
      double w = s.b.aweights[idx[0]] * s.b.aweights[idx[1]];
      if (D == 3) w *= s.b.aweights[idx[2]];
      double ue[5];
      initial_condition(s.eq, ic, params, &xa[(size_t)node * D], t, ue);
      for (int v = 0; v < NV; ++v) {
        const double diff = ue[v] - ua[(size_t)node * NV + v];
        loc[v] += diff * diff * (w * vj);
        LI[v] = std::max(LI[v], std::fabs(diff));
      }
    }
    for (int v = 0; v < NV; ++v) L2[v] += loc[v];
  }
  double vol = s.m.length0;
  vol = D == 2 ? vol * vol : vol * vol * vol;
  for (int v = 0; v < NV; ++v) {
    l2[v] = std::sqrt(L2[v] / vol);
    linf[v] = LI[v];
  }
}

// integrate_via_indices(u -> u[v]), analysis_dg2d.jl:313-336, without
// normalisation: the domain totals of the conserved variables, plus the total
// mathematical entropy (compressible_euler_2d.jl:2236-2255) and kinetic energy.
void orc_integrals(void* h, const double* u, double* out) {
  const Solver& s = *(Solver*)h;
  const int n = s.b.n, D = s.eq.D, NV = s.eq.NV;
  double acc[7] = {0, 0, 0, 0, 0, 0, 0};
  for (int64_t e = 0; e < s.m.nelem; ++e) {
    double vj = 1.0 / s.m.inverse_jacobian[e];
    vj = D == 2 ? vj * vj : vj * vj * vj;
    for (int node = 0; node < s.nn; ++node) {
      int idx[3] = {node % n, (node / n) % n, node / (n * n)};
      double w = s.b.weights[idx[0]] * s.b.weights[idx[1]];
      if (D == 3) w *= s.b.weights[idx[2]];
      const double* un = &u[uidx(s, e, node, 0)];
      for (int v = 0; v < NV; ++v) acc[v] += vj * w * un[v];
      double m2 = 0;
      for (int d = 0; d < D; ++d) m2 += un[1 + d] * un[1 + d];
      const double p = (s.eq.gamma - 1) * (un[NV - 1] - 0.5 * m2 / un[0]);
      const double sth = std::log(p) - s.eq.gamma * std::log(un[0]);
      acc[5] += vj * w * (-sth * un[0] * s.eq.inv_gamma_minus_one);
      acc[6] += vj * w * (m2 / (2 * un[0]));
    }
  }
  for (int v = 0; v < NV; ++v) out[v] = acc[v];
  out[NV] = acc[5];
  out[NV + 1] = acc[6];
}

// analyze(entropy_timederivative, ...), analysis_dg2d.jl:460-472: the
// normalised integral of cons2entropy(u) . du with du = rhs(u, t);
// cons2entropy, compressible_euler_2d.jl:2049-2066.
double orc_entropy_timederivative(void* h, const double* u, double t) {
  Solver& s = *(Solver*)h;
  const int n = s.b.n, D = s.eq.D, NV = s.eq.NV;
  std::vector<double> du((size_t)s.ndofs() * NV);
  rhs(s, du.data(), u, t);
  const double g = s.eq.gamma;
  double acc = 0;
  for (int64_t e = 0; e < s.m.nelem; ++e) {
    double vj = 1.0 / s.m.inverse_jacobian[e];
    vj = D == 2 ? vj * vj : vj * vj * vj;
    for (int node = 0; node < s.nn; ++node) {
      int idx[3] = {node % n, (node / n) % n, node / (n * n)};
      double w = s.b.weights[idx[0]] * s.b.weights[idx[1]];
      if (D == 3) w *= s.b.weights[idx[2]];
      const double* un = &u[uidx(s, e, node, 0)];
      const double* dn = &du[uidx(s, e, node, 0)];
      double v[3], v2 = 0;
      for (int d = 0; d < D; ++d) {
        v[d] = un[1 + d] / un[0];
        v2 += v[d] * v[d];
      }
      const double p = (g - 1) * (un[NV - 1] - 0.5 * un[0] * v2);
      const double sth = std::log(p) - g * std::log(un[0]);
      const double rho_p = un[0] / p;
      double dot = ((g - sth) * s.eq.inv_gamma_minus_one - 0.5 * rho_p * v2) * dn[0];
      for (int d = 0; d < D; ++d) dot += rho_p * v[d] * dn[1 + d];
      dot += -rho_p * dn[NV - 1];
      acc += vj * w * dot;
    }
  }
  double vol = s.m.length0;
  vol = D == 2 ? vol * vol : vol * vol * vol;
  return acc / vol;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Curvilinear 2D meshes: StructuredMesh and P4estMesh built from a brick of
// trees (src/meshes/structured_mesh.jl, p4est_mesh.jl:189-244) with DGSEM on
// the mapped elements (src/solvers/dgsem_structured/*_2d.jl,
// dgsem_p4est/dg_2d.jl).  The caller gives the element node coordinates and
// the neighbours of every element (periodic bricks: all four exist); the
// metric terms are computed here.
// ---------------------------------------------------------------------------

namespace orc {

// flux(u, normal_direction), compressible_euler_2d.jl:436-448
static inline void flux_n(const Eq& eq, const double* u, const double* n, double* f) {
  double w[4];
  cons2prim(eq, u, w);
  const double vn = w[1] * n[0] + w[2] * n[1];
  const double rvn = w[0] * vn;
  f[0] = rvn;
  f[1] = rvn * w[1] + w[3] * n[0];
  f[2] = rvn * w[2] + w[3] * n[1];
  f[3] = (u[3] + w[3]) * vn;
}

// flux_ranocha(u_ll, u_rr, normal_direction), compressible_euler_2d.jl:724-753
static inline void flux_ranocha_n(const Eq& eq, const double* ul, const double* ur,
                                  const double* n, double* f) {
  double a[4], b[4];
  cons2prim(eq, ul, a);
  cons2prim(eq, ur, b);
  const double vna = a[1] * n[0] + a[2] * n[1];
  const double vnb = b[1] * n[0] + b[2] * n[1];
  const double rho_mean = ln_mean(a[0], b[0]);
  const double inv_rho_p_mean = a[3] * b[3] * inv_ln_mean(a[0] * b[3], b[0] * a[3]);
  const double v1 = 0.5 * (a[1] + b[1]), v2 = 0.5 * (a[2] + b[2]);
  const double p_avg = 0.5 * (a[3] + b[3]);
  const double vsq = 0.5 * (a[1] * b[1] + a[2] * b[2]);
  const double f1 = rho_mean * 0.5 * (vna + vnb);
  f[0] = f1;
  f[1] = std::fma(f1, v1, p_avg * n[0]);
  f[2] = std::fma(f1, v2, p_avg * n[1]);
  f[3] = f1 * (vsq + inv_rho_p_mean * eq.inv_gamma_minus_one) +
         0.5 * (a[3] * vnb + b[3] * vna);
}

// flux_shima_etal(u_ll, u_rr, normal_direction), compressible_euler_2d.jl:497-526
static inline void flux_shima_n(const Eq& eq, const double* ul, const double* ur,
                                const double* n, double* f) {
  double a[4], b[4];
  cons2prim(eq, ul, a);
  cons2prim(eq, ur, b);
  const double vna = a[1] * n[0] + a[2] * n[1];
  const double vnb = b[1] * n[0] + b[2] * n[1];
  const double rho_avg = 0.5 * (a[0] + b[0]);
  const double v1 = 0.5 * (a[1] + b[1]), v2 = 0.5 * (a[2] + b[2]);
  const double vn_avg = 0.5 * (vna + vnb);
  const double p_avg = 0.5 * (a[3] + b[3]);
  const double vsq = 0.5 * (a[1] * b[1] + a[2] * b[2]);
  const double f1 = rho_avg * vn_avg;
  f[0] = f1;
  f[1] = std::fma(f1, v1, p_avg * n[0]);
  f[2] = std::fma(f1, v2, p_avg * n[1]);
  f[3] = f1 * vsq + p_avg * vn_avg * eq.inv_gamma_minus_one + 0.5 * (a[3] * vnb + b[3] * vna);
}

// flux_chandrashekar(u_ll, u_rr, normal_direction), compressible_euler_2d.jl:639-670
static inline void flux_chandrashekar_n(const Eq& eq, const double* ul, const double* ur,
                                        const double* n, double* f) {
  double a[4], b[4];
  cons2prim(eq, ul, a);
  cons2prim(eq, ur, b);
  const double vna = a[1] * n[0] + a[2] * n[1];
  const double vnb = b[1] * n[0] + b[2] * n[1];
  const double beta_a = 0.5 * a[0] / a[3], beta_b = 0.5 * b[0] / b[3];
  const double kin_a = 0.5 * (a[1] * a[1] + a[2] * a[2]);
  const double kin_b = 0.5 * (b[1] * b[1] + b[2] * b[2]);
  const double rho_avg = 0.5 * (a[0] + b[0]);
  const double rho_mean = ln_mean(a[0], b[0]);
  const double beta_mean = ln_mean(beta_a, beta_b);
  const double beta_avg = 0.5 * (beta_a + beta_b);
  const double v1 = 0.5 * (a[1] + b[1]), v2 = 0.5 * (a[2] + b[2]);
  const double p_mean = 0.5 * rho_avg / beta_avg;
  const double vsq_avg = kin_a + kin_b;
  const double f1 = rho_mean * 0.5 * (vna + vnb);
  f[0] = f1;
  f[1] = std::fma(f1, v1, p_mean * n[0]);
  f[2] = std::fma(f1, v2, p_mean * n[1]);
  f[3] = f1 * 0.5 * (1 / (eq.gamma - 1) / beta_mean - vsq_avg) + f[1] * v1 + f[2] * v2;
}

// max_abs_speed(_naive)(u_ll, u_rr, normal_direction), compressible_euler_2d.jl:1443-1509
static inline double max_abs_speed_n(const Eq& eq, const double* ul, const double* ur,
                                     const double* n, bool naive) {
  double a[4], b[4];
  cons2prim(eq, ul, a);
  cons2prim(eq, ur, b);
  const double va = a[1] * n[0] + a[2] * n[1];
  const double vb = b[1] * n[0] + b[2] * n[1];
  const double ca = std::sqrt(eq.gamma * a[3] / a[0]);
  const double cb = std::sqrt(eq.gamma * b[3] / b[0]);
  const double nn = std::sqrt(n[0] * n[0] + n[1] * n[1]);
  if (naive) return std::max(std::fabs(va), std::fabs(vb)) + std::max(ca, cb) * nn;
  return std::max(std::fabs(va) + ca * nn, std::fabs(vb) + cb * nn);
}

// Two-point fluxes along a normal direction (volume and surface)
static inline void two_point_flux_n(const Eq& eq, int kind, const double* ul, const double* ur,
                                    const double* n, double* f) {
  switch (kind) {
    case FLUX_CENTRAL:
    case FLUX_LAX_FRIEDRICHS:
    case FLUX_LAX_FRIEDRICHS_NAIVE: {
      // flux_central, numerical_fluxes.jl:17-25, plus DissipationLocalLaxFriedrichs
      double fl[4], fr[4];
      flux_n(eq, ul, n, fl);
      flux_n(eq, ur, n, fr);
      for (int v = 0; v < 4; ++v) f[v] = 0.5 * (fl[v] + fr[v]);
      if (kind != FLUX_CENTRAL) {
        const double lam = max_abs_speed_n(eq, ul, ur, n, kind == FLUX_LAX_FRIEDRICHS_NAIVE);
        for (int v = 0; v < 4; ++v) f[v] = f[v] + (-0.5 * lam * (ur[v] - ul[v]));
      }
      return;
    }
    case FLUX_RANOCHA: flux_ranocha_n(eq, ul, ur, n, f); return;
    case FLUX_SHIMA_ETAL: flux_shima_n(eq, ul, ur, n, f); return;
    case FLUX_CHANDRASHEKAR: flux_chandrashekar_n(eq, ul, ur, n, f); return;
    default: for (int v = 0; v < 4; ++v) f[v] = NAN;
  }
}

struct Curved {
  Eq eq;
  Basis b;
  int n = 0, nn = 0;
  int64_t E = 0;
  int vi = VI_WEAK, vf = FLUX_CENTRAL, sf = FLUX_LAX_FRIEDRICHS, source = SRC_NONE;
  std::vector<double> x;     // [E][nn][2] node coordinates, node = i + n j
  std::vector<int64_t> nbr;  // [E][4]: neighbours across -x, +x, -y, +y
  std::vector<double> Ja;    // [E][nn][4]: Ja^1 (x, y), Ja^2 (x, y)
  std::vector<double> invJ;  // [E][nn]
  // faces without a neighbour (nbr < 0): BoundaryConditionDirichlet of an
  // initial condition (bc_ic, bc_par)
  int bc_ic = -1;
  double bc_par[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  // VolumeIntegralShockCapturingHG: indicator parameters, the FV flux and the
  // subcell normal vectors [E][dir][N - 1][n][2] (calc_normalvectors_subcell_fv!)
  double alpha_max = 0.5, alpha_min = 0.001;
  bool alpha_smooth = true;
  int fvflux = FLUX_LAX_FRIEDRICHS;
  std::vector<double> snv;
  size_t ui(int64_t e, int node) const { return ((size_t)e * nn + node) * 4; }
};

// calc_normalvectors_subcell_fv! (dgsem_structured/containers_2d.jl:200-298):
// the normal of the subcell interface between nodes i and i + 1 of a line is
// Ja at the first node plus the partial sums of w_m D[m, :] Ja along the line,
// which keeps the finite-volume subcells free-stream preserving.
static void curved_subcell_normals(Curved& c) {
  const int n = c.n, nn = c.nn;
  const std::vector<double>& Dm = c.b.D;
  const std::vector<double>& w = c.b.weights;
  c.snv.assign((size_t)c.E * 2 * (n - 1) * n * 2, 0.0);
  for (int64_t e = 0; e < c.E; ++e)
    for (int dir = 0; dir < 2; ++dir)
      for (int l = 0; l < n; ++l) {
        // node a of line l in direction dir
        auto q = [&](int a) { return dir == 0 ? a + n * l : l + n * a; };
        double acc[2];
        for (int xy = 0; xy < 2; ++xy) acc[xy] = c.Ja[((size_t)e * nn + q(0)) * 4 + 2 * dir + xy];
        for (int i = 0; i < n - 1; ++i) {
          for (int m = 0; m < n; ++m) {
            const double wd = w[i] * Dm[i * n + m];
            for (int xy = 0; xy < 2; ++xy)
              acc[xy] += wd * c.Ja[((size_t)e * nn + q(m)) * 4 + 2 * dir + xy];
          }
          for (int xy = 0; xy < 2; ++xy)
            c.snv[((((size_t)e * 2 + dir) * (n - 1) + i) * n + l) * 2 + xy] = acc[xy];
        }
      }
}

// IndicatorHennemannGassner on density_pressure (indicators.jl:114-148,
// indicators_2d.jl:30-136) per element of a curvilinear mesh, smoothed over
// the element neighbours
static void curved_hg_alpha(const Curved& c, const double* u, std::vector<double>& alpha) {
  const int n = c.n, nn = c.nn;
  const double threshold = 0.5 * std::pow(10.0, -1.8 * std::pow((double)n, 0.25));
  const double parameter_s = std::log((1 - 0.0001) / 0.0001);
  alpha.assign(c.E, 0.0);
  const double* V = c.b.Vinv.data();
  for (int64_t e = 0; e < c.E; ++e) {
    double ind[64], t1[64];
    for (int q = 0; q < nn; ++q) ind[q] = density_pressure(c.eq, &u[c.ui(e, q)]);
    double modal[64];
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        double r = 0;
        for (int ii = 0; ii < n; ++ii) r += V[i * n + ii] * ind[ii + n * j];
        t1[i + n * j] = r;
      }
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        double r = 0;
        for (int jj = 0; jj < n; ++jj) r += V[j * n + jj] * t1[i + n * jj];
        modal[i + n * j] = r;
      }
    double e_clip2 = 0, e_clip1 = 0, e_tot = 0;
    for (int q = 0; q < nn; ++q) {
      const int mx = std::max(q % n, q / n);
      const double m2 = modal[q] * modal[q];
      if (mx <= n - 3) e_clip2 += m2;
      if (mx <= n - 2) e_clip1 += m2;
      e_tot += m2;
    }
    const double f1 = e_tot != 0 ? (e_tot - e_clip1) / e_tot : 0.0;
    const double f2 = e_clip1 != 0 ? (e_clip1 - e_clip2) / e_clip1 : 0.0;
    const double energy = std::max(f1, f2);
    double a = 1 / (1 + std::exp(-parameter_s / threshold * (energy - threshold)));
    if (a < c.alpha_min) a = 0;
    if (a > 1 - c.alpha_min) a = 1;
    alpha[e] = std::min(c.alpha_max, a);
  }
  if (c.alpha_smooth) {
    const std::vector<double> tmp = alpha;
    for (int64_t e = 0; e < c.E; ++e)
      for (int o = 0; o < 2; ++o) {
        const int64_t r = c.nbr[e * 4 + 2 * o + 1];  // interface (e, r) in direction o
        if (r < 0) continue;
        alpha[e] = std::max({tmp[e], 0.5 * tmp[r], alpha[e]});
        alpha[r] = std::max({tmp[r], 0.5 * tmp[e], alpha[r]});
      }
  }
}

// calc_jacobian_matrix!, calc_contravariant_vectors!, calc_inverse_jacobian!
// (dgsem_structured/containers_2d.jl:61-152)
static void curved_metric(Curved& c) {
  const int n = c.n, nn = c.nn;
  const std::vector<double>& Dm = c.b.D;
  c.Ja.assign((size_t)c.E * nn * 4, 0.0);
  c.invJ.assign((size_t)c.E * nn, 0.0);
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < c.E; ++e) {
    const double* X = &c.x[(size_t)e * nn * 2];
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        double J[2][2];  // J[xy][dir]
        for (int xy = 0; xy < 2; ++xy) {
          double r1 = 0, r2 = 0;
          for (int k = 0; k < n; ++k) {
            r1 += Dm[i * n + k] * X[(k + n * j) * 2 + xy];
            r2 += Dm[j * n + k] * X[(i + n * k) * 2 + xy];
          }
          J[xy][0] = r1;
          J[xy][1] = r2;
        }
        double* a = &c.Ja[((size_t)e * nn + i + n * j) * 4];
        a[0] = J[1][1];
        a[1] = -J[0][1];
        a[2] = -J[1][0];
        a[3] = J[0][0];
        c.invJ[(size_t)e * nn + i + n * j] = 1.0 / (J[0][0] * J[1][1] - J[0][1] * J[1][0]);
      }
  }
}

// rhs! of a curvilinear 2D mesh: volume integral (weak_form_kernel! /
// flux_differencing_kernel!, dgsem_structured/dg_2d.jl:34-139), interface
// fluxes with the normal of the element on the + side (dg_2d.jl:551-606),
// surface integral (dgsem_tree/dg_2d.jl:1245-1287), apply_jacobian! per node
// (dgsem_structured/dg_2d.jl:751-771) and sources (dg_2d.jl:1366-1386).
static void curved_rhs(const Curved& c, double* du, const double* u, double t) {
  const int n = c.n, nn = c.nn;
  const Basis& b = c.b;
  const Eq& eq = c.eq;
  std::vector<double> sfv((size_t)c.E * 4 * n * 4);  // [E][dir][l][v]
  // VolumeIntegralShockCapturingHG (calc_volume_integral.jl:231-272): the
  // blending factor per element, FD weighted by 1 - alpha, FV by alpha
  const bool hg = c.vi == VI_SHOCKCAPTURING_HG;
  std::vector<double> alpha;
  if (hg) curved_hg_alpha(c, u, alpha);
  const double atol = std::max(100 * 2.220446049250313e-16, std::pow(2.220446049250313e-16, 0.75));
  // interface fluxes: for each element, the faces towards its -x and -y neighbours
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < c.E; ++e) {
    for (int o = 0; o < 2; ++o) {
      const int64_t left = c.nbr[e * 4 + 2 * o];
      if (left < 0) continue;
      for (int l = 0; l < n; ++l) {
        const int nr = o == 0 ? n * l : l;                        // (1, l) / (l, 1) of e
        const int nl = o == 0 ? (n - 1) + n * l : l + n * (n - 1);  // (N, l) / (l, N) of left
        const double sj = c.invJ[(size_t)e * nn + nr] >= 0 ? 1.0 : -1.0;
        const double* a = &c.Ja[((size_t)e * nn + nr) * 4 + 2 * o];
        const double nd[2] = {sj * a[0], sj * a[1]};
        double F[4];
        two_point_flux_n(eq, c.sf, &u[c.ui(left, nl)], &u[c.ui(e, nr)], nd, F);
        for (int v = 0; v < 4; ++v) {
          F[v] *= sj;
          sfv[(((size_t)e * 4 + 2 * o) * n + l) * 4 + v] = F[v];
          sfv[(((size_t)left * 4 + 2 * o + 1) * n + l) * 4 + v] = F[v];
        }
      }
    }
  }
  // Dirichlet boundary faces (calc_boundary_flux!, dgsem_structured/dg_2d.jl:680-750,
  // dg.jl:124-163; BoundaryConditionDirichlet, equations.jl:183-211): the flux
  // along the element's own contravariant vector, the boundary value on the
  // outer side
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < c.E; ++e) {
    for (int dir = 0; dir < 4; ++dir) {
      if (c.nbr[e * 4 + dir] >= 0) continue;
      const int o = dir >> 1;
      for (int l = 0; l < n; ++l) {
        const int q = o == 0 ? ((dir & 1) ? (n - 1) + n * l : n * l)
                             : ((dir & 1) ? l + n * (n - 1) : l);
        const double sj = c.invJ[(size_t)e * nn + q] >= 0 ? 1.0 : -1.0;
        const double* a = &c.Ja[((size_t)e * nn + q) * 4 + 2 * o];
        const double nd[2] = {sj * a[0], sj * a[1]};
        double ub[5];
        initial_condition(c.eq, c.bc_ic, c.bc_par, &c.x[((size_t)e * nn + q) * 2], t, ub);
        double F[4];
        if (dir & 1)
          two_point_flux_n(eq, c.sf, &u[c.ui(e, q)], ub, nd, F);
        else
          two_point_flux_n(eq, c.sf, ub, &u[c.ui(e, q)], nd, F);
        for (int v = 0; v < 4; ++v) sfv[(((size_t)e * 4 + dir) * n + l) * 4 + v] = sj * F[v];
      }
    }
  }
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < c.E; ++e) {
    double* de = du + (size_t)e * nn * 4;
    const double* ue = u + (size_t)e * nn * 4;
    const double* Ja = &c.Ja[(size_t)e * nn * 4];
    for (int k = 0; k < nn * 4; ++k) de[k] = 0;
    if (c.vi == VI_WEAK) {
      for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) {
          const int q = i + n * j;
          double f1[5] = {}, f2[5] = {};
          flux_phys(eq, ue + q * 4, 0, f1);
          flux_phys(eq, ue + q * 4, 1, f2);
          const double* a = Ja + q * 4;
          double cf1[4], cf2[4];
          for (int v = 0; v < 4; ++v) {
            cf1[v] = std::fma(a[0], f1[v], a[1] * f2[v]);
            cf2[v] = std::fma(a[2], f1[v], a[3] * f2[v]);
          }
          for (int ii = 0; ii < n; ++ii)
            for (int v = 0; v < 4; ++v)
              de[(ii + n * j) * 4 + v] = std::fma(b.Dhat[ii * n + i], cf1[v], de[(ii + n * j) * 4 + v]);
          for (int jj = 0; jj < n; ++jj)
            for (int v = 0; v < 4; ++v)
              de[(i + n * jj) * 4 + v] = std::fma(b.Dhat[jj * n + j], cf2[v], de[(i + n * jj) * 4 + v]);
        }
    } else {
      const double ae = hg ? alpha[e] : 0.0;
      const bool dg_only = !hg || std::fabs(ae) <= atol;
      const double fdw = dg_only ? 1.0 : 1.0 - ae;
      for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) {
          const int q = i + n * j;
          for (int ii = i + 1; ii < n; ++ii) {
            const int r = ii + n * j;
            const double avg[2] = {0.5 * (Ja[q * 4] + Ja[r * 4]), 0.5 * (Ja[q * 4 + 1] + Ja[r * 4 + 1])};
            double F[4];
            two_point_flux_n(eq, c.vf, ue + q * 4, ue + r * 4, avg, F);
            for (int v = 0; v < 4; ++v) {
              de[q * 4 + v] = std::fma(fdw * b.Dsplit[i * n + ii], F[v], de[q * 4 + v]);
              de[r * 4 + v] = std::fma(fdw * b.Dsplit[ii * n + i], F[v], de[r * 4 + v]);
            }
          }
          for (int jj = j + 1; jj < n; ++jj) {
            const int r = i + n * jj;
            const double avg[2] = {0.5 * (Ja[q * 4 + 2] + Ja[r * 4 + 2]),
                                   0.5 * (Ja[q * 4 + 3] + Ja[r * 4 + 3])};
            double F[4];
            two_point_flux_n(eq, c.vf, ue + q * 4, ue + r * 4, avg, F);
            for (int v = 0; v < 4; ++v) {
              de[q * 4 + v] = std::fma(fdw * b.Dsplit[j * n + jj], F[v], de[q * 4 + v]);
              de[r * 4 + v] = std::fma(fdw * b.Dsplit[jj * n + j], F[v], de[r * 4 + v]);
            }
          }
        }
      if (!dg_only) {
        // fv_kernel! / calcflux_fv! (dgsem_structured/dg_2d.jl:304-345): subcell
        // fluxes along the free-stream preserving subcell normals, zero at the
        // element faces
        for (int dir = 0; dir < 2; ++dir)
          for (int l = 0; l < n; ++l) {
            double fst[9][4] = {};
            auto qn = [&](int a) { return dir == 0 ? a + n * l : l + n * a; };
            for (int i = 1; i < n; ++i) {
              const double* nv = &c.snv[((((size_t)e * 2 + dir) * (n - 1) + (i - 1)) * n + l) * 2];
              two_point_flux_n(eq, c.fvflux, ue + qn(i - 1) * 4, ue + qn(i) * 4, nv, fst[i]);
            }
            for (int i = 0; i < n; ++i)
              for (int v = 0; v < 4; ++v)
                de[qn(i) * 4 + v] += ae * (b.inv_weights[i] * (fst[i + 1][v] - fst[i][v]));
          }
      }
    }
    // surface integral
    const double factor = b.inv_weights[0];
    const double* sf = &sfv[(size_t)e * 4 * n * 4];
    for (int l = 0; l < n; ++l)
      for (int v = 0; v < 4; ++v) {
        double& a0 = de[(n * l) * 4 + v];
        a0 = a0 - sf[(0 * n + l) * 4 + v] * factor;
        double& a1 = de[((n - 1) + n * l) * 4 + v];
        a1 = a1 + sf[(1 * n + l) * 4 + v] * factor;
        double& a2 = de[l * 4 + v];
        a2 = a2 - sf[(2 * n + l) * 4 + v] * factor;
        double& a3 = de[(l + n * (n - 1)) * 4 + v];
        a3 = a3 + sf[(3 * n + l) * 4 + v] * factor;
      }
    for (int q = 0; q < nn; ++q) {
      const double fac = -c.invJ[(size_t)e * nn + q];
      for (int v = 0; v < 4; ++v) de[q * 4 + v] *= fac;
      if (c.source == SRC_CONVERGENCE_TEST) {
        double s[5];
        source_convergence(eq, &c.x[((size_t)e * nn + q) * 2], t, s);
        for (int v = 0; v < 4; ++v) de[q * 4 + v] += s[v];
      }
    }
  }
}

// max_dt of a curvilinear 2D mesh (stepsize_dg2d.jl:114-157)
static double curved_max_dt(const Curved& c, const double* u) {
  double mss = 4.9406564584124654e-324;  // nextfloat(0.0)
  for (int64_t e = 0; e < c.E; ++e) {
    double m1 = 0, m2 = 0;
    for (int q = 0; q < c.nn; ++q) {
      double lam[2];
      max_abs_speeds(c.eq, &u[c.ui(e, q)], lam);
      const double* a = &c.Ja[((size_t)e * c.nn + q) * 4];
      const double l1 = std::fabs(a[0] * lam[0] + a[1] * lam[1]);
      const double l2 = std::fabs(a[2] * lam[0] + a[3] * lam[1]);
      const double ij = std::fabs(c.invJ[(size_t)e * c.nn + q]);
      m1 = std::max(m1, l1 * ij);
      m2 = std::max(m2, l2 * ij);
    }
    mss = std::max(mss, m1 + m2);
  }
  return 2 / (c.n * mss);
}

// calc_error_norms of a curvilinear 2D mesh (analysis_dg2d.jl:141-197)
static void curved_errors(const Curved& c, const double* u, double t, int ic, const double* par,
                          double* l2, double* linf) {
  const Basis& b = c.b;
  const int n = c.n, na = b.na;
  for (int v = 0; v < 4; ++v) l2[v] = linf[v] = 0;
  double vol = 0;
  std::vector<double> tmp((size_t)na * n * 4), ua((size_t)na * na * 4), xt((size_t)na * n * 2),
      xa((size_t)na * na * 2), jt((size_t)na * n), ja((size_t)na * na);
  for (int64_t e = 0; e < c.E; ++e) {
    // interpolate along i, then along j (multiply_dimensionwise!)
    for (int j = 0; j < n; ++j)
      for (int a = 0; a < na; ++a) {
        double s4[4] = {0, 0, 0, 0}, s2[2] = {0, 0}, s1 = 0;
        for (int i = 0; i < n; ++i) {
          const double w = b.avand[a * n + i];
          const int q = i + n * j;
          for (int v = 0; v < 4; ++v) s4[v] += w * u[c.ui(e, q) + v];
          for (int d = 0; d < 2; ++d) s2[d] += w * c.x[((size_t)e * c.nn + q) * 2 + d];
          s1 += w * (1.0 / c.invJ[(size_t)e * c.nn + q]);
        }
        for (int v = 0; v < 4; ++v) tmp[(a + na * j) * 4 + v] = s4[v];
        for (int d = 0; d < 2; ++d) xt[(a + na * j) * 2 + d] = s2[d];
        jt[a + na * j] = s1;
      }
    for (int bb = 0; bb < na; ++bb)
      for (int a = 0; a < na; ++a) {
        double s4[4] = {0, 0, 0, 0}, s2[2] = {0, 0}, s1 = 0;
        for (int j = 0; j < n; ++j) {
          const double w = b.avand[bb * n + j];
          for (int v = 0; v < 4; ++v) s4[v] += w * tmp[(a + na * j) * 4 + v];
          for (int d = 0; d < 2; ++d) s2[d] += w * xt[(a + na * j) * 2 + d];
          s1 += w * jt[a + na * j];
        }
        double ue[4];
        initial_condition(c.eq, ic, par, s2, t, ue);
        const double wj = b.aweights[a] * b.aweights[bb] * std::fabs(s1);
        for (int v = 0; v < 4; ++v) {
          const double d = ue[v] - s4[v];
          l2[v] += d * d * wj;
          linf[v] = std::max(linf[v], std::fabs(d));
        }
        vol += wj;
      }
  }
  for (int v = 0; v < 4; ++v) l2[v] = std::sqrt(l2[v] / vol);
}

}  // namespace orc

extern "C" {

// Curvilinear 2D solver on element node coordinates x[E][n][n][2] (i fastest)
// and neighbours nbr[E][4] (0-based, -x, +x, -y, +y).
void* orc_curved_create(int polydeg, int64_t nelements, const double* x, const int64_t* nbr,
                        double gamma, int volume_integral, int volume_flux, int surface_flux,
                        int source) {
  Curved* c = new Curved();
  c->eq.D = 2;
  c->eq.NV = 4;
  c->eq.gamma = gamma;
  c->eq.inv_gamma_minus_one = 1 / (gamma - 1);
  c->b = make_basis(polydeg);
  c->n = polydeg + 1;
  c->nn = c->n * c->n;
  c->E = nelements;
  c->vi = volume_integral;
  c->vf = volume_flux;
  c->sf = surface_flux;
  c->source = source;
  c->x.assign(x, x + (size_t)nelements * c->nn * 2);
  c->nbr.assign(nbr, nbr + (size_t)nelements * 4);
  curved_metric(*c);
  return c;
}

void orc_curved_destroy(void* h) { delete (Curved*)h; }

// VolumeIntegralShockCapturingHG settings (the volume integral must be
// VI_SHOCKCAPTURING_HG): indicator parameters and the FV subcell flux
void orc_curved_set_hg(void* h, double alpha_max, double alpha_min, int alpha_smooth, int fvflux) {
  Curved& c = *(Curved*)h;
  c.alpha_max = alpha_max;
  c.alpha_min = alpha_min;
  c.alpha_smooth = alpha_smooth != 0;
  c.fvflux = fvflux;
  curved_subcell_normals(c);
}

// Smoothed blending factors of a state (VI_SHOCKCAPTURING_HG), alpha[E]
void orc_curved_alpha(void* h, const double* u, double* alpha) {
  std::vector<double> a;
  curved_hg_alpha(*(const Curved*)h, u, a);
  std::copy(a.begin(), a.end(), alpha);
}

// Dirichlet values (an initial condition and its parameters) of the faces
// without a neighbour
void orc_curved_set_dirichlet(void* h, int ic, const double* params) {
  Curved& c = *(Curved*)h;
  c.bc_ic = ic;
  for (int k = 0; k < 8; ++k) c.bc_par[k] = params ? params[k] : 0.0;
}

// contravariant_vectors [E][n][n][2 (dir)][2 (xy)], inverse_jacobian [E][n][n]
void orc_curved_metric(void* h, double* contravariant, double* inverse_jacobian) {
  Curved& c = *(Curved*)h;
  std::copy(c.Ja.begin(), c.Ja.end(), contravariant);
  std::copy(c.invJ.begin(), c.invJ.end(), inverse_jacobian);
}

void orc_curved_initial_condition(void* h, int ic, const double* params, double t, double* u) {
  Curved& c = *(Curved*)h;
  for (int64_t e = 0; e < c.E; ++e)
    for (int q = 0; q < c.nn; ++q)
      initial_condition(c.eq, ic, params, &c.x[((size_t)e * c.nn + q) * 2], t, &u[c.ui(e, q)]);
}

void orc_curved_rhs(void* h, double* du, const double* u, double t) {
  curved_rhs(*(Curved*)h, du, u, t);
}

double orc_curved_max_dt(void* h, const double* u) { return curved_max_dt(*(Curved*)h, u); }

// SimpleIntegrator2N + StepsizeCallback(cfl), as orc_solve
int orc_curved_solve(void* h, double* u, double t0, double t_end, double cfl, int64_t max_steps,
                     double* t_out, int64_t* nsteps_out) {
  Curved& c = *(Curved*)h;
  const int64_t ndof = c.E * c.nn * 4;
  std::vector<double> du(ndof), u_tmp(ndof);
  double t = t0;
  double dt = cfl * curved_max_dt(c, u);
  int64_t iter = 0;
  bool finalstep = false;
  while (!finalstep && iter < max_steps) {
    if (std::isnan(dt)) {
      *t_out = t;
      *nsteps_out = iter;
      return -1;
    }
    if (t + dt > t_end || isapprox(t + dt, t_end)) {
      dt = t_end - t;
      finalstep = true;
    }
    std::fill(u_tmp.begin(), u_tmp.end(), 0.0);
    for (int stage = 0; stage < 5; ++stage) {
      curved_rhs(c, du.data(), u, t + dt * CK_C[stage]);
      rk_update(ndof, u, u_tmp.data(), du.data(), CK_A[stage], CK_B[stage] * dt);
    }
    iter += 1;
    t += dt;
    dt = cfl * curved_max_dt(c, u);
  }
  *t_out = t;
  *nsteps_out = iter;
  return 0;
}

void orc_curved_errors(void* h, const double* u, double t, int ic, const double* params,
                       double* l2, double* linf) {
  curved_errors(*(Curved*)h, u, t, ic, params, l2, linf);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Curvilinear 3D meshes (StructuredMesh{3}): the element node coordinates and
// neighbours come from the caller; metric terms in the invariant curl form
// (dgsem_structured/containers_3d.jl:67-286); rhs! of dgsem_structured/dg_3d.jl.
// ---------------------------------------------------------------------------

namespace orc {

// flux(u, normal_direction) and the two-point fluxes along a normal,
// compressible_euler_3d.jl (normal-direction methods)
static inline void flux3_n(const Eq& eq, const double* u, const double* n, double* f) {
  double w[5];
  cons2prim(eq, u, w);
  const double vn = w[1] * n[0] + w[2] * n[1] + w[3] * n[2];
  const double rvn = w[0] * vn;
  f[0] = rvn;
  for (int d = 0; d < 3; ++d) f[1 + d] = std::fma(rvn, w[1 + d], w[4] * n[d]);
  f[4] = (u[4] + w[4]) * vn;
}

static inline void two_point3_n(const Eq& eq, int kind, const double* ul, const double* ur,
                                const double* n, double* f) {
  double a[5], b[5];
  cons2prim(eq, ul, a);
  cons2prim(eq, ur, b);
  const double vna = a[1] * n[0] + a[2] * n[1] + a[3] * n[2];
  const double vnb = b[1] * n[0] + b[2] * n[1] + b[3] * n[2];
  double vavg[3], vsq = 0;
  for (int d = 0; d < 3; ++d) {
    vavg[d] = 0.5 * (a[1 + d] + b[1 + d]);
    vsq += a[1 + d] * b[1 + d];
  }
  vsq *= 0.5;
  const double p_avg = 0.5 * (a[4] + b[4]);
  switch (kind) {
    case FLUX_RANOCHA: {
      const double rho_mean = ln_mean(a[0], b[0]);
      const double irpm = a[4] * b[4] * inv_ln_mean(a[0] * b[4], b[0] * a[4]);
      const double f1 = rho_mean * 0.5 * (vna + vnb);
      f[0] = f1;
      for (int d = 0; d < 3; ++d) f[1 + d] = std::fma(f1, vavg[d], p_avg * n[d]);
      f[4] = f1 * (vsq + irpm * eq.inv_gamma_minus_one) + 0.5 * (a[4] * vnb + b[4] * vna);
      return;
    }
    case FLUX_SHIMA_ETAL: {
      const double rho_avg = 0.5 * (a[0] + b[0]);
      const double vn_avg = 0.5 * (vna + vnb);
      const double f1 = rho_avg * vn_avg;
      f[0] = f1;
      for (int d = 0; d < 3; ++d) f[1 + d] = std::fma(f1, vavg[d], p_avg * n[d]);
      f[4] = f1 * vsq + p_avg * vn_avg * eq.inv_gamma_minus_one + 0.5 * (a[4] * vnb + b[4] * vna);
      return;
    }
    case FLUX_CHANDRASHEKAR: {
      // compressible_euler_3d.jl:693-729
      const double beta_a = 0.5 * a[0] / a[4], beta_b = 0.5 * b[0] / b[4];
      const double kin_a = 0.5 * (a[1] * a[1] + a[2] * a[2] + a[3] * a[3]);
      const double kin_b = 0.5 * (b[1] * b[1] + b[2] * b[2] + b[3] * b[3]);
      const double rho_avg = 0.5 * (a[0] + b[0]);
      const double rho_mean = ln_mean(a[0], b[0]);
      const double beta_mean = ln_mean(beta_a, beta_b);
      const double beta_avg = 0.5 * (beta_a + beta_b);
      const double p_mean = 0.5 * rho_avg / beta_avg;
      const double f1 = rho_mean * 0.5 * (vna + vnb);
      f[0] = f1;
      for (int d = 0; d < 3; ++d) f[1 + d] = f1 * vavg[d] + p_mean * n[d];
      f[4] = f1 * 0.5 * (1 / (eq.gamma - 1) / beta_mean - (kin_a + kin_b)) + f[1] * vavg[0] +
             f[2] * vavg[1] + f[3] * vavg[2];
      return;
    }
    default: break;
  }
  double fl[5], fr[5];
  flux3_n(eq, ul, n, fl);
  flux3_n(eq, ur, n, fr);
  for (int v = 0; v < 5; ++v) f[v] = 0.5 * (fl[v] + fr[v]);
  if (kind == FLUX_LAX_FRIEDRICHS || kind == FLUX_LAX_FRIEDRICHS_NAIVE) {
    // max_abs_speed(_naive)(u_ll, u_rr, normal_direction), compressible_euler_3d.jl
    const double ca = std::sqrt(eq.gamma * a[4] / a[0]), cb = std::sqrt(eq.gamma * b[4] / b[0]);
    const double nn = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    const double lam = kind == FLUX_LAX_FRIEDRICHS_NAIVE
                           ? std::max(std::fabs(vna), std::fabs(vnb)) + std::max(ca, cb) * nn
                           : std::max(std::fabs(vna) + ca * nn, std::fabs(vnb) + cb * nn);
    for (int v = 0; v < 5; ++v) f[v] = f[v] + (-0.5 * lam * (ur[v] - ul[v]));
  }
}

struct Curved3 {
  Eq eq;
  Basis b;
  int n = 0, nn = 0;
  int64_t E = 0;
  int vi = VI_WEAK, vf = FLUX_CENTRAL, sf = FLUX_LAX_FRIEDRICHS, source = SRC_NONE;
  std::vector<double> x;     // [E][nn][3], node = i + n j + n^2 k
  std::vector<int64_t> nbr;  // [E][6]: -x, +x, -y, +y, -z, +z (< 0: Dirichlet face)
  std::vector<double> Ja;    // [E][nn][9]: Ja^d_c at d * 3 + c
  std::vector<double> invJ;  // [E][nn]
  int bc_ic = -1;
  double bc_par[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  // VolumeIntegralShockCapturingHG: indicator parameters, the FV flux and the
  // subcell normals [E][d][l][n - 1][3] (calc_normalvectors_subcell_fv!,
  // containers_3d.jl:352-470): direction d, line l = the two other indices
  // (lower one fastest), subcell interface between nodes i and i + 1
  double alpha_max = 0.5, alpha_min = 0.001;
  bool alpha_smooth = true;
  int fvflux = FLUX_LAX_FRIEDRICHS;
  std::vector<double> snv;
  size_t ui(int64_t e, int q) const { return ((size_t)e * nn + q) * 5; }
  int node(int i, int j, int k) const { return i + n * (j + n * k); }
  // node a of line l = (l0, l1) in direction d
  int line_node(int d, int l, int a) const {
    const int l0 = l % n, l1 = l / n;
    return d == 0 ? node(a, l0, l1) : (d == 1 ? node(l0, a, l1) : node(l0, l1, a));
  }
};

// calc_normalvectors_subcell_fv! (3D): per direction, Ja^d at the line's first
// node plus the partial sums of w_i D[i, :] Ja^d along the line
static void curved3_subcell_normals(Curved3& c) {
  const int n = c.n, nn = c.nn, nf = n * n;
  const std::vector<double>& Dm = c.b.D;
  const std::vector<double>& w = c.b.weights;
  c.snv.assign((size_t)c.E * 3 * nf * (n - 1) * 3, 0.0);
  for (int64_t e = 0; e < c.E; ++e)
    for (int d = 0; d < 3; ++d)
      for (int l = 0; l < nf; ++l) {
        double acc[3];
        for (int xyz = 0; xyz < 3; ++xyz)
          acc[xyz] = c.Ja[((size_t)e * nn + c.line_node(d, l, 0)) * 9 + 3 * d + xyz];
        for (int i = 0; i < n - 1; ++i) {
          for (int m = 0; m < n; ++m) {
            const double wd = w[i] * Dm[i * n + m];
            for (int xyz = 0; xyz < 3; ++xyz)
              acc[xyz] += wd * c.Ja[((size_t)e * nn + c.line_node(d, l, m)) * 9 + 3 * d + xyz];
          }
          for (int xyz = 0; xyz < 3; ++xyz)
            c.snv[((((size_t)e * 3 + d) * nf + l) * (n - 1) + i) * 3 + xyz] = acc[xyz];
        }
      }
}

// IndicatorHennemannGassner on density_pressure (indicators.jl:114-148,
// indicators_3d.jl:39-123) per element, smoothed over the face neighbours
static void curved3_hg_alpha(const Curved3& c, const double* u, std::vector<double>& alpha) {
  const int n = c.n, nn = c.nn;
  const double threshold = 0.5 * std::pow(10.0, -1.8 * std::pow((double)n, 0.25));
  const double parameter_s = std::log((1 - 0.0001) / 0.0001);
  alpha.assign(c.E, 0.0);
  const double* V = c.b.Vinv.data();
  std::vector<double> a(nn), t(nn);
  for (int64_t e = 0; e < c.E; ++e) {
    for (int q = 0; q < nn; ++q) a[q] = density_pressure(c.eq, &u[c.ui(e, q)]);
    // multiply_scalar_dimensionwise!: x, then y, then z
    for (int d = 0; d < 3; ++d) {
      for (int k = 0; k < n; ++k)
        for (int j = 0; j < n; ++j)
          for (int i = 0; i < n; ++i) {
            const int idx[3] = {i, j, k};
            double r = 0;
            for (int s = 0; s < n; ++s) {
              int id2[3] = {i, j, k};
              id2[d] = s;
              r += V[idx[d] * n + s] * a[c.node(id2[0], id2[1], id2[2])];
            }
            t[c.node(i, j, k)] = r;
          }
      std::swap(a, t);
    }
    double e_clip2 = 0, e_clip1 = 0, e_tot = 0;
    for (int q = 0; q < nn; ++q) {
      const int mx = std::max({q % n, (q / n) % n, q / (n * n)});
      const double m2 = a[q] * a[q];
      if (mx <= n - 3) e_clip2 += m2;
      if (mx <= n - 2) e_clip1 += m2;
      e_tot += m2;
    }
    const double f1 = e_tot != 0 ? (e_tot - e_clip1) / e_tot : 0.0;
    const double f2 = e_clip1 != 0 ? (e_clip1 - e_clip2) / e_clip1 : 0.0;
    const double energy = std::max(f1, f2);
    double al = 1 / (1 + std::exp(-parameter_s / threshold * (energy - threshold)));
    if (al < c.alpha_min) al = 0;
    if (al > 1 - c.alpha_min) al = 1;
    alpha[e] = std::min(c.alpha_max, al);
  }
  if (c.alpha_smooth) {
    const std::vector<double> tmp = alpha;
    for (int64_t e = 0; e < c.E; ++e)
      for (int o = 0; o < 3; ++o) {
        const int64_t r = c.nbr[e * 6 + 2 * o + 1];  // interface (e, r) in direction o
        if (r < 0) continue;
        alpha[e] = std::max({tmp[e], 0.5 * tmp[r], alpha[e]});
        alpha[r] = std::max({tmp[r], 0.5 * tmp[e], alpha[r]});
      }
  }
}

// calc_jacobian_matrix!, calc_contravariant_vectors! (curl form),
// calc_inverse_jacobian! (containers_3d.jl:67-286)
static void curved3_metric(Curved3& c) {
  const int n = c.n, nn = c.nn;
  const std::vector<double>& Dm = c.b.D;
  c.Ja.assign((size_t)c.E * nn * 9, 0.0);
  c.invJ.assign((size_t)c.E * nn, 0.0);
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < c.E; ++e) {
    const double* X = &c.x[(size_t)e * nn * 3];
    std::vector<double> J((size_t)nn * 9);  // J[q][c * 3 + d] = dX_c / dxi_d
    for (int k = 0; k < n; ++k)
      for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) {
          const int q = c.node(i, j, k);
          for (int cc = 0; cc < 3; ++cc) {
            double r0 = 0, r1 = 0, r2 = 0;
            for (int s = 0; s < n; ++s) {
              r0 += Dm[i * n + s] * X[c.node(s, j, k) * 3 + cc];
              r1 += Dm[j * n + s] * X[c.node(i, s, k) * 3 + cc];
              r2 += Dm[k * n + s] * X[c.node(i, j, s) * 3 + cc];
            }
            J[q * 9 + cc * 3 + 0] = r0;
            J[q * 9 + cc * 3 + 1] = r1;
            J[q * 9 + cc * 3 + 2] = r2;
          }
        }
    // (X_m dX_l/dxi_d - X_l dX_m/dxi_d) at node q
    auto g = [&](int q, int m, int l, int d) {
      return X[q * 3 + m] * J[q * 9 + l * 3 + d] - X[q * 3 + l] * J[q * 9 + m * 3 + d];
    };
    double* Ja = &c.Ja[(size_t)e * nn * 9];
    for (int k = 0; k < n; ++k)
      for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) {
          const int q = c.node(i, j, k);
          for (int cn = 0; cn < 3; ++cn) {
            const int m = (cn + 1) % 3, l = (cn + 2) % 3;
            double a1 = 0, a2 = 0, b1 = 0, b2 = 0, c1 = 0, c2 = 0;
            for (int s = 0; s < n; ++s) {
              a1 += 0.5 * Dm[j * n + s] * g(c.node(i, s, k), m, l, 2);  // (.)_zeta, d/deta
              a2 += 0.5 * Dm[k * n + s] * g(c.node(i, j, s), m, l, 1);  // (.)_eta, d/dzeta
              b1 += 0.5 * Dm[k * n + s] * g(c.node(i, j, s), m, l, 0);  // (.)_xi, d/dzeta
              b2 += 0.5 * Dm[i * n + s] * g(c.node(s, j, k), m, l, 2);  // (.)_zeta, d/dxi
              c1 += 0.5 * Dm[i * n + s] * g(c.node(s, j, k), m, l, 1);  // (.)_eta, d/dxi
              c2 += 0.5 * Dm[j * n + s] * g(c.node(i, s, k), m, l, 0);  // (.)_xi, d/deta
            }
            Ja[q * 9 + 0 * 3 + cn] = a1 - a2;
            Ja[q * 9 + 1 * 3 + cn] = b1 - b2;
            Ja[q * 9 + 2 * 3 + cn] = c1 - c2;
          }
          const double* M = &J[q * 9];
          const double det = M[0] * M[4] * M[8] + M[1] * M[5] * M[6] + M[2] * M[3] * M[7] -
                             M[2] * M[4] * M[6] - M[1] * M[3] * M[8] - M[0] * M[5] * M[7];
          c.invJ[(size_t)e * nn + q] = 1.0 / det;
        }
  }
}

}  // namespace orc

namespace orc {

// rhs! on a curvilinear 3D mesh (dgsem_structured/dg_3d.jl: weak form and flux
// differencing with contravariant fluxes, interface fluxes along the + side
// element's contravariant vector, Dirichlet faces, surface integral,
// per-node Jacobian, sources)
static void curved3_rhs(const Curved3& c, double* du, const double* u, double t) {
  const int n = c.n, nn = c.nn, nf = n * n;
  const Basis& b = c.b;
  const Eq& eq = c.eq;
  std::vector<double> sfv((size_t)c.E * 6 * nf * 5);  // [E][dir][face node][v]
  // VolumeIntegralShockCapturingHG (calc_volume_integral.jl:231-272)
  const bool hg = c.vi == VI_SHOCKCAPTURING_HG;
  std::vector<double> alpha;
  if (hg) curved3_hg_alpha(c, u, alpha);
  const double atol = std::max(100 * 2.220446049250313e-16, std::pow(2.220446049250313e-16, 0.75));
  // face node (a, b) of direction o at the - side (s = 0) or + side (s = n - 1)
  auto fnode = [&](int o, int a, int bb, int s) {
    return o == 0 ? c.node(s, a, bb) : (o == 1 ? c.node(a, s, bb) : c.node(a, bb, s));
  };
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < c.E; ++e)
    for (int o = 0; o < 3; ++o) {
      const int64_t left = c.nbr[e * 6 + 2 * o];
      if (left < 0) continue;
      for (int bb = 0; bb < n; ++bb)
        for (int a = 0; a < n; ++a) {
          const int qr = fnode(o, a, bb, 0), ql = fnode(o, a, bb, n - 1);
          const double sj = c.invJ[(size_t)e * nn + qr] >= 0 ? 1.0 : -1.0;
          const double* J = &c.Ja[((size_t)e * nn + qr) * 9 + 3 * o];
          const double nd[3] = {sj * J[0], sj * J[1], sj * J[2]};
          double F[5];
          two_point3_n(eq, c.sf, &u[c.ui(left, ql)], &u[c.ui(e, qr)], nd, F);
          const int l = a + n * bb;
          for (int v = 0; v < 5; ++v) {
            sfv[(((size_t)e * 6 + 2 * o) * nf + l) * 5 + v] = sj * F[v];
            sfv[(((size_t)left * 6 + 2 * o + 1) * nf + l) * 5 + v] = sj * F[v];
          }
        }
    }
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < c.E; ++e)
    for (int dir = 0; dir < 6; ++dir) {
      if (c.nbr[e * 6 + dir] >= 0) continue;
      const int o = dir >> 1;
      for (int bb = 0; bb < n; ++bb)
        for (int a = 0; a < n; ++a) {
          const int q = fnode(o, a, bb, (dir & 1) ? n - 1 : 0);
          const double sj = c.invJ[(size_t)e * nn + q] >= 0 ? 1.0 : -1.0;
          const double* J = &c.Ja[((size_t)e * nn + q) * 9 + 3 * o];
          const double nd[3] = {sj * J[0], sj * J[1], sj * J[2]};
          double ub[5], F[5];
          initial_condition(c.eq, c.bc_ic, c.bc_par, &c.x[((size_t)e * nn + q) * 3], t, ub);
          if (dir & 1)
            two_point3_n(eq, c.sf, &u[c.ui(e, q)], ub, nd, F);
          else
            two_point3_n(eq, c.sf, ub, &u[c.ui(e, q)], nd, F);
          for (int v = 0; v < 5; ++v) sfv[(((size_t)e * 6 + dir) * nf + a + n * bb) * 5 + v] = sj * F[v];
        }
    }
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < c.E; ++e) {
    double* de = du + (size_t)e * nn * 5;
    const double* ue = u + (size_t)e * nn * 5;
    const double* Ja = &c.Ja[(size_t)e * nn * 9];
    for (int k = 0; k < nn * 5; ++k) de[k] = 0;
    const double ae = hg ? alpha[e] : 0.0;
    const bool dg_only = !hg || std::fabs(ae) <= atol;
    const double fdw = dg_only ? 1.0 : 1.0 - ae;
    for (int k = 0; k < n; ++k)
      for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) {
          const int q = c.node(i, j, k);
          const int idx[3] = {i, j, k};
          if (c.vi == VI_WEAK) {
            double f[3][5] = {};
            for (int o = 0; o < 3; ++o) flux_phys(eq, ue + q * 5, o, f[o]);
            for (int d = 0; d < 3; ++d) {
              const double* a = Ja + q * 9 + 3 * d;
              double cf[5];
              for (int v = 0; v < 5; ++v)
                cf[v] = std::fma(a[2], f[2][v], std::fma(a[1], f[1][v], a[0] * f[0][v]));
              for (int s = 0; s < n; ++s) {
                int id2[3] = {i, j, k};
                id2[d] = s;
                const int r = c.node(id2[0], id2[1], id2[2]);
                for (int v = 0; v < 5; ++v)
                  de[r * 5 + v] = std::fma(b.Dhat[s * n + idx[d]], cf[v], de[r * 5 + v]);
              }
            }
          } else {
            for (int d = 0; d < 3; ++d)
              for (int s = idx[d] + 1; s < n; ++s) {
                int id2[3] = {i, j, k};
                id2[d] = s;
                const int r = c.node(id2[0], id2[1], id2[2]);
                const double* aq = Ja + q * 9 + 3 * d;
                const double* ar = Ja + r * 9 + 3 * d;
                const double avg[3] = {0.5 * (aq[0] + ar[0]), 0.5 * (aq[1] + ar[1]),
                                       0.5 * (aq[2] + ar[2])};
                double F[5];
                two_point3_n(eq, c.vf, ue + q * 5, ue + r * 5, avg, F);
                for (int v = 0; v < 5; ++v) {
                  de[q * 5 + v] = std::fma(fdw * b.Dsplit[idx[d] * n + s], F[v], de[q * 5 + v]);
                  de[r * 5 + v] = std::fma(fdw * b.Dsplit[s * n + idx[d]], F[v], de[r * 5 + v]);
                }
              }
          }
        }
    if (!dg_only) {
      // fv_kernel! / calcflux_fv! (dgsem_structured/dg_3d.jl): subcell fluxes
      // along the subcell normals, zero at the element faces
      for (int d = 0; d < 3; ++d)
        for (int l = 0; l < nf; ++l) {
          double fst[9][5] = {};
          for (int i = 1; i < n; ++i) {
            const double* nv = &c.snv[((((size_t)e * 3 + d) * nf + l) * (n - 1) + (i - 1)) * 3];
            two_point3_n(eq, c.fvflux, ue + c.line_node(d, l, i - 1) * 5,
                         ue + c.line_node(d, l, i) * 5, nv, fst[i]);
          }
          for (int i = 0; i < n; ++i)
            for (int v = 0; v < 5; ++v)
              de[c.line_node(d, l, i) * 5 + v] += ae * (b.inv_weights[i] * (fst[i + 1][v] - fst[i][v]));
        }
    }
    const double factor = b.inv_weights[0];
    const double* sf = &sfv[(size_t)e * 6 * nf * 5];
    for (int o = 0; o < 3; ++o)
      for (int bb = 0; bb < n; ++bb)
        for (int a = 0; a < n; ++a) {
          const int l = a + n * bb;
          const int q0 = fnode(o, a, bb, 0), q1 = fnode(o, a, bb, n - 1);
          for (int v = 0; v < 5; ++v) {
            de[q0 * 5 + v] = de[q0 * 5 + v] - sf[((2 * o) * nf + l) * 5 + v] * factor;
            de[q1 * 5 + v] = de[q1 * 5 + v] + sf[((2 * o + 1) * nf + l) * 5 + v] * factor;
          }
        }
    for (int q = 0; q < nn; ++q) {
      const double fac = -c.invJ[(size_t)e * nn + q];
      for (int v = 0; v < 5; ++v) de[q * 5 + v] *= fac;
      if (c.source == SRC_CONVERGENCE_TEST) {
        double s[5] = {0, 0, 0, 0, 0};
        source_convergence(eq, &c.x[((size_t)e * nn + q) * 3], t, s);
        for (int v = 0; v < 5; ++v) de[q * 5 + v] += s[v];
      }
    }
  }
}

// max_dt on a curvilinear 3D mesh (stepsize_dg3d.jl, curvilinear method)
static double curved3_max_dt(const Curved3& c, const double* u) {
  double mss = 4.9406564584124654e-324;
  for (int64_t e = 0; e < c.E; ++e) {
    double m[3] = {0, 0, 0};
    for (int q = 0; q < c.nn; ++q) {
      double lam[3];
      max_abs_speeds(c.eq, &u[c.ui(e, q)], lam);
      const double* a = &c.Ja[((size_t)e * c.nn + q) * 9];
      const double ij = std::fabs(c.invJ[(size_t)e * c.nn + q]);
      for (int d = 0; d < 3; ++d)
        m[d] = std::max(m[d], std::fabs(a[3 * d] * lam[0] + a[3 * d + 1] * lam[1] +
                                        a[3 * d + 2] * lam[2]) * ij);
    }
    mss = std::max(mss, m[0] + m[1] + m[2]);
  }
  return 2 / (c.n * mss);
}

// calc_error_norms on a curvilinear 3D mesh (analysis_dg3d.jl, curvilinear method)
static void curved3_errors(const Curved3& c, const double* u, double t, int ic, const double* par,
                           double* l2, double* linf) {
  const Basis& b = c.b;
  const int n = c.n, na = b.na, nn = c.nn;
  for (int v = 0; v < 5; ++v) l2[v] = linf[v] = 0;
  double vol = 0;
  // fields per node: 5 state values, 3 coordinates, J
  const int NFLD = 9;
  std::vector<double> f0((size_t)nn * NFLD), f1((size_t)na * n * n * NFLD),
      f2((size_t)na * na * n * NFLD), f3((size_t)na * na * na * NFLD);
  for (int64_t e = 0; e < c.E; ++e) {
    for (int q = 0; q < nn; ++q) {
      for (int v = 0; v < 5; ++v) f0[q * NFLD + v] = u[c.ui(e, q) + v];
      for (int d = 0; d < 3; ++d) f0[q * NFLD + 5 + d] = c.x[((size_t)e * nn + q) * 3 + d];
      f0[q * NFLD + 8] = 1.0 / c.invJ[(size_t)e * nn + q];
    }
    // interpolate along i, j, k in turn (multiply_dimensionwise!)
    for (int k = 0; k < n; ++k)
      for (int j = 0; j < n; ++j)
        for (int a = 0; a < na; ++a)
          for (int f = 0; f < NFLD; ++f) {
            double s = 0;
            for (int i = 0; i < n; ++i) s += b.avand[a * n + i] * f0[(i + n * (j + n * k)) * NFLD + f];
            f1[(a + na * (j + n * k)) * NFLD + f] = s;
          }
    for (int k = 0; k < n; ++k)
      for (int bb = 0; bb < na; ++bb)
        for (int a = 0; a < na; ++a)
          for (int f = 0; f < NFLD; ++f) {
            double s = 0;
            for (int j = 0; j < n; ++j) s += b.avand[bb * n + j] * f1[(a + na * (j + n * k)) * NFLD + f];
            f2[(a + na * (bb + na * k)) * NFLD + f] = s;
          }
    for (int cc = 0; cc < na; ++cc)
      for (int bb = 0; bb < na; ++bb)
        for (int a = 0; a < na; ++a) {
          double* p = &f3[(a + na * (bb + na * cc)) * NFLD];
          for (int f = 0; f < NFLD; ++f) {
            double s = 0;
            for (int k = 0; k < n; ++k) s += b.avand[cc * n + k] * f2[(a + na * (bb + na * k)) * NFLD + f];
            p[f] = s;
          }
          double ue[5];
          initial_condition(c.eq, ic, par, p + 5, t, ue);
          const double wj = b.aweights[a] * b.aweights[bb] * b.aweights[cc] * std::fabs(p[8]);
          for (int v = 0; v < 5; ++v) {
            const double d = ue[v] - p[v];
            l2[v] += d * d * wj;
            linf[v] = std::max(linf[v], std::fabs(d));
          }
          vol += wj;
        }
  }
  for (int v = 0; v < 5; ++v) l2[v] = std::sqrt(l2[v] / vol);
}

}  // namespace orc

extern "C" {

// Curvilinear 3D solver on element node coordinates x[E][n][n][n][3] (i
// fastest) and neighbours nbr[E][6] (0-based; -1: Dirichlet face).
void* orc_curved3_create(int polydeg, int64_t nelements, const double* x, const int64_t* nbr,
                         double gamma, int volume_integral, int volume_flux, int surface_flux,
                         int source) {
  Curved3* c = new Curved3();
  c->eq.D = 3;
  c->eq.NV = 5;
  c->eq.gamma = gamma;
  c->eq.inv_gamma_minus_one = 1 / (gamma - 1);
  c->b = make_basis(polydeg);
  c->n = polydeg + 1;
  c->nn = c->n * c->n * c->n;
  c->E = nelements;
  c->vi = volume_integral;
  c->vf = volume_flux;
  c->sf = surface_flux;
  c->source = source;
  c->x.assign(x, x + (size_t)nelements * c->nn * 3);
  c->nbr.assign(nbr, nbr + (size_t)nelements * 6);
  curved3_metric(*c);
  return c;
}

void orc_curved3_destroy(void* h) { delete (Curved3*)h; }

// VolumeIntegralShockCapturingHG settings of a 3D curvilinear mesh
void orc_curved3_set_hg(void* h, double alpha_max, double alpha_min, int alpha_smooth, int fvflux) {
  Curved3& c = *(Curved3*)h;
  c.alpha_max = alpha_max;
  c.alpha_min = alpha_min;
  c.alpha_smooth = alpha_smooth != 0;
  c.fvflux = fvflux;
  curved3_subcell_normals(c);
}

// Smoothed blending factors of a state, alpha[E]
void orc_curved3_alpha(void* h, const double* u, double* alpha) {
  std::vector<double> a;
  curved3_hg_alpha(*(const Curved3*)h, u, a);
  std::copy(a.begin(), a.end(), alpha);
}

void orc_curved3_set_dirichlet(void* h, int ic, const double* params) {
  Curved3& c = *(Curved3*)h;
  c.bc_ic = ic;
  for (int k = 0; k < 8; ++k) c.bc_par[k] = params ? params[k] : 0.0;
}

// contravariant_vectors [E][n][n][n][3 (dir)][3 (xyz)], inverse_jacobian [E][n][n][n]
void orc_curved3_metric(void* h, double* contravariant, double* inverse_jacobian) {
  Curved3& c = *(Curved3*)h;
  std::copy(c.Ja.begin(), c.Ja.end(), contravariant);
  std::copy(c.invJ.begin(), c.invJ.end(), inverse_jacobian);
}

void orc_curved3_initial_condition(void* h, int ic, const double* params, double t, double* u) {
  Curved3& c = *(Curved3*)h;
  for (int64_t e = 0; e < c.E; ++e)
    for (int q = 0; q < c.nn; ++q)
      initial_condition(c.eq, ic, params, &c.x[((size_t)e * c.nn + q) * 3], t, &u[c.ui(e, q)]);
}

void orc_curved3_rhs(void* h, double* du, const double* u, double t) {
  curved3_rhs(*(Curved3*)h, du, u, t);
}

double orc_curved3_max_dt(void* h, const double* u) { return curved3_max_dt(*(Curved3*)h, u); }

int orc_curved3_solve(void* h, double* u, double t0, double t_end, double cfl, int64_t max_steps,
                      double* t_out, int64_t* nsteps_out) {
  Curved3& c = *(Curved3*)h;
  const int64_t ndof = c.E * c.nn * 5;
  std::vector<double> du(ndof), u_tmp(ndof);
  double t = t0;
  double dt = cfl * curved3_max_dt(c, u);
  int64_t iter = 0;
  bool finalstep = false;
  while (!finalstep && iter < max_steps) {
    if (std::isnan(dt)) {
      *t_out = t;
      *nsteps_out = iter;
      return -1;
    }
    if (t + dt > t_end || isapprox(t + dt, t_end)) {
      dt = t_end - t;
      finalstep = true;
    }
    std::fill(u_tmp.begin(), u_tmp.end(), 0.0);
    for (int stage = 0; stage < 5; ++stage) {
      curved3_rhs(c, du.data(), u, t + dt * CK_C[stage]);
      rk_update(ndof, u, u_tmp.data(), du.data(), CK_A[stage], CK_B[stage] * dt);
    }
    iter += 1;
    t += dt;
    dt = cfl * curved3_max_dt(c, u);
  }
  *t_out = t;
  *nsteps_out = iter;
  return 0;
}

void orc_curved3_errors(void* h, const double* u, double t, int ic, const double* params,
                        double* l2, double* linf) {
  curved3_errors(*(Curved3*)h, u, t, ic, params, l2, linf);
}

}  // extern "C"
