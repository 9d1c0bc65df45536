// Compressible Euler physics for the GB300 DGSEM kernels, templated on the
// compute type R (double for the FP64 path, float for the mixed path) and on
// the dimension D.  State vectors live in registers: u[NV] conservative,
// w[NV] primitive (rho, v_1..v_D, p), NV = D + 2.
//
// Formulas follow src/equations/compressible_euler_{2,3}d.jl,
// src/equations/numerical_fluxes.jl and src/auxiliary/math.jl of Trixi.jl.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace tg {

enum VolumeIntegralKind { VI_WEAK = 0, VI_FD = 1, VI_HG = 2 };
enum FluxKind {
  FLUX_CENTRAL = 0,
  FLUX_RANOCHA = 1,
  FLUX_SHIMA_ETAL = 2,
  FLUX_LLF = 3,
  FLUX_LLF_NAIVE = 4,
  FLUX_HLLC = 5,
  FLUX_CHANDRASHEKAR = 6,
  FLUX_HLLE = 7
};
enum SourceKind { SRC_NONE = 0, SRC_CONVERGENCE_TEST = 1 };
// boundary conditions of a non-periodic TreeMesh, per direction
enum BoundaryKind { BC_PERIODIC = 0, BC_DIRICHLET = 1, BC_SLIP_WALL = 2 };
// initial conditions a Dirichlet boundary can take its values from
enum InitialConditionKind {
  IC_CONSTANT = 0,
  IC_CONVERGENCE_TEST = 1,
  IC_ISENTROPIC_VORTEX = 2,
  IC_WEAK_BLAST_WAVE = 3,
  IC_KELVIN_HELMHOLTZ = 4,
  IC_TAYLOR_GREEN = 5,
  IC_GAUSSIAN_BLAST = 6
};

template <typename R>
struct Real;

template <>
struct Real<double> {
  static __host__ __device__ __forceinline__ double log(double x) { return ::log(x); }
  static __host__ __device__ __forceinline__ double sqrt(double x) { return ::sqrt(x); }
  static __host__ __device__ __forceinline__ double sin(double x) { return ::sin(x); }
  static __host__ __device__ __forceinline__ double cos(double x) { return ::cos(x); }
  static __host__ __device__ __forceinline__ double exp(double x) { return ::exp(x); }
};

template <>
struct Real<float> {
  // logf / sinf / cosf / expf are CUDA's accurate single-precision functions;
  // division and sqrt follow the translation unit's -prec-div/-prec-sqrt.
  static __host__ __device__ __forceinline__ float log(float x) { return ::logf(x); }
  static __host__ __device__ __forceinline__ float sqrt(float x) { return ::sqrtf(x); }
  static __host__ __device__ __forceinline__ float sin(float x) { return ::sinf(x); }
  static __host__ __device__ __forceinline__ float cos(float x) { return ::cosf(x); }
  static __host__ __device__ __forceinline__ float exp(float x) { return ::expf(x); }
};

// ---------------------------------------------------------------------------
// Logarithmic mean (math.jl:198-250).
//
// FP64: Trixi's algorithm as is -- the series in f^2 = ((y-x)/(y+x))^2 below
// f^2 < 1e-4, else (y - x) / log(y / x).
//
// FP32: the same series, one term longer (2/9 f^8), used below f^2 < 0.05.
// Its truncation error is f^10 / 11 < 3e-8 there, under FP32 rounding, and
// above the switch y/x > 1.58 so log(y/x) > 0.45 keeps the direct formula
// well conditioned; f is formed as (y-x)/(y+x) instead of Trixi's
// cancellation-prone quotient of quadratics.
// ---------------------------------------------------------------------------
__host__ __device__ __forceinline__ double ln_mean(double x, double y) {
  const double f2 = (x * (x - 2 * y) + y * y) / (x * (x + 2 * y) + y * y);
  if (f2 < 1.0e-4)
    return (x + y) / (2.0 + f2 * (2.0 / 3.0 + f2 * (2.0 / 5.0 + f2 * (2.0 / 7.0))));
  return (y - x) / ::log(y / x);
}
__host__ __device__ __forceinline__ double inv_ln_mean(double x, double y) {
  const double f2 = (x * (x - 2 * y) + y * y) / (x * (x + 2 * y) + y * y);
  if (f2 < 1.0e-4)
    return (2.0 + f2 * (2.0 / 3.0 + f2 * (2.0 / 5.0 + f2 * (2.0 / 7.0)))) / (x + y);
  return ::log(y / x) / (y - x);
}
__host__ __device__ __forceinline__ float ln_mean(float x, float y) {
  const float f = (y - x) / (y + x);
  const float f2 = f * f;
  if (f2 < 0.05f)
    return (x + y) /
           (2.0f + f2 * (2.0f / 3.0f + f2 * (2.0f / 5.0f + f2 * (2.0f / 7.0f + f2 * (2.0f / 9.0f)))));
  return (y - x) / ::logf(y / x);
}
__host__ __device__ __forceinline__ float inv_ln_mean(float x, float y) {
  const float f = (y - x) / (y + x);
  const float f2 = f * f;
  if (f2 < 0.05f)
    return (2.0f + f2 * (2.0f / 3.0f + f2 * (2.0f / 5.0f + f2 * (2.0f / 7.0f + f2 * (2.0f / 9.0f))))) /
           (x + y);
  return ::logf(y / x) / (y - x);
}

template <int D, typename R>
struct Euler {
  static constexpr int NV = D + 2;
  static constexpr int P = D + 1;

  // cons2prim, compressible_euler_2d.jl:2038-2046
  static __host__ __device__ __forceinline__ void cons2prim(const R* u, R* w, R gamma) {
    const R rho = u[0];
    const R inv_rho = R(1) / rho;
    R ke = 0;
#pragma unroll
    for (int d = 0; d < D; ++d) {
      w[1 + d] = u[1 + d] * inv_rho;
      ke += u[1 + d] * w[1 + d];
    }
    w[0] = rho;
    w[P] = (gamma - R(1)) * (u[P] - R(0.5) * ke);
  }

  // Component o (0-based direction) of a D-vector stored at a[0..D-1], with a
  // runtime o but compile-time indexing only (keeps arrays in registers).
  static __host__ __device__ __forceinline__ R pick(const R* a, int o) {
    R r = a[0];
#pragma unroll
    for (int d = 1; d < D; ++d) r = (o == d) ? a[d] : r;
    return r;
  }

  // flux(u, orientation), compressible_euler_2d.jl:415-432, 3d.jl:420-447
  static __host__ __device__ __forceinline__ void flux(const R* u, const R* w, int o, R* f) {
    const R rvo = pick(u + 1, o);
    const R vo = pick(w + 1, o);
    f[0] = rvo;
#pragma unroll
    for (int d = 0; d < D; ++d) f[1 + d] = (d == o) ? rvo * w[1 + d] + w[P] : rvo * w[1 + d];
    f[P] = (u[P] + w[P]) * vo;
  }

  // flux_ranocha, compressible_euler_2d.jl:686-722, 3d.jl:746-792
  static __host__ __device__ __forceinline__ void flux_ranocha(const R* wl, const R* wr, int o,
                                                       R inv_gm1, R* f) {
    const R rho_mean = ln_mean(wl[0], wr[0]);
    const R inv_rho_p_mean = wl[P] * wr[P] * inv_ln_mean(wl[0] * wr[P], wr[0] * wl[P]);
    R vavg[D];
    R vsq = 0;
#pragma unroll
    for (int d = 0; d < D; ++d) {
      vavg[d] = R(0.5) * (wl[1 + d] + wr[1 + d]);
      vsq += wl[1 + d] * wr[1 + d];
    }
    vsq *= R(0.5);
    const R p_avg = R(0.5) * (wl[P] + wr[P]);
    const R f1 = rho_mean * pick(vavg, o);
    f[0] = f1;
#pragma unroll
    for (int d = 0; d < D; ++d) f[1 + d] = (d == o) ? f1 * vavg[d] + p_avg : f1 * vavg[d];
    f[P] = f1 * (vsq + inv_rho_p_mean * inv_gm1) +
           R(0.5) * (wl[P] * pick(wr + 1, o) + wr[P] * pick(wl + 1, o));
  }

  // flux_chandrashekar, compressible_euler_2d.jl (orientation method), 3d.jl:640-692
  static __host__ __device__ __forceinline__ void flux_chandrashekar(const R* wl, const R* wr, int o,
                                                             R inv_gm1, R* f) {
    const R beta_ll = R(0.5) * wl[0] / wl[P], beta_rr = R(0.5) * wr[0] / wr[P];
    R kin = 0, vavg[D];
#pragma unroll
    for (int d = 0; d < D; ++d) {
      kin += wl[1 + d] * wl[1 + d] + wr[1 + d] * wr[1 + d];
      vavg[d] = R(0.5) * (wl[1 + d] + wr[1 + d]);
    }
    const R rho_mean = ln_mean(wl[0], wr[0]);
    const R beta_mean = ln_mean(beta_ll, beta_rr);
    const R p_mean = R(0.5) * (R(0.5) * (wl[0] + wr[0])) / (R(0.5) * (beta_ll + beta_rr));
    const R f1 = rho_mean * pick(vavg, o);
    f[0] = f1;
    R e = f1 * R(0.5) * (inv_gm1 / beta_mean - R(0.5) * kin);
#pragma unroll
    for (int d = 0; d < D; ++d) {
      f[1 + d] = (d == o) ? f1 * vavg[d] + p_mean : f1 * vavg[d];
      e += f[1 + d] * vavg[d];
    }
    f[P] = e;
  }

  // flux_hlle = FluxHLL(min_max_speed_einfeldt): numerical_fluxes.jl:422-457,
  // compressible_euler_2d.jl:1925-1963 (3d analogue)
  static __host__ __device__ __forceinline__ void flux_hlle(const R* ul, const R* wl, const R* ur,
                                                    const R* wr, int o, R gamma, R* F) {
    R lmin, lmax;
    einfeldt(ul, wl, ur, wr, o, gamma, lmin, lmax);
    if (lmin >= R(0) && lmax >= R(0)) {
      flux(ul, wl, o, F);
      return;
    }
    if (lmax <= R(0) && lmin <= R(0)) {
      flux(ur, wr, o, F);
      return;
    }
    R fl[NV], fr[NV];
    flux(ul, wl, o, fl);
    flux(ur, wr, o, fr);
    const R id = R(1) / (lmax - lmin);
    const R a = lmax * id, b = lmin * id, c = lmin * lmax * id;
#pragma unroll
    for (int v = 0; v < NV; ++v) F[v] = a * fl[v] - b * fr[v] + c * (ur[v] - ul[v]);
  }

  // min_max_speed_einfeldt, compressible_euler_2d.jl:1925-1963
  static __host__ __device__ __forceinline__ void einfeldt(const R* ul, const R* wl, const R* ur,
                                                   const R* wr, int o, R gamma, R& lmin, R& lmax) {
    const R Hl = (ul[P] + wl[P]) / wl[0], Hr = (ur[P] + wr[P]) / wr[0];
    const R cl = Real<R>::sqrt(gamma * wl[P] / wl[0]), cr = Real<R>::sqrt(gamma * wr[P] / wr[0]);
    const R sl = Real<R>::sqrt(wl[0]), sr = Real<R>::sqrt(wr[0]);
    const R inv = R(1) / (sl + sr);
    R vroe2 = 0, vroe_o = 0;
#pragma unroll
    for (int d = 0; d < D; ++d) {
      const R vr = (sl * wl[1 + d] + sr * wr[1 + d]) * inv;
      vroe2 += vr * vr;
      if (d == o) vroe_o = vr;
    }
    const R H_roe = (sl * Hl + sr * Hr) * inv;
    const R c_roe = Real<R>::sqrt((gamma - R(1)) * (H_roe - R(0.5) * vroe2));
    const R beta = Real<R>::sqrt(R(0.5) * (gamma - R(1)) / gamma);
    lmin = fmin(fmin(vroe_o - c_roe, pick(wl + 1, o) - beta * cl), R(0));
    lmax = fmax(fmax(vroe_o + c_roe, pick(wr + 1, o) + beta * cr), R(0));
  }

  // flux_shima_etal, compressible_euler_2d.jl:466-495
  static __host__ __device__ __forceinline__ void flux_shima(const R* wl, const R* wr, int o, R inv_gm1,
                                                     R* f) {
    const R rho_avg = R(0.5) * (wl[0] + wr[0]);
    R vavg[D];
    R kin = 0;
#pragma unroll
    for (int d = 0; d < D; ++d) {
      vavg[d] = R(0.5) * (wl[1 + d] + wr[1 + d]);
      kin += wl[1 + d] * wr[1 + d];
    }
    kin *= R(0.5);
    const R p_avg = R(0.5) * (wl[P] + wr[P]);
    const R vo = pick(vavg, o);
    const R pv_avg = R(0.5) * (wl[P] * pick(wr + 1, o) + wr[P] * pick(wl + 1, o));
    const R f1 = rho_avg * vo;
    f[0] = f1;
#pragma unroll
    for (int d = 0; d < D; ++d) f[1 + d] = (d == o) ? f1 * vavg[d] + p_avg : f1 * vavg[d];
    f[P] = p_avg * vo * inv_gm1 + f1 * kin + pv_avg;
  }

  // flux_central, numerical_fluxes.jl:17-25
  static __host__ __device__ __forceinline__ void flux_central(const R* ul, const R* wl, const R* ur,
                                                       const R* wr, int o, R* f) {
    R fl[NV], fr[NV];
    flux(ul, wl, o, fl);
    flux(ur, wr, o, fr);
#pragma unroll
    for (int v = 0; v < NV; ++v) f[v] = R(0.5) * (fl[v] + fr[v]);
  }

  // FluxLaxFriedrichs(max_abs_speed[_naive]), numerical_fluxes.jl:166-178, 222-253,
  // max_abs_speed(_naive), compressible_euler_2d.jl:1423-1482
  static __host__ __device__ __forceinline__ void flux_llf(const R* ul, const R* wl, const R* ur,
                                                   const R* wr, int o, bool naive, R gamma,
                                                   R* f) {
    flux_central(ul, wl, ur, wr, o, f);
    const R cl = Real<R>::sqrt(gamma * wl[P] / wl[0]);
    const R cr = Real<R>::sqrt(gamma * wr[P] / wr[0]);
    const R al = fabs(pick(wl + 1, o)), ar = fabs(pick(wr + 1, o));
    const R lam = naive ? fmax(al, ar) + fmax(cl, cr) : fmax(al + cl, ar + cr);
#pragma unroll
    for (int v = 0; v < NV; ++v) f[v] = f[v] + (R(-0.5) * lam * (ur[v] - ul[v]));
  }

  // flux_hllc, compressible_euler_2d.jl:1720-1816, 3d.jl:1423-1541: Toro's HLLC
  // with signal speeds bounded by the Roe average
  static __host__ __device__ __forceinline__ void flux_hllc(const R* ul, const R* wl, const R* ur,
                                                    const R* wr, int o, R gamma, R* F) {
    const R rl = wl[0], rr = wr[0], pl = wl[P], pr = wr[P];
    const R cl = Real<R>::sqrt(gamma * pl / rl), cr = Real<R>::sqrt(gamma * pr / rr);
    const R sl = Real<R>::sqrt(rl), sr = Real<R>::sqrt(rr), ss = sl + sr;
    const R vel_L = pick(wl + 1, o), vel_R = pick(wr + 1, o);
    const R vel_roe = (sl * vel_L + sr * vel_R) / ss;
    R vroe2 = 0;
#pragma unroll
    for (int d = 0; d < D; ++d) {
      const R vroe = sl * wl[1 + d] + sr * wr[1 + d];
      vroe2 += vroe * vroe;
    }
    const R Hl = (ul[P] + pl) / rl, Hr = (ur[P] + pr) / rr;
    const R H_roe = (sl * Hl + sr * Hr) / ss;
    const R c_roe = Real<R>::sqrt((gamma - R(1)) * (H_roe - R(0.5) * (vroe2 / (ss * ss))));
    const R Ssl = fmin(vel_L - cl, vel_roe - c_roe);
    const R Ssr = fmax(vel_R + cr, vel_roe + c_roe);
    if (Ssl >= R(0)) {
      flux(ul, wl, o, F);
      return;
    }
    if (Ssr <= R(0)) {
      flux(ur, wr, o, F);
      return;
    }
    const R sMu_L = Ssl - vel_L, sMu_R = Ssr - vel_R;
    const R SStar = (pr - pl + rl * vel_L * sMu_L - rr * vel_R * sMu_R) / (rl * sMu_L - rr * sMu_R);
    const bool left = SStar >= R(0);
    const R* u = left ? ul : ur;
    const R* w = left ? wl : wr;
    const R S = left ? Ssl : Ssr, sMu = left ? sMu_L : sMu_R;
    const R rho = w[0], vel = left ? vel_L : vel_R, p = w[P];
    flux(u, w, o, F);
    const R densStar = rho * sMu / (S - SStar);
    const R enerStar = u[P] / rho + (SStar - vel) * (SStar + p / (rho * sMu));
    F[0] += S * (densStar - u[0]);
#pragma unroll
    for (int d = 0; d < D; ++d) F[1 + d] += S * (densStar * (d == o ? SStar : w[1 + d]) - u[1 + d]);
    F[P] += S * (densStar * enerStar - u[P]);
  }

  static __host__ __device__ __forceinline__ void two_point(int kind, const R* ul, const R* wl,
                                                    const R* ur, const R* wr, int o, R gamma,
                                                    R inv_gm1, R* f) {
    switch (kind) {
      case FLUX_RANOCHA: flux_ranocha(wl, wr, o, inv_gm1, f); break;
      case FLUX_SHIMA_ETAL: flux_shima(wl, wr, o, inv_gm1, f); break;
      case FLUX_LLF: flux_llf(ul, wl, ur, wr, o, false, gamma, f); break;
      case FLUX_LLF_NAIVE: flux_llf(ul, wl, ur, wr, o, true, gamma, f); break;
      case FLUX_HLLC: flux_hllc(ul, wl, ur, wr, o, gamma, f); break;
      case FLUX_CHANDRASHEKAR: flux_chandrashekar(wl, wr, o, inv_gm1, f); break;
      case FLUX_HLLE: flux_hlle(ul, wl, ur, wr, o, gamma, f); break;
      default: flux_central(ul, wl, ur, wr, o, f); break;
    }
  }

  // source_terms_convergence_test, compressible_euler_2d.jl:116-145, 3d.jl:127-150
  static __host__ __device__ __forceinline__ void source_convergence(const R* x, R t, R gamma, R* s) {
    const R c = 2, A = R(0.1);
    const R omega = R(3.141592653589793);  // 2 * pi * (1/2)
    R arg = x[0] + x[1];
    if (D == 3) arg += x[D == 3 ? 2 : 0];
    arg = omega * (arg - t);
    const R si = Real<R>::sin(arg), co = Real<R>::cos(arg);
    const R rho = c + A * si;
    const R rho_x = omega * A * co;
    if (D == 2) {
      const R tmp = (2 * rho - 1) * (gamma - 1);
      s[0] = rho_x;
      s[1] = rho_x * (1 + tmp);
      s[2] = s[1];
      s[P] = 2 * rho_x * (rho + tmp);
    } else {
      const R tmp = (2 * rho - R(1.5)) * (gamma - 1);
      s[0] = 2 * rho_x;
      s[1] = rho_x * (2 + tmp);
      s[2] = s[1];
      s[D] = s[1];
      s[P] = rho_x * (4 * rho + 3 * tmp);
    }
  }

  // density_pressure, compressible_euler_2d.jl:2205-2210
  static __host__ __device__ __forceinline__ R density_pressure(const R* u, R gamma) {
    R m2 = 0;
#pragma unroll
    for (int d = 0; d < D; ++d) m2 += u[1 + d] * u[1 + d];
    return (gamma - R(1)) * (u[0] * u[P] - R(0.5) * m2);
  }
};

// ---------------------------------------------------------------------------
// Boundary values and boundary fluxes of a non-periodic TreeMesh (FP64)
// ---------------------------------------------------------------------------

// Conservative state of an initial condition at x, t: the value a
// BoundaryConditionDirichlet(initial_condition) imposes (equations.jl:164-182).
// par: the free constants of the configurable conditions (see each case).
template <int D>
__host__ __device__ inline void boundary_value(int ic, const double* par, const double* x, double t,
                                               double gamma, double* u) {
  constexpr int NV = D + 2, P = D + 1;
  const double igm1 = 1.0 / (gamma - 1.0);
  double w[NV];
  switch (ic) {
    case IC_CONSTANT:  // compressible_euler_2d.jl:71-78, 3d.jl:71-79
      u[0] = 1.0;
      u[1] = 0.1;
      u[2] = -0.2;
      if (D == 3) u[3] = 0.7;
      u[P] = 10.0;
      return;
    case IC_CONVERGENCE_TEST: {  // compressible_euler_2d.jl:87-104, 3d.jl:93-110
      double s = x[0];
      for (int d = 1; d < D; ++d) s += x[d];
      const double ini = 2.0 + 0.1 * sin(3.141592653589793 * (s - t));
      for (int v = 0; v < P; ++v) u[v] = ini;
      u[P] = ini * ini;
      return;
    }
    case IC_ISENTROPIC_VORTEX: {  // elixir_euler_vortex.jl:18-52; par = {p_inf, amplitude}
      const double p0 = par[0], amp = par[1];
      const double c0 = -x[1], c1 = x[0];
      const double du = amp / (2.0 * 3.141592653589793) * exp(0.5 * (1.0 - (c0 * c0 + c1 * c1)));
      const double dtemp = -(gamma - 1.0) / (2.0 * gamma * p0) * du * du;
      w[0] = pow(1.0 + dtemp, igm1);
      w[1] = 1.0 + du * c0;
      w[2] = 1.0 + du * c1;
      w[P] = p0 * pow(1.0 + dtemp, gamma * igm1);
      break;
    }
    case IC_WEAK_BLAST_WAVE: {  // compressible_euler_2d.jl:245-264, 3d.jl:241-263
      double r2 = 0;
      for (int d = 0; d < D; ++d) r2 += x[d] * x[d];
      const double r = sqrt(r2);
      const bool out = r > 0.5;
      const double phi = atan2(x[1], x[0]);
      w[0] = out ? 1.0 : 1.1691;
      w[P] = out ? 1.0 : 1.245;
      if (D == 2) {
        w[1] = out ? 0.0 : 0.1882 * cos(phi);
        w[2] = out ? 0.0 : 0.1882 * sin(phi);
      } else {
        const double theta = r == 0.0 ? 0.0 : acos(x[D - 1] / r);
        w[1] = out ? 0.0 : 0.1882 * cos(phi) * sin(theta);
        w[2] = out ? 0.0 : 0.1882 * sin(phi) * sin(theta);
        w[D] = out ? 0.0 : 0.1882 * cos(theta);
      }
      break;
    }
    case IC_KELVIN_HELMHOLTZ: {  // elixir_euler_kelvin_helmholtz_instability.jl:18-31
      const double B = tanh(15.0 * x[1] + 7.5) - tanh(15.0 * x[1] - 7.5);
      w[0] = 0.5 + 0.75 * B;
      w[1] = 0.5 * (B - 1.0);
      w[2] = 0.1 * sinpi(2.0 * x[0]);
      for (int d = 3; d <= D; ++d) w[d] = 0.0;
      w[P] = 1.0;
      break;
    }
    case IC_TAYLOR_GREEN: {  // elixir_euler_taylor_green_vortex.jl:14-30; par = {Ma}
      const double Ms = par[0];
      w[0] = 1.0;
      w[1] = sin(x[0]) * cos(x[1]) * cos(x[D - 1]);
      w[2] = -cos(x[0]) * sin(x[1]) * cos(x[D - 1]);
      if (D == 3) w[3] = 0.0;
      w[P] = (1.0 / Ms) * (1.0 / Ms) / gamma +
             1.0 / 16.0 * (cos(2 * x[0]) * cos(2 * x[D - 1]) + 2 * cos(2 * x[1]) + 2 * cos(2 * x[0]) +
                           cos(2 * x[1]) * cos(2 * x[D - 1]));
      break;
    }
    case IC_GAUSSIAN_BLAST: {  // energy deposit; par = {p_bg, E, width}
      const double pbg = par[0], E = par[1], wd = par[2];
      double r2 = 0;
      for (int d = 0; d < D; ++d) r2 += x[d] * x[d];
      const double area = 3.141592653589793 * wd * wd;
      const double norm = D == 2 ? area : area * sqrt(area);
      w[0] = 1.0;
      for (int d = 1; d <= D; ++d) w[d] = 0.0;
      w[P] = pbg + (gamma - 1.0) * E * exp(-r2 / (wd * wd)) / norm;
      break;
    }
    default:
      for (int v = 0; v < NV; ++v) u[v] = NAN;
      return;
  }
  double ke = 0;
  u[0] = w[0];
  for (int d = 0; d < D; ++d) {
    u[1 + d] = w[0] * w[1 + d];
    ke += u[1 + d] * w[1 + d];
  }
  u[P] = w[P] * igm1 + 0.5 * ke;
}

// Pressure of boundary_condition_slip_wall (compressible_euler_2d.jl:322-371,
// 3d.jl:315-373): the 1D pressure Riemann problem of density rho, pressure p
// and outward normal velocity vn; the wall flux is this pressure in the
// normal momentum and zero elsewhere.
template <typename R>
__host__ __device__ inline R slip_wall_pressure(R rho, R vn, R p, R gamma, R igm1) {
  if (vn <= R(0)) {
    const R c = Real<R>::sqrt(gamma * p / rho);
    const R base = R(1) + R(0.5) * (gamma - R(1)) * vn / c;
    return base >= R(0) ? p * pow(base, R(2) * gamma * igm1) : R(0);
  }
  const R A = R(2) / ((gamma + R(1)) * rho);
  const R B = p * (gamma - R(1)) / (gamma + R(1));
  return p + R(0.5) * vn / A * (vn + Real<R>::sqrt(vn * vn + R(4) * A * (p + B)));
}

}  // namespace tg
