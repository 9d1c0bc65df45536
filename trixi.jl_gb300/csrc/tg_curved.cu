// Curvilinear 2D stage kernels (declarations and references in tg_curved.cuh).
//
// Layout as in the TreeMesh kernels: one block owns EPB consecutive elements
// and stages their state in shared memory; one thread owns one (direction,
// line) of an element, evaluates the N(N-1)/2 two-point fluxes of its line
// once each (or the weak-form fluxes) and the two face fluxes at its ends,
// accumulating the line's node contributions in registers; a node phase sums
// the two directions, applies the per-node inverse Jacobian and the sources
// and performs the 2N stage update.  Each interface flux is evaluated by both
// elements with the element on the negative side as the left state: the FP64
// kernel along the contravariant vector of the element on the positive side
// (as Trixi, so both elements evaluate the same flux), the mixed kernel along
// its own element's vector of the shared face (equal up to the rounding of
// the node coordinates the metric was built from).
//
// The mixed kernel evaluates the fluxes in deviation form relative to a
// per-element reference state as the TreeMesh mixed kernel does.  The
// two-point fluxes are linear in the normal direction n, so the deviation of
// a flux along n is n_x times its deviation along x plus n_y times its
// deviation along y; the reference flux f(w_e) . n drops out because the
// metric terms satisfy the discrete metric identities (the scheme preserves
// free streams), which is the curvilinear form of the cancellation used on
// Cartesian elements.  The Lax-Friedrichs dissipation takes its speed from
// the normal velocity and |n|.
#include <cuda_runtime.h>

#include "tg_curved.cuh"

namespace tg {

int curved_epb(int N) { return N == 3 || N == 4 ? 16 : (N == 5 ? 8 : 0); }

// ---------------------------------------------------------------------------
// FP64 fluxes along a normal direction, compressible_euler_2d.jl
// ---------------------------------------------------------------------------
struct FluxN {
  using Eu = Euler<2, double>;

  // flux(u, normal_direction), :436-448
  static __device__ __forceinline__ void phys(const double* u, const double* w, double n0, double n1,
                                              double* f) {
    const double vn = w[1] * n0 + w[2] * n1;
    const double rvn = w[0] * vn;
    f[0] = rvn;
    f[1] = fma(rvn, w[1], w[3] * n0);
    f[2] = fma(rvn, w[2], w[3] * n1);
    f[3] = (u[3] + w[3]) * vn;
  }

  // flux_ranocha(u_ll, u_rr, normal_direction), :724-753
  static __device__ __forceinline__ void ranocha(const double* a, const double* b, double n0,
                                                 double n1, double igm1, double* f) {
    const double vna = a[1] * n0 + a[2] * n1, vnb = b[1] * n0 + b[2] * n1;
    const double rho_mean = ln_mean(a[0], b[0]);
    const double irpm = a[3] * b[3] * inv_ln_mean(a[0] * b[3], b[0] * a[3]);
    const double v1 = 0.5 * (a[1] + b[1]), v2 = 0.5 * (a[2] + b[2]);
    const double p_avg = 0.5 * (a[3] + b[3]);
    const double vsq = 0.5 * (a[1] * b[1] + a[2] * b[2]);
    const double f1 = rho_mean * 0.5 * (vna + vnb);
    f[0] = f1;
    f[1] = fma(f1, v1, p_avg * n0);
    f[2] = fma(f1, v2, p_avg * n1);
    f[3] = f1 * (vsq + irpm * igm1) + 0.5 * (a[3] * vnb + b[3] * vna);
  }

  // flux_shima_etal(u_ll, u_rr, normal_direction), :497-526
  static __device__ __forceinline__ void shima(const double* a, const double* b, double n0,
                                               double n1, double igm1, double* f) {
    const double vna = a[1] * n0 + a[2] * n1, vnb = b[1] * n0 + b[2] * n1;
    const double rho_avg = 0.5 * (a[0] + b[0]);
    const double v1 = 0.5 * (a[1] + b[1]), v2 = 0.5 * (a[2] + b[2]);
    const double vn_avg = 0.5 * (vna + vnb);
    const double p_avg = 0.5 * (a[3] + b[3]);
    const double vsq = 0.5 * (a[1] * b[1] + a[2] * b[2]);
    const double f1 = rho_avg * vn_avg;
    f[0] = f1;
    f[1] = fma(f1, v1, p_avg * n0);
    f[2] = fma(f1, v2, p_avg * n1);
    f[3] = f1 * vsq + p_avg * vn_avg * igm1 + 0.5 * (a[3] * vnb + b[3] * vna);
  }

  // flux_chandrashekar(u_ll, u_rr, normal_direction), :639-670
  static __device__ __forceinline__ void chandrashekar(const double* a, const double* b, double n0,
                                                       double n1, double gamma, double* f) {
    const double vna = a[1] * n0 + a[2] * n1, vnb = b[1] * n0 + b[2] * n1;
    const double beta_a = 0.5 * a[0] / a[3], beta_b = 0.5 * b[0] / b[3];
    const double kin_a = 0.5 * (a[1] * a[1] + a[2] * a[2]);
    const double kin_b = 0.5 * (b[1] * b[1] + b[2] * b[2]);
    const double rho_avg = 0.5 * (a[0] + b[0]);
    const double rho_mean = ln_mean(a[0], b[0]);
    const double beta_mean = ln_mean(beta_a, beta_b);
    const double beta_avg = 0.5 * (beta_a + beta_b);
    const double v1 = 0.5 * (a[1] + b[1]), v2 = 0.5 * (a[2] + b[2]);
    const double p_mean = 0.5 * rho_avg / beta_avg;
    const double f1 = rho_mean * 0.5 * (vna + vnb);
    f[0] = f1;
    f[1] = fma(f1, v1, p_mean * n0);
    f[2] = fma(f1, v2, p_mean * n1);
    f[3] = f1 * 0.5 * (1 / (gamma - 1) / beta_mean - (kin_a + kin_b)) + f[1] * v1 + f[2] * v2;
  }

  // two-point flux of kind k between states (u, w) a and b along (n0, n1):
  // central (+ local Lax-Friedrichs dissipation, max_abs_speed(_naive) along
  // the normal, :1443-1509, numerical_fluxes.jl:17-45, 166-253), ranocha,
  // shima_etal, chandrashekar
  static __device__ __forceinline__ void two_point(int k, const double* ua, const double* wa,
                                                   const double* ub, const double* wb, double n0,
                                                   double n1, double gamma, double igm1,
                                                   double* f) {
    switch (k) {
      case FLUX_RANOCHA: ranocha(wa, wb, n0, n1, igm1, f); return;
      case FLUX_SHIMA_ETAL: shima(wa, wb, n0, n1, igm1, f); return;
      case FLUX_CHANDRASHEKAR: chandrashekar(wa, wb, n0, n1, gamma, f); return;
      default: break;
    }
    double fa[4], fb[4];
    phys(ua, wa, n0, n1, fa);
    phys(ub, wb, n0, n1, fb);
#pragma unroll
    for (int v = 0; v < 4; ++v) f[v] = 0.5 * (fa[v] + fb[v]);
    if (k == FLUX_LLF || k == FLUX_LLF_NAIVE) {
      const double va = wa[1] * n0 + wa[2] * n1, vb = wb[1] * n0 + wb[2] * n1;
      const double ca = sqrt(gamma * wa[3] / wa[0]), cb = sqrt(gamma * wb[3] / wb[0]);
      const double nn = sqrt(n0 * n0 + n1 * n1);
      const double lam = k == FLUX_LLF_NAIVE ? fmax(fabs(va), fabs(vb)) + fmax(ca, cb) * nn
                                             : fmax(fabs(va) + ca * nn, fabs(vb) + cb * nn);
#pragma unroll
      for (int v = 0; v < 4; ++v) f[v] = f[v] + (-0.5 * lam * (ub[v] - ua[v]));
    }
  }
};


}  // namespace tg

namespace tg {


// ---------------------------------------------------------------------------
// FP64 stage kernel
// ---------------------------------------------------------------------------
template <int N, int VI, int EPB>
__global__ void __launch_bounds__(CurvedK<N, EPB>::NT)
    curved_kernel_f64(const CurvedParams P, const StageArgs A) {
  using K = CurvedK<N, EPB>;
  using Eu = Euler<2, double>;
  constexpr int NN = K::NN, NV = 4, NT = K::NT, SP = K::SP, CHUNK = K::CHUNK;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double* s_u = reinterpret_cast<double*>(smem_raw);
  double* s_fu = s_u + CHUNK;
  double* s_part = s_fu + K::FACE;                       // [2][NV][SP]
  unsigned long long* s_smax = reinterpret_cast<unsigned long long*>(s_part + 2 * NV * SP);
  double* s_alpha = reinterpret_cast<double*>(s_smax + 2 * EPB);  // [EPB] (VI_HG)

  const int tid = threadIdx.x;
  const int64_t e0 = (int64_t)blockIdx.x * EPB;
  const int nel = (int)min((int64_t)EPB, P.nelements - e0);
  const size_t gofs = (size_t)e0 * NN * NV;
  const int nval = nel * NN * NV;
  const double gamma = P.gamma, igm1 = P.inv_gamma_minus_one;

  if (A.mode == MODE_STAGE && A.clock->skip) {
    for (int k = tid; k < nval; k += NT) A.u_out[gofs + k] = A.u_in[gofs + k];
    return;
  }
  for (int k = tid; k < nval; k += NT) s_u[k] = __ldg(A.u_in + gofs + k);
  for (int k = tid; k < nel * 4 * N; k += NT) {
    const int sl = k / (4 * N);
    const int dir = (k / N) & 3;
    const int fn = k % N;
    const int32_t nb = P.nbr[(e0 + sl) * 4 + dir];
    if (nb >= e0 && nb < e0 + nel) continue;  // read from s_u below
    if (nb < 0) {
      // Dirichlet boundary face: the boundary value at this face node
      const double* x = P.xy + ((size_t)(e0 + sl) * NN + cface_own<N>(dir, fn)) * 2;
      const double tt = A.mode == MODE_STAGE ? A.clock->t + A.c * A.clock->dt : A.t_rhs;
      double xv[2] = {x[0], x[1]}, ub[NV];
      boundary_value<2>(P.bc_ic, P.bc_par, xv, tt, gamma, ub);
#pragma unroll
      for (int v = 0; v < NV; ++v) s_fu[k * NV + v] = ub[v];
      continue;
    }
    const double* g = A.u_in + ((size_t)nb * NN + cface_partner<N>(dir, fn)) * NV;
#pragma unroll
    for (int v = 0; v < NV; ++v) s_fu[k * NV + v] = __ldg(g + v);
  }
  if (tid < 2 * EPB) s_smax[tid] = 0ull;
  if (VI == VI_HG && tid < nel) {
    // apply_smoothing! as a gather (indicators_2d.jl:104-136)
    const double* raw = static_cast<const double*>(A.alpha_raw);
    const int64_t e = e0 + tid;
    double a = raw[e];
    if (P.alpha_smooth)
#pragma unroll
      for (int f = 0; f < 4; ++f) {
        const int32_t nb = P.nbr[e * 4 + f];
        if (nb >= 0) a = fmax(a, 0.5 * raw[nb]);
      }
    s_alpha[tid] = a;
    if (A.alpha_out) static_cast<double*>(A.alpha_out)[e] = a;
  }
  __syncthreads();

  // ---- lines ---------------------------------------------------------------------
  {
    const int dd = tid / (EPB * N);
    const int r = tid - dd * (EPB * N);
    const int sl = r / N;
    const int line = r - sl * N;
    if (sl < nel) {
      const int64_t e = e0 + sl;
      double uu[N][NV], ww[N][NV], ja[N][2];
#pragma unroll
      for (int a = 0; a < N; ++a) {
        const int q = cline_node<N>(line, dd, a);
#pragma unroll
        for (int v = 0; v < NV; ++v) uu[a][v] = s_u[(sl * NN + q) * NV + v];
        Eu::cons2prim(uu[a], ww[a], gamma);
        const double* m = P.met + ((size_t)e * NN + q) * 5 + 2 * dd;
        ja[a][0] = m[0];
        ja[a][1] = m[1];
      }
      double acc[N][NV];
#pragma unroll
      for (int a = 0; a < N; ++a)
#pragma unroll
        for (int v = 0; v < NV; ++v) acc[a][v] = 0.0;
      if (VI == VI_WEAK) {
#pragma unroll
        for (int a = 0; a < N; ++a) {
          double f[NV];
          FluxN::phys(uu[a], ww[a], ja[a][0], ja[a][1], f);
#pragma unroll
          for (int ii = 0; ii < N; ++ii) {
            const double c = P.Dhat[ii * N + a];
#pragma unroll
            for (int v = 0; v < NV; ++v) acc[ii][v] = fma(c, f[v], acc[ii][v]);
          }
        }
      } else {
#pragma unroll
        for (int a = 0; a < N; ++a)
#pragma unroll
          for (int b = a + 1; b < N; ++b) {
            double F[NV];
            FluxN::two_point(P.volume_flux, uu[a], ww[a], uu[b], ww[b], 0.5 * (ja[a][0] + ja[b][0]),
                             0.5 * (ja[a][1] + ja[b][1]), gamma, igm1, F);
            const double cab = P.Dsplit[a * N + b], cba = P.Dsplit[b * N + a];
#pragma unroll
            for (int v = 0; v < NV; ++v) {
              acc[a][v] = fma(cab, F[v], acc[a][v]);
              acc[b][v] = fma(cba, F[v], acc[b][v]);
            }
          }
      }
      if (VI == VI_HG) {
        // VolumeIntegralShockCapturingHG (calc_volume_integral.jl:231-272):
        // flux differencing weighted by 1 - alpha, the FV subcell fluxes of
        // the line (fv_kernel!, calcflux_fv!, dgsem_structured/dg_2d.jl:
        // 304-345) by alpha; the subcell fluxes at the element faces are zero
        const double ae = s_alpha[sl];
        if (!(fabs(ae) <= P.alpha_atol)) {
#pragma unroll
          for (int a = 0; a < N; ++a)
#pragma unroll
            for (int v = 0; v < NV; ++v) acc[a][v] *= 1.0 - ae;
          const double2* nv = P.snv + (((size_t)e * 2 + dd) * N + line) * (N - 1);
          double fl[NV] = {0.0, 0.0, 0.0, 0.0};  // subcell flux on the node's lower side
#pragma unroll
          for (int i = 0; i < N; ++i) {
            double fr[NV] = {0.0, 0.0, 0.0, 0.0};
            if (i < N - 1) {
              const double2 n = nv[i];
              FluxN::two_point(P.fv_flux, uu[i], ww[i], uu[i + 1], ww[i + 1], n.x, n.y, gamma,
                               igm1, fr);
            }
#pragma unroll
            for (int v = 0; v < NV; ++v) {
              acc[i][v] += ae * (P.inv_weights[i] * (fr[v] - fl[v]));
              fl[v] = fr[v];
            }
          }
        }
      }
      // faces -dd (node 0) and +dd (node N-1), along this element's
      // contravariant vector, negative-side element as the left state
      const double factor = P.inv_weights[0];
#pragma unroll
      for (int side = 0; side < 2; ++side) {
        const int dir = 2 * dd + side;
        const int32_t nb = P.nbr[e * 4 + dir];
        const int own = side ? N - 1 : 0;
        const double* src = (nb >= e0 && nb < e0 + nel)
                                ? s_u + (((int)(nb - e0)) * NN + cface_partner<N>(dir, line)) * NV
                                : s_fu + ((sl * 4 + dir) * N + line) * NV;
        double un[NV], wn[NV], F[NV];
#pragma unroll
        for (int v = 0; v < NV; ++v) un[v] = src[v];
        Eu::cons2prim(un, wn, gamma);
        if (side) {
          // an interface takes the contravariant vector of the element on its
          // positive side (calc_interface_flux!, dgsem_structured/dg_2d.jl:
          // 551-606), so both elements evaluate the same flux; boundary faces
          // take their own
          double n0 = ja[own][0], n1 = ja[own][1];
          if (nb >= 0) {
            const double* m = P.met + ((size_t)nb * NN + cface_partner<N>(dir, line)) * 5 + 2 * dd;
            n0 = m[0];
            n1 = m[1];
          }
          FluxN::two_point(P.surface_flux, uu[own], ww[own], un, wn, n0, n1, gamma, igm1, F);
        } else
          FluxN::two_point(P.surface_flux, un, wn, uu[own], ww[own], ja[own][0], ja[own][1], gamma,
                           igm1, F);
#pragma unroll
        for (int v = 0; v < NV; ++v)
          acc[own][v] = side ? acc[own][v] + F[v] * factor : acc[own][v] - F[v] * factor;
      }
#pragma unroll
      for (int a = 0; a < N; ++a) {
        const int q = cline_node<N>(line, dd, a);
#pragma unroll
        for (int v = 0; v < NV; ++v) s_part[(dd * NV + v) * SP + sl * NN + q] = acc[a][v];
      }
    }
  }
  __syncthreads();

  // ---- nodes -----------------------------------------------------------------------
  const bool stage = A.mode == MODE_STAGE;
  const double bdt = stage ? A.b * A.clock->dt : 0.0;
  bool bad = false;
  for (int n = tid; n < nel * NN; n += NT) {
    const int sl = n / NN;
    const int q = n - sl * NN;
    const int64_t e = e0 + sl;
    const double* m = P.met + ((size_t)e * NN + q) * 5;
    const double jfac = -m[4];
    double du[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) du[v] = (s_part[v * SP + n] + s_part[(NV + v) * SP + n]) * jfac;
    if (P.source == SRC_CONVERGENCE_TEST) {
      double x[2], s[NV];
      x[0] = P.xy[((size_t)e * NN + q) * 2];
      x[1] = P.xy[((size_t)e * NN + q) * 2 + 1];
      const double tt = stage ? A.clock->t + A.c * A.clock->dt : A.t_rhs;
      Eu::source_convergence(x, tt, gamma, s);
#pragma unroll
      for (int v = 0; v < NV; ++v) du[v] += s[v];
    }
    const size_t g = gofs + (size_t)n * NV;
    if (!stage) {
#pragma unroll
      for (int v = 0; v < NV; ++v) A.du_out[g + v] = du[v];
      continue;
    }
    double* ut = reinterpret_cast<double*>(A.u_tmp) + g;
    double un[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      const double t0 = A.zero_tmp ? 0.0 : ut[v];
      const double t1 = du[v] - t0 * A.a;
      ut[v] = t1;
      un[v] = s_u[n * NV + v] + t1 * bdt;
      A.u_out[g + v] = un[v];
      bad |= !(un[v] == un[v]);
    }
    if (A.speed_bits) {
      double w[NV];
      Eu::cons2prim(un, w, gamma);
      const double cs = sqrt(gamma * w[3] / w[0]);
      bad |= !(w[0] > 0.0) || !(w[3] > 0.0);
      const double l1 = fabs(w[1]) + cs, l2 = fabs(w[2]) + cs;
      const double ij = fabs(m[4]);
      const double s1 = fabs(m[0] * l1 + m[1] * l2) * ij;
      const double s2 = fabs(m[2] * l1 + m[3] * l2) * ij;
      if (s1 == s1) atomicMax(&s_smax[2 * sl], (unsigned long long)__double_as_longlong(s1));
      if (s2 == s2) atomicMax(&s_smax[2 * sl + 1], (unsigned long long)__double_as_longlong(s2));
    }
  }
  if (bad) atomicOr(A.status, 1);
  if (stage && A.speed_bits) {
    __syncthreads();
    if (tid < nel) {
      const double sp = __longlong_as_double((long long)s_smax[2 * tid]) +
                        __longlong_as_double((long long)s_smax[2 * tid + 1]);
      if (sp == sp) atomicMax(A.speed_bits, (unsigned long long)__double_as_longlong(sp));
    }
  }
}

}  // namespace tg


namespace tg {

__device__ __forceinline__ double cstate(double x) { return x; }
__device__ __forceinline__ double cstate(float2 x) { return (double)x.x + (double)x.y; }

// max_dt of a curvilinear mesh (stepsize_dg2d.jl:114-157), one thread per
// node (consecutive threads read consecutive nodes): FP64 for an FP64 state,
// the stage kernel's FP32 arithmetic on the hi parts for a float-float state.
// A block holds EB = 128 / NN elements; per-element maxima meet in shared
// memory (positive doubles order like their bit patterns).
template <typename TS>
__global__ void __launch_bounds__(128) curved_speed_kernel(const CurvedParams P,
                                                           const TS* __restrict__ u, int NN,
                                                           unsigned long long* __restrict__ speed_bits,
                                                           int32_t* __restrict__ status) {
  __shared__ unsigned long long s_m[2 * 128];
  constexpr bool FF = !std::is_same<TS, double>::value;
  const int EB = 128 / NN;
  const int tid = threadIdx.x;
  const int sl = tid / NN;
  const int64_t e = (int64_t)blockIdx.x * EB + sl;
  if (tid < 2 * EB) s_m[tid] = 0ull;
  __syncthreads();
  bool bad = false;
  if (sl < EB && e < P.nelements) {
    const size_t gq = (size_t)e * NN + (tid - sl * NN);
    const TS* p = u + gq * 4;
    double s1, s2;
    if constexpr (FF) {
      float hi[4], w[4];
      for (int v = 0; v < 4; ++v) hi[v] = reinterpret_cast<const float2*>(p)[v].x;
      Euler<2, float>::cons2prim(hi, w, P.eos.gamma);
      const float cs = sqrtf(P.eos.gamma * w[3] / w[0]);
      bad |= !(w[0] > 0.0f) || !(w[3] > 0.0f);
      const float l1 = fabsf(w[1]) + cs, l2 = fabsf(w[2]) + cs;
      const float4 j = P.ja32[gq];
      const float ij = fabsf(P.invj32[gq]);
      s1 = (double)(fabsf(j.x * l1 + j.y * l2) * ij);
      s2 = (double)(fabsf(j.z * l1 + j.w * l2) * ij);
    } else {
      double uu[4], w[4];
      for (int v = 0; v < 4; ++v) uu[v] = cstate(p[v]);
      Euler<2, double>::cons2prim(uu, w, P.gamma);
      const double cs = sqrt(P.gamma * w[3] / w[0]);
      bad |= !(w[0] > 0) || !(w[3] > 0);
      const double l1 = fabs(w[1]) + cs, l2 = fabs(w[2]) + cs;
      const double* m = P.met + gq * 5;
      s1 = fabs(m[0] * l1 + m[1] * l2) * fabs(m[4]);
      s2 = fabs(m[2] * l1 + m[3] * l2) * fabs(m[4]);
    }
    if (s1 == s1 && s2 == s2) {
      atomicMax(&s_m[2 * sl], (unsigned long long)__double_as_longlong(s1));
      atomicMax(&s_m[2 * sl + 1], (unsigned long long)__double_as_longlong(s2));
    } else {
      bad = true;
    }
  }
  __syncthreads();
  if (tid < EB && (int64_t)blockIdx.x * EB + tid < P.nelements) {
    const double sp = __longlong_as_double((long long)s_m[2 * tid]) +
                      __longlong_as_double((long long)s_m[2 * tid + 1]);
    atomicMax(speed_bits, (unsigned long long)__double_as_longlong(sp));
  }
  if (bad) atomicOr(status, 2);
}

// Per-element FP64 integrals with the per-node Jacobian |J| = 1/|invJ|
// (integrate_via_indices, analysis_dg2d.jl:313-336): conserved totals,
// mathematical entropy and kinetic energy, as element_integrals_kernel.
template <typename TS>
__global__ void curved_integrals_kernel(const CurvedParams P, const TS* __restrict__ u,
                                        const double* __restrict__ weights, int N,
                                        double* __restrict__ partial) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= P.nelements) return;
  const int NN = N * N;
  const double g = P.gamma;
  double acc[6] = {0, 0, 0, 0, 0, 0};
  for (int q = 0; q < NN; ++q) {
    const size_t gq = (size_t)e * NN + q;
    const double w = weights[q % N] * weights[q / N] / fabs(P.met[gq * 5 + 4]);
    double p[4];
    for (int v = 0; v < 4; ++v) p[v] = cstate(u[gq * 4 + v]);
    const double m2 = p[1] * p[1] + p[2] * p[2];
    for (int v = 0; v < 4; ++v) acc[v] += w * p[v];
    const double pr = (g - 1) * (p[3] - 0.5 * m2 / p[0]);
    const double s = log(pr) - g * log(p[0]);
    acc[4] += w * (-s * p[0] / (g - 1));
    acc[5] += w * (m2 / (2 * p[0]));
  }
  for (int k = 0; k < 6; ++k) partial[(size_t)e * 6 + k] = acc[k];
}

template <int N, int VI>
static int launch_curved_n(const CurvedParams& P, const StageArgs* A64, const MixedArgs* A32,
                           cudaStream_t stream) {
  constexpr int EPB = N == 5 ? 8 : 16;
  using K = CurvedK<N, EPB>;
  const unsigned nb = (unsigned)((P.nelements + EPB - 1) / EPB);
  if (A64) {
    const size_t smem = sizeof(double) * (K::CHUNK + K::FACE + 2 * 4 * K::SP) +
                        sizeof(unsigned long long) * 2 * EPB + sizeof(double) * EPB;
    static bool attr = false;
    if (!attr) {
      cudaFuncSetAttribute(curved_kernel_f64<N, VI, EPB>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      attr = true;
    }
    curved_kernel_f64<N, VI, EPB><<<nb, K::NT, smem, stream>>>(P, *A64);
  } else {
    return launch_curved_mixed2(P, *A32, stream);
  }
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int launch_curved(const CurvedParams& P, const StageArgs* A64, const MixedArgs* A32,
                  cudaStream_t stream) {
  if ((A64 == nullptr) == (A32 == nullptr)) return -2;
  switch (P.vi) {
    case VI_WEAK:
      switch (P.N) {
        case 3: return launch_curved_n<3, VI_WEAK>(P, A64, A32, stream);
        case 4: return launch_curved_n<4, VI_WEAK>(P, A64, A32, stream);
        case 5: return launch_curved_n<5, VI_WEAK>(P, A64, A32, stream);
      }
      break;
    case VI_FD:
      switch (P.N) {
        case 3: return launch_curved_n<3, VI_FD>(P, A64, A32, stream);
        case 4: return launch_curved_n<4, VI_FD>(P, A64, A32, stream);
        case 5: return launch_curved_n<5, VI_FD>(P, A64, A32, stream);
      }
      break;
    case VI_HG:
      switch (P.N) {
        case 3: return launch_curved_n<3, VI_HG>(P, A64, A32, stream);
        case 4: return launch_curved_n<4, VI_HG>(P, A64, A32, stream);
        case 5: return launch_curved_n<5, VI_HG>(P, A64, A32, stream);
      }
      break;
  }
  return -3;
}

__global__ void curved_ghost_kernel(const CurvedParams P, int64_t B, const Clock* clock, double c_s,
                                    double t_rhs, int mode, float2* __restrict__ ghost) {
  const int N = P.N, NN = N * N;
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= B * N) return;
  const int64_t b = k / N;
  const int fn = (int)(k - b * N);
  const int64_t e = P.bface[2 * b];
  const int dir = P.bface[2 * b + 1];
  int node;
  switch (dir) {
    case 0: node = N * fn; break;
    case 1: node = (N - 1) + N * fn; break;
    case 2: node = fn; break;
    default: node = fn + N * (N - 1); break;
  }
  const double* x = P.xy + ((size_t)e * NN + node) * 2;
  double xv[2] = {x[0], x[1]}, out[4];
  const double t = mode == MODE_RHS ? t_rhs : clock->t + c_s * clock->dt;
  boundary_value<2>(P.bc_ic, P.bc_par, xv, t, P.gamma, out);
  for (int v = 0; v < 4; ++v) {
    const float hi = (float)out[v];
    ghost[k * 4 + v] = make_float2(hi, (float)(out[v] - (double)hi));
  }
}

int launch_curved_ghost(const CurvedParams& P, int64_t B, const Clock* clock, double c_s,
                        double t_rhs, int mode, float2* ghost, cudaStream_t stream) {
  const int64_t nk = B * P.N;
  curved_ghost_kernel<<<(unsigned)((nk + 127) / 128), 128, 0, stream>>>(P, B, clock, c_s, t_rhs,
                                                                      mode, ghost);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int launch_curved_speed(const CurvedParams& P, const void* u, bool ff, unsigned long long* dst,
                        int32_t* status, cudaStream_t stream) {
  const int eb = 128 / (P.N * P.N);  // elements per block (N <= 5: at least 5)
  const unsigned nb = (unsigned)((P.nelements + eb - 1) / eb);
  if (ff)
    curved_speed_kernel<float2><<<nb, 128, 0, stream>>>(P, (const float2*)u, P.N * P.N, dst, status);
  else
    curved_speed_kernel<double><<<nb, 128, 0, stream>>>(P, (const double*)u, P.N * P.N, dst, status);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int launch_curved_integrals(const CurvedParams& P, const void* u, bool ff, const double* weights,
                            double* partial, cudaStream_t stream) {
  const unsigned nb = (unsigned)((P.nelements + 127) / 128);
  if (ff)
    curved_integrals_kernel<float2><<<nb, 128, 0, stream>>>(P, (const float2*)u, weights, P.N,
                                                            partial);
  else
    curved_integrals_kernel<double><<<nb, 128, 0, stream>>>(P, (const double*)u, weights, P.N,
                                                            partial);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace tg
