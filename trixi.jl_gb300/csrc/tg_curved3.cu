// Curvilinear 3D stage kernels (StructuredMesh{3}), FP64 and mixed precision
// (weak form and flux differencing, polydeg 3 and 5).
//
// The 3D form of the FP64 kernel of tg_curved.cu: volume integrals with
// contravariant fluxes along the three reference directions
// (dgsem_structured/dg_3d.jl: weak_form_kernel!, flux_differencing_kernel!),
// interface fluxes along the contravariant vector of the element face, with
// the element on the negative side as the left state, Dirichlet faces
// (calc_boundary_flux!, dg_3d.jl; BoundaryConditionDirichlet,
// equations.jl:183-211), the surface integral, apply_jacobian! with the
// per-node inverse Jacobian, sources at the node coordinates, and the
// curvilinear CFL reduction (stepsize_dg3d.jl).  The metric terms come from
// the caller (Trixi's contravariant_vectors, invariant curl form,
// containers_3d.jl:125-246).
//
// One block holds EPB elements; one thread owns one (direction, line) of an
// element (3 N^2 lines), evaluates its N(N-1)/2 two-point fluxes (or the N
// weak-form fluxes) and its two face fluxes, and accumulates the line's node
// contributions in registers; a node phase sums the three directions.
#include <cuda_runtime.h>

#include "tg_curved.cuh"

namespace tg {

namespace {

// FP64 fluxes along a normal direction, compressible_euler_3d.jl
// (normal-direction methods of flux, flux_ranocha, flux_shima_etal,
// flux_chandrashekar, max_abs_speed(_naive))
struct FluxN3 {
  static __device__ __forceinline__ void phys(const double* u, const double* w, const double* n,
                                              double* f) {
    const double vn = w[1] * n[0] + w[2] * n[1] + w[3] * n[2];
    const double rvn = w[0] * vn;
    f[0] = rvn;
#pragma unroll
    for (int d = 0; d < 3; ++d) f[1 + d] = fma(rvn, w[1 + d], w[4] * n[d]);
    f[4] = (u[4] + w[4]) * vn;
  }

  static __device__ __forceinline__ void two_point(int k, const double* ua, const double* a,
                                                   const double* ub, const double* b,
                                                   const double* n, double gamma, double igm1,
                                                   double* f) {
    const double vna = a[1] * n[0] + a[2] * n[1] + a[3] * n[2];
    const double vnb = b[1] * n[0] + b[2] * n[1] + b[3] * n[2];
    double vavg[3], vsq = 0;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      vavg[d] = 0.5 * (a[1 + d] + b[1 + d]);
      vsq += a[1 + d] * b[1 + d];
    }
    vsq *= 0.5;
    const double p_avg = 0.5 * (a[4] + b[4]);
    if (k == FLUX_RANOCHA) {
      const double rho_mean = ln_mean(a[0], b[0]);
      const double irpm = a[4] * b[4] * inv_ln_mean(a[0] * b[4], b[0] * a[4]);
      const double f1 = rho_mean * 0.5 * (vna + vnb);
      f[0] = f1;
#pragma unroll
      for (int d = 0; d < 3; ++d) f[1 + d] = fma(f1, vavg[d], p_avg * n[d]);
      f[4] = f1 * (vsq + irpm * igm1) + 0.5 * (a[4] * vnb + b[4] * vna);
      return;
    }
    if (k == FLUX_SHIMA_ETAL) {
      const double rho_avg = 0.5 * (a[0] + b[0]);
      const double vn_avg = 0.5 * (vna + vnb);
      const double f1 = rho_avg * vn_avg;
      f[0] = f1;
#pragma unroll
      for (int d = 0; d < 3; ++d) f[1 + d] = fma(f1, vavg[d], p_avg * n[d]);
      f[4] = f1 * vsq + p_avg * vn_avg * igm1 + 0.5 * (a[4] * vnb + b[4] * vna);
      return;
    }
    if (k == FLUX_CHANDRASHEKAR) {
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
#pragma unroll
      for (int d = 0; d < 3; ++d) f[1 + d] = fma(f1, vavg[d], p_mean * n[d]);
      f[4] = f1 * 0.5 * (1 / (gamma - 1) / beta_mean - (kin_a + kin_b)) + f[1] * vavg[0] +
             f[2] * vavg[1] + f[3] * vavg[2];
      return;
    }
    double fa[5], fb[5];
    phys(ua, a, n, fa);
    phys(ub, b, n, fb);
#pragma unroll
    for (int v = 0; v < 5; ++v) f[v] = 0.5 * (fa[v] + fb[v]);
    if (k == FLUX_LLF || k == FLUX_LLF_NAIVE) {
      const double ca = sqrt(gamma * a[4] / a[0]), cb = sqrt(gamma * b[4] / b[0]);
      const double nn = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
      const double lam = k == FLUX_LLF_NAIVE ? fmax(fabs(vna), fabs(vnb)) + fmax(ca, cb) * nn
                                             : fmax(fabs(vna) + ca * nn, fabs(vnb) + cb * nn);
#pragma unroll
      for (int v = 0; v < 5; ++v) f[v] = f[v] + (-0.5 * lam * (ub[v] - ua[v]));
    }
  }
};

template <int N, int EPB>
struct Curved3K {
  static constexpr int NF = N * N, NN = N * N * N, NV = 5, NT = EPB * 3 * NF;
  static constexpr int CHUNK = EPB * NN * NV;
  static constexpr int FACE = EPB * 6 * NF * NV;
  static constexpr int SP = EPB * NN;
  static constexpr size_t smem() {
    return sizeof(double) * (CHUNK + FACE + 3 * NV * SP) + sizeof(unsigned long long) * 3 * EPB +
           sizeof(double) * EPB;  // blending factors (VI_HG)
  }
};

}  // namespace

}  // namespace tg

namespace tg {

namespace {

// met: [E][NN][10] = Ja^d_c at d * 3 + c, then the inverse Jacobian
template <int N, int VI, int EPB>
__global__ void __launch_bounds__(Curved3K<N, EPB>::NT)
    curved3_kernel_f64(const CurvedParams P, const StageArgs A) {
  using K = Curved3K<N, EPB>;
  using Eu = Euler<3, double>;
  constexpr int NN = K::NN, NF = K::NF, NV = 5, NT = K::NT, SP = K::SP, CHUNK = K::CHUNK;
  constexpr int MS = 10;  // metric values per node
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double* s_u = reinterpret_cast<double*>(smem_raw);
  double* s_fu = s_u + CHUNK;                 // [EPB][6][NF][NV] neighbour / boundary traces
  double* s_part = s_fu + K::FACE;            // [3][NV][SP]
  unsigned long long* s_smax = reinterpret_cast<unsigned long long*>(s_part + 3 * NV * SP);
  double* s_alpha = reinterpret_cast<double*>(s_smax + 3 * EPB);  // [EPB] (VI_HG)

  const int tid = threadIdx.x;
  const int64_t e0 = (int64_t)blockIdx.x * EPB;
  const int nel = (int)min((int64_t)EPB, P.nelements - e0);
  const size_t gofs = (size_t)e0 * NN * NV;
  const int nval = nel * NN * NV;
  const double gamma = P.gamma, igm1 = P.inv_gamma_minus_one;
  const bool stage = A.mode == MODE_STAGE;

  if (stage && A.clock->skip) {
    for (int k = tid; k < nval; k += NT) A.u_out[gofs + k] = A.u_in[gofs + k];
    return;
  }
  for (int k = tid; k < nval; k += NT) s_u[k] = __ldg(A.u_in + gofs + k);
  for (int k = tid; k < nel * 6 * NF; k += NT) {
    const int sl = k / (6 * NF);
    const int rem = k - sl * (6 * NF);
    const int dir = rem / NF;
    const int fn = rem - dir * NF;
    const int32_t nb = P.nbr[(e0 + sl) * 6 + dir];
    if (nb >= e0 && nb < e0 + nel) continue;  // read from s_u below
    if (nb < 0) {
      const double* x = P.xy + ((size_t)(e0 + sl) * NN + face_own3<N>(dir, fn)) * 3;
      const double tt = stage ? A.clock->t + A.c * A.clock->dt : A.t_rhs;
      double xv[3] = {x[0], x[1], x[2]}, ub[NV];
      boundary_value<3>(P.bc_ic, P.bc_par, xv, tt, gamma, ub);
#pragma unroll
      for (int v = 0; v < NV; ++v) s_fu[k * NV + v] = ub[v];
      continue;
    }
    const double* g = A.u_in + ((size_t)nb * NN + face_partner3<N>(dir, fn)) * NV;
#pragma unroll
    for (int v = 0; v < NV; ++v) s_fu[k * NV + v] = __ldg(g + v);
  }
  if (tid < 3 * EPB) s_smax[tid] = 0ull;
  if (VI == VI_HG && tid < nel) {
    // apply_smoothing! as a gather over the face neighbours
    const double* raw = static_cast<const double*>(A.alpha_raw);
    const int64_t e = e0 + tid;
    double a = raw[e];
    if (P.alpha_smooth)
#pragma unroll
      for (int f = 0; f < 6; ++f) {
        const int32_t nb = P.nbr[e * 6 + f];
        if (nb >= 0) a = fmax(a, 0.5 * raw[nb]);
      }
    s_alpha[tid] = a;
    if (A.alpha_out) static_cast<double*>(A.alpha_out)[e] = a;
  }
  __syncthreads();

  // ---- lines ---------------------------------------------------------------------
  {
    const int dd = tid / (EPB * NF);
    const int r = tid - dd * (EPB * NF);
    const int sl = r / NF;
    const int line = r - sl * NF;
    if (sl < nel) {
      const int64_t e = e0 + sl;
      double uu[N][NV], ww[N][NV], ja[N][3];
#pragma unroll
      for (int a = 0; a < N; ++a) {
        const int q = line3<N>(line, dd, a);
#pragma unroll
        for (int v = 0; v < NV; ++v) uu[a][v] = s_u[(sl * NN + q) * NV + v];
        Eu::cons2prim(uu[a], ww[a], gamma);
        const double* m = P.met + ((size_t)e * NN + q) * MS + 3 * dd;
        ja[a][0] = m[0];
        ja[a][1] = m[1];
        ja[a][2] = m[2];
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
          FluxN3::phys(uu[a], ww[a], ja[a], f);
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
            const double avg[3] = {0.5 * (ja[a][0] + ja[b][0]), 0.5 * (ja[a][1] + ja[b][1]),
                                   0.5 * (ja[a][2] + ja[b][2])};
            double F[NV];
            FluxN3::two_point(P.volume_flux, uu[a], ww[a], uu[b], ww[b], avg, gamma, igm1, F);
            const double cab = P.Dsplit[a * N + b], cba = P.Dsplit[b * N + a];
#pragma unroll
            for (int v = 0; v < NV; ++v) {
              acc[a][v] = fma(cab, F[v], acc[a][v]);
              acc[b][v] = fma(cba, F[v], acc[b][v]);
            }
          }
      }
      if (VI == VI_HG) {
        // (1 - alpha) flux differencing + alpha FV subcell fluxes along the
        // subcell normals, zero at the element faces (calcflux_fv!,
        // dgsem_structured/dg_3d.jl; calc_volume_integral.jl:231-272)
        const double ae = s_alpha[sl];
        if (!(fabs(ae) <= P.alpha_atol)) {
#pragma unroll
          for (int a = 0; a < N; ++a)
#pragma unroll
            for (int v = 0; v < NV; ++v) acc[a][v] *= 1.0 - ae;
          const double* nv = P.snv3 + ((((size_t)e * 3 + dd) * NF + line) * (N - 1)) * 3;
          double fl[NV] = {0.0, 0.0, 0.0, 0.0, 0.0};
#pragma unroll
          for (int i = 0; i < N; ++i) {
            double fr[NV] = {0.0, 0.0, 0.0, 0.0, 0.0};
            if (i < N - 1) {
              const double n3[3] = {nv[3 * i], nv[3 * i + 1], nv[3 * i + 2]};
              FluxN3::two_point(P.fv_flux, uu[i], ww[i], uu[i + 1], ww[i + 1], n3, gamma, igm1, fr);
            }
#pragma unroll
            for (int v = 0; v < NV; ++v) {
              acc[i][v] += ae * (P.inv_weights[i] * (fr[v] - fl[v]));
              fl[v] = fr[v];
            }
          }
        }
      }
      const double factor = P.inv_weights[0];
#pragma unroll
      for (int side = 0; side < 2; ++side) {
        const int dir = 2 * dd + side;
        const int32_t nb = P.nbr[e * 6 + dir];
        const int own = side ? N - 1 : 0;
        const double* src = (nb >= e0 && nb < e0 + nel)
                                ? s_u + (((int)(nb - e0)) * NN + face_partner3<N>(dir, line)) * NV
                                : s_fu + ((sl * 6 + dir) * NF + line) * NV;
        double un[NV], wn[NV], F[NV];
#pragma unroll
        for (int v = 0; v < NV; ++v) un[v] = src[v];
        Eu::cons2prim(un, wn, gamma);
        if (side) {
          // an interface takes the contravariant vector of the element on its
          // positive side (calc_interface_flux!, dgsem_structured/dg_3d.jl), so
          // both elements evaluate the same flux; boundary faces take their own
          double nrm[3] = {ja[own][0], ja[own][1], ja[own][2]};
          if (nb >= 0) {
            const double* m = P.met + ((size_t)nb * NN + face_partner3<N>(dir, line)) * MS + 3 * dd;
            nrm[0] = m[0];
            nrm[1] = m[1];
            nrm[2] = m[2];
          }
          FluxN3::two_point(P.surface_flux, uu[own], ww[own], un, wn, nrm, gamma, igm1, F);
        } else
          FluxN3::two_point(P.surface_flux, un, wn, uu[own], ww[own], ja[own], gamma, igm1, F);
#pragma unroll
        for (int v = 0; v < NV; ++v)
          acc[own][v] = side ? acc[own][v] + F[v] * factor : acc[own][v] - F[v] * factor;
      }
#pragma unroll
      for (int a = 0; a < N; ++a) {
        const int q = line3<N>(line, dd, a);
#pragma unroll
        for (int v = 0; v < NV; ++v) s_part[(dd * NV + v) * SP + sl * NN + q] = acc[a][v];
      }
    }
  }
  __syncthreads();

  // ---- nodes -----------------------------------------------------------------------
  const double bdt = stage ? A.b * A.clock->dt : 0.0;
  bool bad = false;
  for (int n = tid; n < nel * NN; n += NT) {
    const int sl = n / NN;
    const int q = n - sl * NN;
    const int64_t e = e0 + sl;
    const double* m = P.met + ((size_t)e * NN + q) * MS;
    const double jfac = -m[9];
    double du[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v)
      du[v] = (s_part[v * SP + n] + s_part[(NV + v) * SP + n] + s_part[(2 * NV + v) * SP + n]) *
              jfac;
    if (P.source == SRC_CONVERGENCE_TEST) {
      const double* xp = P.xy + ((size_t)e * NN + q) * 3;
      double x[3] = {xp[0], xp[1], xp[2]}, s[NV];
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
      const double cs = sqrt(gamma * w[4] / w[0]);
      bad |= !(w[0] > 0.0) || !(w[4] > 0.0);
      const double l[3] = {fabs(w[1]) + cs, fabs(w[2]) + cs, fabs(w[3]) + cs};
      const double ij = fabs(m[9]);
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const double sd = fabs(m[3 * d] * l[0] + m[3 * d + 1] * l[1] + m[3 * d + 2] * l[2]) * ij;
        if (sd == sd) atomicMax(&s_smax[3 * sl + d], (unsigned long long)__double_as_longlong(sd));
      }
    }
  }
  if (bad) atomicOr(A.status, 1);
  if (stage && A.speed_bits) {
    __syncthreads();
    if (tid < nel) {
      const double sp = __longlong_as_double((long long)s_smax[3 * tid]) +
                        __longlong_as_double((long long)s_smax[3 * tid + 1]) +
                        __longlong_as_double((long long)s_smax[3 * tid + 2]);
      if (sp == sp) atomicMax(A.speed_bits, (unsigned long long)__double_as_longlong(sp));
    }
  }
}


}  // namespace

}  // namespace tg

namespace tg {

namespace {

__device__ __forceinline__ double state3(double x) { return x; }
__device__ __forceinline__ double state3(float2 x) { return (double)x.x + (double)x.y; }

// curvilinear max_dt (stepsize_dg3d.jl), one warp per element, in FP64 on an
// FP64 or a float-float state
template <typename TS>
__global__ void __launch_bounds__(128) curved3_speed_kernel(const CurvedParams P,
                                                            const TS* __restrict__ u, int NN,
                                                            unsigned long long* __restrict__ speed_bits,
                                                            int32_t* __restrict__ status) {
  const int lane = threadIdx.x & 31;
  const int64_t e = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (e >= P.nelements) return;
  double m[3] = {0, 0, 0};
  bool bad = false;
  for (int q = lane; q < NN; q += 32) {
    const size_t gq = (size_t)e * NN + q;
    double uu[5], w[5];
    for (int v = 0; v < 5; ++v) uu[v] = state3(u[gq * 5 + v]);
    Euler<3, double>::cons2prim(uu, w, P.gamma);
    const double cs = sqrt(P.gamma * w[4] / w[0]);
    bad |= !(w[0] > 0) || !(w[4] > 0);
    const double l[3] = {fabs(w[1]) + cs, fabs(w[2]) + cs, fabs(w[3]) + cs};
    const double* mt = P.met + gq * 10;
    for (int d = 0; d < 3; ++d)
      m[d] = fmax(m[d], fabs(mt[3 * d] * l[0] + mt[3 * d + 1] * l[1] + mt[3 * d + 2] * l[2]) *
                            fabs(mt[9]));
  }
  for (int d = 0; d < 3; ++d)
    for (int o = 16; o > 0; o >>= 1) m[d] = fmax(m[d], __shfl_xor_sync(0xffffffffu, m[d], o));
  if (lane == 0) {
    const double sp = m[0] + m[1] + m[2];
    if (sp == sp)
      atomicMax(speed_bits, (unsigned long long)__double_as_longlong(sp));
    else
      bad = true;
  }
  if (bad) atomicOr(status, 2);
}

// per-element FP64 integrals with |J| per node, as element_integrals_kernel
template <typename TS>
__global__ void curved3_integrals_kernel(const CurvedParams P, const TS* __restrict__ u,
                                         const double* __restrict__ weights, int N,
                                         double* __restrict__ partial) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= P.nelements) return;
  const int NN = N * N * N;
  const double g = P.gamma;
  double acc[7] = {0, 0, 0, 0, 0, 0, 0};
  for (int q = 0; q < NN; ++q) {
    const size_t gq = (size_t)e * NN + q;
    const double w = weights[q % N] * weights[(q / N) % N] * weights[q / (N * N)] /
                     fabs(P.met[gq * 10 + 9]);
    double p[5];
    for (int v = 0; v < 5; ++v) p[v] = state3(u[gq * 5 + v]);
    const double m2 = p[1] * p[1] + p[2] * p[2] + p[3] * p[3];
    for (int v = 0; v < 5; ++v) acc[v] += w * p[v];
    const double pr = (g - 1) * (p[4] - 0.5 * m2 / p[0]);
    const double s = log(pr) - g * log(p[0]);
    acc[5] += w * (-s * p[0] / (g - 1));
    acc[6] += w * (m2 / (2 * p[0]));
  }
  for (int k = 0; k < 7; ++k) partial[(size_t)e * 7 + k] = acc[k];
}

template <int N, int VI>
int launch_curved3_n(const CurvedParams& P, const StageArgs* A64, const MixedArgs* A32,
                     cudaStream_t stream) {
  if (A64) {
    constexpr int EPB = N == 3 ? 4 : (N == 4 ? 2 : 1);
    const unsigned nb = (unsigned)((P.nelements + EPB - 1) / EPB);
    using K = Curved3K<N, EPB>;
    static_assert(K::smem() <= 48 * 1024, "curvilinear 3D block exceeds 48 KB of shared memory");
    curved3_kernel_f64<N, VI, EPB><<<nb, K::NT, K::smem(), stream>>>(P, *A64);
  } else {
    return launch_curved_mixed3(P, *A32, stream);
  }
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace

// Built for polydeg 3 and 5 (N = 4, 6: the degrees of Trixi's StructuredMesh3D
// Euler elixirs), each with the weak form and flux differencing, and shock
// capturing at polydeg 3; FP64 and mixed precision.
int curved3_supported(int N) { return N == 4 || N == 6; }

int launch_curved3(const CurvedParams& P, const StageArgs* A64, const MixedArgs* A32,
                   cudaStream_t stream) {
  if ((A64 == nullptr) == (A32 == nullptr)) return -2;
  if (P.vi == VI_HG) return P.N == 4 ? launch_curved3_n<4, VI_HG>(P, A64, A32, stream) : -3;
  const bool fd = P.vi == VI_FD;
  if (!fd && P.vi != VI_WEAK) return -3;
  if (P.N == 4) return fd ? launch_curved3_n<4, VI_FD>(P, A64, A32, stream)
                          : launch_curved3_n<4, VI_WEAK>(P, A64, A32, stream);
  if (P.N == 6) return fd ? launch_curved3_n<6, VI_FD>(P, A64, A32, stream)
                          : launch_curved3_n<6, VI_WEAK>(P, A64, A32, stream);
  return -3;
}

int launch_curved3_speed(const CurvedParams& P, const void* u, bool ff, unsigned long long* dst,
                         int32_t* status, cudaStream_t stream) {
  const unsigned nb = (unsigned)((P.nelements + 3) / 4);  // one warp per element
  const int NN = P.N * P.N * P.N;
  if (ff)
    curved3_speed_kernel<float2><<<nb, 128, 0, stream>>>(P, (const float2*)u, NN, dst, status);
  else
    curved3_speed_kernel<double><<<nb, 128, 0, stream>>>(P, (const double*)u, NN, dst, status);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int launch_curved3_integrals(const CurvedParams& P, const void* u, bool ff, const double* weights,
                             double* partial, cudaStream_t stream) {
  const unsigned nb = (unsigned)((P.nelements + 127) / 128);
  if (ff)
    curved3_integrals_kernel<float2><<<nb, 128, 0, stream>>>(P, (const float2*)u, weights, P.N,
                                                             partial);
  else
    curved3_integrals_kernel<double><<<nb, 128, 0, stream>>>(P, (const double*)u, weights, P.N,
                                                             partial);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace tg
