// Fused DGSEM element kernels for sm_103a.
//
// One CUDA block owns EPB consecutive elements (Trixi's depth-first leaf
// order, so a block holds a compact brick of the mesh); one thread owns one
// LGL node.  A launch evaluates, per element,
//
//   volume integral      weak form      dg_2d.jl:195-221 / dg_3d.jl:133-164
//                        flux diff.     dg_2d.jl:223-259 / dg_3d.jl:166-214
//                        HG blending    calc_volume_integral.jl:231-272,
//                                       fv_kernel! dg_2d.jl:407-464 / dg_3d.jl:268-390
//   interface fluxes     prolong2interfaces! + calc_interface_flux!
//                                       dg_2d.jl:515-541, 600-632 / dg_3d.jl:530-650
//   surface integral     calc_surface_integral! dg_2d.jl:1245-1287 / dg_3d.jl:1337-1394
//   Jacobian             apply_jacobian!        dg_2d.jl:1345-1363 / dg_3d.jl:1396-1414
//   sources              calc_sources!          dg_2d.jl:1366-1386 / dg_3d.jl:1422-1438
//
// and then either writes du (rhs mode, the rhs_hyperbolic! contract) or
// applies the 2N Runge-Kutta stage update methods_2N.jl:153-157 in place
// (stage mode), so that du never reaches HBM.  Stage mode can also reduce the
// CFL wave speed of the new state (stepsize_dg{2,3}d.jl) for the next step.
//
// Each interface flux is evaluated by both adjacent elements with the same
// (left, right) operand order and the same instruction sequence, so the two
// copies are bitwise equal and the scheme stays conservative to round-off.
// Neighbour traces are read straight from the FP64 state (from shared memory
// when the neighbour lives in the same block, else through the read-only
// path, where they are usually L2 hits): no interface arrays exist in HBM.
//
// Shared memory per block holds the FP64 state chunk (staged with coalesced
// loads, reused for the coalesced write-back), the primitive and conservative
// variables in padded SoA form, the face fluxes and the two-point fluxes of
// the volume integral; each symmetric two-point flux is evaluated once per
// node pair (half the pairs of a naive sweep), with pairs dealt out
// round-robin over the nodes of a line.
#pragma once

#include "tg_physics.cuh"

namespace tg {

constexpr int MAXN = 8;

struct DgParams {
  int64_t nelements;
  double gamma, inv_gamma_minus_one;
  double nodes[MAXN];
  double inv_weights[MAXN];
  // n x n matrices packed row-major with the actual n: M[a * n + b] = M[a, b]
  double Dhat[MAXN * MAXN];
  double Dsplit[MAXN * MAXN];
  double Vinv[MAXN * MAXN];  // inverse Legendre Vandermonde
  int32_t volume_flux, surface_flux, fv_flux, source;
  double alpha_max, alpha_min, alpha_atol, hg_threshold, hg_parameter_s;
  int32_t alpha_smooth;
  int32_t hg_variable;    // indicator variable: 0 density_pressure, 1 density
  // [E][2D] neighbour across face (-x,+x,-y,+y,-z,+z); a face without a
  // conforming neighbour has nbr = -1 - b: b < nbc a boundary face, else
  // mortar face slot b - nbc
  const int32_t* nbr;
  const double* inv_jac;  // [E]
  const double* xline;    // [E][D][N] node coordinates along each axis, or null
  // boundary conditions of the faces with nbr < 0 (non-periodic meshes)
  int32_t bc[6];          // per direction, BoundaryKind
  int32_t bc_ic;          // Dirichlet values: InitialConditionKind
  double bc_par[4];       // and its free constants
  // L2 mortars: fluxes of the mortar faces from the mortar pre-pass
  int32_t nbc;            // boundary faces (nbr = -1 - b with b < nbc)
  const double* mflux;    // [mortar face slot][NF][NV]
  const int32_t* mnbr;    // [mortar face slot][4]: elements across it (-1: none)
};

// max(a, 0.5 raw[n]) over the elements n across face `dir` of e: the
// conforming neighbour, or the elements on the other side of a mortar
// (apply_smoothing!, indicators_2d.jl:104-136, indicators_3d.jl:125-166).
template <typename R>
__device__ __forceinline__ R smooth_over_face(R a, int32_t nb, const R* raw, int32_t nbc,
                                              const int32_t* mnbr) {
  if (nb >= 0) return fmax(a, R(0.5) * raw[nb]);
  const int32_t b = -1 - nb - nbc;
  if (b < 0) return a;  // domain boundary
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int32_t m = mnbr[4 * b + q];
    if (m >= 0) a = fmax(a, R(0.5) * raw[m]);
  }
  return a;
}

// Device-resident clock of the time loop (one per context).
struct Clock {
  double t, dt, t_end, cfl;
  unsigned long long speed_bits;  // max scaled wave speed of the state (as bits)
  int32_t skip, finalstep, finished, nan_dt;
  int64_t steps;
  float sin_t[5], cos_t[5];       // sin/cos(pi (t + c_s dt)) of the 2N stages
  float sin_tl[5], cos_tl[5];     // their low parts (float-float)
};

enum StageMode { MODE_RHS = 0, MODE_STAGE = 1 };

struct StageArgs {
  const double* u_in;
  double* u_out;             // MODE_STAGE: new state (must not alias u_in)
  double* du_out;            // MODE_RHS: du
  void* u_tmp;               // MODE_STAGE: 2N register (RT)
  const void* alpha_raw;     // VI_HG: unsmoothed indicator of u_in (R)
  void* alpha_out;           // VI_HG (optional): smoothed blending factor (R)
  const Clock* clock;        // MODE_STAGE: t, dt, skip
  unsigned long long* speed_bits;  // MODE_STAGE (optional): CFL reduction of u_out
  int32_t* status;           // sticky status word
  double t_rhs;              // MODE_RHS time
  double a, b, c;            // 2N coefficients of the stage
  int32_t mode;
  int32_t zero_tmp;          // MODE_STAGE: treat u_tmp as zero (first stage)
};

template <int B, int E>
struct Pow {
  static constexpr int value = B * Pow<B, E - 1>::value;
};
template <int B>
struct Pow<B, 0> {
  static constexpr int value = 1;
};

__host__ __device__ constexpr int ipow(int b, int e) { return e == 0 ? 1 : b * ipow(b, e - 1); }

// Stride of axis d in the node numbering n = i0 + N i1 + N^2 i2.
template <int N>
__device__ __forceinline__ int axis_stride(int d) {
  return d == 0 ? 1 : (d == 1 ? N : N * N);
}
// Index of `node` along axis d.
template <int N>
__device__ __forceinline__ int axis_index(int node, int d) {
  return (node / axis_stride<N>(d)) % N;
}
// Face-node / line index of `node` with axis d removed (Trixi's surface index order).
template <int N>
__device__ __forceinline__ int line_index(int node, int d) {
  const int S = axis_stride<N>(d);
  return (node % S) + (node / (S * N)) * S;
}
// First node (index 0 along d) of line `line` of axis d.
template <int N>
__device__ __forceinline__ int line_base(int line, int d) {
  const int S = axis_stride<N>(d);
  return (line % S) + (line / S) * S * N;
}
// Index of the node pair (a, b), a < b, in the list (0,1),(0,2),..,(0,N-1),(1,2),..
template <int N>
__device__ __forceinline__ int pair_index(int a, int b) {
  return a * N - (a * (a + 1)) / 2 + (b - a - 1);
}

template <int D, int N, typename R, typename RT, int VI, int EPB>
struct ElementKernel {
  static constexpr int NV = D + 2;
  static constexpr int NN = Pow<N, D>::value;
  static constexpr int NF = NN / N;
  static constexpr int NT = EPB * NN;
  static constexpr int SP = EPB * NN + 1;  // padded SoA stride (odd)
  static constexpr int NP = N * (N - 1) / 2;
  static constexpr int CHUNK = EPB * NN * NV;
  static constexpr int VOL_WEAK = D * NV * SP;
  static constexpr int VOL_FD = EPB * D * NF * NP * NV;
  static constexpr int VOL_FV = EPB * D * NF * (N - 1) * NV;
  static constexpr int VOL = VI == VI_WEAK ? VOL_WEAK : (VI == VI_FD ? VOL_FD : VOL_FD + VOL_FV);

  static constexpr size_t smem_bytes() {
    return sizeof(double) * CHUNK                          // s_u
           + sizeof(RT) * CHUNK                            // s_tmp
           + sizeof(R) * (2 * NV * SP                      // s_w, s_c
                          + EPB * 2 * D * NF * NV          // s_face
                          + VOL                            // volume buffers
                          + N * N + N + N * N              // s_mat, s_iw, s_mat2
                          + EPB + 8);                      // s_alpha (+ pad)
  }
};

// Flux through face node `node` of element e on a face without neighbour
// (prolong2boundaries! + calc_boundary_flux!, dg_2d.jl:680-717, 795-860):
// BoundaryConditionDirichlet with the initial condition's values at the node
// and the stage time (u_inner left of + faces), or boundary_condition_slip_wall.
template <int D, int N, typename R>
__device__ inline void boundary_face_flux(const DgParams& P, const StageArgs& A, int64_t e,
                                          int node, int d, int side, const R* uo, R gamma,
                                          R igm1, R* F) {
  using Eu = Euler<D, R>;
  constexpr int NV = D + 2;
  R wo[NV];
  Eu::cons2prim(uo, wo, gamma);
  if (P.bc[2 * d + side] == BC_SLIP_WALL) {
    const R vn = side ? wo[1 + d] : -wo[1 + d];  // outward normal velocity
    const R ps = slip_wall_pressure<R>(wo[0], vn, wo[NV - 1], gamma, igm1);
#pragma unroll
    for (int v = 0; v < NV; ++v) F[v] = R(0);
    F[1 + d] = ps;
    return;
  }
  double x[D];
#pragma unroll
  for (int q = 0; q < D; ++q) x[q] = P.xline[((size_t)e * D + q) * N + axis_index<N>(node, q)];
  const double t = A.mode == MODE_RHS ? A.t_rhs : A.clock->t + A.c * A.clock->dt;
  double ubd[NV];
  boundary_value<D>(P.bc_ic, P.bc_par, x, t, P.gamma, ubd);
  R ub[NV], wb[NV];
#pragma unroll
  for (int v = 0; v < NV; ++v) ub[v] = (R)ubd[v];
  Eu::cons2prim(ub, wb, gamma);
  if (side)
    Eu::two_point(P.surface_flux, uo, wo, ub, wb, d, gamma, igm1, F);
  else
    Eu::two_point(P.surface_flux, ub, wb, uo, wo, d, gamma, igm1, F);
}

template <int D, int N, typename R, typename RT, int VI, int EPB>
__global__ void __launch_bounds__(EPB * Pow<N, D>::value)
    dg_element_kernel(const DgParams P, const StageArgs A) {
  using K = ElementKernel<D, N, R, RT, VI, EPB>;
  using Eu = Euler<D, R>;
  constexpr int NV = K::NV, NN = K::NN, NF = K::NF, NT = K::NT, SP = K::SP, NP = K::NP;
  constexpr int CHUNK = K::CHUNK;

  extern __shared__ __align__(16) unsigned char smem_raw[];
  double* s_u = reinterpret_cast<double*>(smem_raw);
  RT* s_tmp = reinterpret_cast<RT*>(s_u + CHUNK);
  R* s_w = reinterpret_cast<R*>(s_tmp + CHUNK);
  R* s_c = s_w + NV * SP;
  R* s_face = s_c + NV * SP;
  R* s_vol = s_face + EPB * 2 * D * NF * NV;
  R* s_fv = s_vol + K::VOL_FD;  // VI_HG only
  R* s_mat = s_vol + K::VOL;    // Dhat (weak) or Dsplit (FD/HG)
  R* s_iw = s_mat + N * N;
  R* s_alpha = s_iw + N + N * N;

  const int tid = threadIdx.x;
  const int slot = tid / NN;
  const int node = tid - slot * NN;
  const int64_t e0 = (int64_t)blockIdx.x * EPB;
  const int nel = (int)min((int64_t)EPB, P.nelements - e0);
  const bool active = slot < nel;
  const int64_t e = e0 + slot;
  const size_t gofs = (size_t)e0 * NN * NV;
  const int nval = nel * NN * NV;
  const R gamma = (R)P.gamma;
  const R igm1 = (R)P.inv_gamma_minus_one;

  if (A.mode == MODE_STAGE && A.clock->skip) {
    // The time loop has reached t_end: carry the state over unchanged so the
    // ping-pong buffers stay consistent.
    for (int k = tid; k < nval; k += NT) A.u_out[gofs + k] = A.u_in[gofs + k];
    return;
  }

  // ---- stage the element chunk (coalesced) and the basis matrices ----------
  for (int k = tid; k < nval; k += NT) s_u[k] = __ldg(A.u_in + gofs + k);
  if (A.mode == MODE_STAGE) {
    const RT* tg = reinterpret_cast<const RT*>(A.u_tmp) + gofs;
    for (int k = tid; k < nval; k += NT) s_tmp[k] = A.zero_tmp ? RT(0) : tg[k];
  }
  for (int k = tid; k < N * N; k += NT) {
    s_mat[k] = (R)(VI == VI_WEAK ? P.Dhat[k] : P.Dsplit[k]);
  }
  if (tid < N) s_iw[tid] = (R)P.inv_weights[tid];
  if (VI == VI_HG && node == 0 && active) {
    // smoothed blending factor: apply_smoothing!, indicators_2d.jl:104-136
    const R* raw = reinterpret_cast<const R*>(A.alpha_raw);
    R a = raw[e];
    if (P.alpha_smooth) {
#pragma unroll
      for (int dir = 0; dir < 2 * D; ++dir)
        a = smooth_over_face<R>(a, P.nbr[e * 2 * D + dir], raw, P.nbc, P.mnbr);
    }
    s_alpha[slot] = a;
    if (A.alpha_out) reinterpret_cast<R*>(A.alpha_out)[e] = a;
  }
  __syncthreads();

  R uc[NV], w[NV];
  if (active) {
#pragma unroll
    for (int v = 0; v < NV; ++v) uc[v] = (R)s_u[(slot * NN + node) * NV + v];
    Eu::cons2prim(uc, w, gamma);
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      s_c[v * SP + slot * NN + node] = uc[v];
      s_w[v * SP + slot * NN + node] = w[v];
    }
  }
  __syncthreads();

  // ---- interface fluxes of all 2D faces of the block's elements ------------
  for (int it = tid; it < nel * 2 * D * NF; it += NT) {
    const int sl = it / (2 * D * NF);
    const int rem = it - sl * (2 * D * NF);
    const int dir = rem / NF;
    const int fn = rem - dir * NF;
    const int d = dir >> 1;
    const int side = dir & 1;  // 0: face at -d, 1: face at +d
    const int S = axis_stride<N>(d);
    const int base = line_base<N>(fn, d);
    const int own = base + (side ? (N - 1) * S : 0);
    const int nnode = base + (side ? 0 : (N - 1) * S);
    const int64_t nb = P.nbr[(e0 + sl) * 2 * D + dir];
    R uo[NV], un[NV], ul[NV], ur[NV], wl[NV], wr[NV], F[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) uo[v] = s_c[v * SP + sl * NN + own];
    if (nb < 0 && -1 - nb >= P.nbc) {
      // mortar face: flux from the mortar pre-pass
      const double* mf = P.mflux + ((size_t)(-1 - nb - P.nbc) * NF + fn) * NV;
#pragma unroll
      for (int v = 0; v < NV; ++v) s_face[((sl * 2 * D + dir) * NF + fn) * NV + v] = (R)mf[v];
      continue;
    }
    if (nb < 0) {
      boundary_face_flux<D, N, R>(P, A, e0 + sl, own, d, side, uo, gamma, igm1, F);
#pragma unroll
      for (int v = 0; v < NV; ++v) s_face[((sl * 2 * D + dir) * NF + fn) * NV + v] = F[v];
      continue;
    }
    const int64_t nbs = nb - e0;
    if (nbs >= 0 && nbs < nel) {
#pragma unroll
      for (int v = 0; v < NV; ++v) un[v] = s_c[v * SP + (int)nbs * NN + nnode];
    } else {
      const double* p = A.u_in + ((size_t)nb * NN + nnode) * NV;
#pragma unroll
      for (int v = 0; v < NV; ++v) un[v] = (R)__ldg(p + v);
    }
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      ul[v] = side ? uo[v] : un[v];
      ur[v] = side ? un[v] : uo[v];
    }
    Eu::cons2prim(ul, wl, gamma);
    Eu::cons2prim(ur, wr, gamma);
    Eu::two_point(P.surface_flux, ul, wl, ur, wr, d, gamma, igm1, F);
#pragma unroll
    for (int v = 0; v < NV; ++v) s_face[((sl * 2 * D + dir) * NF + fn) * NV + v] = F[v];
  }

  // ---- volume fluxes --------------------------------------------------------
  if (active) {
    if (VI == VI_WEAK) {
#pragma unroll
      for (int d = 0; d < D; ++d) {
        R f[NV];
        Eu::flux(uc, w, d, f);
#pragma unroll
        for (int v = 0; v < NV; ++v) s_vol[(d * NV + v) * SP + slot * NN + node] = f[v];
      }
    } else {
#pragma unroll
      for (int d = 0; d < D; ++d) {
        const int S = axis_stride<N>(d);
        const int i = axis_index<N>(node, d);
        const int line = line_index<N>(node, d);
        const int lb = line_base<N>(line, d);
        for (int p = i; p < NP; p += N) {
          // decode pair p -> (a, b), a < b
          int a = 0, q = p;
          while (q >= N - 1 - a) {
            q -= N - 1 - a;
            ++a;
          }
          const int b = a + 1 + q;
          const int na = slot * NN + lb + a * S, nb2 = slot * NN + lb + b * S;
          R ul[NV], wl[NV], ur[NV], wr[NV], F[NV];
#pragma unroll
          for (int v = 0; v < NV; ++v) {
            ul[v] = s_c[v * SP + na];
            wl[v] = s_w[v * SP + na];
            ur[v] = s_c[v * SP + nb2];
            wr[v] = s_w[v * SP + nb2];
          }
          Eu::two_point(P.volume_flux, ul, wl, ur, wr, d, gamma, igm1, F);
#pragma unroll
          for (int v = 0; v < NV; ++v)
            s_vol[(((slot * D + d) * NF + line) * NP + p) * NV + v] = F[v];
        }
        if (VI == VI_HG && i < N - 1 && fabs(s_alpha[slot]) > (R)P.alpha_atol) {
          // subcell finite-volume flux between nodes i and i+1 (calcflux_fv!)
          const int na = slot * NN + node, nb2 = slot * NN + node + S;
          R ul[NV], wl[NV], ur[NV], wr[NV], F[NV];
#pragma unroll
          for (int v = 0; v < NV; ++v) {
            ul[v] = s_c[v * SP + na];
            wl[v] = s_w[v * SP + na];
            ur[v] = s_c[v * SP + nb2];
            wr[v] = s_w[v * SP + nb2];
          }
          Eu::two_point(P.fv_flux, ul, wl, ur, wr, d, gamma, igm1, F);
#pragma unroll
          for (int v = 0; v < NV; ++v)
            s_fv[(((slot * D + d) * NF + line) * (N - 1) + i) * NV + v] = F[v];
        }
      }
    }
  }
  __syncthreads();

  // ---- gather: volume + surface + Jacobian + sources -------------------------
  R du[NV];
#pragma unroll
  for (int v = 0; v < NV; ++v) du[v] = 0;
  if (active) {
    if (VI == VI_WEAK) {
#pragma unroll
      for (int d = 0; d < D; ++d) {
        const int S = axis_stride<N>(d);
        const int i = axis_index<N>(node, d);
        const int lb = line_base<N>(line_index<N>(node, d), d);
#pragma unroll
        for (int l = 0; l < N; ++l) {
          const R c = s_mat[i * N + l];
          const int src = slot * NN + lb + l * S;
#pragma unroll
          for (int v = 0; v < NV; ++v) du[v] += c * s_vol[(d * NV + v) * SP + src];
        }
      }
    } else {
#pragma unroll
      for (int d = 0; d < D; ++d) {
        const int i = axis_index<N>(node, d);
        const int line = line_index<N>(node, d);
#pragma unroll
        for (int l = 0; l < N; ++l) {
          if (l == i) continue;
          const int p = l > i ? pair_index<N>(i, l) : pair_index<N>(l, i);
          const R c = s_mat[i * N + l];
          const R* F = s_vol + (((slot * D + d) * NF + line) * NP + p) * NV;
#pragma unroll
          for (int v = 0; v < NV; ++v) du[v] += c * F[v];
        }
      }
      if (VI == VI_HG) {
        const R alpha = s_alpha[slot];
        if (fabs(alpha) > (R)P.alpha_atol) {
          R fv[NV];
#pragma unroll
          for (int v = 0; v < NV; ++v) fv[v] = 0;
#pragma unroll
          for (int d = 0; d < D; ++d) {
            const int i = axis_index<N>(node, d);
            const int line = line_index<N>(node, d);
            const R iw = s_iw[i];
            const R* Fb = s_fv + ((slot * D + d) * NF + line) * (N - 1) * NV;
#pragma unroll
            for (int v = 0; v < NV; ++v) {
              const R fr = i < N - 1 ? Fb[i * NV + v] : R(0);
              const R fl = i > 0 ? Fb[(i - 1) * NV + v] : R(0);
              fv[v] += iw * (fr - fl);
            }
          }
#pragma unroll
          for (int v = 0; v < NV; ++v) du[v] = (R(1) - alpha) * du[v] + alpha * fv[v];
        }
      }
    }
    // surface integral (LGL: weighted boundary interpolation = inverse_weights[1])
    const R factor = s_iw[0];
#pragma unroll
    for (int d = 0; d < D; ++d) {
      const int i = axis_index<N>(node, d);
      const int fn = line_index<N>(node, d);
      if (i == 0) {
        const R* F = s_face + ((slot * 2 * D + 2 * d) * NF + fn) * NV;
#pragma unroll
        for (int v = 0; v < NV; ++v) du[v] = du[v] - F[v] * factor;
      }
      if (i == N - 1) {
        const R* F = s_face + ((slot * 2 * D + 2 * d + 1) * NF + fn) * NV;
#pragma unroll
        for (int v = 0; v < NV; ++v) du[v] = du[v] + F[v] * factor;
      }
    }
    const R jfac = -(R)P.inv_jac[e];
#pragma unroll
    for (int v = 0; v < NV; ++v) du[v] *= jfac;
    if (P.source == SRC_CONVERGENCE_TEST) {
      R x[D], s[NV];
      const double* xl = P.xline + (size_t)e * D * N;
#pragma unroll
      for (int d = 0; d < D; ++d) x[d] = (R)xl[d * N + axis_index<N>(node, d)];
      const double tt = A.mode == MODE_RHS ? A.t_rhs : A.clock->t + A.c * A.clock->dt;
      Eu::source_convergence(x, (R)tt, gamma, s);
#pragma unroll
      for (int v = 0; v < NV; ++v) du[v] += s[v];
    }
  }

  if (A.mode == MODE_RHS) {
    if (active) {
#pragma unroll
      for (int v = 0; v < NV; ++v) s_u[(slot * NN + node) * NV + v] = (double)du[v];
    }
    __syncthreads();
    for (int k = tid; k < nval; k += NT) A.du_out[gofs + k] = s_u[k];
    return;
  }

  // ---- 2N stage update: u_tmp = du - a u_tmp; u = u + b dt u_tmp -----------
  const double bdt = A.b * A.clock->dt;
  const RT a_s = (RT)A.a;
  bool bad = false;
  R lam[D];
  if (active) {
    double un_[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      const int k = (slot * NN + node) * NV + v;
      const RT ut = (RT)du[v] - s_tmp[k] * a_s;
      s_tmp[k] = ut;
      un_[v] = s_u[k] + (double)ut * bdt;
      s_u[k] = un_[v];
      bad |= !(un_[v] == un_[v]);
    }
    if (A.speed_bits) {
      // max_abs_speeds of the new state, stepsize_dg{2,3}d.jl
      R uu[NV], ww[NV];
#pragma unroll
      for (int v = 0; v < NV; ++v) uu[v] = (R)un_[v];
      Eu::cons2prim(uu, ww, gamma);
      const R cs = Real<R>::sqrt(gamma * ww[NV - 1] / ww[0]);
      bad |= !(ww[0] > R(0)) || !(ww[NV - 1] > R(0));
#pragma unroll
      for (int d = 0; d < D; ++d) lam[d] = fabs(ww[1 + d]) + cs;
    }
  }
  if (bad) atomicOr(A.status, 1);
  __syncthreads();
  {
    RT* tg = reinterpret_cast<RT*>(A.u_tmp) + gofs;
    for (int k = tid; k < nval; k += NT) {
      A.u_out[gofs + k] = s_u[k];
      tg[k] = s_tmp[k];
    }
  }
  if (A.speed_bits) {
    // element maxima over nodes per direction, then max over elements
    if (active) {
#pragma unroll
      for (int d = 0; d < D; ++d) s_w[d * SP + slot * NN + node] = lam[d];
    }
    __syncthreads();
    if (active && node == 0) {
      R sum = 0;
#pragma unroll
      for (int d = 0; d < D; ++d) {
        R m = 0;
        for (int q = 0; q < NN; ++q) m = fmax(m, s_w[d * SP + slot * NN + q]);
        sum += m;
      }
      const double sp = P.inv_jac[e] * (double)sum;
      if (sp == sp) atomicMax(A.speed_bits, (unsigned long long)__double_as_longlong(sp));
      else atomicOr(A.status, 1);
    }
  }
}

// ---------------------------------------------------------------------------
// Hennemann-Gassner indicator (unsmoothed), one thread per node:
// indicators.jl:114-148, indicators_2d.jl:30-101, indicators_3d.jl:39-123.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double state_value(double x) { return x; }
__device__ __forceinline__ float state_value(float2 x) { return x.x; }

// PT: DgParams (FP64 path) or MixedParams; TS: double or float2 (float-float) state.
template <int D, int N, typename R, int EPB, typename PT, typename TS>
__global__ void __launch_bounds__(EPB * Pow<N, D>::value)
    hg_indicator_kernel(const PT P, const TS* __restrict__ u, R* __restrict__ alpha_raw) {
  constexpr int NV = D + 2, NN = Pow<N, D>::value, NT = EPB * NN;
  __shared__ R s_a[EPB * NN], s_b[EPB * NN], s_v[N * N];
  const int tid = threadIdx.x;
  const int slot = tid / NN, node = tid - slot * NN;
  const int64_t e0 = (int64_t)blockIdx.x * EPB;
  const int nel = (int)min((int64_t)EPB, P.nelements - e0);
  const bool active = slot < nel;
  const int64_t e = e0 + slot;
  for (int k = tid; k < N * N; k += NT) s_v[k] = (R)P.Vinv[k];
  if (active) {
    R uu[NV];
    const TS* p = u + ((size_t)e * NN + node) * NV;
#pragma unroll
    for (int v = 0; v < NV; ++v) uu[v] = (R)state_value(p[v]);
    s_a[tid] = P.hg_variable == 1 ? uu[0] : Euler<D, R>::density_pressure(uu, (R)P.gamma);
  }
  __syncthreads();
  // multiply_scalar_dimensionwise!: x, then y, then z
  R* in = s_a;
  R* out = s_b;
#pragma unroll
  for (int d = 0; d < D; ++d) {
    if (active) {
      const int S = axis_stride<N>(d);
      const int i = axis_index<N>(node, d);
      const int lb = line_base<N>(line_index<N>(node, d), d);
      R r = 0;
#pragma unroll
      for (int k = 0; k < N; ++k) r += s_v[i * N + k] * in[slot * NN + lb + k * S];
      out[tid] = r;
    }
    __syncthreads();
    R* t = in;
    in = out;
    out = t;
  }
  if (active && node == 0) {
    R clip2 = 0, clip1 = 0, tot = 0;
    for (int q = 0; q < NN; ++q) {
      int mx = 0;
#pragma unroll
      for (int d = 0; d < D; ++d) mx = max(mx, axis_index<N>(q, d));
      const R m = in[slot * NN + q];
      const R m2 = m * m;
      if (mx <= N - 3) clip2 += m2;
      if (mx <= N - 2) clip1 += m2;
      tot += m2;
    }
    const R f1 = tot != R(0) ? (tot - clip1) / tot : R(0);
    const R f2 = clip1 != R(0) ? (clip1 - clip2) / clip1 : R(0);
    const R energy = fmax(f1, f2);
    const R thr = (R)P.hg_threshold;
    R a = R(1) / (R(1) + Real<R>::exp(-(R)P.hg_parameter_s / thr * (energy - thr)));
    if (a < (R)P.alpha_min) a = 0;
    if (a > R(1) - (R)P.alpha_min) a = 1;
    alpha_raw[e] = fmin((R)P.alpha_max, a);
  }
}

// Host-side launch helpers (defined in the instantiation units).
int launch_element(int D, int N, bool fp64, int vi, int epb, const DgParams& P,
                   const StageArgs& A, cudaStream_t s);
int launch_indicator(int D, int N, bool fp64, const DgParams& P, const double* u,
                     void* alpha_raw, cudaStream_t s);
int default_epb(int D, int N);
bool supported_epb(int D, int N, int epb);

}  // namespace tg
