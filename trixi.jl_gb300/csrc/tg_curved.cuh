// Fused DGSEM stage kernels of curvilinear 2D meshes (StructuredMesh and
// P4estMesh bricks), FP64 and mixed precision, for sm_103a.
//
// The element work follows dgsem_structured/dg_2d.jl: volume integrals with
// contravariant fluxes (weak_form_kernel! :34-75 with Ja^i . f, and
// flux_differencing_kernel! :77-139 with the two-point flux along the averaged
// contravariant vector), interface fluxes along the contravariant vector of
// the element face (calc_interface_flux!, :551-606; dgsem_p4est/dg_2d.jl:263-
// 434), the surface integral of dgsem_tree/dg_2d.jl:1245-1287, apply_jacobian!
// with the per-node inverse Jacobian (dgsem_structured/dg_2d.jl:751-771) and
// sources at the node coordinates.  The CFL reduction is the curvilinear
// max_dt (stepsize_dg2d.jl:114-157).
#pragma once

#include "tg_mixed.cuh"

namespace tg {

struct CurvedParams {
  int64_t nelements;
  int32_t N;                // nodes per direction
  int32_t vi;               // VI_WEAK, VI_FD or VI_HG (2D)
  int32_t volume_flux, surface_flux, source;
  double gamma, inv_gamma_minus_one;
  EosF eos;
  // n x n matrices row-major with the actual n: M[a * n + b] = M[a, b]
  double Dhat[MAXN * MAXN], Dsplit[MAXN * MAXN], inv_weights[MAXN];
  float Dhat32[MAXN * MAXN], Dsplit32[MAXN * MAXN], inv_weights32[MAXN];
  const int32_t* nbr;       // [E][4]: element across -x, +x, -y, +y
  const double* met;        // [E][NN][5]: Ja^1_x, Ja^1_y, Ja^2_x, Ja^2_y, inverse Jacobian
  const float4* ja32;       // [E][NN]: Ja^1_x, Ja^1_y, Ja^2_x, Ja^2_y (3D: see below)
  const float* invj32;      // [E][NN] (2D)
  const double* xy;         // [E][NN][2] node coordinates (FP64 sources)
  const float4* sc;         // [E][NN] sin/cos(pi (x + y)): (sin hi, cos hi, sin lo, cos lo)
  // Faces at a non-periodic edge have nbr = -1 - b (b: boundary face number,
  // bface[b] = element, direction) and take BoundaryConditionDirichlet of the
  // initial condition bc_ic (dgsem_structured/dg_2d.jl:680-750, dg.jl:124-163):
  // the FP64 kernel evaluates it at the face node (xy); the mixed kernel reads
  // ghost[b][face node] (float-float), written by launch_curved_ghost.
  int32_t bc_ic;
  double bc_par[4];
  const int32_t* bface;     // [B][2]
  const float2* ghost;      // [B][N][4]
  // VI_HG (VolumeIntegralShockCapturingHG, dgsem_structured/dg_2d.jl:304-345):
  // the FV flux, apply_smoothing! of the raw indicator (the stage arguments'
  // alpha_raw), the blending threshold (calc_volume_integral.jl:242-245) and
  // the free-stream preserving subcell normals (containers_2d.jl:200-298):
  // snv[e][d][l][i] = normal of the interface between nodes i and i + 1 of
  // line l in direction d, i = 0 .. N - 2 (FP64 pairs; FP32 copy for mixed)
  int32_t fv_flux, alpha_smooth;
  double alpha_atol;
  const double2* snv;       // [E][2][N][N - 1]
  const float2* snv32;
  // 3D: the same per direction d and line l (the two other node indices,
  // lower one fastest): [E][3][N^2][N - 1], FP64 triples and FP32 (x, y, z, 0)
  const double* snv3;
  const float4* snv3_32;
};

// ---------------------------------------------------------------------------
// Flux deviations along a normal direction n (the mixed kernels): the
// two-point flux between nodes a and b of the element with reference state R
// minus the reference's physical flux f(w_ref) . n
// ---------------------------------------------------------------------------

// x . n with the products summed left to right
template <int D>
__device__ __forceinline__ float dot_n(const float* x, const float* n) {
  float r = x[0] * n[0];
#pragma unroll
  for (int d = 1; d < D; ++d) r = fmaf(x[d], n[d], r);
  return r;
}

// Flux of kind KIND (or `kind` at run time): the fluxes are linear in n, so
// the deviation along n is the sum over d of n_d times the deviation along
// axis d.
template <int D, int KIND>
__device__ __forceinline__ void dev_flux_n(int kind, const RefState<D>& R, const Node<D>& a,
                                           const Node<D>& b, const float* n, const EosF& eos,
                                           float* F) {
  using Dv = Dev<D>;
  constexpr int NV = D + 2;
#pragma unroll
  for (int d = 0; d < D; ++d) {
    Node<D> ad = a, bd = b;
    Dv::orient(ad, d);
    Dv::orient(bd, d);
    float fd[NV];
    Dv::template flux2<KIND>(kind, R, ad, bd, d, R.v[d], eos, fd);
#pragma unroll
    for (int v = 0; v < NV; ++v) F[v] = d == 0 ? n[0] * fd[v] : fmaf(n[d], fd[v], F[v]);
  }
}

// flux_ranocha(a, b, n) - f(w_ref) . n in one pass (compressible_euler_2d.jl:
// 724-753, compressible_euler_3d.jl normal-direction method): Dev::dranocha
// with the axis replaced by the normal -- the reference normal velocity
// v_ref . n, the nodes' normal-velocity deviations dv . n and the pressure
// term dp_avg n -- so the two logarithmic means are evaluated once instead of
// once per axis.  Algebraically equal to dev_flux_n<D, FLUX_RANOCHA>.
template <int D>
__device__ __forceinline__ void dev_ranocha_n(const RefState<D>& R, const Node<D>& a,
                                              const Node<D>& b, const float* n, const EosF& eos,
                                              float* f) {
  using Dv = Dev<D>;
  constexpr int P = D + 1;
  const float igm1 = eos.igm1;
  const float drho_ln = Dv::dev_ln_mean(R.rho, a.dw[0], b.dw[0], a.w[0], b.w[0]);
  const float dq_ln = Dv::dev_ln_mean(R.q, a.dq, b.dq, R.q + a.dq, R.q + b.dq);
  const float q_ln = R.q + dq_ln;
  float dvavg[D], vavg[D];
  float dvsq = 0, vsq = 0;
#pragma unroll
  for (int d = 0; d < D; ++d) {
    dvavg[d] = 0.5f * (a.dw[1 + d] + b.dw[1 + d]);
    vavg[d] = R.v[d] + dvavg[d];
    dvsq += R.v[d] * (a.dw[1 + d] + b.dw[1 + d]) + a.dw[1 + d] * b.dw[1 + d];
    vsq += a.w[1 + d] * b.w[1 + d];
  }
  dvsq *= 0.5f;
  const float dpavg = 0.5f * (a.dw[P] + b.dw[P]);
  const float vrn = dot_n<D>(R.v, n);
  const float dvan = dot_n<D>(a.dw + 1, n), dvbn = dot_n<D>(b.dw + 1, n);
  const float F1r = R.rho * vrn;
  const float dvavgn = 0.5f * (dvan + dvbn);
  const float d1 = R.rho * dvavgn + drho_ln * (vrn + dvavgn);
  f[0] = d1;
#pragma unroll
  for (int d = 0; d < D; ++d) f[1 + d] = d1 * vavg[d] + F1r * dvavg[d] + dpavg * n[d];
  const float H = 0.5f * vsq + igm1 / q_ln;
  const float dH = dvsq + igm1 * (R.rq - R.p * dq_ln) / (R.rho * q_ln);
  const float dpv = 0.5f * (R.p * (dvan + dvbn) + vrn * (a.dw[P] + b.dw[P]) + a.dw[P] * dvbn +
                            b.dw[P] * dvan);
  f[P] = d1 * H + F1r * dH + dpv;
}

// Surface (or FV subcell) flux deviation along n: the linear fluxes as above;
// the Lax-Friedrichs fluxes as the central flux plus the dissipation
// -lambda/2 (u_b - u_a) with lambda from the normal velocities and |n|
// (max_abs_speed(_naive) along a normal).  Needs the nodes' du.
template <int D>
__device__ __forceinline__ void dev_surface_n(int kind, const RefState<D>& R, const Node<D>& a,
                                              const Node<D>& b, const float* n, const EosF& eos,
                                              float* F) {
  constexpr int NV = D + 2, P = D + 1;
  if (kind == FLUX_RANOCHA) {
    dev_ranocha_n<D>(R, a, b, n, eos, F);
    return;
  }
  if (kind != FLUX_LLF && kind != FLUX_LLF_NAIVE) {
    dev_flux_n<D, -1>(kind, R, a, b, n, eos, F);
    return;
  }
  dev_flux_n<D, FLUX_CENTRAL>(FLUX_CENTRAL, R, a, b, n, eos, F);
  const float va = dot_n<D>(a.w + 1, n), vb = dot_n<D>(b.w + 1, n);
  const float ca = sqrtf(eos.gamma * a.w[P] / a.w[0]), cb = sqrtf(eos.gamma * b.w[P] / b.w[0]);
  const float nn = sqrtf(dot_n<D>(n, n));
  const float lam = kind == FLUX_LLF_NAIVE ? fmaxf(fabsf(va), fabsf(vb)) + fmaxf(ca, cb) * nn
                                           : fmaxf(fabsf(va) + ca * nn, fabsf(vb) + cb * nn);
#pragma unroll
  for (int v = 0; v < NV; ++v) F[v] = F[v] + (-0.5f * lam * (b.du[v] - a.du[v]));
}

// dev_surface_n with the flux kind fixed at compile time (KIND >= 0; the
// flux-specialised mixed kernels) or dispatched at run time (KIND < 0).
template <int D, int KIND>
__device__ __forceinline__ void dev_surface_k(int kind, const RefState<D>& R, const Node<D>& a,
                                              const Node<D>& b, const float* n, const EosF& eos,
                                              float* F) {
  if constexpr (KIND < 0) {
    dev_surface_n<D>(kind, R, a, b, n, eos, F);
  } else if constexpr (KIND == FLUX_RANOCHA) {
    dev_ranocha_n<D>(R, a, b, n, eos, F);
  } else if constexpr (KIND == FLUX_LLF || KIND == FLUX_LLF_NAIVE) {
    constexpr int NV = D + 2, P = D + 1;
    dev_flux_n<D, FLUX_CENTRAL>(FLUX_CENTRAL, R, a, b, n, eos, F);
    const float va = dot_n<D>(a.w + 1, n), vb = dot_n<D>(b.w + 1, n);
    const float ca = sqrtf(eos.gamma * a.w[P] / a.w[0]), cb = sqrtf(eos.gamma * b.w[P] / b.w[0]);
    const float nn = sqrtf(dot_n<D>(n, n));
    const float lam = KIND == FLUX_LLF_NAIVE ? fmaxf(fabsf(va), fabsf(vb)) + fmaxf(ca, cb) * nn
                                             : fmaxf(fabsf(va) + ca * nn, fabsf(vb) + cb * nn);
#pragma unroll
    for (int v = 0; v < NV; ++v) F[v] = F[v] + (-0.5f * lam * (b.du[v] - a.du[v]));
  } else {
    dev_flux_n<D, KIND>(KIND, R, a, b, n, eos, F);
  }
}

// ---------------------------------------------------------------------------
// Node indexing and block shape of the 2D curvilinear kernels
// ---------------------------------------------------------------------------
template <int N>
__device__ __forceinline__ int cline_node(int line, int dd, int a) {
  // node a of line `line` in direction dd (node index q = i + N j)
  return dd == 0 ? a + N * line : line + N * a;
}

// Node of the neighbour across face dir of an element that meets face node fn.
template <int N>
__device__ __forceinline__ int cface_partner(int dir, int fn) {
  switch (dir) {
    case 0: return (N - 1) + N * fn;  // -x: neighbour's +x face
    case 1: return N * fn;            // +x: neighbour's -x face
    case 2: return fn + N * (N - 1);  // -y: neighbour's +y face
    default: return fn;               // +y: neighbour's -y face
  }
}

// Node of this element at face dir that meets face node fn.
template <int N>
__device__ __forceinline__ int cface_own(int dir, int fn) {
  switch (dir) {
    case 0: return N * fn;
    case 1: return (N - 1) + N * fn;
    case 2: return fn;
    default: return fn + N * (N - 1);
  }
}

// Position of block node n (= slot * N^2 + node) in the mixed kernel's
// per-node shared arrays.  For N = 4 the low and high halves of the node index
// are XORed with bits 1-2 of the element slot: a warp holds the x-lines (or the
// y-lines) of 8 elements, whose same-parity elements would otherwise fall on
// the same 8 banks (4-way conflicts); with the permutation the 32 lanes of
// every line-phase access and of the node phase hit 32 different banks.
template <int N>
__device__ __forceinline__ int cpos(int n) {
  if constexpr (N == 4) {
    const int g = (n >> 5) & 3;  // bits 1-2 of the slot n >> 4
    return n ^ (g | (g << 2));
  } else {
    return n;
  }
}

template <int N, int EPB>
struct CurvedK {
  static constexpr int NN = N * N, NV = 4, NT = EPB * 2 * N;
  static constexpr int CHUNK = EPB * NN * NV;  // state values of a block
  static constexpr int FACE = EPB * 4 * N * NV;
  static constexpr int SP = EPB * NN;          // field stride of the partial sums
  // resident blocks per SM asked of the mixed kernel: for N <= 4 five blocks
  // fit its shared memory (44 KB at N = 4) and 96 registers per thread
  static constexpr int MINB_MIXED = N <= 4 ? 5 : 1;
};

// Elements per block of the curvilinear kernels (0: polydeg not compiled);
// the mixed 2D weak-form kernel at polydeg 3 runs 8 (tg_curved_mixed_2d.cu).
int curved_epb(int N);

// The mixed-precision 2D stage kernels (tg_curved_mixed_2d.cu, compiled with
// the FP32 flags of the mixed units).
int launch_curved_mixed2(const CurvedParams& P, const MixedArgs& A, cudaStream_t stream);

// ---------------------------------------------------------------------------
// Node indexing of the 3D curvilinear kernels
// ---------------------------------------------------------------------------
// node a of line `line` (0 .. N^2 - 1) in direction dd, node q = i + N j + N^2 k
template <int N>
__device__ __forceinline__ int line3(int line, int dd, int a) {
  if (dd == 0) return a + N * line;                           // line = j + N k
  if (dd == 1) return (line % N) + N * a + N * N * (line / N);  // line = i + N k
  return line + N * N * a;                                    // line = i + N j
}

// face node fn of face dir (fn runs over the two tangential indices, the
// lower one fastest): this element's node there, and the neighbour's node
template <int N>
__device__ __forceinline__ int face_own3(int dir, int fn) {
  switch (dir) {
    case 0: return N * fn;
    case 1: return (N - 1) + N * fn;
    case 2: return (fn % N) + N * N * (fn / N);
    case 3: return (fn % N) + N * (N - 1) + N * N * (fn / N);
    case 4: return fn;
    default: return fn + N * N * (N - 1);
  }
}

template <int N>
__device__ __forceinline__ int face_partner3(int dir, int fn) {
  return face_own3<N>(dir ^ 1, fn);
}

// The mixed-precision 3D stage kernels (tg_curved_mixed_3d.cu, compiled with
// the FP32 flags of the mixed units).
int launch_curved_mixed3(const CurvedParams& P, const MixedArgs& A, cudaStream_t stream);

// One stage (or rhs) launch; exactly one of A64 (FP64 context) and A32
// (mixed context) is non-null.
int launch_curved(const CurvedParams& P, const StageArgs* A64, const MixedArgs* A32,
                  cudaStream_t stream);

// Mixed contexts with boundary faces: the float-float Dirichlet states of the
// B boundary faces for the stage with weight c_s (MODE_STAGE: t + c_s dt of
// the clock) or at t_rhs (MODE_RHS), into ghost.
int launch_curved_ghost(const CurvedParams& P, int64_t B, const Clock* clock, double c_s,
                        double t_rhs, int mode, float2* ghost, cudaStream_t stream);

// max_dt reduction of a state (FP64 values, or the float-float state of a
// mixed context in that context's FP32 arithmetic) into dst (double bits).
int launch_curved_speed(const CurvedParams& P, const void* u, bool ff, unsigned long long* dst,
                        int32_t* status, cudaStream_t stream);

// Per-element FP64 integrals (conserved totals, entropy, kinetic energy) with
// the per-node Jacobian, as element_integrals_kernel.
int launch_curved_integrals(const CurvedParams& P, const void* u, bool ff, const double* weights,
                            double* partial, cudaStream_t stream);

// 3D curvilinear meshes (tg_curved3.cu): P.met holds [E][NN][10] (Ja^d_c at
// d * 3 + c, then the inverse Jacobian), P.xy [E][NN][3], P.nbr [E][6]; mixed
// contexts also P.ja32 as [E][NN][3] float4 {Ja^d_x, Ja^d_y, Ja^d_z, (d = 0:
// inverse Jacobian)} and, with MMS sources, P.sc with the phase x + y + z.
// Exactly one of A64 (FP64 context) and A32 (mixed context) is non-null; u is
// the context's state (float-float when ff), the speed and the integrals are
// evaluated in FP64.
int curved3_supported(int N);
int launch_curved3(const CurvedParams& P, const StageArgs* A64, const MixedArgs* A32,
                   cudaStream_t stream);
int launch_curved3_speed(const CurvedParams& P, const void* u, bool ff, unsigned long long* dst,
                         int32_t* status, cudaStream_t stream);
int launch_curved3_integrals(const CurvedParams& P, const void* u, bool ff, const double* weights,
                             double* partial, cudaStream_t stream);

}  // namespace tg
