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
  const float4* ja32;       // [E][NN]: Ja^1_x, Ja^1_y, Ja^2_x, Ja^2_y
  const float* invj32;      // [E][NN]
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
};

// Elements per block of the curvilinear kernels (0: polydeg not compiled).
int curved_epb(int N);

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

// 3D curvilinear meshes (tg_curved3.cu), FP64 contexts only: P.met holds
// [E][NN][10] (Ja^d_c at d * 3 + c, then the inverse Jacobian), P.xy [E][NN][3],
// P.nbr [E][6].
int curved3_supported(int N);
int launch_curved3(const CurvedParams& P, const StageArgs& A, cudaStream_t stream);
int launch_curved3_speed(const CurvedParams& P, const double* u, unsigned long long* dst,
                         int32_t* status, cudaStream_t stream);
int launch_curved3_integrals(const CurvedParams& P, const double* u, const double* weights,
                             double* partial, cudaStream_t stream);

}  // namespace tg
