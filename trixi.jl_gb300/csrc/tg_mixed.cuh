// Mixed-precision path of the fused DGSEM stage kernel (sm_103a).
//
// GB300 runs FP64 at a small fraction of its FP32 rate, so this path keeps
// FP64 instructions out of the per-node work entirely:
//
// 1. The solution is stored in HBM as float-float pairs (hi, lo), 8 bytes per
//    value like FP64, with |lo| <= ulp(hi)/2 (about 48 significant bits).  The
//    2N stage update u += b dt u_tmp is a float-float addition (TwoSum, then
//    Fast2Sum), so the stage accumulation keeps ~1e-14 relative precision.
//
// 2. Deviation form.  Within element e all fluxes are evaluated as deviations
//    F(a, b) - f(w_e) from the physical flux of a reference state w_e (the
//    primitives of node 0's `hi` part), using algebra that involves only node
//    deviations from w_e.  Those deviations are formed exactly from the
//    float-float state ((hi_i - hi_ref) + lo_i), so FP32 rounding is relative
//    to |u_i - u_ref| instead of |u_i|.  The reference flux drops out exactly:
//    the split-form and weak-form derivative matrices have zero interior row
//    sums and +-1/w at the end rows, where it cancels against the same
//    reference flux inside the surface term (calc_surface_integral!), and the
//    subcell finite-volume sums telescope.  Without this, FP32 rounding of the
//    state is amplified by the derivative operator (|D| ~ N^2/dx) and sets an
//    error floor above the scheme's own error on fine meshes.
//
// Everything else (block/thread layout, both-sided interface fluxes, pair
// sweep, surface lift, Jacobian, sources, coalesced staging) mirrors the FP64
// kernel in tg_dg.cuh; see there for the reference citations.
#pragma once

#include "tg_dg.cuh"

namespace tg {

struct MixedParams {
  int64_t nelements;
  float gamma, inv_gamma_minus_one;
  float inv_weights[MAXN];
  float Dhat[MAXN * MAXN];
  float Dsplit[MAXN * MAXN];
  float Vinv[MAXN * MAXN];
  int32_t volume_flux, surface_flux, fv_flux, source;
  float alpha_max, alpha_min, alpha_atol, hg_threshold, hg_parameter_s;
  int32_t alpha_smooth;
  const int32_t* nbr;       // [E][2D]
  const float* inv_jac;     // [E]
  const float* xline;       // [E][D][N] or null
};

struct MixedArgs {
  const float2* u_in;       // float-float state (hi, lo) per value
  float2* u_out;            // MODE_STAGE
  double* du_out;           // MODE_RHS (FP64 du, Trixi layout)
  float* u_tmp;             // MODE_STAGE
  const float* alpha_raw;   // VI_HG
  float* alpha_out;         // VI_HG (optional)
  const Clock* clock;
  unsigned long long* speed_bits;
  int32_t* status;
  double t_rhs;
  double a, b, c;           // 2N coefficients of the stage
  int32_t mode;
  int32_t zero_tmp;
};

// ---------------------------------------------------------------------------
// Reference state of an element and node deviations
// ---------------------------------------------------------------------------
template <int D>
struct RefState {
  float rho, v[D], p;   // reference primitives w_e
  float q, rq;          // q = rho/p and its residual rho - q p (exact by FMA)
  float hi[D + 2];      // conservative reference (hi of node 0)
  float r[D + 2];       // hi - cons(w_e): momentum residual exact, energy to FP32
};

template <int D>
struct Node {
  float du[D + 2];      // conservative deviation from cons(w_e)
  float dw[D + 2];      // primitive deviation (drho, dv_1..dv_D, dp)
  float w[D + 2];       // full primitives
};

template <int D>
struct Dev {
  static constexpr int NV = D + 2, P = D + 1;

  static __host__ __device__ __forceinline__ void make_ref(const float* hi, float gamma, float igm1,
                                                   RefState<D>& R) {
    R.rho = hi[0];
    const float irho = 1.0f / R.rho;
    float ke = 0;
#pragma unroll
    for (int d = 0; d < D; ++d) {
      R.v[d] = hi[1 + d] * irho;
      ke += hi[1 + d] * R.v[d];
    }
    R.p = (gamma - 1.0f) * (hi[P] - 0.5f * ke);
    R.q = R.rho / R.p;
    R.rq = fmaf(-R.q, R.p, R.rho);
    float v2 = 0;
#pragma unroll
    for (int d = 0; d < D; ++d) v2 += R.v[d] * R.v[d];
#pragma unroll
    for (int v = 0; v < NV; ++v) R.hi[v] = hi[v];
    R.r[0] = 0.0f;
#pragma unroll
    for (int d = 0; d < D; ++d) R.r[1 + d] = fmaf(-R.v[d], R.rho, hi[1 + d]);
    // energy residual hi - (p igm1 + rho |v|^2 / 2): the product error of p igm1
    // is recovered exactly by an FMA and hi - p igm1 is exact (Sterbenz) unless
    // the kinetic energy dominates, so the residual is good to FP32 rounding of
    // the (small) kinetic part instead of a unit in the last place of E.
    const float pe = R.p * igm1;
    const float pe_err = fmaf(R.p, igm1, -pe);
    R.r[P] = ((hi[P] - pe) - pe_err) - 0.5f * R.rho * v2;
  }

  // Node state (hi, lo) -> deviations relative to R and full primitives.
  static __host__ __device__ __forceinline__ void make_node(const float* hi, const float* lo,
                                                    const RefState<D>& R, float gamma, Node<D>& n) {
#pragma unroll
    for (int v = 0; v < NV; ++v) n.du[v] = ((hi[v] - R.hi[v]) + lo[v]) + R.r[v];
    const float drho = n.du[0];
    const float rho = R.rho + drho;
    const float irho = 1.0f / rho;
    float kin = 0;
    float vbar2 = 0;
#pragma unroll
    for (int d = 0; d < D; ++d) {
      const float dv = (n.du[1 + d] - R.v[d] * drho) * irho;
      n.dw[1 + d] = dv;
      n.w[1 + d] = R.v[d] + dv;
      kin += dv * (2.0f * R.v[d] + dv);
      vbar2 += R.v[d] * R.v[d];
    }
    // rho|v|^2 - rho_ref|v_ref|^2 = drho |v_ref|^2 + rho (2 v_ref.dv + |dv|^2)
    const float dkin = drho * vbar2 + rho * kin;
    const float dp = (gamma - 1.0f) * (n.du[P] - 0.5f * dkin);
    n.dw[0] = drho;
    n.w[0] = rho;
    n.dw[P] = dp;
    n.w[P] = R.p + dp;
  }

  static __host__ __device__ __forceinline__ float pick(const float* a, int o) {
    float r = a[0];
#pragma unroll
    for (int d = 1; d < D; ++d) r = (o == d) ? a[d] : r;
    return r;
  }

  // ln_mean(x_ref + dx, x_ref + dy) - x_ref (series below f^2 < 0.05, see
  // tg_physics.cuh for the FP32 threshold)
  static __host__ __device__ __forceinline__ float dev_ln_mean(float xr, float dx, float dy, float x,
                                                       float y) {
    const float s = x + y;
    const float f = (dy - dx) / s;
    const float f2 = f * f;
    if (f2 < 0.05f) {
      const float P1 = f2 * (1.0f / 3.0f + f2 * (1.0f / 5.0f + f2 * (1.0f / 7.0f + f2 * (1.0f / 9.0f))));
      return ((dx + dy) - 2.0f * xr * P1) / (2.0f * (1.0f + P1));
    }
    return (y - x) / logf(y / x) - xr;
  }

  // physical flux deviation f(w) - f(w_ref), orientation o
  static __host__ __device__ __forceinline__ void dflux(const RefState<D>& R, const Node<D>& a, int o,
                                                float gamma, float igm1, float* f) {
    const float vro = pick(R.v, o), vo = pick(a.w + 1, o), dvo = pick(a.dw + 1, o);
    const float d1 = a.dw[0] * vro + a.w[0] * dvo;
    const float F1r = R.rho * vro;
    f[0] = d1;
    float dk = 0, k = 0;
#pragma unroll
    for (int d = 0; d < D; ++d) {
      f[1 + d] = d1 * a.w[1 + d] + F1r * a.dw[1 + d] + ((d == o) ? a.dw[P] : 0.0f);
      dk += a.dw[1 + d] * (R.v[d] + 0.5f * a.dw[1 + d]);
      k += a.w[1 + d] * a.w[1 + d];
    }
    f[P] = d1 * (0.5f * k) + F1r * dk + gamma * igm1 * (a.dw[P] * vo + R.p * dvo);
  }

  static __host__ __device__ __forceinline__ void dcentral(const RefState<D>& R, const Node<D>& a,
                                                   const Node<D>& b, int o, float gamma,
                                                   float igm1, float* f) {
    float fa[NV], fb[NV];
    dflux(R, a, o, gamma, igm1, fa);
    dflux(R, b, o, gamma, igm1, fb);
#pragma unroll
    for (int v = 0; v < NV; ++v) f[v] = 0.5f * (fa[v] + fb[v]);
  }

  static __host__ __device__ __forceinline__ void dllf(const RefState<D>& R, const Node<D>& a,
                                               const Node<D>& b, int o, bool naive, float gamma,
                                               float igm1, float* f) {
    dcentral(R, a, b, o, gamma, igm1, f);
    const float ca = sqrtf(gamma * a.w[P] / a.w[0]);
    const float cb = sqrtf(gamma * b.w[P] / b.w[0]);
    const float va = fabsf(pick(a.w + 1, o)), vb = fabsf(pick(b.w + 1, o));
    const float lam = naive ? fmaxf(va, vb) + fmaxf(ca, cb) : fmaxf(va + ca, vb + cb);
#pragma unroll
    for (int v = 0; v < NV; ++v) f[v] = f[v] + (-0.5f * lam * (b.du[v] - a.du[v]));
  }

  // flux_ranocha(a, b) - f(w_ref)
  static __host__ __device__ __forceinline__ void dranocha(const RefState<D>& R, const Node<D>& a,
                                                   const Node<D>& b, int o, float igm1, float* f) {
    const float drho_ln = dev_ln_mean(R.rho, a.dw[0], b.dw[0], a.w[0], b.w[0]);
    // q = rho / p relative to R.q, with the exact residual R.rq = rho_ref - q_ref p_ref
    const float dqa = (R.rq + a.dw[0] - R.q * a.dw[P]) / a.w[P];
    const float dqb = (R.rq + b.dw[0] - R.q * b.dw[P]) / b.w[P];
    const float dq_ln = dev_ln_mean(R.q, dqa, dqb, R.q + dqa, R.q + dqb);
    const float q_ln = R.q + dq_ln;
    float dvavg[D], vavg[D];
    float dvsq = 0;
#pragma unroll
    for (int d = 0; d < D; ++d) {
      dvavg[d] = 0.5f * (a.dw[1 + d] + b.dw[1 + d]);
      vavg[d] = R.v[d] + dvavg[d];
      dvsq += R.v[d] * (a.dw[1 + d] + b.dw[1 + d]) + a.dw[1 + d] * b.dw[1 + d];
    }
    dvsq *= 0.5f;
    const float dpavg = 0.5f * (a.dw[P] + b.dw[P]);
    const float vro = pick(R.v, o);
    const float F1r = R.rho * vro;
    const float d1 = R.rho * pick(dvavg, o) + drho_ln * pick(vavg, o);
    f[0] = d1;
#pragma unroll
    for (int d = 0; d < D; ++d) f[1 + d] = d1 * vavg[d] + F1r * dvavg[d] + ((d == o) ? dpavg : 0.0f);
    float vsq = 0;
#pragma unroll
    for (int d = 0; d < D; ++d) vsq += a.w[1 + d] * b.w[1 + d];
    const float H = 0.5f * vsq + igm1 / q_ln;
    const float dH = dvsq + igm1 * (R.rq - R.p * dq_ln) / (R.rho * q_ln);
    const float dvao = pick(a.dw + 1, o), dvbo = pick(b.dw + 1, o);
    const float dpv = 0.5f * (R.p * (dvao + dvbo) + vro * (a.dw[P] + b.dw[P]) +
                              a.dw[P] * dvbo + b.dw[P] * dvao);
    f[P] = d1 * H + F1r * dH + dpv;
  }

  // flux_shima_etal(a, b) - f(w_ref)
  static __host__ __device__ __forceinline__ void dshima(const RefState<D>& R, const Node<D>& a,
                                                 const Node<D>& b, int o, float igm1, float* f) {
    const float drho = 0.5f * (a.dw[0] + b.dw[0]);
    float dvavg[D], vavg[D];
    float dkin = 0, kin = 0;
#pragma unroll
    for (int d = 0; d < D; ++d) {
      dvavg[d] = 0.5f * (a.dw[1 + d] + b.dw[1 + d]);
      vavg[d] = R.v[d] + dvavg[d];
      dkin += R.v[d] * (a.dw[1 + d] + b.dw[1 + d]) + a.dw[1 + d] * b.dw[1 + d];
      kin += a.w[1 + d] * b.w[1 + d];
    }
    dkin *= 0.5f;
    kin *= 0.5f;
    const float dpavg = 0.5f * (a.dw[P] + b.dw[P]);
    const float vro = pick(R.v, o);
    const float F1r = R.rho * vro;
    const float d1 = R.rho * pick(dvavg, o) + drho * pick(vavg, o);
    f[0] = d1;
#pragma unroll
    for (int d = 0; d < D; ++d) f[1 + d] = d1 * vavg[d] + F1r * dvavg[d] + ((d == o) ? dpavg : 0.0f);
    const float dvao = pick(a.dw + 1, o), dvbo = pick(b.dw + 1, o);
    const float dpv = 0.5f * (R.p * (dvao + dvbo) + vro * (a.dw[P] + b.dw[P]) +
                              a.dw[P] * dvbo + b.dw[P] * dvao);
    f[P] = igm1 * (dpavg * pick(vavg, o) + R.p * pick(dvavg, o)) + d1 * kin + F1r * dkin + dpv;
  }

  static __host__ __device__ __forceinline__ void two_point(int kind, const RefState<D>& R,
                                                    const Node<D>& a, const Node<D>& b, int o,
                                                    float gamma, float igm1, float* f) {
    switch (kind) {
      case FLUX_RANOCHA: dranocha(R, a, b, o, igm1, f); break;
      case FLUX_SHIMA_ETAL: dshima(R, a, b, o, igm1, f); break;
      case FLUX_LLF: dllf(R, a, b, o, false, gamma, igm1, f); break;
      case FLUX_LLF_NAIVE: dllf(R, a, b, o, true, gamma, igm1, f); break;
      default: dcentral(R, a, b, o, gamma, igm1, f); break;
    }
  }
};

// float-float addition (hi, lo) + x -> normalised (hi, lo): TwoSum, then Fast2Sum
__device__ __forceinline__ float2 ff_add(float2 u, float x) {
  const float s = __fadd_rn(u.x, x);
  const float bp = __fsub_rn(s, u.x);
  const float e = __fadd_rn(__fsub_rn(u.x, __fsub_rn(s, bp)), __fsub_rn(x, bp));
  const float t = __fadd_rn(u.y, e);
  const float h = __fadd_rn(s, t);
  const float l = __fsub_rn(t, __fsub_rn(h, s));
  return make_float2(h, l);
}

template <int D, int N, int VI, int EPB>
struct MixedKernel {
  static constexpr int NV = D + 2;
  static constexpr int NN = Pow<N, D>::value;
  static constexpr int NF = NN / N;
  static constexpr int NT = EPB * NN;
  static constexpr int SP = EPB * NN + 1;
  static constexpr int NP = N * (N - 1) / 2;
  static constexpr int CHUNK = EPB * NN * NV;
  static constexpr int VOL_WEAK = D * NV * SP;
  static constexpr int VOL_FD = EPB * D * NF * NP * NV;
  static constexpr int VOL_FV = EPB * D * NF * (N - 1) * NV;
  static constexpr int VOL = VI == VI_WEAK ? VOL_WEAK : (VI == VI_FD ? VOL_FD : VOL_FD + VOL_FV);
  static constexpr int REFW = (sizeof(RefState<D>) + 3) / 4;  // floats per reference

  static constexpr size_t smem_bytes() {
    return sizeof(float2) * CHUNK + sizeof(float) * CHUNK  // state, u_tmp
           + sizeof(float) * (3 * NV * SP                  // du, dw, w (SoA)
                              + EPB * 2 * D * NF * NV      // face fluxes
                              + VOL                        // volume fluxes
                              + N * N + N                  // matrix, inverse weights
                              + EPB * REFW                 // references
                              + EPB * (D + 1) + 4 + 8);    // alpha, scalars, speed maxima
  }
};

template <int D, int N, int VI, int EPB>
__global__ void __launch_bounds__(EPB * Pow<N, D>::value)
    mixed_element_kernel(const MixedParams P, const MixedArgs A) {
  using K = MixedKernel<D, N, VI, EPB>;
  using Dv = Dev<D>;
  constexpr int NV = K::NV, NN = K::NN, NF = K::NF, NT = K::NT, SP = K::SP, NP = K::NP;
  constexpr int CHUNK = K::CHUNK;
  constexpr int PP = D + 1;

  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* s_u = reinterpret_cast<float2*>(smem_raw);
  float* s_tmp = reinterpret_cast<float*>(s_u + CHUNK);
  float* s_du = s_tmp + CHUNK;
  float* s_dw = s_du + NV * SP;
  float* s_w = s_dw + NV * SP;
  float* s_face = s_w + NV * SP;
  float* s_vol = s_face + EPB * 2 * D * NF * NV;
  float* s_fv = s_vol + K::VOL_FD;
  float* s_mat = s_vol + K::VOL;
  float* s_iw = s_mat + N * N;
  RefState<D>* s_ref = reinterpret_cast<RefState<D>*>(s_iw + N);
  float* s_alpha = reinterpret_cast<float*>(s_ref + EPB);
  float* s_scal = s_alpha + EPB;  // [0] stage time, [1] b dt, [2] a
  unsigned int* s_smax = reinterpret_cast<unsigned int*>(s_scal + 4);

  const int tid = threadIdx.x;
  const int slot = tid / NN;
  const int node = tid - slot * NN;
  const int64_t e0 = (int64_t)blockIdx.x * EPB;
  const int nel = (int)min((int64_t)EPB, P.nelements - e0);
  const bool active = slot < nel;
  const int64_t e = e0 + slot;
  const size_t gofs = (size_t)e0 * NN * NV;
  const int nval = nel * NN * NV;
  const float gamma = P.gamma, igm1 = P.inv_gamma_minus_one;

  if (A.mode == MODE_STAGE && A.clock->skip) {
    for (int k = tid; k < nval; k += NT) A.u_out[gofs + k] = A.u_in[gofs + k];
    return;
  }

  // ---- stage chunk, matrices, references --------------------------------------
  for (int k = tid; k < nval; k += NT) s_u[k] = __ldg(A.u_in + gofs + k);
  if (A.mode == MODE_STAGE) {
    for (int k = tid; k < nval; k += NT) s_tmp[k] = A.zero_tmp ? 0.0f : A.u_tmp[gofs + k];
  }
  for (int k = tid; k < N * N; k += NT) s_mat[k] = VI == VI_WEAK ? P.Dhat[k] : P.Dsplit[k];
  if (tid < N) s_iw[tid] = P.inv_weights[tid];
  if (tid < EPB * D) s_smax[tid] = 0u;
  if (tid == 0) {
    // the only FP64 arithmetic of the kernel: a few scalars per block
    if (A.mode == MODE_RHS) {
      s_scal[0] = (float)A.t_rhs;
      s_scal[1] = 0.0f;
    } else {
      const double dt = A.clock->dt;
      s_scal[0] = (float)(A.clock->t + A.c * dt);
      s_scal[1] = (float)(A.b * dt);
    }
    s_scal[2] = (float)A.a;
  }
  __syncthreads();
  if (active && node == 0) {
    float hi[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) hi[v] = s_u[slot * NN * NV + v].x;
    Dv::make_ref(hi, gamma, igm1, s_ref[slot]);
    if (VI == VI_HG) {
      float a = A.alpha_raw[e];
      if (P.alpha_smooth) {
#pragma unroll
        for (int dir = 0; dir < 2 * D; ++dir)
          a = fmaxf(a, 0.5f * A.alpha_raw[P.nbr[e * 2 * D + dir]]);
      }
      s_alpha[slot] = a;
      if (A.alpha_out) A.alpha_out[e] = a;
    }
  }
  __syncthreads();

  if (active) {
    float hi[NV], lo[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      const float2 x = s_u[(slot * NN + node) * NV + v];
      hi[v] = x.x;
      lo[v] = x.y;
    }
    Node<D> nd;
    Dv::make_node(hi, lo, s_ref[slot], gamma, nd);
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      s_du[v * SP + tid] = nd.du[v];
      s_dw[v * SP + tid] = nd.dw[v];
      s_w[v * SP + tid] = nd.w[v];
    }
  }
  __syncthreads();

  auto load_node = [&](int idx, Node<D>& n) {
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      n.du[v] = s_du[v * SP + idx];
      n.dw[v] = s_dw[v * SP + idx];
      n.w[v] = s_w[v * SP + idx];
    }
  };

  // ---- interface fluxes (deviation form, own element's reference) -----------
  for (int it = tid; it < nel * 2 * D * NF; it += NT) {
    const int sl = it / (2 * D * NF);
    const int rem = it - sl * (2 * D * NF);
    const int dir = rem / NF;
    const int fn = rem - dir * NF;
    const int d = dir >> 1;
    const int side = dir & 1;
    const int S = axis_stride<N>(d);
    const int base = line_base<N>(fn, d);
    const int own = base + (side ? (N - 1) * S : 0);
    const int nnode = base + (side ? 0 : (N - 1) * S);
    const int64_t nb = P.nbr[(e0 + sl) * 2 * D + dir];
    const RefState<D>& R = s_ref[sl];
    Node<D> no, nn_;
    load_node(sl * NN + own, no);
    {
      float hi[NV], lo[NV];
      const int64_t nbs = nb - e0;
      if (nbs >= 0 && nbs < nel) {
#pragma unroll
        for (int v = 0; v < NV; ++v) {
          const float2 x = s_u[((int)nbs * NN + nnode) * NV + v];
          hi[v] = x.x;
          lo[v] = x.y;
        }
      } else {
        const float2* p = A.u_in + ((size_t)nb * NN + nnode) * NV;
#pragma unroll
        for (int v = 0; v < NV; ++v) {
          const float2 x = __ldg(p + v);
          hi[v] = x.x;
          lo[v] = x.y;
        }
      }
      Dv::make_node(hi, lo, R, gamma, nn_);
    }
    float F[NV];
    if (side)
      Dv::two_point(P.surface_flux, R, no, nn_, d, gamma, igm1, F);
    else
      Dv::two_point(P.surface_flux, R, nn_, no, d, gamma, igm1, F);
#pragma unroll
    for (int v = 0; v < NV; ++v) s_face[((sl * 2 * D + dir) * NF + fn) * NV + v] = F[v];
  }

  // ---- volume fluxes -----------------------------------------------------------
  if (active) {
    const RefState<D>& R = s_ref[slot];
    if (VI == VI_WEAK) {
      Node<D> nd;
      load_node(tid, nd);
#pragma unroll
      for (int d = 0; d < D; ++d) {
        float f[NV];
        Dv::dflux(R, nd, d, gamma, igm1, f);
#pragma unroll
        for (int v = 0; v < NV; ++v) s_vol[(d * NV + v) * SP + tid] = f[v];
      }
    } else {
#pragma unroll
      for (int d = 0; d < D; ++d) {
        const int S = axis_stride<N>(d);
        const int i = axis_index<N>(node, d);
        const int line = line_index<N>(node, d);
        const int lb = line_base<N>(line, d);
        for (int p = i; p < NP; p += N) {
          int a = 0, q = p;
          while (q >= N - 1 - a) {
            q -= N - 1 - a;
            ++a;
          }
          const int b = a + 1 + q;
          Node<D> na, nb2;
          load_node(slot * NN + lb + a * S, na);
          load_node(slot * NN + lb + b * S, nb2);
          float F[NV];
          Dv::two_point(P.volume_flux, R, na, nb2, d, gamma, igm1, F);
#pragma unroll
          for (int v = 0; v < NV; ++v)
            s_vol[(((slot * D + d) * NF + line) * NP + p) * NV + v] = F[v];
        }
        if (VI == VI_HG && i < N - 1 && fabsf(s_alpha[slot]) > P.alpha_atol) {
          Node<D> na, nb2;
          load_node(tid, na);
          load_node(tid + S, nb2);
          float F[NV];
          Dv::two_point(P.fv_flux, R, na, nb2, d, gamma, igm1, F);
#pragma unroll
          for (int v = 0; v < NV; ++v)
            s_fv[(((slot * D + d) * NF + line) * (N - 1) + i) * NV + v] = F[v];
        }
      }
    }
  }
  __syncthreads();

  // ---- gather --------------------------------------------------------------------
  float du[NV];
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
          const float c = s_mat[i * N + l];
          const int src = slot * NN + lb + l * S;
#pragma unroll
          for (int v = 0; v < NV; ++v) du[v] = fmaf(c, s_vol[(d * NV + v) * SP + src], du[v]);
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
          const float c = s_mat[i * N + l];
          const float* F = s_vol + (((slot * D + d) * NF + line) * NP + p) * NV;
#pragma unroll
          for (int v = 0; v < NV; ++v) du[v] = fmaf(c, F[v], du[v]);
        }
      }
      if (VI == VI_HG) {
        const float alpha = s_alpha[slot];
        if (fabsf(alpha) > P.alpha_atol) {
          float fv[NV];
#pragma unroll
          for (int v = 0; v < NV; ++v) fv[v] = 0;
#pragma unroll
          for (int d = 0; d < D; ++d) {
            const int i = axis_index<N>(node, d);
            const int line = line_index<N>(node, d);
            const float iw = s_iw[i];
            const float* Fb = s_fv + ((slot * D + d) * NF + line) * (N - 1) * NV;
#pragma unroll
            for (int v = 0; v < NV; ++v) {
              const float fr = i < N - 1 ? Fb[i * NV + v] : 0.0f;
              const float fl = i > 0 ? Fb[(i - 1) * NV + v] : 0.0f;
              fv[v] += iw * (fr - fl);
            }
          }
#pragma unroll
          for (int v = 0; v < NV; ++v) du[v] = (1.0f - alpha) * du[v] + alpha * fv[v];
        }
      }
    }
    const float factor = s_iw[0];
#pragma unroll
    for (int d = 0; d < D; ++d) {
      const int i = axis_index<N>(node, d);
      const int fn = line_index<N>(node, d);
      if (i == 0) {
        const float* F = s_face + ((slot * 2 * D + 2 * d) * NF + fn) * NV;
#pragma unroll
        for (int v = 0; v < NV; ++v) du[v] = du[v] - F[v] * factor;
      }
      if (i == N - 1) {
        const float* F = s_face + ((slot * 2 * D + 2 * d + 1) * NF + fn) * NV;
#pragma unroll
        for (int v = 0; v < NV; ++v) du[v] = du[v] + F[v] * factor;
      }
    }
    const float jfac = -P.inv_jac[e];
#pragma unroll
    for (int v = 0; v < NV; ++v) du[v] *= jfac;
    if (P.source == SRC_CONVERGENCE_TEST) {
      float x[D], s[NV];
      const float* xl = P.xline + (size_t)e * D * N;
#pragma unroll
      for (int d = 0; d < D; ++d) x[d] = xl[d * N + axis_index<N>(node, d)];
      Euler<D, float>::source_convergence(x, s_scal[0], gamma, s);
#pragma unroll
      for (int v = 0; v < NV; ++v) du[v] += s[v];
    }
  }
  if (A.mode == MODE_RHS) {
    __syncthreads();
    // du in FP64 through the (now free) float state buffer as two halves
    double* s_d = reinterpret_cast<double*>(s_u);
    if (active) {
#pragma unroll
      for (int v = 0; v < NV; ++v) s_d[tid * NV + v] = (double)du[v];
    }
    __syncthreads();
    for (int k = tid; k < nval; k += NT) A.du_out[gofs + k] = s_d[k];
    return;
  }

  // ---- 2N stage update in float-float ------------------------------------------
  const float bdt = s_scal[1];
  const float a_s = s_scal[2];
  bool bad = false;
  if (active) {
    float hi[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      const int k = tid * NV + v;
      const float ut = du[v] - s_tmp[k] * a_s;
      s_tmp[k] = ut;
      const float2 un = ff_add(s_u[k], ut * bdt);
      s_u[k] = un;
      hi[v] = un.x;
      bad |= !(un.x == un.x);
    }
    if (A.speed_bits) {
      float w[NV];
      Euler<D, float>::cons2prim(hi, w, gamma);
      const float cs = sqrtf(gamma * w[PP] / w[0]);
      bad |= !(w[0] > 0.0f) || !(w[PP] > 0.0f);
#pragma unroll
      for (int d = 0; d < D; ++d) {
        const float lam = fabsf(w[1 + d]) + cs;
        if (lam == lam) atomicMax(&s_smax[slot * D + d], __float_as_uint(lam));
      }
    }
  }
  if (bad) atomicOr(A.status, 1);
  __syncthreads();
  for (int k = tid; k < nval; k += NT) {
    A.u_out[gofs + k] = s_u[k];
    A.u_tmp[gofs + k] = s_tmp[k];
  }
  if (A.speed_bits && active && node == 0) {
    float sum = 0;
#pragma unroll
    for (int d = 0; d < D; ++d) sum += __uint_as_float(s_smax[slot * D + d]);
    const float sp = P.inv_jac[e] * sum;
    if (sp == sp) atomicMax(A.speed_bits, (unsigned long long)__double_as_longlong((double)sp));
  }
}

}  // namespace tg
