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
//    primitives of the mean `hi` of two opposite corner nodes), using algebra
//    that involves only node deviations from w_e.  Those are formed from the
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
#include "tg_tcgen05.cuh"

namespace tg {

// FP32 equation-of-state constants, each rounded once from the FP64 gamma.
// gamma - 1 multiplies every pressure and pressure deviation; rounded to a
// float it is off by up to 3e-8 in the same direction everywhere, which acts
// like a slightly different gas and shifts the whole solution coherently over
// a long run, so it is carried as a float-float pair (hi + lo).  For gamma =
// 1.4 the other two are exact (2.5 and 3.5).
struct EosF {
  float gamma, gm1, gm1_lo, igm1, gigm1;  // gamma, gamma-1 (hi, lo), 1/(gamma-1), gamma/(gamma-1)
  __host__ __device__ __forceinline__ float pressure(float x) const {
    return fmaf(gm1_lo, x, gm1 * x);  // (gamma - 1) x with one rounding
  }
};

struct MixedParams {
  int64_t nelements;
  float gamma, inv_gamma_minus_one;
  EosF eos;                 // the same constants, consistent for the flux algebra
  float inv_weights[MAXN];
  float Dhat[MAXN * MAXN];
  float Dsplit[MAXN * MAXN];
  float Vinv[MAXN * MAXN];
  int32_t volume_flux, surface_flux, fv_flux, source;
  float alpha_max, alpha_min, alpha_atol, hg_threshold, hg_parameter_s;
  int32_t alpha_smooth;
  int32_t hg_variable;      // indicator variable: 0 density_pressure, 1 density
  const int32_t* nbr;       // [E][2D]
  const float* inv_jac;     // [E]
  const float* xline;       // [E][D][N] or null (unused by the stage kernel)
  // source phase pi (sum_d x_d - t) as float-float sin/cos parts
  // (sin_hi, cos_hi, sin_lo, cos_lo): of the first node of each element, and
  // of each node's offset from the first node (one table per element size)
  const float4* sc0;        // [E]
  const float4* scn;        // [size class][NN]
  const int8_t* scls;       // [E] size class of each element
  // Faces without a conforming neighbour have nbr = -1 - b.  b < nbc: a
  // boundary face of a non-periodic mesh; ghost[b][face node][v] holds, for
  // the current stage, the Dirichlet state (float-float) or, on slip walls
  // (bc), the wall flux (float-float), written by a pre-pass from the stage's
  // input state.  b >= nbc: a mortar face; ghost[b] holds its flux from the
  // mortar pre-pass, and mnbr[b - nbc] the elements across it.
  int32_t bc[6];            // per direction, BoundaryKind
  int32_t has_direct;       // any face whose flux is given (slip wall, mortar)
  int32_t nbc;
  const float2* ghost;      // [B][NF][NV]
  const int32_t* mnbr;      // [mortar face slot][4]
};

struct MixedArgs {
  const float2* u_in;       // float-float state (hi, lo) per value
  float2* u_out;            // MODE_STAGE
  double* du_out;           // MODE_RHS (FP64 du, Trixi layout)
  float* u_tmp;             // MODE_STAGE
  const float* alpha_raw;   // VI_HG
  const float* alpha_smoothed;  // VI_HG, persistent 2D kernel: alpha_raw after apply_smoothing!
  // VI_HG, persistent 2D kernel on a mesh without mortars: alpha_smoothed
  // holds the raw factors and the kernel applies apply_smoothing! itself,
  // from the face neighbours' raw factors gathered with the face traces
  int32_t alpha_gather;
  float* alpha_out;         // VI_HG (optional)
  // MODE_STAGE (optional): rho*p of u_out per node (FP32 on the hi parts, as
  // the indicators compute it), read by the next stage's indicator instead of
  // the whole state
  float* rp_out;
  const Clock* clock;
  unsigned long long* speed_bits;
  int32_t* status;
  double t_rhs;
  double a, b, c;           // 2N coefficients of the stage
  int32_t mode;
  int32_t zero_tmp;
  int32_t stage;            // MODE_STAGE: index into the clock's per-stage phase
  float sin_t, cos_t;       // MODE_RHS: sin/cos(pi t), float-float
  float sin_tl, cos_tl;
};

// ---------------------------------------------------------------------------
// Reference state of an element and node deviations
// ---------------------------------------------------------------------------
template <int D>
struct RefState {
  float rho, v[D], p;   // reference primitives w_e
  float q, rq;          // q = rho/p and its residual rho - q p (exact by FMA)
  float hi[D + 2];      // conservative reference (mean hi of opposite corners)
  float r[D + 2];       // hi - cons(w_e): momentum residual exact, energy to FP32
};

template <int D>
struct Node {
  float du[D + 2];      // conservative deviation from cons(w_e)
  float dw[D + 2];      // primitive deviation (drho, dv_1..dv_D, dp)
  float w[D + 2];       // full primitives
  float dq;             // deviation of rho/p from the reference q
  float vo, dvo;        // velocity along the current direction and its deviation
};

template <int D>
struct Dev {
  static constexpr int NV = D + 2, P = D + 1;

  static __host__ __device__ __forceinline__ void make_ref(const float* hi, const EosF& eos,
                                                   RefState<D>& R) {
    const float igm1 = eos.igm1;
    R.rho = hi[0];
    const float irho = 1.0f / R.rho;
    float ke = 0;
#pragma unroll
    for (int d = 0; d < D; ++d) {
      R.v[d] = hi[1 + d] * irho;
      ke += hi[1 + d] * R.v[d];
    }
    R.p = eos.pressure(hi[P] - 0.5f * ke);
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
                                                    const RefState<D>& R, const EosF& eos, Node<D>& n) {
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
    const float dp = eos.pressure(n.du[P] - 0.5f * dkin);
    n.dw[0] = drho;
    n.w[0] = rho;
    n.dw[P] = dp;
    n.w[P] = R.p + dp;
    n.dq = (R.rq + drho - R.q * dp) / n.w[P];
  }

  // Conservative deviation of a node from its float-float state (as make_node).
  static __host__ __device__ __forceinline__ void node_du(const float2* x, const RefState<D>& R,
                                                  float* du) {
#pragma unroll
    for (int v = 0; v < NV; ++v) du[v] = ((x[v].x - R.hi[v]) + x[v].y) + R.r[v];
  }

  // A boundary flux given as float-float values (the slip-wall flux of the
  // pre-pass) as a deviation from the reference state's physical flux along o.
  static __device__ __forceinline__ void wall_flux(const RefState<D>& R, const float2* fw, int o,
                                                   float vro, const EosF& eos, float* f) {
    const float m = R.rho * vro;
    float v2 = 0;
#pragma unroll
    for (int d = 0; d < D; ++d) v2 += R.v[d] * R.v[d];
    f[0] = (fw[0].x - m) + fw[0].y;
#pragma unroll
    for (int d = 0; d < D; ++d)
      f[1 + d] = (fw[1 + d].x - ((d == o) ? fmaf(m, R.v[d], R.p) : m * R.v[d])) + fw[1 + d].y;
    f[P] = (fw[P].x - ((R.p * eos.igm1 + 0.5f * R.rho * v2) + R.p) * vro) + fw[P].y;
  }

  // Full primitives from deviations (nodes stored as dw + dq only).
  static __host__ __device__ __forceinline__ void complete(const RefState<D>& R, Node<D>& n) {
    n.w[0] = R.rho + n.dw[0];
#pragma unroll
    for (int d = 0; d < D; ++d) n.w[1 + d] = R.v[d] + n.dw[1 + d];
    n.w[P] = R.p + n.dw[P];
  }

  static __host__ __device__ __forceinline__ float pick(const float* a, int o) {
    float r = a[0];
#pragma unroll
    for (int d = 1; d < D; ++d) r = (o == d) ? a[d] : r;
    return r;
  }

  // Velocity components along direction o, selected once per node and line
  // (the fluxes below use n.vo / n.dvo and the reference's vro = v_ref[o]).
  static __host__ __device__ __forceinline__ void orient(Node<D>& n, int o) {
    n.vo = pick(n.w + 1, o);
    n.dvo = pick(n.dw + 1, o);
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
                                                float vro, const EosF& eos, float* f) {
    const float vo = a.vo, dvo = a.dvo;
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
    f[P] = d1 * (0.5f * k) + F1r * dk + eos.gigm1 * (a.dw[P] * vo + R.p * dvo);
  }

  static __host__ __device__ __forceinline__ void dcentral(const RefState<D>& R, const Node<D>& a,
                                                   const Node<D>& b, int o, float vro,
                                                   const EosF& eos, float* f) {
    float fa[NV], fb[NV];
    dflux(R, a, o, vro, eos, fa);
    dflux(R, b, o, vro, eos, fb);
#pragma unroll
    for (int v = 0; v < NV; ++v) f[v] = 0.5f * (fa[v] + fb[v]);
  }

  static __host__ __device__ __forceinline__ void dllf(const RefState<D>& R, const Node<D>& a,
                                               const Node<D>& b, int o, float vro, bool naive,
                                               const EosF& eos, float* f) {
    dcentral(R, a, b, o, vro, eos, f);
    const float ca = sqrtf(eos.gamma * a.w[P] / a.w[0]);
    const float cb = sqrtf(eos.gamma * b.w[P] / b.w[0]);
    const float va = fabsf(a.vo), vb = fabsf(b.vo);
    const float lam = naive ? fmaxf(va, vb) + fmaxf(ca, cb) : fmaxf(va + ca, vb + cb);
#pragma unroll
    for (int v = 0; v < NV; ++v) f[v] = f[v] + (-0.5f * lam * (b.du[v] - a.du[v]));
  }

  // flux_ranocha(a, b) - f(w_ref)
  static __host__ __device__ __forceinline__ void dranocha(const RefState<D>& R, const Node<D>& a,
                                                   const Node<D>& b, int o, float vro, const EosF& eos,
                                                   float* f) {
    const float igm1 = eos.igm1;
    const float drho_ln = dev_ln_mean(R.rho, a.dw[0], b.dw[0], a.w[0], b.w[0]);
    // q = rho / p relative to R.q (node deviations a.dq, b.dq from make_node)
    const float dq_ln = dev_ln_mean(R.q, a.dq, b.dq, R.q + a.dq, R.q + b.dq);
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
    const float F1r = R.rho * vro;
    const float dvavgo = 0.5f * (a.dvo + b.dvo);
    const float d1 = R.rho * dvavgo + drho_ln * (vro + dvavgo);
    f[0] = d1;
#pragma unroll
    for (int d = 0; d < D; ++d) f[1 + d] = d1 * vavg[d] + F1r * dvavg[d] + ((d == o) ? dpavg : 0.0f);
    float vsq = 0;
#pragma unroll
    for (int d = 0; d < D; ++d) vsq += a.w[1 + d] * b.w[1 + d];
    const float H = 0.5f * vsq + igm1 / q_ln;
    const float dH = dvsq + igm1 * (R.rq - R.p * dq_ln) / (R.rho * q_ln);
    const float dvao = a.dvo, dvbo = b.dvo;
    const float dpv = 0.5f * (R.p * (dvao + dvbo) + vro * (a.dw[P] + b.dw[P]) +
                              a.dw[P] * dvbo + b.dw[P] * dvao);
    f[P] = d1 * H + F1r * dH + dpv;
  }

  // flux_shima_etal(a, b) - f(w_ref)
  static __host__ __device__ __forceinline__ void dshima(const RefState<D>& R, const Node<D>& a,
                                                 const Node<D>& b, int o, float vro, const EosF& eos,
                                                 float* f) {
    const float igm1 = eos.igm1;
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
    const float F1r = R.rho * vro;
    const float dvavgo = 0.5f * (a.dvo + b.dvo);
    const float vavgo = vro + dvavgo;
    const float d1 = R.rho * dvavgo + drho * vavgo;
    f[0] = d1;
#pragma unroll
    for (int d = 0; d < D; ++d) f[1 + d] = d1 * vavg[d] + F1r * dvavg[d] + ((d == o) ? dpavg : 0.0f);
    const float dvao = a.dvo, dvbo = b.dvo;
    const float dpv = 0.5f * (R.p * (dvao + dvbo) + vro * (a.dw[P] + b.dw[P]) +
                              a.dw[P] * dvbo + b.dw[P] * dvao);
    f[P] = igm1 * (dpavg * vavgo + R.p * dvavgo) + d1 * kin + F1r * dkin + dpv;
  }

  // KIND >= 0 selects the flux at compile time; KIND < 0 dispatches on `kind`.
  // flux_chandrashekar(a, b) - f(w_ref).  With beta = q / 2 (q = rho / p) its
  // energy flux is f1 (igm1 / q_ln + v_a . v_b / 2) + p_mean v_avg,o: the
  // enthalpy term of flux_ranocha, with p_mean = rho_avg / q_avg in place of the
  // arithmetic mean pressure, so p_mean - p_ref = (rq_ref + drho_avg -
  // p_ref dq_avg) / q_avg in deviations.
  static __host__ __device__ __forceinline__ void dchandrashekar(const RefState<D>& R,
                                                         const Node<D>& a, const Node<D>& b,
                                                         int o, float vro, const EosF& eos,
                                                         float* f) {
    const float igm1 = eos.igm1;
    const float drho_ln = dev_ln_mean(R.rho, a.dw[0], b.dw[0], a.w[0], b.w[0]);
    const float dq_ln = dev_ln_mean(R.q, a.dq, b.dq, R.q + a.dq, R.q + b.dq);
    const float q_ln = R.q + dq_ln;
    const float dq_avg = 0.5f * (a.dq + b.dq);
    const float dp_mean = (R.rq + 0.5f * (a.dw[0] + b.dw[0]) - R.p * dq_avg) / (R.q + dq_avg);
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
    const float F1r = R.rho * vro;
    const float dvavgo = 0.5f * (a.dvo + b.dvo);
    const float d1 = R.rho * dvavgo + drho_ln * (vro + dvavgo);
    f[0] = d1;
#pragma unroll
    for (int d = 0; d < D; ++d) f[1 + d] = d1 * vavg[d] + F1r * dvavg[d] + ((d == o) ? dp_mean : 0.0f);
    const float H = 0.5f * vsq + igm1 / q_ln;
    const float dH = dvsq + igm1 * (R.rq - R.p * dq_ln) / (R.rho * q_ln);
    f[P] = d1 * H + F1r * dH + (R.p * dvavgo + dp_mean * (vro + dvavgo));
  }

  // flux_hlle(a, b) - f(w_ref): FluxHLL with min_max_speed_einfeldt
  // (numerical_fluxes.jl:422-457, compressible_euler_2d.jl:1925-1963).  The
  // HLL combination is linear in the two physical fluxes, so it is exact in
  // their deviations and in the conservative deviations b.du - a.du.
  static __host__ __device__ __forceinline__ void dhlle(const RefState<D>& R, const Node<D>& a,
                                                const Node<D>& b, int o, float vro,
                                                const EosF& eos, float* f) {
    const float g = eos.gamma;
    const float rl = a.w[0], rr = b.w[0], pl = a.w[P], pr = b.w[P];
    const float cl = sqrtf(g * pl / rl), cr = sqrtf(g * pr / rr);
    const float sl = sqrtf(rl), sr = sqrtf(rr), iss = 1.0f / (sl + sr);
    float vroe2 = 0, kl = 0, kr = 0;
#pragma unroll
    for (int d = 0; d < D; ++d) {
      const float vr = (sl * a.w[1 + d] + sr * b.w[1 + d]) * iss;
      vroe2 += vr * vr;
      kl += a.w[1 + d] * a.w[1 + d];
      kr += b.w[1 + d] * b.w[1 + d];
    }
    const float vroe_o = (sl * a.vo + sr * b.vo) * iss;
    const float Hl = (pl * eos.gigm1 + 0.5f * rl * kl) / rl;
    const float Hr = (pr * eos.gigm1 + 0.5f * rr * kr) / rr;
    const float c_roe = sqrtf(eos.pressure((sl * Hl + sr * Hr) * iss - 0.5f * vroe2));
    const float beta = sqrtf(0.5f * eos.gm1 / g);
    const float lmin = fminf(fminf(vroe_o - c_roe, a.vo - beta * cl), 0.0f);
    const float lmax = fmaxf(fmaxf(vroe_o + c_roe, b.vo + beta * cr), 0.0f);
    if (lmin >= 0.0f && lmax >= 0.0f) {
      dflux(R, a, o, vro, eos, f);
      return;
    }
    if (lmax <= 0.0f && lmin <= 0.0f) {
      dflux(R, b, o, vro, eos, f);
      return;
    }
    float fb[NV];
    dflux(R, a, o, vro, eos, f);
    dflux(R, b, o, vro, eos, fb);
    const float id = 1.0f / (lmax - lmin);
    const float ca = lmax * id, cb = lmin * id, cd = lmin * lmax * id;
#pragma unroll
    for (int v = 0; v < NV; ++v) f[v] = ca * f[v] - cb * fb[v] + cd * (b.du[v] - a.du[v]);
  }

  // flux_hllc(a, b) - f(w_ref) (compressible_euler_2d.jl:1720-1816, 3d.jl:1423-1541).
  // Signal speeds from the full primitives (they only weight the terms).  The
  // outer branches are physical-flux deviations; the star-state correction is
  // written in terms of SStar - v of the upwind side, which comes from the
  // pressure and velocity deviations without cancellation:
  //   SStar - v_L = (p_R - p_L + rho_R sMu_R (v_L - v_R)) / den,
  //   SStar - v_R = (p_R - p_L + rho_L sMu_L (v_L - v_R)) / den,
  //   den = rho_L sMu_L - rho_R sMu_R,
  // and rho* - rho = rho (SStar - v) / (S - SStar), so every correction term is
  // proportional to SStar - v.
  static __host__ __device__ __forceinline__ void dhllc(const RefState<D>& R, const Node<D>& a,
                                                const Node<D>& b, int o, float vro,
                                                const EosF& eos, float* f) {
    const float g = eos.gamma;
    const float rl = a.w[0], rr = b.w[0], pl = a.w[P], pr = b.w[P];
    const float cl = sqrtf(g * pl / rl), cr = sqrtf(g * pr / rr);
    const float sl = sqrtf(rl), sr = sqrtf(rr), iss = 1.0f / (sl + sr);
    const float vel_L = a.vo, vel_R = b.vo;
    const float vel_roe = (sl * vel_L + sr * vel_R) * iss;
    float vroe2 = 0, kl = 0, kr = 0;
#pragma unroll
    for (int d = 0; d < D; ++d) {
      const float vroe = sl * a.w[1 + d] + sr * b.w[1 + d];
      vroe2 += vroe * vroe;
      kl += a.w[1 + d] * a.w[1 + d];
      kr += b.w[1 + d] * b.w[1 + d];
    }
    const float El = pl * eos.igm1 + 0.5f * rl * kl, Er = pr * eos.igm1 + 0.5f * rr * kr;
    const float H_roe = (sl * ((El + pl) / rl) + sr * ((Er + pr) / rr)) * iss;
    const float c_roe = sqrtf(eos.pressure(H_roe - 0.5f * vroe2 * iss * iss));
    const float Ssl = fminf(vel_L - cl, vel_roe - c_roe);
    const float Ssr = fmaxf(vel_R + cr, vel_roe + c_roe);
    if (Ssl >= 0.0f) {
      dflux(R, a, o, vro, eos, f);
      return;
    }
    if (Ssr <= 0.0f) {
      dflux(R, b, o, vro, eos, f);
      return;
    }
    const float sMu_L = Ssl - vel_L, sMu_R = Ssr - vel_R;
    const float iden = 1.0f / (rl * sMu_L - rr * sMu_R);
    const float dv = a.dvo - b.dvo;     // v_L - v_R
    const float dp = b.dw[P] - a.dw[P];  // p_R - p_L
    const float ds_L = (dp + rr * sMu_R * dv) * iden;
    const float SStar = vel_L + ds_L;
    const bool left = SStar >= 0.0f;
    const Node<D>& X = left ? a : b;
    const float S = left ? Ssl : Ssr, sMu = left ? sMu_L : sMu_R;
    const float ds = left ? ds_L : (dp + rl * sMu_L * dv) * iden;
    const float rho = X.w[0], vel = X.vo;
    const float dr = rho * ds / (S - SStar);  // rho* - rho
    const float rs = rho + dr;
    const float e = (left ? El : Er) / rho;
    dflux(R, X, o, vro, eos, f);
    f[0] += S * dr;
#pragma unroll
    for (int d = 0; d < D; ++d) f[1 + d] += S * ((d == o) ? fmaf(rs, ds, vel * dr) : X.w[1 + d] * dr);
    f[P] += S * (e * dr + rs * ds * (SStar + X.w[P] / (rho * sMu)));
  }

  template <int KIND>
  static __host__ __device__ __forceinline__ void flux2(int kind, const RefState<D>& R,
                                                         const Node<D>& a, const Node<D>& b, int o,
                                                         float vro, const EosF& eos, float* f) {
    if constexpr (KIND == FLUX_RANOCHA) dranocha(R, a, b, o, vro, eos, f);
    else if constexpr (KIND == FLUX_SHIMA_ETAL) dshima(R, a, b, o, vro, eos, f);
    else if constexpr (KIND == FLUX_LLF) dllf(R, a, b, o, vro, false, eos, f);
    else if constexpr (KIND == FLUX_LLF_NAIVE) dllf(R, a, b, o, vro, true, eos, f);
    else if constexpr (KIND == FLUX_CENTRAL) dcentral(R, a, b, o, vro, eos, f);
    else if constexpr (KIND == FLUX_HLLC) dhllc(R, a, b, o, vro, eos, f);
    else if constexpr (KIND == FLUX_CHANDRASHEKAR) dchandrashekar(R, a, b, o, vro, eos, f);
    else if constexpr (KIND == FLUX_HLLE) dhlle(R, a, b, o, vro, eos, f);
    else two_point(kind, R, a, b, o, vro, eos, f);
  }

  static __host__ __device__ __forceinline__ void two_point(int kind, const RefState<D>& R,
                                                    const Node<D>& a, const Node<D>& b, int o,
                                                    float vro, const EosF& eos, float* f) {
    switch (kind) {
      case FLUX_RANOCHA: dranocha(R, a, b, o, vro, eos, f); break;
      case FLUX_SHIMA_ETAL: dshima(R, a, b, o, vro, eos, f); break;
      case FLUX_LLF: dllf(R, a, b, o, vro, false, eos, f); break;
      case FLUX_LLF_NAIVE: dllf(R, a, b, o, vro, true, eos, f); break;
      case FLUX_HLLC: dhllc(R, a, b, o, vro, eos, f); break;
      case FLUX_CHANDRASHEKAR: dchandrashekar(R, a, b, o, vro, eos, f); break;
      case FLUX_HLLE: dhlle(R, a, b, o, vro, eos, f); break;
      default: dcentral(R, a, b, o, vro, eos, f); break;
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

// (ah + al)(bh + bl) + (ch + cl)(dh + dl) as a normalised float-float pair:
// exact products and TwoSum of the leading terms, cross terms added to the
// low part (relative error a few units of 2^-46).  The _rn intrinsics keep
// the compiler from contracting the error-free transformations into FMAs.
__device__ __forceinline__ float2 ff_dot2(float ah, float al, float bh, float bl, float ch, float cl,
                                          float dh, float dl) {
  const float p = __fmul_rn(ah, bh), q = __fmul_rn(ch, dh);
  const float ep = fmaf(ah, bh, -p), eq = fmaf(ch, dh, -q);
  const float s = __fadd_rn(p, q);
  const float bp = __fsub_rn(s, p);
  const float es = __fadd_rn(__fsub_rn(p, __fsub_rn(s, bp)), __fsub_rn(q, bp));
  const float lo = es + ep + eq + fmaf(ah, bl, fmaf(al, bh, fmaf(ch, dl, cl * dh)));
  const float hi = __fadd_rn(s, lo);
  return make_float2(hi, __fsub_rn(lo, __fsub_rn(hi, s)));
}

// cp.async (sm_80+ asynchronous global->shared copies) helpers
__device__ __forceinline__ void cp_async8(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async4(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;" ::: "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_all;\n" ::: "memory");
}

// Thread layout: one thread per (direction, line) of each element, lines
// ordered direction-major so that a warp works on one direction.  A line
// thread evaluates the N(N-1)/2 two-point fluxes of its line (or the N
// physical fluxes of the weak form, and the subcell fluxes of the HG blend)
// and its two face fluxes, accumulating the line's N nodal contributions in
// registers; the D partial sums per node meet once in shared memory.  All
// global reads of a block (state chunk, u_tmp chunk and the neighbour traces
// of faces between blocks) are issued up front as cp.async copies.
// Position of node n of block slot `slot` inside one SoA field of the node
// arrays (for 3D polydeg 3, the production case, see pos()).
template <int D, int N, int EPB>
struct NodeLayout {
  static constexpr int NN = Pow<N, D>::value;
  // polydeg 3: swizzled layouts whose x-lines are 4 contiguous, 16-byte
  // aligned nodes (read and written as float4)
  static constexpr bool PADDED = N == 4;
  static constexpr int SS = D == 3 && PADDED ? 80 : NN;
  static constexpr int FS = PADDED ? EPB * SS : EPB * NN + 1;  // field stride
  static __host__ __device__ __forceinline__ int pos(int slot, int n) {
    if constexpr (D == 3 && PADDED) {
      // 3D: an XOR swizzle of bits 2-3 of the node index by bits 4-5 (a
      // permutation of each element's 64 nodes) with an 80-float element
      // stride.  A warp holds 16 lines of one direction of two elements: with
      // it the node-field reads and partial-sum writes of x-lines (float4), y-
      // and z-lines (scalar) and the node phase (32 consecutive nodes) each
      // take one shared-memory wavefront.
      return slot * SS + (n ^ (((n >> 4) & 1) << 2) ^ (((n >> 5) & 1) << 3));
    } else if constexpr (PADDED) {
      // 2D: the y index (bits 2-3 of the node) XORed with bits 1-2 of the
      // element slot.  A warp holds the 4 lines of one direction of 8
      // elements: x-lines read 8 x 4 distinct 16-byte groups, y-lines (node
      // line + 4 a) land in 32 distinct banks, the node phase permutes within
      // each element.
      return slot * SS + (n ^ (((slot >> 1) & 3) << 2));
    } else {
      return slot * SS + n;
    }
  }
};

template <int D, int N, int VI, int EPB>
struct MixedKernel {
  static constexpr int NV = D + 2;
  static constexpr int NN = Pow<N, D>::value;
  static constexpr int NF = NN / N;          // lines per direction = nodes per face
  static constexpr int L = D * NF;           // lines per element
  static constexpr int NT = EPB * L;         // threads per block
  static constexpr int SP = NodeLayout<D, N, EPB>::FS;  // field stride of node arrays
  // node fields: dw[NV], dq and, for shock capturing (whose subcell and
  // surface Lax-Friedrichs fluxes need them at every node), du[NV]
  static constexpr int NFLD = NV + 1 + (VI == VI_HG ? NV : 0);
  static constexpr int CHUNK = EPB * NN * NV;
  static constexpr int FACE = EPB * 2 * D * NF * NV;  // neighbour traces (float2)
  static constexpr int REFW = (sizeof(RefState<D>) + 3) / 4;
  static constexpr int MINB = NT <= 192 ? 4 : (NT <= 256 ? 3 : 1);  // resident blocks per SM

  static constexpr int PADF = (CHUNK + FACE) & 1;  // keeps node fields 16-byte aligned

  static constexpr size_t smem_bytes() {
    return sizeof(float2) * (CHUNK + FACE + PADF)               // state, traces
           + sizeof(float) * (NFLD * SP + D * NV * SP               // node fields, partial du
                              + EPB * REFW + EPB * 8 + 8            // references, per element
                              + EPB * D                             // speed maxima
                              + N * N + N + 4)                      // matrix, inverse weights
           + 16;                                                    // staging mbarrier
  }
};

template <int D>
struct SourceMMS {
  // source_terms_convergence_test, compressible_euler_2d.jl:116-145, 3d.jl:127-150,
  // given sin/cos of the phase omega (x+y(+z)-t)
  static __device__ __forceinline__ void eval(float si, float co, const EosF& eos, float* s) {
    // A omega = 0.1 pi as a float-float pair: one rounded constant would bias
    // the source by the same relative amount at every node and stage
    constexpr double AW = 0.1 * 3.14159265358979323846;
    constexpr float aw_hi = (float)AW;
    constexpr float aw_lo = (float)(AW - (double)aw_hi);
    const float rho = 2.0f + 0.1f * si;
    const float rho_x = fmaf(co, aw_lo, co * aw_hi);
    if (D == 2) {
      const float tmp = eos.pressure(2.0f * rho - 1.0f);
      s[0] = rho_x;
      s[1] = rho_x * (1.0f + tmp);
      s[2] = s[1];
      s[D + 1] = 2.0f * rho_x * (rho + tmp);
    } else {
      const float tmp = eos.pressure(2.0f * rho - 1.5f);
      s[0] = 2.0f * rho_x;
      s[1] = rho_x * (2.0f + tmp);
      s[2] = s[1];
      s[D] = s[1];
      s[D + 1] = rho_x * (4.0f * rho + 3.0f * tmp);
    }
  }
};

template <int D, int N, int VI, int VF, int SF, int EPB, bool DIRECT = false>
__device__ __forceinline__ void mixed_line(const MixedParams& P, const RefState<D>& R,
                                           const float2* s_u, const float2* s_fu,
                                           const float* s_nd, float* s_part, const float* s_mat,
                                           const float* s_iw, float alpha, int slot, int line,
                                           int dd, int64_t e, int64_t e0, int nel,
                                           const int32_t* nbr_row) {
  using K = MixedKernel<D, N, VI, EPB>;
  using Lay = NodeLayout<D, N, EPB>;
  using Dv = Dev<D>;
  constexpr int NV = K::NV, NN = K::NN, SP = K::SP, NF = K::NF;
  const EosF& eos = P.eos;
  const int S = axis_stride<N>(dd);
  const int lb = line_base<N>(line, dd);
  const float vro = Dv::pick(R.v, dd);
  // conservative deviations at every node: for the Lax-Friedrichs jumps of the
  // subcell fluxes and of a Lax-Friedrichs volume flux (the weak form's volume
  // term is the physical flux: its face nodes get them below)
  constexpr bool NEED_DU =
      VI == VI_HG || (VI != VI_WEAK && (VF < 0 || VF == FLUX_LLF || VF == FLUX_LLF_NAIVE));
  // node a of the line sits at field position pos(slot, lb + a S)
  const bool vec4 = Lay::PADDED && dd == 0;  // x-line: 4 contiguous, aligned nodes
  Node<D> nd[N];
  {
    constexpr int NLOAD = K::NFLD;  // dw, dq (and du for shock capturing)
#pragma unroll
    for (int f = 0; f < NLOAD; ++f) {
      float x[N];
      if constexpr (N == 4) {
        if (vec4) {
          const float4 q = *reinterpret_cast<const float4*>(s_nd + f * SP + Lay::pos(slot, lb));
          x[0] = q.x;
          x[1] = q.y;
          x[2] = q.z;
          x[3] = q.w;
        } else {
#pragma unroll
          for (int a = 0; a < N; ++a) x[a] = s_nd[f * SP + Lay::pos(slot, lb + a * S)];
        }
      } else {
#pragma unroll
        for (int a = 0; a < N; ++a) x[a] = s_nd[f * SP + Lay::pos(slot, lb + a * S)];
      }
#pragma unroll
      for (int a = 0; a < N; ++a) {
        if (f < NV)
          nd[a].dw[f] = x[a];
        else if (f == NV)
          nd[a].dq = x[a];
        else
          nd[a].du[f - NV - 1] = x[a];
      }
    }
#pragma unroll
    for (int a = 0; a < N; ++a) {
      Dv::complete(R, nd[a]);
      Dv::orient(nd[a], dd);
      // conservative deviations (jumps of Lax-Friedrichs fluxes) from the
      // staged state where the node phase did not store them
      if (NEED_DU && VI != VI_HG)
        Dv::node_du(s_u + ((size_t)slot * NN + lb + a * S) * NV, R, nd[a].du);
    }
  }
  float acc[N][NV];
#pragma unroll
  for (int a = 0; a < N; ++a)
#pragma unroll
    for (int v = 0; v < NV; ++v) acc[a][v] = 0.0f;

  if (VI == VI_WEAK) {
    // weak_form_kernel!: du[ii] += Dhat[ii, a] f(u_a)
#pragma unroll
    for (int a = 0; a < N; ++a) {
      float f[NV];
      Dv::dflux(R, nd[a], dd, vro, eos, f);
#pragma unroll
      for (int ii = 0; ii < N; ++ii) {
        const float c = s_mat[ii * N + a];
#pragma unroll
        for (int v = 0; v < NV; ++v) acc[ii][v] = fmaf(c, f[v], acc[ii][v]);
      }
    }
  } else {
    // flux_differencing_kernel!: each pair once, both nodes updated
#pragma unroll
    for (int a = 0; a < N; ++a)
#pragma unroll
      for (int b = a + 1; b < N; ++b) {
        float F[NV];
        Dv::template flux2<VF>(P.volume_flux, R, nd[a], nd[b], dd, vro, eos, F);
        const float cab = s_mat[a * N + b], cba = s_mat[b * N + a];
#pragma unroll
        for (int v = 0; v < NV; ++v) {
          acc[a][v] = fmaf(cab, F[v], acc[a][v]);
          acc[b][v] = fmaf(cba, F[v], acc[b][v]);
        }
      }
    if (VI == VI_HG && fabsf(alpha) > P.alpha_atol) {
      // (1 - alpha) FD + alpha FV (fv_kernel!, zero-padded subcell fluxes)
#pragma unroll
      for (int a = 0; a < N; ++a)
#pragma unroll
        for (int v = 0; v < NV; ++v) acc[a][v] *= (1.0f - alpha);
#pragma unroll
      for (int a = 0; a + 1 < N; ++a) {
        float F[NV];
        // flux-specialised instances run only where the subcell flux is the
        // surface flux (launch_mixed_n4); the others dispatch at run time
        if constexpr (SF >= 0)
          Dv::template flux2<SF>(SF, R, nd[a], nd[a + 1], dd, vro, eos, F);
        else
          Dv::two_point(P.fv_flux, R, nd[a], nd[a + 1], dd, vro, eos, F);
        const float ca = alpha * s_iw[a], cb = alpha * s_iw[a + 1];
#pragma unroll
        for (int v = 0; v < NV; ++v) {
          acc[a][v] = fmaf(ca, F[v], acc[a][v]);
          acc[a + 1][v] = fmaf(-cb, F[v], acc[a + 1][v]);
        }
      }
    }
  }

  // faces -dd (node 0) and +dd (node N-1): interface fluxes with the
  // neighbour's trace expressed relative to this element's reference
  const float factor = s_iw[0];
#pragma unroll
  for (int side = 0; side < 2; ++side) {
    const int dir = 2 * dd + side;
    const int64_t nb = nbr_row[dir];
    const int own_node = lb + (side ? (N - 1) * S : 0);
    Node<D>& own = side ? nd[N - 1] : nd[0];
    if (!NEED_DU) Dv::node_du(s_u + ((size_t)slot * NN + own_node) * NV, R, own.du);
    // neighbour trace: in this block, or staged (other blocks, and the ghost
    // trace of a boundary face)
    const int64_t nbs = nb - e0;
    const float2* src = (nb >= 0 && nbs < nel && nbs >= 0)
                            ? s_u + ((int)nbs * NN + lb + (side ? 0 : (N - 1) * S)) * NV
                            : s_fu + ((slot * 2 * D + dir) * NF + line) * NV;
    float F[NV];
    // faces with a given flux (slip walls, mortars) are compiled into the
    // run-time flux kernels and the DIRECT instances only: contexts with such
    // faces use those (the other flux-specialised instances keep registers
    // for the conforming hot path)
    bool wall = false;
    if constexpr (SF < 0 || DIRECT)
      wall = nb < 0 && (-1 - nb >= P.nbc || P.bc[dir] == BC_SLIP_WALL);
    if (wall) {
      Dv::wall_flux(R, src, dd, vro, eos, F);
    } else {
      float hi[NV], lo[NV];
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        const float2 x = src[v];
        hi[v] = x.x;
        lo[v] = x.y;
      }
      Node<D> nn_;
      Dv::make_node(hi, lo, R, eos, nn_);
      Dv::orient(nn_, dd);
      if (side)
        Dv::template flux2<SF>(P.surface_flux, R, own, nn_, dd, vro, eos, F);
      else
        Dv::template flux2<SF>(P.surface_flux, R, nn_, own, dd, vro, eos, F);
    }
    if (side) {
#pragma unroll
      for (int v = 0; v < NV; ++v) acc[N - 1][v] = fmaf(F[v], factor, acc[N - 1][v]);
    } else {
#pragma unroll
      for (int v = 0; v < NV; ++v) acc[0][v] = fmaf(-F[v], factor, acc[0][v]);
    }
  }
#pragma unroll
  for (int v = 0; v < NV; ++v) {
    float* dst = s_part + (dd * NV + v) * SP;
    if constexpr (N == 4) {
      if (vec4) {
        *reinterpret_cast<float4*>(dst + Lay::pos(slot, lb)) =
            make_float4(acc[0][v], acc[1][v], acc[2][v], acc[3][v]);
        continue;
      }
    }
#pragma unroll
    for (int a = 0; a < N; ++a) dst[Lay::pos(slot, lb + a * S)] = acc[a][v];
  }
}

// Status bit of a stage kernel block whose (bounded) wait for its staged
// inputs gave up; the block stops.
constexpr int32_t STATUS_STAGING_TIMEOUT = 8;
constexpr uint32_t STAGING_WAIT_POLLS = 1u << 22;

// ---------------------------------------------------------------------------
// Phases of one block's work (EPB elements of one mesh).  Every thread of the
// block runs each phase; blockDim.x == MixedKernel::NT.
// ---------------------------------------------------------------------------

// Per element: blending factor (VI_HG: `alpha_pre` when a pre-pass smoothed
// it, or raw with `alpha_nb` the raw factors across its faces, else alpha_raw
// smoothed here from global memory), the reference state (mean `hi` of two
// opposite corner nodes, read from `chunk`, the block's state in global or
// shared memory) and the element part of the source phase.
template <int D, int N, int VI, int EPB>
__device__ __forceinline__ void mixed_setup_elements(const MixedParams& P, const MixedArgs& A,
                                                     int64_t e0, int nel, const float2* chunk,
                                                     const float* alpha_pre, RefState<D>* s_ref,
                                                     float* s_elem,
                                                     const float* alpha_nb = nullptr) {
  using K = MixedKernel<D, N, VI, EPB>;
  using Dv = Dev<D>;
  constexpr int NV = K::NV, NN = K::NN;
  const int tid = threadIdx.x;
  if (tid >= nel) return;
  const int64_t e = e0 + tid;
  if (VI == VI_HG) {
    float a;
    if (alpha_pre) {
      a = alpha_pre[tid];
      // alpha_nb: the raw factors across the element's faces, NaN at a domain
      // boundary (fmax keeps `a` there), in smooth_over_face's order
      if (alpha_nb) {
#pragma unroll
        for (int dir = 0; dir < 2 * D; ++dir) a = fmax(a, 0.5f * alpha_nb[tid * 2 * D + dir]);
      }
    } else {
      a = A.alpha_raw[e];
      if (P.alpha_smooth) {
#pragma unroll
        for (int dir = 0; dir < 2 * D; ++dir)
          a = smooth_over_face<float>(a, P.nbr[e * 2 * D + dir], A.alpha_raw, P.nbc, P.mnbr);
      }
    }
    s_elem[tid * 8 + 0] = a;
    if (A.alpha_out) A.alpha_out[e] = a;
  }
  // reference = mean of two opposite corner nodes: the element centre for a
  // linear state, which makes the deviations (and their FP32 rounding) about
  // three times smaller in rms than those from a corner
  const float2* ue = chunk + (size_t)tid * NN * NV;
  float hi[NV];
#pragma unroll
  for (int v = 0; v < NV; ++v) hi[v] = 0.5f * (ue[v].x + ue[(NN - 1) * NV + v].x);
  Dv::make_ref(hi, P.eos, s_ref[tid]);
  if (P.source == SRC_CONVERGENCE_TEST) {
    // sin/cos of pi (x_first - t) in float-float by the angle-difference
    // formula: sin(a - b) = sa cb - ca sb, cos(a - b) = ca cb + sa sb
    float st, ct, stl, ctl;
    if (A.mode == MODE_RHS) {
      st = A.sin_t, ct = A.cos_t, stl = A.sin_tl, ctl = A.cos_tl;
    } else {
      st = A.clock->sin_t[A.stage], ct = A.clock->cos_t[A.stage];
      stl = A.clock->sin_tl[A.stage], ctl = A.clock->cos_tl[A.stage];
    }
    const float4 a = P.sc0[e];
    const float2 sn = ff_dot2(a.x, a.z, ct, ctl, -a.y, -a.w, st, stl);
    const float2 cs = ff_dot2(a.y, a.w, ct, ctl, a.x, a.z, st, stl);
    float* el = s_elem + tid * 8;
    el[1] = sn.x;
    el[2] = cs.x;
    el[3] = sn.y;
    el[4] = cs.y;
    el[5] = (float)P.scls[e];
  }
}

// Node deviations from the element's reference state -> s_nd (padded SoA).
template <int D, int N, int VI, int EPB>
__device__ __forceinline__ void mixed_node_deviations(const MixedParams& P, const float2* s_u,
                                                      const RefState<D>* s_ref, float* s_nd,
                                                      int nel) {
  using K = MixedKernel<D, N, VI, EPB>;
  using Lay = NodeLayout<D, N, EPB>;
  using Dv = Dev<D>;
  constexpr int NV = K::NV, NN = K::NN, NT = K::NT, SP = K::SP;
  for (int n = threadIdx.x; n < nel * NN; n += NT) {
    const int sl = n / NN;
    float hi[NV], lo[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      const float2 x = s_u[n * NV + v];
      hi[v] = x.x;
      lo[v] = x.y;
    }
    Node<D> nd;
    Dv::make_node(hi, lo, s_ref[sl], P.eos, nd);
    const int ps = Lay::pos(sl, n - sl * NN);
#pragma unroll
    for (int v = 0; v < NV; ++v) s_nd[v * SP + ps] = nd.dw[v];
    s_nd[NV * SP + ps] = nd.dq;
    if (VI == VI_HG) {
#pragma unroll
      for (int v = 0; v < NV; ++v) s_nd[(NV + 1 + v) * SP + ps] = nd.du[v];
    }
  }
}

// Lines: volume + surface contributions of this thread's line -> s_part.
// nbr_rows: the face-neighbour rows of the block's elements ([nel][2D]).
template <int D, int N, int VI, int VF, int SF, int EPB, bool DIRECT>
__device__ __forceinline__ void mixed_lines(const MixedParams& P, const RefState<D>* s_ref,
                                            const float2* s_u, const float2* s_fu,
                                            const float* s_nd, float* s_part, const float* s_mat,
                                            const float* s_iw, const float* s_elem,
                                            const int32_t* nbr_rows, int64_t e0, int nel) {
  using K = MixedKernel<D, N, VI, EPB>;
  constexpr int NF = K::NF;
  const int tid = threadIdx.x;
  const int dd = tid / (EPB * NF);
  const int r = tid - dd * (EPB * NF);
  const int sl = r / NF;
  const int line = r - sl * NF;
  if (sl < nel)
    mixed_line<D, N, VI, VF, SF, EPB, DIRECT>(P, s_ref[sl], s_u, s_fu, s_nd, s_part, s_mat, s_iw,
                                              VI == VI_HG ? s_elem[sl * 8] : 0.0f, sl, line, dd,
                                              e0 + sl, e0, nel, nbr_rows + sl * 2 * D);
}

// Nodes: sum of directions, Jacobian, sources, then either du (MODE_RHS) or
// the 2N update written straight to HBM and the CFL wave-speed reduction of
// the new state.  ut_old[k] holds the 2N register of this thread's k-th node
// (zero at the first stage); inv_jac the inverse Jacobians of the block's
// elements (global or shared memory).
template <int D, int N, int VI, int EPB>
__device__ __forceinline__ void mixed_node_update(const MixedParams& P, const MixedArgs& A,
                                                  int64_t e0, int nel, const float2* s_u,
                                                  const float* s_part, const float* s_elem,
                                                  const float* s_scal, unsigned int* s_smax,
                                                  const float* inv_jac,
                                                  const float (&ut_pre)[(EPB * Pow<N, D>::value +
                                                                         MixedKernel<D, N, VI, EPB>::NT - 1) /
                                                                        MixedKernel<D, N, VI, EPB>::NT]
                                                                       [D + 2]) {
  using K = MixedKernel<D, N, VI, EPB>;
  using Lay = NodeLayout<D, N, EPB>;
  constexpr int NV = K::NV, NN = K::NN, NT = K::NT, SP = K::SP;
  constexpr int PP = D + 1;
  constexpr int NPT = (EPB * NN + NT - 1) / NT;
  const int tid = threadIdx.x;
  const size_t gofs = (size_t)e0 * NN * NV;
  const float gamma = P.gamma;
  const bool stage = A.mode == MODE_STAGE;
  const float bdt = s_scal[0], bdt_lo = s_scal[6];
  const float a_s = s_scal[1], a_lo = s_scal[7];
  bool bad = false;
#pragma unroll
  for (int k = 0; k < NPT; ++k) {
    const int n = tid + k * NT;
    if (n >= nel * NN) continue;
    const int sl = n / NN;
    const int node = n - sl * NN;
    const size_t g = gofs + (size_t)n * NV;
    const float* ut_old = ut_pre[k];
    const float jfac = -inv_jac[sl];
    const int ps = Lay::pos(sl, node);
    float du[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      float s = 0;
#pragma unroll
      for (int d = 0; d < D; ++d) s += s_part[(d * NV + v) * SP + ps];
      du[v] = s * jfac;
    }
    if (P.source == SRC_CONVERGENCE_TEST) {
      // phase of this node: element part + node offset, each float-float, so
      // that the only rounding is the final one (which varies with t instead
      // of repeating the same pattern every stage)
      const float* el = s_elem + sl * 8;
      const float4 o = P.scn[(int)el[5] * NN + node];
      const float2 sn = ff_dot2(el[1], el[3], o.y, o.w, el[2], el[4], o.x, o.z);
      const float2 cs = ff_dot2(el[2], el[4], o.y, o.w, -el[1], -el[3], o.x, o.z);
      float src[NV];
      SourceMMS<D>::eval(sn.x, cs.x, P.eos, src);
#pragma unroll
      for (int v = 0; v < NV; ++v) du[v] += src[v];
    }
    if (!stage) {
#pragma unroll
      for (int v = 0; v < NV; ++v) A.du_out[g + v] = (double)du[v];
      continue;
    }
    float hi[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      const float ut = fmaf(-a_lo, ut_old[v], fmaf(-a_s, ut_old[v], du[v]));
      A.u_tmp[g + v] = ut;
      const float2 un = ff_add(s_u[n * NV + v], fmaf(ut, bdt_lo, ut * bdt));
      A.u_out[g + v] = un;
      hi[v] = un.x;
      bad |= !(un.x == un.x);
    }
    if (A.rp_out) A.rp_out[g / NV] = Euler<D, float>::density_pressure(hi, gamma);
    if (A.speed_bits) {
      float w[NV];
      Euler<D, float>::cons2prim(hi, w, gamma);
      const float cs = sqrtf(gamma * w[PP] / w[0]);
      bad |= !(w[0] > 0.0f) || !(w[PP] > 0.0f);
#pragma unroll
      for (int d = 0; d < D; ++d) {
        const float lam = fabsf(w[1 + d]) + cs;
        if (lam == lam) atomicMax(&s_smax[sl * D + d], __float_as_uint(lam));
      }
    }
  }
  if (bad) atomicOr(A.status, 1);
  if (stage && A.speed_bits) {
    // the block's largest element speed, one atomic per block: the first
    // warp reduces the element speeds
    __syncthreads();
    if (tid < 32) {
      unsigned long long b = 0;
      for (int k = tid; k < nel; k += 32) {
        float sum = 0;
#pragma unroll
        for (int d = 0; d < D; ++d) sum += __uint_as_float(s_smax[k * D + d]);
        const float sp = inv_jac[k] * sum;
        if (sp == sp) {
          const unsigned long long x = (unsigned long long)__double_as_longlong((double)sp);
          b = x > b ? x : b;
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long other = __shfl_xor_sync(0xffffffffu, b, o);
        b = other > b ? other : b;
      }
      if (tid == 0 && b) atomicMax(A.speed_bits, b);
    }
  }
}

// Per-kernel constants of a block: derivative matrix, inverse weights, the
// 2N coefficients (b dt and a as float-float pairs: rounded once they would
// perturb the 2N weights by the same amount every step, a drift of the time
// axis) and the cleared speed maxima.
template <int D, int N, int VI>
__device__ __forceinline__ void mixed_block_constants(const MixedParams& P, const MixedArgs& A,
                                                      int nthreads, float* s_mat, float* s_iw,
                                                      float* s_scal) {
  const int tid = threadIdx.x;
  for (int k = tid; k < N * N; k += nthreads) s_mat[k] = VI == VI_WEAK ? P.Dhat[k] : P.Dsplit[k];
  if (tid < N) s_iw[tid] = P.inv_weights[tid];
  if (tid == 0) {
    const double bdt = A.mode == MODE_RHS ? 0.0 : A.b * A.clock->dt;
    const float bh = (float)bdt, ah = (float)A.a;
    s_scal[0] = bh;
    s_scal[6] = (float)(bdt - (double)bh);
    s_scal[1] = ah;
    s_scal[7] = (float)(A.a - (double)ah);
  }
}

// The work of one block: EPB elements (block index blk) of one mesh.  It is
// the body of mixed_element_kernel and of the ensemble kernel, which runs it
// on work items of many meshes (tg_ensemble.cu).  Every thread of the block
// calls it with the same arguments, blockDim.x == NT, and smem_raw holds
// MixedKernel::smem_bytes() bytes.  All global reads of a block are issued up
// front: the state chunk as one bulk (TMA) copy completed on an mbarrier, the
// neighbour traces of faces between blocks as cp.async copies; each element's
// reference state is built from direct loads of its two corner nodes while
// the copies are in flight.
template <int D, int N, int VI, int VF, int SF, int EPB, bool DIRECT = false>
__device__ __forceinline__ void mixed_element_block(const MixedParams& P, const MixedArgs& A,
                                                    int64_t blk, unsigned char* smem_raw) {
  using K = MixedKernel<D, N, VI, EPB>;
  constexpr int NV = K::NV, NN = K::NN, NF = K::NF, NT = K::NT, SP = K::SP;
  constexpr int CHUNK = K::CHUNK, NFLD = K::NFLD, FACE = K::FACE;

  float2* s_u = reinterpret_cast<float2*>(smem_raw);
  float2* s_fu = s_u + CHUNK;                               // neighbour traces
  float* s_nd = reinterpret_cast<float*>(s_fu + FACE + K::PADF);
  float* s_part = s_nd + NFLD * SP;
  RefState<D>* s_ref = reinterpret_cast<RefState<D>*>(s_part + D * NV * SP);
  // [EPB][8]: alpha, then sin/cos (hi, hi, lo, lo) of pi (x_first - t)
  float* s_elem = reinterpret_cast<float*>(s_ref + EPB);
  // b dt, a, (unused: 2..5), b dt lo, a lo
  float* s_scal = s_elem + EPB * 8;
  unsigned int* s_smax = reinterpret_cast<unsigned int*>(s_scal + 8);
  float* s_mat = reinterpret_cast<float*>(s_smax + EPB * D);
  float* s_iw = s_mat + N * N;
  uint64_t* s_bar = reinterpret_cast<uint64_t*>(
      (reinterpret_cast<uintptr_t>(s_iw + N + 4) + 7) & ~static_cast<uintptr_t>(7));

  const int tid = threadIdx.x;
  const int64_t e0 = blk * EPB;
  const int nel = (int)min((int64_t)EPB, P.nelements - e0);
  const size_t gofs = (size_t)e0 * NN * NV;
  const int nval = nel * NN * NV;

  if (A.mode == MODE_STAGE && A.clock->skip) {
    for (int k = tid; k < nval; k += NT) A.u_out[gofs + k] = A.u_in[gofs + k];
    return;
  }

  // ---- asynchronous staging of the block's state (one bulk copy when the
  //      chunk starts and ends on 16-byte boundaries, else 8-byte cp.async)
  //      and of the face traces of neighbours in other blocks ---------------------
  const bool bulk = (gofs & 1) == 0 && (nval & 1) == 0;
  if (bulk && tid == 0) {
    tc::mbar_init(s_bar, 1);
    tc::fence_mbar_init();
    tc::mbar_arrive_expect_tx(s_bar, (uint32_t)(sizeof(float2) * nval));
    tc::bulk_g2s(s_u, A.u_in + gofs, (uint32_t)(sizeof(float2) * nval), s_bar);
  }
  if (!bulk)
    for (int k = tid; k < nval; k += NT) cp_async8(s_u + k, A.u_in + gofs + k);
  for (int k = tid; k < nel * 2 * D * NF; k += NT) {
    const int sl = k / (2 * D * NF);
    const int rem = k - sl * (2 * D * NF);
    const int dir = rem / NF;
    const int fn = rem - dir * NF;
    const int64_t nb = P.nbr[(e0 + sl) * 2 * D + dir];
    if (nb >= e0 && nb < e0 + nel) continue;  // in this block
    const int dd = dir >> 1;
    const int nnode = line_base<N>(fn, dd) + ((dir & 1) ? 0 : (N - 1) * axis_stride<N>(dd));
    const float2* g = nb >= 0 ? A.u_in + ((size_t)nb * NN + nnode) * NV
                              : P.ghost + ((size_t)(-1 - nb) * NF + fn) * NV;  // boundary face
#pragma unroll
    for (int v = 0; v < NV; ++v) cp_async8(s_fu + k * NV + v, g + v);
  }
  mixed_block_constants<D, N, VI>(P, A, NT, s_mat, s_iw, s_scal);
  if (tid < EPB * D) s_smax[tid] = 0u;
  // ---- per element, while the copies are in flight ---------------------------
  mixed_setup_elements<D, N, VI, EPB>(P, A, e0, nel, A.u_in + gofs, nullptr, s_ref, s_elem);
  cp_async_wait_all();
  __syncthreads();  // also orders the mbarrier's initialisation before the waits
  if (bulk && __syncthreads_or(!tc::mbar_wait_bounded(s_bar, 0u, STAGING_WAIT_POLLS))) {
    // the bulk copy did not land in time: report it and leave the block
    // (a second bounded wait for the copy still in flight first)
    if (tid == 0) atomicOr(A.status, STATUS_STAGING_TIMEOUT);
    tc::mbar_wait_bounded(s_bar, 0u, STAGING_WAIT_POLLS);
    return;
  }

  mixed_node_deviations<D, N, VI, EPB>(P, s_u, s_ref, s_nd, nel);
  __syncthreads();

  mixed_lines<D, N, VI, VF, SF, EPB, DIRECT>(P, s_ref, s_u, s_fu, s_nd, s_part, s_mat, s_iw,
                                             s_elem, P.nbr + e0 * 2 * D, e0, nel);
  // 2N register of this thread's node-phase nodes (zero at the first stage),
  // loaded before the barrier so that its latency overlaps the wait
  constexpr int NPT = (EPB * NN + NT - 1) / NT;  // nodes per thread in the node phase
  const bool stage = A.mode == MODE_STAGE;
  float ut_pre[NPT][NV];
#pragma unroll
  for (int k = 0; k < NPT; ++k) {
    const int n = tid + k * NT;
    const bool ld = stage && !A.zero_tmp && n < nel * NN;
#pragma unroll
    for (int v = 0; v < NV; ++v) ut_pre[k][v] = ld ? A.u_tmp[gofs + (size_t)n * NV + v] : 0.0f;
  }
  __syncthreads();

  mixed_node_update<D, N, VI, EPB>(P, A, e0, nel, s_u, s_part, s_elem, s_scal, s_smax,
                                   P.inv_jac + e0, ut_pre);
  if (bulk) {
    // the ensemble kernel calls this body again on the same shared memory:
    // retire the mbarrier (its one phase has completed) before it is re-made
    __syncthreads();
    if (tid == 0) tc::mbar_inval(s_bar);
  }
}

template <int D, int N, int VI, int VF, int SF, int EPB, bool DIRECT = false>
__global__ void __launch_bounds__(MixedKernel<D, N, VI, EPB>::NT, MixedKernel<D, N, VI, EPB>::MINB)
    mixed_element_kernel(const MixedParams P, const MixedArgs A) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  mixed_element_block<D, N, VI, VF, SF, EPB, DIRECT>(P, A, blockIdx.x, smem_raw);
}

// ---------------------------------------------------------------------------
// Persistent, double-buffered form of the stage kernel (2D meshes).
//
// Each block walks element blocks blk = blockIdx.x, + gridDim.x, ...  The
// inputs of the next element block are fetched while the current one
// computes:
//   - one thread issues bulk (TMA) copies of its state chunk, its 2N register
//     chunk (after stage 0), its face-neighbour rows, its pre-smoothed blending
//     factors and its inverse Jacobians into the other of two buffers, before
//     the lines phase; they complete on that buffer's mbarrier;
//   - after the lines phase (the last reader of the face traces), every thread
//     issues cp.async copies of the next block's neighbour traces of faces to
//     other blocks, addressed by the neighbour rows that have arrived by then;
//     they land during the node phase.
// The waits are bounded: a block that gives up sets STATUS_STAGING_TIMEOUT in
// the status word, waits (bounded) for its copies in flight and stops.  The
// arithmetic is that of mixed_element_block, phase by phase, so both give the
// same bits.
// ---------------------------------------------------------------------------
template <int D, int N, int VI, int EPB>
struct MixedPipe {
  using K = MixedKernel<D, N, VI, EPB>;
  static constexpr int NV = K::NV, NN = K::NN, NF = K::NF, NT = K::NT, SP = K::SP;
  static __host__ __device__ constexpr size_t up(size_t x) { return (x + 15) / 16 * 16; }
  // one buffer: state, u_tmp, neighbour rows, alpha, inverse Jacobian
  static constexpr size_t B_U = 0;
  static constexpr size_t B_UT = B_U + up(sizeof(float2) * K::CHUNK);
  static constexpr size_t B_NBR = B_UT + up(sizeof(float) * K::CHUNK);
  static constexpr size_t B_AL = B_NBR + up(sizeof(int32_t) * EPB * 2 * D);
  static constexpr size_t B_IJ = B_AL + up(sizeof(float) * EPB);
  static constexpr size_t BUF = B_IJ + up(sizeof(float) * EPB);
  // single copies
  static constexpr size_t O_FU = 2 * BUF;
  static constexpr size_t O_ND = O_FU + up(sizeof(float2) * K::FACE);
  static constexpr size_t O_PART = O_ND + up(sizeof(float) * K::NFLD * SP);
  static constexpr size_t O_REF = O_PART + up(sizeof(float) * D * NV * SP);
  static constexpr size_t O_ELEM = O_REF + up(sizeof(RefState<D>) * EPB);
  static constexpr size_t O_SCAL = O_ELEM + up(sizeof(float) * EPB * 8);
  static constexpr size_t O_SMAX = O_SCAL + up(sizeof(float) * 8);
  static constexpr size_t O_MAT = O_SMAX + up(sizeof(unsigned) * EPB * D);
  static constexpr size_t O_IW = O_MAT + up(sizeof(float) * N * N);
  static constexpr size_t O_ANB = O_IW + up(sizeof(float) * N);  // neighbours' raw factors
  static constexpr size_t O_BAR = O_ANB + up(sizeof(float) * EPB * 2 * D);
  static constexpr size_t SMEM = O_BAR + 16;
  // the per-element float rows (blending factor, inverse Jacobian) of a block
  // start on 16-byte boundaries only for EPB % 4 == 0; otherwise they are read
  // with plain loads when the block starts
  static constexpr bool ROWS_BULK = EPB % 4 == 0;
  // resident blocks per SM asked of the register allocator: the 3D form runs
  // small blocks (2 elements, 96 threads), six of them per SM
  static constexpr int MINB = (D == 3 && EPB == 2) ? 6 : K::MINB;
};

// Bulk copies of element block blk's contiguous inputs into buffer `buf`
// (thread 0).  The state and u_tmp chunks are multiples of 16 bytes for every
// polydeg in 2D and for even N^3 in 3D; the neighbour rows (2D ints per
// element) and the per-element float arrays are read in whole 16-byte groups
// (allocated with padding), starting on 16-byte boundaries for EPB % 4 == 0.
template <int D, int N, int VI, int EPB>
__device__ __forceinline__ void mixed_pipe_issue(const MixedParams& P, const MixedArgs& A,
                                                 int64_t blk, unsigned char* buf, uint64_t* mbar) {
  using Q = MixedPipe<D, N, VI, EPB>;
  constexpr int NN = Q::NN, NV = Q::NV;
  const int64_t e0 = blk * EPB;
  const int nel = (int)min((int64_t)EPB, P.nelements - e0);
  const size_t gofs = (size_t)e0 * NN * NV;
  const uint32_t b_u = (uint32_t)(sizeof(float2) * nel * NN * NV);
  const bool need_ut = A.mode == MODE_STAGE && !A.zero_tmp;
  const uint32_t b_ut = need_ut ? (uint32_t)(sizeof(float) * nel * NN * NV) : 0u;
  // every source address below is 16-byte aligned: e0 is a multiple of EPB,
  // the neighbour rows of EPB elements are whole 16-byte groups and the float
  // rows are copied in bulk only where EPB % 4 == 0 (Q::ROWS_BULK)
  static_assert((Pow<N, D>::value * (D + 2)) % 2 == 0, "state chunks of whole 16-byte groups");
  static_assert((EPB * 2 * D * sizeof(int32_t)) % 16 == 0, "neighbour rows of whole 16-byte groups");
  const uint32_t b_nbr = (uint32_t)Q::up(sizeof(int32_t) * nel * 2 * D);
  const uint32_t b_el = Q::ROWS_BULK ? (uint32_t)Q::up(sizeof(float) * nel) : 0u;
  const uint32_t b_al = VI == VI_HG ? b_el : 0u;
  tc::mbar_arrive_expect_tx(mbar, b_u + b_ut + b_nbr + b_al + b_el);
  tc::bulk_g2s(buf + Q::B_U, A.u_in + gofs, b_u, mbar);
  if (need_ut) tc::bulk_g2s(buf + Q::B_UT, A.u_tmp + gofs, b_ut, mbar);
  tc::bulk_g2s(buf + Q::B_NBR, P.nbr + e0 * 2 * D, b_nbr, mbar);
  if constexpr (Q::ROWS_BULK) {
    if (VI == VI_HG) tc::bulk_g2s(buf + Q::B_AL, A.alpha_smoothed + e0, b_al, mbar);
    tc::bulk_g2s(buf + Q::B_IJ, P.inv_jac + e0, b_el, mbar);
  }
}

// cp.async copies of the neighbour traces of element block blk's faces to
// other blocks (and of ghost traces) into `fu`, addressed by the block's
// staged neighbour rows, then a commit.
template <int D, int N, int VI, int EPB>
__device__ __forceinline__ void mixed_pipe_faces(const MixedParams& P, const MixedArgs& A,
                                                 int64_t blk, const int32_t* s_nbr, float2* fu,
                                                 float* anb) {
  using Q = MixedPipe<D, N, VI, EPB>;
  constexpr int NF = Q::NF, NT = Q::NT, NN = Q::NN, NV = Q::NV;
  const int64_t e0 = blk * EPB;
  const int nel = (int)min((int64_t)EPB, P.nelements - e0);
  if (VI == VI_HG && A.alpha_gather && (int)threadIdx.x < nel) {
    // the raw blending factors across the faces of element threadIdx.x, by
    // the thread that smooths its factor in the setup phase (which waits for
    // its own copies only)
    const int t = threadIdx.x;
#pragma unroll
    for (int dir = 0; dir < 2 * D; ++dir) {
      const int32_t nb = s_nbr[t * 2 * D + dir];
      if (nb >= 0)
        cp_async4(anb + t * 2 * D + dir, A.alpha_smoothed + nb);
      else
        anb[t * 2 * D + dir] = __int_as_float(0x7fffffff);  // domain boundary (no mortars here)
    }
  }
  for (int k = threadIdx.x; k < nel * 2 * D * NF; k += NT) {
    const int sl = k / (2 * D * NF);
    const int rem = k - sl * (2 * D * NF);
    const int dir = rem / NF;
    const int fn = rem - dir * NF;
    const int64_t nb = s_nbr[sl * 2 * D + dir];
    if (nb >= e0 && nb < e0 + nel) continue;  // in the block
    const int dd = dir >> 1;
    const int nnode = line_base<N>(fn, dd) + ((dir & 1) ? 0 : (N - 1) * axis_stride<N>(dd));
    const float2* g = nb >= 0 ? A.u_in + ((size_t)nb * NN + nnode) * NV
                              : P.ghost + ((size_t)(-1 - nb) * NF + fn) * NV;
#pragma unroll
    for (int v = 0; v < NV; ++v) cp_async8(fu + k * NV + v, g + v);
  }
  cp_async_commit();
}

template <int D, int N, int VI, int VF, int SF, int EPB, bool DIRECT = false>
__global__ void __launch_bounds__(MixedKernel<D, N, VI, EPB>::NT, MixedPipe<D, N, VI, EPB>::MINB)
    mixed_element_pipe_kernel(const MixedParams P, const MixedArgs A) {
  using K = MixedKernel<D, N, VI, EPB>;
  using Q = MixedPipe<D, N, VI, EPB>;
  constexpr int NV = K::NV, NN = K::NN, NT = K::NT;
  constexpr int NPT = (EPB * NN + NT - 1) / NT;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* s_fu = reinterpret_cast<float2*>(smem_raw + Q::O_FU);
  float* s_nd = reinterpret_cast<float*>(smem_raw + Q::O_ND);
  float* s_part = reinterpret_cast<float*>(smem_raw + Q::O_PART);
  RefState<D>* s_ref = reinterpret_cast<RefState<D>*>(smem_raw + Q::O_REF);
  float* s_elem = reinterpret_cast<float*>(smem_raw + Q::O_ELEM);
  float* s_scal = reinterpret_cast<float*>(smem_raw + Q::O_SCAL);
  unsigned int* s_smax = reinterpret_cast<unsigned int*>(smem_raw + Q::O_SMAX);
  float* s_mat = reinterpret_cast<float*>(smem_raw + Q::O_MAT);
  float* s_iw = reinterpret_cast<float*>(smem_raw + Q::O_IW);
  float* s_anb = reinterpret_cast<float*>(smem_raw + Q::O_ANB);
  uint64_t* mbar = reinterpret_cast<uint64_t*>(smem_raw + Q::O_BAR);

  const int tid = threadIdx.x;
  const int64_t nblocks = (P.nelements + EPB - 1) / EPB;
  if (A.mode == MODE_STAGE && A.clock->skip) {
    // past t_end: the state passes through unchanged (no copies issued)
    for (int64_t blk = blockIdx.x; blk < nblocks; blk += gridDim.x) {
      const int64_t e0 = blk * EPB;
      const size_t gofs = (size_t)e0 * NN * NV;
      const int nval = (int)min((int64_t)EPB, P.nelements - e0) * NN * NV;
      for (int k = tid; k < nval; k += NT) A.u_out[gofs + k] = A.u_in[gofs + k];
    }
    return;
  }
  const bool need_ut = A.mode == MODE_STAGE && !A.zero_tmp;
  if (tid == 0) {
    tc::mbar_init(&mbar[0], 1);
    tc::mbar_init(&mbar[1], 1);
    tc::fence_mbar_init();
  }
  mixed_block_constants<D, N, VI>(P, A, NT, s_mat, s_iw, s_scal);
  __syncthreads();

  // prologue: the first element block's inputs
  int64_t blk = blockIdx.x;
  int failed_it = -1;
  if (tid == 0) mixed_pipe_issue<D, N, VI, EPB>(P, A, blk, smem_raw, &mbar[0]);
  if (__syncthreads_or(!tc::mbar_wait_bounded(&mbar[0], 0u, STAGING_WAIT_POLLS))) {
    failed_it = 0;
  } else {
    mixed_pipe_faces<D, N, VI, EPB>(P, A, blk,
                                    reinterpret_cast<const int32_t*>(smem_raw + Q::B_NBR), s_fu,
                                    s_anb);
  }
  for (int it = 0; failed_it < 0 && blk < nblocks; ++it, blk += gridDim.x) {
    const int b = it & 1;
    unsigned char* cur = smem_raw + b * Q::BUF;
    unsigned char* nxt_buf = smem_raw + (b ^ 1) * Q::BUF;
    const int64_t nxt = blk + gridDim.x;
    const int64_t e0 = blk * EPB;
    const int nel = (int)min((int64_t)EPB, P.nelements - e0);
    const float2* s_u = reinterpret_cast<const float2*>(cur + Q::B_U);
    // ---- this block's bulk data: waited for at the end of the previous
    //      iteration (or in the prologue), so this returns at once ------------------
    if (__syncthreads_or(!tc::mbar_wait_bounded(&mbar[b], (uint32_t)((it >> 1) & 1),
                                                 STAGING_WAIT_POLLS))) {
      failed_it = it;
      break;
    }
    if (tid < EPB * D) s_smax[tid] = 0u;
    if constexpr (!Q::ROWS_BULK) {
      // the per-element float rows, by the thread that sets its element up;
      // the other threads read them after the barrier below.  The buffer is
      // overwritten by bulk copies two blocks later: async-proxy ordering.
      if (tid < nel) {
        reinterpret_cast<float*>(cur + Q::B_IJ)[tid] = P.inv_jac[e0 + tid];
        if (VI == VI_HG) reinterpret_cast<float*>(cur + Q::B_AL)[tid] = A.alpha_smoothed[e0 + tid];
        tc::fence_proxy_async_smem();
      }
    }
    cp_async_wait_all();  // this thread's copies of this block's face traces (and factors)
    mixed_setup_elements<D, N, VI, EPB>(P, A, e0, nel, s_u,
                                        VI == VI_HG ? reinterpret_cast<const float*>(cur + Q::B_AL)
                                                    : nullptr,
                                        s_ref, s_elem,
                                        VI == VI_HG && A.alpha_gather ? s_anb : nullptr);
    __syncthreads();

    mixed_node_deviations<D, N, VI, EPB>(P, s_u, s_ref, s_nd, nel);
    __syncthreads();

    // ---- the next block's bulk inputs, into the other buffer (last read one
    //      iteration ago, before two barriers) ------------------------------------
    if (tid == 0 && nxt < nblocks) mixed_pipe_issue<D, N, VI, EPB>(P, A, nxt, nxt_buf, &mbar[b ^ 1]);

    mixed_lines<D, N, VI, VF, SF, EPB, DIRECT>(
        P, s_ref, s_u, s_fu, s_nd, s_part, s_mat, s_iw, s_elem,
        reinterpret_cast<const int32_t*>(cur + Q::B_NBR), e0, nel);
    __syncthreads();

    // ---- the next block's face traces (the face buffer is free now) -------------
    if (nxt < nblocks) {
      if (__syncthreads_or(!tc::mbar_wait_bounded(&mbar[b ^ 1], (uint32_t)(((it + 1) >> 1) & 1),
                                                   STAGING_WAIT_POLLS))) {
        failed_it = it + 1;
        break;
      }
      mixed_pipe_faces<D, N, VI, EPB>(P, A, nxt,
                                      reinterpret_cast<const int32_t*>(nxt_buf + Q::B_NBR), s_fu,
                                      s_anb);
    }

    const float* s_ut = reinterpret_cast<const float*>(cur + Q::B_UT);
    float ut_pre[NPT][NV];
#pragma unroll
    for (int k = 0; k < NPT; ++k) {
      const int n = tid + k * NT;
      const bool ld = need_ut && n < nel * NN;
#pragma unroll
      for (int v = 0; v < NV; ++v) ut_pre[k][v] = ld ? s_ut[n * NV + v] : 0.0f;
    }
    mixed_node_update<D, N, VI, EPB>(P, A, e0, nel, s_u, s_part, s_elem, s_scal, s_smax,
                                     reinterpret_cast<const float*>(cur + Q::B_IJ), ut_pre);
    __syncthreads();
  }
  if (failed_it >= 0) {
    if (tid == 0) atomicOr(A.status, STATUS_STAGING_TIMEOUT);
    cp_async_wait_all();
    // the bulk copies that were waited for, if they are still landing
    tc::mbar_wait_bounded(&mbar[failed_it & 1], (uint32_t)((failed_it >> 1) & 1),
                          STAGING_WAIT_POLLS);
  }
}

}  // namespace tg
