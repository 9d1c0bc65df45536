// Mixed-precision stage kernels of curvilinear 3D meshes (float-float state,
// FP32 deviation fluxes along the contravariant vectors), compiled with the
// FP32 flags of the mixed units (approximate FP32 division and square root,
// flush to zero).
//
// Flux-specialised instances at polydeg 3 (VF, SF >= 0: the volume and the
// surface flux compiled in, the shock-capturing subcell flux being the
// surface flux) keep the common configurations free of the run-time flux
// dispatch; every other choice takes the run-time instance (VF = SF = -1).
#include <cuda_runtime.h>

#include "tg_curved.cuh"

namespace tg {

namespace {

// ---------------------------------------------------------------------------
// Mixed-precision kernel: float-float state, FP32 flux deviations along the
// contravariant vectors (the 2D mixed kernel's algebra, tg_curved.cu, with
// three directions).  Per node the metric is three float4 {Ja^d_x, Ja^d_y,
// Ja^d_z, (d = 0: inverse Jacobian)}; with MMS sources a float4 of
// sin/cos(pi (x + y + z)) as float-float pairs.  Dirichlet faces take the
// FP64 boundary value of the face node, split into a float-float pair, while
// the block stages its neighbour traces.
// ---------------------------------------------------------------------------
template <int N, int EPB>
struct Curved3M {
  static constexpr int NF = N * N, NN = N * N * N, NV = 5, NT = EPB * 3 * NF;
  static constexpr int CHUNK = EPB * NN * NV;     // float2 state values of a block
  static constexpr int FACE = EPB * 6 * NF * NV;  // float2 neighbour / boundary traces
  static constexpr int SP = EPB * NN;
  static constexpr size_t smem() {
    return sizeof(float2) * (CHUNK + FACE) + sizeof(float4) * 4 * SP +
           sizeof(float) * (NV * SP + (NV + 1) * SP + 3 * NV * SP) + sizeof(RefState<3>) * EPB +
           sizeof(float) * 4 + sizeof(unsigned int) * 3 * EPB + sizeof(float) * EPB;
  }
};

template <int N, int VI, int EPB, int VF, int SF>
__global__ void __launch_bounds__(Curved3M<N, EPB>::NT)
    curved3_kernel_mixed(const CurvedParams P, const MixedArgs A) {
  using K = Curved3M<N, EPB>;
  using Dv = Dev<3>;
  constexpr int NN = K::NN, NF = K::NF, NV = 5, NT = K::NT, SP = K::SP, CHUNK = K::CHUNK;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* s_u = reinterpret_cast<float2*>(smem_raw);
  float2* s_fu = s_u + CHUNK;                                // [EPB][6][NF][NV]
  float4* s_ja = reinterpret_cast<float4*>(s_fu + K::FACE);  // [SP][3]
  float4* s_sc = s_ja + 3 * SP;                              // [SP]
  float* s_ut = reinterpret_cast<float*>(s_sc + SP);         // [SP][NV]
  float* s_nd = s_ut + SP * NV;                              // [NV + 1][SP]: dw, dq
  float* s_part = s_nd + (NV + 1) * SP;                      // [3][NV][SP]
  RefState<3>* s_ref = reinterpret_cast<RefState<3>*>(s_part + 3 * NV * SP);
  float* s_scal = reinterpret_cast<float*>(s_ref + EPB);     // b dt, a (hi, lo)
  unsigned int* s_smax = reinterpret_cast<unsigned int*>(s_scal + 4);
  float* s_alpha = reinterpret_cast<float*>(s_smax + 3 * EPB);  // [EPB] (VI_HG)

  const int tid = threadIdx.x;
  const int64_t e0 = (int64_t)blockIdx.x * EPB;
  const int nel = (int)min((int64_t)EPB, P.nelements - e0);
  const size_t gofs = (size_t)e0 * NN * NV;
  const int nval = nel * NN * NV;
  const EosF& eos = P.eos;
  const bool stage = A.mode == MODE_STAGE;

  if (stage && A.clock->skip) {
    for (int k = tid; k < nval; k += NT) A.u_out[gofs + k] = A.u_in[gofs + k];
    return;
  }
  {
    // NN * NV is even for the compiled degrees: the chunk starts on a 16-byte
    // boundary and holds an even number of values
    const float4* src = reinterpret_cast<const float4*>(A.u_in + gofs);
    float4* dst = reinterpret_cast<float4*>(s_u);
    for (int k = tid; k < nval / 2; k += NT) cp_async16(dst + k, src + k);
  }
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
      boundary_value<3>(P.bc_ic, P.bc_par, xv, tt, P.gamma, ub);
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        const float hi = (float)ub[v];
        s_fu[k * NV + v] = make_float2(hi, (float)(ub[v] - (double)hi));
      }
      continue;
    }
    const float2* g = A.u_in + ((size_t)nb * NN + face_partner3<N>(dir, fn)) * NV;
#pragma unroll
    for (int v = 0; v < NV; ++v) cp_async8(s_fu + k * NV + v, g + v);
  }
  {
    const int nn = nel * NN;
    const float4* ja = P.ja32 + (size_t)e0 * NN * 3;
    for (int k = tid; k < 3 * nn; k += NT) cp_async16(s_ja + k, ja + k);
    if (P.source == SRC_CONVERGENCE_TEST) {
      const float4* sc = P.sc + (size_t)e0 * NN;
      for (int k = tid; k < nn; k += NT) cp_async16(s_sc + k, sc + k);
    }
    if (stage && !A.zero_tmp) {
      // u_tmp rows of a block start on 16-byte boundaries (NN * NV * 4 bytes)
      const float4* ut = reinterpret_cast<const float4*>(A.u_tmp + gofs);
      for (int k = tid; k < nval / 4; k += NT)
        cp_async16(reinterpret_cast<float4*>(s_ut) + k, ut + k);
    }
  }
  if (tid < 3 * EPB) s_smax[tid] = 0u;
  if (tid == 0) {
    const double bdt = stage ? A.b * A.clock->dt : 0.0;
    const float bh = (float)bdt, ah = (float)A.a;
    s_scal[0] = bh;
    s_scal[1] = (float)(bdt - (double)bh);
    s_scal[2] = ah;
    s_scal[3] = (float)(A.a - (double)ah);
  }
  if (tid < nel) {
    // reference state: mean hi of two opposite corner nodes
    const float2* ue = A.u_in + (size_t)(e0 + tid) * NN * NV;
    float hi[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) hi[v] = 0.5f * (ue[v].x + ue[(NN - 1) * NV + v].x);
    Dv::make_ref(hi, eos, s_ref[tid]);
    if (VI == VI_HG) {
      // apply_smoothing! as a gather over the face neighbours
      const int64_t e = e0 + tid;
      float a = A.alpha_raw[e];
      if (P.alpha_smooth)
#pragma unroll
        for (int f = 0; f < 6; ++f) {
          const int32_t nb = P.nbr[e * 6 + f];
          if (nb >= 0) a = fmaxf(a, 0.5f * A.alpha_raw[nb]);
        }
      s_alpha[tid] = a;
      if (A.alpha_out) A.alpha_out[e] = a;
    }
  }
  cp_async_wait_all();
  __syncthreads();

  for (int n = tid; n < nel * NN; n += NT) {
    const int sl = n / NN;
    float hi[NV], lo[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      const float2 x = s_u[n * NV + v];
      hi[v] = x.x;
      lo[v] = x.y;
    }
    Node<3> nd;
    Dv::make_node(hi, lo, s_ref[sl], eos, nd);
#pragma unroll
    for (int v = 0; v < NV; ++v) s_nd[v * SP + n] = nd.dw[v];
    s_nd[NV * SP + n] = nd.dq;
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
      const RefState<3>& R = s_ref[sl];
      Node<3> nd[N];
      float ja[N][3];
#pragma unroll
      for (int a = 0; a < N; ++a) {
        const int n = sl * NN + line3<N>(line, dd, a);
#pragma unroll
        for (int v = 0; v < NV; ++v) nd[a].dw[v] = s_nd[v * SP + n];
        nd[a].dq = s_nd[NV * SP + n];
        Dv::complete(R, nd[a]);
        const float4 j = s_ja[n * 3 + dd];
        ja[a][0] = j.x;
        ja[a][1] = j.y;
        ja[a][2] = j.z;
      }
      float acc[N][NV];
#pragma unroll
      for (int a = 0; a < N; ++a)
#pragma unroll
        for (int v = 0; v < NV; ++v) acc[a][v] = 0.0f;
      if (VI == VI_WEAK) {
#pragma unroll
        for (int a = 0; a < N; ++a) {
          float cf[NV];
#pragma unroll
          for (int d = 0; d < 3; ++d) {
            Node<3> ad = nd[a];
            Dv::orient(ad, d);
            float fd[NV];
            Dv::dflux(R, ad, d, R.v[d], eos, fd);
#pragma unroll
            for (int v = 0; v < NV; ++v) cf[v] = d == 0 ? ja[a][0] * fd[v] : fmaf(ja[a][d], fd[v], cf[v]);
          }
#pragma unroll
          for (int ii = 0; ii < N; ++ii) {
            const float c = P.Dhat32[ii * N + a];
#pragma unroll
            for (int v = 0; v < NV; ++v) acc[ii][v] = fmaf(c, cf[v], acc[ii][v]);
          }
        }
      } else {
#pragma unroll
        for (int a = 0; a < N; ++a)
#pragma unroll
          for (int b = a + 1; b < N; ++b) {
            float F[NV];
            const float n[3] = {0.5f * (ja[a][0] + ja[b][0]), 0.5f * (ja[a][1] + ja[b][1]),
                                0.5f * (ja[a][2] + ja[b][2])};
            if constexpr (VF == FLUX_RANOCHA)
              dev_ranocha_n<3>(R, nd[a], nd[b], n, eos, F);
            else if constexpr (VF >= 0)
              dev_flux_n<3, VF>(VF, R, nd[a], nd[b], n, eos, F);
            else if (P.volume_flux == FLUX_RANOCHA)
              dev_ranocha_n<3>(R, nd[a], nd[b], n, eos, F);
            else
              dev_flux_n<3, -1>(P.volume_flux, R, nd[a], nd[b], n, eos, F);
            const float cab = P.Dsplit32[a * N + b], cba = P.Dsplit32[b * N + a];
#pragma unroll
            for (int v = 0; v < NV; ++v) {
              acc[a][v] = fmaf(cab, F[v], acc[a][v]);
              acc[b][v] = fmaf(cba, F[v], acc[b][v]);
            }
          }
      }
      if (VI == VI_HG) {
        // the FP64 kernel's blend in deviation form (as in 2D, tg_curved.cu)
        const float ae = s_alpha[sl];
        if (!(fabsf(ae) <= (float)P.alpha_atol)) {
#pragma unroll
          for (int a = 0; a < N; ++a) {
#pragma unroll
            for (int v = 0; v < NV; ++v) acc[a][v] *= 1.0f - ae;
            Dv::node_du(s_u + ((size_t)sl * NN + line3<N>(line, dd, a)) * NV, R, nd[a].du);
          }
          const float4* nv = P.snv3_32 + (((size_t)e * 3 + dd) * NF + line) * (N - 1);
          float fl[NV] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
          for (int i = 0; i < N; ++i) {
            float fr[NV] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
            if (i < N - 1) {
              const float4 n4 = nv[i];
              const float n3[3] = {n4.x, n4.y, n4.z};
              dev_surface_k<3, SF>(P.fv_flux, R, nd[i], nd[i + 1], n3, eos, fr);
            }
#pragma unroll
            for (int v = 0; v < NV; ++v) {
              acc[i][v] = fmaf(ae, P.inv_weights32[i] * (fr[v] - fl[v]), acc[i][v]);
              fl[v] = fr[v];
            }
          }
        }
      }
      const float factor = P.inv_weights32[0];
#pragma unroll
      for (int side = 0; side < 2; ++side) {
        const int dir = 2 * dd + side;
        const int32_t nb = P.nbr[e * 6 + dir];
        const int own = side ? N - 1 : 0;
        Dv::node_du(s_u + ((size_t)sl * NN + line3<N>(line, dd, own)) * NV, R, nd[own].du);
        const float2* src = (nb >= e0 && nb < e0 + nel)
                                ? s_u + (((int)(nb - e0)) * NN + face_partner3<N>(dir, line)) * NV
                                : s_fu + ((sl * 6 + dir) * NF + line) * NV;
        float hi[NV], lo[NV];
#pragma unroll
        for (int v = 0; v < NV; ++v) {
          hi[v] = src[v].x;
          lo[v] = src[v].y;
        }
        Node<3> other;
        Dv::make_node(hi, lo, R, eos, other);
        float F[NV];
        if (side)
          dev_surface_k<3, SF>(P.surface_flux, R, nd[own], other, ja[own], eos, F);
        else
          dev_surface_k<3, SF>(P.surface_flux, R, other, nd[own], ja[own], eos, F);
#pragma unroll
        for (int v = 0; v < NV; ++v) acc[own][v] = fmaf(side ? F[v] : -F[v], factor, acc[own][v]);
      }
#pragma unroll
      for (int a = 0; a < N; ++a) {
        const int n = sl * NN + line3<N>(line, dd, a);
#pragma unroll
        for (int v = 0; v < NV; ++v) s_part[(dd * NV + v) * SP + n] = acc[a][v];
      }
    }
  }
  __syncthreads();

  // ---- nodes -----------------------------------------------------------------------
  const float bdt = s_scal[0], bdt_lo = s_scal[1], a_s = s_scal[2], a_lo = s_scal[3];
  float st = 0, ct = 0, stl = 0, ctl = 0;
  if (P.source == SRC_CONVERGENCE_TEST) {
    if (stage) {
      st = A.clock->sin_t[A.stage];
      ct = A.clock->cos_t[A.stage];
      stl = A.clock->sin_tl[A.stage];
      ctl = A.clock->cos_tl[A.stage];
    } else {
      st = A.sin_t, ct = A.cos_t, stl = A.sin_tl, ctl = A.cos_tl;
    }
  }
  bool bad = false;
  for (int n = tid; n < nel * NN; n += NT) {
    const int sl = n / NN;
    const float4 j0 = s_ja[n * 3], j1 = s_ja[n * 3 + 1], j2 = s_ja[n * 3 + 2];
    const float jfac = -j0.w;
    float du[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v)
      du[v] = (s_part[v * SP + n] + s_part[(NV + v) * SP + n] + s_part[(2 * NV + v) * SP + n]) *
              jfac;
    if (P.source == SRC_CONVERGENCE_TEST) {
      // sin/cos(pi (x + y + z - t)) by the angle-difference formula in float-float
      const float4 o = s_sc[n];
      const float2 sn = ff_dot2(o.x, o.z, ct, ctl, -o.y, -o.w, st, stl);
      const float2 cs = ff_dot2(o.y, o.w, ct, ctl, o.x, o.z, st, stl);
      float sv[NV];
      SourceMMS<3>::eval(sn.x, cs.x, eos, sv);
#pragma unroll
      for (int v = 0; v < NV; ++v) du[v] += sv[v];
    }
    const size_t g = gofs + (size_t)n * NV;
    if (!stage) {
#pragma unroll
      for (int v = 0; v < NV; ++v) A.du_out[g + v] = (double)du[v];
      continue;
    }
    float hi[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      const float old = A.zero_tmp ? 0.0f : s_ut[n * NV + v];
      const float ut = fmaf(-a_lo, old, fmaf(-a_s, old, du[v]));
      A.u_tmp[g + v] = ut;
      const float2 un = ff_add(s_u[n * NV + v], fmaf(ut, bdt_lo, ut * bdt));
      A.u_out[g + v] = un;
      hi[v] = un.x;
      bad |= !(un.x == un.x);
    }
    if (A.speed_bits) {
      float w[NV];
      Euler<3, float>::cons2prim(hi, w, eos.gamma);
      const float cs = sqrtf(eos.gamma * w[4] / w[0]);
      bad |= !(w[0] > 0.0f) || !(w[4] > 0.0f);
      const float l[3] = {fabsf(w[1]) + cs, fabsf(w[2]) + cs, fabsf(w[3]) + cs};
      const float ij = fabsf(j0.w);
      const float4 jd[3] = {j0, j1, j2};
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const float sd = fabsf(jd[d].x * l[0] + jd[d].y * l[1] + jd[d].z * l[2]) * ij;
        if (sd == sd) atomicMax(&s_smax[3 * sl + d], __float_as_uint(sd));
      }
    }
  }
  if (bad) atomicOr(A.status, 1);
  if (stage && A.speed_bits) {
    __syncthreads();
    if (tid < nel) {
      const float sp = __uint_as_float(s_smax[3 * tid]) + __uint_as_float(s_smax[3 * tid + 1]) +
                       __uint_as_float(s_smax[3 * tid + 2]);
      if (sp == sp) atomicMax(A.speed_bits, (unsigned long long)__double_as_longlong((double)sp));
    }
  }
}


template <int N, int VI, int VF, int SF>
int launch_mixed3_one(const CurvedParams& P, const MixedArgs& A, cudaStream_t stream) {
  // 2 elements per block at polydeg 3 (at 32^3 on the warped cube: 2.50 ms
  // per step, against 2.87 with 4 and 3.19 with 8)
  constexpr int EPB = N == 4 ? 2 : 1;
  const unsigned nb = (unsigned)((P.nelements + EPB - 1) / EPB);
  using K = Curved3M<N, EPB>;
  static_assert(K::smem() <= 227 * 1024, "curvilinear 3D block exceeds the shared memory");
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(curved3_kernel_mixed<N, VI, EPB, VF, SF>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)K::smem());
    attr = true;
  }
  curved3_kernel_mixed<N, VI, EPB, VF, SF><<<nb, K::NT, K::smem(), stream>>>(P, A);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

// polydeg 3: flux_ranocha volume flux with the Lax-Friedrichs or ranocha
// surface fluxes, the weak form with the Lax-Friedrichs ones
template <int VI>
int launch_mixed3_n4(const CurvedParams& P, const MixedArgs& A, cudaStream_t stream) {
  const int sf = P.surface_flux;
  const bool lf = sf == FLUX_LLF || sf == FLUX_LLF_NAIVE;
  if constexpr (VI == VI_WEAK) {
    if (sf == FLUX_LLF) return launch_mixed3_one<4, VI, -1, FLUX_LLF>(P, A, stream);
    if (sf == FLUX_LLF_NAIVE) return launch_mixed3_one<4, VI, -1, FLUX_LLF_NAIVE>(P, A, stream);
  } else if constexpr (VI == VI_FD) {
    if (P.volume_flux == FLUX_RANOCHA) {
      if (sf == FLUX_LLF) return launch_mixed3_one<4, VI, FLUX_RANOCHA, FLUX_LLF>(P, A, stream);
      if (sf == FLUX_LLF_NAIVE)
        return launch_mixed3_one<4, VI, FLUX_RANOCHA, FLUX_LLF_NAIVE>(P, A, stream);
      if (sf == FLUX_RANOCHA)
        return launch_mixed3_one<4, VI, FLUX_RANOCHA, FLUX_RANOCHA>(P, A, stream);
    }
  } else {
    if (P.volume_flux == FLUX_RANOCHA && lf && P.fv_flux == sf) {
      if (sf == FLUX_LLF) return launch_mixed3_one<4, VI, FLUX_RANOCHA, FLUX_LLF>(P, A, stream);
      return launch_mixed3_one<4, VI, FLUX_RANOCHA, FLUX_LLF_NAIVE>(P, A, stream);
    }
  }
  return launch_mixed3_one<4, VI, -1, -1>(P, A, stream);
}

}  // namespace

// Instances as launch_curved3: polydeg 3 and 5 with the weak form and flux
// differencing, shock capturing at polydeg 3.
int launch_curved_mixed3(const CurvedParams& P, const MixedArgs& A, cudaStream_t stream) {
  if (P.vi == VI_HG) return P.N == 4 ? launch_mixed3_n4<VI_HG>(P, A, stream) : -3;
  const bool fd = P.vi == VI_FD;
  if (!fd && P.vi != VI_WEAK) return -3;
  if (P.N == 4) return fd ? launch_mixed3_n4<VI_FD>(P, A, stream) : launch_mixed3_n4<VI_WEAK>(P, A, stream);
  if (P.N == 6)
    return fd ? launch_mixed3_one<6, VI_FD, -1, -1>(P, A, stream)
              : launch_mixed3_one<6, VI_WEAK, -1, -1>(P, A, stream);
  return -3;
}

}  // namespace tg
