// Mixed-precision stage kernels of curvilinear 2D meshes (float-float state,
// FP32 deviation fluxes along the contravariant vectors; the algebra is
// described in tg_curved.cu).  Compiled with the FP32 flags of the mixed
// units (approximate FP32 division and square root, flush to zero).
//
// Flux-specialised instances at polydeg 3 (VF, SF >= 0: the volume and the
// surface flux compiled in, the shock-capturing subcell flux being the
// surface flux) keep the common configurations free of the run-time flux
// dispatch; every other choice takes the run-time instance (VF = SF = -1).
#include <cuda_runtime.h>

#include "tg_curved.cuh"

namespace tg {

// ---------------------------------------------------------------------------
// Mixed-precision stage kernel (float-float state, FP32 deviation fluxes)
// ---------------------------------------------------------------------------

template <int N, int VI, int EPB, int VF, int SF>
__global__ void __launch_bounds__(CurvedK<N, EPB>::NT, CurvedK<N, EPB>::MINB_MIXED)
    curved_kernel_mixed(const CurvedParams P, const MixedArgs A) {
  using K = CurvedK<N, EPB>;
  using Dv = Dev<2>;
  constexpr int NN = K::NN, NV = 4, NT = K::NT, SP = K::SP, CHUNK = K::CHUNK;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* s_u = reinterpret_cast<float2*>(smem_raw);
  float2* s_fu = s_u + CHUNK;
  // per-node metric, source phase, inverse Jacobian and 2N register of the
  // block, staged with the state so that no phase waits on global loads
  float4* s_ja = reinterpret_cast<float4*>(s_fu + K::FACE);  // [SP]
  float4* s_sc = s_ja + SP;                                   // [SP]
  float* s_ut = reinterpret_cast<float*>(s_sc + SP);          // [SP][NV]
  float* s_ij = s_ut + SP * NV;                               // [SP]
  float* s_nd = s_ij + SP;                                    // [NV + 1][SP]: dw, dq
  float* s_part = s_nd + (NV + 1) * SP;                     // [2][NV][SP]
  RefState<2>* s_ref = reinterpret_cast<RefState<2>*>(s_part + 2 * NV * SP);
  float* s_scal = reinterpret_cast<float*>(s_ref + EPB);    // b dt, a (hi, lo)
  unsigned int* s_smax = reinterpret_cast<unsigned int*>(s_scal + 4);
  float* s_alpha = reinterpret_cast<float*>(s_smax + 2 * EPB);  // [EPB] (VI_HG)

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
    // gofs is even (NN * NV is), so the chunk is 16-byte aligned; nval is even
    const float4* src = reinterpret_cast<const float4*>(A.u_in + gofs);
    float4* dst = reinterpret_cast<float4*>(s_u);
    for (int k = tid; k < nval / 2; k += NT) cp_async16(dst + k, src + k);
  }
  for (int k = tid; k < nel * 4 * N; k += NT) {
    const int sl = k / (4 * N);
    const int dir = (k / N) & 3;
    const int fn = k % N;
    const int32_t nb = P.nbr[(e0 + sl) * 4 + dir];
    if (nb >= e0 && nb < e0 + nel) continue;
    const float2* g = nb >= 0 ? A.u_in + ((size_t)nb * NN + cface_partner<N>(dir, fn)) * NV
                              : P.ghost + ((size_t)(-1 - nb) * N + fn) * NV;  // boundary face
#pragma unroll
    for (int v = 0; v < NV; ++v) cp_async8(s_fu + k * NV + v, g + v);
  }
  {
    // metric (one float4 per node) and inverse Jacobian; u_tmp rows are
    // 16-byte aligned (NV = 4 floats per node)
    const int nn = nel * NN;
    const float4* ja = P.ja32 + (size_t)e0 * NN;
    for (int k = tid; k < nn; k += NT) cp_async16(s_ja + k, ja + k);
    const float* ij = P.invj32 + (size_t)e0 * NN;
    for (int k = tid; k < nn; k += NT) cp_async4(s_ij + k, ij + k);
    if (P.source == SRC_CONVERGENCE_TEST) {
      const float4* sc = P.sc + (size_t)e0 * NN;
      for (int k = tid; k < nn; k += NT) cp_async16(s_sc + k, sc + k);
    }
    if (stage && !A.zero_tmp) {
      const float4* ut = reinterpret_cast<const float4*>(A.u_tmp + gofs);
      for (int k = tid; k < nval / 4; k += NT) cp_async16(reinterpret_cast<float4*>(s_ut) + k, ut + k);
    }
  }
  if (tid < 2 * EPB) s_smax[tid] = 0u;
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
      // apply_smoothing! as a gather (indicators_2d.jl:104-136)
      const int64_t e = e0 + tid;
      float a = A.alpha_raw[e];
      if (P.alpha_smooth)
#pragma unroll
        for (int f = 0; f < 4; ++f) {
          const int32_t nb = P.nbr[e * 4 + f];
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
    Node<2> nd;
    Dv::make_node(hi, lo, s_ref[sl], eos, nd);
    const int pn = cpos<N>(n);
#pragma unroll
    for (int v = 0; v < NV; ++v) s_nd[v * SP + pn] = nd.dw[v];
    s_nd[NV * SP + pn] = nd.dq;
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
      const RefState<2>& R = s_ref[sl];
      Node<2> nd[N];
      float ja[N][2];
#pragma unroll
      for (int a = 0; a < N; ++a) {
        const int q = cline_node<N>(line, dd, a);
        const int n = sl * NN + q;
#pragma unroll
        for (int v = 0; v < NV; ++v) nd[a].dw[v] = s_nd[v * SP + cpos<N>(n)];
        nd[a].dq = s_nd[NV * SP + cpos<N>(n)];
        Dv::complete(R, nd[a]);
        const float4 j = s_ja[n];
        ja[a][0] = dd ? j.z : j.x;
        ja[a][1] = dd ? j.w : j.y;
      }
      float acc[N][NV];
#pragma unroll
      for (int a = 0; a < N; ++a)
#pragma unroll
        for (int v = 0; v < NV; ++v) acc[a][v] = 0.0f;
      if (VI == VI_WEAK) {
#pragma unroll
        for (int a = 0; a < N; ++a) {
          Node<2> ax = nd[a], ay = nd[a];
          Dv::orient(ax, 0);
          Dv::orient(ay, 1);
          float fx[NV], fy[NV];
          Dv::dflux(R, ax, 0, R.v[0], eos, fx);
          Dv::dflux(R, ay, 1, R.v[1], eos, fy);
#pragma unroll
          for (int ii = 0; ii < N; ++ii) {
            const float c = P.Dhat32[ii * N + a];
#pragma unroll
            for (int v = 0; v < NV; ++v)
              acc[ii][v] = fmaf(c, fmaf(ja[a][1], fy[v], ja[a][0] * fx[v]), acc[ii][v]);
          }
        }
      } else {
#pragma unroll
        for (int a = 0; a < N; ++a)
#pragma unroll
          for (int b = a + 1; b < N; ++b) {
            float F[NV];
            const float n[2] = {0.5f * (ja[a][0] + ja[b][0]), 0.5f * (ja[a][1] + ja[b][1])};
            if constexpr (VF == FLUX_RANOCHA)
              dev_ranocha_n<2>(R, nd[a], nd[b], n, eos, F);
            else if constexpr (VF >= 0)
              dev_flux_n<2, VF>(VF, R, nd[a], nd[b], n, eos, F);
            else if (P.volume_flux == FLUX_RANOCHA)
              dev_ranocha_n<2>(R, nd[a], nd[b], n, eos, F);
            else
              dev_flux_n<2, -1>(P.volume_flux, R, nd[a], nd[b], n, eos, F);
            const float cab = P.Dsplit32[a * N + b], cba = P.Dsplit32[b * N + a];
#pragma unroll
            for (int v = 0; v < NV; ++v) {
              acc[a][v] = fmaf(cab, F[v], acc[a][v]);
              acc[b][v] = fmaf(cba, F[v], acc[b][v]);
            }
          }
      }
      if (VI == VI_HG) {
        // the FP64 kernel's blend in deviation form: the subcell flux
        // deviations F - f(w_ref) . n along the subcell normals, zero at the
        // element faces.  The dropped reference terms of the FD, FV and
        // surface parts cancel as for the unblended scheme: both volume
        // integrals are free-stream preserving with the same surface fluxes
        const float ae = s_alpha[sl];
        if (!(fabsf(ae) <= (float)P.alpha_atol)) {
#pragma unroll
          for (int a = 0; a < N; ++a) {
#pragma unroll
            for (int v = 0; v < NV; ++v) acc[a][v] *= 1.0f - ae;
            Dv::node_du(s_u + ((size_t)sl * NN + cline_node<N>(line, dd, a)) * NV, R, nd[a].du);
          }
          const float2* nv = P.snv32 + (((size_t)e * 2 + dd) * N + line) * (N - 1);
          float fl[NV] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
          for (int i = 0; i < N; ++i) {
            float fr[NV] = {0.0f, 0.0f, 0.0f, 0.0f};
            if (i < N - 1) {
              const float2 n2 = nv[i];
              const float n[2] = {n2.x, n2.y};
              dev_surface_k<2, SF>(P.fv_flux, R, nd[i], nd[i + 1], n, eos, fr);
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
        const int32_t nb = P.nbr[e * 4 + dir];
        const int own = side ? N - 1 : 0;
        Dv::node_du(s_u + ((size_t)sl * NN + cline_node<N>(line, dd, own)) * NV, R, nd[own].du);
        const float2* src = (nb >= e0 && nb < e0 + nel)
                                ? s_u + (((int)(nb - e0)) * NN + cface_partner<N>(dir, line)) * NV
                                : s_fu + ((sl * 4 + dir) * N + line) * NV;
        float hi[NV], lo[NV];
#pragma unroll
        for (int v = 0; v < NV; ++v) {
          hi[v] = src[v].x;
          lo[v] = src[v].y;
        }
        Node<2> other;
        Dv::make_node(hi, lo, R, eos, other);
        float F[NV];
        if (side)
          dev_surface_k<2, SF>(P.surface_flux, R, nd[own], other, ja[own], eos, F);
        else
          dev_surface_k<2, SF>(P.surface_flux, R, other, nd[own], ja[own], eos, F);
#pragma unroll
        for (int v = 0; v < NV; ++v) acc[own][v] = fmaf(side ? F[v] : -F[v], factor, acc[own][v]);
      }
#pragma unroll
      for (int a = 0; a < N; ++a) {
        const int q = cline_node<N>(line, dd, a);
#pragma unroll
        for (int v = 0; v < NV; ++v) s_part[(dd * NV + v) * SP + cpos<N>(sl * NN + q)] = acc[a][v];
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
    const float jfac = -s_ij[n];
    float du[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v)
      du[v] = (s_part[v * SP + cpos<N>(n)] + s_part[(NV + v) * SP + cpos<N>(n)]) * jfac;
    if (P.source == SRC_CONVERGENCE_TEST) {
      // sin/cos(pi (x + y - t)) by the angle-difference formula in float-float
      const float4 o = s_sc[n];
      const float2 sn = ff_dot2(o.x, o.z, ct, ctl, -o.y, -o.w, st, stl);
      const float2 cs = ff_dot2(o.y, o.w, ct, ctl, o.x, o.z, st, stl);
      float s[NV];
      SourceMMS<2>::eval(sn.x, cs.x, eos, s);
#pragma unroll
      for (int v = 0; v < NV; ++v) du[v] += s[v];
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
      Euler<2, float>::cons2prim(hi, w, eos.gamma);
      const float cs = sqrtf(eos.gamma * w[3] / w[0]);
      bad |= !(w[0] > 0.0f) || !(w[3] > 0.0f);
      const float l1 = fabsf(w[1]) + cs, l2 = fabsf(w[2]) + cs;
      const float4 j = s_ja[n];
      const float ij = fabsf(s_ij[n]);
      const float s1 = fabsf(j.x * l1 + j.y * l2) * ij;
      const float s2 = fabsf(j.z * l1 + j.w * l2) * ij;
      if (s1 == s1) atomicMax(&s_smax[2 * sl], __float_as_uint(s1));
      if (s2 == s2) atomicMax(&s_smax[2 * sl + 1], __float_as_uint(s2));
    }
  }
  if (bad) atomicOr(A.status, 1);
  if (stage && A.speed_bits) {
    __syncthreads();
    if (tid < nel) {
      const float sp = __uint_as_float(s_smax[2 * tid]) + __uint_as_float(s_smax[2 * tid + 1]);
      if (sp == sp) atomicMax(A.speed_bits, (unsigned long long)__double_as_longlong((double)sp));
    }
  }
}


template <int N, int VI, int VF, int SF>
static int launch_mixed2_one(const CurvedParams& P, const MixedArgs& A, cudaStream_t stream) {
  // elements per block: 8 for the polydeg-3 weak form (at 512^2 on the waving
  // flag 0.194 ms per stage against 0.208 with 16; flux differencing and shock
  // capturing were 3-4 % slower with 8); both give the same bits
  constexpr int EPB = (N == 5 || (N == 4 && VI == VI_WEAK)) ? 8 : 16;
  using K = CurvedK<N, EPB>;
  const unsigned nb = (unsigned)((P.nelements + EPB - 1) / EPB);
  const size_t smem = sizeof(float2) * (K::CHUNK + K::FACE) + sizeof(float4) * 2 * K::SP +
                      sizeof(float) * (4 * K::SP + K::SP) +
                      sizeof(float) * ((4 + 1) * K::SP + 2 * 4 * K::SP) +
                      sizeof(RefState<2>) * EPB + sizeof(float) * 4 +
                      sizeof(unsigned int) * 2 * EPB + sizeof(float) * EPB;
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(curved_kernel_mixed<N, VI, EPB, VF, SF>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    attr = true;
  }
  curved_kernel_mixed<N, VI, EPB, VF, SF><<<nb, K::NT, smem, stream>>>(P, A);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

// polydeg 3: flux_ranocha volume flux (flux differencing, shock capturing)
// with the Lax-Friedrichs or ranocha surface fluxes, the weak form with the
// Lax-Friedrichs ones
template <int VI>
static int launch_mixed2_n4(const CurvedParams& P, const MixedArgs& A, cudaStream_t stream) {
  const int sf = P.surface_flux;
  const bool lf = sf == FLUX_LLF || sf == FLUX_LLF_NAIVE;
  if constexpr (VI == VI_WEAK) {
    if (sf == FLUX_LLF) return launch_mixed2_one<4, VI, -1, FLUX_LLF>(P, A, stream);
    if (sf == FLUX_LLF_NAIVE) return launch_mixed2_one<4, VI, -1, FLUX_LLF_NAIVE>(P, A, stream);
  } else if constexpr (VI == VI_FD) {
    if (P.volume_flux == FLUX_RANOCHA) {
      if (sf == FLUX_LLF) return launch_mixed2_one<4, VI, FLUX_RANOCHA, FLUX_LLF>(P, A, stream);
      if (sf == FLUX_LLF_NAIVE)
        return launch_mixed2_one<4, VI, FLUX_RANOCHA, FLUX_LLF_NAIVE>(P, A, stream);
      if (sf == FLUX_RANOCHA)
        return launch_mixed2_one<4, VI, FLUX_RANOCHA, FLUX_RANOCHA>(P, A, stream);
    }
  } else {
    if (P.volume_flux == FLUX_RANOCHA && lf && P.fv_flux == sf) {
      if (sf == FLUX_LLF) return launch_mixed2_one<4, VI, FLUX_RANOCHA, FLUX_LLF>(P, A, stream);
      return launch_mixed2_one<4, VI, FLUX_RANOCHA, FLUX_LLF_NAIVE>(P, A, stream);
    }
  }
  return launch_mixed2_one<4, VI, -1, -1>(P, A, stream);
}

int launch_curved_mixed2(const CurvedParams& P, const MixedArgs& A, cudaStream_t stream) {
  switch (P.vi) {
    case VI_WEAK:
      switch (P.N) {
        case 3: return launch_mixed2_one<3, VI_WEAK, -1, -1>(P, A, stream);
        case 4: return launch_mixed2_n4<VI_WEAK>(P, A, stream);
        case 5: return launch_mixed2_one<5, VI_WEAK, -1, -1>(P, A, stream);
      }
      break;
    case VI_FD:
      switch (P.N) {
        case 3: return launch_mixed2_one<3, VI_FD, -1, -1>(P, A, stream);
        case 4: return launch_mixed2_n4<VI_FD>(P, A, stream);
        case 5: return launch_mixed2_one<5, VI_FD, -1, -1>(P, A, stream);
      }
      break;
    case VI_HG:
      switch (P.N) {
        case 3: return launch_mixed2_one<3, VI_HG, -1, -1>(P, A, stream);
        case 4: return launch_mixed2_n4<VI_HG>(P, A, stream);
        case 5: return launch_mixed2_one<5, VI_HG, -1, -1>(P, A, stream);
      }
      break;
  }
  return -3;
}

}  // namespace tg
