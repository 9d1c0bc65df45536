// Explicit instantiation of the mixed-precision element kernels (tg_mixed.cuh)
// for one (dimension, volume integral) pair; each tg_inst_*_mixed_*.cu unit
// defines TG_D, TG_VI and TG_SUFFIX and includes this file.
#include <algorithm>

#include "tg_mixed.cuh"

namespace tg {

template <int D, int N, int VI, int VF, int SF, int EPB, bool DIRECT = false>
static int launch_mixed_one(const MixedParams& P, const MixedArgs& A, cudaStream_t s) {
  using K = MixedKernel<D, N, VI, EPB>;
  const int64_t nblocks = (P.nelements + EPB - 1) / EPB;
  if (nblocks <= 0) return 0;
  // 2D: the persistent, double-buffered kernel with bulk-copy staging, one
  // block per resident slot (it needs the pre-smoothed blending factors).
  // Every bulk copy of an element block starts on a 16-byte boundary and
  // moves whole 16-byte groups: the per-element float rows (4 bytes per
  // element) need EPB % 4 == 0, the state chunks an even N^D (D + 2).  (The
  // same kernel on the 3D MMS mesh at 32^3, 4 elements per block, took 0.195
  // ms per stage against the per-block kernel's 0.186: 3 resident blocks of
  // 68 KB against 4 of 53 KB.)
  // 3D: the same kernel with 2 elements (96 threads) per block, 6 blocks per
  // SM, without shock capturing (whose 3D factors are smoothed inside the
  // per-block kernel)
  if constexpr ((Pow<N, D>::value * (D + 2)) % 2 == 0 &&
                ((D == 2 && EPB % 4 == 0) || (D == 3 && EPB == 2 && VI != VI_HG))) {
    if (VI != VI_HG || A.alpha_smoothed) {
      using Q = MixedPipe<D, N, VI, EPB>;
      auto kern = mixed_element_pipe_kernel<D, N, VI, VF, SF, EPB, DIRECT>;
      static int resident[64] = {0};
      static int sms[64] = {0};
      int dev = 0;
      if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return -1;
      if (resident[dev] == 0) {
        int occ = 0;
        if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)Q::SMEM) != cudaSuccess ||
            cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 (int)cudaSharedmemCarveoutMaxShared) != cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, K::NT, Q::SMEM) !=
                cudaSuccess ||
            cudaDeviceGetAttribute(&sms[dev], cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
          return -1;
        resident[dev] = occ > 0 ? occ : 1;
      }
      const int64_t grid = std::min<int64_t>(nblocks, (int64_t)sms[dev] * resident[dev]);
      kern<<<(unsigned)grid, K::NT, Q::SMEM, s>>>(P, A);
      return cudaGetLastError() == cudaSuccess ? 0 : -1;
    }
  }
  auto kern = mixed_element_kernel<D, N, VI, VF, SF, EPB, DIRECT>;
  static bool configured = false;
  const size_t smem = K::smem_bytes();
  if (!configured) {
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
      return -1;
    configured = true;
  }
  kern<<<(unsigned)nblocks, K::NT, smem, s>>>(P, A);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

// Flux-specialised instances for polydeg 3 (flux_ranocha volume flux with the
// two Lax-Friedrichs surface fluxes, and for shock capturing the surface flux
// as the subcell flux too); every other choice dispatches at run time.
// Meshes with faces of a given flux (slip walls, mortars) take the DIRECT
// instances, built for the default elements per block (DEF) only; other block
// sizes run those meshes through the run-time flux kernel.
template <int D, int VI, int EPB, bool DEF>
static int launch_mixed_n4(const MixedParams& P, const MixedArgs& A, cudaStream_t s) {
  constexpr int VF = VI == VI_WEAK ? -1 : FLUX_RANOCHA;
  const bool ranocha = (VI == VI_WEAK || P.volume_flux == FLUX_RANOCHA) &&
                       (VI != VI_HG || P.fv_flux == P.surface_flux);
  if (ranocha && !P.has_direct) {
    if (P.surface_flux == FLUX_LLF) return launch_mixed_one<D, 4, VI, VF, FLUX_LLF, EPB>(P, A, s);
    if (P.surface_flux == FLUX_LLF_NAIVE)
      return launch_mixed_one<D, 4, VI, VF, FLUX_LLF_NAIVE, EPB>(P, A, s);
  }
  if constexpr (DEF) {
    if (ranocha && P.has_direct) {
      if (P.surface_flux == FLUX_LLF)
        return launch_mixed_one<D, 4, VI, VF, FLUX_LLF, EPB, true>(P, A, s);
      if (P.surface_flux == FLUX_LLF_NAIVE)
        return launch_mixed_one<D, 4, VI, VF, FLUX_LLF_NAIVE, EPB, true>(P, A, s);
    }
  }
  return launch_mixed_one<D, 4, VI, -1, -1, EPB>(P, A, s);
}

#define TG_CAT2(a, b) a##b
#define TG_CAT(a, b) TG_CAT2(a, b)

// Elements per block (threads = EPB x lines per element); the first is the default.
int TG_CAT(launch_mixed_, TG_SUFFIX)(int N, int epb, const MixedParams& P, const MixedArgs& A,
                                     cudaStream_t s) {
#if TG_D == 2
  switch (N) {
    case 2: return launch_mixed_one<2, 2, TG_VI, -1, -1, 32>(P, A, s);
    case 3: return launch_mixed_one<2, 3, TG_VI, -1, -1, 32>(P, A, s);
    case 4:
      if (epb == 8) return launch_mixed_n4<2, TG_VI, 8, false>(P, A, s);
      if (epb == 32) return launch_mixed_n4<2, TG_VI, 32, false>(P, A, s);
      return launch_mixed_n4<2, TG_VI, 16, true>(P, A, s);
    case 5: return launch_mixed_one<2, 5, TG_VI, -1, -1, 16>(P, A, s);
    case 6: return launch_mixed_one<2, 6, TG_VI, -1, -1, 16>(P, A, s);
  }
#else
  switch (N) {
    case 2: return launch_mixed_one<3, 2, TG_VI, -1, -1, 16>(P, A, s);
    case 3: return launch_mixed_one<3, 3, TG_VI, -1, -1, 8>(P, A, s);
    case 4:
      // 2 elements per block (the persistent kernel without shock capturing,
      // the default) and 4 (shock capturing) both have the instances for
      // faces of a given flux
#if TG_VI != 2
      if (epb == 2) return launch_mixed_n4<3, TG_VI, 2, true>(P, A, s);
#else
      if (epb == 2) return launch_mixed_n4<3, TG_VI, 2, false>(P, A, s);
#endif
      if (epb == 8) return launch_mixed_n4<3, TG_VI, 8, false>(P, A, s);
      return launch_mixed_n4<3, TG_VI, 4, true>(P, A, s);
    case 5: return launch_mixed_one<3, 5, TG_VI, -1, -1, 2>(P, A, s);
  }
#endif
  return -2;
}

#if TG_VI == 2
template <int D, int N, int EPB>
static int launch_ind_mixed(const MixedParams& P, const float2* u, float* alpha, cudaStream_t s) {
  const int64_t nblocks = (P.nelements + EPB - 1) / EPB;
  if (nblocks <= 0) return 0;
  hg_indicator_kernel<D, N, float, EPB, MixedParams, float2>
      <<<(unsigned)nblocks, EPB * Pow<N, D>::value, 0, s>>>(P, u, alpha);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int TG_CAT(launch_indicator_mixed_, TG_D)(int N, const MixedParams& P, const float2* u,
                                          float* alpha, cudaStream_t s) {
#if TG_D == 2
  switch (N) {
    case 2: return launch_ind_mixed<2, 2, 64>(P, u, alpha, s);
    case 3: return launch_ind_mixed<2, 3, 28>(P, u, alpha, s);
    case 4: return launch_ind_mixed<2, 4, 16>(P, u, alpha, s);
    case 5: return launch_ind_mixed<2, 5, 10>(P, u, alpha, s);
    case 6: return launch_ind_mixed<2, 6, 7>(P, u, alpha, s);
  }
#else
  switch (N) {
    case 2: return launch_ind_mixed<3, 2, 32>(P, u, alpha, s);
    case 3: return launch_ind_mixed<3, 3, 9>(P, u, alpha, s);
    case 4: return launch_ind_mixed<3, 4, 4>(P, u, alpha, s);
    case 5: return launch_ind_mixed<3, 5, 2>(P, u, alpha, s);
  }
#endif
  return -2;
}

#if TG_D == 2
// IndicatorHennemannGassner from rho*p of the nodes ([E][N^2], the previous
// stage kernel's output) instead of the state: hg_indicator_kernel's modal
// transform (x, then y), energy and logistic in the same order, one thread per
// element.
template <int N>
__global__ void __launch_bounds__(128) hg_alpha_rp_kernel(const MixedParams P,
                                                          const float* __restrict__ rp,
                                                          float* __restrict__ alpha_raw) {
  constexpr int NN = N * N;
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= P.nelements) return;
  float a[NN], b[NN];
#pragma unroll
  for (int q = 0; q < NN; ++q) a[q] = __ldg(rp + e * NN + q);
#pragma unroll
  for (int j = 0; j < N; ++j)
#pragma unroll
    for (int i = 0; i < N; ++i) {
      float r = 0;
#pragma unroll
      for (int k = 0; k < N; ++k) r += P.Vinv[i * N + k] * a[k + N * j];
      b[i + N * j] = r;
    }
#pragma unroll
  for (int j = 0; j < N; ++j)
#pragma unroll
    for (int i = 0; i < N; ++i) {
      float r = 0;
#pragma unroll
      for (int k = 0; k < N; ++k) r += P.Vinv[j * N + k] * b[i + N * k];
      a[i + N * j] = r;
    }
  float clip2 = 0, clip1 = 0, tot = 0;
#pragma unroll
  for (int q = 0; q < NN; ++q) {
    const int mx = max(q % N, q / N);
    const float m2 = a[q] * a[q];
    if (mx <= N - 3) clip2 += m2;
    if (mx <= N - 2) clip1 += m2;
    tot += m2;
  }
  const float f1 = tot != 0.0f ? (tot - clip1) / tot : 0.0f;
  const float f2 = clip1 != 0.0f ? (clip1 - clip2) / clip1 : 0.0f;
  const float energy = fmaxf(f1, f2);
  const float thr = P.hg_threshold;
  float al = 1.0f / (1.0f + Real<float>::exp(-P.hg_parameter_s / thr * (energy - thr)));
  if (al < P.alpha_min) al = 0;
  if (al > 1.0f - P.alpha_min) al = 1;
  alpha_raw[e] = fminf(P.alpha_max, al);
}

int launch_hg_alpha_rp(int N, const MixedParams& P, const float* rp, float* alpha,
                       cudaStream_t s) {
  const unsigned nb = (unsigned)((P.nelements + 127) / 128);
  if (nb == 0) return 0;
  switch (N) {
    case 2: hg_alpha_rp_kernel<2><<<nb, 128, 0, s>>>(P, rp, alpha); break;
    case 3: hg_alpha_rp_kernel<3><<<nb, 128, 0, s>>>(P, rp, alpha); break;
    case 4: hg_alpha_rp_kernel<4><<<nb, 128, 0, s>>>(P, rp, alpha); break;
    case 5: hg_alpha_rp_kernel<5><<<nb, 128, 0, s>>>(P, rp, alpha); break;
    case 6: hg_alpha_rp_kernel<6><<<nb, 128, 0, s>>>(P, rp, alpha); break;
    default: return -2;
  }
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}
#endif
#endif

}  // namespace tg
